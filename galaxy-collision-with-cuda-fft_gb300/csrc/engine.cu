// Fused PM step: the force chain of accel_fn (sim.py:320-325) and the KDK kicks
// and drift of kdk_step (integrator.py:100-131) in four device passes:
//   1. int64 fixed-point CIC deposit (run-aggregated for cell-sorted particles)
//   2. q -> b = 4 pi G h^2 rho, exact integer moments, ||b||, q cleared
//   3. FP64 multipole faces + adaptive multigrid on the double-float potential
//   4. one particle pass: gather of -grad(phi) computed on the fly, the closing
//      half-kick, FP64 diagnostics at the synchronised time, the opening
//      half-kick and the drift.
// The state between ADVANCE calls is (x_n, v_{n-1/2}); PRIME and CLOSE enter and
// leave the synchronised state, so PRIME + (K-1) ADVANCE + CLOSE reproduce K
// calls of kdk_step after the priming force evaluation.
#include "common.cuh"

#include <math.h>

#include <new>

// Phases 1-3: deposit, b0 + moments, initial guess, faces and V-cycles.
static int pm_solve(gc_ctx *ctx, const gc_particles *p, const gc_step_params *sp, gc_mg_stats *mst) {
  int s;
  const size_t g3 = (size_t)ctx->G * ctx->G * ctx->G;
  // 1. deposit (the quantum is fixed at PRIME: the masses do not change)
  if (sp->mode == GC_STEP_PRIME) {
    if ((s = gc_fixed_point_setup(ctx, p->m, p->n, sp->fixed_point_bits, GC_S_MASS_PM, GC_S_QEXP_PM))) return s;
  }
  // the previous particle pass may have deposited these positions already
  const bool have_q = ctx->q_next_ready && sp->mode != GC_STEP_PRIME && (sp->flags & GC_STEP_DEPOSIT_NEXT);
  ctx->q_next_ready = 0;
  if (!have_q && (s = gc_deposit_q(ctx, p->x, p->y, p->z, p->m, p->n, ctx->dsmall + GC_S_QEXP_PM))) return s;
  // 2. b0, moments, ||b0||
  if ((s = gc_convert_q(ctx, ctx->dsmall + GC_S_QEXP_PM, nullptr, ctx->b0))) return s;
  // 3. initial guess and faces, then V-cycles
  const int warm = sp->warm_start && ctx->solved_once;
  if (!warm) {
    GC_CUDA(ctx, cudaMemsetAsync(ctx->hi, 0, g3 * sizeof(float), ctx->stream));
    GC_CUDA(ctx, cudaMemsetAsync(ctx->lo, 0, g3 * sizeof(float), ctx->stream));
  }
  // The faces (FP64-bound) on the fork stream, beside the learned / extrapolated
  // correction of the previous potential and the sample recording (bound by
  // memory, and they leave the face nodes alone); joined before the V-cycles.
  if (!ctx->fork) {
    GC_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->fork, cudaStreamNonBlocking));
    GC_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming));
    GC_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming));
  }
  GC_CUDA(ctx, cudaEventRecord(ctx->ev_fork, ctx->stream));
  GC_CUDA(ctx, cudaStreamWaitEvent(ctx->fork, ctx->ev_fork, 0));
  {
    cudaStream_t main = ctx->stream;
    ctx->stream = ctx->fork;
    s = gc_faces_from_moments(ctx);
    ctx->stream = main;
    if (s) return s;
  }
  GC_CUDA(ctx, cudaEventRecord(ctx->ev_join, ctx->fork));
  if ((s = gc_ws_pre_solve(ctx, warm, sp->mode))) return s;
  GC_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ctx->ev_join, 0));
  return gc_mg_run(ctx, &sp->mg, mst);
}

// Phase 4: the particle pass, diagnostics, state and stats.
static int pm_push(gc_ctx *ctx, const gc_particles *p, const gc_step_params *sp, const gc_mg_stats &mst,
                   gc_step_stats *st) {
  int s;
  const size_t g3 = (size_t)ctx->G * ctx->G * ctx->G;
  int nparts = 0;
  int deposited = 0;
  if ((s = gc_gather_kick_drift(ctx, p, sp->dt, sp->mode, sp->diagnostics, (sp->flags & GC_STEP_GRAD_GRID) != 0,
                                (sp->flags & GC_STEP_DEPOSIT_NEXT) != 0, nullptr, nullptr, nullptr, &nparts,
                                &deposited)))
    return s;
  ctx->q_next_ready = deposited;
  if (sp->diagnostics) {
    if ((s = gc_finalize(ctx, ctx->red, nparts, 11, ctx->ddiag))) return s;
    if ((s = gc_dot_async(ctx, ctx->b0, ctx->hi, g3, ctx->ddiag + 11))) return s;
  }
  ctx->last_step_valid = (sp->mode != GC_STEP_CLOSE);
  if (st) {
    memset(st, 0, sizeof(*st));
    st->mg = mst;
    if (sp->diagnostics) {
      double h[12];
      GC_CUDA(ctx, cudaMemcpyAsync(h, ctx->ddiag, 12 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
      GC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
      for (int i = 0; i < 11; ++i) st->diag[i] = h[i];
      // sum rho phi = sum b0 phi / (4 pi G h^2)
      const double bfac = 4.0 * M_PI * ctx->grav * ctx->dx * ctx->dx;
      st->grid_pe_raw = bfac != 0.0 ? h[11] / bfac : 0.0;
    }
  }
  return GC_OK;
}

extern "C" int gc_pm_step(gc_ctx *ctx, const gc_particles *p, const gc_step_params *sp, gc_step_stats *st) {
  if (!ctx) return GC_ERR_ARG;
  GC_REQUIRE(ctx, p && sp, "gc_pm_step: NULL argument");
  GC_REQUIRE(ctx, p->n >= 0 && p->n < (1LL << 31), "particle count out of range");
  GC_REQUIRE(ctx, p->n == 0 || (p->x && p->y && p->z && p->vx && p->vy && p->vz && p->m),
             "gc_pm_step: particle arrays required");
  GC_REQUIRE(ctx, sp->mode >= GC_STEP_PRIME && sp->mode <= GC_STEP_CLOSE, "gc_pm_step: bad mode %d", sp->mode);
  GC_REQUIRE(ctx, sp->dt == sp->dt, "gc_pm_step: dt must be finite");
  GC_REQUIRE(ctx, sp->fixed_point_bits >= 24 && sp->fixed_point_bits <= gc_max_fixed_point_bits(ctx),
             "fixed_point_bits must be in [24, %d] for a %d^3 grid", gc_max_fixed_point_bits(ctx), ctx->G);
  if (sp->mode != GC_STEP_PRIME && !ctx->last_step_valid) {
    gc_set_error(ctx, "gc_pm_step: ADVANCE/CLOSE before PRIME");
    return GC_ERR_STATE;
  }
  int s = gc_mg_check_params(ctx, &sp->mg);
  if (s) return s;
  const int solve_only = (sp->flags & GC_STEP_SOLVE_ONLY) != 0, push_only = (sp->flags & GC_STEP_PUSH_ONLY) != 0;
  GC_REQUIRE(ctx, !(solve_only && push_only), "gc_pm_step: SOLVE_ONLY and PUSH_ONLY are exclusive");
  GC_REQUIRE(ctx, push_only == ctx->pending_push, "gc_pm_step: %s",
             push_only ? "PUSH_ONLY without a SOLVE_ONLY step before it" : "a SOLVE_ONLY step awaits its PUSH_ONLY");
  gc_mg_stats mst;
  memset(&mst, 0, sizeof(mst));
  if (push_only) {
    ctx->pending_push = 0;
    mst = ctx->last_stats;
  } else {
    if ((s = pm_solve(ctx, p, sp, &mst))) return s;
    if (solve_only) {  // the particle pass (and the history update) come with PUSH_ONLY
      ctx->pending_push = 1;
      if (st) {
        memset(st, 0, sizeof(*st));
        st->mg = mst;
      }
      return GC_OK;
    }
  }
  if ((s = gc_ws_post_solve(ctx))) return s;
  return pm_push(ctx, p, sp, mst, st);
}

// More V-cycles on the current potential until ||r|| < tol ||b|| (between a
// SOLVE_ONLY and a PUSH_ONLY step); adds the cycles run to *cycles.
extern "C" int gc_pm_refine(gc_ctx *ctx, const gc_mg_params *p, int *cycles) {
  if (!ctx) return GC_ERR_ARG;
  GC_REQUIRE(ctx, p, "gc_pm_refine: NULL params");
  int s = gc_mg_check_params(ctx, p);
  if (s) return s;
  gc_mg_params q = *p;
  q.flags &= ~GC_MG_FIXED_CYCLES;
  q.min_cycles = 0;
  const gc_mg_stats before = ctx->last_stats;
  gc_mg_stats st;
  if ((s = gc_mg_run(ctx, &q, &st))) return s;
  ctx->last_stats = before;
  ctx->last_stats.cycles += st.cycles;
  ctx->last_stats.converged = st.converged;
  ctx->last_stats.rhs_norm = st.rhs_norm;
  ctx->last_stats.res_norm = st.res_norm;
  if (cycles) *cycles = st.cycles;
  return GC_OK;
}

// Relative residual of the last fixed-cycle solve from the pinned host mirror the
// solve wrote (no copy, no synchronisation: the caller synchronised already).
extern "C" int gc_pm_residual_host(const gc_ctx *ctx, double *rel) {
  if (!ctx || !rel) return GC_ERR_ARG;
  const double b2 = ctx->hsmall[GC_S_BNORM2], r2 = ctx->hsmall[GC_S_RNORM2];
  *rel = b2 > 0.0 ? sqrt(r2) / sqrt(b2) : 0.0;
  return GC_OK;
}

extern "C" int gc_pm_last_residual(gc_ctx *ctx, double *rel) {
  if (!ctx) return GC_ERR_ARG;
  GC_REQUIRE(ctx, rel, "gc_pm_last_residual: NULL output");
  double h[2];
  GC_CUDA(ctx, cudaMemcpyAsync(&h[0], ctx->dsmall + GC_S_BNORM2, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  GC_CUDA(ctx, cudaMemcpyAsync(&h[1], ctx->dsmall + GC_S_RNORM2, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  GC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  *rel = h[0] > 0.0 ? sqrt(h[1]) / sqrt(h[0]) : 0.0;
  return GC_OK;
}

extern "C" int gc_pm_copy_potential(gc_ctx *ctx, float *phi) {
  if (!ctx) return GC_ERR_ARG;
  GC_REQUIRE(ctx, phi, "gc_pm_copy_potential: NULL phi");
  const size_t g3 = (size_t)ctx->G * ctx->G * ctx->G;
  GC_CUDA(ctx, cudaMemcpyAsync(phi, ctx->hi, g3 * sizeof(float), cudaMemcpyDeviceToDevice, ctx->stream));
  return GC_OK;
}

// ---- the whole step as one CUDA graph ------------------------------------------
// One ADVANCE step (deposit, conversion, initial guess, faces, the adaptive
// multigrid with its stopping rule decided on the device by a conditional while
// node, the particle pass) captured from the context's stream and instantiated.
// A replay makes no host synchronisation and runs exactly the kernels of an
// eager gc_pm_step, so the state is the same bit for bit. Host-side state that
// a step advances (warm-start history depth, pending deposit) must be stationary:
// capture after at least three steps with the same flags.
struct gc_graph {
  gc_ctx *ctx;
  cudaGraphExec_t exec;
  long long fixed_launches;  // kernels outside the V-cycle loop
  long long body_launches;   // kernels per V-cycle
};

extern "C" int gc_pm_graph_create(gc_ctx *ctx, const gc_particles *p, const gc_step_params *sp, gc_graph **out) {
  if (!ctx) return GC_ERR_ARG;
  GC_REQUIRE(ctx, p && sp && out, "gc_pm_graph_create: NULL argument");
  *out = nullptr;
  GC_REQUIRE(ctx, sp->mode == GC_STEP_ADVANCE, "gc_pm_graph_create: only ADVANCE steps are captured");
  GC_REQUIRE(ctx, !(sp->flags & (GC_STEP_SOLVE_ONLY | GC_STEP_PUSH_ONLY)), "gc_pm_graph_create: split steps");
  GC_REQUIRE(ctx, !sp->diagnostics, "gc_pm_graph_create: diagnostics steps read the host");
  GC_REQUIRE(ctx, ctx->stream != nullptr, "gc_pm_graph_create: set a non-default stream (gc_set_stream) first");
  GC_REQUIRE(ctx, ctx->last_step_valid && ctx->solved_once && !ctx->pending_push,
             "gc_pm_graph_create: needs an open engine that has stepped");
  GC_REQUIRE(ctx, p->n > 0 && p->n < (1LL << 31) && p->x && p->y && p->z && p->vx && p->vy && p->vz && p->m,
             "gc_pm_graph_create: particle arrays required");
  int s = gc_mg_check_params(ctx, &sp->mg);
  if (s) return s;
  if (!ctx->side) GC_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking));
  GC_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeRelaxed));
  ctx->capturing = 1;
  ctx->cap_body_launches = 0;
  const long long before = gc_launch_total(ctx);
  gc_mg_stats mst;
  memset(&mst, 0, sizeof(mst));
  s = pm_solve(ctx, p, sp, &mst);
  if (!s) s = gc_ws_post_solve(ctx);
  if (!s) s = pm_push(ctx, p, sp, mst, nullptr);
  const long long total = gc_launch_total(ctx) - before;
  ctx->capturing = 0;
  cudaGraph_t g = nullptr;
  const cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
  if (s || e != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    if (!s) {
      gc_set_error(ctx, "gc_pm_graph_create: capture failed: %s", cudaGetErrorString(e));
      s = GC_ERR_CUDA;
    }
    return s;
  }
  cudaGraphExec_t exec = nullptr;
  const cudaError_t ei = cudaGraphInstantiate(&exec, g, 0);
  cudaGraphDestroy(g);
  if (ei != cudaSuccess) {
    gc_set_error(ctx, "gc_pm_graph_create: instantiate failed: %s", cudaGetErrorString(ei));
    return GC_ERR_CUDA;
  }
  gc_graph *gr = new (std::nothrow) gc_graph();
  if (!gr) {
    cudaGraphExecDestroy(exec);
    return GC_ERR_CUDA;
  }
  gr->ctx = ctx;
  gr->exec = exec;
  gr->body_launches = ctx->cap_body_launches;
  gr->fixed_launches = total - ctx->cap_body_launches;
  *out = gr;
  return GC_OK;
}

extern "C" int gc_pm_graph_launch(gc_graph *g) {
  if (!g) return GC_ERR_ARG;
  gc_ctx *ctx = g->ctx;
  GC_CUDA(ctx, cudaGraphLaunch(g->exec, ctx->stream));
  return GC_OK;
}

extern "C" int gc_pm_graph_info(const gc_graph *g, long long *fixed_launches, long long *body_launches) {
  if (!g) return GC_ERR_ARG;
  if (fixed_launches) *fixed_launches = g->fixed_launches;
  if (body_launches) *body_launches = g->body_launches;
  return GC_OK;
}

extern "C" int gc_pm_graph_destroy(gc_graph *g) {
  if (!g) return GC_OK;
  cudaGraphExecDestroy(g->exec);
  delete g;
  return GC_OK;
}

// V-cycles, converged flag and relative residual of the last graph-replayed
// solve, from the pinned mirror its graph wrote (no copy, no synchronisation:
// the caller has synchronised the stream).
extern "C" int gc_pm_graph_stats(const gc_ctx *ctx, int *cycles, int *converged, double *rel) {
  if (!ctx) return GC_ERR_ARG;
  const double b2 = ctx->hsmall[GC_S_BNORM2], r2 = ctx->hsmall[GC_S_RNORM2];
  if (cycles) *cycles = (int)ctx->hsmall[GC_S_CYCLES];
  if (converged) *converged = ctx->hsmall[GC_S_CONVERGED] != 0.0;
  if (rel) *rel = b2 > 0.0 ? sqrt(r2) / sqrt(b2) : 0.0;
  return GC_OK;
}

// Solves decided on the device (graph replays) since the last reset: count,
// total V-cycles and the largest relative residual they ended with.
// Synchronises; reset clears the counters afterwards.
extern "C" int gc_pm_solve_counters(gc_ctx *ctx, double out[3], int reset) {
  if (!ctx) return GC_ERR_ARG;
  GC_REQUIRE(ctx, out, "gc_pm_solve_counters: NULL output");
  double h[3];
  GC_CUDA(ctx, cudaMemcpyAsync(h, ctx->dsmall + GC_S_SOLVES, 3 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  GC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  out[0] = h[0];
  out[1] = h[1];
  out[2] = sqrt(h[2]);
  if (reset) {
    GC_CUDA(ctx, cudaMemsetAsync(ctx->dsmall + GC_S_SOLVES, 0, 3 * sizeof(double), ctx->stream));
    GC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  }
  return GC_OK;
}
