// Context lifetime, error reporting and scratch management.
#include "common.cuh"

#include <stdlib.h>

static char g_create_err[512] = "";

const char *const gc_kernel_names[GK_COUNT] = {
    "deposit", "deposit_runs", "convert_q", "mass_setup", "smooth0", "resid0", "restrict", "smooth",
    "resid", "prolong", "prolong0", "tail", "faces", "moments", "rhs", "reduce", "gather_kick_drift",
    "grad", "gather", "axpy", "cell_keys", "radix_sort", "permute", "diag", "radial_hist", "resid64", "copy",
    "update0", "project_ngp", "warmstart", "viz", "ic", "resid0e", "coarse"};

int gc_prof_slot(gc_ctx *ctx, int kid) {
  gc_profiler &p = ctx->prof;
  if (p.nrec >= GC_PROF_MAX_EVENTS) return -1;
  const int slot = p.nrec;
  if (slot >= p.nev_created) {
    if (cudaEventCreate(&p.ev[2 * slot]) != cudaSuccess) return -1;
    if (cudaEventCreate(&p.ev[2 * slot + 1]) != cudaSuccess) return -1;
    p.nev_created = slot + 1;
  }
  p.kid[slot] = kid;
  p.nrec++;
  return slot;
}

extern "C" int gc_profile_enable(gc_ctx *ctx, int enable) {
  if (!ctx) return GC_ERR_ARG;
  ctx->prof.enabled = enable ? 1 : 0;
  return GC_OK;
}

extern "C" int gc_num_kernel_ids(void) { return GK_COUNT; }

extern "C" const char *gc_kernel_name(int kid) { return (kid >= 0 && kid < GK_COUNT) ? gc_kernel_names[kid] : ""; }

// Fold the recorded event pairs into per-kernel totals (synchronises), then
// report launches (always counted), timed launches and milliseconds of kid.
extern "C" int gc_profile_read(gc_ctx *ctx, int kid, long long *launches, long long *timed, double *ms) {
  if (!ctx || kid < 0 || kid >= GK_COUNT) return GC_ERR_ARG;
  gc_profiler &p = ctx->prof;
  if (p.nrec > 0) {
    GC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (int i = 0; i < p.nrec; ++i) {
      float t = 0.f;
      if (cudaEventElapsedTime(&t, p.ev[2 * i], p.ev[2 * i + 1]) == cudaSuccess) {
        p.ms[p.kid[i]] += t;
        p.timed[p.kid[i]]++;
      }
    }
    p.nrec = 0;
  }
  if (launches) *launches = p.launches[kid];
  if (timed) *timed = p.timed[kid];
  if (ms) *ms = p.ms[kid];
  return GC_OK;
}

extern "C" int gc_profile_reset(gc_ctx *ctx) {
  if (!ctx) return GC_ERR_ARG;
  GC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  gc_profiler &p = ctx->prof;
  p.nrec = 0;
  for (int k = 0; k < GK_COUNT; ++k) {
    p.launches[k] = 0;
    p.timed[k] = 0;
    p.ms[k] = 0.0;
  }
  return GC_OK;
}

unsigned gc_sms(void) {
  static int cache[64];  // 0: not queried yet
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 1;
  int v = __atomic_load_n(&cache[dev], __ATOMIC_RELAXED);
  if (v <= 0) {
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) v = 1;
    __atomic_store_n(&cache[dev], v, __ATOMIC_RELAXED);
  }
  return (unsigned)v;
}

void gc_set_error(gc_ctx *ctx, const char *fmt, ...) {
  char *dst = ctx ? ctx->err : g_create_err;
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(dst, 512, fmt, ap);
  va_end(ap);
}

int gc_check_launch(gc_ctx *ctx, const char *what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    gc_set_error(ctx, "kernel %s: %s", what, cudaGetErrorString(e));
    return GC_ERR_CUDA;
  }
  return GC_OK;
}

int gc_ensure_red(gc_ctx *ctx, size_t ndoubles) {
  if (ctx->red_cap >= ndoubles) return GC_OK;
  if (ctx->red) {
    GC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    cudaFree(ctx->red);
    ctx->red = nullptr;
  }
  size_t cap = ndoubles < 4096 ? 4096 : ndoubles;
  GC_CUDA(ctx, cudaMalloc(&ctx->red, cap * sizeof(double)));
  ctx->red_cap = cap;
  return GC_OK;
}

int gc_ensure_particle_scratch(gc_ctx *ctx, size_t n) {
  if (ctx->pcap >= n) return GC_OK;
  ctx->import_n = 0;  // a kept import order or export rank lives in these buffers
  ctx->import_perm = nullptr;
  ctx->export_n = 0;
  GC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  cudaFree(ctx->keys); cudaFree(ctx->keys2); cudaFree(ctx->vals); cudaFree(ctx->vals2);
  ctx->keys = ctx->keys2 = ctx->vals = ctx->vals2 = nullptr;
  ctx->pcap = 0;
  size_t cap = n + n / 8 + 1024;
  GC_CUDA(ctx, cudaMalloc(&ctx->keys, cap * sizeof(uint32_t)));
  GC_CUDA(ctx, cudaMalloc(&ctx->keys2, cap * sizeof(uint32_t)));
  GC_CUDA(ctx, cudaMalloc(&ctx->vals, cap * sizeof(uint32_t)));
  GC_CUDA(ctx, cudaMalloc(&ctx->vals2, cap * sizeof(uint32_t)));
  ctx->pcap = cap;
  return GC_OK;
}

extern "C" int gc_abi_version(void) { return GC_ABI_VERSION; }

extern "C" const char *gc_last_error(const gc_ctx *ctx) { return ctx ? ctx->err : g_create_err; }

extern "C" int gc_ctx_create(gc_ctx **out, int grid_size, double dx, double grav_constant) {
  if (!out) {
    gc_set_error(nullptr, "gc_ctx_create: out is NULL");
    return GC_ERR_ARG;
  }
  *out = nullptr;
  if (grid_size < 2 || grid_size > 1024) {
    gc_set_error(nullptr, "grid_size must be in [2, 1024], got %d", grid_size);
    return GC_ERR_ARG;
  }
  if (!(dx > 0.0) || !(dx < 1e30)) {
    gc_set_error(nullptr, "dx must be positive and finite, got %g", dx);
    return GC_ERR_ARG;
  }
  if (!(grav_constant == grav_constant)) {
    gc_set_error(nullptr, "grav_constant must be finite");
    return GC_ERR_ARG;
  }
  gc_ctx *ctx = (gc_ctx *)calloc(1, sizeof(gc_ctx));
  if (!ctx) {
    gc_set_error(nullptr, "out of host memory");
    return GC_ERR_ARG;
  }
  ctx->G = grid_size;
  ctx->dx = dx;
  ctx->grav = grav_constant;
  ctx->stream = 0;
  cudaError_t e = cudaGetDevice(&ctx->device);
  int st = GC_OK;
  if (e != cudaSuccess) {
    gc_set_error(nullptr, "cudaGetDevice: %s", cudaGetErrorString(e));
    free(ctx);
    return GC_ERR_CUDA;
  }
  st = gc_mg_build_levels(ctx);
  if (st == GC_OK) st = gc_mg_alloc(ctx);
  if (st == GC_OK) {
    size_t g3 = (size_t)grid_size * grid_size * grid_size;
    if (cudaMalloc(&ctx->q, g3 * sizeof(long long)) != cudaSuccess ||
        cudaMemset(ctx->q, 0, g3 * sizeof(long long)) != cudaSuccess ||
        cudaMalloc(&ctx->dmom, 16 * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&ctx->dsmall, GC_S_NSLOTS * sizeof(double)) != cudaSuccess ||
        cudaMemset(ctx->dsmall, 0, GC_S_NSLOTS * sizeof(double)) != cudaSuccess ||
        cudaMallocHost(&ctx->hsmall, GC_S_NSLOTS * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&ctx->dstatus, sizeof(unsigned)) != cudaSuccess ||
        cudaMemset(ctx->dstatus, 0, sizeof(unsigned)) != cudaSuccess ||
        cudaMalloc(&ctx->ddiag, 32 * sizeof(double)) != cudaSuccess) {
      snprintf(ctx->err, sizeof(ctx->err), "device allocation failed: %s",
               cudaGetErrorString(cudaGetLastError()));
      st = GC_ERR_CUDA;
    }
  }
  if (st == GC_OK) st = gc_ensure_red(ctx, 1 << 16);
  if (st == GC_OK) {
    cudaError_t se = cudaDeviceSynchronize();
    if (se != cudaSuccess) {
      snprintf(ctx->err, sizeof(ctx->err), "synchronize after create: %s", cudaGetErrorString(se));
      st = GC_ERR_CUDA;
    }
  }
  if (st != GC_OK) {
    snprintf(g_create_err, sizeof(g_create_err), "%s", ctx->err);
    gc_ctx_destroy(ctx);
    return st;
  }
  *out = ctx;
  return GC_OK;
}

extern "C" int gc_ctx_destroy(gc_ctx *ctx) {
  if (!ctx) return GC_OK;
  cudaStreamSynchronize(ctx->stream);
  gc_mg_free(ctx);
  cudaFree(ctx->q);
  cudaFree(ctx->g4);
  cudaFree(ctx->ws_buf);
  cudaFree(ctx->red);
  cudaFree(ctx->dmom);
  cudaFree(ctx->dsmall);
  if (ctx->hsmall) cudaFreeHost(ctx->hsmall);
  cudaFree(ctx->dstatus);
  cudaFree(ctx->ddiag);
  cudaFree(ctx->keys); cudaFree(ctx->keys2); cudaFree(ctx->vals); cudaFree(ctx->vals2);
  cudaFree(ctx->hist); cudaFree(ctx->hist_aux);
  for (int i = 0; i < 2 * ctx->prof.nev_created; ++i) cudaEventDestroy(ctx->prof.ev[i]);
  if (ctx->side) cudaStreamDestroy(ctx->side);
  if (ctx->fork) cudaStreamDestroy(ctx->fork);
  if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
  if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
  free(ctx);
  return GC_OK;
}

extern "C" int gc_set_stream(gc_ctx *ctx, void *stream) {
  if (!ctx) return GC_ERR_ARG;
  ctx->stream = (cudaStream_t)stream;
  return GC_OK;
}

extern "C" int gc_status(gc_ctx *ctx, uint32_t *flags_out, int clear) {
  if (!ctx) return GC_ERR_ARG;
  unsigned h = 0;
  GC_CUDA(ctx, cudaMemcpyAsync(&h, ctx->dstatus, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
  GC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (clear) GC_CUDA(ctx, cudaMemsetAsync(ctx->dstatus, 0, sizeof(unsigned), ctx->stream));
  if (flags_out) *flags_out = h;
  return GC_OK;
}

extern "C" int gc_num_levels(const gc_ctx *ctx) { return ctx ? ctx->nlev : 0; }

extern "C" int gc_level_info(const gc_ctx *ctx, int level, int *n_nodes, int *last_interior,
                             double *far_face) {
  if (!ctx || level < 0 || level >= ctx->nlev) return GC_ERR_ARG;
  if (n_nodes) *n_nodes = ctx->lev[level].n;
  if (last_interior) *last_interior = ctx->lev[level].J;
  if (far_face) *far_face = (double)(ctx->G - 1) / (double)(1 << level);
  return GC_OK;
}

extern "C" void gc_mg_default_params(gc_mg_params *p) {
  if (!p) return;
  p->pre_sweeps = 2;
  p->post_sweeps = 2;
  p->coarse_sweeps = 40;
  p->max_cycles = 20;
  p->min_cycles = 1;
  p->flags = 0;
  p->tol = 1e-3;
}
