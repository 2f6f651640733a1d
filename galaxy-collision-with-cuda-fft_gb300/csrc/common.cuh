// Internal definitions shared by the gcpm translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <stdarg.h>
#include <string.h>

#include <utility>

#include "../../include/gcpm.h"

#define GC_MAX_LEVELS 24
// Levels with at most this many nodes per axis are relaxed together by one CTA.
#ifndef GC_TAIL_MAX_N
#define GC_TAIL_MAX_N 17
#endif

struct LevelGeom {
  int n;        // nodes per axis (array extent)
  int J;        // last interior index; interior is 1..J on every axis
  float a;      // Shortley-Weller weight of the west neighbour at i == J
  float dB;     // Shortley-Weller diagonal contribution of the boundary axis at i == J
  float p;      // far face position in this level's node units, (G-1)/2^l
};

// Slots of ctx->dsmall.
enum {
  GC_S_BNORM2 = 0,   // ||b0||^2 (h^2-scaled rhs, all nodes)
  GC_S_RNORM2 = 1,   // ||r0||^2 (interior) of the last residual evaluation
  GC_S_RHO_BAD = 4,  // count of non-finite density values (as double)
  GC_S_RNORM64 = 5,  // FP64 residual norm^2 (verification kernel)
  GC_S_GRIDPE = 6,   // Sum b0*phi (engine grid energy, h^2 4 pi G units)
  GC_S_MASS_PM = 7,  // engine: total density-mass of its particles
  GC_S_QEXP_PM = 8,  // engine: quantum exponent
  GC_S_CYCLES = 2,   // V-cycles of the last device-decided (graph-captured) solve
  GC_S_CONVERGED = 3,// 1 if that solve met its tolerance
  GC_S_MIRROR = 4,   // slots [0, 4) are copied to the pinned mirror by captured solves
  GC_S_GRIDBAR = 10, // [10, 12): grid-barrier words of the persistent coarse launches
  GC_S_MASS = 12,    // total deposited density-mass used for the fixed-point quantum
  GC_S_QEXP = 13,    // quantum exponent E: quantum = 2^E (density units)
  GC_S_SOLVES = 14,  // device-decided solves since the counters were reset ...
  GC_S_CYC_TOTAL = 15, // ... their V-cycles ...
  GC_S_MAXREL2 = 16, // ... and the largest (||r|| / ||b||)^2 they ended with
  GC_S_TICKET = 17,  // block ticket of the last-block grid reductions (an unsigned, 0 between them)
  GC_S_FIN_TMP = 128, // [128, 256): chunk partials of gc_finalize
  GC_S_NSLOTS = 256
};

// Kernel ids for launch counting and event timing (gc_profile_*).
enum gc_kernel_id {
  GK_DEPOSIT = 0, GK_DEPOSIT_RUNS, GK_CONVERT_Q, GK_MASS, GK_SMOOTH0, GK_RESID0, GK_RESTRICT, GK_SMOOTH,
  GK_RESID, GK_PROLONG, GK_PROLONG0, GK_TAIL, GK_FACES, GK_MOMENTS, GK_RHS, GK_REDUCE, GK_GATHER_KD,
  GK_GRAD, GK_GATHER, GK_AXPY, GK_KEYS, GK_SORT, GK_PERMUTE, GK_DIAG, GK_HIST, GK_RESID64, GK_COPY,
  GK_UPDATE0, GK_PROJECT, GK_WARMSTART, GK_VIZ, GK_IC, GK_RESIDE, GK_COARSE, GK_COUNT
};
extern const char *const gc_kernel_names[GK_COUNT];

#define GC_PROF_MAX_EVENTS 8192

struct gc_profiler {
  int enabled;
  long long launches[GK_COUNT];      // always counted
  int nrec;                          // recorded (start, stop) pairs since the last read
  int kid[GC_PROF_MAX_EVENTS];
  cudaEvent_t ev[2 * GC_PROF_MAX_EVENTS];
  int nev_created;
  double ms[GK_COUNT];               // accumulated by gc_profile_read
  long long timed[GK_COUNT];
};

struct gc_ctx {
  int G;
  double dx;
  double grav;
  cudaStream_t stream;
  int device;

  int coarse_blocks;    // CTAs of the persistent coarse-level launches (0: not sized yet)
  int capturing;        // a gc_pm_graph_create capture is in progress (no host reads, no events)
  cudaStream_t side;    // stream the V-cycle body of a captured solve is recorded on
  cudaStream_t fork;    // second stream of the engine step (the faces beside the warm-start passes)
  cudaEvent_t ev_fork, ev_join;  // its fork and join (no timing)
  long long cap_body_launches;  // kernel launches in that body (one V-cycle)
  int nlev;             // multigrid levels (0 = finest)
  int tail;             // first level handled by the single-CTA tail kernel (== nlev if none)
  LevelGeom lev[GC_MAX_LEVELS];

  // finest level: double-float potential hi + lo, h^2-scaled right-hand side b0,
  // natural-layout scratch r0 (residual of the correction, the restriction's
  // input); colour-split correction e0s and potential residual r0s (two halves
  // of half0 = G*G*H0 nodes, H0 = (G+1)/2); natural-layout correction and
  // residual e0n, r0n of the validation path (GC_MG_NATURAL_LAYOUT, lazily)
  float *hi, *lo, *b0, *r0;
  float *e0s, *r0s, *e0n, *r0n;
  size_t half0;
  int H0;
  // coarse levels (index >= 1): correction e and h^2-scaled right-hand side b
  float *e[GC_MAX_LEVELS];
  float *b[GC_MAX_LEVELS];
  float *rc;            // residual scratch for coarse levels (sized for level 1)

  long long *q;         // int64 fixed-point mass grid (G^3)
  void *g4;             // float4 node field -grad(phi) (G^3), allocated on first use
  double *red;          // reduction scratch (block partials)
  size_t red_cap;       // doubles in red
  double *dmom;         // 10 moments
  double *dsmall;       // GC_S_NSLOTS device scalars, see GC_S_* below
  double *hsmall;       // pinned host mirror of dsmall
  unsigned *dstatus;    // device status word
  double *ddiag;        // 16 doubles for diagnostics

  // particle scratch (grown on demand)
  uint32_t *keys, *keys2, *vals, *vals2;
  unsigned *hist;       // radix histogram (digits x blocks)
  unsigned *hist_aux;   // scan auxiliaries
  size_t pcap;          // capacity of the particle scratch (elements)
  size_t hist_cap;

  double mass_sum_cache; // sum of masses for the engine's fixed-point quantum
  int last_step_valid;
  int q_next_ready;     // q holds the deposit of the current positions (made by the last particle pass)
  int gt_smem_set;      // the TMA particle-pass kernels' dynamic shared-memory limit has been raised
  const uint32_t *import_perm;  // gc_pm_import_order's permutation (in the sort scratch) ...
  int64_t import_n;             // ... for this many particles (0: none pending)
  int64_t export_n;             // gc_pm_export_order's ranks (in ctx->keys) are for this many particles (0: none)
  const int32_t *export_pid;    // ... and for the particle set with this pid array
  int solved_once;
  gc_mg_stats last_stats;

  gc_profiler prof;

  // warm-start hook (coarse history of the potential on the (G/2)^3 grid)
  struct gc_ws *ws;     // attached network (learned mode), not owned
  int ws_mode;          // GC_WS_PLAIN / GC_WS_LEARNED / GC_WS_EXTRAPOLATE
  int ws_track;         // maintain the warm-start history (previous potential)
  int ws_coarse;        // also the coarse history and network features (learned mode or track = 1)
  int ws_hist;          // solves recorded in the history (0, 1, 2+)
  void *ws_record;      // one-shot f16 [5][R^3] sample destination
  int ws_skip;          // this step leaves the history alone (PRIME after CLOSE)
  int pending_push;     // a SOLVE_ONLY step awaits its PUSH_ONLY step
  float *ws_buf;        // rho_c, phi_c, delta_c, y (R^3 each) + scalars + partials
  size_t ws_buf_cap;

  char err[512];
};

int gc_ws_pre_solve(gc_ctx *ctx, int warm, int mode);
int gc_ws_post_solve(gc_ctx *ctx);

// Launch `k` on ctx's stream, counting it under `kid` and bracketing it with
// CUDA events when profiling is enabled.
int gc_prof_slot(gc_ctx *ctx, int kid);
template <typename... KArgs, typename... Args>
static inline void gc_launch(gc_ctx *ctx, int kid, void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem,
                             Args &&...args) {
  ctx->prof.launches[kid]++;
  const int slot = ctx->prof.enabled && !ctx->capturing ? gc_prof_slot(ctx, kid) : -1;
  if (slot >= 0) cudaEventRecord(ctx->prof.ev[2 * slot], ctx->stream);
  k<<<grid, block, smem, ctx->stream>>>(std::forward<Args>(args)...);
  if (slot >= 0) cudaEventRecord(ctx->prof.ev[2 * slot + 1], ctx->stream);
}

// Kernel launches counted on ctx so far (all ids).
static inline long long gc_launch_total(const gc_ctx *ctx) {
  long long t = 0;
  for (int k = 0; k < GK_COUNT; ++k) t += ctx->prof.launches[k];
  return t;
}

// ---- error helpers -----------------------------------------------------------
void gc_set_error(gc_ctx *ctx, const char *fmt, ...);
int gc_check_launch(gc_ctx *ctx, const char *what);

#define GC_CUDA(ctx, call)                                                              \
  do {                                                                                  \
    cudaError_t _e = (call);                                                            \
    if (_e != cudaSuccess) {                                                            \
      gc_set_error((ctx), "%s failed: %s (%s:%d)", #call, cudaGetErrorString(_e),       \
                   __FILE__, __LINE__);                                                 \
      return GC_ERR_CUDA;                                                               \
    }                                                                                   \
  } while (0)

#define GC_LAUNCH_CHECK(ctx, what)                                                      \
  do {                                                                                  \
    int _s = gc_check_launch((ctx), (what));                                            \
    if (_s != GC_OK) return _s;                                                         \
  } while (0)

#define GC_REQUIRE(ctx, cond, ...)                                                      \
  do {                                                                                  \
    if (!(cond)) {                                                                      \
      gc_set_error((ctx), __VA_ARGS__);                                                 \
      return GC_ERR_ARG;                                                                \
    }                                                                                   \
  } while (0)

int gc_ensure_red(gc_ctx *ctx, size_t ndoubles);
int gc_ensure_particle_scratch(gc_ctx *ctx, size_t n);

// Streaming multiprocessors of the current device (queried once per device and
// cached); persistent and grid-capped launches size their grids from it.
unsigned gc_sms(void);

static inline unsigned gc_blocks(long long n, int threads) {
  long long b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  return (unsigned)b;
}

// ---- double-float (FP32 pair) arithmetic ---------------------------------------
// Error-free transforms with explicit round-to-nearest intrinsics so that no
// contraction or reassociation can break them.
__device__ __forceinline__ void df_two_sum(float a, float b, float &s, float &e) {
  s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
__device__ __forceinline__ void df_fast_two_sum(float a, float b, float &s, float &e) {
  s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
}

// ---- reference CIC geometry (deposit.py:62-70) ---------------------------------
// gx = x/dx (IEEE f32 division), ix = floor(gx), fx = gx - ix. Non-finite or
// far-outside coordinates are reported as "no deposit" before any cast.
struct CellPos {
  int ix, iy, iz;
  float fx, fy, fz;
};

__device__ __forceinline__ bool gc_cell_of(float x, float y, float z, float dx, int G, CellPos &c) {
  float gx = __fdiv_rn(x, dx), gy = __fdiv_rn(y, dx), gz = __fdiv_rn(z, dx);
  // Every node the particle could touch is in [ix, ix+1]; keep -1 <= ix <= G-1.
  const float lo = -1.0f, hi = (float)G;  // gx < G  <=>  floor(gx) <= G-1
  if (!(gx >= lo && gx < hi && gy >= lo && gy < hi && gz >= lo && gz < hi)) return false;
  float flx = floorf(gx), fly = floorf(gy), flz = floorf(gz);
  c.ix = (int)flx; c.iy = (int)fly; c.iz = (int)flz;
  c.fx = __fsub_rn(gx, flx); c.fy = __fsub_rn(gy, fly); c.fz = __fsub_rn(gz, flz);
  return true;
}

// Parameters of the deposit kernels.
struct DepCtx {
  float dx;
  float inv_vol;  // 1/(dx*dx*dx) in f32, as the reference (deposit.py:58)
  int G;
};

// ---- exact int64 <-> f32 conversions in integer arithmetic --------------------
// cvt between f32 and 64-bit integers issues on the FP64 pipe, a small fraction
// of the FP32 rate on this part; these give the same results (round to nearest
// even) from the float bits and a leading-zero count, on the integer ALUs.
__device__ __forceinline__ long long f32_to_i64_rn(float v) {
  const unsigned u = __float_as_uint(v);
  int ex = (int)((u >> 23) & 0xffu);
  const unsigned mant = (u & 0x7fffffu) | (ex ? 0x800000u : 0u);
  if (ex == 0) ex = 1;
  const int sh = ex - 150;  // |v| = mant * 2^sh
  long long r;
  if (sh >= 0) {
    r = (long long)((unsigned long long)mant << sh);  // callers keep |v| < 2^62
  } else if (sh < -25) {
    r = 0;  // |v| < 0.25
  } else {
    const int rs = -sh;
    const unsigned long long m = mant;
    unsigned long long q = m >> rs;
    const unsigned long long rem = m & ((1ull << rs) - 1ull);
    const unsigned long long half = 1ull << (rs - 1);
    if (rem > half || (rem == half && (q & 1ull))) q += 1ull;
    r = (long long)q;
  }
  return (u >> 31) ? -r : r;
}

__device__ __forceinline__ float i64_to_f32_rn(long long q) {
  if (q == 0) return 0.0f;
  const unsigned long long a = q < 0 ? (0ull - (unsigned long long)q) : (unsigned long long)q;
  int msb = 63 - __clzll((long long)a);
  unsigned bits;
  if (msb <= 23) {
    bits = ((unsigned)(msb + 127) << 23) | ((unsigned)(a << (23 - msb)) & 0x7fffffu);
  } else {
    const int rs = msb - 23;
    unsigned long long m = a >> rs;
    const unsigned long long rem = a & ((1ull << rs) - 1ull);
    const unsigned long long half = 1ull << (rs - 1);
    if (rem > half || (rem == half && (m & 1ull))) {
      m += 1ull;
      if (m == (1ull << 24)) {
        m >>= 1;
        msb += 1;
      }
    }
    bits = ((unsigned)(msb + 127) << 23) | ((unsigned)m & 0x7fffffu);
  }
  if (q < 0) bits |= 0x80000000u;
  return __uint_as_float(bits);
}

// Is (x,y,z) finite? Used to raise GC_FLAG_NONFINITE_POS.
__device__ __forceinline__ bool gc_finite3(float x, float y, float z) {
  return isfinite(x) && isfinite(y) && isfinite(z);
}

// Block reduction: every thread passes NV values; thread 0 of the block writes
// their block sums to out[0..NV). Deterministic (fixed shuffle tree).
template <int NV>
__device__ __forceinline__ void block_partials(double (&v)[NV], double *out) {
  __shared__ double sh[32][NV];
  // flat thread index: the 2-D launches (32 x 8) have one warp per threadIdx.y row
  const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int lane = tid & 31;
  const int wid = tid >> 5;
  const int nw = (blockDim.x * blockDim.y * blockDim.z + 31) >> 5;
#pragma unroll
  for (int i = 0; i < NV; ++i) {
    double x = v[i];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    v[i] = x;
  }
  if (lane == 0) {
#pragma unroll
    for (int i = 0; i < NV; ++i) sh[wid][i] = v[i];
  }
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      double x = lane < nw ? sh[lane][i] : 0.0;
      for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
      if (lane == 0) out[i] = x;
    }
  }
}

// Single-value block sum reduced in FP32 (for norms, where ~1e-6 relative
// accuracy is ample) and written as a double partial; avoids per-element FP64,
// which runs at a small fraction of the FP32 rate on this part.
__device__ __forceinline__ void block_sum_f32(float v, double *out) {
  __shared__ float shf[32];
  const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int lane = tid & 31;
  const int wid = tid >> 5;
  const int nw = (blockDim.x * blockDim.y * blockDim.z + 31) >> 5;
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if (lane == 0) shf[wid] = v;
  __syncthreads();
  if (wid == 0) {
    float x = lane < nw ? shf[lane] : 0.0f;
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) *out = (double)x;
  }
}

// Last-block finish of a grid reduction of NV values per block, for grids of a
// few hundred blocks (every block takes a ticket on one counter). Every block
// has written its NV partials to parts[bid * NV + v] from its thread 0 (and
// calls this with all its threads); the block that takes the last ticket sums
// the nparts rows in a fixed order, writes the NV sums to dst[v] and resets
// the ticket to 0, so the sums do not depend on which block finishes last and
// no second launch is needed. Thread t adds value v = t mod NV of the rows
// g, g + P, ... (g = t / NV, P = T / NV threads per value) into eight
// accumulators; a warp per value then adds the P partials in order. Returns
// true in the last block.
template <int NV>
__device__ bool grid_finish_sum(const double *parts, unsigned nparts, unsigned *ticket, double *dst) {
  __shared__ bool last_s;
  __shared__ double part_s[1024];
  const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int nthr = blockDim.x * blockDim.y * blockDim.z;
  const int lane = tid & 31, wid = tid >> 5, nw = (nthr + 31) >> 5;
  __syncthreads();
  if (tid == 0) {
    __threadfence();  // this block's partials (written by thread 0) before its ticket
    last_s = atomicAdd(ticket, 1u) == nparts - 1u;
  }
  __syncthreads();
  if (!last_s) return false;
  __threadfence();  // every other block's partials after the last ticket
  const int P = nthr / NV, v = tid % NV, g = tid / NV;
  double xs[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  if (g < P) {
    for (unsigned q0 = (unsigned)g; q0 < nparts; q0 += 8u * (unsigned)P) {
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const unsigned q = q0 + (unsigned)u * (unsigned)P;
        if (q < nparts) xs[u] += __ldcg(parts + (size_t)q * NV + v);
      }
    }
  }
  part_s[tid] = ((xs[0] + xs[1]) + (xs[2] + xs[3])) + ((xs[4] + xs[5]) + (xs[6] + xs[7]));
  __syncthreads();
  for (int vv = wid; vv < NV; vv += nw) {
    double x = 0.0;
    for (int gg = lane; gg < P; gg += 32) x += part_s[gg * NV + vv];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) dst[vv] = x;
  }
  if (tid == 0) *ticket = 0u;
  __syncthreads();  // dst complete for every thread of the block
  return true;
}

// Internals shared between translation units
int gc_mg_build_levels(gc_ctx *ctx);
int gc_mg_alloc(gc_ctx *ctx);
void gc_mg_free(gc_ctx *ctx);
int gc_mg_run(gc_ctx *ctx, const gc_mg_params *p, gc_mg_stats *st);
int gc_faces_from_moments(gc_ctx *ctx);
int gc_finalize(gc_ctx *ctx, const double *parts, int nparts, int nv, double *dst);
// Sum of m/dx^3 (FP64, deterministic) into dsmall[mass_slot] and the fixed-point
// exponent E (quantum 2^E, total <= 2^bits quanta) into dsmall[exp_slot].
int gc_fixed_point_setup(gc_ctx *ctx, const float *m, int64_t n, int bits, int mass_slot, int exp_slot);
// int64 fixed-point CIC deposit into ctx->q (which must be zero on entry). Any
// particle order; runs of equal cells (cell-sorted input) are summed in registers.
int gc_deposit_q(gc_ctx *ctx, const float *x, const float *y, const float *z, const float *m, int64_t n,
                 const double *qexp);
// Read ctx->q, write rho (may be NULL) and b = f32(q 2^E 4 pi G h^2) (may be NULL),
// zero q, and reduce the ten moments into ctx->dmom and ||b||^2 into dsmall[GC_S_BNORM2].
int gc_convert_q(gc_ctx *ctx, const double *qexp, float *rho_out, float *b_out);
int gc_mg_check_params(gc_ctx *ctx, const gc_mg_params *p);
// The exact integer column moments of the fixed-point grid need
// (G-1) * 2^bits < 2^62: the largest allowed fixed_point_bits for this grid.
int gc_max_fixed_point_bits(const gc_ctx *ctx);
// Fused gather(-grad phi of ctx->hi) + kicks + drift over p (mode: gc_step_mode).
// With diag, writes nparts rows of 11 FP64 partials into ctx->red.
// With deposit_next (and a drifting mode) the bulk-streamed pass also deposits
// the new positions into ctx->q; *deposited tells whether it did.
int gc_gather_kick_drift(gc_ctx *ctx, const gc_particles *p, float dt, int mode, int diag, int grad_grid,
                         int deposit_next, float *axo, float *ayo, float *azo, int *nparts_out, int *deposited);
// dst = sum a*b in FP64 (async).
int gc_dot_async(gc_ctx *ctx, const float *a, const float *b, size_t n, double *dst);
// Stable LSD radix sort of (keys, vals) pairs on the low `bits` bits; the results
// are in the context's key/value scratch (*keys_out, *vals_out; the inputs may be
// one of its buffers). vals_in == NULL sorts the identity values 0 .. n-1.
int gc_radix_sort_pairs(gc_ctx *ctx, const uint32_t *keys_in, const uint32_t *vals_in, int64_t n, int bits,
                        uint32_t **keys_out, uint32_t **vals_out);
