// Open-boundary multigrid Poisson solver for laplacian(phi) = 4 pi G rho.
//
// The discrete problem is the reference's (src/galaxy_collision/solver/multigrid.py):
// 7-point Laplacian on the finest node grid, Dirichlet faces from the monopole +
// quadrupole of rho about its centre of mass (multigrid.py:261-295), residual
// ||rhs - L phi||_2 against ||rhs||_2 (multigrid.py:473-485). Only the finest
// level defines the answer (multigrid.py:8-15), so the hierarchy is free:
//
//  * Level l has its far face at p_l = (G-1)/2^l (in level-l node units). Coarse
//    node J <-> fine node 2J. When p_l is fractional the last interior node J_l
//    uses a Shortley-Weller stencil with the Dirichlet face at distance
//    delta = p_l - J_l, and the transfer operators interpolate to that face. The
//    reference instead cuts the coarse grid at fine node 2(n/2)-2 and converges
//    at ~0.6-0.7 per V-cycle; this hierarchy converges at ~0.1.
//  * The finest level relaxes the potential itself as a double-float pair
//    (hi + lo, both FP32): each red-black Gauss-Seidel update is computed from
//    an accurate local residual (exact neighbour differences summed with
//    error-free transforms), so the residual can be driven below the FP32 floor
//    (~6e-5 relative in the reference) with FP32 arithmetic only. This is the
//    defect-correction loop: coarse levels relax FP32 corrections of that
//    residual, the coarsest level is solved in FP64.
//  * All arrays are C-order [i][j][k], k fastest. Right-hand sides are stored
//    h^2-scaled (b = h^2 * rhs) so stencils need no division by h^2.
#include "common.cuh"

#include <math.h>
#include <stdlib.h>

#define RB_TX 32
#define RB_TY 8

// ------------------------------------------------------------------------------
// level geometry
// ------------------------------------------------------------------------------
int gc_mg_build_levels(gc_ctx *ctx) {
  const int G = ctx->G;
  ctx->nlev = 0;
  ctx->tail = 0;
  if (G - 2 < 1) return GC_OK;  // no interior node: the solve is the boundary alone
  LevelGeom g0;
  g0.n = G;
  g0.J = G - 2;
  g0.a = 1.0f;
  g0.dB = 2.0f;
  g0.p = (float)(G - 1);
  ctx->lev[0] = g0;
  int nl = 1;
  for (int l = 1; l < GC_MAX_LEVELS; ++l) {
    double p = (double)(G - 1) / (double)(1 << l);
    int J = (int)ceil(p) - 1;
    if (J < 1) break;
    double delta = p - (double)J;
    LevelGeom g;
    g.n = J + 2;
    g.J = J;
    g.a = (float)(2.0 / (1.0 + delta));
    g.dB = (float)(2.0 / delta);
    g.p = (float)p;
    ctx->lev[nl++] = g;
  }
  ctx->nlev = nl;
  int tail = nl;
  for (int l = 1; l < nl; ++l) {
    if (ctx->lev[l].n <= GC_TAIL_MAX_N) {
      tail = l;
      break;
    }
  }
  ctx->tail = tail;
  return GC_OK;
}

static size_t tail_smem_bytes(const gc_ctx *ctx) {
  size_t bytes = 0;
  for (int l = ctx->tail; l < ctx->nlev; ++l) {
    size_t n3 = (size_t)ctx->lev[l].n * ctx->lev[l].n * ctx->lev[l].n;
    if (l == ctx->nlev - 1)
      bytes += 2 * n3 * sizeof(double);
    else
      bytes += 3 * n3 * sizeof(float);
    bytes = (bytes + 15) & ~(size_t)15;
  }
  return bytes;
}

int gc_mg_alloc(gc_ctx *ctx) {
  const size_t G = ctx->G;
  const size_t g3 = G * G * G;
  ctx->H0 = (ctx->G + 1) / 2;
  ctx->half0 = G * G * (size_t)ctx->H0;
  GC_CUDA(ctx, cudaMalloc(&ctx->hi, g3 * sizeof(float)));
  GC_CUDA(ctx, cudaMalloc(&ctx->lo, g3 * sizeof(float)));
  GC_CUDA(ctx, cudaMalloc(&ctx->b0, g3 * sizeof(float)));
  GC_CUDA(ctx, cudaMalloc(&ctx->r0, g3 * sizeof(float)));
  GC_CUDA(ctx, cudaMemset(ctx->hi, 0, g3 * sizeof(float)));
  GC_CUDA(ctx, cudaMemset(ctx->lo, 0, g3 * sizeof(float)));
  GC_CUDA(ctx, cudaMemset(ctx->b0, 0, g3 * sizeof(float)));
  GC_CUDA(ctx, cudaMemset(ctx->r0, 0, g3 * sizeof(float)));
  // colour-split correction and residual of the finest level (faces stay zero)
  GC_CUDA(ctx, cudaMalloc(&ctx->e0s, 2 * ctx->half0 * sizeof(float)));
  GC_CUDA(ctx, cudaMalloc(&ctx->r0s, 2 * ctx->half0 * sizeof(float)));
  GC_CUDA(ctx, cudaMemset(ctx->e0s, 0, 2 * ctx->half0 * sizeof(float)));
  GC_CUDA(ctx, cudaMemset(ctx->r0s, 0, 2 * ctx->half0 * sizeof(float)));
  size_t rc_n = 0;
  for (int l = 1; l < ctx->nlev; ++l) {
    size_t n3 = (size_t)ctx->lev[l].n * ctx->lev[l].n * ctx->lev[l].n;
    GC_CUDA(ctx, cudaMalloc(&ctx->e[l], n3 * sizeof(float)));
    GC_CUDA(ctx, cudaMalloc(&ctx->b[l], n3 * sizeof(float)));
    GC_CUDA(ctx, cudaMemset(ctx->e[l], 0, n3 * sizeof(float)));
    GC_CUDA(ctx, cudaMemset(ctx->b[l], 0, n3 * sizeof(float)));
    if (l < ctx->tail && n3 > rc_n) rc_n = n3;
  }
  if (rc_n) {
    GC_CUDA(ctx, cudaMalloc(&ctx->rc, rc_n * sizeof(float)));
    GC_CUDA(ctx, cudaMemset(ctx->rc, 0, rc_n * sizeof(float)));
  }
  return GC_OK;
}

// Natural-layout correction and residual of the finest level, for
// GC_MG_NATURAL_LAYOUT (allocated on first use).
static int mg_alloc_natural(gc_ctx *ctx) {
  if (ctx->e0n) return GC_OK;
  const size_t g3 = (size_t)ctx->G * ctx->G * ctx->G;
  GC_CUDA(ctx, cudaMalloc(&ctx->e0n, g3 * sizeof(float)));
  GC_CUDA(ctx, cudaMalloc(&ctx->r0n, g3 * sizeof(float)));
  GC_CUDA(ctx, cudaMemset(ctx->e0n, 0, g3 * sizeof(float)));
  GC_CUDA(ctx, cudaMemset(ctx->r0n, 0, g3 * sizeof(float)));
  return GC_OK;
}

void gc_mg_free(gc_ctx *ctx) {
  cudaFree(ctx->hi); cudaFree(ctx->lo);
  cudaFree(ctx->b0); cudaFree(ctx->r0);
  cudaFree(ctx->e0s); cudaFree(ctx->r0s); cudaFree(ctx->e0n); cudaFree(ctx->r0n);
  for (int l = 1; l < GC_MAX_LEVELS; ++l) {
    cudaFree(ctx->e[l]); cudaFree(ctx->b[l]);
    ctx->e[l] = ctx->b[l] = nullptr;
  }
  cudaFree(ctx->rc);
  ctx->hi = ctx->lo = ctx->b0 = ctx->r0 = ctx->rc = nullptr;
  ctx->e0s = ctx->r0s = ctx->e0n = ctx->r0n = nullptr;
}

// ------------------------------------------------------------------------------
// reductions: per-block partials written in a fixed order, then one block sums them
// ------------------------------------------------------------------------------
// Sum nparts rows of nv partials into dst[0..nv), deterministically (a fixed
// association for given nparts and nv). FP64 runs at a small fraction of the
// f32 rate on this GPU, so the adds are spread: warp w of one block sums value
// w (lanes take rows lane, lane + 32, ...); a long single-value list is first
// cut into GC_FIN_CHUNKS contiguous chunks summed by as many blocks.
#define GC_FIN_NV 32
#define GC_FIN_CHUNKS 128
__global__ void __launch_bounds__(1024)
    k_fin_warps(const double *__restrict__ parts, int nparts, int nv, double *__restrict__ dst) {
  const int lane = threadIdx.x & 31, v = threadIdx.x >> 5;
  if (v >= nv) return;
  double s = 0.0;
  for (int i = lane; i < nparts; i += 32) s += parts[(size_t)i * nv + v];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if (lane == 0) dst[v] = s;
}

__global__ void __launch_bounds__(256)
    k_fin_chunks(const double *__restrict__ parts, int nparts, double *__restrict__ out) {
  __shared__ double sh[8];
  const int per = (nparts + gridDim.x - 1) / gridDim.x;
  const int i0 = blockIdx.x * per, i1 = min(nparts, i0 + per);
  double s = 0.0;
  for (int i = i0 + (int)threadIdx.x; i < i1; i += 256) s += parts[i];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double x = 0.0;
    for (int w = 0; w < 8; ++w) x += sh[w];
    out[blockIdx.x] = x;
  }
}

// ------------------------------------------------------------------------------
// finest level: double-float red-black Gauss-Seidel, residual, prolongation
// ------------------------------------------------------------------------------
// Accurate residual r = b - L_h2(hi + lo) at an interior node (h^2 units) from
// the pair at the node (hc, lc) and at its six neighbours in the order
// i+1, i-1, j+1, j-1, k+1, k-1: exact neighbour differences summed with
// error-free transforms, the lo parts' Laplacian added in f32.
__device__ __forceinline__ float df_residual_v(float hc, float lc, const float (&h)[6], const float (&l)[6],
                                               float bc) {
  const float d0 = __fsub_rn(h[0], hc);
  const float d1 = __fsub_rn(h[1], hc);
  const float d2 = __fsub_rn(h[2], hc);
  const float d3 = __fsub_rn(h[3], hc);
  const float d4 = __fsub_rn(h[4], hc);
  const float d5 = __fsub_rn(h[5], hc);
  float s, e, t;
  df_two_sum(d0, d1, s, e);
  df_two_sum(s, d2, s, t); e = __fadd_rn(e, t);
  df_two_sum(s, d3, s, t); e = __fadd_rn(e, t);
  df_two_sum(s, d4, s, t); e = __fadd_rn(e, t);
  df_two_sum(s, d5, s, t); e = __fadd_rn(e, t);
  const float ln = ((((l[0] + l[1]) + l[2]) + l[3]) + l[4]) + l[5];
  const float ll = __fsub_rn(ln, __fmul_rn(6.0f, lc));
  float r1, r1e;
  df_two_sum(bc, -s, r1, r1e);
  return __fadd_rn(r1, __fsub_rn(r1e, __fadd_rn(e, ll)));
}

__device__ __forceinline__ float df_residual(const float *__restrict__ hi, const float *__restrict__ lo,
                                             float bc, size_t c, size_t sj, size_t si, float &hc_out,
                                             float &lc_out) {
  const float h[6] = {hi[c + si], hi[c - si], hi[c + sj], hi[c - sj], hi[c + 1], hi[c - 1]};
  const float l[6] = {lo[c + si], lo[c - si], lo[c + sj], lo[c - sj], lo[c + 1], lo[c - 1]};
  hc_out = hi[c];
  lc_out = lo[c];
  return df_residual_v(hc_out, lc_out, h, l, bc);
}

// FP64 verification residual: phi = (double)hi + (double)lo, or hi alone when lo is NULL.
__global__ void __launch_bounds__(256)
    k_resid64(const float *__restrict__ hi, const float *__restrict__ lo, const float *__restrict__ b,
              double *__restrict__ parts, int G) {
  const int k = blockIdx.x * 32 + threadIdx.x + 1;
  const int j = blockIdx.y * 8 + threadIdx.y + 1;
  const int i = blockIdx.z + 1;
  double acc[1] = {0.0};
  if (k <= G - 2 && j <= G - 2) {
    const size_t sj = (size_t)G, si = (size_t)G * G;
    const size_t c = (size_t)i * si + (size_t)j * sj + k;
    auto P = [&](size_t q) { return lo ? (double)hi[q] + (double)lo[q] : (double)hi[q]; };
    const double pc = P(c);
    const double lap = (P(c + si) - pc) + (P(c - si) - pc) + (P(c + sj) - pc) + (P(c - sj) - pc) +
                       (P(c + 1) - pc) + (P(c - 1) - pc);
    const double rv = (double)b[c] - lap;
    acc[0] = rv * rv;
  }
  const size_t bid = ((size_t)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
  block_partials<1>(acc, parts + bid);
}

// ------------------------------------------------------------------------------
// coarse levels (FP32 corrections, Shortley-Weller far faces)
// ------------------------------------------------------------------------------
struct AxisTerm {
  float s;  // weighted neighbour sum along the axis
  float d;  // diagonal contribution
};

__device__ __forceinline__ AxisTerm sw_axis(const float *__restrict__ e, size_t c, size_t stride, int idx,
                                            const LevelGeom &g) {
  AxisTerm t;
  if (idx == g.J) {
    t.s = g.a * e[c - stride];
    t.d = g.dB;
  } else {
    t.s = e[c + stride] + e[c - stride];
    t.d = 2.0f;
  }
  return t;
}

__device__ __forceinline__ void sw_stencil(const float *__restrict__ e, size_t c, int i, int j, int k,
                                           const LevelGeom &g, float &sum, float &diag) {
  const size_t n = (size_t)g.n;
  const AxisTerm ax = sw_axis(e, c, n * n, i, g);
  const AxisTerm ay = sw_axis(e, c, n, j, g);
  const AxisTerm az = sw_axis(e, c, 1, k, g);
  sum = (ax.s + ay.s) + az.s;
  diag = (ax.d + ay.d) + az.d;
}

// Gauss-Seidel value (sum - b) / diag. The common diagonal 6 (every node off a
// Shortley-Weller face) multiplies by the correctly rounded 1/6 instead of
// dividing; every smoother of every level and layout uses this one rule, with
// explicitly rounded products so that no contraction can differ between them.
#define GC_SIXTH 0.16666667f
__device__ __forceinline__ float gs_value(float sum, float b, float diag) {
  return diag == 6.0f ? __fmul_rn(sum - b, GC_SIXTH) : (sum - b) / diag;
}

__global__ void __launch_bounds__(RB_TX *RB_TY)
    k_smooth(float *__restrict__ e, const float *__restrict__ b, LevelGeom g, int color) {
  const int kk = blockIdx.x * RB_TX + threadIdx.x;
  const int j = blockIdx.y * RB_TY + threadIdx.y + 1;
  const int i = blockIdx.z + 1;
  if (j > g.J) return;
  const int k = 2 * kk + ((color + i + j) & 1);
  if (k < 1 || k > g.J) return;
  const size_t n = g.n;
  const size_t c = ((size_t)i * n + j) * n + k;
  float sum, diag;
  sw_stencil(e, c, i, j, k, g, sum, diag);
  e[c] = gs_value(sum, b[c], diag);
}

__global__ void __launch_bounds__(256)
    k_resid(const float *__restrict__ e, const float *__restrict__ b, float *__restrict__ r, LevelGeom g) {
  const int k = blockIdx.x * 32 + threadIdx.x + 1;
  const int j = blockIdx.y * 8 + threadIdx.y + 1;
  const int i = blockIdx.z + 1;
  if (k > g.J || j > g.J) return;
  const size_t n = g.n;
  const size_t c = ((size_t)i * n + j) * n + k;
  float sum, diag;
  sw_stencil(e, c, i, j, k, g, sum, diag);
  r[c] = b[c] - (sum - diag * e[c]);
}

// 1-D restriction weight of fine node 2J'+o into coarse node J' (transpose of the prolongation / 2).
__device__ __forceinline__ float restrict_w(int Jc, int o, const LevelGeom &f, const LevelGeom &cg) {
  const int i = 2 * Jc + o;
  if (i < 1 || i > f.J) return 0.0f;
  if (o == 0) return 0.5f;
  if (o < 0) return 0.25f;
  if (Jc < cg.J) return 0.25f;
  return 0.5f * (f.p - (float)i) / (f.p - (float)(2 * Jc));
}

// b_c = 4 * R(r_f) at coarse node (I, Jj, K): full weighting (transpose of
// trilinear prolongation), summed separably: the three k terms of each of the
// nine (i, j) fine rows, then the rows' j weights, then the i weights. Terms of
// weight zero (fine nodes on a face) are not read.
__device__ __forceinline__ void restrict_node(const float *__restrict__ rf, const LevelGeom &f,
                                              float *__restrict__ bc, const LevelGeom &cg, int I, int Jj, int K) {
  float wi[3], wj[3], wk[3];
#pragma unroll
  for (int o = -1; o <= 1; ++o) {
    wi[o + 1] = restrict_w(I, o, f, cg);
    wj[o + 1] = restrict_w(Jj, o, f, cg);
    wk[o + 1] = restrict_w(K, o, f, cg);
  }
  const size_t n = f.n;
  const float *base = rf + ((size_t)(2 * I - 1) * n + (size_t)(2 * Jj - 1)) * n + (size_t)(2 * K - 1);
  float acc = 0.0f;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    if (wi[a] == 0.0f) continue;
    float ta = 0.0f;
#pragma unroll
    for (int bb = 0; bb < 3; ++bb) {
      if (wj[bb] == 0.0f) continue;
      const float *row = base + ((size_t)a * n + (size_t)bb) * n;
      float sab = wk[1] * row[1];
      if (wk[0] != 0.0f) sab += wk[0] * row[0];
      if (wk[2] != 0.0f) sab += wk[2] * row[2];
      ta += wj[bb] * sab;
    }
    acc += wi[a] * ta;
  }
  const size_t m = cg.n;
  bc[((size_t)I * m + Jj) * m + K] = 4.0f * acc;
}

__global__ void __launch_bounds__(256)
    k_restrict(const float *__restrict__ rf, LevelGeom f, float *__restrict__ bc, LevelGeom cg) {
  const int K = blockIdx.x * 32 + threadIdx.x + 1;
  const int Jj = blockIdx.y * 8 + threadIdx.y + 1;
  const int I = blockIdx.z + 1;
  if (K > cg.J || Jj > cg.J) return;
  restrict_node(rf, f, bc, cg, I, Jj, K);
}

// 1-D prolongation weights of fine node i from the coarse level.
__device__ __forceinline__ int prolong_w(int i, const LevelGeom &f, const LevelGeom &cg, int &c0, float &w0,
                                         float &w1) {
  c0 = i >> 1;
  if ((i & 1) == 0) {
    w0 = 1.0f;
    w1 = 0.0f;
    return 1;
  }
  if (c0 + 1 <= cg.J) {
    w0 = 0.5f;
    w1 = 0.5f;
    return 2;
  }
  w0 = (f.p - (float)i) / (f.p - (float)(2 * c0));
  w1 = 0.0f;
  return 1;
}

__device__ __forceinline__ float prolong_value(const float *__restrict__ ec, int i, int j, int k,
                                               const LevelGeom &f, const LevelGeom &cg) {
  int ci, cj, ck;
  float wi0, wi1, wj0, wj1, wk0, wk1;
  const int ni = prolong_w(i, f, cg, ci, wi0, wi1);
  const int nj = prolong_w(j, f, cg, cj, wj0, wj1);
  const int nk = prolong_w(k, f, cg, ck, wk0, wk1);
  const size_t m = cg.n;
  float val = 0.0f;
  for (int a = 0; a < ni; ++a) {
    const float wa = a ? wi1 : wi0;
    for (int bb = 0; bb < nj; ++bb) {
      const float wb = bb ? wj1 : wj0;
      const size_t row = ((size_t)(ci + a) * m + (cj + bb)) * m + ck;
      const float wab = wa * wb;
      val += wab * wk0 * ec[row];
      if (nk == 2) val += wab * wk1 * ec[row + 1];
    }
  }
  return val;
}

__global__ void __launch_bounds__(256)
    k_prolong(const float *__restrict__ ec, LevelGeom cg, float *__restrict__ ef, LevelGeom f) {
  const int k = blockIdx.x * 32 + threadIdx.x + 1;
  const int j = blockIdx.y * 8 + threadIdx.y + 1;
  const int i = blockIdx.z + 1;
  if (k > f.J || j > f.J) return;
  const size_t n = f.n;
  ef[((size_t)i * n + j) * n + k] += prolong_value(ec, i, j, k, f, cg);
}

// ------------------------------------------------------------------------------
// coarse levels in two persistent launches
// ------------------------------------------------------------------------------
// Levels 1 .. tail-1 are relaxed grid-wide by one cooperative launch on the way
// down (pre-smoothing, residual, restriction per level) and one on the way up
// (prolongation, post-smoothing), with a grid barrier between phases instead of
// a kernel boundary. The arithmetic per node is that of k_smooth / k_resid /
// k_restrict / k_prolong, so the result equals the per-phase launches bit for
// bit. The first half-sweep of a level starts from a zero correction and reads
// no neighbour, so the level needs no clearing.
struct GridBar {
  unsigned count;  // arrivals since the start of the solve (grows by the grid size per barrier)
  unsigned pad0;
  unsigned abort;  // set by a CTA that gave up waiting
  unsigned pad1;
};

struct CoarseDesc {
  int l0, l1;  // levels l0 .. l1-1
  int pre, post;
  long long budget;  // SM clocks a CTA waits at one barrier before it gives up
  GridBar *bar;
  unsigned *status;
  float *rc;
  LevelGeom g[GC_MAX_LEVELS];
  float *e[GC_MAX_LEVELS];
  float *b[GC_MAX_LEVELS];
};

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Grid-wide barrier of a cooperative launch on a monotonic arrival count: thread
// 0 of each CTA adds one arrival (a release reduction, no return value) and
// waits with acquire loads until the count reaches its target, a multiple of
// the grid size. The count is cleared before every solve and only grows within
// it; a launch starts from the count rounded down to a multiple of the grid
// size (every barrier of earlier launches has completed, and a CTA that reads
// it late can see at most the other CTAs' first arrivals). The wait is bounded
// by `budget` clocks: a CTA that gives up raises GC_FLAG_TIMEOUT and the abort
// word (so the others stop waiting too) and the kernel returns.
__device__ __forceinline__ unsigned grid_barrier_base(GridBar *gb) {
  return (ld_acquire_u32(&gb->count) / gridDim.x) * gridDim.x;
}

__device__ __forceinline__ bool grid_barrier(GridBar *gb, unsigned &target, unsigned *status, long long budget) {
  __shared__ int ok_s;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    target += gridDim.x;
    __threadfence();
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(&gb->count), "r"(1u) : "memory");
    const long long t0 = clock64();
    unsigned spins = 0;
    while ((int)(ld_acquire_u32(&gb->count) - target) < 0) {
      if ((++spins & 63u) == 0 && (ld_acquire_u32(&gb->abort) || clock64() - t0 > budget)) {
        ok = 0;
        atomicOr(status, GC_FLAG_TIMEOUT);
        atomicExch(&gb->abort, 1u);
        break;
      }
    }
    ok_s = ok;
  }
  __syncthreads();
  return ok_s != 0;
}

// A phase deals the rows (i, j), 1 <= i, j <= J, of its level to the grid's
// warps round robin, PR rows per warp per round, and the lanes of a warp take
// the nodes k of a row (SK per lane per group of 32 * SK): one division per
// row instead of per node, coalesced row accesses, and up to PR * SK nodes per
// lane whose loads are all issued before any result is stored, so that a lane
// has several independent L2 round trips in flight. Within a phase no node
// reads a value that the phase writes (a half-sweep reads only the other
// colour; the residual, restriction and prolongation write other arrays or
// only the node itself), so deferring the stores changes nothing.
#define PR 1  // (2 and 4 rows per round measured slower: more registers, fewer warps)
#define SK 2
__device__ __forceinline__ unsigned p_warp() { return (blockIdx.x * blockDim.x + threadIdx.x) >> 5; }
__device__ __forceinline__ unsigned p_nwarps() { return (gridDim.x * blockDim.x) >> 5; }

// One red-black half-sweep of level g (k_smooth's slots and arithmetic): row
// (i, j) holds the nodes k = 2 kk + ((color + i + j) & 1), kk = 0 .. J/2.
__device__ void p_smooth(float *__restrict__ e, const float *__restrict__ b, const LevelGeom &g, int color,
                         bool first) {
  const int J = g.J, n = g.n, nkk = J / 2 + 1;
  const unsigned rows = (unsigned)J * (unsigned)J, NW = p_nwarps(), lane = threadIdx.x & 31u;
  for (unsigned r0 = p_warp(); r0 < rows; r0 += PR * NW) {
    for (int kk0 = 0; kk0 < nkk; kk0 += 32 * SK) {
      float val[PR][SK];
      unsigned at[PR][SK];  // coarse levels have < 2^32 nodes
      bool ok[PR][SK];
#pragma unroll
      for (int u = 0; u < PR; ++u) {
        const unsigned r = r0 + u * NW;
        const int i = (int)(r / (unsigned)J) + 1, j = (int)(r % (unsigned)J) + 1;
        const int par = (color + i + j) & 1;
#pragma unroll
        for (int q = 0; q < SK; ++q) {
          const int k = 2 * (kk0 + (int)lane + 32 * q) + par;
          ok[u][q] = r < rows && k >= 1 && k <= J;
          if (!ok[u][q]) continue;
          const size_t c = ((size_t)i * n + j) * n + k;
          float sum, diag;
          if (first) {  // zero neighbours: the diagonal alone
            sum = 0.0f;
            diag = ((i == J ? g.dB : 2.0f) + (j == J ? g.dB : 2.0f)) + (k == J ? g.dB : 2.0f);
          } else {
            sw_stencil(e, c, i, j, k, g, sum, diag);
          }
          val[u][q] = gs_value(sum, b[c], diag);
          at[u][q] = (unsigned)c;
        }
      }
#pragma unroll
      for (int u = 0; u < PR; ++u)
#pragma unroll
        for (int q = 0; q < SK; ++q)
          if (ok[u][q]) e[at[u][q]] = val[u][q];
    }
  }
}

__device__ void p_zero(float *__restrict__ e, const LevelGeom &g) {
  const size_t tot = (size_t)g.n * g.n * g.n, T = (size_t)gridDim.x * blockDim.x;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < tot; t += T) e[t] = 0.0f;
}

// The nodes k = k0 + lane + 32 q (1 <= k <= J) of RR rows per round, for the
// residual and the prolongation: node(i, j, k, v) returns the node's index in
// `out` and sets its new value v; all of a lane's values are stored after all
// of its nodes are computed.
template <int RR, typename F>
__device__ __forceinline__ void p_node_rows(int J, float *__restrict__ out, F node) {
  const unsigned rows = (unsigned)J * (unsigned)J, NW = p_nwarps(), lane = threadIdx.x & 31u;
  for (unsigned r0 = p_warp(); r0 < rows; r0 += RR * NW) {
    for (int k0 = 1; k0 <= J; k0 += 32 * SK) {
      float val[RR][SK];
      unsigned at[RR][SK];  // coarse levels have < 2^32 nodes
      bool ok[RR][SK];
#pragma unroll
      for (int u = 0; u < RR; ++u) {
        const unsigned r = r0 + u * NW;
        const int i = (int)(r / (unsigned)J) + 1, j = (int)(r % (unsigned)J) + 1;
#pragma unroll
        for (int q = 0; q < SK; ++q) {
          const int k = k0 + (int)lane + 32 * q;
          ok[u][q] = r < rows && k <= J;
          if (ok[u][q]) at[u][q] = node(i, j, k, val[u][q]);
        }
      }
#pragma unroll
      for (int u = 0; u < RR; ++u)
#pragma unroll
        for (int q = 0; q < SK; ++q)
          if (ok[u][q]) out[at[u][q]] = val[u][q];
    }
  }
}

__device__ void p_resid(const float *__restrict__ e, const float *__restrict__ b, float *__restrict__ r_out,
                        const LevelGeom &g) {
  const size_t n = (size_t)g.n;
  p_node_rows<1>(g.J, r_out, [&](int i, int j, int k, float &v) {
    const size_t c = ((size_t)i * n + j) * n + k;
    float sum, diag;
    sw_stencil(e, c, i, j, k, g, sum, diag);
    v = b[c] - (sum - diag * e[c]);
    return (unsigned)c;
  });
}

__device__ void p_restrict(const float *__restrict__ rf, const LevelGeom &f, float *__restrict__ bc,
                           const LevelGeom &cg) {
  const int J = cg.J;
  const unsigned rows = (unsigned)J * (unsigned)J, NW = p_nwarps(), lane = threadIdx.x & 31u;
  for (unsigned r = p_warp(); r < rows; r += NW) {
    const int I = (int)(r / (unsigned)J) + 1, Jj = (int)(r % (unsigned)J) + 1;
    for (int K = 1 + (int)lane; K <= J; K += 32) restrict_node(rf, f, bc, cg, I, Jj, K);
  }
}

__device__ void p_prolong(const float *__restrict__ ec, const LevelGeom &cg, float *__restrict__ ef,
                          const LevelGeom &f) {
  const size_t n = (size_t)f.n;
  // one row per round: the prolongation's weights take the registers
  p_node_rows<1>(f.J, ef, [&](int i, int j, int k, float &v) {
    const size_t c = ((size_t)i * n + j) * n + k;
    v = ef[c] + prolong_value(ec, i, j, k, f, cg);
    return (unsigned)c;
  });
}

#define COARSE_THREADS 512

// Down: for each level, pre-smoothing, residual, restriction into b[l+1].
__global__ void __launch_bounds__(COARSE_THREADS, 2) k_coarse_down(CoarseDesc d) {
  unsigned tgt = threadIdx.x == 0 ? grid_barrier_base(d.bar) : 0u;
  for (int l = d.l0; l < d.l1; ++l) {
    const LevelGeom &g = d.g[l];
    if (d.pre == 0) {
      p_zero(d.e[l], g);
      if (!grid_barrier(d.bar, tgt, d.status, d.budget)) return;
    }
    for (int h = 0; h < 2 * d.pre; ++h) {
      p_smooth(d.e[l], d.b[l], g, h & 1, h == 0);
      if (!grid_barrier(d.bar, tgt, d.status, d.budget)) return;
    }
    p_resid(d.e[l], d.b[l], d.rc, g);
    if (!grid_barrier(d.bar, tgt, d.status, d.budget)) return;
    p_restrict(d.rc, g, d.b[l + 1], d.g[l + 1]);
    if (l + 1 < d.l1 && !grid_barrier(d.bar, tgt, d.status, d.budget)) return;
  }
}

// Up: for each level from l1-1 down to l0, prolongation of e[l+1], post-smoothing.
__global__ void __launch_bounds__(COARSE_THREADS, 2) k_coarse_up(CoarseDesc d) {
  unsigned tgt = threadIdx.x == 0 ? grid_barrier_base(d.bar) : 0u;
  for (int l = d.l1 - 1; l >= d.l0; --l) {
    const LevelGeom &g = d.g[l];
    p_prolong(d.e[l + 1], d.g[l + 1], d.e[l], g);
    for (int h = 0; h < 2 * d.post; ++h) {
      if (!grid_barrier(d.bar, tgt, d.status, d.budget)) return;
      p_smooth(d.e[l], d.b[l], g, h & 1, false);
    }
    if (l > d.l0 && !grid_barrier(d.bar, tgt, d.status, d.budget)) return;
  }
}

// ------------------------------------------------------------------------------
// finest level: defect correction with FP32 corrections in colour-split storage
// ------------------------------------------------------------------------------
// Each V-cycle solves L e = r for a correction e of the current potential
// (phi = hi + lo, double-float) with FP32 red-black Gauss-Seidel, then adds it:
// phi += e, and forms the new residual r = b - L phi accurately from the pair.
// The correction and the residual are stored colour-split: node (i,j,k) of
// colour c = (i+j+k)&1 lives in half c at s = (i*G + j)*H + (k>>1), H = (G+1)/2
// (the same-colour nodes of a row are every other k, so k>>1 is unique). A
// half-sweep of colour c then reads only the other colour's half and its own
// right-hand side and writes its own half: a Gauss-Seidel update does not use
// the node's old value. Neighbours of node s of colour c in the other half:
// i +- 1 at s +- G*H, j +- 1 at s +- H, k +- 1 at s + p and s + p - 1 with
// p = k & 1. Face nodes are never written and stay zero (homogeneous
// correction). The arithmetic is that of k_smooth / k_resid / k_prolong on the
// level-0 geometry in natural layout (GC_MG_NATURAL_LAYOUT runs those), term for
// term, so both layouts give identical potentials.
struct Split0 {
  int G, H;
  size_t half;  // nodes per colour half: G * G * H
};

__device__ __forceinline__ float split_nbr_sum(const float *__restrict__ o, size_t s, size_t GH, int H, int p) {
  const float ax = o[s + GH] + o[s - GH];
  const float ay = o[s + H] + o[s - H];
  const float az = o[s + p] + o[s + p - 1];
  return (ax + ay) + az;
}

// One half-sweep of colour `color` on the interior; FIRST: the correction
// starts at zero, so e = (0 - r)/6 and nothing is read but r.
template <bool FIRST>
__global__ void __launch_bounds__(256)
    k_rb0(float *__restrict__ e, const float *__restrict__ r, Split0 d, int color) {
  const int kk = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int i = blockIdx.z + 1;
  if (kk >= d.H || j > d.G - 2) return;
  const int p = (color + i + j) & 1;
  const int k = 2 * kk + p;
  if (k < 1 || k > d.G - 2) return;
  const size_t s = ((size_t)i * d.G + j) * d.H + kk;
  float *own = e + (size_t)color * d.half;
  const float *oth = e + (size_t)(color ^ 1) * d.half;
  const float rv = r[(size_t)color * d.half + s];
  const float sum = FIRST ? 0.0f : split_nbr_sum(oth, s, (size_t)d.G * d.H, d.H, p);
  own[s] = __fmul_rn(sum - rv, GC_SIXTH);
}

// phi += e at natural node c: double-float add (or a plain f32 add).
template <bool PLAIN>
__device__ __forceinline__ void phi_add(float *__restrict__ hi, float *__restrict__ lo, size_t c, float ev) {
  if (PLAIN) {
    hi[c] = __fadd_rn(hi[c], ev);
  } else {
    float s1, e1, h, l;
    df_two_sum(hi[c], ev, s1, e1);
    const float ln = __fadd_rn(lo[c], e1);
    df_fast_two_sum(s1, ln, h, l);
    hi[c] = h;
    lo[c] = l;
  }
}

// The last half-sweep (black) fused with the update phi += e: thread kk of row
// (i,j) relaxes the black node 2kk + pb and adds the final corrections of that
// node and of the red node 2kk + (1 - pb) into the potential. The correction is
// dead afterwards, so the black value is not stored.
template <bool PLAIN>
__global__ void __launch_bounds__(256)
    k_rb0_last(const float *__restrict__ e, const float *__restrict__ r, float *__restrict__ hi,
               float *__restrict__ lo, Split0 d) {
  const int kk = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int i = blockIdx.z + 1;
  if (kk >= d.H || j > d.G - 2) return;
  const int pb = (1 + i + j) & 1;
  const int kb = 2 * kk + pb, kr = 2 * kk + (pb ^ 1);
  const size_t s = ((size_t)i * d.G + j) * d.H + kk;
  const size_t row = ((size_t)i * d.G + j) * d.G;
  if (kb >= 1 && kb <= d.G - 2) {
    const float sum = split_nbr_sum(e, s, (size_t)d.G * d.H, d.H, pb);
    const float eb = __fmul_rn(sum - r[d.half + s], GC_SIXTH);
    phi_add<PLAIN>(hi, lo, row + kb, eb);
  }
  if (kr >= 1 && kr <= d.G - 2) phi_add<PLAIN>(hi, lo, row + kr, e[s]);
}

// phi += e at every interior node (natural-layout correction), the update of
// the natural-layout path and of cycles without post-smoothing.
template <bool PLAIN, bool SPLIT>
__global__ void __launch_bounds__(256)
    k_update0(const float *__restrict__ e, float *__restrict__ hi, float *__restrict__ lo, Split0 d) {
  const int k = blockIdx.x * 32 + threadIdx.x + 1;
  const int j = blockIdx.y * 8 + threadIdx.y + 1;
  const int i = blockIdx.z + 1;
  if (k > d.G - 2 || j > d.G - 2) return;
  const size_t c = ((size_t)i * d.G + j) * d.G + k;
  const float ev = SPLIT ? e[(size_t)((i + j + k) & 1) * d.half + ((size_t)i * d.G + j) * d.H + (k >> 1)] : e[c];
  phi_add<PLAIN>(hi, lo, c, ev);
}

// Plain FP32 residual b - L(hi) (the reference's left-to-right neighbour sum).
__device__ __forceinline__ float f32_residual(const float *__restrict__ hi, float bc, size_t c, size_t sj, size_t si) {
  const float s6 = ((((hi[c + si] + hi[c - si]) + hi[c + sj]) + hi[c - sj]) + hi[c + 1]) + hi[c - 1];
  return bc - (s6 - 6.0f * hi[c]);
}

// Residual r = b - L phi of the potential (double-float, or f32 when PLAIN) at
// every interior node, stored colour-split (SPLIT) or natural; block partials of
// sum r^2. With e_first (split only), the first half-sweep of the next cycle's
// pre-smoothing (red, from a zero correction) is written as well.
template <bool PLAIN, bool SPLIT>
__global__ void __launch_bounds__(256)
    k_resid0(const float *__restrict__ hi, const float *__restrict__ lo, const float *__restrict__ b,
             float *__restrict__ rout, float *__restrict__ e_first, double *__restrict__ parts, Split0 d) {
  const int G = d.G;
  const int k = blockIdx.x * 32 + threadIdx.x + 1;
  const int j = blockIdx.y * 8 + threadIdx.y + 1;
  const int i = blockIdx.z + 1;
  float acc = 0.0f;
  if (k <= G - 2 && j <= G - 2) {
    const size_t sj = (size_t)G, si = (size_t)G * G;
    const size_t c = (size_t)i * si + (size_t)j * sj + k;
    float rv;
    if (PLAIN) {
      rv = f32_residual(hi, b[c], c, sj, si);
    } else {
      float hc, lc;
      rv = df_residual(hi, lo, b[c], c, sj, si, hc, lc);
    }
    if (SPLIT) {
      const int col = (i + j + k) & 1;
      const size_t s = ((size_t)i * G + j) * d.H + (k >> 1);
      rout[(size_t)col * d.half + s] = rv;
      if (e_first && col == 0) e_first[s] = __fmul_rn(0.0f - rv, GC_SIXTH);
    } else {
      rout[c] = rv;
    }
    acc = rv * rv;
  }
  const size_t bid = ((size_t)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
  block_sum_f32(acc, parts + bid);
}

// Residual of the correction equation, r - L e (e, r colour-split), written in
// natural layout for the restriction: the arithmetic of k_resid on level 0.
__global__ void __launch_bounds__(256)
    k_resid0e(const float *__restrict__ e, const float *__restrict__ r, float *__restrict__ rc, Split0 d) {
  const int G = d.G;
  const int k = blockIdx.x * 32 + threadIdx.x + 1;
  const int j = blockIdx.y * 8 + threadIdx.y + 1;
  const int i = blockIdx.z + 1;
  if (k > G - 2 || j > G - 2) return;
  const int col = (i + j + k) & 1;
  const size_t s = ((size_t)i * G + j) * d.H + (k >> 1);
  const float *own = e + (size_t)col * d.half;
  const float *oth = e + (size_t)(col ^ 1) * d.half;
  const float sum = split_nbr_sum(oth, s, (size_t)G * d.H, d.H, k & 1);
  const float diag = 6.0f;
  rc[((size_t)i * G + j) * G + k] = r[(size_t)col * d.half + s] - (sum - diag * own[s]);
}

// Add the level-1 correction into the colour-split level-0 correction: black
// nodes only when a red half-sweep follows (it overwrites the red half without
// reading it), both colours otherwise.
__global__ void __launch_bounds__(256)
    k_prolong0s(const float *__restrict__ ec, LevelGeom cg, float *__restrict__ e, LevelGeom f, Split0 d,
                int both) {
  const int kk = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int i = blockIdx.z + 1;
  if (kk >= d.H || j > d.G - 2) return;
  const size_t s = ((size_t)i * d.G + j) * d.H + kk;
  for (int col = both ? 0 : 1; col < 2; ++col) {
    const int k = 2 * kk + ((col + i + j) & 1);
    if (k < 1 || k > d.G - 2) continue;
    e[(size_t)col * d.half + s] += prolong_value(ec, i, j, k, f, cg);
  }
}

// ---- the same finest-level kernels, vectorised (G % 4 == 0) --------------------
// With G a multiple of 4 the split row length H = G/2 is even, so slot pairs
// (2t, 2t+1) start on 8-byte boundaries, and natural rows of G nodes split into
// 16-byte quads. Each thread then handles two slots of one colour (half-sweeps,
// prolongation) or four consecutive nodes (residuals, update) with vector
// loads; the arithmetic of every node is that of the scalar kernels above.
__device__ __forceinline__ float2 ld2(const float *p) { return *reinterpret_cast<const float2 *>(p); }
__device__ __forceinline__ float4 ld4(const float *p) { return *reinterpret_cast<const float4 *>(p); }
__device__ __forceinline__ void st2(float *p, float a, float b) { *reinterpret_cast<float2 *>(p) = make_float2(a, b); }
__device__ __forceinline__ void st4(float *p, float4 v) { *reinterpret_cast<float4 *>(p) = v; }
__device__ __forceinline__ float f4get(const float4 &v, int q) { return q == 0 ? v.x : q == 1 ? v.y : q == 2 ? v.z : v.w; }
__device__ __forceinline__ void f4set(float4 &v, int q, float x) {
  if (q == 0) v.x = x; else if (q == 1) v.y = x; else if (q == 2) v.z = x; else v.w = x;
}

// Half-sweep of colour `color`, slots 2t and 2t+1 of a row. Face slots (k = 0 or
// G-1) are written back as zero, their value in the homogeneous correction.
template <bool FIRST>
__global__ void __launch_bounds__(256)
    k_rb0x2(float *__restrict__ e, const float *__restrict__ r, Split0 d, int color) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int i = blockIdx.z + 1;
  const int kk0 = 2 * t;
  if (kk0 >= d.H || j > d.G - 2) return;
  const int p = (color + i + j) & 1;
  const int k0 = 2 * kk0 + p;  // the pair's nodes are k0 and k0 + 2
  const size_t s = ((size_t)i * d.G + j) * d.H + kk0;
  const float2 rv = ld2(r + (size_t)color * d.half + s);
  float v0, v1;
  if (FIRST) {
    v0 = __fmul_rn(0.0f - rv.x, GC_SIXTH);
    v1 = __fmul_rn(0.0f - rv.y, GC_SIXTH);
  } else {
    const float *o = e + (size_t)(color ^ 1) * d.half;
    const size_t GH = (size_t)d.G * d.H;
    const float2 xp = ld2(o + s + GH), xm = ld2(o + s - GH), yp = ld2(o + s + d.H), ym = ld2(o + s - d.H);
    const float2 zc = ld2(o + s);
    const float zo = p ? o[s + 2] : o[s - 1];
    const float az0 = p ? zc.y + zc.x : zc.x + zo;  // (k+1) + (k-1) of node k0
    const float az1 = p ? zo + zc.y : zc.y + zc.x;  // ... of node k0 + 2
    const float sum0 = ((xp.x + xm.x) + (yp.x + ym.x)) + az0;
    const float sum1 = ((xp.y + xm.y) + (yp.y + ym.y)) + az1;
    v0 = __fmul_rn(sum0 - rv.x, GC_SIXTH);
    v1 = __fmul_rn(sum1 - rv.y, GC_SIXTH);
  }
  if (k0 < 1) v0 = 0.0f;
  if (k0 + 2 > d.G - 2) v1 = 0.0f;
  st2(e + (size_t)color * d.half + s, v0, v1);
}

// Last (black) half-sweep fused with phi += e on four consecutive nodes
// 4t .. 4t+3 of a row: the black slots 2t, 2t+1 and the red ones beside them.
template <bool PLAIN>
__global__ void __launch_bounds__(256)
    k_rb0_lastx4(const float *__restrict__ e, const float *__restrict__ r, float *__restrict__ hi,
                 float *__restrict__ lo, Split0 d) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int i = blockIdx.z + 1;
  const int kk0 = 2 * t;
  if (kk0 >= d.H || j > d.G - 2) return;
  const int pb = (1 + i + j) & 1;  // k parity of the black nodes of the row
  const size_t s = ((size_t)i * d.G + j) * d.H + kk0;
  const size_t GH = (size_t)d.G * d.H;
  const float *o = e;  // red half: the neighbours of the black nodes, and the red corrections
  const float2 xp = ld2(o + s + GH), xm = ld2(o + s - GH), yp = ld2(o + s + d.H), ym = ld2(o + s - d.H);
  const float2 zc = ld2(o + s);
  const float zo = pb ? o[s + 2] : o[s - 1];
  const float az0 = pb ? zc.y + zc.x : zc.x + zo;
  const float az1 = pb ? zo + zc.y : zc.y + zc.x;
  const float2 rb = ld2(r + d.half + s);
  const float eb0 = __fmul_rn((((xp.x + xm.x) + (yp.x + ym.x)) + az0) - rb.x, GC_SIXTH);
  const float eb1 = __fmul_rn((((xp.y + xm.y) + (yp.y + ym.y)) + az1) - rb.y, GC_SIXTH);
  const size_t c0 = ((size_t)i * d.G + j) * d.G + 2 * kk0;
  float4 h = ld4(hi + c0);
  float4 l = PLAIN ? make_float4(0.f, 0.f, 0.f, 0.f) : ld4(lo + c0);
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int k = 2 * kk0 + q;
    if (k < 1 || k > d.G - 2) continue;
    const bool black = (q & 1) == pb;
    const float ev = black ? (q < 2 ? eb0 : eb1) : (q < 2 ? zc.x : zc.y);
    if (PLAIN) {
      f4set(h, q, __fadd_rn(f4get(h, q), ev));
    } else {
      float s1, e1, hh, llo;
      df_two_sum(f4get(h, q), ev, s1, e1);
      const float ln = __fadd_rn(f4get(l, q), e1);
      df_fast_two_sum(s1, ln, hh, llo);
      f4set(h, q, hh);
      f4set(l, q, llo);
    }
  }
  st4(hi + c0, h);
  if (!PLAIN) st4(lo + c0, l);
}

// Residual of the potential on four consecutive nodes 4t .. 4t+3 (see k_resid0).
template <bool PLAIN>
__global__ void __launch_bounds__(256)
    k_resid0x4(const float *__restrict__ hi, const float *__restrict__ lo, const float *__restrict__ b,
               float *__restrict__ rout, float *__restrict__ e_first, double *__restrict__ parts, Split0 d) {
  const int G = d.G;
  const int t = blockIdx.x * 32 + threadIdx.x;
  const int j = blockIdx.y * 8 + threadIdx.y + 1;
  const int i = blockIdx.z + 1;
  float acc = 0.0f;
  if (4 * t < G && j <= G - 2) {
    const size_t sj = (size_t)G, si = (size_t)G * G;
    const size_t c0 = (size_t)i * si + (size_t)j * sj + 4 * t;
    const float4 hc = ld4(hi + c0), hxp = ld4(hi + c0 + si), hxm = ld4(hi + c0 - si), hyp = ld4(hi + c0 + sj),
                 hym = ld4(hi + c0 - sj);
    const float hzm = hi[c0 - 1], hzp = hi[c0 + 4];
    float4 lc = make_float4(0.f, 0.f, 0.f, 0.f), lxp = lc, lxm = lc, lyp = lc, lym = lc;
    float lzm = 0.f, lzp = 0.f;
    if (!PLAIN) {
      lc = ld4(lo + c0); lxp = ld4(lo + c0 + si); lxm = ld4(lo + c0 - si); lyp = ld4(lo + c0 + sj);
      lym = ld4(lo + c0 - sj);
      lzm = lo[c0 - 1]; lzp = lo[c0 + 4];
    }
    const float4 bv = ld4(b + c0);
    float rv[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const float hk = f4get(hc, q);
      const float hkp = q < 3 ? f4get(hc, q + 1) : hzp, hkm = q > 0 ? f4get(hc, q - 1) : hzm;
      if (PLAIN) {
        const float s6 = ((((f4get(hxp, q) + f4get(hxm, q)) + f4get(hyp, q)) + f4get(hym, q)) + hkp) + hkm;
        rv[q] = f4get(bv, q) - (s6 - 6.0f * hk);
      } else {
        const float lkp = q < 3 ? f4get(lc, q + 1) : lzp, lkm = q > 0 ? f4get(lc, q - 1) : lzm;
        const float h6[6] = {f4get(hxp, q), f4get(hxm, q), f4get(hyp, q), f4get(hym, q), hkp, hkm};
        const float l6[6] = {f4get(lxp, q), f4get(lxm, q), f4get(lyp, q), f4get(lym, q), lkp, lkm};
        rv[q] = df_residual_v(hk, f4get(lc, q), h6, l6, f4get(bv, q));
      }
      const int k = 4 * t + q;
      if (k < 1 || k > G - 2) rv[q] = 0.0f;  // faces: no residual, zero correction
    }
    // nodes 4t, 4t+2 share a colour (slots 2t, 2t+1), as do 4t+1, 4t+3
    const int c0col = (i + j) & 1;  // colour of node 4t
    const size_t sl = ((size_t)i * G + j) * d.H + 2 * t;
    st2(rout + (size_t)c0col * d.half + sl, rv[0], rv[2]);
    st2(rout + (size_t)(c0col ^ 1) * d.half + sl, rv[1], rv[3]);
    if (e_first) {  // red = colour 0
      if (c0col == 0) st2(e_first + sl, __fmul_rn(0.0f - rv[0], GC_SIXTH), __fmul_rn(0.0f - rv[2], GC_SIXTH));
      else st2(e_first + sl, __fmul_rn(0.0f - rv[1], GC_SIXTH), __fmul_rn(0.0f - rv[3], GC_SIXTH));
    }
    acc = ((rv[0] * rv[0] + rv[1] * rv[1]) + rv[2] * rv[2]) + rv[3] * rv[3];
  }
  const size_t bid = ((size_t)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
  block_sum_f32(acc, parts + bid);
}

// Residual of the correction equation on four consecutive nodes, natural output.
__global__ void __launch_bounds__(256)
    k_resid0ex4(const float *__restrict__ e, const float *__restrict__ r, float *__restrict__ rc, Split0 d) {
  const int G = d.G;
  const int t = blockIdx.x * 32 + threadIdx.x;
  const int j = blockIdx.y * 8 + threadIdx.y + 1;
  const int i = blockIdx.z + 1;
  if (4 * t >= G || j > G - 2) return;
  const int ca = (i + j) & 1;  // colour of nodes 4t, 4t+2 (half A); 4t+1, 4t+3 are half B
  const size_t s0 = ((size_t)i * G + j) * d.H + 2 * t;
  const size_t GH = (size_t)G * d.H;
  const float *A = e + (size_t)ca * d.half, *B = e + (size_t)(ca ^ 1) * d.half;
  const float2 a0 = ld2(A + s0), axp = ld2(A + s0 + GH), axm = ld2(A + s0 - GH), ayp = ld2(A + s0 + d.H),
               aym = ld2(A + s0 - d.H);
  const float a2 = A[s0 + 2];
  const float2 b0 = ld2(B + s0), bxp = ld2(B + s0 + GH), bxm = ld2(B + s0 - GH), byp = ld2(B + s0 + d.H),
               bym = ld2(B + s0 - d.H);
  const float bm = B[s0 - 1];
  const float2 ra = ld2(r + (size_t)ca * d.half + s0), rb = ld2(r + (size_t)(ca ^ 1) * d.half + s0);
  // node q: own value, other-colour sums (i, j, k) in split_nbr_sum's order
  const float sum0 = ((bxp.x + bxm.x) + (byp.x + bym.x)) + (b0.x + bm);
  const float sum1 = ((axp.x + axm.x) + (ayp.x + aym.x)) + (a0.y + a0.x);
  const float sum2 = ((bxp.y + bxm.y) + (byp.y + bym.y)) + (b0.y + b0.x);
  const float sum3 = ((axp.y + axm.y) + (ayp.y + aym.y)) + (a2 + a0.y);
  const float diag = 6.0f;
  float4 out;
  out.x = ra.x - (sum0 - diag * a0.x);
  out.y = rb.x - (sum1 - diag * b0.x);
  out.z = ra.y - (sum2 - diag * a0.y);
  out.w = rb.y - (sum3 - diag * b0.y);
  if (4 * t == 0) out.x = 0.0f;           // face k = 0
  if (4 * t + 3 == G - 1) out.w = 0.0f;  // face k = G-1
  st4(rc + ((size_t)i * G + j) * G + 4 * t, out);
}

// Level-1 correction into the black half, slots 2t and 2t+1 of a row (the two
// nodes share their i and j weights).
__global__ void __launch_bounds__(256)
    k_prolong0bx2(const float *__restrict__ ec, LevelGeom cg, float *__restrict__ e, LevelGeom f, Split0 d) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int i = blockIdx.z + 1;
  const int kk0 = 2 * t;
  if (kk0 >= d.H || j > d.G - 2) return;
  const int pb = (1 + i + j) & 1;
  const int k0 = 2 * kk0 + pb, k1 = k0 + 2;
  int ci, cj, ck0, ck1;
  float wi0, wi1, wj0, wj1, a0, a1, b0, b1;
  const int ni = prolong_w(i, f, cg, ci, wi0, wi1);
  const int nj = prolong_w(j, f, cg, cj, wj0, wj1);
  const int nk0 = prolong_w(k0, f, cg, ck0, a0, a1);
  const int nk1 = prolong_w(k1, f, cg, ck1, b0, b1);
  const size_t m = cg.n;
  float v0 = 0.0f, v1 = 0.0f;
  for (int a = 0; a < ni; ++a) {
    const float wa = a ? wi1 : wi0;
    for (int bb = 0; bb < nj; ++bb) {
      const float wb = bb ? wj1 : wj0;
      const size_t row = ((size_t)(ci + a) * m + (cj + bb)) * m;
      const float wab = wa * wb;
      v0 += wab * a0 * ec[row + ck0];
      if (nk0 == 2) v0 += wab * a1 * ec[row + ck0 + 1];
      v1 += wab * b0 * ec[row + ck1];
      if (nk1 == 2) v1 += wab * b1 * ec[row + ck1 + 1];
    }
  }
  if (k0 < 1) v0 = 0.0f;
  if (k1 > d.G - 2) v1 = 0.0f;
  float *blk = e + d.half + ((size_t)i * d.G + j) * d.H + kk0;
  const float2 old = ld2(blk);
  st2(blk, old.x + v0, old.y + v1);
}

// ------------------------------------------------------------------------------
// tail: all levels with n <= GC_TAIL_MAX_N relaxed by one CTA in shared memory
// ------------------------------------------------------------------------------
struct TailDesc {
  int nl;                       // number of tail levels
  int pre, post, coarse;
  LevelGeom g[GC_MAX_LEVELS];   // g[0] = first tail level
  LevelGeom gf;                 // level above the tail (for nothing but completeness)
};

template <typename T>
__device__ void t_zero(T *a, int n3) {
  for (int i = threadIdx.x; i < n3; i += blockDim.x) a[i] = (T)0;
}

// Tail levels have J <= 15 (n <= GC_TAIL_MAX_N = 17), and the tail runs with
// 1024 threads, so node indices come from the thread index by shifts: for a
// half-sweep thread (kk, j, i0) = (t & 7, (t >> 3) & 15, t >> 7) takes the
// colour slots k = 2 kk + parity of row (i, j) for i = i0 + 1, i0 + 9; for the
// other phases (k, j, i0) = (t & 15, (t >> 4) & 15, t >> 8) takes i = i0 + 1,
// i0 + 5, ...
template <typename T>
__device__ void t_smooth(T *e, const T *b, const LevelGeom &g, int sweeps) {
  const int n = g.n, J = g.J;
  const int kk = threadIdx.x & 7, j = ((threadIdx.x >> 3) & 15) + 1, i0 = (threadIdx.x >> 7) + 1;
  for (int s = 0; s < sweeps; ++s) {
    for (int color = 0; color < 2; ++color) {
      if (j <= J) {
        for (int i = i0; i <= J; i += 8) {
          const int k = 2 * kk + ((color + i + j) & 1);
          if (k < 1 || k > J) continue;
          const int c = (i * n + j) * n + k;
          T sx, sy, sz, dx_, dy_, dz_;
          if (i == J) { sx = (T)g.a * e[c - n * n]; dx_ = (T)g.dB; } else { sx = e[c + n * n] + e[c - n * n]; dx_ = 2; }
          if (j == J) { sy = (T)g.a * e[c - n]; dy_ = (T)g.dB; } else { sy = e[c + n] + e[c - n]; dy_ = 2; }
          if (k == J) { sz = (T)g.a * e[c - 1]; dz_ = (T)g.dB; } else { sz = e[c + 1] + e[c - 1]; dz_ = 2; }
          if constexpr (sizeof(T) == sizeof(float))
            e[c] = gs_value((sx + sy) + sz, b[c], (dx_ + dy_) + dz_);  // the shared rule: 1/6 off the far faces
          else
            e[c] = ((sx + sy + sz) - b[c]) / (dx_ + dy_ + dz_);
        }
      }
      __syncthreads();
    }
  }
}

__device__ void t_resid(const float *e, const float *b, float *r, const LevelGeom &g) {
  const int n = g.n, J = g.J;
  const int k = (threadIdx.x & 15) + 1, j = ((threadIdx.x >> 4) & 15) + 1;
  if (k <= J && j <= J) {
    for (int i = (threadIdx.x >> 8) + 1; i <= J; i += 4) {
      const int c = (i * n + j) * n + k;
      float sum, diag;
      sw_stencil(e, (size_t)c, i, j, k, g, sum, diag);
      r[c] = b[c] - (sum - diag * e[c]);
    }
  }
  __syncthreads();
}

// 1-D transfer weights of a tail level pair (fine f, coarse cg), computed once
// per launch into shared memory so that the restriction and prolongation loops
// are table lookups (the far-face weights take a division): restriction weight
// rw[3 I + a + 1] = restrict_w(I, a, f, cg); prolongation of fine index i:
// coarse index pc[2 i], node count pc[2 i + 1], weights pw[2 i], pw[2 i + 1].
#define TAIL_TAB 16  // indices 0 .. GC_TAIL_MAX_N - 2
static_assert(GC_TAIL_MAX_N - 1 <= TAIL_TAB, "tail transfer tables too small");
struct TailTab {
  float rw[TAIL_TAB * 3];
  float pw[TAIL_TAB * 2];
  int pc[TAIL_TAB * 2];
};

__device__ void t_tables(TailTab &t, const LevelGeom &f, const LevelGeom &cg) {
  for (int q = threadIdx.x; q < TAIL_TAB * 3; q += blockDim.x) {
    const int I = q / 3, a = q % 3 - 1;
    t.rw[q] = I >= 1 && I <= cg.J ? restrict_w(I, a, f, cg) : 0.0f;
  }
  for (int i = threadIdx.x; i < TAIL_TAB; i += blockDim.x) {
    int c0 = 0, cnt = 0;
    float w0 = 0.0f, w1 = 0.0f;
    if (i >= 1 && i <= f.J) cnt = prolong_w(i, f, cg, c0, w0, w1);
    t.pc[2 * i] = c0;
    t.pc[2 * i + 1] = cnt;
    t.pw[2 * i] = w0;
    t.pw[2 * i + 1] = w1;
  }
}

template <typename T>
__device__ void t_restrict(const float *rf, const LevelGeom &f, T *bc, const LevelGeom &cg, const TailTab &tb) {
  const int J = cg.J, m = cg.n, n = f.n;
  const int K = (threadIdx.x & 15) + 1, Jj = ((threadIdx.x >> 4) & 15) + 1;
  if (K <= J && Jj <= J) {
    for (int I = (threadIdx.x >> 8) + 1; I <= J; I += 4) {
      float acc = 0.0f;
      for (int a = -1; a <= 1; ++a) {
        const float wa = tb.rw[3 * I + a + 1];
        if (wa == 0.0f) continue;
        for (int bb = -1; bb <= 1; ++bb) {
          const float wb = tb.rw[3 * Jj + bb + 1];
          if (wb == 0.0f) continue;
          for (int c = -1; c <= 1; ++c) {
            const float wc = tb.rw[3 * K + c + 1];
            if (wc == 0.0f) continue;
            acc += wa * wb * wc * rf[((2 * I + a) * n + (2 * Jj + bb)) * n + (2 * K + c)];
          }
        }
      }
      bc[(I * m + Jj) * m + K] = (T)(4.0f * acc);
    }
  }
  __syncthreads();
}

template <typename T>
__device__ void t_prolong(const T *ec, const LevelGeom &cg, float *ef, const LevelGeom &f, const TailTab &tb) {
  const int J = f.J, n = f.n, m = cg.n;
  const int k = (threadIdx.x & 15) + 1, j = ((threadIdx.x >> 4) & 15) + 1;
  if (k <= J && j <= J) {
    const int cj = tb.pc[2 * j], nj = tb.pc[2 * j + 1], ck = tb.pc[2 * k], nk = tb.pc[2 * k + 1];
    const float wj0 = tb.pw[2 * j], wj1 = tb.pw[2 * j + 1], wk0 = tb.pw[2 * k], wk1 = tb.pw[2 * k + 1];
    for (int i = (threadIdx.x >> 8) + 1; i <= J; i += 4) {
      const int ci = tb.pc[2 * i], ni = tb.pc[2 * i + 1];
      const float wi0 = tb.pw[2 * i], wi1 = tb.pw[2 * i + 1];
      float val = 0.0f;
      for (int a = 0; a < ni; ++a)
        for (int bb = 0; bb < nj; ++bb)
          for (int c = 0; c < nk; ++c) {
            const float w = (a ? wi1 : wi0) * (bb ? wj1 : wj0) * (c ? wk1 : wk0);
            val += w * (float)ec[((ci + a) * m + (cj + bb)) * m + (ck + c)];
          }
      ef[(i * n + j) * n + k] += val;
    }
  }
  __syncthreads();
}

__global__ void __launch_bounds__(1024) k_tail(const float *__restrict__ b_in, float *__restrict__ e_out, TailDesc d) {
  extern __shared__ __align__(16) unsigned char tsm[];
  float *E[GC_MAX_LEVELS], *B[GC_MAX_LEVELS], *R[GC_MAX_LEVELS];
  double *E64 = nullptr, *B64 = nullptr;
  size_t off = 0;
  for (int l = 0; l < d.nl; ++l) {
    const int n3 = d.g[l].n * d.g[l].n * d.g[l].n;
    if (l == d.nl - 1) {
      E64 = (double *)(tsm + off);
      B64 = E64 + n3;
      off += 2 * (size_t)n3 * sizeof(double);
    } else {
      E[l] = (float *)(tsm + off);
      B[l] = E[l] + n3;
      R[l] = B[l] + n3;
      off += 3 * (size_t)n3 * sizeof(float);
    }
    off = (off + 15) & ~(size_t)15;
  }
  // transfer weights of every level pair (the first CTA barrier below orders them)
  __shared__ TailTab tabs[GC_MAX_LEVELS];
  for (int l = 0; l + 1 < d.nl; ++l) t_tables(tabs[l], d.g[l], d.g[l + 1]);
  const int n0 = d.g[0].n * d.g[0].n * d.g[0].n;
  if (d.nl == 1) {
    for (int i = threadIdx.x; i < n0; i += blockDim.x) {
      B64[i] = (double)b_in[i];
      E64[i] = 0.0;
    }
    __syncthreads();
    t_smooth<double>(E64, B64, d.g[0], d.coarse);
    for (int i = threadIdx.x; i < n0; i += blockDim.x) e_out[i] = (float)E64[i];
    return;
  }
  for (int i = threadIdx.x; i < n0; i += blockDim.x) {
    B[0][i] = b_in[i];
    E[0][i] = 0.0f;
    R[0][i] = 0.0f;
  }
  for (int l = 1; l < d.nl - 1; ++l) {
    const int n3 = d.g[l].n * d.g[l].n * d.g[l].n;
    t_zero<float>(R[l], n3);
    t_zero<float>(B[l], n3);
  }
  {
    const int n3 = d.g[d.nl - 1].n * d.g[d.nl - 1].n * d.g[d.nl - 1].n;
    t_zero<double>(B64, n3);
  }
  __syncthreads();
  for (int l = 0; l < d.nl - 1; ++l) {
    if (l > 0) {
      t_zero<float>(E[l], d.g[l].n * d.g[l].n * d.g[l].n);
      __syncthreads();
    }
    t_smooth<float>(E[l], B[l], d.g[l], d.pre);
    t_resid(E[l], B[l], R[l], d.g[l]);
    if (l + 1 == d.nl - 1)
      t_restrict<double>(R[l], d.g[l], B64, d.g[l + 1], tabs[l]);
    else
      t_restrict<float>(R[l], d.g[l], B[l + 1], d.g[l + 1], tabs[l]);
  }
  {
    const LevelGeom &gc = d.g[d.nl - 1];
    t_zero<double>(E64, gc.n * gc.n * gc.n);
    __syncthreads();
    t_smooth<double>(E64, B64, gc, d.coarse);
  }
  for (int l = d.nl - 2; l >= 0; --l) {
    if (l + 1 == d.nl - 1)
      t_prolong<double>(E64, d.g[l + 1], E[l], d.g[l], tabs[l]);
    else
      t_prolong<float>(E[l + 1], d.g[l + 1], E[l], d.g[l], tabs[l]);
    t_smooth<float>(E[l], B[l], d.g[l], d.post);
  }
  for (int i = threadIdx.x; i < n0; i += blockDim.x) e_out[i] = E[0][i];
}

// ------------------------------------------------------------------------------
// boundary faces, moments, scaling
// ------------------------------------------------------------------------------
// Multipole Dirichlet faces (multigrid.py:261-295) evaluated in FP64 from the raw
// moments (multigrid.py:378-389), written as double-float pairs.
__global__ void __launch_bounds__(256)
    k_faces(float *__restrict__ hi, float *__restrict__ lo, int G,
            double dx, double grav, const double *__restrict__ mom) {
  // centre of mass and second moments about it, once per block (FP64 runs at a
  // small fraction of the f32 rate: each face node keeps only its own terms)
  __shared__ double sm[11];
  if (threadIdx.x == 0) {
    const double M = mom[0];
    const double cx = M > 0.0 ? mom[1] / M : 0.0, cy = M > 0.0 ? mom[2] / M : 0.0, cz = M > 0.0 ? mom[3] / M : 0.0;
    sm[0] = M; sm[1] = cx; sm[2] = cy; sm[3] = cz;
    sm[4] = mom[4] - M * cx * cx; sm[5] = mom[5] - M * cy * cy; sm[6] = mom[6] - M * cz * cz;
    sm[7] = mom[7] - M * cx * cy; sm[8] = mom[8] - M * cx * cz; sm[9] = mom[9] - M * cy * cz;
    sm[10] = sm[4] + sm[5] + sm[6];
  }
  __syncthreads();
  const int GG = G * G;  // 6 G^2 < 2^31 for G <= 1024
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 6 * GG) return;
  const int face = t / GG;
  const int rem = t - face * GG;
  const int u = rem / G, v = rem - u * G;
  int i, j, k;
  switch (face) {
    case 0: i = 0; j = u; k = v; break;
    case 1: i = G - 1; j = u; k = v; break;
    case 2: j = 0; i = u; k = v; break;
    case 3: j = G - 1; i = u; k = v; break;
    case 4: k = 0; i = u; j = v; break;
    default: k = G - 1; i = u; j = v; break;
  }
  const double M = sm[0];
  double phi = 0.0;
  if (M > 0.0) {
    const double rx = i * dx - sm[1], ry = j * dx - sm[2], rz = k * dx - sm[3];
    const double d2 = rx * rx + ry * ry + rz * rz + 1e-12;
    // 1/sqrt(d2): the f32 estimate refined by two Newton steps y <- y (3 - d2 y^2) / 2
    // in FP64 (relative error 2^-23 -> 2^-46 -> below the FP64 rounding), a
    // handful of FP64 operations instead of a square root and a division
    double inv = (double)rsqrtf((float)d2);
    inv = inv * (1.5 - 0.5 * d2 * inv * inv);
    inv = inv * (1.5 - 0.5 * d2 * inv * inv);
    // n.S.n d^2 as the quadratic form of r (no normalised n)
    const double rsr = rx * (rx * sm[4] + 2.0 * (ry * sm[7] + rz * sm[8])) + ry * (ry * sm[5] + 2.0 * rz * sm[9]) +
                       rz * rz * sm[6];
    const double inv2 = inv * inv;
    const double quad = 3.0 * rsr * inv2 - sm[10];
    // Phi = -G (M/d + (3 n.S.n - tr S) / (2 d^3)), multigrid.py:261-295
    phi = -grav * (M * inv + quad * (0.5 * inv2 * inv));
  }
  const size_t c = ((size_t)i * G + j) * G + k;
  const float h = (float)phi;
  const float l = (float)(phi - (double)h);
  hi[c] = h;
  lo[c] = l;
}

// Column moments of an f32 density: one warp per (i,j) column, Kahan-compensated
// FP32 sums along k, FP64 across columns (the reference's column scheme,
// multigrid.py:192-221, finished in FP64). Block partials of the ten raw moments.
__global__ void __launch_bounds__(256)
    k_moments_rho(const float *__restrict__ rho, int G, double dx, double *__restrict__ parts, unsigned *status) {
  const int lane = threadIdx.x & 31;
  const long long col = (long long)blockIdx.x * 8 + (threadIdx.x >> 5);
  double v[10];
#pragma unroll
  for (int q = 0; q < 10; ++q) v[q] = 0.0;
  if (col < (long long)G * G) {
    const int i = (int)(col / G), j = (int)(col % G);
    const float *p = rho + (size_t)col * G;
    float s0 = 0.f, c0 = 0.f, s1 = 0.f, c1 = 0.f, s2 = 0.f, c2 = 0.f;
    bool bad = false;
    for (int k = lane; k < G; k += 32) {
      const float r = p[k];
      if (!isfinite(r)) { bad = true; continue; }
      const float fk = (float)k;
      float y, t;
      y = r - c0; t = s0 + y; c0 = (t - s0) - y; s0 = t;
      const float r1 = r * fk;
      y = r1 - c1; t = s1 + y; c1 = (t - s1) - y; s1 = t;
      const float r2 = r1 * fk;
      y = r2 - c2; t = s2 + y; c2 = (t - s2) - y; s2 = t;
    }
    if (bad) atomicOr(status, GC_FLAG_NONFINITE_RHO);
    double S0 = (double)s0 - (double)c0, S1 = (double)s1 - (double)c1, S2 = (double)s2 - (double)c2;
    for (int o = 16; o > 0; o >>= 1) {
      S0 += __shfl_down_sync(0xffffffffu, S0, o);
      S1 += __shfl_down_sync(0xffffffffu, S1, o);
      S2 += __shfl_down_sync(0xffffffffu, S2, o);
    }
    if (lane == 0) {
      const double vol = dx * dx * dx;
      const double x = i * dx, y = j * dx;
      const double m0 = S0 * vol, m1 = S1 * vol * dx, m2 = S2 * vol * dx * dx;
      v[0] = m0; v[1] = m0 * x; v[2] = m0 * y; v[3] = m1;
      v[4] = m0 * x * x; v[5] = m0 * y * y; v[6] = m2;
      v[7] = m0 * x * y; v[8] = m1 * x; v[9] = m1 * y;
    }
  }
  block_partials<10>(v, parts + (size_t)blockIdx.x * 10);
}

// b0 = h^2 * f32(f32(4 pi G) * rho); partial sums of b0^2 over all nodes.
__global__ void __launch_bounds__(256)
    k_rhs_from_rho(const float *__restrict__ rho, float *__restrict__ b0, size_t n, float fpg, float h2,
                   double *__restrict__ parts) {
  float acc = 0.0f;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    const float rhs = __fmul_rn(fpg, rho[t]);
    const float bv = __fmul_rn(rhs, h2);
    b0[t] = bv;
    acc += bv * bv;
  }
  block_sum_f32(acc, parts + blockIdx.x);
}

__global__ void __launch_bounds__(256) k_sumsq(const float *__restrict__ a, size_t n, double *__restrict__ parts) {
  float acc = 0.0f;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
    acc += a[t] * a[t];
  block_sum_f32(acc, parts + blockIdx.x);
}

// Zero the interior nodes 1 .. G-2 of a G^3 array (node_grid launch shape).
__global__ void __launch_bounds__(256) k_zero_interior(float *__restrict__ a, int G) {
  const int k = blockIdx.x * 32 + threadIdx.x + 1, j = blockIdx.y * 8 + threadIdx.y + 1, i = blockIdx.z + 1;
  if (k <= G - 2 && j <= G - 2) a[((size_t)i * G + j) * G + k] = 0.0f;
}

__global__ void k_copy_hi_to(const float *__restrict__ hi, float *__restrict__ out, size_t n) {
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
    out[t] = hi[t];
}

// ------------------------------------------------------------------------------
// device-side stopping rule of the adaptive loop (graph-captured solves)
// ------------------------------------------------------------------------------
// The host loop of gc_mg_run, evaluated on the device after every residual: the
// cycle count lives in dsmall[GC_S_CYCLES]; the loop continues while fewer than
// max_cycles cycles ran and not (at least max(1, min_cycles) cycles ran and
// ||r|| < tol ||b|| with ||b|| > 0). The verdict goes to the conditional node
// that repeats the V-cycle body, the converged flag to dsmall[GC_S_CONVERGED].
__global__ void k_mg_decide(cudaGraphConditionalHandle h, double *__restrict__ small, double tol, int min_c,
                            int max_c, int first) {
  if (threadIdx.x != 0) return;
  const int c = first ? 0 : (int)small[GC_S_CYCLES] + 1;
  small[GC_S_CYCLES] = (double)c;
  const double b2 = small[GC_S_BNORM2], r2 = small[GC_S_RNORM2];
  const int minc = min_c > 1 ? min_c : 1;
  const bool conv = c >= minc && b2 > 0.0 && sqrt(r2) < tol * sqrt(b2);
  small[GC_S_CONVERGED] = conv ? 1.0 : 0.0;
  const bool more = !conv && c < max_c;
  if (!more) {  // the solve ends here: count it
    small[GC_S_SOLVES] += 1.0;
    small[GC_S_CYC_TOTAL] += (double)c;
    const double rel2 = b2 > 0.0 ? r2 / b2 : 0.0;
    if (rel2 > small[GC_S_MAXREL2]) small[GC_S_MAXREL2] = rel2;
  }
  cudaGraphSetConditional(h, more ? 1u : 0u);
}

// ------------------------------------------------------------------------------
// host orchestration
// ------------------------------------------------------------------------------
static dim3 rb_grid(const LevelGeom &g) {
  const int nkk = g.n / 2 + 1;
  return dim3(gc_blocks(nkk, RB_TX), gc_blocks(g.J, RB_TY), (unsigned)g.J);
}
static dim3 node_grid(const LevelGeom &g) { return dim3(gc_blocks(g.J, 32), gc_blocks(g.J, 8), (unsigned)g.J); }
// Sweeps each way on the levels below the finest.
static int coarse_pre(const gc_mg_params *p) { return (p->flags & GC_MG_COARSE_ONE_SWEEP) ? 1 : p->pre_sweeps; }
static int coarse_post(const gc_mg_params *p) { return (p->flags & GC_MG_COARSE_ONE_SWEEP) ? 1 : p->post_sweeps; }

static int launch_smooth(gc_ctx *ctx, int l, int sweeps) {
  const LevelGeom &g = ctx->lev[l];
  for (int s = 0; s < sweeps; ++s)
    for (int color = 0; color < 2; ++color)
      gc_launch(ctx, GK_SMOOTH, k_smooth, dim3(rb_grid(g)), dim3(dim3(RB_TX, RB_TY)), 0, ctx->e[l], ctx->b[l], g, color);
  GC_LAUNCH_CHECK(ctx, "smooth");
  return GC_OK;
}

static int launch_tail(gc_ctx *ctx, const gc_mg_params *p) {
  TailDesc d;
  memset(&d, 0, sizeof(d));
  d.nl = ctx->nlev - ctx->tail;
  d.pre = coarse_pre(p);
  d.post = coarse_post(p);
  for (int l = 0; l < d.nl; ++l) d.g[l] = ctx->lev[ctx->tail + l];
  // The coarsest level has at most 3^3 unknowns: a few FP64 Gauss-Seidel sweeps
  // solve it far below the V-cycle's contraction (J = 1 is exact in one sweep).
  const int Jc = d.g[d.nl - 1].J;
  d.coarse = Jc == 1 ? 1 : (p->coarse_sweeps < 8 * Jc ? p->coarse_sweeps : 8 * Jc);
  const size_t smem = tail_smem_bytes(ctx);
  static int attr_set_for = -1;
  if (smem > 48 * 1024 && attr_set_for != (int)smem) {
    GC_CUDA(ctx, cudaFuncSetAttribute(k_tail, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr_set_for = (int)smem;
  }
  gc_launch(ctx, GK_TAIL, k_tail, dim3(1), dim3(1024), smem, ctx->b[ctx->tail], ctx->e[ctx->tail], d);
  GC_LAUNCH_CHECK(ctx, "tail");
  return GC_OK;
}

static int finalize_to(gc_ctx *ctx, int nparts, int nv, int slot);

static Split0 split0(const gc_ctx *ctx) {
  Split0 d;
  d.G = ctx->G;
  d.H = ctx->H0;
  d.half = ctx->half0;
  return d;
}
// (kk, j, i) over the interior rows of the colour-split finest level
static dim3 split_grid(const gc_ctx *ctx) {
  return dim3(gc_blocks(ctx->H0, 64), gc_blocks(ctx->G - 2, 4), (unsigned)(ctx->G - 2));
}
#define SPLIT_BLOCK dim3(64, 4)
// slot pairs (vectorised kernels, G % 4 == 0)
static dim3 split_grid2(const gc_ctx *ctx) {
  return dim3(gc_blocks(ctx->H0 / 2, 64), gc_blocks(ctx->G - 2, 4), (unsigned)(ctx->G - 2));
}
// node quads of the interior rows (vectorised kernels, G % 4 == 0)
static dim3 quad_grid(const gc_ctx *ctx) {
  return dim3(gc_blocks(ctx->G / 4, 32), gc_blocks(ctx->G - 2, 8), (unsigned)(ctx->G - 2));
}
static bool vec4(const gc_ctx *ctx) { return ctx->G % 4 == 0; }

// CTAs of the persistent coarse launches: as many as fit at once (a cooperative
// launch needs them all resident), at most two per SM (fewer arrivals per grid
// barrier), and no more than the largest phase has work for.
static int coarse_grid(gc_ctx *ctx) {
  if (ctx->coarse_blocks > 0) return GC_OK;
  int occ_d = 0, occ_u = 0;
  GC_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_d, k_coarse_down, COARSE_THREADS, 0));
  GC_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_u, k_coarse_up, COARSE_THREADS, 0));
  int per_sm = occ_d < occ_u ? occ_d : occ_u;
  if (per_sm > 2) per_sm = 2;
  if (per_sm < 1) {
    gc_set_error(ctx, "coarse levels: the persistent kernel does not fit on an SM");
    return GC_ERR_CUDA;
  }
  const LevelGeom &g1 = ctx->lev[1];
  const long long rows = (long long)g1.J * g1.J;  // the largest phase: level 1's rows
  long long nb = (long long)gc_sms() * per_sm;
  const long long per_block = (long long)PR * (COARSE_THREADS / 32);
  const long long need = (rows + per_block - 1) / per_block;
  if (nb > need) nb = need;
  ctx->coarse_blocks = (int)(nb < 1 ? 1 : nb);
  return GC_OK;
}

static int launch_coarse(gc_ctx *ctx, const gc_mg_params *p, bool up) {
  CoarseDesc d;
  memset(&d, 0, sizeof(d));
  d.l0 = 1;
  d.l1 = ctx->tail;
  d.pre = coarse_pre(p);
  d.post = coarse_post(p);
  d.budget = 100000000LL;  // ~50 ms of SM clocks; a barrier normally takes microseconds
  d.bar = reinterpret_cast<GridBar *>(ctx->dsmall + GC_S_GRIDBAR);
  d.status = ctx->dstatus;
  d.rc = ctx->rc;
  for (int l = 1; l < ctx->nlev; ++l) {
    d.g[l] = ctx->lev[l];
    d.e[l] = ctx->e[l];
    d.b[l] = ctx->b[l];
  }
  int st = coarse_grid(ctx);
  if (st) return st;
  void *args[] = {&d};
  const void *fn = up ? (const void *)k_coarse_up : (const void *)k_coarse_down;
  ctx->prof.launches[GK_COARSE]++;
  const int slot = ctx->prof.enabled && !ctx->capturing ? gc_prof_slot(ctx, GK_COARSE) : -1;
  if (slot >= 0) cudaEventRecord(ctx->prof.ev[2 * slot], ctx->stream);
  GC_CUDA(ctx, cudaLaunchCooperativeKernel(fn, dim3(ctx->coarse_blocks), dim3(COARSE_THREADS), args, 0, ctx->stream));
  if (slot >= 0) cudaEventRecord(ctx->prof.ev[2 * slot + 1], ctx->stream);
  return GC_OK;
}

// Levels 1 .. nlev-1 of a V-cycle: b[1] in, e[1] out. Default: two persistent
// launches around the single-CTA tail; the validation path (natural layout)
// keeps one launch per phase.
static int coarse_levels(gc_ctx *ctx, const gc_mg_params *p) {
  const int L = ctx->nlev;
  int st;
  if (!(p->flags & (GC_MG_NATURAL_LAYOUT | GC_MG_PHASE_LAUNCHES)) && ctx->tail > 1) {
    if ((st = launch_coarse(ctx, p, false))) return st;
    if (ctx->tail < L && (st = launch_tail(ctx, p))) return st;
    return launch_coarse(ctx, p, true);
  }
  for (int l = 1; l < ctx->tail; ++l) {
    const LevelGeom &g = ctx->lev[l];
    const size_t n3 = (size_t)g.n * g.n * g.n;
    GC_CUDA(ctx, cudaMemsetAsync(ctx->e[l], 0, n3 * sizeof(float), ctx->stream));
    if ((st = launch_smooth(ctx, l, coarse_pre(p)))) return st;
    gc_launch(ctx, GK_RESID, k_resid, dim3(node_grid(g)), dim3(dim3(32, 8)), 0, ctx->e[l], ctx->b[l], ctx->rc, g);
    gc_launch(ctx, GK_RESTRICT, k_restrict, dim3(node_grid(ctx->lev[l + 1])), dim3(dim3(32, 8)), 0, ctx->rc, g,
              ctx->b[l + 1], ctx->lev[l + 1]);
    GC_LAUNCH_CHECK(ctx, "resid/restrict");
  }
  if (ctx->tail < L) {
    if ((st = launch_tail(ctx, p))) return st;
  }
  for (int l = ctx->tail - 1; l >= 1; --l) {
    gc_launch(ctx, GK_PROLONG, k_prolong, dim3(node_grid(ctx->lev[l])), dim3(dim3(32, 8)), 0, ctx->e[l + 1],
              ctx->lev[l + 1], ctx->e[l], ctx->lev[l]);
    GC_LAUNCH_CHECK(ctx, "prolong");
    if ((st = launch_smooth(ctx, l, coarse_post(p)))) return st;
  }
  return GC_OK;
}

// r = b0 - L phi on the finest interior (colour-split, or natural for the
// validation path), with ||r||^2 into dsmall[GC_S_RNORM2] (async). The split
// path also writes the first red half-sweep of the next pre-smoothing.
static int residual0(gc_ctx *ctx, const gc_mg_params *p) {
  const LevelGeom &g0 = ctx->lev[0];
  const dim3 grid = node_grid(g0);
  const size_t nb = (size_t)grid.x * grid.y * grid.z;
  int st = gc_ensure_red(ctx, nb);
  if (st) return st;
  const bool plain = (p->flags & GC_MG_PLAIN_F32) != 0;
  const Split0 d = split0(ctx);
  if (p->flags & GC_MG_NATURAL_LAYOUT) {
    if ((st = mg_alloc_natural(ctx))) return st;
    if (plain)
      gc_launch(ctx, GK_RESID0, k_resid0<true, false>, grid, dim3(32, 8), 0, ctx->hi, ctx->lo, ctx->b0, ctx->r0n,
                nullptr, ctx->red, d);
    else
      gc_launch(ctx, GK_RESID0, k_resid0<false, false>, grid, dim3(32, 8), 0, ctx->hi, ctx->lo, ctx->b0, ctx->r0n,
                nullptr, ctx->red, d);
  } else if (vec4(ctx)) {
    const int pre = ctx->nlev == 1 ? p->coarse_sweeps : p->pre_sweeps;
    float *ef = pre >= 1 ? ctx->e0s : nullptr;
    const dim3 qg = quad_grid(ctx);
    const size_t nq = (size_t)qg.x * qg.y * qg.z;
    if ((st = gc_ensure_red(ctx, nq))) return st;
    if (plain)
      gc_launch(ctx, GK_RESID0, k_resid0x4<true>, qg, dim3(32, 8), 0, ctx->hi, ctx->lo, ctx->b0, ctx->r0s, ef,
                ctx->red, d);
    else
      gc_launch(ctx, GK_RESID0, k_resid0x4<false>, qg, dim3(32, 8), 0, ctx->hi, ctx->lo, ctx->b0, ctx->r0s, ef,
                ctx->red, d);
    GC_LAUNCH_CHECK(ctx, "resid0");
    // (a last-block sum of the 16k block partials in this kernel was slower: the
    // blocks' tickets serialise on one counter)
    return finalize_to(ctx, (int)nq, 1, GC_S_RNORM2);
  } else {
    const int pre = ctx->nlev == 1 ? p->coarse_sweeps : p->pre_sweeps;
    float *ef = pre >= 1 ? ctx->e0s : nullptr;
    if (plain)
      gc_launch(ctx, GK_RESID0, k_resid0<true, true>, grid, dim3(32, 8), 0, ctx->hi, ctx->lo, ctx->b0, ctx->r0s, ef,
                ctx->red, d);
    else
      gc_launch(ctx, GK_RESID0, k_resid0<false, true>, grid, dim3(32, 8), 0, ctx->hi, ctx->lo, ctx->b0, ctx->r0s, ef,
                ctx->red, d);
  }
  GC_LAUNCH_CHECK(ctx, "resid0");
  return finalize_to(ctx, (int)nb, 1, GC_S_RNORM2);
}

// One V-cycle of the defect correction: relax L e = r from e = 0 (FP32,
// colour-split), restrict its residual, coarse correction, prolong, relax, then
// phi += e and the new residual r = b0 - L phi with its norm. Expects r (and,
// when pre-smoothing, the first red half-sweep) from the previous residual0.
static int vcycle(gc_ctx *ctx, const gc_mg_params *p) {
  const int L = ctx->nlev;
  if (L == 0) return GC_OK;
  const bool plain = (p->flags & GC_MG_PLAIN_F32) != 0;
  const int pre = L == 1 ? p->coarse_sweeps : p->pre_sweeps;  // one level: relaxation alone
  const int post = L == 1 ? 0 : p->post_sweeps;
  const LevelGeom &g0 = ctx->lev[0];
  const Split0 d = split0(ctx);
  int st;
  if (p->flags & GC_MG_NATURAL_LAYOUT) {
    // the same cycle with the generic kernels on a natural-layout correction
    const size_t g3 = (size_t)ctx->G * ctx->G * ctx->G;
    GC_CUDA(ctx, cudaMemsetAsync(ctx->e0n, 0, g3 * sizeof(float), ctx->stream));
    for (int h = 0; h < 2 * pre; ++h)
      gc_launch(ctx, GK_SMOOTH0, k_smooth, rb_grid(g0), dim3(RB_TX, RB_TY), 0, ctx->e0n, ctx->r0n, g0, h & 1);
    if (L > 1) {
      gc_launch(ctx, GK_RESIDE, k_resid, node_grid(g0), dim3(32, 8), 0, ctx->e0n, ctx->r0n, ctx->r0, g0);
      gc_launch(ctx, GK_RESTRICT, k_restrict, node_grid(ctx->lev[1]), dim3(32, 8), 0, ctx->r0, g0, ctx->b[1],
                ctx->lev[1]);
      GC_LAUNCH_CHECK(ctx, "natural resid/restrict");
      if ((st = coarse_levels(ctx, p))) return st;
      gc_launch(ctx, GK_PROLONG0, k_prolong, node_grid(g0), dim3(32, 8), 0, ctx->e[1], ctx->lev[1], ctx->e0n, g0);
      for (int h = 0; h < 2 * post; ++h)
        gc_launch(ctx, GK_SMOOTH0, k_smooth, rb_grid(g0), dim3(RB_TX, RB_TY), 0, ctx->e0n, ctx->r0n, g0, h & 1);
    }
    if (plain)
      gc_launch(ctx, GK_UPDATE0, k_update0<true, false>, node_grid(g0), dim3(32, 8), 0, (const float *)ctx->e0n,
                ctx->hi, ctx->lo, d);
    else
      gc_launch(ctx, GK_UPDATE0, k_update0<false, false>, node_grid(g0), dim3(32, 8), 0, (const float *)ctx->e0n,
                ctx->hi, ctx->lo, d);
    GC_LAUNCH_CHECK(ctx, "natural cycle");
    return residual0(ctx, p);
  }
  const dim3 sg = split_grid(ctx), sg2 = split_grid2(ctx), qg = quad_grid(ctx);
  const bool v4 = vec4(ctx);
  auto half_sweep = [&](int color) {
    if (v4)
      gc_launch(ctx, GK_SMOOTH0, k_rb0x2<false>, sg2, SPLIT_BLOCK, 0, ctx->e0s, (const float *)ctx->r0s, d, color);
    else
      gc_launch(ctx, GK_SMOOTH0, k_rb0<false>, sg, SPLIT_BLOCK, 0, ctx->e0s, (const float *)ctx->r0s, d, color);
  };
  if (pre == 0) GC_CUDA(ctx, cudaMemsetAsync(ctx->e0s, 0, 2 * ctx->half0 * sizeof(float), ctx->stream));
  // half-sweep 0 (red, from zero) came with the residual
  for (int h = 1; h < 2 * pre; ++h) half_sweep(h & 1);
  if (L > 1) {
    if (v4)
      gc_launch(ctx, GK_RESIDE, k_resid0ex4, qg, dim3(32, 8), 0, (const float *)ctx->e0s, (const float *)ctx->r0s,
                ctx->r0, d);
    else
      gc_launch(ctx, GK_RESIDE, k_resid0e, node_grid(g0), dim3(32, 8), 0, (const float *)ctx->e0s,
                (const float *)ctx->r0s, ctx->r0, d);
    gc_launch(ctx, GK_RESTRICT, k_restrict, node_grid(ctx->lev[1]), dim3(32, 8), 0, ctx->r0, g0, ctx->b[1],
              ctx->lev[1]);
    GC_LAUNCH_CHECK(ctx, "resid0e/restrict");
    if ((st = coarse_levels(ctx, p))) return st;
    if (v4 && post >= 1)
      gc_launch(ctx, GK_PROLONG0, k_prolong0bx2, sg2, SPLIT_BLOCK, 0, (const float *)ctx->e[1], ctx->lev[1], ctx->e0s,
                g0, d);
    else
      gc_launch(ctx, GK_PROLONG0, k_prolong0s, sg, SPLIT_BLOCK, 0, (const float *)ctx->e[1], ctx->lev[1], ctx->e0s,
                g0, d, post == 0 ? 1 : 0);
    for (int h = 0; h < 2 * post - 1; ++h) half_sweep(h & 1);
  }
  if (post >= 1 && v4) {  // last half-sweep (black) and phi += e in one pass
    if (plain)
      gc_launch(ctx, GK_UPDATE0, k_rb0_lastx4<true>, sg2, SPLIT_BLOCK, 0, (const float *)ctx->e0s,
                (const float *)ctx->r0s, ctx->hi, ctx->lo, d);
    else
      gc_launch(ctx, GK_UPDATE0, k_rb0_lastx4<false>, sg2, SPLIT_BLOCK, 0, (const float *)ctx->e0s,
                (const float *)ctx->r0s, ctx->hi, ctx->lo, d);
  } else if (post >= 1) {  // last half-sweep (black) and phi += e in one pass
    if (plain)
      gc_launch(ctx, GK_UPDATE0, k_rb0_last<true>, sg, SPLIT_BLOCK, 0, (const float *)ctx->e0s,
                (const float *)ctx->r0s, ctx->hi, ctx->lo, d);
    else
      gc_launch(ctx, GK_UPDATE0, k_rb0_last<false>, sg, SPLIT_BLOCK, 0, (const float *)ctx->e0s,
                (const float *)ctx->r0s, ctx->hi, ctx->lo, d);
  } else {
    if (plain)
      gc_launch(ctx, GK_UPDATE0, k_update0<true, true>, node_grid(g0), dim3(32, 8), 0, (const float *)ctx->e0s,
                ctx->hi, ctx->lo, d);
    else
      gc_launch(ctx, GK_UPDATE0, k_update0<false, true>, node_grid(g0), dim3(32, 8), 0, (const float *)ctx->e0s,
                ctx->hi, ctx->lo, d);
  }
  GC_LAUNCH_CHECK(ctx, "finest cycle");
  return residual0(ctx, p);
}

int gc_finalize(gc_ctx *ctx, const double *parts, int nparts, int nv, double *dst) {
  GC_REQUIRE(ctx, nv >= 1 && nv <= GC_FIN_NV, "gc_finalize: %d values per row (at most %d)", nv, GC_FIN_NV);
  if (nv == 1 && nparts > 32 * GC_FIN_CHUNKS) {
    double *tmp = ctx->dsmall + GC_S_FIN_TMP;
    gc_launch(ctx, GK_REDUCE, k_fin_chunks, dim3(GC_FIN_CHUNKS), dim3(256), 0, parts, nparts, tmp);
    gc_launch(ctx, GK_REDUCE, k_fin_warps, dim3(1), dim3(32), 0, (const double *)tmp, GC_FIN_CHUNKS, 1, dst);
  } else {
    gc_launch(ctx, GK_REDUCE, k_fin_warps, dim3(1), dim3(32 * nv), 0, parts, nparts, nv, dst);
  }
  GC_LAUNCH_CHECK(ctx, "finalize");
  return GC_OK;
}

static int finalize_to(gc_ctx *ctx, int nparts, int nv, int slot) {
  return gc_finalize(ctx, ctx->red, nparts, nv, ctx->dsmall + slot);
}

static int read_small(gc_ctx *ctx, int slot, int count) {
  GC_CUDA(ctx, cudaMemcpyAsync(ctx->hsmall + slot, ctx->dsmall + slot, count * sizeof(double), cudaMemcpyDeviceToHost,
                               ctx->stream));
  GC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return GC_OK;
}

// ||b0||^2 into dsmall[GC_S_BNORM2] (async).
int gc_norm_b(gc_ctx *ctx) {
  const size_t g3 = (size_t)ctx->G * ctx->G * ctx->G;
  const int nb = 2048;
  int st = gc_ensure_red(ctx, nb);
  if (st) return st;
  gc_launch(ctx, GK_REDUCE, k_sumsq, dim3(nb), dim3(256), 0, ctx->b0, g3, ctx->red);
  GC_LAUNCH_CHECK(ctx, "sumsq");
  return finalize_to(ctx, nb, 1, GC_S_BNORM2);
}

int gc_faces_from_moments(gc_ctx *ctx) {
  const long long tot = 6LL * ctx->G * ctx->G;
  gc_launch(ctx, GK_FACES, k_faces, dim3(gc_blocks(tot, 256)), dim3(256), 0, ctx->hi, ctx->lo, ctx->G, ctx->dx, ctx->grav, ctx->dmom);
  GC_LAUNCH_CHECK(ctx, "faces");
  return GC_OK;
}

// The adaptive loop inside a stream capture: the residual of the initial guess
// and the first decision, then a conditional while node whose body (captured on
// the context's side stream) is one V-cycle, its residual and the next decision.
// Same kernels in the same order as the host loop, so the same potential. The
// cycle count, the converged flag and both norms are left in dsmall and copied
// to the pinned host mirror at the end.
static int mg_run_captured(gc_ctx *ctx, const gc_mg_params *p) {
  int s;
  if (ctx->nlev == 0) return GC_OK;
  if ((s = residual0(ctx, p))) return s;
  cudaStreamCaptureStatus cs;
  cudaGraph_t graph = nullptr;
  const cudaGraphNode_t *deps = nullptr;
  size_t nd = 0;
  GC_CUDA(ctx, cudaStreamGetCaptureInfo(ctx->stream, &cs, nullptr, &graph, &deps, nullptr, &nd));
  GC_REQUIRE(ctx, cs == cudaStreamCaptureStatusActive, "captured solve outside a stream capture");
  cudaGraphConditionalHandle h;
  GC_CUDA(ctx, cudaGraphConditionalHandleCreate(&h, graph, 0, 0));
  gc_launch(ctx, GK_REDUCE, k_mg_decide, dim3(1), dim3(32), 0, h, ctx->dsmall, p->tol, p->min_cycles, p->max_cycles, 1);
  GC_LAUNCH_CHECK(ctx, "decide");
  GC_CUDA(ctx, cudaStreamGetCaptureInfo(ctx->stream, &cs, nullptr, &graph, &deps, nullptr, &nd));
  cudaGraphNodeParams np = {};
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = h;
  np.conditional.type = cudaGraphCondTypeWhile;
  np.conditional.size = 1;
  cudaGraphNode_t cond;
  GC_CUDA(ctx, cudaGraphAddNode(&cond, graph, deps, nullptr, nd, &np));
  cudaGraph_t body = np.conditional.phGraph_out[0];
  cudaStream_t main = ctx->stream;
  GC_CUDA(ctx, cudaStreamBeginCaptureToGraph(ctx->side, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
  ctx->stream = ctx->side;
  const long long before = gc_launch_total(ctx);
  s = vcycle(ctx, p);
  if (!s) {
    gc_launch(ctx, GK_REDUCE, k_mg_decide, dim3(1), dim3(32), 0, h, ctx->dsmall, p->tol, p->min_cycles,
              p->max_cycles, 0);
    s = gc_check_launch(ctx, "decide");
  }
  ctx->cap_body_launches = gc_launch_total(ctx) - before;
  cudaGraph_t got = nullptr;
  const cudaError_t e = cudaStreamEndCapture(ctx->side, &got);
  ctx->stream = main;
  if (s) return s;
  GC_CUDA(ctx, e);
  GC_CUDA(ctx, cudaStreamUpdateCaptureDependencies(main, &cond, nullptr, 1, cudaStreamSetCaptureDependencies));
  GC_CUDA(ctx, cudaMemcpyAsync(ctx->hsmall, ctx->dsmall, GC_S_MIRROR * sizeof(double), cudaMemcpyDeviceToHost, main));
  return GC_OK;
}

// Adaptive V-cycling (multigrid.py:473-485): at least one cycle, then stop once
// ||r|| < tol ||b|| (never before min_cycles; no test when ||b|| = 0), at most
// max_cycles. Expects b0, faces and the initial interior guess in place and
// ||b0||^2 in dsmall. The residual of the initial guess is formed first; every
// cycle ends with the residual of its result and its norm.
int gc_mg_run(gc_ctx *ctx, const gc_mg_params *p, gc_mg_stats *stats) {
  gc_mg_stats st;
  memset(&st, 0, sizeof(st));
  int s;
  // the persistent coarse launches' grid barrier starts every solve clean
  GC_CUDA(ctx, cudaMemsetAsync(ctx->dsmall + GC_S_GRIDBAR, 0, 2 * sizeof(double), ctx->stream));
  if (ctx->capturing && !(p->flags & GC_MG_FIXED_CYCLES)) {
    if ((s = mg_run_captured(ctx, p))) return s;
    st.cycles = -1;  // decided on the device: read them with gc_pm_graph_stats
    st.converged = -1;
    st.rhs_norm = st.res_norm = NAN;
    ctx->last_stats = st;
    ctx->solved_once = 1;
    if (stats) *stats = st;
    return GC_OK;
  }
  if (ctx->nlev > 0 && (s = residual0(ctx, p))) return s;
  if (p->flags & GC_MG_FIXED_CYCLES) {
    // exactly max_cycles V-cycles and no host read: the residual norm is left on
    // the device (gc_pm_last_residual reads it), so the solve can be captured in
    // a CUDA graph
    for (int c = 0; c < p->max_cycles && ctx->nlev > 0; ++c)
      if ((s = vcycle(ctx, p))) return s;
    // ||b0||^2 and ||r0||^2 (slots 0 and 1) to the pinned host mirror, stream
    // ordered: after a synchronisation the caller reads them without a copy
    GC_CUDA(ctx, cudaMemcpyAsync(ctx->hsmall, ctx->dsmall, 2 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    st.cycles = ctx->nlev > 0 ? p->max_cycles : 0;
    st.converged = -1;
    st.rhs_norm = st.res_norm = NAN;
    ctx->last_stats = st;
    ctx->solved_once = 1;
    if (stats) *stats = st;
    return GC_OK;
  }
  if ((s = read_small(ctx, GC_S_BNORM2, 2))) return s;
  const double bnorm = sqrt(ctx->hsmall[GC_S_BNORM2]);
  const double h2 = ctx->dx * ctx->dx;
  st.rhs_norm = bnorm / h2;
  if (ctx->nlev == 0) {
    st.cycles = 0;
    st.converged = 1;
    st.res_norm = 0.0;
  } else {
    double rnorm = sqrt(ctx->hsmall[GC_S_RNORM2]);
    const int min_c = p->min_cycles > 1 ? p->min_cycles : 1;
    int c = 0;
    for (;;) {
      if (c >= min_c && bnorm > 0.0 && rnorm < p->tol * bnorm) {
        st.converged = 1;
        break;
      }
      if (c >= p->max_cycles) break;
      if ((s = vcycle(ctx, p))) return s;
      ++c;
      if ((s = read_small(ctx, GC_S_RNORM2, 1))) return s;
      rnorm = sqrt(ctx->hsmall[GC_S_RNORM2]);
    }
    st.cycles = c;
    st.res_norm = rnorm / h2;
  }
  ctx->last_stats = st;
  ctx->solved_once = 1;
  if (stats) *stats = st;
  return GC_OK;
}

int gc_mg_check_params(gc_ctx *ctx, const gc_mg_params *p) {
  GC_REQUIRE(ctx, p->pre_sweeps >= 0 && p->post_sweeps >= 0 && p->pre_sweeps + p->post_sweeps >= 1,
             "sweep counts must be >= 0 with at least one smoothing sweep");
  GC_REQUIRE(ctx, p->coarse_sweeps >= 1, "coarse_sweeps must be >= 1");
  GC_REQUIRE(ctx, p->max_cycles >= 0 && p->max_cycles <= 100000, "max_cycles out of range");
  GC_REQUIRE(ctx, p->tol >= 0.0, "tol must be >= 0");
  return GC_OK;
}

// Moments of an f32 density into ctx->dmom (async). Raises GC_FLAG_NONFINITE_RHO.
static int moments_rho_async(gc_ctx *ctx, const float *rho) {
  const long long cols = (long long)ctx->G * ctx->G;
  const unsigned nb = gc_blocks(cols, 8);
  int s = gc_ensure_red(ctx, (size_t)nb * 10);
  if (s) return s;
  gc_launch(ctx, GK_MOMENTS, k_moments_rho, dim3(nb), dim3(256), 0, rho, ctx->G, ctx->dx, ctx->red, ctx->dstatus);
  GC_LAUNCH_CHECK(ctx, "moments");
  if ((s = gc_finalize(ctx, ctx->red, (int)nb, 10, ctx->dmom))) return s;
  GC_LAUNCH_CHECK(ctx, "moments finalize");
  return GC_OK;
}

extern "C" int gc_moments(gc_ctx *ctx, const float *rho, double out[10]) {
  if (!ctx) return GC_ERR_ARG;
  GC_REQUIRE(ctx, rho && out, "gc_moments: NULL pointer");
  int s = moments_rho_async(ctx, rho);
  if (s) return s;
  GC_CUDA(ctx, cudaMemcpyAsync(out, ctx->dmom, 10 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  GC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return GC_OK;
}

extern "C" int gc_mg_solve(gc_ctx *ctx, const float *rho, float *phi, int warm_start, const gc_mg_params *params,
                           gc_mg_stats *stats) {
  if (!ctx) return GC_ERR_ARG;
  GC_REQUIRE(ctx, rho && phi, "gc_mg_solve: NULL rho or phi");
  gc_mg_params p;
  if (params)
    p = *params;
  else
    gc_mg_default_params(&p);
  int s = gc_mg_check_params(ctx, &p);
  if (s) return s;
  const size_t g3 = (size_t)ctx->G * ctx->G * ctx->G;
  // moments (multigrid.py:364-389), on the device, no host round trip
  if ((s = moments_rho_async(ctx, rho))) return s;
  // b0 = h^2 * 4 pi G rho (multigrid.py:463) and ||b0||^2 (multigrid.py:477)
  {
    const int nb = 2048;
    if ((s = gc_ensure_red(ctx, nb))) return s;
    const float fpg = (float)(4.0 * M_PI * ctx->grav);
    const float h2 = (float)(ctx->dx * ctx->dx);
    gc_launch(ctx, GK_RHS, k_rhs_from_rho, dim3(nb), dim3(256), 0, rho, ctx->b0, g3, fpg, h2, ctx->red);
    GC_LAUNCH_CHECK(ctx, "rhs");
    if ((s = finalize_to(ctx, nb, 1, GC_S_BNORM2))) return s;
  }
  // initial guess (multigrid.py:464-467): previous phi or zero; the lo part starts at zero
  if (p.flags & GC_MG_FACES_GIVEN) {  // faces (and the guess) from phi
    GC_CUDA(ctx, cudaMemcpyAsync(ctx->hi, phi, g3 * sizeof(float), cudaMemcpyDeviceToDevice, ctx->stream));
    if (!warm_start && ctx->nlev > 0) {
      gc_launch(ctx, GK_COPY, k_zero_interior, dim3(node_grid(ctx->lev[0])), dim3(32, 8), 0, ctx->hi, ctx->G);
      GC_LAUNCH_CHECK(ctx, "zero interior");
    }
  } else if (warm_start) {
    GC_CUDA(ctx, cudaMemcpyAsync(ctx->hi, phi, g3 * sizeof(float), cudaMemcpyDeviceToDevice, ctx->stream));
  } else {
    GC_CUDA(ctx, cudaMemsetAsync(ctx->hi, 0, g3 * sizeof(float), ctx->stream));
  }
  GC_CUDA(ctx, cudaMemsetAsync(ctx->lo, 0, g3 * sizeof(float), ctx->stream));
  if (!(p.flags & GC_MG_FACES_GIVEN) && (s = gc_faces_from_moments(ctx))) return s;
  if ((s = gc_mg_run(ctx, &p, stats))) return s;
  // phi = f32(hi + lo) == hi (the pair is normalised)
  gc_launch(ctx, GK_COPY, k_copy_hi_to, dim3(1024), dim3(256), 0, ctx->hi, phi, g3);
  GC_LAUNCH_CHECK(ctx, "copy phi");
  uint32_t flags = 0;
  if ((s = gc_status(ctx, &flags, 0))) return s;
  if (flags & GC_FLAG_NONFINITE_RHO) {
    gc_set_error(ctx, "rho contains non-finite values");
    return GC_ERR_NONFINITE;
  }
  if (flags & GC_FLAG_TIMEOUT) {
    gc_set_error(ctx, "a bounded device wait of the solve timed out (the potential is incomplete)");
    return GC_ERR_TIMEOUT;
  }
  return GC_OK;
}

extern "C" int gc_mg_residual_norm(gc_ctx *ctx, const float *phi_f32, double *out) {
  if (!ctx) return GC_ERR_ARG;
  GC_REQUIRE(ctx, out, "gc_mg_residual_norm: NULL out");
  if (ctx->nlev == 0) {
    *out = 0.0;
    return GC_OK;
  }
  const LevelGeom &g0 = ctx->lev[0];
  const dim3 grid = node_grid(g0);
  const size_t nb = (size_t)grid.x * grid.y * grid.z;
  int s = gc_ensure_red(ctx, nb);
  if (s) return s;
  if (phi_f32)
    gc_launch(ctx, GK_RESID64, k_resid64, dim3(grid), dim3(dim3(32, 8)), 0, phi_f32, nullptr, ctx->b0, ctx->red, ctx->G);
  else
    gc_launch(ctx, GK_RESID64, k_resid64, dim3(grid), dim3(dim3(32, 8)), 0, ctx->hi, ctx->lo, ctx->b0, ctx->red, ctx->G);
  GC_LAUNCH_CHECK(ctx, "resid64");
  if ((s = finalize_to(ctx, (int)nb, 1, GC_S_RNORM64))) return s;
  if ((s = read_small(ctx, GC_S_RNORM64, 1))) return s;
  *out = sqrt(ctx->hsmall[GC_S_RNORM64]) / (ctx->dx * ctx->dx);
  return GC_OK;
}

extern "C" const float *gc_pm_potential(const gc_ctx *ctx) { return ctx ? ctx->hi : nullptr; }
