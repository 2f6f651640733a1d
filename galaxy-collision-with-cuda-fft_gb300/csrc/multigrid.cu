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
  GC_CUDA(ctx, cudaMalloc(&ctx->hi, g3 * sizeof(float)));
  GC_CUDA(ctx, cudaMalloc(&ctx->lo, g3 * sizeof(float)));
  GC_CUDA(ctx, cudaMalloc(&ctx->hi2, g3 * sizeof(float)));
  GC_CUDA(ctx, cudaMalloc(&ctx->lo2, g3 * sizeof(float)));
  GC_CUDA(ctx, cudaMemset(ctx->hi2, 0, g3 * sizeof(float)));
  GC_CUDA(ctx, cudaMemset(ctx->lo2, 0, g3 * sizeof(float)));
  GC_CUDA(ctx, cudaMalloc(&ctx->b0, g3 * sizeof(float)));
  GC_CUDA(ctx, cudaMalloc(&ctx->r0, g3 * sizeof(float)));
  GC_CUDA(ctx, cudaMemset(ctx->hi, 0, g3 * sizeof(float)));
  GC_CUDA(ctx, cudaMemset(ctx->lo, 0, g3 * sizeof(float)));
  GC_CUDA(ctx, cudaMemset(ctx->b0, 0, g3 * sizeof(float)));
  GC_CUDA(ctx, cudaMemset(ctx->r0, 0, g3 * sizeof(float)));
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

void gc_mg_free(gc_ctx *ctx) {
  cudaFree(ctx->hi); cudaFree(ctx->lo); cudaFree(ctx->hi2); cudaFree(ctx->lo2);
  cudaFree(ctx->b0); cudaFree(ctx->r0);
  for (int l = 1; l < GC_MAX_LEVELS; ++l) {
    cudaFree(ctx->e[l]); cudaFree(ctx->b[l]);
    ctx->e[l] = ctx->b[l] = nullptr;
  }
  cudaFree(ctx->rc);
  ctx->hi = ctx->lo = ctx->hi2 = ctx->lo2 = ctx->b0 = ctx->r0 = ctx->rc = nullptr;
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
// Accurate residual r = b - L_h2(hi + lo) at interior node c (h^2 units).
__device__ __forceinline__ float df_residual(const float *__restrict__ hi, const float *__restrict__ lo,
                                             float bc, size_t c, size_t sj, size_t si, float &hc_out,
                                             float &lc_out) {
  const float hc = hi[c];
  const float d0 = __fsub_rn(hi[c + si], hc);
  const float d1 = __fsub_rn(hi[c - si], hc);
  const float d2 = __fsub_rn(hi[c + sj], hc);
  const float d3 = __fsub_rn(hi[c - sj], hc);
  const float d4 = __fsub_rn(hi[c + 1], hc);
  const float d5 = __fsub_rn(hi[c - 1], hc);
  float s, e, t;
  df_two_sum(d0, d1, s, e);
  df_two_sum(s, d2, s, t); e = __fadd_rn(e, t);
  df_two_sum(s, d3, s, t); e = __fadd_rn(e, t);
  df_two_sum(s, d4, s, t); e = __fadd_rn(e, t);
  df_two_sum(s, d5, s, t); e = __fadd_rn(e, t);
  const float lc = lo[c];
  const float ln = ((((lo[c + si] + lo[c - si]) + lo[c + sj]) + lo[c - sj]) + lo[c + 1]) + lo[c - 1];
  const float ll = __fsub_rn(ln, __fmul_rn(6.0f, lc));
  float r1, r1e;
  df_two_sum(bc, -s, r1, r1e);
  hc_out = hc;
  lc_out = lc;
  return __fadd_rn(r1, __fsub_rn(r1e, __fadd_rn(e, ll)));
}

__global__ void __launch_bounds__(RB_TX *RB_TY)
    k_smooth0(float *__restrict__ hi, float *__restrict__ lo, const float *__restrict__ b, int G, int color) {
  const int kk = blockIdx.x * RB_TX + threadIdx.x;
  const int j = blockIdx.y * RB_TY + threadIdx.y + 1;
  const int i = blockIdx.z + 1;
  if (j > G - 2) return;
  const int k = 2 * kk + ((color + i + j) & 1);
  if (k < 1 || k > G - 2) return;
  const size_t sj = (size_t)G, si = (size_t)G * G;
  const size_t c = (size_t)i * si + (size_t)j * sj + k;
  float hc, lc;
  const float r = df_residual(hi, lo, b[c], c, sj, si, hc, lc);
  // Gauss-Seidel: phi_new = (sum6 - h^2 rhs)/6 = phi - r/6
  const float delta = __fmul_rn(r, -0.16666667f);
  float s2, e2, h3, l3;
  df_two_sum(hc, delta, s2, e2);
  const float ln = __fadd_rn(lc, e2);
  df_fast_two_sum(s2, ln, h3, l3);
  hi[c] = h3;
  lo[c] = l3;
}

// Residual on the finest interior (r may be NULL) and per-block partial of sum r^2.
__global__ void __launch_bounds__(256)
    k_resid0(const float *__restrict__ hi, const float *__restrict__ lo, const float *__restrict__ b,
             float *__restrict__ r, double *__restrict__ parts, int G) {
  const int k = blockIdx.x * 32 + threadIdx.x + 1;
  const int j = blockIdx.y * 8 + threadIdx.y + 1;
  const int i = blockIdx.z + 1;
  float acc = 0.0f;
  if (k <= G - 2 && j <= G - 2) {
    const size_t sj = (size_t)G, si = (size_t)G * G;
    const size_t c = (size_t)i * si + (size_t)j * sj + k;
    float hc, lc;
    const float rv = df_residual(hi, lo, b[c], c, sj, si, hc, lc);
    if (r) r[c] = rv;
    acc = rv * rv;
  }
  if (parts) {
    const size_t bid = ((size_t)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
    block_sum_f32(acc, parts + bid);
  }
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
  e[c] = (sum - b[c]) / diag;
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

// b_c = 4 * R(r_f): full weighting (transpose of trilinear prolongation).
__global__ void __launch_bounds__(256)
    k_restrict(const float *__restrict__ rf, LevelGeom f, float *__restrict__ bc, LevelGeom cg) {
  const int K = blockIdx.x * 32 + threadIdx.x + 1;
  const int Jj = blockIdx.y * 8 + threadIdx.y + 1;
  const int I = blockIdx.z + 1;
  if (K > cg.J || Jj > cg.J) return;
  float wi[3], wj[3], wk[3];
#pragma unroll
  for (int o = -1; o <= 1; ++o) {
    wi[o + 1] = restrict_w(I, o, f, cg);
    wj[o + 1] = restrict_w(Jj, o, f, cg);
    wk[o + 1] = restrict_w(K, o, f, cg);
  }
  const size_t n = f.n;
  float acc = 0.0f;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    if (wi[a] == 0.0f) continue;
    const size_t fi = (size_t)(2 * I + a - 1);
#pragma unroll
    for (int bb = 0; bb < 3; ++bb) {
      if (wj[bb] == 0.0f) continue;
      const size_t fj = (size_t)(2 * Jj + bb - 1);
      const float wij = wi[a] * wj[bb];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        if (wk[c] == 0.0f) continue;
        const size_t fk = (size_t)(2 * K + c - 1);
        acc += wij * wk[c] * rf[(fi * n + fj) * n + fk];
      }
    }
  }
  const size_t m = cg.n;
  bc[((size_t)I * m + Jj) * m + K] = 4.0f * acc;
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

// Finest level: add the coarse correction into the double-float pair.
__global__ void __launch_bounds__(256)
    k_prolong0(const float *__restrict__ ec, LevelGeom cg, float *__restrict__ hi, float *__restrict__ lo,
               LevelGeom f) {
  const int k = blockIdx.x * 32 + threadIdx.x + 1;
  const int j = blockIdx.y * 8 + threadIdx.y + 1;
  const int i = blockIdx.z + 1;
  if (k > f.J || j > f.J) return;
  const size_t n = f.n;
  const size_t c = ((size_t)i * n + j) * n + k;
  const float v = prolong_value(ec, i, j, k, f, cg);
  float s, e, h, l;
  df_two_sum(hi[c], v, s, e);
  const float ln = __fadd_rn(lo[c], e);
  df_fast_two_sum(s, ln, h, l);
  hi[c] = h;
  lo[c] = l;
}

// The same, two nodes (k, k+1), k even, per thread: the pair shares its coarse
// loads (the even node reads coarse column k/2, the odd one k/2 and k/2 + 1)
// and moves hi/lo as float2. Each node's sum is formed exactly as in
// prolong_value (same weights, same order), so the result is identical.
__global__ void __launch_bounds__(256)
    k_prolong0x2(const float *__restrict__ ec, LevelGeom cg, float *__restrict__ hi, float *__restrict__ lo,
                 LevelGeom f) {
  const int k = 2 * (blockIdx.x * 32 + threadIdx.x);
  const int j = blockIdx.y * 8 + threadIdx.y + 1;
  const int i = blockIdx.z + 1;
  if (j > f.J || k > f.J) return;  // k + 1 <= f.J + 1 = n - 1 stays inside the row (n even: c is even)
  const size_t n = f.n;
  const size_t c = ((size_t)i * n + j) * n + k;
  const bool u0 = k >= 1, u1 = k + 1 <= f.J;  // interior nodes of the pair
  int ci, cj, ck0, ck1;
  float wi0, wi1, wj0, wj1, a0, a1, b0, b1;
  const int ni = prolong_w(i, f, cg, ci, wi0, wi1);
  const int nj = prolong_w(j, f, cg, cj, wj0, wj1);
  const int nk0 = prolong_w(k, f, cg, ck0, a0, a1);      // even: one coarse column, weight 1
  const int nk1 = prolong_w(k + 1, f, cg, ck1, b0, b1);  // odd: ck1 == ck0, one or two columns
  const size_t m = cg.n;
  float v0 = 0.0f, v1 = 0.0f;
  for (int a = 0; a < ni; ++a) {
    const float wa = a ? wi1 : wi0;
    for (int bb = 0; bb < nj; ++bb) {
      const float wb = bb ? wj1 : wj0;
      const size_t row = ((size_t)(ci + a) * m + (cj + bb)) * m;
      const float wab = wa * wb;
      const float e0 = ec[row + ck0];
      const float e1 = (nk0 == 2 || nk1 == 2) ? ec[row + ck0 + 1] : 0.0f;
      v0 += wab * a0 * e0;
      if (nk0 == 2) v0 += wab * a1 * e1;
      v1 += wab * b0 * (ck1 == ck0 ? e0 : e1);
      if (nk1 == 2) v1 += wab * b1 * ec[row + ck1 + 1];
    }
  }
  float2 h = *reinterpret_cast<const float2 *>(hi + c);
  float2 l = *reinterpret_cast<const float2 *>(lo + c);
  if (u0) {
    float s1, e1, hh, ll;
    df_two_sum(h.x, v0, s1, e1);
    df_fast_two_sum(s1, __fadd_rn(l.x, e1), hh, ll);
    h.x = hh;
    l.x = ll;
  }
  if (u1) {
    float s1, e1, hh, ll;
    df_two_sum(h.y, v1, s1, e1);
    df_fast_two_sum(s1, __fadd_rn(l.y, e1), hh, ll);
    h.y = hh;
    l.y = ll;
  }
  *reinterpret_cast<float2 *>(hi + c) = h;
  *reinterpret_cast<float2 *>(lo + c) = l;
}

// ------------------------------------------------------------------------------
// finest level, fused: one red-black sweep per pass, streamed along i
// ------------------------------------------------------------------------------
// A CTA owns a SW_TJ x SW_TK tile of (j,k) columns and a chunk of i planes. It
// streams the planes through a ring in shared memory (hi, lo with a halo of 2
// in j and k; b likewise), loading plane p+1 with cp.async while it works on
// plane p: it relaxes the red nodes of plane p-1 on the tile plus a one-node
// ring (from old black values only), then the black nodes of plane p-2 on the
// tile (from the new red values), and stores plane p-2. Reading one potential
// buffer and writing the other keeps every CTA on old values outside its own
// tile, so the result is exactly the two in-place half-sweeps of k_smooth0,
// with each datum read and written once per sweep. Thread t relaxes one red
// node of the tile (plus one of the ring for the first 50 threads) and one
// black node per plane.
#define SW_TJ 16
#define SW_TK 32
#define SW_H 2                   // halo in j
#define SW_KO 5                  // smem column of k0 (rows start 16-byte aligned at k0 - 5)
#define SW_EJ (SW_TJ + 2 * SW_H)
#define SW_EK 40                 // k0 - 5 .. k0 + 34: the halo of 2 plus alignment
#define SW_THREADS 256
#define SW_NS 6  // potential planes in flight: p-3 .. p+2
#define SW_NB 5  // right-hand-side planes in flight: p-2 .. p+2

struct SweepSmem {
  float hi[SW_NS][SW_EJ][SW_EK];
  float lo[SW_NS][SW_EJ][SW_EK];
  float b[SW_NB][SW_EJ][SW_EK];
};

__device__ __forceinline__ int sw_slot(int p) { return (p + 10 * SW_NS) % SW_NS; }
__device__ __forceinline__ int sw_bslot(int p) { return (p + 10 * SW_NB) % SW_NB; }

// 16-byte asynchronous copy global -> shared; zero-filled (and no global read) when !valid.
__device__ __forceinline__ void sw_cp16(float *smem, const float *gmem, bool valid) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"((uint32_t)__cvta_generic_to_shared(smem)),
               "l"(gmem), "r"(valid ? 16 : 0)
               : "memory");
}

// The red-black Gauss-Seidel update of one node from the ring (same arithmetic
// order as df_residual + k_smooth0).
__device__ __forceinline__ void sw_update(SweepSmem &S, int sm, int sc, int sp, int bs, int jj, int kk) {
  const float hc = S.hi[sc][jj][kk];
  const float d0 = __fsub_rn(S.hi[sp][jj][kk], hc);
  const float d1 = __fsub_rn(S.hi[sm][jj][kk], hc);
  const float d2 = __fsub_rn(S.hi[sc][jj + 1][kk], hc);
  const float d3 = __fsub_rn(S.hi[sc][jj - 1][kk], hc);
  const float d4 = __fsub_rn(S.hi[sc][jj][kk + 1], hc);
  const float d5 = __fsub_rn(S.hi[sc][jj][kk - 1], hc);
  float s, e, t;
  df_two_sum(d0, d1, s, e);
  df_two_sum(s, d2, s, t); e = __fadd_rn(e, t);
  df_two_sum(s, d3, s, t); e = __fadd_rn(e, t);
  df_two_sum(s, d4, s, t); e = __fadd_rn(e, t);
  df_two_sum(s, d5, s, t); e = __fadd_rn(e, t);
  const float lc = S.lo[sc][jj][kk];
  const float ln = ((((S.lo[sp][jj][kk] + S.lo[sm][jj][kk]) + S.lo[sc][jj + 1][kk]) + S.lo[sc][jj - 1][kk]) +
                    S.lo[sc][jj][kk + 1]) + S.lo[sc][jj][kk - 1];
  const float ll = __fsub_rn(ln, __fmul_rn(6.0f, lc));
  float r1, r1e;
  df_two_sum(S.b[bs][jj][kk], -s, r1, r1e);
  const float r = __fadd_rn(r1, __fsub_rn(r1e, __fadd_rn(e, ll)));
  const float delta = __fmul_rn(r, -0.16666667f);
  float s2, e2, h3, l3;
  df_two_sum(hc, delta, s2, e2);
  const float lnew = __fadd_rn(lc, e2);
  df_fast_two_sum(s2, lnew, h3, l3);
  S.hi[sc][jj][kk] = h3;
  S.lo[sc][jj][kk] = l3;
}

// G must be a multiple of 4 (rows 16-byte aligned; a 16-byte group is wholly
// inside or outside the grid).
__global__ void __launch_bounds__(SW_THREADS)
    k_sweep0(const float *__restrict__ hi_in, const float *__restrict__ lo_in, const float *__restrict__ b,
             float *__restrict__ hi_out, float *__restrict__ lo_out, int G, int chunk) {
  extern __shared__ __align__(16) unsigned char sw_raw[];
  SweepSmem &S = *reinterpret_cast<SweepSmem *>(sw_raw);
  const int tid = threadIdx.x;
  const int j0 = 1 + blockIdx.y * SW_TJ;
  const int k0 = 1 + blockIdx.x * SW_TK;
  const int i0 = 1 + blockIdx.z * chunk;
  const int i1 = min(i0 + chunk, G - 1);  // planes [i0, i1) are relaxed and stored
  const size_t sj = (size_t)G, si = (size_t)G * G;
  auto load_plane = [&](int p) {  // issue the copies of plane p into its slots (16-byte groups)
    const int s = sw_slot(p), bs = sw_bslot(p);
    for (int t = tid; t < SW_EJ * (SW_EK / 4); t += SW_THREADS) {
      const int jj = t / (SW_EK / 4), q4 = t - jj * (SW_EK / 4);
      const int j = j0 - SW_H + jj, k = k0 - SW_KO + 4 * q4;
      const bool v = p >= 0 && p < G && j >= 0 && j < G && k >= 0 && k < G;
      const size_t c = v ? (size_t)p * si + (size_t)j * sj + k : 0;
      sw_cp16(&S.hi[s][jj][4 * q4], hi_in + c, v);
      sw_cp16(&S.lo[s][jj][4 * q4], lo_in + c, v);
      sw_cp16(&S.b[bs][jj][4 * q4], b + c, v);
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
  };
  load_plane(i0 - 2);
  load_plane(i0 - 1);
  for (int p = i0 - 2; p <= i1 + 1; ++p) {
    if (p + 2 <= i1 + 1) {
      load_plane(p + 2);
      asm volatile("cp.async.wait_group 2;" ::: "memory");  // plane p has landed
    } else if (p + 1 <= i1 + 1) {
      asm volatile("cp.async.wait_group 1;" ::: "memory");
    } else {
      asm volatile("cp.async.wait_group 0;" ::: "memory");
    }
    __syncthreads();
    const int q = p - 1;  // red on plane q, tile + 1 halo
    if (q >= i0 - 1 && q <= i1 && q >= 1 && q <= G - 2) {
      const int sc = sw_slot(q), sm = sw_slot(q - 1), sp = sw_slot(q + 1), bs = sw_bslot(q);
      for (int idx = tid; idx < (SW_EJ - 2) * 17; idx += SW_THREADS) {
        const int row = idx / 17, m = idx - row * 17;
        const int jj = 1 + row, j = j0 - SW_H + jj;
        const int kk = SW_KO - 1 + 2 * m + ((q + j + k0 - 1) & 1), k = k0 - SW_KO + kk;
        if (j < 1 || j > G - 2 || k < 1 || k > G - 2) continue;
        sw_update(S, sm, sc, sp, bs, jj, kk);
      }
    }
    __syncthreads();
    const int r = p - 2;  // black on plane r, tile only; then store plane r
    if (r >= i0 && r < i1) {
      const int sc = sw_slot(r), sm = sw_slot(r - 1), sp = sw_slot(r + 1), bs = sw_bslot(r);
      {
        const int row = tid >> 4, m = tid & 15;
        const int jj = SW_H + row, j = j0 + row;
        const int kk = SW_KO + 2 * m + (((r + j + k0) & 1) ? 0 : 1), k = k0 - SW_KO + kk;
        if (j <= G - 2 && k <= G - 2) sw_update(S, sm, sc, sp, bs, jj, kk);
      }
      __syncthreads();
      for (int idx = tid; idx < SW_TJ * SW_TK; idx += SW_THREADS) {
        const int row = idx >> 5, col = idx & 31;
        const int j = j0 + row, k = k0 + col;
        if (j > G - 2 || k > G - 2) continue;
        const size_t c = (size_t)r * si + (size_t)j * sj + k;
        hi_out[c] = S.hi[sc][SW_H + row][SW_KO + col];
        lo_out[c] = S.lo[sc][SW_H + row][SW_KO + col];
      }
    }
    __syncthreads();
  }
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

template <typename T>
__device__ void t_smooth(T *e, const T *b, const LevelGeom &g, int sweeps) {
  const int n = g.n, J = g.J;
  const int m = J * J * J;
  for (int s = 0; s < sweeps; ++s) {
    for (int color = 0; color < 2; ++color) {
      for (int t = threadIdx.x; t < m; t += blockDim.x) {
        const int k = t % J + 1, j = (t / J) % J + 1, i = t / (J * J) + 1;
        if (((i + j + k) & 1) != color) continue;
        const int c = (i * n + j) * n + k;
        T sx, sy, sz, dx_, dy_, dz_;
        if (i == J) { sx = (T)g.a * e[c - n * n]; dx_ = (T)g.dB; } else { sx = e[c + n * n] + e[c - n * n]; dx_ = 2; }
        if (j == J) { sy = (T)g.a * e[c - n]; dy_ = (T)g.dB; } else { sy = e[c + n] + e[c - n]; dy_ = 2; }
        if (k == J) { sz = (T)g.a * e[c - 1]; dz_ = (T)g.dB; } else { sz = e[c + 1] + e[c - 1]; dz_ = 2; }
        e[c] = ((sx + sy + sz) - b[c]) / (dx_ + dy_ + dz_);
      }
      __syncthreads();
    }
  }
}

__device__ void t_resid(const float *e, const float *b, float *r, const LevelGeom &g) {
  const int n = g.n, J = g.J;
  const int m = J * J * J;
  for (int t = threadIdx.x; t < m; t += blockDim.x) {
    const int k = t % J + 1, j = (t / J) % J + 1, i = t / (J * J) + 1;
    const int c = (i * n + j) * n + k;
    float sum, diag;
    sw_stencil(e, (size_t)c, i, j, k, g, sum, diag);
    r[c] = b[c] - (sum - diag * e[c]);
  }
  __syncthreads();
}

template <typename T>
__device__ void t_restrict(const float *rf, const LevelGeom &f, T *bc, const LevelGeom &cg) {
  const int J = cg.J, m = cg.n, n = f.n;
  const int tot = J * J * J;
  for (int t = threadIdx.x; t < tot; t += blockDim.x) {
    const int K = t % J + 1, Jj = (t / J) % J + 1, I = t / (J * J) + 1;
    float acc = 0.0f;
    for (int a = -1; a <= 1; ++a) {
      const float wa = restrict_w(I, a, f, cg);
      if (wa == 0.0f) continue;
      for (int bb = -1; bb <= 1; ++bb) {
        const float wb = restrict_w(Jj, bb, f, cg);
        if (wb == 0.0f) continue;
        for (int c = -1; c <= 1; ++c) {
          const float wc = restrict_w(K, c, f, cg);
          if (wc == 0.0f) continue;
          acc += wa * wb * wc * rf[((2 * I + a) * n + (2 * Jj + bb)) * n + (2 * K + c)];
        }
      }
    }
    bc[(I * m + Jj) * m + K] = (T)(4.0f * acc);
  }
  __syncthreads();
}

template <typename T>
__device__ void t_prolong(const T *ec, const LevelGeom &cg, float *ef, const LevelGeom &f) {
  const int J = f.J, n = f.n, m = cg.n;
  const int tot = J * J * J;
  for (int t = threadIdx.x; t < tot; t += blockDim.x) {
    const int k = t % J + 1, j = (t / J) % J + 1, i = t / (J * J) + 1;
    int ci, cj, ck;
    float wi0, wi1, wj0, wj1, wk0, wk1;
    const int ni = prolong_w(i, f, cg, ci, wi0, wi1);
    const int nj = prolong_w(j, f, cg, cj, wj0, wj1);
    const int nk = prolong_w(k, f, cg, ck, wk0, wk1);
    float val = 0.0f;
    for (int a = 0; a < ni; ++a)
      for (int bb = 0; bb < nj; ++bb)
        for (int c = 0; c < nk; ++c) {
          const float w = (a ? wi1 : wi0) * (bb ? wj1 : wj0) * (c ? wk1 : wk0);
          val += w * (float)ec[((ci + a) * m + (cj + bb)) * m + (ck + c)];
        }
    ef[(i * n + j) * n + k] += val;
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
      t_restrict<double>(R[l], d.g[l], B64, d.g[l + 1]);
    else
      t_restrict<float>(R[l], d.g[l], B[l + 1], d.g[l + 1]);
  }
  {
    const LevelGeom &gc = d.g[d.nl - 1];
    t_zero<double>(E64, gc.n * gc.n * gc.n);
    __syncthreads();
    t_smooth<double>(E64, B64, gc, d.coarse);
  }
  for (int l = d.nl - 2; l >= 0; --l) {
    if (l + 1 == d.nl - 1)
      t_prolong<double>(E64, d.g[l + 1], E[l], d.g[l]);
    else
      t_prolong<float>(E[l + 1], d.g[l + 1], E[l], d.g[l]);
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
    k_faces(float *__restrict__ hi, float *__restrict__ lo, float *__restrict__ hi2, float *__restrict__ lo2, int G,
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
    const double inv = 1.0 / sqrt(d2);
    const double nx = rx * inv, ny = ry * inv, nz = rz * inv;
    const double nsn = nx * nx * sm[4] + ny * ny * sm[5] + nz * nz * sm[6] +
                       2.0 * (nx * ny * sm[7] + nx * nz * sm[8] + ny * nz * sm[9]);
    const double quad = 3.0 * nsn - sm[10];
    // Phi = -G (M/d + (3 n.S.n - tr S) / (2 d^3)), multigrid.py:261-295
    phi = -grav * (M * inv + quad * (0.5 * inv * inv * inv));
  }
  const size_t c = ((size_t)i * G + j) * G + k;
  const float h = (float)phi;
  const float l = (float)(phi - (double)h);
  hi[c] = h;
  lo[c] = l;
  hi2[c] = h;  // both buffers of the streaming sweep carry the faces
  lo2[c] = l;
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

__global__ void k_copy_hi_to(const float *__restrict__ hi, float *__restrict__ out, size_t n) {
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
    out[t] = hi[t];
}

// ------------------------------------------------------------------------------
// host orchestration
// ------------------------------------------------------------------------------
static dim3 rb_grid(const LevelGeom &g) {
  const int nkk = g.n / 2 + 1;
  return dim3(gc_blocks(nkk, RB_TX), gc_blocks(g.J, RB_TY), (unsigned)g.J);
}
static dim3 node_grid(const LevelGeom &g) { return dim3(gc_blocks(g.J, 32), gc_blocks(g.J, 8), (unsigned)g.J); }
// pairs (k, k+1), k = 0, 2, ..., J: J/2 + 1 pairs per row
static dim3 pair_grid(const LevelGeom &g) {
  return dim3(gc_blocks(g.J / 2 + 1, 32), gc_blocks(g.J, 8), (unsigned)g.J);
}

// Add the level-1 correction into the finest double-float potential: pairs of
// nodes per thread when rows have an even length (so every pair starts on an
// 8-byte boundary), one node per thread otherwise.
static void launch_prolong0(gc_ctx *ctx, const LevelGeom &g) {
  if (g.n % 2 == 0)
    gc_launch(ctx, GK_PROLONG0, k_prolong0x2, dim3(pair_grid(g)), dim3(dim3(32, 8)), 0, ctx->e[1], ctx->lev[1],
              ctx->hi, ctx->lo, g);
  else
    gc_launch(ctx, GK_PROLONG0, k_prolong0, dim3(node_grid(g)), dim3(dim3(32, 8)), 0, ctx->e[1], ctx->lev[1],
              ctx->hi, ctx->lo, g);
}

// Finest-level smoothing: `sweeps` red-black sweeps, the first one preceded by
// the prolongation of the level-1 correction when `with_corr` is set. Default:
// in-place red and black half-sweep kernels. GC_MG_FUSED_SWEEP streams each
// sweep from (hi, lo) into (hi2, lo2) and swaps the buffers (same arithmetic).
static int launch_smooth0(gc_ctx *ctx, int sweeps, int with_corr, int flags) {
  const LevelGeom &g = ctx->lev[0];
  const int G = ctx->G;
  if (!(flags & GC_MG_FUSED_SWEEP) || sweeps == 0 || G % 4 != 0) {
    if (with_corr) {
      launch_prolong0(ctx, g);
    }
    for (int s = 0; s < sweeps; ++s)
      for (int color = 0; color < 2; ++color)
        gc_launch(ctx, GK_SMOOTH0, k_smooth0, dim3(rb_grid(g)), dim3(dim3(RB_TX, RB_TY)), 0, ctx->hi, ctx->lo,
                  ctx->b0, ctx->G, color);
    GC_LAUNCH_CHECK(ctx, "smooth0");
    return GC_OK;
  }
  if (with_corr)  // the coarse correction first (the streaming sweep starts from the corrected potential)
    launch_prolong0(ctx, g);
  if (!ctx->sw_smem_set) {  // 54 KB of dynamic shared memory: opt in once per context
    GC_CUDA(ctx, cudaFuncSetAttribute(k_sweep0, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SweepSmem)));
    ctx->sw_smem_set = 1;
  }
  const int tk = (G - 2 + SW_TK - 1) / SW_TK, tj = (G - 2 + SW_TJ - 1) / SW_TJ;
  int nchunks = ((int)gc_sms() * 4 + tk * tj - 1) / (tk * tj);  // ~4 CTAs per SM
  const int max_chunks = (G - 2 + 15) / 16;            // chunks of at least 16 planes
  if (nchunks > max_chunks) nchunks = max_chunks;
  if (nchunks < 1) nchunks = 1;
  const int chunk = (G - 2 + nchunks - 1) / nchunks;
  nchunks = (G - 2 + chunk - 1) / chunk;
  // pairs of streaming sweeps (each swaps the buffers, so a pair leaves the
  // potential where it started); an odd last sweep as two half-sweeps
  for (int s = 0; s < (sweeps & ~1); ++s) {
    gc_launch(ctx, GK_SWEEP0, k_sweep0, dim3(tk, tj, nchunks), dim3(SW_THREADS), sizeof(SweepSmem), ctx->hi,
              ctx->lo, ctx->b0, ctx->hi2, ctx->lo2, G, chunk);
    float *t = ctx->hi; ctx->hi = ctx->hi2; ctx->hi2 = t;
    t = ctx->lo; ctx->lo = ctx->lo2; ctx->lo2 = t;
  }
  if (sweeps & 1)
    for (int color = 0; color < 2; ++color)
      gc_launch(ctx, GK_SMOOTH0, k_smooth0, dim3(rb_grid(g)), dim3(dim3(RB_TX, RB_TY)), 0, ctx->hi, ctx->lo,
                ctx->b0, ctx->G, color);
  GC_LAUNCH_CHECK(ctx, "sweep0");
  return GC_OK;
}

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
  d.pre = p->pre_sweeps;
  d.post = p->post_sweeps;
  for (int l = 0; l < d.nl; ++l) d.g[l] = ctx->lev[ctx->tail + l];
  // The coarsest level has at most 3^3 unknowns: a few FP64 Gauss-Seidel sweeps
  // solve it far below the V-cycle's contraction (J = 1 is exact in one sweep).
  const int Jc = d.g[d.nl - 1].J;
  d.coarse = p->coarse_sweeps < 8 * Jc ? p->coarse_sweeps : 8 * Jc;
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

static int vcycle(gc_ctx *ctx, const gc_mg_params *p) {
  const int L = ctx->nlev;
  if (L == 0) return GC_OK;
  if (L == 1) return launch_smooth0(ctx, p->coarse_sweeps, 0, p->flags);
  int st;
  if ((st = launch_smooth0(ctx, p->pre_sweeps, 0, p->flags))) return st;
  const LevelGeom &g0 = ctx->lev[0];
  gc_launch(ctx, GK_RESID0, k_resid0, dim3(node_grid(g0)), dim3(dim3(32, 8)), 0, ctx->hi, ctx->lo, ctx->b0, ctx->r0, nullptr, ctx->G);
  gc_launch(ctx, GK_RESTRICT, k_restrict, dim3(node_grid(ctx->lev[1])), dim3(dim3(32, 8)), 0, ctx->r0, g0, ctx->b[1], ctx->lev[1]);
  GC_LAUNCH_CHECK(ctx, "resid0/restrict");
  for (int l = 1; l < ctx->tail; ++l) {
    const LevelGeom &g = ctx->lev[l];
    const size_t n3 = (size_t)g.n * g.n * g.n;
    GC_CUDA(ctx, cudaMemsetAsync(ctx->e[l], 0, n3 * sizeof(float), ctx->stream));
    if ((st = launch_smooth(ctx, l, p->pre_sweeps))) return st;
    gc_launch(ctx, GK_RESID, k_resid, dim3(node_grid(g)), dim3(dim3(32, 8)), 0, ctx->e[l], ctx->b[l], ctx->rc, g);
    gc_launch(ctx, GK_RESTRICT, k_restrict, dim3(node_grid(ctx->lev[l + 1])), dim3(dim3(32, 8)), 0, ctx->rc, g, ctx->b[l + 1], ctx->lev[l + 1]);
    GC_LAUNCH_CHECK(ctx, "resid/restrict");
  }
  if (ctx->tail < L) {
    if ((st = launch_tail(ctx, p))) return st;
  }
  for (int l = ctx->tail - 1; l >= 1; --l) {
    gc_launch(ctx, GK_PROLONG, k_prolong, dim3(node_grid(ctx->lev[l])), dim3(dim3(32, 8)), 0, ctx->e[l + 1], ctx->lev[l + 1], ctx->e[l], ctx->lev[l]);
    GC_LAUNCH_CHECK(ctx, "prolong");
    if ((st = launch_smooth(ctx, l, p->post_sweeps))) return st;
  }
  return launch_smooth0(ctx, p->post_sweeps, 1, p->flags);
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

// ||r0||^2 into dsmall[GC_S_RNORM2] (async).
static int resid_norm_async(gc_ctx *ctx) {
  const LevelGeom &g0 = ctx->lev[0];
  const dim3 grid = node_grid(g0);
  const size_t nb = (size_t)grid.x * grid.y * grid.z;
  int st = gc_ensure_red(ctx, nb);
  if (st) return st;
  gc_launch(ctx, GK_RESID0, k_resid0, dim3(grid), dim3(dim3(32, 8)), 0, ctx->hi, ctx->lo, ctx->b0, nullptr, ctx->red, ctx->G);
  GC_LAUNCH_CHECK(ctx, "resid0 norm");
  return finalize_to(ctx, (int)nb, 1, GC_S_RNORM2);
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
  gc_launch(ctx, GK_FACES, k_faces, dim3(gc_blocks(tot, 256)), dim3(256), 0, ctx->hi, ctx->lo, ctx->hi2, ctx->lo2, ctx->G, ctx->dx, ctx->grav, ctx->dmom);
  GC_LAUNCH_CHECK(ctx, "faces");
  return GC_OK;
}

// Adaptive V-cycling (multigrid.py:473-485). Expects b0, faces and the initial
// interior guess in place and ||b0||^2 in dsmall.
int gc_mg_run(gc_ctx *ctx, const gc_mg_params *p, gc_mg_stats *stats) {
  gc_mg_stats st;
  memset(&st, 0, sizeof(st));
  int s;
  if (p->flags & GC_MG_FIXED_CYCLES) {
    // exactly max_cycles V-cycles and no host read: the residual norm is left on
    // the device (gc_pm_last_residual reads it), so the solve can be captured in
    // a CUDA graph
    for (int c = 0; c < p->max_cycles && ctx->nlev > 0; ++c)
      if ((s = vcycle(ctx, p))) return s;
    if (ctx->nlev > 0 && (s = resid_norm_async(ctx))) return s;
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
  s = read_small(ctx, GC_S_BNORM2, 1);
  if (s) return s;
  const double bnorm = sqrt(ctx->hsmall[GC_S_BNORM2]);
  const double h2 = ctx->dx * ctx->dx;
  st.rhs_norm = bnorm / h2;
  st.cycles = p->max_cycles;
  st.converged = 0;
  double rnorm = NAN;
  if (ctx->nlev == 0) {
    st.cycles = 0;
    st.converged = 1;
    st.res_norm = 0.0;
  } else {
    for (int c = 0; c < p->max_cycles; ++c) {
      if ((s = vcycle(ctx, p))) return s;
      if (c + 1 >= p->min_cycles && bnorm > 0.0) {
        if ((s = resid_norm_async(ctx))) return s;
        if ((s = read_small(ctx, GC_S_RNORM2, 1))) return s;
        rnorm = sqrt(ctx->hsmall[GC_S_RNORM2]);
        if (rnorm < p->tol * bnorm) {
          st.cycles = c + 1;
          st.converged = 1;
          break;
        }
      }
    }
    if (!(rnorm == rnorm)) {
      if ((s = resid_norm_async(ctx))) return s;
      if ((s = read_small(ctx, GC_S_RNORM2, 1))) return s;
      rnorm = sqrt(ctx->hsmall[GC_S_RNORM2]);
    }
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
  if (warm_start) {
    GC_CUDA(ctx, cudaMemcpyAsync(ctx->hi, phi, g3 * sizeof(float), cudaMemcpyDeviceToDevice, ctx->stream));
  } else {
    GC_CUDA(ctx, cudaMemsetAsync(ctx->hi, 0, g3 * sizeof(float), ctx->stream));
  }
  GC_CUDA(ctx, cudaMemsetAsync(ctx->lo, 0, g3 * sizeof(float), ctx->stream));
  if ((s = gc_faces_from_moments(ctx))) return s;
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
