// Particle <-> grid kernels of the PM force chain.
//
// Arithmetic follows the reference kernels in src/galaxy_collision/deposit.py
// and integrator.py operation by operation in f32 with explicit
// round-to-nearest intrinsics (no FMA contraction), so the CPU restatement can
// reproduce them bit for bit. The deposit accumulates the reference's per-corner
// contributions m*wx*wy*wz into an int64 fixed-point grid: the partial product
// (m/dx^3*wx)*wy is rounded to f32 as the reference rounds it, and its exact
// product with wz is rounded once to the nearest quantum (one fused
// multiply-add). Integer addition is associative, so the density is
// bit-identical whatever the particle order or atomic interleaving.
#include "common.cuh"
#include "umma.cuh"

#include <math.h>

#include <cmath>
#include <cstdint>

// ------------------------------------------------------------------------------
// fixed-point set-up: total density-mass and quantum exponent
// ------------------------------------------------------------------------------
// The quantum must not depend on the particle order (sorting permutes the
// particles), so the total S = sum m/dx^3 is formed exactly: every positive
// finite term is truncated to an integer multiple of 2^-s, with s chosen from
// the largest term (an order-independent maximum) so that the integer sum of
// all n terms stays below 2^62, and the integers are summed exactly.
__global__ void __launch_bounds__(256) k_mass_max(const float *__restrict__ m, long long n, float inv_vol,
                                                  unsigned *__restrict__ maxbits) {
  unsigned best = 0;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    const float mm = __fmul_rn(m[p], inv_vol);
    if (isfinite(mm) && mm > 0.0f) best = max(best, __float_as_uint(mm));
  }
  best = __reduce_max_sync(0xffffffffu, best);
  if ((threadIdx.x & 31) == 0 && best) atomicMax(maxbits, best);
}

__device__ __forceinline__ int mass_shift(unsigned maxbits, int log2n) {
  const int emax = (int)((maxbits >> 23) & 0xffu) - 127;  // max term < 2^(emax+1)
  return 62 - log2n - (emax + 1);
}

__global__ void __launch_bounds__(256) k_mass_isum(const float *__restrict__ m, long long n, float inv_vol,
                                                   const unsigned *__restrict__ maxbits, int log2n,
                                                   unsigned long long *__restrict__ isum) {
  const int s = mass_shift(*maxbits, log2n);
  unsigned long long acc = 0;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    const float mm = __fmul_rn(m[p], inv_vol);
    if (isfinite(mm) && mm > 0.0f) {  // floor(mm * 2^s) from the float bits (no FP64)
      const unsigned u = __float_as_uint(mm);
      int ex = (int)((u >> 23) & 0xffu);
      const unsigned long long mant = (u & 0x7fffffu) | (ex ? 0x800000u : 0u);
      if (ex == 0) ex = 1;
      const int e2 = ex - 150 + s;
      acc += e2 >= 0 ? (mant << e2) : (e2 > -64 ? (mant >> -e2) : 0ull);
    }
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0 && acc) atomicAdd(isum, acc);
}

// E = exponent(S) - bits so that the whole mass is at most 2^bits quanta.
__global__ void k_qexp(const unsigned *__restrict__ maxbits, const unsigned long long *__restrict__ isum, int log2n,
                       double *__restrict__ small, int mass_slot, int exp_slot, int bits) {
  if (threadIdx.x != 0) return;
  double S = 0.0;
  if (*maxbits) S = ldexp((double)(*isum), -mass_shift(*maxbits, log2n));
  int ex = 0;
  if (S > 0.0) frexp(S, &ex);  // S = f * 2^ex, f in [0.5, 1)
  int E = ex - bits;
  if (E < -120) E = -120;      // keep 2^-E a normal f32
  if (E > 120) E = 120;
  small[mass_slot] = S;
  small[exp_slot] = (double)E;
}

static int ceil_log2(long long n) {
  int L = 0;
  while ((1LL << L) < n) ++L;
  return L;
}

int gc_fixed_point_setup(gc_ctx *ctx, const float *m, int64_t n, int bits, int mass_slot, int exp_slot) {
  const float dxf = (float)ctx->dx;
  const float inv_vol = 1.0f / ((dxf * dxf) * dxf);
  // two integer scratch words live in the reduction buffer
  int s = gc_ensure_red(ctx, 4);
  if (s) return s;
  unsigned *maxbits = (unsigned *)ctx->red;
  unsigned long long *isum = (unsigned long long *)(ctx->red + 1);
  GC_CUDA(ctx, cudaMemsetAsync(ctx->red, 0, 2 * sizeof(double), ctx->stream));
  unsigned nb = gc_blocks(n, 256);
  if (nb > gc_sms() * 8u) nb = gc_sms() * 8u;
  const int L = ceil_log2((long long)n);
  gc_launch(ctx, GK_MASS, k_mass_max, dim3(nb), dim3(256), 0, m, (long long)n, inv_vol, maxbits);
  gc_launch(ctx, GK_MASS, k_mass_isum, dim3(nb), dim3(256), 0, m, (long long)n, inv_vol, maxbits, L, isum);
  gc_launch(ctx, GK_MASS, k_qexp, dim3(1), dim3(32), 0, maxbits, isum, L, ctx->dsmall, mass_slot, exp_slot, bits);
  GC_LAUNCH_CHECK(ctx, "fixed-point set-up");
  return GC_OK;
}

// ------------------------------------------------------------------------------
// deposit (deposit.py:47-82)
// ------------------------------------------------------------------------------
// RNE(a * b * 2^k) as an int64, for finite a, b and |a * b * 2^k| < 2^62: the
// product of the two 24-bit significands is exact in 64 bits, so the rounding
// is the single rounding of the exact product (integer ALUs only).
__device__ __forceinline__ long long prod_to_i64_rn(float a, float b, int k) {
  const unsigned ua = __float_as_uint(a), ub = __float_as_uint(b);
  int ea = (int)((ua >> 23) & 0xffu), eb = (int)((ub >> 23) & 0xffu);
  const unsigned long long ma = (ua & 0x7fffffu) | (ea ? 0x800000u : 0u);
  const unsigned long long mb = (ub & 0x7fffffu) | (eb ? 0x800000u : 0u);
  if (ea == 0) ea = 1;
  if (eb == 0) eb = 1;
  const unsigned long long prod = ma * mb;  // < 2^48
  const int sh = ea + eb - 300 + k;          // |a * b * 2^k| = prod * 2^sh
  long long r;
  if (sh >= 0) {
    r = (long long)(prod << sh);
  } else if (sh <= -49) {
    r = 0;  // below 1/2
  } else {
    const int rs = -sh;
    unsigned long long q = prod >> rs;
    const unsigned long long rem = prod & ((1ull << rs) - 1ull), half = 1ull << (rs - 1);
    if (rem > half || (rem == half && (q & 1ull))) q += 1ull;
    r = (long long)q;
  }
  return ((ua ^ ub) >> 31) ? -r : r;
}

// The exponent k of a power of two 2^k held in a normal f32.
__device__ __forceinline__ int pow2_exponent(float p) { return (int)((__float_as_uint(p) >> 23) & 0xffu) - 127; }

// Per-corner int64 contributions of one particle; corners outside the box are 0.
// Returns false when the particle deposits nothing.
__device__ __forceinline__ bool cic_contrib(float x, float y, float z, float mass, const DepCtx &d, float qscale,
                                            CellPos &c, long long (&q)[8]) {
  if (!gc_cell_of(x, y, z, d.dx, d.G, c)) return false;
  const float mm = __fmul_rn(mass, d.inv_vol);
  const int qk = pow2_exponent(qscale);
  const float wx[2] = {__fsub_rn(1.0f, c.fx), c.fx};
  const float wy[2] = {__fsub_rn(1.0f, c.fy), c.fy};
  const float wz[2] = {__fsub_rn(1.0f, c.fz), c.fz};
#pragma unroll
  for (int cx = 0; cx < 2; ++cx)
#pragma unroll
    for (int cy = 0; cy < 2; ++cy)
#pragma unroll
      for (int cz = 0; cz < 2; ++cz) {
        const int jx = c.ix + cx, jy = c.iy + cy, jz = c.iz + cz;
        const bool in = (unsigned)jx < (unsigned)d.G && (unsigned)jy < (unsigned)d.G && (unsigned)jz < (unsigned)d.G;
        const float b = __fmul_rn(__fmul_rn(mm, wx[cx]), wy[cy]);
        q[(cx * 2 + cy) * 2 + cz] = in ? prod_to_i64_rn(b, wz[cz], qk) : 0LL;
      }
  return true;
}

__device__ __forceinline__ void flush_corners(long long *__restrict__ qg, int ix, int iy, int iz, int G,
                                              const long long (&q)[8]) {
#pragma unroll
  for (int cx = 0; cx < 2; ++cx)
#pragma unroll
    for (int cy = 0; cy < 2; ++cy)
#pragma unroll
      for (int cz = 0; cz < 2; ++cz) {
        const long long v = q[(cx * 2 + cy) * 2 + cz];
        const int jx = ix + cx, jy = iy + cy, jz = iz + cz;
        if (v != 0 && (unsigned)jx < (unsigned)G && (unsigned)jy < (unsigned)G && (unsigned)jz < (unsigned)G) {
          const size_t idx = ((size_t)jx * G + jy) * G + jz;
          atomicAdd((unsigned long long *)(qg + idx), (unsigned long long)v);
        }
      }
}

// One particle per thread; when a whole warp shares one cell its 8 corner sums
// are reduced in registers and flushed by one lane.
__global__ void __launch_bounds__(256)
    k_deposit(const float *__restrict__ x, const float *__restrict__ y, const float *__restrict__ z,
              const float *__restrict__ m, long long n, DepCtx d, const double *__restrict__ qexp,
              long long *__restrict__ qg, unsigned *__restrict__ status) {
  const float qscale = ldexpf(1.0f, -(int)(*qexp));
  const int lane = threadIdx.x & 31;
  const long long warp0 = (blockIdx.x * (long long)blockDim.x + (threadIdx.x & ~31));
  const long long wstride = (long long)gridDim.x * blockDim.x;
  for (long long base = warp0; base < n; base += wstride) {
    const long long p = base + lane;
    CellPos c;
    long long q[8];
    bool ok = false;
    if (p < n) {
      const float px = x[p], py = y[p], pz = z[p];
      if (!gc_finite3(px, py, pz)) atomicOr(status, GC_FLAG_NONFINITE_POS);
      ok = cic_contrib(px, py, pz, m[p], d, qscale, c, q);
    }
    const unsigned key = ok ? (unsigned)(((c.ix + 1) * (d.G + 1) + (c.iy + 1)) * (d.G + 1) + (c.iz + 1))
                            : (0x80000000u | (unsigned)lane);
    int all_same = 0;
    __match_all_sync(0xffffffffu, key, &all_same);
    if (all_same) {
#pragma unroll
      for (int t = 0; t < 8; ++t) {
        long long v = q[t];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        q[t] = v;
      }
      if (lane == 0) flush_corners(qg, c.ix, c.iy, c.iz, d.G, q);
    } else if (ok) {
      flush_corners(qg, c.ix, c.iy, c.iz, d.G, q);
    }
  }
}

// Cell-sorted particles, warp-contiguous. Lane L of warp w takes the particles
// t0 + 256 w + 32 j + L (j = 0..7) of the CTA's tile of 2048, so the 32
// particles a warp handles at once are adjacent in the array: after the cell
// sort they share one or two cells, and the particles that drifted into a
// neighbouring cell since the sort are scattered among them.
//
// Per particle the 8 corner contributions are the reference's products
// m/dx^3 * wx * wy * wz (deposit.py:69-82) scaled by the quantum (a power of
// two: exact) and rounded to the nearest integer (dep_corners: the last
// multiplication fused with the rounding, two corners per packed f32x2
// instruction). The bias of the rounding is subtracted in integer arithmetic,
// and the corner values are summed in int32, which is exact because every
// partial sum fits.
//
// Into the shared-memory box (below) the warp keeps a run cell (dep_warp_runs):
// lanes in it add their corners in registers, and the run is reduced across the
// warp with one redux.sync per corner when the warp leaves the cell. Directly
// into the grid (dep_warp_pass) the cells of lane 0 and lane 31 are the warp's
// "main" cells, each reduced with one full-warp redux.sync per corner. In both,
// lanes in any other cell (drifted particles, or sparse regions where every
// particle has its own cell) add their own corners. A redux.sync over the full
// warp costs the same whatever the keys, unlike one per group of equal keys,
// which serialises over the groups.
//
// Each warp owns an int32 box of nodes in shared memory (no block-wide
// barriers: warps never wait for each other). Corners go to it when the cells
// of the warp's 256 particles fit DEP_WBOX nodes (the box is the cell range of
// their coordinate range: x/dx is monotone) and their total quanta bound every
// node below 2^31; the box is added to the int64 grid with one atomic per
// nonzero node when the warp moves on. Otherwise corners go to the grid
// directly. Particles whose contribution reaches 2^22 quanta (point masses) are
// deposited out of line at the end of the tile with the general int64
// rounding. Correct for any particle order;
// the sort makes it fast.
#define DEP_NONE 0xffffffffu
#define DEP_PER 8
#define DEP_TILE (256 * DEP_PER)
#define DEP_BOX 8192
#define DEP_WBOX (DEP_BOX / 8)  // nodes of one warp's box
static_assert(DEP_WBOX <= 1024, "the box flush's reciprocal quotients are exact below 2^10 nodes");
#define DEP_BIAS 0x4B400000u

// Packed f32x2 arithmetic (two lanes of a 64-bit register, IEEE round to
// nearest per lane).
__device__ __forceinline__ float2 f2_mul(float2 a, float2 b) {
  float2 r;
  asm("{\n\t.reg .b64 A, B, D;\n\tmov.b64 A, {%2, %3};\n\tmov.b64 B, {%4, %5};\n\t"
      "mul.rn.f32x2 D, A, B;\n\tmov.b64 {%0, %1}, D;\n\t}"
      : "=f"(r.x), "=f"(r.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return r;
}
__device__ __forceinline__ float2 f2_fma(float2 a, float2 b, float2 c) {
  float2 r;
  asm("{\n\t.reg .b64 A, B, C, D;\n\tmov.b64 A, {%2, %3};\n\tmov.b64 B, {%4, %5};\n\tmov.b64 C, {%6, %7};\n\t"
      "fma.rn.f32x2 D, A, B, C;\n\tmov.b64 {%0, %1}, D;\n\t}"
      : "=f"(r.x), "=f"(r.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
  return r;
}

// The 8 corner values of a particle of s quanta (|s| < 2^22) with weights
// (wx0, fx), (wy0, fy), (wz0, fz), as the bits of 1.5 * 2^23 + RNE(b * wz)
// (corner order (cx, cy, cz)): the partial products a = s*wx and b = a*wy are
// rounded to f32, and b * wz + 1.5 * 2^23 is one fused multiply-add, whose single
// rounding (spacing 1 in [2^23, 2^24)) is the rounding of the exact product to
// the nearest integer. Two corners per packed instruction.
__device__ __forceinline__ void dep_corners(float s, float wx0, float fx, float wy0, float fy, float wz0, float fz,
                                            unsigned (&r)[8]) {
  const float2 a = f2_mul(make_float2(s, s), make_float2(wx0, fx));
  const float2 wy = make_float2(wy0, fy), wz = make_float2(wz0, fz), M = make_float2(12582912.0f, 12582912.0f);
  const float2 b0 = f2_mul(make_float2(a.x, a.x), wy), b1 = f2_mul(make_float2(a.y, a.y), wy);
  const float2 r01 = f2_fma(make_float2(b0.x, b0.x), wz, M), r23 = f2_fma(make_float2(b0.y, b0.y), wz, M);
  const float2 r45 = f2_fma(make_float2(b1.x, b1.x), wz, M), r67 = f2_fma(make_float2(b1.y, b1.y), wz, M);
  r[0] = __float_as_uint(r01.x); r[1] = __float_as_uint(r01.y);
  r[2] = __float_as_uint(r23.x); r[3] = __float_as_uint(r23.y);
  r[4] = __float_as_uint(r45.x); r[5] = __float_as_uint(r45.y);
  r[6] = __float_as_uint(r67.x); r[7] = __float_as_uint(r67.y);
}

// Corner contributions of a particle whose mass exceeds 2^22 quanta.
__device__ __forceinline__ void cic_q_large(float mm, float fx, float fy, float fz, float qscale, long long (&q)[8]) {
  const float wx[2] = {__fsub_rn(1.0f, fx), fx};
  const float wy[2] = {__fsub_rn(1.0f, fy), fy};
  const float wz[2] = {__fsub_rn(1.0f, fz), fz};
  const int qk = pow2_exponent(qscale);
#pragma unroll
  for (int c = 0; c < 8; ++c)
    q[c] = prod_to_i64_rn(__fmul_rn(__fmul_rn(mm, wx[c >> 2]), wy[(c >> 1) & 1]), wz[c & 1], qk);
}

// Add 8 corner values to the int64 grid, dropping corners outside it.
__device__ __forceinline__ void corners_to_grid(long long *__restrict__ qg, int G, int ix, int iy, int iz,
                                                const long long (&q)[8]) {
  const bool interior = ix >= 0 && iy >= 0 && iz >= 0 && ix + 1 < G && iy + 1 < G && iz + 1 < G;
  if (interior) {
    const int base = (ix * G + iy) * G + iz;  // G^3 < 2^31
#pragma unroll
    for (int c = 0; c < 8; ++c)
      if (q[c] != 0)
        atomicAdd((unsigned long long *)(qg + base + ((c >> 2) * G + ((c >> 1) & 1)) * G + (c & 1)),
                  (unsigned long long)q[c]);
  } else {
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      const int jx = ix + (c >> 2), jy = iy + ((c >> 1) & 1), jz = iz + (c & 1);
      if (q[c] != 0 && (unsigned)jx < (unsigned)G && (unsigned)jy < (unsigned)G && (unsigned)jz < (unsigned)G)
        atomicAdd((unsigned long long *)(qg + ((size_t)jx * G + jy) * G + jz), (unsigned long long)q[c]);
    }
  }
}

// A particle whose contribution reaches 2^22 quanta goes to the grid on its own.
__device__ __noinline__ void large_to_grid(long long *__restrict__ qg, int G, int ix, int iy, int iz, float mm,
                                           float fx, float fy, float fz, float qscale) {
  long long q[8];
  cic_q_large(mm, fx, fy, fz, qscale, q);
  corners_to_grid(qg, G, ix, iy, iz, q);
}

// The tile's box of nodes [x0, x0+nx) x [y0, y0+ny) x [z0, z0+nz) in shared memory.
struct DepBox {
  int *b;
  int x0, y0, z0, ny, nz, nyz;
};

template <bool BOX>
__device__ __forceinline__ void dep_out(const DepBox &bx, long long *__restrict__ qg, int G, int ix, int iy, int iz,
                                        const int (&t)[8]) {
  if (BOX) {
    int *b = bx.b + ((ix - bx.x0) * bx.ny + (iy - bx.y0)) * bx.nz + (iz - bx.z0);
    const int nz = bx.nz, nyz = bx.nyz;
    atomicAdd(b, t[0]); atomicAdd(b + 1, t[1]); atomicAdd(b + nz, t[2]); atomicAdd(b + nz + 1, t[3]);
    atomicAdd(b + nyz, t[4]); atomicAdd(b + nyz + 1, t[5]); atomicAdd(b + nyz + nz, t[6]);
    atomicAdd(b + nyz + nz + 1, t[7]);
  } else {
    const long long q[8] = {t[0], t[1], t[2], t[3], t[4], t[5], t[6], t[7]};
    corners_to_grid(qg, G, ix, iy, iz, q);
  }
}

// dep_out with the lane's box node already located.
template <bool BOX>
__device__ __forceinline__ void dep_put(int bo, const DepBox &bx, long long *__restrict__ qg, int G, int ix, int iy,
                                        int iz, const int (&t)[8]) {
  if (BOX) {
    int *bp = bx.b + bo;
    const int nz = bx.nz, nyz = bx.nyz;
    atomicAdd(bp, t[0]); atomicAdd(bp + 1, t[1]); atomicAdd(bp + nz, t[2]); atomicAdd(bp + nz + 1, t[3]);
    atomicAdd(bp + nyz, t[4]); atomicAdd(bp + nyz + 1, t[5]); atomicAdd(bp + nyz + nz, t[6]);
    atomicAdd(bp + nyz + nz + 1, t[7]);
  } else {
    const long long q[8] = {t[0], t[1], t[2], t[3], t[4], t[5], t[6], t[7]};
    corners_to_grid(qg, G, ix, iy, iz, q);
  }
}

// The DEP_PER particles of one lane (registers), 32 adjacent particles of the
// warp at a time. Sets bit j of `large` for particles left to the out-of-line pass.
template <bool POW2, bool BOX, int NJ = DEP_PER>
__device__ __forceinline__ void dep_warp_pass(const float (&px)[NJ], const float (&py)[NJ],
                                              const float (&pz)[NJ], const float (&pm)[NJ], long long nrem,
                                              const DepCtx &d, float inv_dx, float qscale, const DepBox &bx,
                                              long long *__restrict__ qg, unsigned *__restrict__ status, int lane,
                                              unsigned &large) {
  const int G1 = d.G + 1;
  const float hi = (float)d.G;
#pragma unroll
  for (int j = 0; j < NJ; ++j) {
    float gx, gy, gz;
    if (POW2) {  // x / dx == x * (1/dx) exactly when dx is a power of two
      gx = __fmul_rn(px[j], inv_dx); gy = __fmul_rn(py[j], inv_dx); gz = __fmul_rn(pz[j], inv_dx);
    } else {
      gx = __fdiv_rn(px[j], d.dx); gy = __fdiv_rn(py[j], d.dx); gz = __fdiv_rn(pz[j], d.dx);
    }
    const bool inr = gx >= -1.0f && gx < hi && gy >= -1.0f && gy < hi && gz >= -1.0f && gz < hi;
    const int ix = __float2int_rd(gx), iy = __float2int_rd(gy), iz = __float2int_rd(gz);
    const float fx = __fsub_rn(gx, __int2float_rn(ix)), fy = __fsub_rn(gy, __int2float_rn(iy)),
                fz = __fsub_rn(gz, __int2float_rn(iz));
    const float mmq = __fmul_rn(__fmul_rn(pm[j], d.inv_vol), qscale);
    const bool small = fabsf(mmq) < 4194304.0f;
    if (!inr && 32 * j < nrem && !gc_finite3(px[j], py[j], pz[j])) atomicOr(status, GC_FLAG_NONFINITE_POS);
    if (inr && !small) large |= 1u << j;
    const bool ok = inr && small;
    const float s = ok ? mmq : 0.0f;
    const float wx0 = __fsub_rn(1.0f, fx), wy0 = __fsub_rn(1.0f, fy), wz0 = __fsub_rn(1.0f, fz);
    unsigned r[8];
    dep_corners(s, wx0, fx, wy0, fy, wz0, fz, r);
    const unsigned key = ok ? (unsigned)(((ix + 1) * G1 + (iy + 1)) * G1 + (iz + 1)) : DEP_NONE;
    const unsigned kA = __shfl_sync(0xffffffffu, key, 0), kB = __shfl_sync(0xffffffffu, key, 31);
    const bool inA = key == kA, inB = key == kB;
    // the lane's corner values, unbiased once for every use below (lanes without
    // a key are never summed into an output: their products may be NaN)
    int v[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) v[c] = (int)(r[c] - DEP_BIAS);
    // the lane's node in the box, shared by the three outputs (unsigned: a lane
    // without a key may hold any cell)
    const int bo = BOX ? (int)((((unsigned)ix - (unsigned)bx.x0) * (unsigned)bx.ny + ((unsigned)iy - (unsigned)bx.y0)) *
                                   (unsigned)bx.nz +
                               ((unsigned)iz - (unsigned)bx.z0))
                       : 0;
    int t[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) t[c] = __reduce_add_sync(0xffffffffu, inA ? v[c] : 0);
    if (lane == 0 && kA != DEP_NONE) dep_put<BOX>(bo, bx, qg, d.G, ix, iy, iz, t);
    if (kB != kA) {
#pragma unroll
      for (int c = 0; c < 8; ++c) t[c] = __reduce_add_sync(0xffffffffu, inB ? v[c] : 0);
      if (lane == 31 && kB != DEP_NONE) dep_put<BOX>(bo, bx, qg, d.G, ix, iy, iz, t);
    }
    if (!inA && !inB && key != DEP_NONE) dep_put<BOX>(bo, bx, qg, d.G, ix, iy, iz, v);
  }
}

// The box path with warp runs: after the cell sort the warp's 32 particles
// of one step mostly share one cell with those of the next steps, so the warp
// keeps a run cell K (warp-uniform) and each lane adds its corner values for K
// in registers; the run's 8 sums are reduced across the warp (redux.sync) and
// added to the box only when no lane is in K any more, and at the end. Lane 31's
// cell, when it differs from K (the warp reaching the next cell), is reduced at
// once; particles in any other cell (drifted since the sort) add their own
// corners. The sums are those of dep_warp_pass regrouped: integer, exact
// (every partial sum of the warp's 256 particles is below 2^30 on this path).
template <bool POW2, int NJ = DEP_PER>
__device__ __forceinline__ void dep_warp_runs(const float (&px)[NJ], const float (&py)[NJ], const float (&pz)[NJ],
                                              const float (&pm)[NJ], long long nrem, const DepCtx &d, float inv_dx,
                                              float qscale, const DepBox &bx, unsigned *__restrict__ status, int lane,
                                              unsigned &large) {
  const int G1 = d.G + 1;
  const float hi = (float)d.G;
  unsigned K = DEP_NONE;  // the run's cell (warp-uniform) ...
  int Kbo = 0;            // ... and its node in the box
  int acc[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) acc[c] = 0;
#pragma unroll
  for (int j = 0; j < NJ; ++j) {
    float gx, gy, gz;
    if (POW2) {  // x / dx == x * (1/dx) exactly when dx is a power of two
      gx = __fmul_rn(px[j], inv_dx); gy = __fmul_rn(py[j], inv_dx); gz = __fmul_rn(pz[j], inv_dx);
    } else {
      gx = __fdiv_rn(px[j], d.dx); gy = __fdiv_rn(py[j], d.dx); gz = __fdiv_rn(pz[j], d.dx);
    }
    const bool inr = gx >= -1.0f && gx < hi && gy >= -1.0f && gy < hi && gz >= -1.0f && gz < hi;
    const int ix = __float2int_rd(gx), iy = __float2int_rd(gy), iz = __float2int_rd(gz);
    const float fx = __fsub_rn(gx, __int2float_rn(ix)), fy = __fsub_rn(gy, __int2float_rn(iy)),
                fz = __fsub_rn(gz, __int2float_rn(iz));
    const float mmq = __fmul_rn(__fmul_rn(pm[j], d.inv_vol), qscale);
    const bool small = fabsf(mmq) < 4194304.0f;
    if (!inr && 32 * j < nrem && !gc_finite3(px[j], py[j], pz[j])) atomicOr(status, GC_FLAG_NONFINITE_POS);
    if (inr && !small) large |= 1u << j;
    const bool ok = inr && small;
    const float s = ok ? mmq : 0.0f;
    const float wx0 = __fsub_rn(1.0f, fx), wy0 = __fsub_rn(1.0f, fy), wz0 = __fsub_rn(1.0f, fz);
    unsigned r[8];
    dep_corners(s, wx0, fx, wy0, fy, wz0, fz, r);
    int v[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) v[c] = (int)(r[c] - DEP_BIAS);
    const unsigned key = ok ? (unsigned)(((ix + 1) * G1 + (iy + 1)) * G1 + (iz + 1)) : DEP_NONE;
    // the lane's node in the box (unsigned: a lane without a key may hold any cell)
    const int bo = (int)((((unsigned)ix - (unsigned)bx.x0) * (unsigned)bx.ny + ((unsigned)iy - (unsigned)bx.y0)) *
                             (unsigned)bx.nz +
                         ((unsigned)iz - (unsigned)bx.z0));
    if (!__any_sync(0xffffffffu, K != DEP_NONE && key == K)) {  // the run has ended (warp-uniform)
      if (K != DEP_NONE) {
        int t[8];
#pragma unroll
        for (int c = 0; c < 8; ++c) t[c] = __reduce_add_sync(0xffffffffu, acc[c]);
        if (lane == 0) dep_put<true>(Kbo, bx, nullptr, d.G, 0, 0, 0, t);
      }
      const unsigned have = __ballot_sync(0xffffffffu, key != DEP_NONE);
      const int src = have ? __ffs(have) - 1 : 0;
      K = have ? __shfl_sync(0xffffffffu, key, src) : DEP_NONE;
      Kbo = __shfl_sync(0xffffffffu, bo, src);
#pragma unroll
      for (int c = 0; c < 8; ++c) acc[c] = 0;
    }
    const bool inK = K != DEP_NONE && key == K;
    if (inK) {
#pragma unroll
      for (int c = 0; c < 8; ++c) acc[c] += v[c];
    }
    const unsigned kB = __shfl_sync(0xffffffffu, key, 31);
    const bool bnext = kB != K && kB != DEP_NONE;  // lane 31 already in another cell (warp-uniform)
    const bool inB = bnext && key == kB;
    if (bnext) {
      int t[8];
#pragma unroll
      for (int c = 0; c < 8; ++c) t[c] = __reduce_add_sync(0xffffffffu, inB ? v[c] : 0);
      if (lane == 31) dep_put<true>(bo, bx, nullptr, d.G, 0, 0, 0, t);
    }
    if (key != DEP_NONE && !inK && !inB) dep_put<true>(bo, bx, nullptr, d.G, 0, 0, 0, v);
  }
  if (K != DEP_NONE) {
    int t[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) t[c] = __reduce_add_sync(0xffffffffu, acc[c]);
    if (lane == 0) dep_put<true>(Kbo, bx, nullptr, d.G, 0, 0, 0, t);
  }
}

// The warp's particles straight into the grid (a tile whose cells do not fit the
// box): out of line, reloading the particles, so that the registers of the box
// path are not shaped by this rare one. Returns the `large` bits.
template <bool POW2>
__device__ __noinline__ unsigned dep_warp_direct(const float *__restrict__ x, const float *__restrict__ y,
                                                 const float *__restrict__ z, const float *__restrict__ m, long long wb,
                                                 long long nrem, const DepCtx d, float inv_dx, float qscale,
                                                 long long *__restrict__ qg, unsigned *__restrict__ status, int lane) {
  float px[DEP_PER], py[DEP_PER], pz[DEP_PER], pm[DEP_PER];
#pragma unroll
  for (int j = 0; j < DEP_PER; ++j) {
    if (32 * j < nrem) {
      px[j] = __ldg(x + wb + 32 * j); py[j] = __ldg(y + wb + 32 * j); pz[j] = __ldg(z + wb + 32 * j);
      pm[j] = __ldg(m + wb + 32 * j);
    } else {
      px[j] = py[j] = pz[j] = __int_as_float(0x7fc00000);
      pm[j] = 0.0f;
    }
  }
  DepBox bx = {};
  unsigned large = 0;
  dep_warp_pass<POW2, false>(px, py, pz, pm, nrem, d, inv_dx, qscale, bx, qg, status, lane, large);
  return large;
}

template <bool POW2>
__global__ void __launch_bounds__(256, 4)
    k_deposit_sorted(const float *__restrict__ x, const float *__restrict__ y, const float *__restrict__ z,
                     const float *__restrict__ m, long long n, DepCtx d, float inv_dx,
                     const double *__restrict__ qexp, long long *__restrict__ qg, unsigned *__restrict__ status) {
  __shared__ int box[DEP_BOX];
  const float qscale = ldexpf(1.0f, -(int)(*qexp));
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  int *wbox = box + warp * DEP_WBOX;  // each warp owns a box: no block-wide barriers
  for (int i = lane; i < DEP_WBOX; i += 32) wbox[i] = 0;  // every flush zeroes what it read
  __syncwarp();
  for (long long t0 = (long long)blockIdx.x * DEP_TILE; t0 < n; t0 += (long long)gridDim.x * DEP_TILE) {
    const long long wb = t0 + warp * (32 * DEP_PER) + lane;
    const long long nrem = n - wb;  // particle j of this lane exists when 32 j < nrem
    if (nrem + lane <= 0) continue;  // this warp's part of the last tile is empty (warp-uniform)
    float px[DEP_PER], py[DEP_PER], pz[DEP_PER], pm[DEP_PER];
#pragma unroll
    for (int j = 0; j < DEP_PER; ++j) {
      if (32 * j < nrem) {
        px[j] = __ldg(x + wb + 32 * j); py[j] = __ldg(y + wb + 32 * j); pz[j] = __ldg(z + wb + 32 * j);
        pm[j] = __ldg(m + wb + 32 * j);
      } else {  // missing: NaN position (ignored by the bounds, deposits nothing), zero mass
        px[j] = py[j] = pz[j] = __int_as_float(0x7fc00000);
        pm[j] = 0.0f;
      }
    }
    // the warp's cell range from its coordinate range (fminf/fmaxf skip NaN),
    // clamped to the cells -1 .. G-1 that receive mass, and its largest |m|
    DepBox bx;
    bx.b = wbox;
    bool use_box;
    int nx;
    {
      float xl = 3.0e38f, yl = 3.0e38f, zl = 3.0e38f, xh = -3.0e38f, yh = -3.0e38f, zh = -3.0e38f;
      unsigned mb = 0;
#pragma unroll
      for (int j = 0; j < DEP_PER; ++j) {
        xl = fminf(xl, px[j]); xh = fmaxf(xh, px[j]);
        yl = fminf(yl, py[j]); yh = fmaxf(yh, py[j]);
        zl = fminf(zl, pz[j]); zh = fmaxf(zh, pz[j]);
        mb = max(mb, __float_as_uint(pm[j]) & 0x7fffffffu);
      }
      const float gl = -1.0f, gh = (float)d.G - 1.0f;
      const float cl[3] = {xl, yl, zl}, ch[3] = {xh, yh, zh};
      int lo[3], hi[3];
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        float l = POW2 ? __fmul_rn(cl[a], inv_dx) : __fdiv_rn(cl[a], d.dx);
        float h = POW2 ? __fmul_rn(ch[a], inv_dx) : __fdiv_rn(ch[a], d.dx);
        l = fminf(fmaxf(floorf(l), gl), gh);
        h = fminf(fmaxf(floorf(h), gl), gh);
        const bool any_pt = cl[a] <= ch[a];
        lo[a] = __reduce_min_sync(0xffffffffu, any_pt ? (int)l : 0x7fffffff);
        hi[a] = __reduce_max_sync(0xffffffffu, any_pt ? (int)h : -0x7fffffff);
      }
      mb = __reduce_max_sync(0xffffffffu, mb);
      bx.x0 = lo[0]; bx.y0 = lo[1]; bx.z0 = lo[2];
      nx = hi[0] - lo[0] + 2;
      bx.ny = hi[1] - lo[1] + 2;
      bx.nz = hi[2] - lo[2] + 2;
      bx.nyz = bx.ny * bx.nz;
      // every small corner is at most min(largest |m| in quanta, 2^22) + 1/2
      const float mq = __fmul_rn(__fmul_rn(__uint_as_float(mb), d.inv_vol), qscale);
      use_box = hi[0] >= lo[0] && (long long)nx * bx.nyz <= DEP_WBOX &&
                __fmul_rn(fminf(mq, 4194304.0f) + 1.0f, (float)(32 * DEP_PER)) < 1073741824.0f;
    }
    unsigned large = 0;
    if (use_box)
      dep_warp_runs<POW2>(px, py, pz, pm, nrem, d, inv_dx, qscale, bx, status, lane, large);
    else
      large = dep_warp_direct<POW2>(x, y, z, m, wb, nrem, d, inv_dx, qscale, qg, status, lane);
    while (large) {  // rare: point masses
      const int j = __ffs(large) - 1;
      large &= large - 1;
      const long long p = wb + 32 * j;
      const float gx = POW2 ? __fmul_rn(x[p], inv_dx) : __fdiv_rn(x[p], d.dx);
      const float gy = POW2 ? __fmul_rn(y[p], inv_dx) : __fdiv_rn(y[p], d.dx);
      const float gz = POW2 ? __fmul_rn(z[p], inv_dx) : __fdiv_rn(z[p], d.dx);
      const int ix = __float2int_rd(gx), iy = __float2int_rd(gy), iz = __float2int_rd(gz);
      large_to_grid(qg, d.G, ix, iy, iz, __fmul_rn(m[p], d.inv_vol), __fsub_rn(gx, __int2float_rn(ix)),
                    __fsub_rn(gy, __int2float_rn(iy)), __fsub_rn(gz, __int2float_rn(iz)), qscale);
    }
    if (use_box) {
      __syncwarp();
      // the warp's box to the grid, one atomic per nonzero node; zeroed as read.
      // Node coordinates by correctly rounded reciprocals instead of integer
      // divisions: for i < 2^10 the product (i + 1/2) * (1/nyz) is off by less
      // than the distance to the next integer, so truncating it is the quotient.
      const int vol = nx * bx.nyz;
      const float inv_nyz = __frcp_rn((float)bx.nyz), inv_nz = __frcp_rn((float)bx.nz);
      for (int i = lane; i < vol; i += 32) {
        const int v = wbox[i];
        if (v == 0) continue;
        wbox[i] = 0;
        const int rx = (int)(((float)i + 0.5f) * inv_nyz), rem = i - rx * bx.nyz;
        const int ry = (int)(((float)rem + 0.5f) * inv_nz), rz = rem - ry * bx.nz;
        const int jx = bx.x0 + rx, jy = bx.y0 + ry, jz = bx.z0 + rz;
        if ((unsigned)jx < (unsigned)d.G && (unsigned)jy < (unsigned)d.G && (unsigned)jz < (unsigned)d.G)
          atomicAdd((unsigned long long *)(qg + ((size_t)jx * d.G + jy) * d.G + jz), (unsigned long long)(long long)v);
      }
      __syncwarp();
    }
  }
}

int gc_deposit_q(gc_ctx *ctx, const float *x, const float *y, const float *z, const float *m, int64_t n,
                 const double *qexp) {
  if (n <= 0) return GC_OK;
  DepCtx d;
  d.dx = (float)ctx->dx;
  d.inv_vol = 1.0f / ((d.dx * d.dx) * d.dx);
  d.G = ctx->G;
  const long long ntiles = (n + DEP_TILE - 1) / DEP_TILE;
  const unsigned nb = (unsigned)(ntiles < (long long)gc_sms() * 4 ? ntiles : (long long)gc_sms() * 4);  // 4 CTAs per SM, persistent
  int fe = 0;
  const bool pow2 = std::frexp(d.dx, &fe) == 0.5f;
  const float inv_dx = pow2 ? std::ldexp(1.0f, 1 - fe) : 0.0f;
  if (pow2)
    gc_launch(ctx, GK_DEPOSIT_RUNS, k_deposit_sorted<true>, dim3(nb), dim3(256), 0, x, y, z, m, (long long)n, d,
              inv_dx, qexp, ctx->q, ctx->dstatus);
  else
    gc_launch(ctx, GK_DEPOSIT_RUNS, k_deposit_sorted<false>, dim3(nb), dim3(256), 0, x, y, z, m, (long long)n, d,
              inv_dx, qexp, ctx->q, ctx->dstatus);
  GC_LAUNCH_CHECK(ctx, "deposit");
  return GC_OK;
}

// ------------------------------------------------------------------------------
// q -> rho / b, zero q, exact integer column moments, ||b||^2
// ------------------------------------------------------------------------------
// One warp per (i,j) column, persistent over the columns. Column sums S0 = sum q,
// S1 = sum q k and S2 = sum q k^2 are exact in integers (S2 split at bit 32),
// combined across columns in FP64 in a fixed order. Partials per block: 10
// moments + ||b||^2.
__global__ void __launch_bounds__(256)
    k_convert_q(long long *__restrict__ qg, int G, double dx, const double *__restrict__ qexp, float *__restrict__ rho,
                float *__restrict__ b, double bfac, double *__restrict__ parts, unsigned *__restrict__ ticket,
                double *__restrict__ mom, double *__restrict__ bnorm2) {
  __shared__ double wsum[8][11];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int E = (int)(*qexp);
  const float qinv = ldexpf(1.0f, E);
  const float bscale = (float)(ldexp(1.0, E) * bfac);
  const double msc = ldexp(1.0, E) * dx * dx * dx;  // mass of one quantum
  double v[11];
#pragma unroll
  for (int t = 0; t < 11; ++t) v[t] = 0.0;
  const long long ncols = (long long)G * G;
  for (long long col = (long long)blockIdx.x * 8 + wid; col < ncols; col += (long long)gridDim.x * 8) {
    const int i = (int)(col / G), j = (int)(col - (long long)i * G);
    long long *p = qg + (size_t)col * G;
    float *rp = rho ? rho + (size_t)col * G : nullptr;
    float *bp = b ? b + (size_t)col * G : nullptr;
    long long S0 = 0, S1 = 0, S2h = 0;
    unsigned long long S2l = 0;
    float bb = 0.0f;
    for (int k0 = 0; k0 < G; k0 += 32 * 8) {
      long long qv[8];
      bool nz = false;
#pragma unroll
      for (int t = 0; t < 8; ++t) {  // all loads of the lane in flight together
        const int k = k0 + 32 * t + lane;
        qv[t] = k < G ? p[k] : 0;
        nz |= qv[t] != 0;
      }
      if (!__any_sync(0xffffffffu, nz)) {  // an empty stretch (most of a disk's box): zeros out, q stays 0
#pragma unroll
        for (int t = 0; t < 8; ++t) {
          const int k = k0 + 32 * t + lane;
          if (k >= G) continue;
          if (rp) rp[k] = 0.0f;
          if (bp) bp[k] = 0.0f;
        }
        continue;
      }
#pragma unroll
      for (int t = 0; t < 8; ++t) {
        const int k = k0 + 32 * t + lane;
        if (k >= G) continue;
        if (qv[t] != 0) p[k] = 0;  // clear for the next deposit (zeros need no store)
        const float qf = i64_to_f32_rn(qv[t]);  // one rounding, as (float)q
        if (rp) rp[k] = __fmul_rn(qf, qinv);
        const float bv = __fmul_rn(qf, bscale);
        if (bp) bp[k] = bv;
        bb += bv * bv;
        const long long kk = k;
        S0 += qv[t];
        S1 += qv[t] * kk;
        S2h += (qv[t] >> 32) * (kk * kk);
        S2l += (unsigned long long)(qv[t] & 0xffffffffLL) * (unsigned long long)(kk * kk);
      }
    }
    // exact integer warp sums (no FP64 per lane)
    for (int o = 16; o > 0; o >>= 1) {
      S0 += __shfl_down_sync(0xffffffffu, S0, o);
      S1 += __shfl_down_sync(0xffffffffu, S1, o);
      S2h += __shfl_down_sync(0xffffffffu, S2h, o);
      S2l += __shfl_down_sync(0xffffffffu, S2l, o);
      bb += __shfl_down_sync(0xffffffffu, bb, o);
    }
    if (lane == 0) v[10] += (double)bb;
    if (lane == 0 && (S0 | S1 | S2h | (long long)S2l) != 0) {
      const double d0 = (double)S0, d1 = (double)S1, d2 = (double)S2h * 4294967296.0 + (double)S2l;
      const double x = i * dx, y = j * dx;
      const double m0 = d0 * msc, m1 = d1 * msc * dx, m2 = d2 * msc * dx * dx;
      v[0] += m0; v[1] += m0 * x; v[2] += m0 * y; v[3] += m1;
      v[4] += m0 * x * x; v[5] += m0 * y * y; v[6] += m2;
      v[7] += m0 * x * y; v[8] += m1 * x; v[9] += m1 * y;
    }
  }
  // lane 0 of each warp holds the warp's totals: sum the 8 warps in order
  if (lane == 0) {
#pragma unroll
    for (int t = 0; t < 11; ++t) wsum[wid][t] = v[t];
  }
  __syncthreads();
  if (threadIdx.x == 0) {  // one writer: the last-block reduction below fences its stores
#pragma unroll 1
    for (int t = 0; t < 11; ++t) {
      double a = 0.0;
      for (int w = 0; w < 8; ++w) a += wsum[w][t];
      parts[(size_t)blockIdx.x * 11 + t] = a;
    }
  }
  // the moments and ||b||^2 from the block partials by the last block
  if (ticket && grid_finish_sum<11>(parts, gridDim.x, ticket, mom) && threadIdx.x == 0) *bnorm2 = mom[10];
}

int gc_max_fixed_point_bits(const gc_ctx *ctx) {
  int lg = 0;
  while ((1 << lg) < ctx->G) ++lg;
  const int b = 62 - lg;
  return b > 60 ? 60 : b;
}

int gc_convert_q(gc_ctx *ctx, const double *qexp, float *rho_out, float *b_out) {
  const long long cols = (long long)ctx->G * ctx->G;
  unsigned nb = gc_blocks(cols, 8);
  if (nb > gc_sms() * 3u) nb = gc_sms() * 3u;  // persistent: 3 CTAs per SM (80 registers)
  int s = gc_ensure_red(ctx, (size_t)nb * 11);
  if (s) return s;
  const double bfac = 4.0 * M_PI * ctx->grav * ctx->dx * ctx->dx;
  gc_launch(ctx, GK_CONVERT_Q, k_convert_q, dim3(nb), dim3(256), 0, ctx->q, ctx->G, ctx->dx, qexp, rho_out, b_out,
            bfac, ctx->red, reinterpret_cast<unsigned *>(ctx->dsmall + GC_S_TICKET), ctx->dmom,
            ctx->dsmall + GC_S_BNORM2);
  GC_LAUNCH_CHECK(ctx, "convert q");
  return GC_OK;
}

extern "C" int gc_deposit_cic(gc_ctx *ctx, const float *x, const float *y, const float *z, const float *m, int64_t n,
                              int fixed_point_bits, float *rho) {
  if (!ctx) return GC_ERR_ARG;
  GC_REQUIRE(ctx, rho, "gc_deposit_cic: NULL rho");
  GC_REQUIRE(ctx, n >= 0 && n < (1LL << 31), "particle count out of range: %lld", (long long)n);
  GC_REQUIRE(ctx, n == 0 || (x && y && z && m), "gc_deposit_cic: NULL particle array");
  GC_REQUIRE(ctx, fixed_point_bits >= 24 && fixed_point_bits <= gc_max_fixed_point_bits(ctx),
             "fixed_point_bits must be in [24, %d] for a %d^3 grid", gc_max_fixed_point_bits(ctx), ctx->G);
  int s;
  if (n > 0) {
    if ((s = gc_fixed_point_setup(ctx, m, n, fixed_point_bits, GC_S_MASS, GC_S_QEXP))) return s;
    if ((s = gc_deposit_q(ctx, x, y, z, m, n, ctx->dsmall + GC_S_QEXP))) return s;
  }
  return gc_convert_q(ctx, ctx->dsmall + GC_S_QEXP, rho, nullptr);
}

// ------------------------------------------------------------------------------
// gradient (deposit.py:132-174)
// ------------------------------------------------------------------------------
__device__ __forceinline__ float grad_comp(const float *__restrict__ phi, size_t c, size_t stride, int idx, int G,
                                           float inv_dx, float inv_2dx) {
  if (idx == 0) return -__fmul_rn(__fsub_rn(phi[c + stride], phi[c]), inv_dx);
  if (idx == G - 1) return -__fmul_rn(__fsub_rn(phi[c], phi[c - stride]), inv_dx);
  return -__fmul_rn(__fsub_rn(phi[c + stride], phi[c - stride]), inv_2dx);
}

struct GradCtx {
  int G;
  float inv_dx, inv_2dx;
};

__host__ static GradCtx make_grad(const gc_ctx *ctx) {
  GradCtx g;
  g.G = ctx->G;
  const float dx = (float)ctx->dx;
  g.inv_dx = 1.0f / dx;
  g.inv_2dx = 1.0f / (2.0f * dx);
  return g;
}

__global__ void __launch_bounds__(256)
    k_grad(const float *__restrict__ phi, float *__restrict__ ax, float *__restrict__ ay, float *__restrict__ az,
           GradCtx g) {
  const int k = blockIdx.x * 32 + threadIdx.x;
  const int j = blockIdx.y * 8 + threadIdx.y;
  const int i = blockIdx.z;
  if (k >= g.G || j >= g.G) return;
  const size_t G = g.G;
  const size_t c = ((size_t)i * G + j) * G + k;
  ax[c] = grad_comp(phi, c, G * G, i, g.G, g.inv_dx, g.inv_2dx);
  ay[c] = grad_comp(phi, c, G, j, g.G, g.inv_dx, g.inv_2dx);
  az[c] = grad_comp(phi, c, 1, k, g.G, g.inv_dx, g.inv_2dx);
}

extern "C" int gc_potential_to_accel(gc_ctx *ctx, const float *phi, float *ax, float *ay, float *az) {
  if (!ctx) return GC_ERR_ARG;
  GC_REQUIRE(ctx, phi && ax && ay && az, "gc_potential_to_accel: NULL pointer");
  const GradCtx g = make_grad(ctx);
  gc_launch(ctx, GK_GRAD, k_grad, dim3(dim3(gc_blocks(g.G, 32), gc_blocks(g.G, 8), g.G)), dim3(dim3(32, 8)), 0, phi, ax, ay, az, g);
  GC_LAUNCH_CHECK(ctx, "grad");
  return GC_OK;
}

// ------------------------------------------------------------------------------
// gather (deposit.py:85-129)
// ------------------------------------------------------------------------------
__global__ void __launch_bounds__(256)
    k_gather(const float *__restrict__ x, const float *__restrict__ y, const float *__restrict__ z, long long n,
             const float *__restrict__ axg, const float *__restrict__ ayg, const float *__restrict__ azg,
             float *__restrict__ ax, float *__restrict__ ay, float *__restrict__ az, float dx, int G) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    float sx = 0.0f, sy = 0.0f, sz = 0.0f;
    CellPos c;
    if (gc_cell_of(x[p], y[p], z[p], dx, G, c)) {
      const float wx[2] = {__fsub_rn(1.0f, c.fx), c.fx};
      const float wy[2] = {__fsub_rn(1.0f, c.fy), c.fy};
      const float wz[2] = {__fsub_rn(1.0f, c.fz), c.fz};
#pragma unroll
      for (int cx = 0; cx < 2; ++cx)
#pragma unroll
        for (int cy = 0; cy < 2; ++cy)
#pragma unroll
          for (int cz = 0; cz < 2; ++cz) {
            const int jx = c.ix + cx, jy = c.iy + cy, jz = c.iz + cz;
            if ((unsigned)jx < (unsigned)G && (unsigned)jy < (unsigned)G && (unsigned)jz < (unsigned)G) {
              const float w = __fmul_rn(__fmul_rn(wx[cx], wy[cy]), wz[cz]);
              const size_t idx = ((size_t)jx * G + jy) * G + jz;
              sx = __fadd_rn(sx, __fmul_rn(w, axg[idx]));
              sy = __fadd_rn(sy, __fmul_rn(w, ayg[idx]));
              sz = __fadd_rn(sz, __fmul_rn(w, azg[idx]));
            }
          }
    }
    ax[p] = sx;
    ay[p] = sy;
    az[p] = sz;
  }
}

extern "C" int gc_gather_accel(gc_ctx *ctx, const float *x, const float *y, const float *z, int64_t n,
                               const float *ax_g, const float *ay_g, const float *az_g, float *acc_x, float *acc_y,
                               float *acc_z) {
  if (!ctx) return GC_ERR_ARG;
  GC_REQUIRE(ctx, n >= 0 && n < (1LL << 31), "particle count out of range");
  if (n == 0) return GC_OK;
  GC_REQUIRE(ctx, x && y && z && ax_g && ay_g && az_g && acc_x && acc_y && acc_z, "gc_gather_accel: NULL pointer");
  unsigned nb = gc_blocks(n, 256);
  if (nb > gc_sms() * 32u) nb = gc_sms() * 32u;
  gc_launch(ctx, GK_GATHER, k_gather, dim3(nb), dim3(256), 0, x, y, z, (long long)n, ax_g, ay_g, az_g, acc_x, acc_y, acc_z,
                                        (float)ctx->dx, ctx->G);
  GC_LAUNCH_CHECK(ctx, "gather");
  return GC_OK;
}

// ------------------------------------------------------------------------------
// kick / drift (integrator.py:27-59)
// ------------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_axpy3(float *__restrict__ u, float *__restrict__ v, float *__restrict__ w,
                                               const float *__restrict__ a, const float *__restrict__ b,
                                               const float *__restrict__ c, long long n, float dt) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    u[p] = __fadd_rn(u[p], __fmul_rn(a[p], dt));
    v[p] = __fadd_rn(v[p], __fmul_rn(b[p], dt));
    w[p] = __fadd_rn(w[p], __fmul_rn(c[p], dt));
  }
}

static int axpy3(gc_ctx *ctx, float *u, float *v, float *w, const float *a, const float *b, const float *c,
                 int64_t n, float dt, const char *what) {
  GC_REQUIRE(ctx, n >= 0 && n < (1LL << 31), "particle count out of range");
  if (n == 0) return GC_OK;
  GC_REQUIRE(ctx, u && v && w && a && b && c, "%s: NULL pointer", what);
  unsigned nb = gc_blocks(n, 256);
  if (nb > gc_sms() * 32u) nb = gc_sms() * 32u;
  gc_launch(ctx, GK_AXPY, k_axpy3, dim3(nb), dim3(256), 0, u, v, w, a, b, c, (long long)n, dt);
  GC_LAUNCH_CHECK(ctx, what);
  return GC_OK;
}

extern "C" int gc_kick(gc_ctx *ctx, float *vx, float *vy, float *vz, const float *ax, const float *ay, const float *az,
                       int64_t n, float dt) {
  if (!ctx) return GC_ERR_ARG;
  return axpy3(ctx, vx, vy, vz, ax, ay, az, n, dt, "kick");
}

extern "C" int gc_drift(gc_ctx *ctx, float *px, float *py, float *pz, const float *vx, const float *vy,
                        const float *vz, int64_t n, float dt) {
  if (!ctx) return GC_ERR_ARG;
  return axpy3(ctx, px, py, pz, vx, vy, vz, n, dt, "drift");
}

// ------------------------------------------------------------------------------
// fused: gather of -grad(phi) computed on the fly + KDK kicks + drift
// ------------------------------------------------------------------------------
struct FusedCtx {
  float dx, inv_dx, inv_2dx;
  int G;
  float h, dt;
  int mode;
  int diag;
};

// Acceleration at a particle: the CIC gather of the node field g = -grad(phi),
// each node's g formed exactly as _potential_to_accel does (deposit.py:148-174).
__device__ __forceinline__ void gather_grad(const float *__restrict__ phi, float x, float y, float z,
                                            const FusedCtx &f, float &ax, float &ay, float &az) {
  ax = ay = az = 0.0f;
  CellPos c;
  if (!gc_cell_of(x, y, z, f.dx, f.G, c)) return;
  const int G = f.G;
  const size_t sG = (size_t)G;
  const float wx[2] = {__fsub_rn(1.0f, c.fx), c.fx};
  const float wy[2] = {__fsub_rn(1.0f, c.fy), c.fy};
  const float wz[2] = {__fsub_rn(1.0f, c.fz), c.fz};
#pragma unroll
  for (int cx = 0; cx < 2; ++cx)
#pragma unroll
    for (int cy = 0; cy < 2; ++cy)
#pragma unroll
      for (int cz = 0; cz < 2; ++cz) {
        const int jx = c.ix + cx, jy = c.iy + cy, jz = c.iz + cz;
        if ((unsigned)jx < (unsigned)G && (unsigned)jy < (unsigned)G && (unsigned)jz < (unsigned)G) {
          const size_t idx = ((size_t)jx * sG + jy) * sG + jz;
          const float gx = grad_comp(phi, idx, sG * sG, jx, G, f.inv_dx, f.inv_2dx);
          const float gy = grad_comp(phi, idx, sG, jy, G, f.inv_dx, f.inv_2dx);
          const float gz = grad_comp(phi, idx, 1, jz, G, f.inv_dx, f.inv_2dx);
          const float w = __fmul_rn(__fmul_rn(wx[cx], wy[cy]), wz[cz]);
          ax = __fadd_rn(ax, __fmul_rn(w, gx));
          ay = __fadd_rn(ay, __fmul_rn(w, gy));
          az = __fadd_rn(az, __fmul_rn(w, gz));
        }
      }
}

// Per-thread diagnostic sums (diagnostics_device.py:56-74: M, KE, P, L, M x) in
// double-float: every product of f32 state is formed exactly (TwoProduct with an
// FMA) or to ~2^-46, and accumulated as an unevaluated sum hi + lo (Knuth's
// TwoSum), all in FP32 instructions; the per-thread totals go to FP64 for the
// block and grid reductions. FP64 arithmetic per particle would run at a small
// fraction of the FP32 rate on this part (it cost ~4 ms per 100M particles).
struct DiagAcc {
  float h[11], l[11];
  __device__ __forceinline__ void zero() {
#pragma unroll
    for (int t = 0; t < 11; ++t) h[t] = l[t] = 0.0f;
  }
  // exact a*b = p + e
  static __device__ __forceinline__ void tp(float a, float b, float &p, float &e) {
    p = __fmul_rn(a, b);
    e = __fmaf_rn(a, b, -p);
  }
  // exact a+b = s + e
  static __device__ __forceinline__ void ts(float a, float b, float &s, float &e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  }
  __device__ __forceinline__ void add(int t, float ph, float pl) {
    float s, e;
    ts(h[t], ph, s, e);
    h[t] = s;
    l[t] = __fadd_rn(l[t], __fadd_rn(e, pl));
  }
  // m (a*b - c*d) to ~2^-46 relative
  static __device__ __forceinline__ void cross(float m, float a, float b, float c, float d, float &q, float &ql) {
    float p1, e1, p2, e2, s, r, qe;
    tp(a, b, p1, e1);
    tp(c, d, p2, e2);
    ts(p1, -p2, s, r);
    const float sl = __fadd_rn(r, __fsub_rn(e1, e2));
    tp(s, m, q, qe);
    ql = __fmaf_rn(sl, m, qe);
  }
  __device__ __forceinline__ void particle(float m, float X, float Y, float Z, float VX, float VY, float VZ) {
    float p, e, q, ql;
    add(0, m, 0.0f);
    {  // 0.5 m |v|^2
      float a1, e1, a2, e2, a3, e3, s1, r1, s2, r2, qe;
      tp(VX, VX, a1, e1);
      tp(VY, VY, a2, e2);
      tp(VZ, VZ, a3, e3);
      ts(a1, a2, s1, r1);
      ts(s1, a3, s2, r2);
      const float sl = __fadd_rn(__fadd_rn(__fadd_rn(e1, e2), e3), __fadd_rn(r1, r2));
      tp(s2, m, q, qe);
      ql = __fmaf_rn(sl, m, qe);
      add(1, __fmul_rn(0.5f, q), __fmul_rn(0.5f, ql));
    }
    tp(m, VX, p, e); add(2, p, e);
    tp(m, VY, p, e); add(3, p, e);
    tp(m, VZ, p, e); add(4, p, e);
    cross(m, Y, VZ, Z, VY, q, ql); add(5, q, ql);
    cross(m, Z, VX, X, VZ, q, ql); add(6, q, ql);
    cross(m, X, VY, Y, VX, q, ql); add(7, q, ql);
    tp(m, X, p, e); add(8, p, e);
    tp(m, Y, p, e); add(9, p, e);
    tp(m, Z, p, e); add(10, p, e);
  }
  __device__ __forceinline__ void to_double(double (&dv)[11]) const {
#pragma unroll
    for (int t = 0; t < 11; ++t) dv[t] = (double)h[t] + (double)l[t];
  }
};

template <bool DIAG>
__global__ void __launch_bounds__(256)
    k_gather_kick_drift(float *__restrict__ x, float *__restrict__ y, float *__restrict__ z, float *__restrict__ vx,
                        float *__restrict__ vy, float *__restrict__ vz, const float *__restrict__ m, long long n,
                        const float *__restrict__ phi, FusedCtx f, float *__restrict__ axo, float *__restrict__ ayo,
                        float *__restrict__ azo, double *__restrict__ parts) {
  DiagAcc acc;
  acc.zero();
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    float px = x[p], py = y[p], pz = z[p];
    float ux = vx[p], uy = vy[p], uz = vz[p];
    float ax, ay, az;
    gather_grad(phi, px, py, pz, f, ax, ay, az);
    if (axo) {
      axo[p] = ax;
      ayo[p] = ay;
      azo[p] = az;
    }
    if (f.mode != GC_STEP_PRIME) {  // closing half-kick of the previous step (integrator.py:131)
      ux = __fadd_rn(ux, __fmul_rn(ax, f.h));
      uy = __fadd_rn(uy, __fmul_rn(ay, f.h));
      uz = __fadd_rn(uz, __fmul_rn(az, f.h));
    }
    if (DIAG) {  // synchronised state (diagnostics_device.py:56-74)
      acc.particle(m[p], px, py, pz, ux, uy, uz);
    }
    if (f.mode != GC_STEP_CLOSE) {  // opening half-kick + drift (integrator.py:128-129)
      ux = __fadd_rn(ux, __fmul_rn(ax, f.h));
      uy = __fadd_rn(uy, __fmul_rn(ay, f.h));
      uz = __fadd_rn(uz, __fmul_rn(az, f.h));
      x[p] = __fadd_rn(px, __fmul_rn(ux, f.dt));
      y[p] = __fadd_rn(py, __fmul_rn(uy, f.dt));
      z[p] = __fadd_rn(pz, __fmul_rn(uz, f.dt));
    }
    vx[p] = ux;
    vy[p] = uy;
    vz[p] = uz;
  }
  if (DIAG) {
    double dv[11];
    acc.to_double(dv);
    block_partials<11>(dv, parts + (size_t)blockIdx.x * 11);
  }
}

// Variant with the node field g = -grad(phi) precomputed as float4 (x, y, z, 0):
// one pass over phi writes it (k_grad4), then each particle reads its 8 corner
// nodes with one 16-byte load each. Same arithmetic as gather_grad.
__global__ void __launch_bounds__(256) k_grad4(const float *__restrict__ phi, float4 *__restrict__ g4, GradCtx g) {
  const int k = blockIdx.x * 32 + threadIdx.x;
  const int j = blockIdx.y * 8 + threadIdx.y;
  const int i = blockIdx.z;
  if (k >= g.G || j >= g.G) return;
  const size_t G = g.G;
  const size_t c = ((size_t)i * G + j) * G + k;
  g4[c] = make_float4(grad_comp(phi, c, G * G, i, g.G, g.inv_dx, g.inv_2dx),
                      grad_comp(phi, c, G, j, g.G, g.inv_dx, g.inv_2dx),
                      grad_comp(phi, c, 1, k, g.G, g.inv_dx, g.inv_2dx), 0.0f);
}

template <bool POW2>
__device__ __forceinline__ void gather_g4(const float4 *__restrict__ g4, float x, float y, float z, const FusedCtx &f,
                                          float &ax, float &ay, float &az) {
  ax = ay = az = 0.0f;
  CellPos c;
  if (POW2) {  // x / dx == x * (1/dx) exactly when dx is a power of two
    const float gx = __fmul_rn(x, f.inv_dx), gy = __fmul_rn(y, f.inv_dx), gz = __fmul_rn(z, f.inv_dx);
    const float hi = (float)f.G;
    if (!(gx >= -1.0f && gx < hi && gy >= -1.0f && gy < hi && gz >= -1.0f && gz < hi)) return;
    const float flx = floorf(gx), fly = floorf(gy), flz = floorf(gz);
    c.ix = (int)flx; c.iy = (int)fly; c.iz = (int)flz;
    c.fx = __fsub_rn(gx, flx); c.fy = __fsub_rn(gy, fly); c.fz = __fsub_rn(gz, flz);
  } else if (!gc_cell_of(x, y, z, f.dx, f.G, c)) {
    return;
  }
  const int G = f.G;
  const float wx[2] = {__fsub_rn(1.0f, c.fx), c.fx};
  const float wy[2] = {__fsub_rn(1.0f, c.fy), c.fy};
  const float wz[2] = {__fsub_rn(1.0f, c.fz), c.fz};
  const bool interior = c.ix >= 0 && c.iy >= 0 && c.iz >= 0 && c.ix + 1 < G && c.iy + 1 < G && c.iz + 1 < G;
  const int base = (c.ix * G + c.iy) * G + c.iz;  // G^3 < 2^31 (G <= 1024)
#pragma unroll
  for (int cx = 0; cx < 2; ++cx)
#pragma unroll
    for (int cy = 0; cy < 2; ++cy)
#pragma unroll
      for (int cz = 0; cz < 2; ++cz) {
        const int jx = c.ix + cx, jy = c.iy + cy, jz = c.iz + cz;
        if (interior || ((unsigned)jx < (unsigned)G && (unsigned)jy < (unsigned)G && (unsigned)jz < (unsigned)G)) {
          const float4 gv = __ldg(g4 + base + (cx * G + cy) * G + cz);
          const float w = __fmul_rn(__fmul_rn(wx[cx], wy[cy]), wz[cz]);
          ax = __fadd_rn(ax, __fmul_rn(w, gv.x));
          ay = __fadd_rn(ay, __fmul_rn(w, gv.y));
          az = __fadd_rn(az, __fmul_rn(w, gv.z));
        }
      }
}

// One particle of the fused pass (closing half-kick, diagnostics, opening
// half-kick, drift) given its acceleration; writes back x, v.
template <bool DIAG>
__device__ __forceinline__ void kd_update(long long p, float px, float py, float pz, float ux, float uy, float uz,
                                          float ax, float ay, float az, float *__restrict__ x, float *__restrict__ y,
                                          float *__restrict__ z, float *__restrict__ vx, float *__restrict__ vy,
                                          float *__restrict__ vz, const float *__restrict__ m, const FusedCtx &f,
                                          DiagAcc &acc) {
  if (f.mode != GC_STEP_PRIME) {
    ux = __fadd_rn(ux, __fmul_rn(ax, f.h));
    uy = __fadd_rn(uy, __fmul_rn(ay, f.h));
    uz = __fadd_rn(uz, __fmul_rn(az, f.h));
  }
  if (DIAG) {
    acc.particle(m[p], px, py, pz, ux, uy, uz);
  }
  if (f.mode != GC_STEP_CLOSE) {
    ux = __fadd_rn(ux, __fmul_rn(ax, f.h));
    uy = __fadd_rn(uy, __fmul_rn(ay, f.h));
    uz = __fadd_rn(uz, __fmul_rn(az, f.h));
    x[p] = __fadd_rn(px, __fmul_rn(ux, f.dt));
    y[p] = __fadd_rn(py, __fmul_rn(uy, f.dt));
    z[p] = __fadd_rn(pz, __fmul_rn(uz, f.dt));
  }
  vx[p] = ux;
  vy[p] = uy;
  vz[p] = uz;
}

template <bool DIAG, bool POW2>
__global__ void __launch_bounds__(256)
    k_gather4_kick_drift(float *__restrict__ x, float *__restrict__ y, float *__restrict__ z, float *__restrict__ vx,
                         float *__restrict__ vy, float *__restrict__ vz, const float *__restrict__ m, long long n,
                         const float4 *__restrict__ g4, FusedCtx f, double *__restrict__ parts) {
  DiagAcc acc;
  acc.zero();
  // software pipelined: the next particle's state is loaded before this one's
  // corner gather, so its DRAM latency overlaps the gather's L2 latency
  const long long stride = (long long)gridDim.x * blockDim.x;
  long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  float nx = 0.0f, ny = 0.0f, nz = 0.0f, nvx = 0.0f, nvy = 0.0f, nvz = 0.0f;
  if (p < n) { nx = x[p]; ny = y[p]; nz = z[p]; nvx = vx[p]; nvy = vy[p]; nvz = vz[p]; }
  for (; p < n; p += stride) {
    const float px = nx, py = ny, pz = nz, ux = nvx, uy = nvy, uz = nvz;
    const long long q = p + stride;
    if (q < n) { nx = x[q]; ny = y[q]; nz = z[q]; nvx = vx[q]; nvy = vy[q]; nvz = vz[q]; }
    float ax, ay, az;
    gather_g4<POW2>(g4, px, py, pz, f, ax, ay, az);
    kd_update<DIAG>(p, px, py, pz, ux, uy, uz, ax, ay, az, x, y, z, vx, vy, vz, m, f, acc);
  }
  if (DIAG) {
    double dv[11];
    acc.to_double(dv);
    block_partials<11>(dv, parts + (size_t)blockIdx.x * 11);
  }
}

// The same particle pass with the particle state streamed by the TMA engine: a
// CTA owns tiles of GT_TILE particles (round robin); one thread arms an
// mbarrier and issues 1-D bulk copies (x, y, z, vx, vy, vz, and m when
// depositing) of the next tile into the other half of a double buffer while all
// threads work on the current one, reading the state from shared memory,
// gathering the corners from the float4 grid, and writing the new state back in
// place; the tile then leaves with six bulk stores. The DRAM streams never wait
// for the gather's dependent loads.
//
// With DEP the pass also deposits the drifted positions (the next step's
// density) into the int64 grid while the stores drain: warp w takes the tile's
// particles [128 w, 128 w + 128) 32 at a time, exactly as k_deposit_sorted does
// (two full-warp reductions for the main cells, direct adds for the others, a
// per-warp shared-memory box), so the density is the one k_deposit_sorted
// would produce from the stored positions, bit for bit.
//
// Full tiles only; the remainder goes through plain loads (and per-particle
// deposits). Waits are bounded (clock budget): a timeout raises
// GC_FLAG_TIMEOUT and the CTA stops issuing.
#define GT_TILE 1024
#define GT_BUDGET 2000000000LL
#define GT_WBOX 512  // nodes of one warp's deposit box
// dynamic shared memory: two buffers of 7 arrays, the warps' boxes
#define GT_SMEM(dep) (2 * ((dep) ? 7 : 6) * GT_TILE * 4 + ((dep) ? 8 * GT_WBOX * 4 : 0))

template <bool POW2>
__device__ __forceinline__ void gt_particle(float *s0, float *s1, float *s2, float *s3, float *s4, float *s5, int i,
                                            const float4 *__restrict__ g4, const FusedCtx &f) {
  const float px = s0[i], py = s1[i], pz = s2[i];
  float ux = s3[i], uy = s4[i], uz = s5[i];
  float ax, ay, az;
  gather_g4<POW2>(g4, px, py, pz, f, ax, ay, az);
  if (f.mode != GC_STEP_PRIME) {
    ux = __fadd_rn(ux, __fmul_rn(ax, f.h));
    uy = __fadd_rn(uy, __fmul_rn(ay, f.h));
    uz = __fadd_rn(uz, __fmul_rn(az, f.h));
  }
  if (f.mode != GC_STEP_CLOSE) {
    ux = __fadd_rn(ux, __fmul_rn(ax, f.h));
    uy = __fadd_rn(uy, __fmul_rn(ay, f.h));
    uz = __fadd_rn(uz, __fmul_rn(az, f.h));
    s0[i] = __fadd_rn(px, __fmul_rn(ux, f.dt));
    s1[i] = __fadd_rn(py, __fmul_rn(uy, f.dt));
    s2[i] = __fadd_rn(pz, __fmul_rn(uz, f.dt));
  }
  s3[i] = ux;
  s4[i] = uy;
  s5[i] = uz;
}

// Deposit of 128 staged particles (warp-contiguous, the k_deposit_sorted rules)
// into the warp's box or the grid.
template <bool POW2>
__device__ __forceinline__ void gt_deposit_warp(const float *s0, const float *s1, const float *s2, const float *s6,
                                                int base, int *wbox, const DepCtx &d, float inv_dx, float qscale,
                                                long long *__restrict__ qg, unsigned *__restrict__ status, int lane) {
  float px[4], py[4], pz[4], pm[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int i = base + 32 * j + lane;
    px[j] = s0[i]; py[j] = s1[i]; pz[j] = s2[i]; pm[j] = s6[i];
  }
  DepBox bx;
  bx.b = wbox;
  bool use_box;
  int nx;
  {
    float xl = 3.0e38f, yl = 3.0e38f, zl = 3.0e38f, xh = -3.0e38f, yh = -3.0e38f, zh = -3.0e38f;
    unsigned mb = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      xl = fminf(xl, px[j]); xh = fmaxf(xh, px[j]);
      yl = fminf(yl, py[j]); yh = fmaxf(yh, py[j]);
      zl = fminf(zl, pz[j]); zh = fmaxf(zh, pz[j]);
      mb = max(mb, __float_as_uint(pm[j]) & 0x7fffffffu);
    }
    const float gl = -1.0f, gh = (float)d.G - 1.0f;
    const float cl[3] = {xl, yl, zl}, ch[3] = {xh, yh, zh};
    int lo[3], hi[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      float l = POW2 ? __fmul_rn(cl[a], inv_dx) : __fdiv_rn(cl[a], d.dx);
      float h = POW2 ? __fmul_rn(ch[a], inv_dx) : __fdiv_rn(ch[a], d.dx);
      l = fminf(fmaxf(floorf(l), gl), gh);
      h = fminf(fmaxf(floorf(h), gl), gh);
      const bool any_pt = cl[a] <= ch[a];
      lo[a] = __reduce_min_sync(0xffffffffu, any_pt ? (int)l : 0x7fffffff);
      hi[a] = __reduce_max_sync(0xffffffffu, any_pt ? (int)h : -0x7fffffff);
    }
    mb = __reduce_max_sync(0xffffffffu, mb);
    bx.x0 = lo[0]; bx.y0 = lo[1]; bx.z0 = lo[2];
    nx = hi[0] - lo[0] + 2;
    bx.ny = hi[1] - lo[1] + 2;
    bx.nz = hi[2] - lo[2] + 2;
    bx.nyz = bx.ny * bx.nz;
    const float mq = __fmul_rn(__fmul_rn(__uint_as_float(mb), d.inv_vol), qscale);
    use_box = hi[0] >= lo[0] && (long long)nx * bx.nyz <= GT_WBOX &&
              __fmul_rn(fminf(mq, 4194304.0f) + 1.0f, 128.0f) < 1073741824.0f;
  }
  unsigned large = 0;
  const long long nrem = 1LL << 40;  // all 128 particles exist
  if (use_box)
    dep_warp_pass<POW2, true, 4>(px, py, pz, pm, nrem, d, inv_dx, qscale, bx, qg, status, lane, large);
  else
    dep_warp_pass<POW2, false, 4>(px, py, pz, pm, nrem, d, inv_dx, qscale, bx, qg, status, lane, large);
  while (large) {  // rare: point masses
    const int j = __ffs(large) - 1;
    large &= large - 1;
    const int i = base + 32 * j + lane;
    const float gx = POW2 ? __fmul_rn(s0[i], inv_dx) : __fdiv_rn(s0[i], d.dx);
    const float gy = POW2 ? __fmul_rn(s1[i], inv_dx) : __fdiv_rn(s1[i], d.dx);
    const float gz = POW2 ? __fmul_rn(s2[i], inv_dx) : __fdiv_rn(s2[i], d.dx);
    const int ix = __float2int_rd(gx), iy = __float2int_rd(gy), iz = __float2int_rd(gz);
    large_to_grid(qg, d.G, ix, iy, iz, __fmul_rn(s6[i], d.inv_vol), __fsub_rn(gx, __int2float_rn(ix)),
                  __fsub_rn(gy, __int2float_rn(iy)), __fsub_rn(gz, __int2float_rn(iz)), qscale);
  }
  if (use_box) {
    __syncwarp();
    const int vol = nx * bx.nyz;
    for (int i = lane; i < vol; i += 32) {
      const int v = wbox[i];
      if (v == 0) continue;
      wbox[i] = 0;
      const int rx = i / bx.nyz, rem = i - rx * bx.nyz, ry = rem / bx.nz, rz = rem - ry * bx.nz;
      const int jx = bx.x0 + rx, jy = bx.y0 + ry, jz = bx.z0 + rz;
      if ((unsigned)jx < (unsigned)d.G && (unsigned)jy < (unsigned)d.G && (unsigned)jz < (unsigned)d.G)
        atomicAdd((unsigned long long *)(qg + ((size_t)jx * d.G + jy) * d.G + jz), (unsigned long long)(long long)v);
    }
    __syncwarp();
  }
}

// One particle of the remainder: its corners straight to the grid.
template <bool POW2>
__device__ __forceinline__ void gt_deposit_one(float px, float py, float pz, float pm, const DepCtx &d, float inv_dx,
                                               float qscale, long long *__restrict__ qg,
                                               unsigned *__restrict__ status) {
  float gx, gy, gz;
  if (POW2) {
    gx = __fmul_rn(px, inv_dx); gy = __fmul_rn(py, inv_dx); gz = __fmul_rn(pz, inv_dx);
  } else {
    gx = __fdiv_rn(px, d.dx); gy = __fdiv_rn(py, d.dx); gz = __fdiv_rn(pz, d.dx);
  }
  const float hi = (float)d.G;
  if (!(gx >= -1.0f && gx < hi && gy >= -1.0f && gy < hi && gz >= -1.0f && gz < hi)) {
    if (!gc_finite3(px, py, pz)) atomicOr(status, GC_FLAG_NONFINITE_POS);
    return;
  }
  const int ix = __float2int_rd(gx), iy = __float2int_rd(gy), iz = __float2int_rd(gz);
  const float fx = __fsub_rn(gx, __int2float_rn(ix)), fy = __fsub_rn(gy, __int2float_rn(iy)),
              fz = __fsub_rn(gz, __int2float_rn(iz));
  large_to_grid(qg, d.G, ix, iy, iz, __fmul_rn(pm, d.inv_vol), fx, fy, fz, qscale);
}

template <bool POW2, bool DEP>
__global__ void __launch_bounds__(256)
    k_gather4_tma(float *__restrict__ x, float *__restrict__ y, float *__restrict__ z, float *__restrict__ vx,
                  float *__restrict__ vy, float *__restrict__ vz, const float *__restrict__ m, long long n,
                  const float4 *__restrict__ g4, FusedCtx f, DepCtx d, float inv_dx, const double *__restrict__ qexp,
                  long long *__restrict__ qg, unsigned *__restrict__ status) {
  using namespace umma;
  constexpr int NA = DEP ? 7 : 6;
  extern __shared__ __align__(128) float gt_smem[];
  float *buf = gt_smem;                               // [2][NA][GT_TILE]
  int *wboxes = reinterpret_cast<int *>(gt_smem + 2 * NA * GT_TILE);  // [8][GT_WBOX] when DEP
  __shared__ __align__(8) uint64_t bar[2];
  const float *src[7] = {x, y, z, vx, vy, vz, m};
  float *const dst[6] = {x, y, z, vx, vy, vz};
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const long long ntiles = n / GT_TILE;
  const float qscale = DEP ? ldexpf(1.0f, -(int)(*qexp)) : 1.0f;
  if (DEP)
    for (int i = tid; i < 8 * GT_WBOX; i += 256) wboxes[i] = 0;  // every flush zeroes what it read
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  const uint32_t tile_bytes = GT_TILE * 4;
  long long t = blockIdx.x;
  if (tid == 0 && t < ntiles) {
    mbar_arrive_expect_tx(&bar[0], NA * tile_bytes);
#pragma unroll
    for (int a = 0; a < NA; ++a) bulk_g2s(buf + a * GT_TILE, src[a] + t * GT_TILE, tile_bytes, &bar[0]);
  }
  for (int it = 0; t < ntiles; ++it, t += gridDim.x) {
    const int b = it & 1;
    float *cur = buf + b * NA * GT_TILE, *nxt = buf + (b ^ 1) * NA * GT_TILE;
    const long long tn = t + gridDim.x;
    if (tid == 0 && tn < ntiles) {  // prefetch the next tile into the other buffer
      bulk_wait_read_all();          // its previous tile's stores have read it
      mbar_arrive_expect_tx(&bar[b ^ 1], NA * tile_bytes);
#pragma unroll
      for (int a = 0; a < NA; ++a) bulk_g2s(nxt + a * GT_TILE, src[a] + tn * GT_TILE, tile_bytes, &bar[b ^ 1]);
    }
    const bool got = mbar_wait(&bar[b], (uint32_t)(it >> 1) & 1u, GT_BUDGET);
    if (!__syncthreads_and(got)) {  // the block leaves together
      if (tid == 0) {  // record it, and give the copies still in flight a bounded time to land
        atomicOr(status, GC_FLAG_TIMEOUT);
        mbar_wait(&bar[b], (uint32_t)(it >> 1) & 1u, GT_BUDGET);
        if (tn < ntiles) mbar_wait(&bar[b ^ 1], (uint32_t)((it + 1) >> 1) & 1u, GT_BUDGET);
        bulk_wait_all();
      }
      return;
    }
    float *s0 = cur, *s1 = cur + GT_TILE, *s2 = cur + 2 * GT_TILE, *s3 = cur + 3 * GT_TILE, *s4 = cur + 4 * GT_TILE,
          *s5 = cur + 5 * GT_TILE;
#pragma unroll 4
    for (int i = tid; i < GT_TILE; i += 256) gt_particle<POW2>(s0, s1, s2, s3, s4, s5, i, g4, f);
    fence_async_smem();  // this thread's shared-memory writes -> visible to the bulk stores
    __syncthreads();
    if (tid == 0) {
#pragma unroll
      for (int a = 0; a < 6; ++a) bulk_s2g(dst[a] + t * GT_TILE, cur + a * GT_TILE, tile_bytes);
      bulk_commit();
    }
    if (DEP) {  // the drifted positions' density while the stores drain
      gt_deposit_warp<POW2>(s0, s1, s2, cur + 6 * GT_TILE, 128 * warp, wboxes + warp * GT_WBOX, d, inv_dx, qscale,
                            qg, status, lane);
      fence_async_smem();
      __syncthreads();  // the buffer is free for the prefetch of the tile after next
    }
  }
  if (tid == 0) bulk_wait_all();
  // the remainder after the full tiles: plain loads, every CTA a slice
  const long long r0 = ntiles * GT_TILE;
  for (long long p = r0 + blockIdx.x * (long long)blockDim.x + tid; p < n; p += (long long)gridDim.x * blockDim.x) {
    float px = x[p], py = y[p], pz = z[p], ux = vx[p], uy = vy[p], uz = vz[p];
    float ax, ay, az;
    gather_g4<POW2>(g4, px, py, pz, f, ax, ay, az);
    if (f.mode != GC_STEP_PRIME) {
      ux = __fadd_rn(ux, __fmul_rn(ax, f.h));
      uy = __fadd_rn(uy, __fmul_rn(ay, f.h));
      uz = __fadd_rn(uz, __fmul_rn(az, f.h));
    }
    if (f.mode != GC_STEP_CLOSE) {
      ux = __fadd_rn(ux, __fmul_rn(ax, f.h));
      uy = __fadd_rn(uy, __fmul_rn(ay, f.h));
      uz = __fadd_rn(uz, __fmul_rn(az, f.h));
      px = __fadd_rn(px, __fmul_rn(ux, f.dt));
      py = __fadd_rn(py, __fmul_rn(uy, f.dt));
      pz = __fadd_rn(pz, __fmul_rn(uz, f.dt));
      x[p] = px;
      y[p] = py;
      z[p] = pz;
    }
    vx[p] = ux;
    vy[p] = uy;
    vz[p] = uz;
    if (DEP) gt_deposit_one<POW2>(px, py, pz, m[p], d, inv_dx, qscale, qg, status);
  }
}

int gc_gather_kick_drift(gc_ctx *ctx, const gc_particles *p, float dt, int mode, int diag, int grad_grid,
                         int deposit_next, float *axo, float *ayo, float *azo, int *nparts_out, int *deposited) {
  if (deposited) *deposited = 0;
  FusedCtx f;
  f.dx = (float)ctx->dx;
  f.inv_dx = 1.0f / f.dx;
  f.inv_2dx = 1.0f / (2.0f * f.dx);
  f.G = ctx->G;
  f.dt = dt;
  f.h = 0.5f * dt;
  f.mode = mode;
  f.diag = diag;
  unsigned nb = gc_blocks(p->n, 256);
  if (nb > gc_sms() * 16u) nb = gc_sms() * 16u;
  int s = gc_ensure_red(ctx, (size_t)nb * 11);
  if (s) return s;
  if (grad_grid && !axo) {
    const size_t g3 = (size_t)ctx->G * ctx->G * ctx->G;
    if (!ctx->g4) GC_CUDA(ctx, cudaMalloc(&ctx->g4, g3 * sizeof(float4)));
    const GradCtx g = make_grad(ctx);
    gc_launch(ctx, GK_GRAD, k_grad4, dim3(gc_blocks(g.G, 32), gc_blocks(g.G, 8), g.G), dim3(32, 8), 0, ctx->hi,
              (float4 *)ctx->g4, g);
    int fe = 0;
    const bool pow2 = std::frexp(f.dx, &fe) == 0.5f;  // then inv_dx is exact
    const uintptr_t al = (uintptr_t)p->x | (uintptr_t)p->y | (uintptr_t)p->z | (uintptr_t)p->vx | (uintptr_t)p->vy |
                         (uintptr_t)p->vz;
    const bool dep = deposit_next && mode != GC_STEP_CLOSE && ((uintptr_t)p->m & 15u) == 0;
    if (!diag && (al & 15u) == 0 && p->n >= GT_TILE) {
      if (!ctx->gt_smem_set) {  // opt in to more than 48 KB of dynamic shared memory (once per context)
        GC_CUDA(ctx, cudaFuncSetAttribute(k_gather4_tma<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, GT_SMEM(false)));
        GC_CUDA(ctx, cudaFuncSetAttribute(k_gather4_tma<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, GT_SMEM(false)));
        GC_CUDA(ctx, cudaFuncSetAttribute(k_gather4_tma<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, GT_SMEM(true)));
        GC_CUDA(ctx, cudaFuncSetAttribute(k_gather4_tma<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, GT_SMEM(true)));
        ctx->gt_smem_set = 1;
      }
      // bulk-streamed state, persistent: 4 CTAs per SM (3 when depositing: 72 KB each)
      const long long ntiles = p->n / GT_TILE;
      const long long per_sm = dep ? 3 : 4;
      const unsigned nbt = (unsigned)(ntiles < (long long)gc_sms() * per_sm ? ntiles : (long long)gc_sms() * per_sm);
      DepCtx d;
      d.dx = (float)ctx->dx;
      d.inv_vol = 1.0f / ((d.dx * d.dx) * d.dx);
      d.G = ctx->G;
      const float inv_dx_dep = pow2 ? std::ldexp(1.0f, 1 - fe) : 0.0f;
      auto k = dep ? (pow2 ? k_gather4_tma<true, true> : k_gather4_tma<false, true>)
                   : (pow2 ? k_gather4_tma<true, false> : k_gather4_tma<false, false>);
      gc_launch(ctx, GK_GATHER_KD, k, dim3(nbt), dim3(256), GT_SMEM(dep), p->x, p->y, p->z, p->vx, p->vy, p->vz, p->m,
                (long long)p->n, (const float4 *)ctx->g4, f, d, inv_dx_dep, (const double *)(ctx->dsmall + GC_S_QEXP_PM),
                ctx->q, ctx->dstatus);
      if (dep && deposited) *deposited = 1;
    } else {
      auto k = diag ? (pow2 ? k_gather4_kick_drift<true, true> : k_gather4_kick_drift<true, false>)
                    : (pow2 ? k_gather4_kick_drift<false, true> : k_gather4_kick_drift<false, false>);
      gc_launch(ctx, GK_GATHER_KD, k, dim3(nb), dim3(256), 0, p->x, p->y, p->z, p->vx, p->vy, p->vz, p->m,
                (long long)p->n, (const float4 *)ctx->g4, f, ctx->red);
    }
  } else if (diag) {
    gc_launch(ctx, GK_GATHER_KD, k_gather_kick_drift<true>, dim3(nb), dim3(256), 0, p->x, p->y, p->z, p->vx, p->vy,
              p->vz, p->m, (long long)p->n, ctx->hi, f, axo, ayo, azo, ctx->red);
  } else {
    gc_launch(ctx, GK_GATHER_KD, k_gather_kick_drift<false>, dim3(nb), dim3(256), 0, p->x, p->y, p->z, p->vx, p->vy,
              p->vz, p->m, (long long)p->n, ctx->hi, f, axo, ayo, azo, ctx->red);
  }
  GC_LAUNCH_CHECK(ctx, "gather_kick_drift");
  if (nparts_out) *nparts_out = (int)nb;
  return GC_OK;
}

// ------------------------------------------------------------------------------
// diagnostics (diagnostics_device.py)
// ------------------------------------------------------------------------------
__global__ void __launch_bounds__(256)
    k_diag_particles(const float *__restrict__ x, const float *__restrict__ y, const float *__restrict__ z,
                     const float *__restrict__ vx, const float *__restrict__ vy, const float *__restrict__ vz,
                     const float *__restrict__ m, long long n, double *__restrict__ parts) {
  DiagAcc acc;
  acc.zero();
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    acc.particle(m[p], x[p], y[p], z[p], vx[p], vy[p], vz[p]);
  }
  double dv[11];
  acc.to_double(dv);
  block_partials<11>(dv, parts + (size_t)blockIdx.x * 11);
}

extern "C" int gc_diag_particles(gc_ctx *ctx, const float *x, const float *y, const float *z, const float *vx,
                                 const float *vy, const float *vz, const float *m, int64_t n, double out[11]) {
  if (!ctx) return GC_ERR_ARG;
  GC_REQUIRE(ctx, out, "gc_diag_particles: NULL out");
  GC_REQUIRE(ctx, n >= 0 && n < (1LL << 31), "particle count out of range");
  GC_REQUIRE(ctx, n == 0 || (x && y && z && vx && vy && vz && m), "gc_diag_particles: NULL pointer");
  const int nb = 512;
  int s = gc_ensure_red(ctx, nb * 11);
  if (s) return s;
  gc_launch(ctx, GK_DIAG, k_diag_particles, dim3(nb), dim3(256), 0, x, y, z, vx, vy, vz, m, (long long)n, ctx->red);
  GC_LAUNCH_CHECK(ctx, "diag particles");
  if ((s = gc_finalize(ctx, ctx->red, nb, 11, ctx->ddiag))) return s;
  GC_CUDA(ctx, cudaMemcpyAsync(out, ctx->ddiag, 11 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  GC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return GC_OK;
}

__global__ void __launch_bounds__(256) k_dot(const float *__restrict__ a, const float *__restrict__ b, size_t n,
                                             double *__restrict__ parts) {
  double acc[1] = {0.0};
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
    acc[0] += (double)a[t] * (double)b[t];
  block_partials<1>(acc, parts + blockIdx.x);
}

int gc_dot_async(gc_ctx *ctx, const float *a, const float *b, size_t n, double *dst) {
  const int nb = 1024;
  int s = gc_ensure_red(ctx, nb);
  if (s) return s;
  gc_launch(ctx, GK_REDUCE, k_dot, dim3(nb), dim3(256), 0, a, b, n, ctx->red);
  GC_LAUNCH_CHECK(ctx, "dot");
  return gc_finalize(ctx, ctx->red, nb, 1, dst);
}

extern "C" int gc_diag_grid_pe(gc_ctx *ctx, const float *rho, const float *phi, double *out) {
  if (!ctx) return GC_ERR_ARG;
  GC_REQUIRE(ctx, rho && phi && out, "gc_diag_grid_pe: NULL pointer");
  const size_t g3 = (size_t)ctx->G * ctx->G * ctx->G;
  int s = gc_dot_async(ctx, rho, phi, g3, ctx->ddiag + 12);
  if (s) return s;
  GC_CUDA(ctx, cudaMemcpyAsync(out, ctx->ddiag + 12, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  GC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return GC_OK;
}

__global__ void __launch_bounds__(256)
    k_radial_hist(const float *__restrict__ x, const float *__restrict__ y, const float *__restrict__ z,
                  const float *__restrict__ m, long long n, double cx, double cy, double cz, double inv_binw, int nbins,
                  double *__restrict__ hist) {
  extern __shared__ double sh[];
  for (int b = threadIdx.x; b < nbins; b += blockDim.x) sh[b] = 0.0;
  __syncthreads();
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    const double rx = (double)x[p] - cx, ry = (double)y[p] - cy, rz = (double)z[p] - cz;
    const double r = sqrt(rx * rx + ry * ry + rz * rz);
    const double fb = r * inv_binw;
    int b = fb >= (double)nbins ? nbins - 1 : (int)fb;
    if (b < 0) b = 0;
    atomicAdd(&sh[b], (double)m[p]);
  }
  __syncthreads();
  for (int b = threadIdx.x; b < nbins; b += blockDim.x)
    if (sh[b] != 0.0) atomicAdd(&hist[b], sh[b]);
}

extern "C" int gc_radial_histogram(gc_ctx *ctx, const float *x, const float *y, const float *z, const float *m,
                                   int64_t n, double cx, double cy, double cz, double inv_binw, int nbins,
                                   double *hist) {
  if (!ctx) return GC_ERR_ARG;
  GC_REQUIRE(ctx, hist, "gc_radial_histogram: NULL hist");
  GC_REQUIRE(ctx, nbins >= 1 && nbins <= 6144, "nbins must be in [1, 6144]");
  GC_REQUIRE(ctx, n >= 0 && n < (1LL << 31), "particle count out of range");
  GC_CUDA(ctx, cudaMemsetAsync(hist, 0, nbins * sizeof(double), ctx->stream));
  if (n == 0) return GC_OK;
  GC_REQUIRE(ctx, x && y && z && m, "gc_radial_histogram: NULL pointer");
  const size_t smem = nbins * sizeof(double);
  if (smem > 48 * 1024)
    GC_CUDA(ctx, cudaFuncSetAttribute(k_radial_hist, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  unsigned nb = gc_blocks(n, 256);
  if (nb > gc_sms() * 4u) nb = gc_sms() * 4u;
  gc_launch(ctx, GK_HIST, k_radial_hist, dim3(nb), dim3(256), smem, x, y, z, m, (long long)n, cx, cy, cz, inv_binw, nbins, hist);
  GC_LAUNCH_CHECK(ctx, "radial hist");
  return GC_OK;
}

// ------------------------------------------------------------------------------
// headless 2-D projection (viz/project.py:26-46)
// ------------------------------------------------------------------------------
// Nearest-bin mass histogram over two in-plane axes: ia = floor((a - lo_a)/binw_a)
// in f32 as the reference; mass outside [0, bins) is dropped.
__global__ void __launch_bounds__(256)
    k_project_ngp(const float *__restrict__ pa, const float *__restrict__ pb, const float *__restrict__ m, long long n,
                  float lo_a, float lo_b, float bw_a, float bw_b, int bins, float *__restrict__ img) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    const float ga = floorf(__fdiv_rn(__fsub_rn(pa[p], lo_a), bw_a));
    const float gb = floorf(__fdiv_rn(__fsub_rn(pb[p], lo_b), bw_b));
    if (!(ga >= 0.0f && ga < (float)bins && gb >= 0.0f && gb < (float)bins)) continue;
    atomicAdd(img + (size_t)(int)ga * bins + (int)gb, m[p]);
  }
}

extern "C" int gc_project_ngp(gc_ctx *ctx, const float *pa, const float *pb, const float *m, int64_t n, double lo_a,
                              double lo_b, double binw_a, double binw_b, int bins, float *img) {
  if (!ctx) return GC_ERR_ARG;
  GC_REQUIRE(ctx, img, "gc_project_ngp: NULL image");
  GC_REQUIRE(ctx, bins >= 1 && bins <= 16384, "bins must be in [1, 16384]");
  GC_REQUIRE(ctx, binw_a > 0.0 && binw_b > 0.0, "bin widths must be positive");
  GC_REQUIRE(ctx, n >= 0 && n < (1LL << 31), "particle count out of range");
  GC_CUDA(ctx, cudaMemsetAsync(img, 0, (size_t)bins * bins * sizeof(float), ctx->stream));
  if (n == 0) return GC_OK;
  GC_REQUIRE(ctx, pa && pb && m, "gc_project_ngp: NULL particle array");
  unsigned nb = gc_blocks(n, 256);
  if (nb > gc_sms() * 16u) nb = gc_sms() * 16u;
  gc_launch(ctx, GK_PROJECT, k_project_ngp, dim3(nb), dim3(256), 0, pa, pb, m, (long long)n, (float)lo_a, (float)lo_b,
            (float)binw_a, (float)binw_b, bins, img);
  GC_LAUNCH_CHECK(ctx, "project");
  return GC_OK;
}

// ------------------------------------------------------------------------------
// self-test of the bounded mbarrier wait (the wait of the TMA particle pass and
// of the tensor-core kernels): one thread arms an mbarrier for one arrival and,
// unless `arrive` is set, nobody arrives; the wait must give up after `budget`
// SM clocks and raise GC_FLAG_TIMEOUT instead of spinning on.
// ------------------------------------------------------------------------------
__global__ void k_selftest_wait(unsigned *__restrict__ status, long long budget, int arrive) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x != 0) return;
  umma::mbar_init(&bar, 1);
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  if (arrive) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(umma::smem_u32(&bar)) : "memory");
  if (!umma::mbar_wait(&bar, 0u, budget)) atomicOr(status, GC_FLAG_TIMEOUT);
}

extern "C" int gc_selftest_wait_timeout(void *stream, uint32_t *status, int64_t budget_cycles, int arrive) {
  if (!status || budget_cycles < 1 || budget_cycles > GT_BUDGET) {
    gc_set_error(nullptr, "gc_selftest_wait_timeout: status required, budget in [1, %lld] clocks",
                 (long long)GT_BUDGET);
    return GC_ERR_ARG;
  }
  k_selftest_wait<<<1, 32, 0, (cudaStream_t)stream>>>((unsigned *)status, (long long)budget_cycles, arrive ? 1 : 0);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    gc_set_error(nullptr, "gc_selftest_wait_timeout: launch failed: %s", cudaGetErrorString(e));
    return GC_ERR_CUDA;
  }
  return GC_OK;
}
