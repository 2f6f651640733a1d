// Learned warm start: BF16 3-D convolutions on the fifth-generation tensor cores.
//
// This file holds the tensor-core kernels of the warm-start network (implicit-GEMM
// convolution forward / data-gradient / weight-gradient) and a single-tile GEMM
// used to check the shared-memory descriptor conventions on the device.
#include <cuda_fp16.h>

#include <algorithm>
#include <vector>

#include "common.cuh"
#include "umma.cuh"

// Clock budget of every mbarrier wait (about one second at 2 GHz).
#define WS_WAIT_BUDGET 2000000000LL
// Warps whose lane 0 issues tensor-core MMAs (each commits once per phase).
#define WS_ISSUERS 4

// ------------------------------------------------------------------------------
// single-tile GEMM check: D (128 x N, f32) = A (128 x K) * B (N x K)^T
// ------------------------------------------------------------------------------
// A and B arrive row-major (bf16 bits) and are staged into shared memory in the
// no-swizzle canonical layout of the requested major-ness:
//   K-major,  R rows: byte(r,k) = (k/8)*R*16 + (r/8)*128 + (r%8)*16 + (k%8)*2
//   MN-major, R rows: byte(r,k) = (r/8)*(K/8)*128 + (k/8)*128 + (k%8)*16 + (r%8)*2
// `swap` exchanges the two byte offsets in the descriptor of MN-major operands.
__device__ __forceinline__ uint32_t st_offset(int r, int k, int R, int K, int mn) {
  return mn ? (uint32_t)((r >> 3) * (K >> 3) * 128 + (k >> 3) * 128 + (k & 7) * 16 + (r & 7) * 2)
            : (uint32_t)((k >> 3) * R * 16 + (r >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

__global__ void __launch_bounds__(128) k_umma_selftest(const uint16_t *__restrict__ A, const uint16_t *__restrict__ B,
                                                       float *__restrict__ D, int N, int K, int a_mn, int b_mn,
                                                       int swap, unsigned *__restrict__ status) {
  extern __shared__ __align__(1024) uint8_t sm[];
  uint8_t *sA = sm;
  uint8_t *sB = sm + 128 * K * 2;
  uint64_t *bar = reinterpret_cast<uint64_t *>(sB + 256 * K * 2);
  uint32_t *tslot = reinterpret_cast<uint32_t *>(bar + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  for (int i = tid; i < 128 * K; i += 128)
    *reinterpret_cast<uint16_t *>(sA + st_offset(i / K, i % K, 128, K, a_mn)) = A[i];
  for (int i = tid; i < N * K; i += 128)
    *reinterpret_cast<uint16_t *>(sB + st_offset(i / K, i % K, N, K, b_mn)) = B[i];
  if (warp == 0) {
    umma::tmem_alloc(tslot, 256);
    umma::tmem_relinquish();
  }
  if (tid == 0) {
    umma::mbar_init(bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  umma::fence_async_smem();
  umma::tc_fence_before();
  __syncthreads();
  umma::tc_fence_after();
  const uint32_t tmem = *tslot;
  if (tid == 0) {
    const uint32_t a_lbo = a_mn ? 128u : 128u * 16u, a_sbo = a_mn ? (uint32_t)(K / 8) * 128u : 128u;
    const uint32_t b_lbo = b_mn ? 128u : (uint32_t)N * 16u, b_sbo = b_mn ? (uint32_t)(K / 8) * 128u : 128u;
    const uint32_t idesc = umma::idesc_bf16(128, N, a_mn, b_mn);
    for (int ks = 0; ks < K / 16; ++ks) {
      const uint32_t aoff = 2u * ks * a_lbo, boff = 2u * ks * b_lbo;  // two core matrices along K
      const uint64_t ad = (a_mn && swap) ? umma::sdesc(umma::smem_u32(sA) + aoff, a_sbo, a_lbo)
                                         : umma::sdesc(umma::smem_u32(sA) + aoff, a_lbo, a_sbo);
      const uint64_t bd = (b_mn && swap) ? umma::sdesc(umma::smem_u32(sB) + boff, b_sbo, b_lbo)
                                         : umma::sdesc(umma::smem_u32(sB) + boff, b_lbo, b_sbo);
      umma::mma_bf16(tmem, ad, bd, idesc, ks > 0 ? 1u : 0u);
    }
    umma::mma_commit(bar);
  }
  __syncwarp();
  const bool ok = umma::mbar_wait(bar, 0, WS_WAIT_BUDGET);
  if (!ok) {
    if (lane == 0) atomicOr(status, 1u);
    umma::mbar_wait(bar, 0, WS_WAIT_BUDGET);  // give in-flight MMAs a second chance before freeing TMEM
  }
  umma::tc_fence_after();
  if (ok) {
    for (int c = 0; c < N; c += 16) {
      uint32_t r[16];
      umma::tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)c, r);
      umma::tmem_wait_ld();
      float *row = D + (size_t)(32 * warp + lane) * N + c;
#pragma unroll
      for (int j = 0; j < 16; ++j) row[j] = __uint_as_float(r[j]);
    }
  }
  umma::tc_fence_before();
  __syncthreads();
  if (warp == 0) umma::tmem_dealloc(tmem, 256);
}

extern "C" int gc_ws_selftest_gemm(const void *A, const void *B, float *D, int N, int K, int a_mn, int b_mn, int swap,
                                   void *stream, unsigned *status) {
  if (!A || !B || !D || !status) return GC_ERR_ARG;
  if (N < 16 || N > 256 || (N % 16) || K < 16 || K > 64 || (K % 16)) return GC_ERR_ARG;
  const size_t smem = (size_t)128 * K * 2 + (size_t)256 * K * 2 + 64;
  cudaStream_t st = (cudaStream_t)stream;
  if (cudaFuncSetAttribute(k_umma_selftest, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return GC_ERR_CUDA;
  k_umma_selftest<<<1, 128, smem, st>>>((const uint16_t *)A, (const uint16_t *)B, D, N, K, a_mn, b_mn, swap, status);
  return cudaGetLastError() == cudaSuccess ? GC_OK : GC_ERR_CUDA;
}

// ------------------------------------------------------------------------------
// activations and weights
// ------------------------------------------------------------------------------
// An activation with C channels on an R^3 grid is stored channel-chunk planar:
// chunk c (channels 8c..8c+7) is an R^3 array of 16-byte rows, one row per voxel
// (x fastest), i.e. element (ch, voxel) at ((ch/8)*R^3 + voxel)*8 + ch%8.
// Convolution weights (3x3x3, tap t = (dz+1)*9 + (dy+1)*3 + (dx+1)) for the
// forward pass are [27][Cin/8][Cout] 16-byte rows of 8 input channels.

__device__ __forceinline__ float bf_lo(uint32_t w) { return __uint_as_float(w << 16); }
__device__ __forceinline__ float bf_hi(uint32_t w) { return __uint_as_float(w & 0xffff0000u); }
__device__ __forceinline__ uint32_t bf_pack(float a, float b) {
  // round to nearest even, NaN kept quiet
  uint32_t ua = __float_as_uint(a), ub = __float_as_uint(b);
  ua = (ua & 0x7fffffffu) > 0x7f800000u ? 0x7fc00000u : ua + 0x7fffu + ((ua >> 16) & 1u);
  ub = (ub & 0x7fffffffu) > 0x7f800000u ? 0x7fc00000u : ub + 0x7fffu + ((ub >> 16) & 1u);
  return (ua >> 16) | (ub & 0xffff0000u);
}
__device__ __forceinline__ void unpack8(const uint4 &v, float (&f)[8]) {
  f[0] = bf_lo(v.x); f[1] = bf_hi(v.x); f[2] = bf_lo(v.y); f[3] = bf_hi(v.y);
  f[4] = bf_lo(v.z); f[5] = bf_hi(v.z); f[6] = bf_lo(v.w); f[7] = bf_hi(v.w);
}
template <int O, int N>
__device__ __forceinline__ uint4 pack8(const float (&f)[N]) {
  return make_uint4(bf_pack(f[O], f[O + 1]), bf_pack(f[O + 2], f[O + 3]), bf_pack(f[O + 4], f[O + 5]),
                    bf_pack(f[O + 6], f[O + 7]));
}

// ------------------------------------------------------------------------------
// convolution as implicit GEMM: out[v][co] = sum_t sum_ci in[v + off_t][ci] W[t][co][ci]
// ------------------------------------------------------------------------------
// A CTA owns BZ planes x BY lines x R voxels of the output. Its input tile with a
// one-voxel halo, (BZ+2) x (BY+2) x (R+2) voxels, is staged channel-chunk planar
// in shared memory: row L (padded linear voxel index) of chunk kc at byte
// (kc*V + L)*16. That is the K-major no-swizzle operand layout with 8-row groups
// 128 bytes apart, so the A operand of tap t for the 128 output rows starting
// at padded index s is simply the descriptor at row s + off_t: no im2col copy.
// Output rows are the padded linear range [L0, L1] cut into 128-row M tiles;
// rows that fall on halo voxels are computed and discarded. Accumulators live
// in Tensor Memory (M tile mt in columns mt*Cout ..). Weights stream through a
// two-slot ring of tap groups; one thread issues the MMAs, completion is
// tracked by tcgen05.commit on one mbarrier per slot.
struct ConvFwd {
  const uint4 *in;
  const uint4 *w;
  const float *bias;   // [Cout] or null
  const uint4 *skip;   // Cout channels or null: added before the activation
  const uint4 *mask;   // Cout channels or null: result zeroed where mask <= 0
  uint4 *out;          // Cout channels or null
  float *out_f32;      // channel 0 as f32 [R^3] or null
  unsigned *status;
  int R, Cin, Cout, BZ, BY;
  int relu;
  int tpg;             // taps per weight group
  int n_mt;
  uint32_t tmem_cols;
};

__host__ __device__ inline void conv_geom(int R, int BZ, int BY, int &W2, int &P, int &V, int &L0, int &L1) {
  W2 = R + 2;
  P = (BY + 2) * W2;
  V = (BZ + 2) * P;
  L0 = P + W2 + 1;
  L1 = V - 1 - L0;
}

__device__ __forceinline__ int tap_offset(int t, int P, int W2) {
  return (t / 9 - 1) * P + ((t / 3) % 3 - 1) * W2 + (t % 3 - 1);
}

// Copy the weights of tap group g (taps g*tpg .. min(27, (g+1)*tpg)) to dst.
__device__ __forceinline__ void load_taps(const uint4 *__restrict__ w, int g, int tpg, uint32_t tap_bytes, uint8_t *dst,
                                          int tid) {
  const int t0 = g * tpg, t1 = min(27, t0 + tpg);
  const uint4 *src = w + (size_t)t0 * (tap_bytes / 16u);
  uint4 *d = reinterpret_cast<uint4 *>(dst);
  const int n16 = (t1 - t0) * (int)(tap_bytes / 16u);
  for (int i = tid; i < n16; i += blockDim.x) umma::cp_async16(d + i, src + i, true);
}

__global__ void __launch_bounds__(256) k_conv_fwd(ConvFwd a) {
  extern __shared__ __align__(1024) uint8_t sm[];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int R = a.R;
  int W2, P, V, L0, L1;
  conv_geom(R, a.BZ, a.BY, W2, P, V, L0, L1);
  const int kci = a.Cin >> 3;
  const size_t R3 = (size_t)R * R * R;
  const int nby = R / a.BY;
  const int z0 = (blockIdx.x / nby) * a.BZ, y0 = (blockIdx.x % nby) * a.BY;
  const uint32_t tile_bytes = (uint32_t)(kci * V + 128) * 16u;
  const uint32_t tap_bytes = (uint32_t)a.Cin * a.Cout * 2u;
  const uint32_t slot_bytes = (uint32_t)a.tpg * tap_bytes;
  uint8_t *tile = sm;
  uint8_t *ring = sm + ((tile_bytes + 1023u) & ~1023u);
  uint64_t *bars = reinterpret_cast<uint64_t *>(ring + 2u * slot_bytes);
  uint32_t *tslot = reinterpret_cast<uint32_t *>(bars + 2);
  const int ngroups = (27 + a.tpg - 1) / a.tpg;

  if (warp == 0) {
    umma::tmem_alloc(tslot, a.tmem_cols);
    umma::tmem_relinquish();
  }
  if (tid == 0) {  // one arrival per issuing warp (WS_ISSUERS commits per phase)
    umma::mbar_init(&bars[0], WS_ISSUERS);
    umma::mbar_init(&bars[1], WS_ISSUERS);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // input tile, zero outside the grid, plus a zero margin read by the last M tile;
  // one warp per padded line, lanes along x
  uint4 *trow = reinterpret_cast<uint4 *>(tile);
  {
    const int nzy = (a.BZ + 2) * (a.BY + 2), nrows = kci * nzy, nwarps = blockDim.x >> 5;
    for (int row = warp; row < nrows; row += nwarps) {
      const int kc = row / nzy, rr = row - kc * nzy;
      const int tz = rr / (a.BY + 2), ty = rr - tz * (a.BY + 2);
      const int gz = z0 - 1 + tz, gy = y0 - 1 + ty;
      const bool rowin = (unsigned)gz < (unsigned)R && (unsigned)gy < (unsigned)R;
      const uint4 *src = a.in + (size_t)kc * R3 + ((size_t)(rowin ? gz : 0) * R + (rowin ? gy : 0)) * R;
      uint4 *dst = trow + (size_t)kc * V + (size_t)rr * W2;
      for (int tx = lane; tx < W2; tx += 32) {
        const int gx = tx - 1;
        const bool in = rowin && (unsigned)gx < (unsigned)R;
        umma::cp_async16(dst + tx, in ? (const void *)(src + gx) : (const void *)a.in, in);
      }
    }
  }
  for (int i = tid; i < 128; i += blockDim.x) trow[kci * V + i] = make_uint4(0u, 0u, 0u, 0u);
  load_taps(a.w, 0, a.tpg, tap_bytes, ring, tid);
  umma::cp_async_wait_all();
  umma::fence_async_smem();
  umma::tc_fence_before();
  __syncthreads();
  umma::tc_fence_after();
  const uint32_t tmem = *tslot;
  const uint32_t idesc = umma::idesc_bf16(128, a.Cout, 0, 0);
  const uint32_t a_lbo = (uint32_t)V * 16u, b_lbo = (uint32_t)a.Cout * 16u;
  const uint32_t tile_u32 = umma::smem_u32(tile), ring_u32 = umma::smem_u32(ring);
  uint32_t ph0 = 0u, ph1 = 0u;  // next completion parity of each slot's barrier
  int last = 0;                  // slot of the last commit
  bool fail = false;
  for (int g = 0; g < ngroups; ++g) {
    const int s = g & 1;
    if (lane == 0 && warp < WS_ISSUERS) {  // issuer w owns the M tiles mt = w (mod WS_ISSUERS)
      umma::tc_fence_after();
      const int t0 = g * a.tpg, t1 = min(27, t0 + a.tpg);
      // descriptors differ only in the start address (bits 0..13, address / 16)
      const uint64_t ad0 = umma::sdesc(tile_u32, a_lbo, 128u), bd0 = umma::sdesc(ring_u32, b_lbo, 128u);
      for (int t = t0; t < t1; ++t) {
        const int off = tap_offset(t, P, W2);
        const uint32_t boff = ((uint32_t)s * slot_bytes + (uint32_t)(t - t0) * tap_bytes) >> 4;
        for (int mt = warp; mt < a.n_mt; mt += WS_ISSUERS) {
          const uint32_t aoff = ((uint32_t)(L0 + 128 * mt + off) * 16u) >> 4;
          for (int ks = 0; ks < kci / 2; ++ks) {
            umma::mma_bf16(tmem + (uint32_t)(mt * a.Cout), ad0 + aoff + ((2u * ks * a_lbo) >> 4),
                           bd0 + boff + ((2u * ks * b_lbo) >> 4), idesc, (t > 0 || ks > 0) ? 1u : 0u);
          }
        }
      }
      umma::mma_commit(&bars[s]);
    }
    last = s;
    if (g + 1 < ngroups) {
      const int s1 = (g + 1) & 1;
      if (g >= 1) {
        fail = !umma::mbar_wait(&bars[s1], s1 ? ph1 : ph0, WS_WAIT_BUDGET);
        if (s1) ph1 ^= 1u; else ph0 ^= 1u;
      }
      if (__syncthreads_or(fail)) { fail = true; break; }
      load_taps(a.w, g + 1, a.tpg, tap_bytes, ring + (uint32_t)s1 * slot_bytes, tid);
      umma::cp_async_wait_all();
      umma::fence_async_smem();
      __syncthreads();
    }
  }
  // completion of every MMA: the last commit (MMAs of one thread complete in order)
  if (!umma::mbar_wait(&bars[last], last ? ph1 : ph0, WS_WAIT_BUDGET)) fail = true;
  fail = __syncthreads_or(fail);
  umma::tc_fence_after();
  if (fail) {
    if (tid == 0) atomicOr(a.status, 1u);
  } else {
    const int quad = warp & 3;
    for (int mt = warp >> 2; mt < a.n_mt; mt += (blockDim.x >> 7)) {
      const int L = L0 + 128 * mt + 32 * quad + lane;
      const int tz = L / P, rem = L - tz * P, ty = rem / W2, tx = rem - ty * W2;
      const bool valid = L <= L1 && tz >= 1 && tz <= a.BZ && ty >= 1 && ty <= a.BY && tx >= 1 && tx <= R;
      const size_t vox = ((size_t)(z0 + tz - 1) * R + (y0 + ty - 1)) * R + (tx - 1);
      for (int c = 0; c < a.Cout; c += 16) {
        uint32_t r[16];
        umma::tmem_ld16(tmem + ((uint32_t)(32 * quad) << 16) + (uint32_t)(mt * a.Cout + c), r);
        umma::tmem_wait_ld();
        if (!valid) continue;
        float v[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]) + (a.bias ? __ldg(a.bias + c + j) : 0.0f);
        if (a.skip) {
          float s0[8], s1[8];
          unpack8(__ldg(a.skip + (size_t)(c >> 3) * R3 + vox), s0);
          unpack8(__ldg(a.skip + (size_t)((c >> 3) + 1) * R3 + vox), s1);
#pragma unroll
          for (int j = 0; j < 8; ++j) { v[j] += s0[j]; v[8 + j] += s1[j]; }
        }
        if (a.relu) {
#pragma unroll
          for (int j = 0; j < 16; ++j) v[j] = fmaxf(v[j], 0.0f);
        }
        if (a.mask) {
          float m0[8], m1[8];
          unpack8(__ldg(a.mask + (size_t)(c >> 3) * R3 + vox), m0);
          unpack8(__ldg(a.mask + (size_t)((c >> 3) + 1) * R3 + vox), m1);
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            v[j] = m0[j] > 0.0f ? v[j] : 0.0f;
            v[8 + j] = m1[j] > 0.0f ? v[8 + j] : 0.0f;
          }
        }
        if (a.out) {
          a.out[(size_t)(c >> 3) * R3 + vox] = pack8<0>(v);
          a.out[(size_t)((c >> 3) + 1) * R3 + vox] = pack8<8>(v);
        }
        if (a.out_f32 && c == 0) a.out_f32[vox] = v[0];
      }
    }
  }
  umma::tc_fence_before();
  __syncthreads();
  if (warp == 0) umma::tmem_dealloc(tmem, a.tmem_cols);
}

// ------------------------------------------------------------------------------
// weight gradient: dW[t][co][ci] = sum_v gy[v][co] x[v + off_t][ci]
// ------------------------------------------------------------------------------
// GEMM with M = co (padded to 128), N = ci, K = voxels. The input tile (with
// halo) is staged exactly as in the forward pass; read MN-major (8 channels of
// one voxel per 16-byte row), the B operand of tap t is again the tile shifted
// by off_t rows. gy arrives in stages of 128 voxels, each voxel's 16-byte rows
// (8 output channels) placed in 2 KB groups of 8 voxels so that every one of the
// 128 M rows addresses shared memory of the stage (rows >= Cout are never read
// back). Voxels outside the CTA's block are zero in gy. Taps are split into
// passes so that a pass's accumulators (tpp x Cin columns) fit Tensor Memory;
// persistent CTAs accumulate over all their blocks and write one partial per
// CTA, summed in a fixed order afterwards.
struct ConvW {
  const uint4 *x;    // layer input, Cin channels
  const uint4 *gy;   // gradient of the pre-activation output, Cout channels
  float *part;       // [gridDim.x][27][Cout][Cin]
  unsigned *status;
  int R, Cin, Cout, BZ, BY;
  int tpp;           // taps per pass
  int nblocks;
  uint32_t tmem_cols;
};

#define WG_STAGE_ROWS 128
#define WG_STAGE_BYTES (16 * 2048)

__global__ void __launch_bounds__(256) k_conv_wgrad(ConvW a) {
  extern __shared__ __align__(1024) uint8_t sm[];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int R = a.R;
  int W2, P, V, L0, L1;
  conv_geom(R, a.BZ, a.BY, W2, P, V, L0, L1);
  const int kci = a.Cin >> 3, kco = a.Cout >> 3;
  const size_t R3 = (size_t)R * R * R;
  const int nby = R / a.BY;
  const int nst = (L1 - L0 + WG_STAGE_ROWS) / WG_STAGE_ROWS;
  const uint32_t tile_bytes = (uint32_t)(kci * V + 128) * 16u;
  uint8_t *tile = sm;
  uint8_t *stg = sm + ((tile_bytes + 1023u) & ~1023u);
  uint64_t *bars = reinterpret_cast<uint64_t *>(stg + 2 * WG_STAGE_BYTES);
  uint32_t *tslot = reinterpret_cast<uint32_t *>(bars + 2);
  if (warp == 0) {
    umma::tmem_alloc(tslot, a.tmem_cols);
    umma::tmem_relinquish();
  }
  if (tid == 0) {  // one arrival per issuing warp
    umma::mbar_init(&bars[0], WS_ISSUERS);
    umma::mbar_init(&bars[1], WS_ISSUERS);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  umma::tc_fence_before();
  __syncthreads();
  umma::tc_fence_after();
  const uint32_t tmem = *tslot;
  const uint32_t idesc = umma::idesc_bf16(128, a.Cin, 1, 1);
  const uint32_t tile_u32 = umma::smem_u32(tile), stg_u32 = umma::smem_u32(stg);
  uint32_t ph0 = 0u, ph1 = 0u;
  bool pend0 = false, pend1 = false;
  bool fail = false;
  long long gs = 0;  // stages issued by this CTA
  uint4 *trow = reinterpret_cast<uint4 *>(tile);
  const int npass = (27 + a.tpp - 1) / a.tpp;
  for (int pass = 0; pass < npass && !fail; ++pass) {
    const int t0 = pass * a.tpp, t1 = min(27, t0 + a.tpp);
    bool first = true;
    for (int b = blockIdx.x; b < a.nblocks && !fail; b += gridDim.x) {
      const int z0 = (b / nby) * a.BZ, y0 = (b % nby) * a.BY;
      // every MMA reading the previous tile must be complete before it is overwritten
      if (pend0) { fail |= !umma::mbar_wait(&bars[0], ph0, WS_WAIT_BUDGET); ph0 ^= 1u; pend0 = false; }
      if (pend1) { fail |= !umma::mbar_wait(&bars[1], ph1, WS_WAIT_BUDGET); ph1 ^= 1u; pend1 = false; }
      if (__syncthreads_or(fail)) { fail = true; break; }
      {
        const int nzy = (a.BZ + 2) * (a.BY + 2), nrows = kci * nzy, nwarps = blockDim.x >> 5;
        for (int row = warp; row < nrows; row += nwarps) {
          const int kc = row / nzy, rr = row - kc * nzy;
          const int tz = rr / (a.BY + 2), ty = rr - tz * (a.BY + 2);
          const int gz = z0 - 1 + tz, gy_ = y0 - 1 + ty;
          const bool rowin = (unsigned)gz < (unsigned)R && (unsigned)gy_ < (unsigned)R;
          const uint4 *src = a.x + (size_t)kc * R3 + ((size_t)(rowin ? gz : 0) * R + (rowin ? gy_ : 0)) * R;
          uint4 *dst = trow + (size_t)kc * V + (size_t)rr * W2;
          for (int tx = lane; tx < W2; tx += 32) {
            const int gx = tx - 1;
            const bool in = rowin && (unsigned)gx < (unsigned)R;
            umma::cp_async16(dst + tx, in ? (const void *)(src + gx) : (const void *)a.x, in);
          }
        }
      }
      for (int i = tid; i < 128; i += blockDim.x) trow[kci * V + i] = make_uint4(0u, 0u, 0u, 0u);
      for (int st = 0; st < nst; ++st, ++gs) {
        const int s = (int)(gs & 1);
        if (s ? pend1 : pend0) {
          fail |= !umma::mbar_wait(&bars[s], s ? ph1 : ph0, WS_WAIT_BUDGET);
          if (s) { ph1 ^= 1u; pend1 = false; } else { ph0 ^= 1u; pend0 = false; }
        }
        if (__syncthreads_or(fail)) { fail = true; break; }
        const int Ls = L0 + WG_STAGE_ROWS * st;
        uint8_t *sbuf = stg + s * WG_STAGE_BYTES;
        for (int i = tid; i < WG_STAGE_ROWS * kco; i += blockDim.x) {
          const int r = i % WG_STAGE_ROWS, c = i / WG_STAGE_ROWS;
          const int L = Ls + r;
          const int tz = L / P, rem = L - tz * P, ty = rem / W2, tx = rem - ty * W2;
          const bool valid = L <= L1 && tz >= 1 && tz <= a.BZ && ty >= 1 && ty <= a.BY && tx >= 1 && tx <= R;
          const uint4 *src =
              valid ? a.gy + (size_t)c * R3 + ((size_t)(z0 + tz - 1) * R + (y0 + ty - 1)) * R + (tx - 1) : a.gy;
          umma::cp_async16(sbuf + (r >> 3) * 2048 + c * 128 + (r & 7) * 16, src, valid);
        }
        umma::cp_async_wait_all();
        umma::fence_async_smem();
        __syncthreads();
        if (lane == 0 && warp < WS_ISSUERS) {  // issuer w owns the taps t0 + w (mod WS_ISSUERS)
          umma::tc_fence_after();
          const uint64_t ad0 = umma::sdesc_mn(stg_u32 + (uint32_t)s * WG_STAGE_BYTES, 2048u, 128u);
          const uint64_t bd0 = umma::sdesc_mn(tile_u32, 128u, (uint32_t)V * 16u);
          for (int t = t0 + warp; t < t1; t += WS_ISSUERS) {
            const int off = tap_offset(t, P, W2);
            for (int ks = 0; ks < WG_STAGE_ROWS / 16; ++ks) {
              umma::mma_bf16(tmem + (uint32_t)((t - t0) * a.Cin), ad0 + (uint32_t)ks * 256u,
                             bd0 + (uint32_t)(Ls + 16 * ks + off), idesc, (first && ks == 0) ? 0u : 1u);
            }
          }
          umma::mma_commit(&bars[s]);
        }
        if (s) pend1 = true; else pend0 = true;
        first = false;
      }
    }
    // pass complete: drain, then read the accumulators out
    if (pend0) { fail |= !umma::mbar_wait(&bars[0], ph0, WS_WAIT_BUDGET); ph0 ^= 1u; pend0 = false; }
    if (pend1) { fail |= !umma::mbar_wait(&bars[1], ph1, WS_WAIT_BUDGET); ph1 ^= 1u; pend1 = false; }
    fail = __syncthreads_or(fail);
    umma::tc_fence_after();
    if (!fail) {
      const int quad = warp & 3;
      const int co = 32 * quad + lane;
      for (int t = t0 + (warp >> 2); t < t1; t += (blockDim.x >> 7)) {
        if (32 * quad >= a.Cout) continue;  // whole warp idle: rows beyond Cout
        for (int c = 0; c < a.Cin; c += 16) {
          uint32_t r[16];
          umma::tmem_ld16(tmem + ((uint32_t)(32 * quad) << 16) + (uint32_t)((t - t0) * a.Cin + c), r);
          umma::tmem_wait_ld();
          if (co < a.Cout) {
            float *dst = a.part + (((size_t)blockIdx.x * 27 + t) * a.Cout + co) * a.Cin + c;
#pragma unroll
            for (int j = 0; j < 16; ++j) dst[j] = first ? 0.0f : __uint_as_float(r[j]);
          }
        }
      }
    }
    umma::tc_fence_before();
    __syncthreads();
  }
  if (fail) {
    if (pend0) umma::mbar_wait(&bars[0], ph0, WS_WAIT_BUDGET);
    if (pend1) umma::mbar_wait(&bars[1], ph1, WS_WAIT_BUDGET);
    if (tid == 0) atomicOr(a.status, 1u);
  }
  umma::tc_fence_before();
  __syncthreads();
  if (warp == 0) umma::tmem_dealloc(tmem, a.tmem_cols);
}

// out[e] = sum over c of part[c*nelem + e] for few elements and many partials:
// one block per element, a fixed strided split and a fixed tree (deterministic).
__global__ void __launch_bounds__(256) k_reduce_cols(const float *__restrict__ part, int nparts, int nelem,
                                                     float *__restrict__ out) {
  __shared__ float red[256];
  const int e = blockIdx.x;
  float s = 0.0f;
  for (int c = threadIdx.x; c < nparts; c += 256) s += part[(size_t)c * nelem + e];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[e] = red[0];
}

// dW[e] = sum over CTAs of the partials, in CTA order.
__global__ void __launch_bounds__(256) k_wgrad_reduce(const float *__restrict__ part, int nparts, int nelem,
                                                      float *__restrict__ dw) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nelem) return;
  float s = 0.0f;
  for (int c = 0; c < nparts; ++c) s += part[(size_t)c * nelem + e];
  dw[e] = s;
}

// ------------------------------------------------------------------------------
// elementwise network stages (bf16 chunk-planar activations)
// ------------------------------------------------------------------------------
// Coarse voxel (I,J,K) of an R/2 grid covers fine voxels (2I..2I+1, 2J.., 2K..).
// The elementwise kernels run one thread per voxel of a line: blockIdx.z = chunk *
// R_line + z, blockIdx.y = y, x from blockIdx.x (no index division).
__device__ __forceinline__ size_t child_index(int R, int I, int J, int K, int c) {
  return ((size_t)(2 * I + (c >> 2)) * R + (2 * J + ((c >> 1) & 1))) * R + (2 * K + (c & 1));
}

static dim3 line_grid(int Rl, int kc, int tpb) { return dim3((Rl + tpb - 1) / tpb, Rl, Rl * kc); }

// out (R/2) = mean of the 8 children of in (R)
__global__ void __launch_bounds__(64) k_pool2(const uint4 *__restrict__ in, uint4 *__restrict__ out, int R) {
  const int Rc = R >> 1;
  const int K = blockIdx.x * blockDim.x + threadIdx.x, J = blockIdx.y, c = blockIdx.z / Rc, I = blockIdx.z - c * Rc;
  if (K >= Rc) return;
  const size_t R3 = (size_t)R * R * R, Rc3 = (size_t)Rc * Rc * Rc;
  float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
  for (int ch = 0; ch < 8; ++ch) {
    float f[8];
    unpack8(__ldg(in + c * R3 + child_index(R, I, J, K, ch)), f);
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[j] += f[j];
  }
#pragma unroll
  for (int j = 0; j < 8; ++j) acc[j] *= 0.125f;
  out[c * Rc3 + ((size_t)I * Rc + J) * Rc + K] = pack8<0>(acc);
}

// out (R) = relu(u[parent] + skip)
__global__ void __launch_bounds__(64) k_up_add_relu(const uint4 *__restrict__ u, const uint4 *__restrict__ skip,
                                                    uint4 *__restrict__ out, int R) {
  const int Rc = R >> 1;
  const int z = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, c = blockIdx.z / R, x = blockIdx.z - c * R;
  if (z >= R) return;
  const size_t R3 = (size_t)R * R * R, Rc3 = (size_t)Rc * Rc * Rc;
  const size_t i = c * R3 + ((size_t)x * R + y) * R + z;
  float a[8], b[8];
  unpack8(__ldg(u + c * Rc3 + ((size_t)(x >> 1) * Rc + (y >> 1)) * Rc + (z >> 1)), a);
  unpack8(__ldg(skip + i), b);
#pragma unroll
  for (int j = 0; j < 8; ++j) a[j] = fmaxf(a[j] + b[j], 0.0f);
  out[i] = pack8<0>(a);
}

// out (R/2) = sum of the 8 children of g (R): adjoint of the nearest-neighbour upsample
__global__ void __launch_bounds__(64) k_up_adjoint(const uint4 *__restrict__ g, uint4 *__restrict__ out, int R) {
  const int Rc = R >> 1;
  const int K = blockIdx.x * blockDim.x + threadIdx.x, J = blockIdx.y, c = blockIdx.z / Rc, I = blockIdx.z - c * Rc;
  if (K >= Rc) return;
  const size_t R3 = (size_t)R * R * R, Rc3 = (size_t)Rc * Rc * Rc;
  float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
  for (int ch = 0; ch < 8; ++ch) {
    float f[8];
    unpack8(__ldg(g + c * R3 + child_index(R, I, J, K, ch)), f);
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[j] += f[j];
  }
  out[c * Rc3 + ((size_t)I * Rc + J) * Rc + K] = pack8<0>(acc);
}

// out (R) = (skipgrad + gp[parent] / 8) where act > 0, else 0: the gradient of an
// encoder activation that feeds both a skip connection and the average pool.
__global__ void __launch_bounds__(64) k_pool_adj_add_mask(const uint4 *__restrict__ skipgrad,
                                                          const uint4 *__restrict__ gp, const uint4 *__restrict__ act,
                                                          uint4 *__restrict__ out, int R) {
  const int Rc = R >> 1;
  const int z = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, c = blockIdx.z / R, x = blockIdx.z - c * R;
  if (z >= R) return;
  const size_t R3 = (size_t)R * R * R, Rc3 = (size_t)Rc * Rc * Rc;
  const size_t i = c * R3 + ((size_t)x * R + y) * R + z;
  float p[8], s[8], m[8];
  unpack8(__ldg(gp + c * Rc3 + ((size_t)(x >> 1) * Rc + (y >> 1)) * Rc + (z >> 1)), p);
  unpack8(__ldg(skipgrad + i), s);
  unpack8(__ldg(act + i), m);
#pragma unroll
  for (int j = 0; j < 8; ++j) p[j] = m[j] > 0.0f ? s[j] + 0.125f * p[j] : 0.0f;
  out[i] = pack8<0>(p);
}

// Per-block partial channel sums of g (C = 8*kc channels): part[block][C].
__global__ void __launch_bounds__(256) k_chan_sum(const uint4 *__restrict__ g, int kc, size_t R3,
                                                  float *__restrict__ part) {
  __shared__ float red[8][8];  // [warp][channel of the chunk]
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int c = 0; c < kc; ++c) {
    float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (size_t v = blockIdx.x * (size_t)blockDim.x + tid; v < R3; v += (size_t)gridDim.x * blockDim.x) {
      float f[8];
      unpack8(__ldg(g + (size_t)c * R3 + v), f);
#pragma unroll
      for (int j = 0; j < 8; ++j) acc[j] += f[j];
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) acc[j] += __shfl_xor_sync(0xffffffffu, acc[j], o);
    }
    if (lane == 0) {
#pragma unroll
      for (int j = 0; j < 8; ++j) red[warp][j] = acc[j];
    }
    __syncthreads();
    if (tid < 8) {
      float s = 0.0f;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w][tid];
      part[(size_t)blockIdx.x * (8 * kc) + 8 * c + tid] = s;
    }
    __syncthreads();
  }
}

// Network input: channels 0..3 from f16 planar features [4][R^3]; channels 4..15 zero.
__global__ void __launch_bounds__(256) k_pack_input(const __half *__restrict__ feat, uint4 *__restrict__ x0, size_t R3) {
  for (size_t v = blockIdx.x * (size_t)blockDim.x + threadIdx.x; v < R3; v += (size_t)gridDim.x * blockDim.x) {
    float f[8] = {__half2float(feat[v]), __half2float(feat[R3 + v]), __half2float(feat[2 * R3 + v]),
                  __half2float(feat[3 * R3 + v]), 0, 0, 0, 0};
    x0[v] = pack8<0>(f);
    x0[R3 + v] = make_uint4(0u, 0u, 0u, 0u);
  }
}

// Loss 0.5 * mean((y - t)^2) over R^3 and its gradient dL/dy (channel 0 of a
// 16-channel bf16 tensor, other channels zero). Per-block partial loss sums.
__global__ void __launch_bounds__(256) k_mse(const float *__restrict__ y, const __half *__restrict__ t, size_t R3,
                                             uint4 *__restrict__ gy, float *__restrict__ part) {
  __shared__ float red[8];
  const float inv_n = 1.0f / (float)R3;
  float acc = 0.0f;
  for (size_t v = blockIdx.x * (size_t)blockDim.x + threadIdx.x; v < R3; v += (size_t)gridDim.x * blockDim.x) {
    const float d = y[v] - __half2float(t[v]);
    acc += d * d;
    float f[8] = {d * inv_n, 0, 0, 0, 0, 0, 0, 0};
    gy[v] = pack8<0>(f);
    gy[R3 + v] = make_uint4(0u, 0u, 0u, 0u);
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    float s = 0.0f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
    part[blockIdx.x] = 0.5f * s * inv_n;
  }
}

// ------------------------------------------------------------------------------
// parameters: Adam and the bf16 packing of the weights
// ------------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_adam(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m,
                                              float *__restrict__ v, size_t n, float lr, float b1, float b2, float eps,
                                              float bc1, float bc2) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
  }
}

// W (f32 [27][Cout][Cin]) -> forward operand [27][Cin/8][Cout][8] and data-gradient
// operand [27][Cout/8][Cin][8] with the tap mirrored (t' = 26 - t).
__global__ void __launch_bounds__(256) k_pack_weights(const float *__restrict__ W, int Cin, int Cout,
                                                      uint16_t *__restrict__ wf, uint16_t *__restrict__ wb) {
  const int n = 27 * Cout * Cin;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int t = i / (Cout * Cin), rem = i - t * Cout * Cin, co = rem / Cin, ci = rem - co * Cin;
    const uint32_t u = bf_pack(W[i], 0.0f) & 0xffffu;
    wf[(((size_t)t * (Cin >> 3) + (ci >> 3)) * Cout + co) * 8 + (ci & 7)] = (uint16_t)u;
    wb[(((size_t)(26 - t) * (Cout >> 3) + (co >> 3)) * Cin + ci) * 8 + (co & 7)] = (uint16_t)u;
  }
}

// ------------------------------------------------------------------------------
// the network object
// ------------------------------------------------------------------------------
// Encoder-decoder over 4 levels (R, R/2, R/4, R/8) with 16-32-64-128 channels:
//   e0 = relu(A x0)            p1 = pool(e0)   e1 = relu(B p1)   p2 = pool(e1)
//   e2 = relu(C p2)            p3 = pool(e2)   e3 = relu(D p3)
//   u2 = E e3                  d2 = relu(up(u2) + e2)            f2 = relu(F d2)
//   u1 = G f2                  d1 = relu(up(u1) + e1)            f1 = relu(H d1)
//   u0 = I f1                  d0 = relu(up(u0) + e0)            f0 = relu(J d0)
//   y  = K f0 (channel 0)
// every capital a 3x3x3 convolution with bias (zero padding), pool a 2x2x2 mean,
// up a nearest-neighbour doubling. x0 has 16 channels, 3 in use.
#define WS_NL 11
static const int kWsLayer[WS_NL][4] = {  // cin, cout, level, relu
    {16, 16, 0, 1}, {16, 32, 1, 1}, {32, 64, 2, 1}, {64, 128, 3, 1}, {128, 64, 3, 0}, {64, 64, 2, 1},
    {64, 32, 2, 0}, {32, 32, 1, 1}, {32, 16, 1, 0}, {16, 16, 0, 1}, {16, 16, 0, 0}};

struct FwdPlan {
  int BZ, BY, tpg, n_mt, grid;
  uint32_t cols;
  size_t smem;
};
struct WgPlan {
  int BZ, BY, tpp, nblocks, grid;
  uint32_t cols;
  size_t smem;
};

struct gc_ws {
  int R;
  int device;
  cudaStream_t stream;
  size_t nparams;
  size_t w_off[WS_NL], b_off[WS_NL];
  float *params, *grads, *adam_m, *adam_v;
  uint16_t *wf[WS_NL], *wb[WS_NL];
  FwdPlan pf[WS_NL], pb[WS_NL];
  WgPlan pw[WS_NL];
  void *arena;
  uint4 *x0, *e0, *d0, *f0, *gy, *g_f0, *g_d0, *g_e0;
  uint4 *p1, *e1, *u0, *d1, *f1, *g_u0, *g_f1, *g_d1, *g_p1, *g_e1;
  uint4 *p2, *e2, *u1, *d2, *f2, *g_u1, *g_f2, *g_d2, *g_p2, *g_e2;
  uint4 *p3, *e3, *u2, *g_u2, *g_e3, *g_p3;
  float *y;
  float *part;
  size_t part_cap;
  float *cpart;
  float *lpart;
  float *loss;
  unsigned *status;
  int sm_count;
  char err[256];
};

static int ws_fail(gc_ws *ws, int code, const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(ws->err, sizeof(ws->err), fmt, ap);
  va_end(ap);
  return code;
}
#define WS_CUDA(ws, call)                                                                        \
  do {                                                                                           \
    cudaError_t e_ = (call);                                                                     \
    if (e_ != cudaSuccess) return ws_fail(ws, GC_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

static uint32_t pow2_cols(int c) {
  uint32_t n = 32;
  while ((int)n < c) n <<= 1;
  return n;
}

// Shared memory that leaves at most `k` CTAs on an SM (so their Tensor Memory fits).
static size_t smem_for_residency(size_t smem, int k) {
  const size_t per_sm = 233472, reserve = 1024;
  const size_t need = per_sm / (size_t)(k + 1) - reserve + 1;
  return std::max(smem, need);
}

static const size_t WS_SMEM_MAX = 232448;

// Tile plans of the forward kernel. Every feasible (BZ, BY) is enumerated; the
// default pick minimises a cycle estimate per SM -- staging the input tile (L2 ->
// shared, ~64 B/clk), the MMAs (one 128 x Cout x 16 step every max(8,
// 128*Cout*16/4096) clocks, issued by four threads) and the epilogue, with at
// most `occ` CTAs overlapping on an SM -- and gc_ws_autotune replaces it by the
// fastest measured candidate.
static std::vector<FwdPlan> enum_fwd(int R, int Cin, int Cout, int sm_count, std::vector<double> *costs) {
  std::vector<FwdPlan> out;
  const int bys[] = {32, 16, 8, 4, 2, 1};
  const int bzs[] = {1, 2, 4, 8};
  for (int BY : bys) {
    if (BY > R || R % BY) continue;
    for (int BZ : bzs) {
      if (BZ > R || R % BZ) continue;
      int W2, P, V, L0, L1;
      conv_geom(R, BZ, BY, W2, P, V, L0, L1);
      const int n_mt = (L1 - L0 + 128) / 128;
      if (n_mt * Cout > 512) continue;
      const size_t tile = (((size_t)(Cin / 8) * V + 128) * 16 + 1023) & ~(size_t)1023;
      const size_t tap = (size_t)Cin * Cout * 2;
      if (tile + 2 * tap + 64 > WS_SMEM_MAX) continue;
      const int tpg = (int)std::min<size_t>(27, (WS_SMEM_MAX - tile - 64) / (2 * tap));
      const int ngroups = (27 + tpg - 1) / tpg;
      const int tpg_even = (27 + ngroups - 1) / ngroups;
      const size_t smem = tile + 2 * (size_t)tpg_even * tap + 64;
      FwdPlan p;
      p.BZ = BZ; p.BY = BY; p.tpg = tpg_even; p.n_mt = n_mt; p.grid = (R / BZ) * (R / BY);
      p.cols = pow2_cols(n_mt * Cout);
      p.smem = smem_for_residency(smem, (int)(512 / p.cols));
      out.push_back(p);
      if (costs) {
        const int occ = std::max(1, std::min(8, (int)(233472 / (p.smem + 1024))));
        const double load = (double)(Cin / 8) * V * 16 / 64.0 + (double)27 * tap / 64.0;
        const double mma = 27.0 * n_mt * (Cin / 16) * std::max(8.0, 128.0 * Cout * 16 / 4096.0) / 4.0 + 300.0;
        const double epi = (double)n_mt * 128 * Cout * 2 / 64.0;
        const double per_cta = load + mma + epi + 2000.0;
        const double busiest = std::max(load, std::max(mma, epi));
        const double waves = std::ceil((double)p.grid / (sm_count * occ));
        costs->push_back(waves * std::max(per_cta, occ * busiest));
      }
    }
  }
  return out;
}

static bool plan_fwd(int R, int Cin, int Cout, int sm_count, FwdPlan &best) {
  std::vector<double> cost;
  const std::vector<FwdPlan> c = enum_fwd(R, Cin, Cout, sm_count, &cost);
  if (c.empty()) return false;
  size_t k = 0;
  for (size_t i = 1; i < c.size(); ++i)
    if (cost[i] < cost[k]) k = i;
  best = c[k];
  return true;
}

static std::vector<WgPlan> enum_wgrad(int R, int Cin, int Cout, int sm_count, std::vector<double> *scores) {
  std::vector<WgPlan> out;
  const int bys[] = {32, 16, 8, 4, 2, 1};
  const int bzs[] = {1, 2, 4};
  const int tpp = std::min(27, 512 / Cin);
  const uint32_t cols = pow2_cols(tpp * Cin);
  for (int BY : bys) {
    if (BY > R || R % BY) continue;
    for (int BZ : bzs) {
      if (BZ > R || R % BZ) continue;
      int W2, P, V, L0, L1;
      conv_geom(R, BZ, BY, W2, P, V, L0, L1);
      const size_t tile = (((size_t)(Cin / 8) * V + 128) * 16 + 1023) & ~(size_t)1023;
      const size_t smem = tile + 2 * WG_STAGE_BYTES + 64;
      if (smem > WS_SMEM_MAX) continue;
      const int nst = (L1 - L0 + WG_STAGE_ROWS) / WG_STAGE_ROWS;
      WgPlan p;
      p.BZ = BZ; p.BY = BY; p.tpp = tpp; p.nblocks = (R / BZ) * (R / BY); p.cols = cols;
      p.smem = smem_for_residency(smem, (int)(512 / cols));
      const int per_sm = std::max(1, (int)(233472 / (p.smem + 1024)));
      p.grid = std::min(p.nblocks, sm_count * per_sm);
      out.push_back(p);
      if (scores) {
        const double useful = (double)BZ * BY * R / (128.0 * nst);
        const double fill = std::min(1.0, (double)p.nblocks / (double)sm_count);
        const double reload = (double)(BZ * BY) / ((BZ + 2.0) * (BY + 2.0));
        scores->push_back(useful * fill * (0.5 + 0.5 * reload));
      }
    }
  }
  return out;
}

static bool plan_wgrad(int R, int Cin, int Cout, int sm_count, WgPlan &best) {
  std::vector<double> sc;
  const std::vector<WgPlan> c = enum_wgrad(R, Cin, Cout, sm_count, &sc);
  if (c.empty()) return false;
  size_t k = 0;
  for (size_t i = 1; i < c.size(); ++i)
    if (sc[i] > sc[k]) k = i;
  best = c[k];
  return true;
}

static unsigned ew_blocks(size_t n, int sm_count) {
  size_t b = (n + 255) / 256;
  const size_t cap = (size_t)sm_count * 8;
  if (b > cap) b = cap;
  return (unsigned)std::max<size_t>(1, b);
}

static int ws_conv(gc_ws *ws, const FwdPlan &p, int R, int Cin, int Cout, const uint4 *in, const uint16_t *w,
                   const float *bias, const uint4 *skip, const uint4 *mask, uint4 *out, float *out_f32, int relu) {
  ConvFwd a;
  a.in = in; a.w = reinterpret_cast<const uint4 *>(w); a.bias = bias; a.skip = skip; a.mask = mask;
  a.out = out; a.out_f32 = out_f32; a.status = ws->status;
  a.R = R; a.Cin = Cin; a.Cout = Cout; a.BZ = p.BZ; a.BY = p.BY; a.relu = relu; a.tpg = p.tpg; a.n_mt = p.n_mt;
  a.tmem_cols = p.cols;
  k_conv_fwd<<<p.grid, 256, p.smem, ws->stream>>>(a);
  WS_CUDA(ws, cudaGetLastError());
  return GC_OK;
}

static int ws_wgrad(gc_ws *ws, int l, const uint4 *x, const uint4 *gy) {
  const int Cin = kWsLayer[l][0], Cout = kWsLayer[l][1], R = ws->R >> kWsLayer[l][2];
  const WgPlan &p = ws->pw[l];
  ConvW a;
  a.x = x; a.gy = gy; a.part = ws->part; a.status = ws->status;
  a.R = R; a.Cin = Cin; a.Cout = Cout; a.BZ = p.BZ; a.BY = p.BY; a.tpp = p.tpp; a.nblocks = p.nblocks;
  a.tmem_cols = p.cols;
  k_conv_wgrad<<<p.grid, 256, p.smem, ws->stream>>>(a);
  WS_CUDA(ws, cudaGetLastError());
  const int nelem = 27 * Cout * Cin;
  k_wgrad_reduce<<<(nelem + 255) / 256, 256, 0, ws->stream>>>(ws->part, p.grid, nelem, ws->grads + ws->w_off[l]);
  WS_CUDA(ws, cudaGetLastError());
  // bias gradient: channel sums of gy
  const size_t R3 = (size_t)R * R * R;
  const unsigned nb = std::min<unsigned>(ew_blocks(R3, ws->sm_count), 1024u);
  k_chan_sum<<<nb, 256, 0, ws->stream>>>(gy, Cout / 8, R3, ws->cpart);
  k_reduce_cols<<<Cout, 256, 0, ws->stream>>>(ws->cpart, (int)nb, Cout, ws->grads + ws->b_off[l]);
  WS_CUDA(ws, cudaGetLastError());
  return GC_OK;
}

static int ws_fwd_layer(gc_ws *ws, int l, const uint4 *in, const uint4 *skip, uint4 *out, float *out_f32) {
  const int R = ws->R >> kWsLayer[l][2];
  return ws_conv(ws, ws->pf[l], R, kWsLayer[l][0], kWsLayer[l][1], in, ws->wf[l], ws->params + ws->b_off[l], skip,
                 nullptr, out, out_f32, kWsLayer[l][3]);
}

// data gradient of layer l: conv of g (Cout channels) with the mirrored weights,
// optionally masked by (act > 0)
static int ws_dgrad(gc_ws *ws, int l, const uint4 *g, const uint4 *mask_act, uint4 *out) {
  const int R = ws->R >> kWsLayer[l][2];
  return ws_conv(ws, ws->pb[l], R, kWsLayer[l][1], kWsLayer[l][0], g, ws->wb[l], nullptr, nullptr, mask_act, out,
                 nullptr, 0);
}

extern "C" int gc_ws_layer_info(int layer, int *cin, int *cout, int *level, int *relu) {
  if (layer < 0 || layer >= WS_NL) return GC_ERR_ARG;
  if (cin) *cin = kWsLayer[layer][0];
  if (cout) *cout = kWsLayer[layer][1];
  if (level) *level = kWsLayer[layer][2];
  if (relu) *relu = kWsLayer[layer][3];
  return GC_OK;
}

extern "C" int gc_ws_create(gc_ws **out, int R) {
  if (!out) return GC_ERR_ARG;
  *out = nullptr;
  if (R < 16 || R > 512 || (R % 8)) return GC_ERR_ARG;
  gc_ws *ws = new (std::nothrow) gc_ws();
  if (!ws) return GC_ERR_CUDA;
  memset(ws, 0, sizeof(*ws));
  ws->R = R;
  cudaGetDevice(&ws->device);
  cudaDeviceGetAttribute(&ws->sm_count, cudaDevAttrMultiProcessorCount, ws->device);
  if (ws->sm_count <= 0) ws->sm_count = (int)gc_sms();
  size_t off = 0;
  for (int l = 0; l < WS_NL; ++l) {
    ws->w_off[l] = off;
    off += (size_t)27 * kWsLayer[l][0] * kWsLayer[l][1];
    ws->b_off[l] = off;
    off += kWsLayer[l][1];
  }
  ws->nparams = off;
  size_t wbytes = 0;
  for (int l = 0; l < WS_NL; ++l) wbytes += (size_t)27 * kWsLayer[l][0] * kWsLayer[l][1] * 2 * 2;
  int rc = GC_OK;
  auto fail = [&](const char *what) {
    snprintf(ws->err, sizeof(ws->err), "gc_ws_create: %s", what);
    rc = GC_ERR_CUDA;
  };
  if (cudaMalloc(&ws->params, 4 * ws->nparams * sizeof(float)) != cudaSuccess) fail("parameters");
  if (rc == GC_OK) {
    ws->grads = ws->params + ws->nparams;
    ws->adam_m = ws->grads + ws->nparams;
    ws->adam_v = ws->adam_m + ws->nparams;
    cudaMemset(ws->params, 0, 4 * ws->nparams * sizeof(float));
  }
  uint16_t *wall = nullptr;
  if (rc == GC_OK && cudaMalloc(&wall, wbytes) != cudaSuccess) fail("bf16 weights");
  if (rc == GC_OK) {
    cudaMemset(wall, 0, wbytes);
    for (int l = 0; l < WS_NL; ++l) {
      const size_t nw = (size_t)27 * kWsLayer[l][0] * kWsLayer[l][1];
      ws->wf[l] = wall;
      ws->wb[l] = wall + nw;
      wall += 2 * nw;
    }
  }
  // activations
  const size_t R3[4] = {(size_t)R * R * R, (size_t)R * R * R / 8, (size_t)R * R * R / 64, (size_t)R * R * R / 512};
  struct Req { uint4 **p; int ch; int lev; };
  const Req reqs[] = {
      {&ws->x0, 16, 0}, {&ws->e0, 16, 0}, {&ws->d0, 16, 0}, {&ws->f0, 16, 0}, {&ws->gy, 16, 0}, {&ws->g_f0, 16, 0},
      {&ws->g_d0, 16, 0}, {&ws->g_e0, 16, 0},
      {&ws->p1, 16, 1}, {&ws->e1, 32, 1}, {&ws->u0, 16, 1}, {&ws->d1, 32, 1}, {&ws->f1, 32, 1}, {&ws->g_u0, 16, 1},
      {&ws->g_f1, 32, 1}, {&ws->g_d1, 32, 1}, {&ws->g_p1, 16, 1}, {&ws->g_e1, 32, 1},
      {&ws->p2, 32, 2}, {&ws->e2, 64, 2}, {&ws->u1, 32, 2}, {&ws->d2, 64, 2}, {&ws->f2, 64, 2}, {&ws->g_u1, 32, 2},
      {&ws->g_f2, 64, 2}, {&ws->g_d2, 64, 2}, {&ws->g_p2, 32, 2}, {&ws->g_e2, 64, 2},
      {&ws->p3, 64, 3}, {&ws->e3, 128, 3}, {&ws->u2, 64, 3}, {&ws->g_u2, 64, 3}, {&ws->g_e3, 128, 3},
      {&ws->g_p3, 64, 3}};
  size_t abytes = 0;
  for (const Req &q : reqs) abytes += ((R3[q.lev] * (q.ch / 8) * 16 + 255) & ~(size_t)255);
  abytes += ((R3[0] * 4 + 255) & ~(size_t)255);  // y
  if (rc == GC_OK && cudaMalloc(&ws->arena, abytes) != cudaSuccess) fail("activations");
  if (rc == GC_OK) {
    cudaMemset(ws->arena, 0, abytes);
    uint8_t *p = (uint8_t *)ws->arena;
    for (const Req &q : reqs) {
      *q.p = (uint4 *)p;
      p += ((R3[q.lev] * (q.ch / 8) * 16 + 255) & ~(size_t)255);
    }
    ws->y = (float *)p;
  }
  // plans
  for (int l = 0; l < WS_NL && rc == GC_OK; ++l) {
    const int Rl = R >> kWsLayer[l][2];
    if (!plan_fwd(Rl, kWsLayer[l][0], kWsLayer[l][1], ws->sm_count, ws->pf[l]) ||
        !plan_fwd(Rl, kWsLayer[l][1], kWsLayer[l][0], ws->sm_count, ws->pb[l]) ||
        !plan_wgrad(Rl, kWsLayer[l][0], kWsLayer[l][1], ws->sm_count, ws->pw[l])) {
      snprintf(ws->err, sizeof(ws->err), "gc_ws_create: no tile plan for layer %d", l);
      rc = GC_ERR_ARG;
    }
  }
  size_t part = 0;  // weight-gradient partials: the largest grid any candidate plan may use
  for (int l = 0; l < WS_NL && rc == GC_OK; ++l) {
    const int Rl = R >> kWsLayer[l][2];
    for (const WgPlan &c : enum_wgrad(Rl, kWsLayer[l][0], kWsLayer[l][1], ws->sm_count, nullptr))
      part = std::max(part, (size_t)c.grid * 27 * kWsLayer[l][0] * kWsLayer[l][1]);
  }
  ws->part_cap = part;
  if (rc == GC_OK && cudaMalloc(&ws->part, part * sizeof(float) + (size_t)(1024 * 128 + 1024 + 16) * sizeof(float) +
                                               64) != cudaSuccess)
    fail("partials");
  if (rc == GC_OK) {
    ws->cpart = ws->part + part;
    ws->lpart = ws->cpart + 1024 * 128;
    ws->loss = ws->lpart + 1024;
    ws->status = (unsigned *)(ws->loss + 8);
    cudaMemset(ws->status, 0, sizeof(unsigned));
  }
  if (rc == GC_OK) {
    if (cudaFuncSetAttribute(k_conv_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)WS_SMEM_MAX) != cudaSuccess ||
        cudaFuncSetAttribute(k_conv_wgrad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)WS_SMEM_MAX) !=
            cudaSuccess)
      fail("shared memory attribute");
  }
  if (rc != GC_OK) {
    char msg[256];
    memcpy(msg, ws->err, sizeof(msg));
    gc_ws_destroy(ws);
    fprintf(stderr, "%s\n", msg);
    return rc;
  }
  *out = ws;
  return GC_OK;
}

extern "C" int gc_ws_destroy(gc_ws *ws) {
  if (!ws) return GC_OK;
  if (ws->params) cudaFree(ws->params);
  if (ws->wf[0]) cudaFree(ws->wf[0]);
  if (ws->arena) cudaFree(ws->arena);
  if (ws->part) cudaFree(ws->part);
  delete ws;
  return GC_OK;
}

extern "C" const char *gc_ws_last_error(const gc_ws *ws) { return ws ? ws->err : "null warm-start object"; }

extern "C" int gc_ws_set_stream(gc_ws *ws, void *stream) {
  if (!ws) return GC_ERR_ARG;
  ws->stream = (cudaStream_t)stream;
  return GC_OK;
}

extern "C" int gc_ws_num_params(const gc_ws *ws, int64_t *n) {
  if (!ws || !n) return GC_ERR_ARG;
  *n = (int64_t)ws->nparams;
  return GC_OK;
}

static int ws_repack(gc_ws *ws) {
  for (int l = 0; l < WS_NL; ++l) {
    const int n = 27 * kWsLayer[l][0] * kWsLayer[l][1];
    k_pack_weights<<<(n + 255) / 256, 256, 0, ws->stream>>>(ws->params + ws->w_off[l], kWsLayer[l][0], kWsLayer[l][1],
                                                            ws->wf[l], ws->wb[l]);
  }
  WS_CUDA(ws, cudaGetLastError());
  return GC_OK;
}

extern "C" int gc_ws_set_params(gc_ws *ws, const float *params) {
  if (!ws || !params) return GC_ERR_ARG;
  WS_CUDA(ws, cudaMemcpyAsync(ws->params, params, ws->nparams * sizeof(float), cudaMemcpyDeviceToDevice, ws->stream));
  WS_CUDA(ws, cudaMemsetAsync(ws->adam_m, 0, 2 * ws->nparams * sizeof(float), ws->stream));
  return ws_repack(ws);
}

extern "C" int gc_ws_get_params(gc_ws *ws, float *params) {
  if (!ws || !params) return GC_ERR_ARG;
  WS_CUDA(ws, cudaMemcpyAsync(params, ws->params, ws->nparams * sizeof(float), cudaMemcpyDeviceToDevice, ws->stream));
  return GC_OK;
}

extern "C" int gc_ws_get_grads(gc_ws *ws, float *grads) {
  if (!ws || !grads) return GC_ERR_ARG;
  WS_CUDA(ws, cudaMemcpyAsync(grads, ws->grads, ws->nparams * sizeof(float), cudaMemcpyDeviceToDevice, ws->stream));
  return GC_OK;
}

extern "C" int gc_ws_status(gc_ws *ws, unsigned *flags, int clear) {
  if (!ws || !flags) return GC_ERR_ARG;
  WS_CUDA(ws, cudaMemcpyAsync(flags, ws->status, sizeof(unsigned), cudaMemcpyDeviceToHost, ws->stream));
  WS_CUDA(ws, cudaStreamSynchronize(ws->stream));
  if (clear) WS_CUDA(ws, cudaMemsetAsync(ws->status, 0, sizeof(unsigned), ws->stream));
  return GC_OK;
}

static int ws_forward_packed(gc_ws *ws, float *y_out) {
  const int R = ws->R;
  int s;
  if ((s = ws_fwd_layer(ws, 0, ws->x0, nullptr, ws->e0, nullptr))) return s;
  k_pool2<<<line_grid(R / 2, 2, 64), 64, 0, ws->stream>>>(ws->e0, ws->p1, R);
  if ((s = ws_fwd_layer(ws, 1, ws->p1, nullptr, ws->e1, nullptr))) return s;
  k_pool2<<<line_grid(R / 4, 4, 64), 64, 0, ws->stream>>>(ws->e1, ws->p2, R / 2);
  if ((s = ws_fwd_layer(ws, 2, ws->p2, nullptr, ws->e2, nullptr))) return s;
  k_pool2<<<line_grid(R / 8, 8, 64), 64, 0, ws->stream>>>(ws->e2, ws->p3, R / 4);
  if ((s = ws_fwd_layer(ws, 3, ws->p3, nullptr, ws->e3, nullptr))) return s;
  if ((s = ws_fwd_layer(ws, 4, ws->e3, nullptr, ws->u2, nullptr))) return s;
  k_up_add_relu<<<line_grid(R / 4, 8, 64), 64, 0, ws->stream>>>(ws->u2, ws->e2, ws->d2, R / 4);
  if ((s = ws_fwd_layer(ws, 5, ws->d2, nullptr, ws->f2, nullptr))) return s;
  if ((s = ws_fwd_layer(ws, 6, ws->f2, nullptr, ws->u1, nullptr))) return s;
  k_up_add_relu<<<line_grid(R / 2, 4, 64), 64, 0, ws->stream>>>(ws->u1, ws->e1, ws->d1, R / 2);
  if ((s = ws_fwd_layer(ws, 7, ws->d1, nullptr, ws->f1, nullptr))) return s;
  if ((s = ws_fwd_layer(ws, 8, ws->f1, nullptr, ws->u0, nullptr))) return s;
  k_up_add_relu<<<line_grid(R, 2, 64), 64, 0, ws->stream>>>(ws->u0, ws->e0, ws->d0, R);
  if ((s = ws_fwd_layer(ws, 9, ws->d0, nullptr, ws->f0, nullptr))) return s;
  if ((s = ws_fwd_layer(ws, 10, ws->f0, nullptr, nullptr, y_out ? y_out : ws->y))) return s;
  WS_CUDA(ws, cudaGetLastError());
  return GC_OK;
}

extern "C" int gc_ws_forward(gc_ws *ws, const void *feat, float *y_out) {
  if (!ws || !feat) return GC_ERR_ARG;
  const size_t R3 = (size_t)ws->R * ws->R * ws->R;
  k_pack_input<<<ew_blocks(R3, ws->sm_count), 256, 0, ws->stream>>>((const __half *)feat, ws->x0, R3);
  WS_CUDA(ws, cudaGetLastError());
  int s = ws_forward_packed(ws, ws->y);
  if (s) return s;
  if (y_out) WS_CUDA(ws, cudaMemcpyAsync(y_out, ws->y, R3 * sizeof(float), cudaMemcpyDeviceToDevice, ws->stream));
  return GC_OK;
}

extern "C" int gc_ws_backward(gc_ws *ws, const void *target, float *loss_out) {
  if (!ws || !target) return GC_ERR_ARG;
  const int R = ws->R;
  const size_t R3 = (size_t)R * R * R;
  const int sm = ws->sm_count;
  int s;
  const unsigned nl = std::min<unsigned>(ew_blocks(R3, sm), 1024u);
  k_mse<<<nl, 256, 0, ws->stream>>>(ws->y, (const __half *)target, R3, ws->gy, ws->lpart);
  k_reduce_cols<<<1, 256, 0, ws->stream>>>(ws->lpart, (int)nl, 1, ws->loss);
  WS_CUDA(ws, cudaGetLastError());
  // K, J
  if ((s = ws_wgrad(ws, 10, ws->f0, ws->gy))) return s;
  if ((s = ws_dgrad(ws, 10, ws->gy, ws->f0, ws->g_f0))) return s;
  if ((s = ws_wgrad(ws, 9, ws->d0, ws->g_f0))) return s;
  if ((s = ws_dgrad(ws, 9, ws->g_f0, ws->d0, ws->g_d0))) return s;
  k_up_adjoint<<<line_grid(R / 2, 2, 64), 64, 0, ws->stream>>>(ws->g_d0, ws->g_u0, R);
  // I, H
  if ((s = ws_wgrad(ws, 8, ws->f1, ws->g_u0))) return s;
  if ((s = ws_dgrad(ws, 8, ws->g_u0, ws->f1, ws->g_f1))) return s;
  if ((s = ws_wgrad(ws, 7, ws->d1, ws->g_f1))) return s;
  if ((s = ws_dgrad(ws, 7, ws->g_f1, ws->d1, ws->g_d1))) return s;
  k_up_adjoint<<<line_grid(R / 4, 4, 64), 64, 0, ws->stream>>>(ws->g_d1, ws->g_u1, R / 2);
  // G, F
  if ((s = ws_wgrad(ws, 6, ws->f2, ws->g_u1))) return s;
  if ((s = ws_dgrad(ws, 6, ws->g_u1, ws->f2, ws->g_f2))) return s;
  if ((s = ws_wgrad(ws, 5, ws->d2, ws->g_f2))) return s;
  if ((s = ws_dgrad(ws, 5, ws->g_f2, ws->d2, ws->g_d2))) return s;
  k_up_adjoint<<<line_grid(R / 8, 8, 64), 64, 0, ws->stream>>>(ws->g_d2, ws->g_u2, R / 4);
  // E, D
  if ((s = ws_wgrad(ws, 4, ws->e3, ws->g_u2))) return s;
  if ((s = ws_dgrad(ws, 4, ws->g_u2, ws->e3, ws->g_e3))) return s;
  if ((s = ws_wgrad(ws, 3, ws->p3, ws->g_e3))) return s;
  if ((s = ws_dgrad(ws, 3, ws->g_e3, nullptr, ws->g_p3))) return s;
  k_pool_adj_add_mask<<<line_grid(R / 4, 8, 64), 64, 0, ws->stream>>>(ws->g_d2, ws->g_p3, ws->e2, ws->g_e2, R / 4);
  // C
  if ((s = ws_wgrad(ws, 2, ws->p2, ws->g_e2))) return s;
  if ((s = ws_dgrad(ws, 2, ws->g_e2, nullptr, ws->g_p2))) return s;
  k_pool_adj_add_mask<<<line_grid(R / 2, 4, 64), 64, 0, ws->stream>>>(ws->g_d1, ws->g_p2, ws->e1, ws->g_e1, R / 2);
  // B
  if ((s = ws_wgrad(ws, 1, ws->p1, ws->g_e1))) return s;
  if ((s = ws_dgrad(ws, 1, ws->g_e1, nullptr, ws->g_p1))) return s;
  k_pool_adj_add_mask<<<line_grid(R, 2, 64), 64, 0, ws->stream>>>(ws->g_d0, ws->g_p1, ws->e0, ws->g_e0, R);
  // A
  if ((s = ws_wgrad(ws, 0, ws->x0, ws->g_e0))) return s;
  WS_CUDA(ws, cudaGetLastError());
  if (loss_out) WS_CUDA(ws, cudaMemcpyAsync(loss_out, ws->loss, sizeof(float), cudaMemcpyDeviceToDevice, ws->stream));
  return GC_OK;
}

// ---- autotuner --------------------------------------------------------------------
// Buffers each layer reads and writes in the forward, data-gradient and
// weight-gradient passes (the autotuner times candidates on them).
struct WsBufs {
  const uint4 *in;
  uint4 *out;
  const uint4 *mask;
  float *outf;
};
static WsBufs fwd_bufs(gc_ws *ws, int l) {
  const uint4 *in[WS_NL] = {ws->x0, ws->p1, ws->p2, ws->p3, ws->e3, ws->d2, ws->f2, ws->d1, ws->f1, ws->d0, ws->f0};
  uint4 *out[WS_NL] = {ws->e0, ws->e1, ws->e2, ws->e3, ws->u2, ws->f2, ws->u1, ws->f1, ws->u0, ws->f0, nullptr};
  return {in[l], out[l], nullptr, l == WS_NL - 1 ? ws->y : nullptr};
}
static WsBufs dgrad_bufs(gc_ws *ws, int l) {  // l >= 1
  const uint4 *in[WS_NL] = {nullptr, ws->g_e1, ws->g_e2, ws->g_e3, ws->g_u2, ws->g_f2, ws->g_u1, ws->g_f1, ws->g_u0,
                            ws->g_f0, ws->gy};
  uint4 *out[WS_NL] = {nullptr, ws->g_p1, ws->g_p2, ws->g_p3, ws->g_e3, ws->g_d2, ws->g_f2, ws->g_d1, ws->g_f1,
                       ws->g_d0, ws->g_f0};
  const uint4 *mask[WS_NL] = {nullptr, nullptr, nullptr, nullptr, ws->e3, ws->d2, ws->f2, ws->d1, ws->f1, ws->d0,
                              ws->f0};
  return {in[l], out[l], mask[l], nullptr};
}
static WsBufs wgrad_bufs(gc_ws *ws, int l) {  // in = layer input, mask = output gradient
  const uint4 *x[WS_NL] = {ws->x0, ws->p1, ws->p2, ws->p3, ws->e3, ws->d2, ws->f2, ws->d1, ws->f1, ws->d0, ws->f0};
  const uint4 *g[WS_NL] = {ws->g_e0, ws->g_e1, ws->g_e2, ws->g_e3, ws->g_u2, ws->g_f2, ws->g_u1, ws->g_f1, ws->g_u0,
                           ws->g_f0, ws->gy};
  return {x[l], nullptr, g[l], nullptr};
}

// Time every feasible tile plan of every layer's three passes (CUDA events,
// `iters` launches after one untimed) and keep the fastest. Activations are
// overwritten. ms_out (host, nullable) receives the best time per pass,
// [layer][forward, data gradient, weight gradient], 0 where a pass does not exist.
extern "C" int gc_ws_autotune(gc_ws *ws, int iters, float *ms_out) {
  if (!ws || iters < 1) return GC_ERR_ARG;
  cudaEvent_t ev0, ev1;
  WS_CUDA(ws, cudaEventCreate(&ev0));
  WS_CUDA(ws, cudaEventCreate(&ev1));
  int rc = GC_OK;
  for (int l = 0; l < WS_NL && rc == GC_OK; ++l) {
    const int Cin = kWsLayer[l][0], Cout = kWsLayer[l][1], R = ws->R >> kWsLayer[l][2];
    for (int kind = 0; kind < 3 && rc == GC_OK; ++kind) {
      float best = 3.0e38f;
      if (kind == 2) {
        const std::vector<WgPlan> c = enum_wgrad(R, Cin, Cout, ws->sm_count, nullptr);
        const WsBufs b = wgrad_bufs(ws, l);
        WgPlan keep = ws->pw[l];
        for (const WgPlan &p : c) {
          ws->pw[l] = p;
          if ((rc = ws_wgrad(ws, l, b.in, b.mask))) break;
          cudaEventRecord(ev0, ws->stream);
          for (int i = 0; i < iters && rc == GC_OK; ++i) rc = ws_wgrad(ws, l, b.in, b.mask);
          cudaEventRecord(ev1, ws->stream);
          cudaEventSynchronize(ev1);
          float ms = 0.0f;
          cudaEventElapsedTime(&ms, ev0, ev1);
          if (ms < best) { best = ms; keep = p; }
        }
        ws->pw[l] = keep;
      } else {
        if (kind == 1 && l == 0) { if (ms_out) ms_out[3 * l + kind] = 0.0f; continue; }
        const int ci = kind == 0 ? Cin : Cout, co = kind == 0 ? Cout : Cin;
        const std::vector<FwdPlan> c = enum_fwd(R, ci, co, ws->sm_count, nullptr);
        const WsBufs b = kind == 0 ? fwd_bufs(ws, l) : dgrad_bufs(ws, l);
        FwdPlan &slot = kind == 0 ? ws->pf[l] : ws->pb[l];
        FwdPlan keep = slot;
        const uint16_t *w = kind == 0 ? ws->wf[l] : ws->wb[l];
        const float *bias = kind == 0 ? ws->params + ws->b_off[l] : nullptr;
        const int relu = kind == 0 ? kWsLayer[l][3] : 0;
        for (const FwdPlan &p : c) {
          if ((rc = ws_conv(ws, p, R, ci, co, b.in, w, bias, nullptr, b.mask, b.out, b.outf, relu))) break;
          cudaEventRecord(ev0, ws->stream);
          for (int i = 0; i < iters && rc == GC_OK; ++i)
            rc = ws_conv(ws, p, R, ci, co, b.in, w, bias, nullptr, b.mask, b.out, b.outf, relu);
          cudaEventRecord(ev1, ws->stream);
          cudaEventSynchronize(ev1);
          float ms = 0.0f;
          cudaEventElapsedTime(&ms, ev0, ev1);
          if (ms < best) { best = ms; keep = p; }
        }
        slot = keep;
      }
      if (ms_out) ms_out[3 * l + kind] = best < 3.0e38f ? best / (float)iters : 0.0f;
    }
  }
  cudaEventDestroy(ev0);
  cudaEventDestroy(ev1);
  if (rc == GC_OK) WS_CUDA(ws, cudaGetLastError());
  return rc;
}

// The plan in use: out[0..4] = BZ, BY, taps per group (or per pass), CTAs, M tiles
// (0 for the weight gradient). kind 0 forward, 1 data gradient, 2 weight gradient.
extern "C" int gc_ws_plan_info(const gc_ws *ws, int layer, int kind, int *out) {
  if (!ws || !out || layer < 0 || layer >= WS_NL || kind < 0 || kind > 2) return GC_ERR_ARG;
  if (kind == 2) {
    const WgPlan &p = ws->pw[layer];
    out[0] = p.BZ; out[1] = p.BY; out[2] = p.tpp; out[3] = p.grid; out[4] = 0;
  } else {
    const FwdPlan &p = kind == 0 ? ws->pf[layer] : ws->pb[layer];
    out[0] = p.BZ; out[1] = p.BY; out[2] = p.tpg; out[3] = p.grid; out[4] = p.n_mt;
  }
  return GC_OK;
}

extern "C" int gc_ws_adam(gc_ws *ws, float lr, float beta1, float beta2, float eps, int step) {
  if (!ws || step < 1 || !(lr >= 0.0f)) return GC_ERR_ARG;
  const float bc1 = 1.0f - powf(beta1, (float)step), bc2 = 1.0f - powf(beta2, (float)step);
  k_adam<<<ew_blocks(ws->nparams, ws->sm_count), 256, 0, ws->stream>>>(ws->params, ws->grads, ws->adam_m, ws->adam_v,
                                                                       ws->nparams, lr, beta1, beta2, eps, bc1, bc2);
  WS_CUDA(ws, cudaGetLastError());
  return ws_repack(ws);
}

// ------------------------------------------------------------------------------
// engine hook: history, input features, applying the prediction
// ------------------------------------------------------------------------------
// Initial guess of step n from the previous potentials:
//   plain        phi(n-1)                                   (the reference's warm start)
//   extrapolate  phi(n-1) + d(n-1),  d(k) = phi(k) - phi(k-1) at full resolution
//   learned      the extrapolation + s * trilinear(y): the network predicts the
//                next second difference dd(n) = d(n) - d(n-1) on the (G/2)^3 grid
//                in units of s = rms(dd_c(n-1)); a zero output is the extrapolation.
// The coarse grid has R = G/2 cells per axis; cell (I,J,K) is the mean of the
// fine nodes (2I..2I+1, 2J.., 2K..), centred at fine coordinate 2I + 0.5.
// Coarse history per context: phi_c(n-1), d_c(n-1), dd_c(n-1). Features of step
// n (f16 [4][R^3]): log(1 + rho_c / mean rho_c), phi_c / rms, d_c / rms(d_c),
// dd_c / rms(dd_c); training target dd_c(n) / rms(dd_c(n-1)).
__global__ void __launch_bounds__(64) k_ws_coarsen(const float *__restrict__ f, int G, float *__restrict__ out) {
  const int R = G >> 1;
  const int K = blockIdx.x * blockDim.x + threadIdx.x, J = blockIdx.y, I = blockIdx.z;
  if (K >= R) return;
  float s = 0.0f;
#pragma unroll
  for (int c = 0; c < 8; ++c) s += __ldg(f + child_index(G, I, J, K, c));
  out[((size_t)I * R + J) * R + K] = 0.125f * s;
}

// per-block sums: rho_c, phi_c^2, d_c^2, dd_c^2
__global__ void __launch_bounds__(256) k_ws_stats(const float *__restrict__ rho, const float *__restrict__ phi,
                                                  const float *__restrict__ dlt, const float *__restrict__ ddl,
                                                  size_t n, float *__restrict__ part) {
  __shared__ float red[4][8];
  float a = 0.0f, b = 0.0f, c = 0.0f, e = 0.0f;
  for (size_t v = blockIdx.x * (size_t)blockDim.x + threadIdx.x; v < n; v += (size_t)gridDim.x * blockDim.x) {
    a += rho[v];
    b += phi[v] * phi[v];
    c += dlt[v] * dlt[v];
    e += ddl[v] * ddl[v];
  }
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
    c += __shfl_xor_sync(0xffffffffu, c, o);
    e += __shfl_xor_sync(0xffffffffu, e, o);
  }
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) { red[0][w] = a; red[1][w] = b; red[2][w] = c; red[3][w] = e; }
  __syncthreads();
  if (threadIdx.x < 4) {
    float s = 0.0f;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += red[threadIdx.x][i];
    part[4 * blockIdx.x + threadIdx.x] = s;
  }
}

// scal: [0] mean rho_c, [1] rms phi_c, [2] rms d_c, [3] d usable, [4] rms dd_c, [5] dd usable
// One block of 256 threads; fixed strided split and tree over the partials.
__global__ void __launch_bounds__(256) k_ws_scales(const float *__restrict__ part, int nb, size_t n, int hist,
                                                   float *__restrict__ scal) {
  __shared__ double red[4][256];
  const int t = threadIdx.x;
  double ta = 0.0, tb = 0.0, tc = 0.0, te = 0.0;
  for (int i = t; i < nb; i += 256) { ta += part[4 * i]; tb += part[4 * i + 1]; tc += part[4 * i + 2]; te += part[4 * i + 3]; }
  red[0][t] = ta; red[1][t] = tb; red[2][t] = tc; red[3][t] = te;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (t < w) {
#pragma unroll
      for (int k = 0; k < 4; ++k) red[k][t] += red[k][t + w];
    }
    __syncthreads();
  }
  if (t != 0) return;
  const double a = red[0][0], b = red[1][0], c = red[2][0], e = red[3][0];
  const double mr = a / (double)n, rp = sqrt(b / (double)n), rd = sqrt(c / (double)n), rdd = sqrt(e / (double)n);
  const double tiny = 1e-30 * (rp > 0.0 ? rp : 1.0);
  scal[0] = mr > 0.0 ? (float)mr : 1.0f;
  scal[1] = (hist >= 1 && rp > 0.0) ? (float)rp : 1.0f;
  const bool dok = hist >= 2 && rd > tiny;
  scal[2] = dok ? (float)rd : 1.0f;
  scal[3] = dok ? 1.0f : 0.0f;
  const bool ddok = hist >= 3 && rdd > tiny;
  scal[4] = ddok ? (float)rdd : 1.0f;
  scal[5] = ddok ? 1.0f : 0.0f;
}

__global__ void __launch_bounds__(256) k_ws_features(const float *__restrict__ rho, const float *__restrict__ phi,
                                                     const float *__restrict__ dlt, const float *__restrict__ ddl,
                                                     const float *__restrict__ scal, int hist, size_t n,
                                                     __half *__restrict__ feat, __half *__restrict__ rec) {
  const float ir = 1.0f / scal[0], ip = 1.0f / scal[1], id = 1.0f / scal[2], idd = 1.0f / scal[4];
  const bool has_p = hist >= 1, has_d = scal[3] != 0.0f, has_dd = scal[5] != 0.0f;
  for (size_t v = blockIdx.x * (size_t)blockDim.x + threadIdx.x; v < n; v += (size_t)gridDim.x * blockDim.x) {
    const __half a = __float2half_rn(log1pf(fmaxf(rho[v] * ir, 0.0f)));
    const __half b = __float2half_rn(has_p ? phi[v] * ip : 0.0f);
    const __half c = __float2half_rn(has_d ? dlt[v] * id : 0.0f);
    const __half e = __float2half_rn(has_dd ? ddl[v] * idd : 0.0f);
    feat[v] = a; feat[n + v] = b; feat[2 * n + v] = c; feat[3 * n + v] = e;
    if (rec) { rec[v] = a; rec[n + v] = b; rec[2 * n + v] = c; rec[3 * n + v] = e; }
  }
}

// Initial guess on every fine node: prev holds phi(n-2) on entry and phi(n-1)
// on exit; hi/lo (phi(n-1) on entry) get + d(n-1) when use_d (extrapolating,
// with two solves in the history) and + s * trilinear(yc) when yc is given.
__global__ void __launch_bounds__(128) k_ws_apply(const float *__restrict__ yc, const float *__restrict__ scal,
                                                  int use_d, int G, float *__restrict__ hi, float *__restrict__ lo,
                                                  float *__restrict__ prev) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, i = blockIdx.z;
  if (k >= G) return;
  // the face nodes are the multipole faces' (computed beside this pass)
  if (i == 0 || j == 0 || k == 0 || i == G - 1 || j == G - 1 || k == G - 1) return;
  const int R = G >> 1;
  const size_t v = ((size_t)i * G + j) * G + k;
  const float h = hi[v], l = lo[v];
  float corr = 0.0f;
  if (use_d) corr = __fsub_rn(h, prev[v]);
  if (yc && scal[5] != 0.0f) {
    int i0[3];
    float f[3];
    const int ii[3] = {i, j, k};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const float c = 0.5f * (float)ii[a] - 0.25f;
      int b = (int)floorf(c);
      b = b < 0 ? 0 : (b > R - 2 ? R - 2 : b);
      i0[a] = b;
      f[a] = fminf(fmaxf(c - (float)b, 0.0f), 1.0f);
    }
    float acc = 0.0f;
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      const int dx = c >> 2, dy = (c >> 1) & 1, dz = c & 1;
      const float w = (dx ? f[0] : 1.0f - f[0]) * (dy ? f[1] : 1.0f - f[1]) * (dz ? f[2] : 1.0f - f[2]);
      acc += w * __ldg(yc + ((size_t)(i0[0] + dx) * R + (i0[1] + dy)) * R + (i0[2] + dz));
    }
    corr += scal[4] * acc;
  }
  prev[v] = h;
  if (corr != 0.0f) {
    float sh, eh;
    df_two_sum(h, corr, sh, eh);
    float h2, l2;
    df_fast_two_sum(sh, __fadd_rn(l, eh), h2, l2);
    hi[v] = h2;
    lo[v] = l2;
  }
}

// after the solve: new phi_c, its first and second differences, the training
// target, history update
__global__ void __launch_bounds__(64) k_ws_post(const float *__restrict__ hi, int G, float *__restrict__ phi,
                                                float *__restrict__ dlt, float *__restrict__ ddl,
                                                const float *__restrict__ scal, int hist, __half *__restrict__ rec) {
  const int R = G >> 1;
  const int K = blockIdx.x * blockDim.x + threadIdx.x, J = blockIdx.y, I = blockIdx.z;
  if (K >= R) return;
  const size_t R3 = (size_t)R * R * R;
  const size_t v = ((size_t)I * R + J) * R + K;
  const float idd = 1.0f / scal[4];
  const bool has_dd = scal[5] != 0.0f;
  float s = 0.0f;
#pragma unroll
  for (int c = 0; c < 8; ++c) s += __ldg(hi + child_index(G, I, J, K, c));
  const float nw = 0.125f * s;
  const float d = hist >= 1 ? nw - phi[v] : 0.0f;
  const float dd = hist >= 2 ? d - dlt[v] : 0.0f;
  if (rec) rec[4 * R3 + v] = __float2half_rn(has_dd ? dd * idd : 0.0f);
  phi[v] = nw;
  dlt[v] = d;
  ddl[v] = dd;
}

static int ws_hook_buffers(gc_ctx *ctx) {
  const int R = ctx->G / 2;
  const size_t R3 = (size_t)R * R * R, G3 = (size_t)ctx->G * ctx->G * ctx->G;
  const size_t need = 5 * R3 + 2 * R3 + 16 + 4 * 1024 + G3;
  if (ctx->ws_buf && ctx->ws_buf_cap >= need) return GC_OK;
  cudaFree(ctx->ws_buf);
  ctx->ws_buf = nullptr;
  GC_CUDA(ctx, cudaMalloc(&ctx->ws_buf, need * sizeof(float)));
  GC_CUDA(ctx, cudaMemsetAsync(ctx->ws_buf, 0, need * sizeof(float), ctx->stream));
  ctx->ws_buf_cap = need;
  return GC_OK;
}

struct WsViews {
  float *rho, *phi, *dlt, *ddl, *y, *scal, *part, *prev;
  __half *feat;
};
static WsViews ws_views(gc_ctx *ctx) {
  const int R = ctx->G / 2;
  const size_t R3 = (size_t)R * R * R;
  WsViews w;
  w.rho = ctx->ws_buf;
  w.phi = w.rho + R3;
  w.dlt = w.phi + R3;
  w.ddl = w.dlt + R3;
  w.y = w.ddl + R3;
  w.feat = reinterpret_cast<__half *>(w.y + R3);  // 4 R^3 halves
  w.scal = w.y + 3 * R3;
  w.part = w.scal + 16;
  w.prev = w.part + 4 * 1024;
  return w;
}

int gc_ws_pre_solve(gc_ctx *ctx, int warm, int mode) {
  ctx->ws_skip = 0;
  if (!ctx->ws_track && !ctx->ws_record) return GC_OK;
  if (ctx->G % 2) return GC_OK;
  // a PRIME after a CLOSE solves at the positions of the last solve again: it
  // neither uses nor extends the history
  if (mode == GC_STEP_PRIME && ctx->ws_hist > 0 && warm) {
    ctx->ws_skip = 1;
    return GC_OK;
  }
  if (!warm) ctx->ws_hist = 0;  // a cold solve restarts the history
  int s;
  if ((s = ws_hook_buffers(ctx))) return s;
  const WsViews w = ws_views(ctx);
  const int R = ctx->G / 2;
  const size_t R3 = (size_t)R * R * R;
  unsigned nb = (unsigned)std::min<size_t>((R3 + 255) / 256, 1024);
  // the coarse history and the network features: for the learned guess, for
  // recording, or when tracking was asked for (the extrapolation needs neither)
  const bool coarse = ctx->ws_coarse || ctx->ws_record;
  if (coarse) {
  gc_launch(ctx, GK_WARMSTART, k_ws_coarsen, dim3((R + 63) / 64, R, R), dim3(64), 0, (const float *)ctx->b0, ctx->G,
            w.rho);
  gc_launch(ctx, GK_WARMSTART, k_ws_stats, dim3(nb), dim3(256), 0, (const float *)w.rho, (const float *)w.phi,
            (const float *)w.dlt, (const float *)w.ddl, R3, w.part);
  gc_launch(ctx, GK_WARMSTART, k_ws_scales, dim3(1), dim3(256), 0, (const float *)w.part, (int)nb, R3, ctx->ws_hist,
            w.scal);
  gc_launch(ctx, GK_WARMSTART, k_ws_features, dim3(nb), dim3(256), 0, (const float *)w.rho, (const float *)w.phi,
            (const float *)w.dlt, (const float *)w.ddl, (const float *)w.scal, ctx->ws_hist, R3, w.feat,
            (__half *)ctx->ws_record);
  GC_LAUNCH_CHECK(ctx, "warm-start features");
  }
  if (!warm || ctx->ws_hist < 1) return GC_OK;
  const float *yc = nullptr;
  if (ctx->ws_mode == GC_WS_LEARNED && ctx->ws_hist >= 3) {
    gc_ws *ws = ctx->ws;
    if (!ws || ws->R != R) {
      gc_set_error(ctx, "learned warm start needs a network with R = G/2 = %d", R);
      return GC_ERR_STATE;
    }
    ws->stream = ctx->stream;
    // the network's convolutions are timed as one warm-start interval (they
    // launch on the network object, not through the context's launcher)
    const int slot = ctx->prof.enabled && !ctx->capturing ? gc_prof_slot(ctx, GK_WARMSTART) : -1;
    if (slot >= 0) cudaEventRecord(ctx->prof.ev[2 * slot], ctx->stream);
    if ((s = gc_ws_forward(ws, w.feat, w.y))) {
      gc_set_error(ctx, "warm-start network: %s", ws->err);
      return s;
    }
    if (slot >= 0) cudaEventRecord(ctx->prof.ev[2 * slot + 1], ctx->stream);
    ctx->prof.launches[GK_WARMSTART] += 18;
    yc = w.y;
  }
  const int use_d = ctx->ws_mode != GC_WS_PLAIN && ctx->ws_hist >= 2;
  gc_launch(ctx, GK_WARMSTART, k_ws_apply, dim3((ctx->G + 127) / 128, ctx->G, ctx->G), dim3(128), 0, yc,
            (const float *)w.scal, use_d, ctx->G, ctx->hi, ctx->lo, w.prev);
  GC_LAUNCH_CHECK(ctx, "warm-start apply");
  return GC_OK;
}

int gc_ws_post_solve(gc_ctx *ctx) {
  if (!ctx->ws_track && !ctx->ws_record) return GC_OK;
  if (ctx->G % 2 || ctx->ws_skip) return GC_OK;
  if (!ctx->ws_coarse && !ctx->ws_record) {
    ctx->ws_hist = ctx->ws_hist < 3 ? ctx->ws_hist + 1 : 3;
    return GC_OK;
  }
  const WsViews w = ws_views(ctx);
  const int R = ctx->G / 2;
  gc_launch(ctx, GK_WARMSTART, k_ws_post, dim3((R + 63) / 64, R, R), dim3(64), 0, (const float *)ctx->hi, ctx->G,
            w.phi, w.dlt, w.ddl, (const float *)w.scal, ctx->ws_hist, (__half *)ctx->ws_record);
  GC_LAUNCH_CHECK(ctx, "warm-start history");
  ctx->ws_hist = ctx->ws_hist < 3 ? ctx->ws_hist + 1 : 3;
  ctx->ws_record = nullptr;
  return GC_OK;
}

extern "C" int gc_pm_set_warmstart(gc_ctx *ctx, gc_ws *ws, int mode, int track) {
  if (!ctx) return GC_ERR_ARG;
  GC_REQUIRE(ctx, mode == GC_WS_PLAIN || mode == GC_WS_LEARNED || mode == GC_WS_EXTRAPOLATE,
             "gc_pm_set_warmstart: bad mode %d", mode);
  GC_REQUIRE(ctx, mode != GC_WS_LEARNED || ws, "gc_pm_set_warmstart: learned mode needs a network");
  GC_REQUIRE(ctx, ctx->G % 2 == 0 || (mode == GC_WS_PLAIN && !track),
             "gc_pm_set_warmstart: the coarse history needs an even grid size");
  GC_REQUIRE(ctx, !ws || ws->R == ctx->G / 2, "gc_pm_set_warmstart: network R=%d, grid needs R=%d", ws ? ws->R : 0,
             ctx->G / 2);
  const int tr = (track || mode != GC_WS_PLAIN) ? 1 : 0;
  const int coarse = (track || mode == GC_WS_LEARNED) ? 1 : 0;
  // the history restarts when what it holds changes
  if ((tr && !ctx->ws_track) || (coarse && !ctx->ws_coarse) || mode != ctx->ws_mode) ctx->ws_hist = 0;
  ctx->ws = ws;
  ctx->ws_mode = mode;
  ctx->ws_track = tr;
  ctx->ws_coarse = coarse;
  return GC_OK;
}

extern "C" int gc_pm_record_sample(gc_ctx *ctx, void *out) {
  if (!ctx) return GC_ERR_ARG;
  GC_REQUIRE(ctx, ctx->G % 2 == 0, "gc_pm_record_sample: the coarse grid needs an even grid size");
  GC_REQUIRE(ctx, ctx->ws_coarse, "gc_pm_record_sample: set the warm start with track = 1 first");
  ctx->ws_record = out;
  return GC_OK;
}
