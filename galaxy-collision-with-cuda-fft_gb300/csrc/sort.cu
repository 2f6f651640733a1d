// Cell keys and a stable LSD radix sort of (key, index) pairs.
//
// The key is the reference's cell index ix = floor(x/dx) (deposit.py:62-67),
// linearised over the (G+1)^3 cells that can receive mass (-1 <= ix <= G-1).
// Each radix pass is reduce-then-scan: per-tile digit histograms, one exclusive
// scan of the digit-major histogram, then a stable scatter in which every warp
// ranks its items round by round (by runs of equal neighbours when a round's
// digits are in order, else with match.any), so equal keys keep their input
// order and the permutation is unique. Digits are up to 9 bits wide (the 25-bit
// cell keys of a 256^3 grid take three passes), tiles 4096 items.
#include "common.cuh"

#include <cmath>

#define RS_MAX_BITS 9                      // widest digit of a pass
#define RS_MAX_RADIX (1 << RS_MAX_BITS)
#define RS_THREADS 256
#define RS_WARPS (RS_THREADS / 32)
#define RS_IPT 16                          // items per thread
#define RS_TILE (RS_THREADS * RS_IPT)      // 4096 items per tile

__global__ void __launch_bounds__(256)
    k_cell_keys(const float *__restrict__ x, const float *__restrict__ y, const float *__restrict__ z, long long n,
                float dx, int G, uint32_t *__restrict__ keys) {
  const uint32_t sentinel = (uint32_t)(G + 1) * (uint32_t)(G + 1) * (uint32_t)(G + 1);
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    CellPos c;
    uint32_t key = sentinel;
    if (gc_cell_of(x[p], y[p], z[p], dx, G, c))
      key = ((uint32_t)(c.ix + 1) * (uint32_t)(G + 1) + (uint32_t)(c.iy + 1)) * (uint32_t)(G + 1) + (uint32_t)(c.iz + 1);
    keys[p] = key;
  }
}

// The lanes 0 .. lane as a mask.
__device__ __forceinline__ unsigned lanes_upto(int lane) { return 0xffffffffu >> (31 - lane); }

// Digit histogram of each tile: hist[d * ntiles + tile], digits of BITS bits
// at `shift`. A thread loads its 16 keys first (16 loads in flight); then, for
// each group of 32 consecutive keys, every run of equal neighbouring digits
// adds its length with one atomic from its first lane, so nearly sorted keys
// do not serialise on one counter and random keys cost one atomic each (a
// digit that recurs after another digit simply starts a second run).
template <int BITS>
__global__ void __launch_bounds__(RS_THREADS)
    k_rs_hist(const uint32_t *__restrict__ keys, long long n, int shift, unsigned *__restrict__ hist, int ntiles) {
  constexpr int RADIX = 1 << BITS;
  __shared__ unsigned cnt[RADIX];
  for (int d = threadIdx.x; d < RADIX; d += RS_THREADS) cnt[d] = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const long long base = (long long)blockIdx.x * RS_TILE;
  uint32_t kk[RS_IPT];
#pragma unroll
  for (int j = 0; j < RS_IPT; ++j) {
    const long long p = base + j * RS_THREADS + threadIdx.x;
    kk[j] = p < n ? keys[p] : 0u;
  }
#pragma unroll
  for (int j = 0; j < RS_IPT; ++j) {
    // the valid lanes of a group are a prefix of it (the tile's tail)
    const bool ok = base + j * RS_THREADS + threadIdx.x < n;
    const unsigned d = (kk[j] >> shift) & (RADIX - 1);
    const unsigned dprev = __shfl_up_sync(0xffffffffu, d, 1);
    const bool head = ok && (lane == 0 || d != dprev);
    const unsigned heads = __ballot_sync(0xffffffffu, head);
    const unsigned nvalid = __popc(__ballot_sync(0xffffffffu, ok));
    const unsigned above = heads & ~lanes_upto(lane);
    const int end = above ? __ffs(above) - 1 : (int)nvalid;  // one past the run
    if (head) atomicAdd(&cnt[d], (unsigned)(end - lane));
  }
  __syncthreads();
  for (int d = threadIdx.x; d < RADIX; d += RS_THREADS) hist[(size_t)d * ntiles + blockIdx.x] = cnt[d];
}

// Exclusive scan of an unsigned array in three phases (tile sums, scan of sums, apply).
#define SC_THREADS 1024
#define SC_TILE 4096

__device__ __forceinline__ unsigned block_excl_scan(unsigned v, unsigned &total) {
  __shared__ unsigned ws[SC_THREADS / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  unsigned x = v;
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) ws[wid] = x;
  __syncthreads();
  if (wid == 0) {
    unsigned w = lane < (int)(blockDim.x / 32) ? ws[lane] : 0u;
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    ws[lane] = w;
  }
  __syncthreads();
  const unsigned prefix = (wid > 0 ? ws[wid - 1] : 0u) + x - v;
  total = ws[blockDim.x / 32 - 1];
  __syncthreads();
  return prefix;
}

__global__ void __launch_bounds__(SC_THREADS) k_scan_tile_sums(const unsigned *__restrict__ a, long long n,
                                                               unsigned *__restrict__ sums) {
  const long long base = (long long)blockIdx.x * SC_TILE;
  unsigned s = 0;
  for (int t = threadIdx.x; t < SC_TILE; t += SC_THREADS) {
    const long long p = base + t;
    if (p < n) s += a[p];
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  __shared__ unsigned ws[SC_THREADS / 32];
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    unsigned w = ws[threadIdx.x];
    for (int o = 16; o > 0; o >>= 1) w += __shfl_down_sync(0xffffffffu, w, o);
    if (threadIdx.x == 0) sums[blockIdx.x] = w;
  }
}

// Single block: in-place exclusive scan of sums[0..m).
__global__ void __launch_bounds__(SC_THREADS) k_scan_sums(unsigned *__restrict__ sums, int m) {
  unsigned carry = 0;
  for (int base = 0; base < m; base += SC_THREADS) {
    const int p = base + threadIdx.x;
    const unsigned v = p < m ? sums[p] : 0u;
    unsigned total;
    const unsigned ex = block_excl_scan(v, total);
    if (p < m) sums[p] = carry + ex;
    carry += total;
  }
}

__global__ void __launch_bounds__(SC_THREADS) k_scan_apply(unsigned *__restrict__ a, long long n,
                                                           const unsigned *__restrict__ sums) {
  const long long base = (long long)blockIdx.x * SC_TILE;
  unsigned carry = sums[blockIdx.x];
  for (int off = 0; off < SC_TILE; off += SC_THREADS) {
    const long long p = base + off + threadIdx.x;
    const unsigned v = p < n ? a[p] : 0u;
    unsigned total;
    const unsigned ex = block_excl_scan(v, total);
    if (p < n) a[p] = carry + ex;
    carry += total;
  }
}

// Stable scatter. Warp w of a tile owns items [w*32*IPT, (w+1)*32*IPT) of the
// tile; round r handles item r*32+lane of that range, so (round, lane) order is
// input order. Ranks within the tile (per-warp digit counts, then across warps
// and digits) place every item at its slot of the tile's digit-sorted order in
// shared memory; the items are then written out from there, so consecutive
// threads write consecutive addresses of one digit's output segment. Dynamic
// shared memory: scatter_smem_bytes<BITS>().
//
// Ranking a round: when the 32 digits are non-decreasing across the lanes
// (nearly sorted keys, most rounds), each digit is one run of neighbours, so
// the run's first lane reads and advances its warp counter by the run length
// and the others take their offset in the run; otherwise the lanes holding
// the same digit are found with match.any. Both give every item the number of
// items with its digit before it in (round, lane) order. The values are read
// only when the items are placed (fewer live registers: four CTAs per SM for
// the 8- and 9-bit digits of the cell keys, measured faster than three or two;
// three for narrower digits, whose kernels would spill at four); vin == NULL
// means the identity values (an item's index).
template <int BITS>
constexpr size_t scatter_smem_bytes() {
  return sizeof(unsigned) * ((size_t)RS_WARPS * (1 << BITS) + 2 * (1 << BITS) + RS_WARPS + 2 * RS_TILE);
}

template <int BITS>
__global__ void __launch_bounds__(RS_THREADS, BITS >= 8 ? 4 : 3)
    k_rs_scatter(const uint32_t *__restrict__ kin, const uint32_t *__restrict__ vin, long long n, int shift,
                 const unsigned *__restrict__ hist, int ntiles, uint32_t *__restrict__ kout,
                 uint32_t *__restrict__ vout) {
  constexpr int RADIX = 1 << BITS;
  constexpr int DPT = (RADIX + RS_THREADS - 1) / RS_THREADS;  // digits per thread in the per-digit phase
  extern __shared__ __align__(16) unsigned rs_smem[];
  unsigned (*whist)[RADIX] = reinterpret_cast<unsigned (*)[RADIX]>(rs_smem);
  unsigned *dstart = rs_smem + RS_WARPS * RADIX;  // first slot of each digit in the tile's sorted order
  unsigned *gofs = dstart + RADIX;                // output index of the tile's first item of each digit
  unsigned *wsum = gofs + RADIX;
  uint32_t *sk = wsum + RS_WARPS, *sv = sk + RS_TILE;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int t = threadIdx.x; t < RS_WARPS * RADIX; t += RS_THREADS) rs_smem[t] = 0;
  __syncthreads();
  const long long tile0 = (long long)blockIdx.x * RS_TILE;
  const int cnt = (int)(n - tile0 < RS_TILE ? n - tile0 : RS_TILE);
  const long long seg = tile0 + (long long)w * 32 * RS_IPT;
  uint32_t k[RS_IPT];
  unsigned rank[RS_IPT];
  const unsigned lt = (1u << lane) - 1u;
#pragma unroll
  for (int r = 0; r < RS_IPT; ++r) {
    const long long p = seg + r * 32 + lane;
    k[r] = p < n ? kin[p] : 0u;
  }
#pragma unroll
  for (int r = 0; r < RS_IPT; ++r) {
    // the valid lanes of a round are a prefix of it (the tile's tail)
    const bool ok = seg + r * 32 + lane < n;
    const unsigned d = (k[r] >> shift) & (RADIX - 1);
    const unsigned dprev = __shfl_up_sync(0xffffffffu, d, 1);
    if (__all_sync(0xffffffffu, !ok || lane == 0 || dprev <= d)) {
      const unsigned heads = __ballot_sync(0xffffffffu, ok && (lane == 0 || d != dprev));
      const unsigned nvalid = __popc(__ballot_sync(0xffffffffu, ok));
      const int hl = 31 - __clz(heads & lanes_upto(lane));  // the run's first lane (-1: no valid lane at all)
      const unsigned above = heads & ~lanes_upto(lane);
      const int end = above ? __ffs(above) - 1 : (int)nvalid;
      unsigned old = 0;
      if (ok && hl == lane) {
        old = whist[w][d];
        whist[w][d] = old + (unsigned)(end - lane);
      }
      __syncwarp();
      rank[r] = __shfl_sync(0xffffffffu, old, hl & 31) + (unsigned)(lane - hl);
    } else {
      const unsigned dd = ok ? d : (unsigned)RADIX + lane;
      const unsigned peers = __match_any_sync(0xffffffffu, dd);
      unsigned old = 0;
      if (ok) old = whist[w][d];
      __syncwarp();
      if (ok && (peers & lt) == 0) whist[w][d] = old + __popc(peers);
      __syncwarp();
      rank[r] = old + __popc(peers & lt);
    }
  }
  __syncthreads();
  // per digit (thread t takes digits t*DPT .. t*DPT+DPT-1): exclusive prefix
  // over the warps, the digit's tile total, and the tile's global offset for it
  unsigned tot[DPT], mine = 0;
#pragma unroll
  for (int q = 0; q < DPT; ++q) {
    const int d = threadIdx.x * DPT + q;
    tot[q] = 0;
    if (d < RADIX) {
      for (int ww = 0; ww < RS_WARPS; ++ww) {
        const unsigned c = whist[ww][d];
        whist[ww][d] = tot[q];
        tot[q] += c;
      }
      gofs[d] = hist[(size_t)d * ntiles + blockIdx.x];
    }
    mine += tot[q];
  }
  // exclusive scan of the digit totals over the block (threads in digit order)
  {
    unsigned x = mine;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) wsum[w] = x;
    __syncthreads();
    unsigned before = 0;
    for (int ww = 0; ww < w; ++ww) before += wsum[ww];
    unsigned at = before + x - mine;
#pragma unroll
    for (int q = 0; q < DPT; ++q) {
      const int d = threadIdx.x * DPT + q;
      if (d < RADIX) dstart[d] = at;
      at += tot[q];
    }
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < RS_IPT; ++r) {
    const long long p = seg + r * 32 + lane;
    if (p < n) {
      const unsigned d = (k[r] >> shift) & (RADIX - 1);
      const unsigned slot = dstart[d] + whist[w][d] + rank[r];
      sk[slot] = k[r];
      sv[slot] = vin ? vin[p] : (uint32_t)p;
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < cnt; i += RS_THREADS) {
    const uint32_t kk = sk[i];
    const unsigned d = (kk >> shift) & (RADIX - 1);
    const unsigned dst = gofs[d] + (unsigned)i - dstart[d];
    kout[dst] = kk;
    vout[dst] = sv[i];
  }
}

// One radix pass with digits of BITS bits at `shift`.
template <int BITS>
static int radix_pass(gc_ctx *ctx, const uint32_t *kin, const uint32_t *vin, long long n, int shift, int ntiles,
                      uint32_t *ko, uint32_t *vo);

static int exclusive_scan(gc_ctx *ctx, unsigned *a, long long n) {
  const long long nt = (n + SC_TILE - 1) / SC_TILE;
  unsigned *sums = ctx->hist_aux;
  gc_launch(ctx, GK_SORT, k_scan_tile_sums, dim3((unsigned)nt), dim3(SC_THREADS), 0, a, n, sums);
  gc_launch(ctx, GK_SORT, k_scan_sums, dim3(1), dim3(SC_THREADS), 0, sums, (int)nt);
  gc_launch(ctx, GK_SORT, k_scan_apply, dim3((unsigned)nt), dim3(SC_THREADS), 0, a, n, sums);
  GC_LAUNCH_CHECK(ctx, "scan");
  return GC_OK;
}

template <int BITS>
static int radix_pass(gc_ctx *ctx, const uint32_t *kin, const uint32_t *vin, long long n, int shift, int ntiles,
                      uint32_t *ko, uint32_t *vo) {
  constexpr size_t smem = scatter_smem_bytes<BITS>();
  static_assert(smem <= 227 * 1024, "scatter tile does not fit shared memory");
  static int attr_device = -1;  // the opt-in above 48 KB, once per device
  if (smem > 48 * 1024 && attr_device != ctx->device) {
    GC_CUDA(ctx, cudaFuncSetAttribute(k_rs_scatter<BITS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr_device = ctx->device;
  }
  gc_launch(ctx, GK_SORT, k_rs_hist<BITS>, dim3(ntiles), dim3(RS_THREADS), 0, kin, n, shift, ctx->hist, ntiles);
  GC_LAUNCH_CHECK(ctx, "radix hist");
  int s = exclusive_scan(ctx, ctx->hist, (long long)ntiles << BITS);
  if (s) return s;
  gc_launch(ctx, GK_SORT, k_rs_scatter<BITS>, dim3(ntiles), dim3(RS_THREADS), smem, kin, vin, n, shift, ctx->hist,
            ntiles, ko, vo);
  GC_LAUNCH_CHECK(ctx, "radix scatter");
  return GC_OK;
}

// Key/value ping-pong buffers and digit histograms for n items (grown, never shrunk).
static int ensure_sort_scratch(gc_ctx *ctx, int64_t n) {
  int s = gc_ensure_particle_scratch(ctx, (size_t)n);
  if (s) return s;
  const size_t ntiles = (ctx->pcap + RS_TILE - 1) / RS_TILE;  // sized for the scratch capacity
  const size_t hn = ntiles * RS_MAX_RADIX;
  if (ctx->hist_cap < hn) {
    GC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    cudaFree(ctx->hist);
    cudaFree(ctx->hist_aux);
    ctx->hist = ctx->hist_aux = nullptr;
    ctx->hist_cap = 0;
    GC_CUDA(ctx, cudaMalloc(&ctx->hist, hn * sizeof(unsigned)));
    GC_CUDA(ctx, cudaMalloc(&ctx->hist_aux, ((hn + SC_TILE - 1) / SC_TILE + 32) * sizeof(unsigned)));
    ctx->hist_cap = hn;
  }
  return GC_OK;
}

extern "C" int gc_pm_reserve(gc_ctx *ctx, int64_t n) {
  if (!ctx) return GC_ERR_ARG;
  GC_REQUIRE(ctx, n >= 0 && n < (1LL << 31), "particle count out of range");
  return n > 0 ? ensure_sort_scratch(ctx, n) : GC_OK;
}

int gc_radix_sort_pairs(gc_ctx *ctx, const uint32_t *keys_in, const uint32_t *vals_in, int64_t n, int bits,
                        uint32_t **keys_out, uint32_t **vals_out) {
  ctx->import_n = 0;  // the scratch is about to be reused: a kept import order is gone
  ctx->import_perm = nullptr;
  ctx->export_n = 0;  // ... and so are kept export ranks
  int s = ensure_sort_scratch(ctx, n);
  if (s) return s;
  const int ntiles = (int)((n + RS_TILE - 1) / RS_TILE);
  const uint32_t *kin = keys_in, *vin = vals_in;
  // ping-pong between (keys, vals) and (keys2, vals2); never write into the caller's input
  uint32_t *ka = ctx->keys, *va = ctx->vals, *kb = ctx->keys2, *vb = ctx->vals2;
  // passes of at most RS_MAX_BITS bits, as even as possible (25 bits: 9 + 8 + 8)
  if (bits < 1) bits = 1;
  const int passes = (bits + RS_MAX_BITS - 1) / RS_MAX_BITS;
  int shift = 0;
  for (int pss = 0; pss < passes; ++pss) {
    const int w = (bits - shift + (passes - pss) - 1) / (passes - pss);
    uint32_t *ko = (pss & 1) ? kb : ka;
    uint32_t *vo = (pss & 1) ? vb : va;
    if (kin == ko) {  // input aliases this pass's output: use the other buffer
      ko = (ko == ka) ? kb : ka;
      vo = (vo == va) ? vb : va;
    }
    switch (w) {
      case 1: s = radix_pass<1>(ctx, kin, vin, n, shift, ntiles, ko, vo); break;
      case 2: s = radix_pass<2>(ctx, kin, vin, n, shift, ntiles, ko, vo); break;
      case 3: s = radix_pass<3>(ctx, kin, vin, n, shift, ntiles, ko, vo); break;
      case 4: s = radix_pass<4>(ctx, kin, vin, n, shift, ntiles, ko, vo); break;
      case 5: s = radix_pass<5>(ctx, kin, vin, n, shift, ntiles, ko, vo); break;
      case 6: s = radix_pass<6>(ctx, kin, vin, n, shift, ntiles, ko, vo); break;
      case 7: s = radix_pass<7>(ctx, kin, vin, n, shift, ntiles, ko, vo); break;
      case 8: s = radix_pass<8>(ctx, kin, vin, n, shift, ntiles, ko, vo); break;
      default: s = radix_pass<9>(ctx, kin, vin, n, shift, ntiles, ko, vo); break;
    }
    if (s) return s;
    shift += w;
    kin = ko;
    vin = vo;
  }
  *keys_out = (uint32_t *)kin;
  *vals_out = (uint32_t *)vin;
  return GC_OK;
}

static int key_bits(int G) {
  const unsigned long long maxkey = (unsigned long long)(G + 1) * (G + 1) * (G + 1);
  int b = 0;
  while ((1ULL << b) <= maxkey) ++b;
  return b;
}

extern "C" int gc_cell_keys(gc_ctx *ctx, const float *x, const float *y, const float *z, int64_t n, uint32_t *keys) {
  if (!ctx) return GC_ERR_ARG;
  GC_REQUIRE(ctx, n >= 0 && n < (1LL << 31), "particle count out of range");
  if (n == 0) return GC_OK;
  GC_REQUIRE(ctx, x && y && z && keys, "gc_cell_keys: NULL pointer");
  GC_REQUIRE(ctx, (unsigned long long)(ctx->G + 1) * (ctx->G + 1) * (ctx->G + 1) < 0xffffffffULL,
             "grid too large for 32-bit cell keys");
  unsigned nb = gc_blocks(n, 256);
  if (nb > gc_sms() * 32u) nb = gc_sms() * 32u;
  gc_launch(ctx, GK_KEYS, k_cell_keys, dim3(nb), dim3(256), 0, x, y, z, (long long)n, (float)ctx->dx, ctx->G, keys);
  GC_LAUNCH_CHECK(ctx, "cell keys");
  return GC_OK;
}

extern "C" int gc_sort_keys(gc_ctx *ctx, const uint32_t *keys, int64_t n, uint32_t *sorted_keys, uint32_t *perm) {
  if (!ctx) return GC_ERR_ARG;
  GC_REQUIRE(ctx, n >= 0 && n < (1LL << 31), "particle count out of range");
  if (n == 0) return GC_OK;
  GC_REQUIRE(ctx, keys && perm, "gc_sort_keys: NULL pointer");
  int s = gc_ensure_particle_scratch(ctx, (size_t)n);
  if (s) return s;
  uint32_t *ko, *vo;
  // full 32-bit keys: any caller key is sorted stably; values: the identity
  if ((s = gc_radix_sort_pairs(ctx, keys, nullptr, n, 32, &ko, &vo))) return s;
  if (sorted_keys) GC_CUDA(ctx, cudaMemcpyAsync(sorted_keys, ko, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, ctx->stream));
  GC_CUDA(ctx, cudaMemcpyAsync(perm, vo, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, ctx->stream));
  return GC_OK;
}

// All arrays of a particle set permuted in one pass: perm is read once and the
// nine gathers of a particle are independent loads.
struct PermSet {
  const float *fin[7];
  float *fout[7];
  const int32_t *iin[2];
  int32_t *iout[2];
};

// Each thread takes PERM_U particles per round (PERM_U perm loads, then all
// their gathers, then the stores), so that a thread keeps many independent
// loads in flight instead of two dependent ones.
#define PERM_U 4
__global__ void __launch_bounds__(256)
    k_permute_set(PermSet s, const uint32_t *__restrict__ perm, long long n) {
  const long long T = (long long)gridDim.x * blockDim.x;
  for (long long p0 = blockIdx.x * (long long)blockDim.x + threadIdx.x; p0 < n; p0 += PERM_U * T) {
    uint32_t q[PERM_U];
#pragma unroll
    for (int u = 0; u < PERM_U; ++u) q[u] = p0 + u * T < n ? __ldg(perm + p0 + u * T) : 0u;
    float fv[7][PERM_U];
    int32_t iv[2][PERM_U];
#pragma unroll
    for (int a = 0; a < 7; ++a)
#pragma unroll
      for (int u = 0; u < PERM_U; ++u)
        if (s.fin[a] && p0 + u * T < n) fv[a][u] = __ldg(s.fin[a] + q[u]);
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
      for (int u = 0; u < PERM_U; ++u)
        if (s.iin[a] && p0 + u * T < n) iv[a][u] = __ldg(s.iin[a] + q[u]);
#pragma unroll
    for (int u = 0; u < PERM_U; ++u) {
      const long long p = p0 + u * T;
      if (p >= n) break;
#pragma unroll
      for (int a = 0; a < 7; ++a)
        if (s.fin[a]) s.fout[a][p] = fv[a][u];
#pragma unroll
      for (int a = 0; a < 2; ++a)
        if (s.iin[a]) s.iout[a][p] = iv[a][u];
    }
  }
}

// Cell keys of the positions predicted tau ahead, x + v tau (f32, rounded per
// operation), or of the current position when the predicted one deposits
// nothing (or v is not finite). Sorting by these keys puts the particles in the
// order of their cells at the middle of the next sort period, so that the
// deposit and gather passes see them drift by half as much.
__global__ void __launch_bounds__(256)
    k_cell_keys_ahead(const float *__restrict__ x, const float *__restrict__ y, const float *__restrict__ z,
                      const float *__restrict__ vx, const float *__restrict__ vy, const float *__restrict__ vz,
                      float tau, long long n, float dx, int G, uint32_t *__restrict__ keys) {
  const uint32_t g1 = (uint32_t)(G + 1), sentinel = g1 * g1 * g1;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    const float px = x[p], py = y[p], pz = z[p];
    CellPos c;
    uint32_t key = sentinel;
    if (gc_cell_of(__fadd_rn(px, __fmul_rn(vx[p], tau)), __fadd_rn(py, __fmul_rn(vy[p], tau)),
                   __fadd_rn(pz, __fmul_rn(vz[p], tau)), dx, G, c) ||
        gc_cell_of(px, py, pz, dx, G, c))
      key = ((uint32_t)(c.ix + 1) * g1 + (uint32_t)(c.iy + 1)) * g1 + (uint32_t)(c.iz + 1);
    keys[p] = key;
  }
}

extern "C" int gc_pm_sort(gc_ctx *ctx, const gc_particles *in, const gc_particles *out) {
  return gc_pm_sort_ahead(ctx, in, out, 0.0f);
}

extern "C" int gc_pm_sort_ahead(gc_ctx *ctx, const gc_particles *in, const gc_particles *out, float tau) {
  if (!ctx) return GC_ERR_ARG;
  GC_REQUIRE(ctx, in && out, "gc_pm_sort: NULL particle set");
  GC_REQUIRE(ctx, std::isfinite(tau), "gc_pm_sort_ahead: tau must be finite, got %g", (double)tau);
  GC_REQUIRE(ctx, tau == 0.0f || (in->vx && in->vy && in->vz), "gc_pm_sort_ahead: velocities required for tau != 0");
  const int64_t n = in->n;
  GC_REQUIRE(ctx, n >= 0 && n < (1LL << 31), "particle count out of range");
  GC_REQUIRE(ctx, out->n == n, "gc_pm_sort: in and out sizes differ");
  if (n == 0) return GC_OK;
  GC_REQUIRE(ctx, in->x && in->y && in->z, "gc_pm_sort: positions required");
  int s = gc_ensure_particle_scratch(ctx, (size_t)n);
  if (s) return s;
  unsigned nb = gc_blocks(n, 256);
  if (nb > gc_sms() * 32u) nb = gc_sms() * 32u;
  if (tau == 0.0f)
    gc_launch(ctx, GK_KEYS, k_cell_keys, dim3(nb), dim3(256), 0, in->x, in->y, in->z, (long long)n, (float)ctx->dx,
              ctx->G, ctx->keys2);
  else
    gc_launch(ctx, GK_KEYS, k_cell_keys_ahead, dim3(nb), dim3(256), 0, in->x, in->y, in->z, in->vx, in->vy, in->vz,
              tau, (long long)n, (float)ctx->dx, ctx->G, ctx->keys2);
  GC_LAUNCH_CHECK(ctx, "cell keys");
  uint32_t *ko, *vo;
  if ((s = gc_radix_sort_pairs(ctx, ctx->keys2, nullptr, n, key_bits(ctx->G), &ko, &vo))) return s;
  PermSet ps;
  const float *fin[7] = {in->x, in->y, in->z, in->vx, in->vy, in->vz, in->m};
  float *fout[7] = {out->x, out->y, out->z, out->vx, out->vy, out->vz, out->m};
  for (int a = 0; a < 7; ++a) {
    GC_REQUIRE(ctx, !fin[a] || (fout[a] && fout[a] != fin[a]), "gc_pm_sort: output array %d missing or aliases its input", a);
    ps.fin[a] = fin[a];
    ps.fout[a] = fin[a] ? fout[a] : nullptr;
  }
  const int32_t *iin[2] = {in->gid, in->pid};
  int32_t *iout[2] = {out->gid, out->pid};
  for (int a = 0; a < 2; ++a) {
    GC_REQUIRE(ctx, !iin[a] || (iout[a] && iout[a] != iin[a]), "gc_pm_sort: id array %d missing or aliases its input", a);
    ps.iin[a] = iin[a];
    ps.iout[a] = iin[a] ? iout[a] : nullptr;
  }
  gc_launch(ctx, GK_PERMUTE, k_permute_set, dim3(nb), dim3(256), 0, ps, vo, (long long)n);
  GC_LAUNCH_CHECK(ctx, "permute");
  return GC_OK;
}

// ---- reference layout <-> engine layout ---------------------------------------
__global__ void __launch_bounds__(256)
    k_pm_import(const float *__restrict__ pos, const float *__restrict__ vel, const float *__restrict__ m,
                const int32_t *__restrict__ gid, double ox, double oy, double oz, gc_particles o, long long n) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    o.x[p] = (float)((double)pos[3 * p] - ox);
    o.y[p] = (float)((double)pos[3 * p + 1] - oy);
    o.z[p] = (float)((double)pos[3 * p + 2] - oz);
    o.vx[p] = vel[3 * p];
    o.vy[p] = vel[3 * p + 1];
    o.vz[p] = vel[3 * p + 2];
    o.m[p] = m[p];
    if (o.gid) o.gid[p] = gid ? gid[p] : 0;
    if (o.pid) o.pid[p] = (int32_t)p;
  }
}

__global__ void __launch_bounds__(256)
    k_pm_export(gc_particles s, double ox, double oy, double oz, float *__restrict__ pos, float *__restrict__ vel,
                float *__restrict__ m, int32_t *__restrict__ gid, long long n, unsigned *__restrict__ status) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    const long long q = s.pid[p];
    if (q < 0 || q >= n) {
      atomicOr(status, GC_FLAG_BAD_PID);
      continue;
    }
    if (pos) {
      pos[3 * q] = (float)((double)s.x[p] + ox);
      pos[3 * q + 1] = (float)((double)s.y[p] + oy);
      pos[3 * q + 2] = (float)((double)s.z[p] + oz);
    }
    if (vel) {
      vel[3 * q] = s.vx[p];
      vel[3 * q + 1] = s.vy[p];
      vel[3 * q + 2] = s.vz[p];
    }
    if (m) m[q] = s.m[p];
    if (gid) gid[q] = s.gid ? s.gid[p] : 0;
  }
}

extern "C" int gc_pm_import(gc_ctx *ctx, const float *pos, const float *vel, const float *m, const int32_t *gid,
                            const double origin[3], const gc_particles *out) {
  if (!ctx) return GC_ERR_ARG;
  GC_REQUIRE(ctx, out && origin, "gc_pm_import: NULL particle set or origin");
  const int64_t n = out->n;
  GC_REQUIRE(ctx, n >= 0 && n < (1LL << 31), "particle count out of range");
  if (n == 0) return GC_OK;
  GC_REQUIRE(ctx, pos && vel && m, "gc_pm_import: NULL input");
  GC_REQUIRE(ctx, out->x && out->y && out->z && out->vx && out->vy && out->vz && out->m,
             "gc_pm_import: output arrays required");
  unsigned nb = gc_blocks(n, 256);
  if (nb > gc_sms() * 32u) nb = gc_sms() * 32u;
  ctx->q_next_ready = 0;  // new positions: no deposit is pending
  gc_launch(ctx, GK_COPY, k_pm_import, dim3(nb), dim3(256), 0, pos, vel, m, gid, origin[0], origin[1], origin[2], *out,
            (long long)n);
  GC_LAUNCH_CHECK(ctx, "import");
  return GC_OK;
}

extern "C" int gc_pm_export(gc_ctx *ctx, const gc_particles *p, const double origin[3], float *pos, float *vel,
                            float *m_out, int32_t *gid_out) {
  if (!ctx) return GC_ERR_ARG;
  GC_REQUIRE(ctx, p && origin, "gc_pm_export: NULL particle set or origin");
  const int64_t n = p->n;
  GC_REQUIRE(ctx, n >= 0 && n < (1LL << 31), "particle count out of range");
  if (n == 0) return GC_OK;
  GC_REQUIRE(ctx, p->pid, "gc_pm_export: pid required");
  GC_REQUIRE(ctx, !pos || (p->x && p->y && p->z), "gc_pm_export: positions missing");
  GC_REQUIRE(ctx, !vel || (p->vx && p->vy && p->vz), "gc_pm_export: velocities missing");
  GC_REQUIRE(ctx, !m_out || p->m, "gc_pm_export: masses missing");
  unsigned nb = gc_blocks(n, 256);
  if (nb > gc_sms() * 32u) nb = gc_sms() * 32u;
  gc_launch(ctx, GK_COPY, k_pm_export, dim3(nb), dim3(256), 0, *p, origin[0], origin[1], origin[2], pos, vel, m_out,
            gid_out, (long long)n, ctx->dstatus);
  GC_LAUNCH_CHECK(ctx, "export");
  return GC_OK;
}

// ---- export as a gather over the original order ---------------------------------
// gc_pm_export scatters (random writes, the whole output at once); this pair
// first inverts pid (rank[pid[i]] = i, in the sort scratch), then writes any
// range [q0, q1) of the original order with coalesced stores, so that a caller
// can copy each finished range to the host while the next one is written.
__global__ void __launch_bounds__(256)
    k_export_rank(const int32_t *__restrict__ pid, long long n, uint32_t *__restrict__ rank,
                  unsigned *__restrict__ status) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    const long long q = pid[p];
    if (q < 0 || q >= n) {
      atomicOr(status, GC_FLAG_BAD_PID);
      continue;
    }
    rank[q] = (uint32_t)p;
  }
}

__global__ void __launch_bounds__(256)
    k_export_range(gc_particles s, const uint32_t *__restrict__ rank, double ox, double oy, double oz,
                   float *__restrict__ pos, float *__restrict__ vel, float *__restrict__ m, int32_t *__restrict__ gid,
                   long long q0, long long q1, unsigned *__restrict__ status) {
  for (long long q = q0 + blockIdx.x * (long long)blockDim.x + threadIdx.x; q < q1;
       q += (long long)gridDim.x * blockDim.x) {
    const uint32_t r = rank[q];
    if (r == 0xffffffffu) {  // no particle claims this original index
      atomicOr(status, GC_FLAG_BAD_PID);
      continue;
    }
    if (pos) {
      pos[3 * q] = (float)((double)s.x[r] + ox);
      pos[3 * q + 1] = (float)((double)s.y[r] + oy);
      pos[3 * q + 2] = (float)((double)s.z[r] + oz);
    }
    if (vel) {
      vel[3 * q] = s.vx[r];
      vel[3 * q + 1] = s.vy[r];
      vel[3 * q + 2] = s.vz[r];
    }
    if (m) m[q] = s.m[r];
    if (gid) gid[q] = s.gid ? s.gid[r] : 0;
  }
}

extern "C" int gc_pm_export_order(gc_ctx *ctx, const gc_particles *p) {
  if (!ctx) return GC_ERR_ARG;
  GC_REQUIRE(ctx, p, "gc_pm_export_order: NULL particle set");
  const int64_t n = p->n;
  GC_REQUIRE(ctx, n >= 0 && n < (1LL << 31), "particle count out of range");
  ctx->export_n = 0;
  if (n == 0) return GC_OK;
  GC_REQUIRE(ctx, p->pid, "gc_pm_export_order: pid required");
  int s = gc_ensure_particle_scratch(ctx, (size_t)n);
  if (s) return s;
  ctx->import_n = 0;  // the ranks take the scratch
  ctx->import_perm = nullptr;
  GC_CUDA(ctx, cudaMemsetAsync(ctx->keys, 0xff, (size_t)n * sizeof(uint32_t), ctx->stream));
  unsigned nb = gc_blocks(n, 256);
  if (nb > gc_sms() * 32u) nb = gc_sms() * 32u;
  gc_launch(ctx, GK_COPY, k_export_rank, dim3(nb), dim3(256), 0, (const int32_t *)p->pid, (long long)n, ctx->keys,
            ctx->dstatus);
  GC_LAUNCH_CHECK(ctx, "export rank");
  ctx->export_n = n;
  ctx->export_pid = p->pid;
  return GC_OK;
}

extern "C" int gc_pm_export_range(gc_ctx *ctx, const gc_particles *p, const double origin[3], float *pos, float *vel,
                                  float *m_out, int32_t *gid_out, int64_t q0, int64_t q1) {
  if (!ctx) return GC_ERR_ARG;
  GC_REQUIRE(ctx, p && origin, "gc_pm_export_range: NULL particle set or origin");
  const int64_t n = p->n;
  GC_REQUIRE(ctx, n >= 0 && n < (1LL << 31), "particle count out of range");
  GC_REQUIRE(ctx, q0 >= 0 && q0 <= q1 && q1 <= n, "gc_pm_export_range: range [%lld, %lld) outside [0, %lld)",
             (long long)q0, (long long)q1, (long long)n);
  if (q0 == q1) return GC_OK;
  GC_REQUIRE(ctx, ctx->export_n == n, "gc_pm_export_range: no gc_pm_export_order of %lld particles before it",
             (long long)n);
  GC_REQUIRE(ctx, ctx->export_pid == p->pid,
             "gc_pm_export_range: the ranks were made by gc_pm_export_order for another particle set (pid array)");
  GC_REQUIRE(ctx, !pos || (p->x && p->y && p->z), "gc_pm_export_range: positions missing");
  GC_REQUIRE(ctx, !vel || (p->vx && p->vy && p->vz), "gc_pm_export_range: velocities missing");
  GC_REQUIRE(ctx, !m_out || p->m, "gc_pm_export_range: masses missing");
  unsigned nb = gc_blocks(q1 - q0, 256);
  if (nb > gc_sms() * 32u) nb = gc_sms() * 32u;
  gc_launch(ctx, GK_COPY, k_export_range, dim3(nb), dim3(256), 0, *p, (const uint32_t *)ctx->keys, origin[0],
            origin[1], origin[2], pos, vel, m_out, gid_out, (long long)q0, (long long)q1, ctx->dstatus);
  GC_LAUNCH_CHECK(ctx, "export range");
  return GC_OK;
}

// ---- import straight into cell order ---------------------------------------------
// Keys from the interleaved physical positions (the origin subtracted in f64,
// as gc_pm_import does), then every particle gathered from the interleaved
// arrays at its sorted slot: one random read of 12 contiguous bytes per vector
// instead of one per component, and no intermediate unsorted copy.
__global__ void __launch_bounds__(256)
    k_cell_keys_aos(const float *__restrict__ pos, double ox, double oy, double oz, long long n, float dx, int G,
                    uint32_t *__restrict__ keys) {
  const uint32_t sentinel = (uint32_t)(G + 1) * (uint32_t)(G + 1) * (uint32_t)(G + 1);
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    const float x = (float)((double)pos[3 * p] - ox);
    const float y = (float)((double)pos[3 * p + 1] - oy);
    const float z = (float)((double)pos[3 * p + 2] - oz);
    CellPos c;
    uint32_t key = sentinel;
    if (gc_cell_of(x, y, z, dx, G, c))
      key = ((uint32_t)(c.ix + 1) * (uint32_t)(G + 1) + (uint32_t)(c.iy + 1)) * (uint32_t)(G + 1) + (uint32_t)(c.iz + 1);
    keys[p] = key;
  }
}

__global__ void __launch_bounds__(256)
    k_import_gather(const float *__restrict__ pos, const float *__restrict__ vel, const float *__restrict__ m,
                    const int32_t *__restrict__ gid, bool zero_gid, double ox, double oy, double oz,
                    const uint32_t *__restrict__ perm, gc_particles o, long long n) {
  // each given input is one uniform branch: a call may gather any subset
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    const long long q = perm[p];
    if (pos) {
      const float px = __ldg(pos + 3 * q), py = __ldg(pos + 3 * q + 1), pz = __ldg(pos + 3 * q + 2);
      o.x[p] = (float)((double)px - ox);
      o.y[p] = (float)((double)py - oy);
      o.z[p] = (float)((double)pz - oz);
      if (o.pid) o.pid[p] = (int32_t)q;
    }
    if (vel) {
      const float vx = __ldg(vel + 3 * q), vy = __ldg(vel + 3 * q + 1), vz = __ldg(vel + 3 * q + 2);
      o.vx[p] = vx;
      o.vy[p] = vy;
      o.vz[p] = vz;
    }
    if (m) o.m[p] = __ldg(m + q);
    if (o.gid && (gid || zero_gid)) o.gid[p] = gid ? __ldg(gid + q) : 0;
  }
}

// Phase 1 of gc_pm_import_sorted: keys from the interleaved positions and the
// stable sort; the permutation stays in the context's scratch for phase 2.
extern "C" int gc_pm_import_order(gc_ctx *ctx, const float *pos, const double origin[3], int64_t n) {
  if (!ctx) return GC_ERR_ARG;
  GC_REQUIRE(ctx, origin && n >= 0 && n < (1LL << 31), "gc_pm_import_order: bad arguments");
  ctx->import_n = 0;
  if (n == 0) return GC_OK;
  GC_REQUIRE(ctx, pos, "gc_pm_import_order: NULL positions");
  int s = ensure_sort_scratch(ctx, n);
  if (s) return s;
  ctx->q_next_ready = 0;  // new positions: no deposit is pending
  unsigned nb = gc_blocks(n, 256);
  if (nb > gc_sms() * 32u) nb = gc_sms() * 32u;
  gc_launch(ctx, GK_KEYS, k_cell_keys_aos, dim3(nb), dim3(256), 0, pos, origin[0], origin[1], origin[2], (long long)n,
            (float)ctx->dx, ctx->G, ctx->keys2);
  GC_LAUNCH_CHECK(ctx, "cell keys");
  uint32_t *ko, *vo;
  if ((s = gc_radix_sort_pairs(ctx, ctx->keys2, nullptr, n, key_bits(ctx->G), &ko, &vo))) return s;
  ctx->import_perm = vo;
  ctx->import_n = n;
  return GC_OK;
}

// Phase 2: every particle gathered from the interleaved arrays into cell order.
extern "C" int gc_pm_import_gather(gc_ctx *ctx, const float *pos, const float *vel, const float *m, const int32_t *gid,
                                   const double origin[3], const gc_particles *out) {
  if (!ctx) return GC_ERR_ARG;
  GC_REQUIRE(ctx, out && origin, "gc_pm_import_gather: NULL particle set or origin");
  const int64_t n = out->n;
  GC_REQUIRE(ctx, n >= 0 && n < (1LL << 31), "particle count out of range");
  if (n == 0) return GC_OK;
  GC_REQUIRE(ctx, ctx->import_n == n && ctx->import_perm,
             "gc_pm_import_gather: no gc_pm_import_order of %lld particles before it", (long long)n);
  GC_REQUIRE(ctx, !pos || (out->x && out->y && out->z), "gc_pm_import_gather: position outputs required");
  GC_REQUIRE(ctx, !vel || (out->vx && out->vy && out->vz), "gc_pm_import_gather: velocity outputs required");
  GC_REQUIRE(ctx, !m || out->m, "gc_pm_import_gather: mass output required");
  if (!pos && !vel && !m && !(gid && out->gid)) return GC_OK;
  unsigned nb = gc_blocks(n, 256);
  if (nb > gc_sms() * 32u) nb = gc_sms() * 32u;
  gc_launch(ctx, GK_PERMUTE, k_import_gather, dim3(nb), dim3(256), 0, pos, vel, m, gid, pos != nullptr, origin[0],
            origin[1], origin[2], ctx->import_perm, *out, (long long)n);
  GC_LAUNCH_CHECK(ctx, "import gather");
  return GC_OK;
}

extern "C" int gc_pm_import_sorted(gc_ctx *ctx, const float *pos, const float *vel, const float *m, const int32_t *gid,
                                   const double origin[3], const gc_particles *out) {
  if (!ctx) return GC_ERR_ARG;
  GC_REQUIRE(ctx, out && origin, "gc_pm_import_sorted: NULL particle set or origin");
  int s = gc_pm_import_order(ctx, pos, origin, out->n);
  if (s) return s;
  return gc_pm_import_gather(ctx, pos, vel, m, gid, origin, out);
}
