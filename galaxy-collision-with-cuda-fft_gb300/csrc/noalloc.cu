// An allocation-free variant of the CIC deposit.
//
// Some callers of this library cannot allocate device memory at the point
// where they need a density: an application whose memory pool has already
// reserved the whole device (cudaMalloc would fail or would have to evict the
// pool), a real-time loop that must not take the implicit device-wide
// synchronisation cudaMalloc/cudaFree can cause, or an embedding with no
// context object to keep scratch in. gc_deposit_cic needs a gc_ctx (created with
// cudaMalloc) for its int64 mass grid and reduction scratch; this entry point
// keeps the same scratch in one file-scope device array instead, sized for grids
// up to GC_NOALLOC_MAX_GRID^3, and calls no allocating routine.
//
// The array lives in this library's module: every GPU that loads the library
// holds it (about 2.2 MiB) until the process exits. The host-side name of the
// array is only a stand-in, never a device address; the device address is looked
// up once per device with cudaGetSymbolAddress on the first call made with that
// device current. That first call should therefore be made before any stream
// capture begins. The cached address is per device ordinal: after
// cudaDeviceReset on a device this entry point must not be called again on it
// in the same process (the array would be mapped anew at another address). All
// calls share the one array: calls whose work overlaps on the GPU (different
// streams, or different host threads on one device) race on it and must be
// serialised by the caller.
//
// A position that is NaN or Inf deposits nothing and raises
// GC_FLAG_NONFINITE_POS. The status word the kernels raise it in is part of the
// shared array and is cleared by the next call, so callers that want to know
// pass their own device word (flags) and the bit is OR-ed into it instead.
#include "common.cuh"

#include <mutex>

#define GC_NOALLOC_MAX_GRID 64
#define GC_NOALLOC_MAX_DEVICES 64

// Kernels of particles.cu reused here (launched with explicit scratch pointers).
__global__ void __launch_bounds__(256) k_mass_max(const float *__restrict__ m, long long n, float inv_vol,
                                                  unsigned *__restrict__ maxbits);
__global__ void __launch_bounds__(256) k_mass_isum(const float *__restrict__ m, long long n, float inv_vol,
                                                   const unsigned *__restrict__ maxbits, int log2n,
                                                   unsigned long long *__restrict__ isum);
__global__ void k_qexp(const unsigned *__restrict__ maxbits, const unsigned long long *__restrict__ isum, int log2n,
                       double *__restrict__ small, int mass_slot, int exp_slot, int bits);
__global__ void __launch_bounds__(256)
    k_deposit(const float *__restrict__ x, const float *__restrict__ y, const float *__restrict__ z,
              const float *__restrict__ m, long long n, DepCtx d, const double *__restrict__ qexp,
              long long *__restrict__ qg, unsigned *__restrict__ status);
__global__ void __launch_bounds__(256)
    k_convert_q(long long *__restrict__ qg, int G, double dx, const double *__restrict__ qexp, float *__restrict__ rho,
                float *__restrict__ b, double bfac, double *__restrict__ parts, unsigned *__restrict__ ticket,
                double *__restrict__ mom, double *__restrict__ bnorm2);

// Layout of the scratch array (byte offsets, each 256-byte aligned).
#define NA_Q_BYTES ((size_t)GC_NOALLOC_MAX_GRID * GC_NOALLOC_MAX_GRID * GC_NOALLOC_MAX_GRID * 8)
#define NA_PARTS_BLOCKS ((GC_NOALLOC_MAX_GRID * GC_NOALLOC_MAX_GRID + 7) / 8)
#define NA_PARTS_BYTES ((size_t)NA_PARTS_BLOCKS * 11 * 8)
#define NA_OFF_Q 0
#define NA_OFF_PARTS (NA_OFF_Q + NA_Q_BYTES)
#define NA_OFF_SMALL (NA_OFF_PARTS + ((NA_PARTS_BYTES + 255) / 256) * 256)
#define NA_SMALL_BYTES 256
#define NA_TOTAL (NA_OFF_SMALL + NA_SMALL_BYTES)

static __device__ __align__(256) unsigned char g_noalloc_scratch[NA_TOTAL];

static std::mutex g_noalloc_mutex;
static unsigned char *g_noalloc_addr[GC_NOALLOC_MAX_DEVICES];

// Device address of the scratch array on the current device (looked up once).
static int noalloc_scratch(unsigned char **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    gc_set_error(nullptr, "gc_deposit_cic_noalloc: cudaGetDevice: %s", cudaGetErrorString(e));
    return GC_ERR_CUDA;
  }
  if (dev < 0 || dev >= GC_NOALLOC_MAX_DEVICES) {
    gc_set_error(nullptr, "gc_deposit_cic_noalloc: device %d beyond the supported %d", dev, GC_NOALLOC_MAX_DEVICES);
    return GC_ERR_ARG;
  }
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_addr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      gc_set_error(nullptr, "gc_deposit_cic_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
      return GC_ERR_CUDA;
    }
    g_noalloc_addr[dev] = (unsigned char *)p;
  }
  *out = g_noalloc_addr[dev];
  return GC_OK;
}

extern "C" int gc_deposit_cic_noalloc(const float *x, const float *y, const float *z, const float *m, int64_t n,
                                      int grid_size, double dx, int fixed_point_bits, float *rho,
                                      uint32_t *flags, void *stream) {
  if (grid_size < 2 || grid_size > GC_NOALLOC_MAX_GRID) {
    gc_set_error(nullptr, "gc_deposit_cic_noalloc: grid_size must be in [2, %d], got %d", GC_NOALLOC_MAX_GRID,
                 grid_size);
    return GC_ERR_ARG;
  }
  if (!(dx > 0.0) || !(dx < 1e30)) {
    gc_set_error(nullptr, "gc_deposit_cic_noalloc: dx must be positive and finite, got %g", dx);
    return GC_ERR_ARG;
  }
  if (n < 0 || n >= (1LL << 31)) {
    gc_set_error(nullptr, "gc_deposit_cic_noalloc: particle count out of range: %lld", (long long)n);
    return GC_ERR_ARG;
  }
  if (!rho || (n > 0 && !(x && y && z && m))) {
    gc_set_error(nullptr, "gc_deposit_cic_noalloc: NULL pointer");
    return GC_ERR_ARG;
  }
  int lg = 0;
  while ((1 << lg) < grid_size) ++lg;
  const int max_bits = 62 - lg > 60 ? 60 : 62 - lg;
  if (fixed_point_bits < 24 || fixed_point_bits > max_bits) {
    gc_set_error(nullptr, "gc_deposit_cic_noalloc: fixed_point_bits must be in [24, %d] for a %d^3 grid", max_bits,
                 grid_size);
    return GC_ERR_ARG;
  }
  unsigned char *base = nullptr;
  int s = noalloc_scratch(&base);
  if (s) return s;
  cudaStream_t st = (cudaStream_t)stream;
  const int G = grid_size;
  const size_t g3 = (size_t)G * G * G;
  long long *q = (long long *)(base + NA_OFF_Q);
  double *parts = (double *)(base + NA_OFF_PARTS);
  double *small = (double *)(base + NA_OFF_SMALL);
  unsigned *maxbits = (unsigned *)(small + 4);
  unsigned long long *isum = (unsigned long long *)(small + 5);
  // the caller's status word when given (it outlives the call), else a scratch slot
  unsigned *status = flags ? (unsigned *)flags : (unsigned *)(small + 6);
  // the array keeps the previous call's contents: clear what must start at zero
  cudaError_t e = cudaMemsetAsync(q, 0, g3 * sizeof(long long), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(small, 0, NA_SMALL_BYTES, st);
  if (e != cudaSuccess) {
    gc_set_error(nullptr, "gc_deposit_cic_noalloc: cudaMemsetAsync: %s", cudaGetErrorString(e));
    return GC_ERR_CUDA;
  }
  const float dxf = (float)dx;
  DepCtx d;
  d.dx = dxf;
  d.inv_vol = 1.0f / ((dxf * dxf) * dxf);
  d.G = G;
  if (n > 0) {
    unsigned nb = gc_blocks(n, 256);
    if (nb > gc_sms() * 8u) nb = gc_sms() * 8u;
    int L = 0;
    while ((1LL << L) < n) ++L;
    k_mass_max<<<nb, 256, 0, st>>>(m, (long long)n, d.inv_vol, maxbits);
    k_mass_isum<<<nb, 256, 0, st>>>(m, (long long)n, d.inv_vol, maxbits, L, isum);
    k_qexp<<<1, 32, 0, st>>>(maxbits, isum, L, small, 0, 1, fixed_point_bits);
    unsigned nd = gc_blocks(n, 256);
    if (nd > gc_sms() * 32u) nd = gc_sms() * 32u;
    k_deposit<<<nd, 256, 0, st>>>(x, y, z, m, (long long)n, d, small + 1, q, status);
  }
  // rho from q (q is cleared again by the conversion); the moments land in parts
  const unsigned nbc = gc_blocks((long long)G * G, 8);
  k_convert_q<<<nbc, 256, 0, st>>>(q, G, dx, small + 1, rho, nullptr, 1.0, parts, nullptr, nullptr, nullptr);
  e = cudaGetLastError();
  if (e != cudaSuccess) {
    gc_set_error(nullptr, "gc_deposit_cic_noalloc: launch failed: %s", cudaGetErrorString(e));
    return GC_ERR_CUDA;
  }
  return GC_OK;
}
