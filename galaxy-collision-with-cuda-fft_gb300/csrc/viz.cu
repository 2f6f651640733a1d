// Headless visualisation kernels: the device side of the reference's viewer
// (src/galaxy_collision/viz/viewer.py) without a graphics API. The 2-D view's
// LogNorm colormap and the 3-D view's subsample, density colouring and point
// drawing all produce device buffers; a caller writes them to image files.
//
// Arithmetic is f32 with explicit round-to-nearest operations (no contraction),
// so the NumPy restatement in the tests reproduces every colour index and
// every rasterised pixel exactly.
#include "common.cuh"

#define GC_LUT_N 256

// Largest value of a (nonnegative) f32 array into *out (the peak that sets the
// colormap's log window, viewer.py:68-73, 98-101). out is cleared first.
__global__ void __launch_bounds__(256) k_max_f32(const float *__restrict__ a, long long n, float *__restrict__ out) {
  float v = 0.0f;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    v = fmaxf(v, a[i]);
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_down_sync(0xffffffffu, v, o));
  // nonnegative floats order like their bit patterns
  if ((threadIdx.x & 31) == 0) atomicMax(reinterpret_cast<unsigned *>(out), __float_as_uint(v));
}

// t = clamp01((ln v - log_vmin) * inv_logspan) (0 for v <= 0), index
// int(t * 255 + 0.5): viewer.py:76-93 and 104-121.
__device__ __forceinline__ int lut_index(float v, float log_vmin, float inv_logspan) {
  float t = 0.0f;
  if (v > 0.0f) t = __fmul_rn(__fsub_rn(logf(v), log_vmin), inv_logspan);
  t = fminf(1.0f, fmaxf(0.0f, t));
  int idx = (int)__fadd_rn(__fmul_rn(t, (float)(GC_LUT_N - 1)), 0.5f);
  return idx < 0 ? 0 : (idx > GC_LUT_N - 1 ? GC_LUT_N - 1 : idx);
}

__global__ void __launch_bounds__(256)
    k_colormap_log(const float *__restrict__ img, long long n, const float *__restrict__ lut, float log_vmin,
                   float inv_logspan, float *__restrict__ rgb) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int idx = lut_index(img[i], log_vmin, inv_logspan);
    rgb[3 * i] = lut[3 * idx];
    rgb[3 * i + 1] = lut[3 * idx + 1];
    rgb[3 * i + 2] = lut[3 * idx + 2];
  }
}

// Every stride-th particle, in a unit cube centred on the origin (viewer.py:52-65).
__global__ void __launch_bounds__(256)
    k_pack_positions(const float *__restrict__ x, const float *__restrict__ y, const float *__restrict__ z,
                     long long stride, float inv_box, long long m, float *__restrict__ out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < m; i += (long long)gridDim.x * blockDim.x) {
    const long long p = i * stride;
    out[3 * i] = __fsub_rn(__fmul_rn(x[p], inv_box), 0.5f);
    out[3 * i + 1] = __fsub_rn(__fmul_rn(y[p], inv_box), 0.5f);
    out[3 * i + 2] = __fsub_rn(__fmul_rn(z[p], inv_box), 0.5f);
  }
}

// Colour of every drawn particle from the density at its nearest node
// (viewer.py:104-121): index clamp(int(x * inv_dx + 0.5)) per axis.
__global__ void __launch_bounds__(256)
    k_density_color(const float *__restrict__ x, const float *__restrict__ y, const float *__restrict__ z,
                    const float *__restrict__ rho, long long stride, long long m, float inv_dx, int G,
                    const float *__restrict__ lut, float log_vmin, float inv_logspan, float *__restrict__ col) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < m; i += (long long)gridDim.x * blockDim.x) {
    const long long p = i * stride;
    int n3[3];
    const float c[3] = {x[p], y[p], z[p]};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const int v = (int)__fadd_rn(__fmul_rn(c[a], inv_dx), 0.5f);
      n3[a] = v < 0 ? 0 : (v > G - 1 ? G - 1 : v);
    }
    const float v = rho[((size_t)n3[0] * G + n3[1]) * G + n3[2]];
    const int idx = lut_index(v, log_vmin, inv_logspan);
    col[3 * i] = lut[3 * idx];
    col[3 * i + 1] = lut[3 * idx + 1];
    col[3 * i + 2] = lut[3 * idx + 2];
  }
}

// ---- point splat: the 3-D view's scene.particles drawn as flat discs -----------
// A point p (unit-cube coordinates) goes through the row-major 4x4 matrix M to
// clip space (products and sums in the order written, f32), then to pixel
// centre (px, py) = ((xc/w + 1) * W/2, (1 - yc/w) * H/2) and depth zc/w. Points
// with w <= 0 or depth outside [0, 1] are not drawn. A disc of radius r pixels
// covers pixel (u, v) when (u + 0.5 - px)^2 + (v + 0.5 - py)^2 <= r^2. Per pixel
// the nearest point wins, ties to the lower index: each covered pixel takes
// atomicMin of (depth bits << 32 | index), then a resolve pass writes RGBA8.
struct SplatCam {
  float m[16];
  int W, H;
  float r;
};

__device__ __forceinline__ bool splat_project(const SplatCam &c, float x, float y, float z, float &px, float &py,
                                              float &depth) {
  const float *M = c.m;
  const float xc = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(M[0], x), __fmul_rn(M[1], y)), __fmul_rn(M[2], z)), M[3]);
  const float yc = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(M[4], x), __fmul_rn(M[5], y)), __fmul_rn(M[6], z)), M[7]);
  const float zc = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(M[8], x), __fmul_rn(M[9], y)), __fmul_rn(M[10], z)), M[11]);
  const float wc = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(M[12], x), __fmul_rn(M[13], y)), __fmul_rn(M[14], z)), M[15]);
  if (!(wc > 0.0f)) return false;
  const float iw = __fdiv_rn(1.0f, wc);
  depth = __fadd_rn(__fmul_rn(zc, iw), 0.0f);  // -0 becomes +0, so depth bits order like depths
  if (!(depth >= 0.0f && depth <= 1.0f)) return false;
  px = __fmul_rn(__fadd_rn(__fmul_rn(xc, iw), 1.0f), __fmul_rn(0.5f, (float)c.W));
  py = __fmul_rn(__fsub_rn(1.0f, __fmul_rn(yc, iw)), __fmul_rn(0.5f, (float)c.H));
  return true;
}

__global__ void __launch_bounds__(256)
    k_splat(const float *__restrict__ pos, long long m, SplatCam c, unsigned long long *__restrict__ zbuf) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < m; i += (long long)gridDim.x * blockDim.x) {
    float px, py, depth;
    if (!splat_project(c, pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], px, py, depth)) continue;
    const float r2 = __fmul_rn(c.r, c.r);
    const int u0 = max(0, (int)floorf(__fsub_rn(px, c.r))), u1 = min(c.W - 1, (int)floorf(__fadd_rn(px, c.r)));
    const int v0 = max(0, (int)floorf(__fsub_rn(py, c.r))), v1 = min(c.H - 1, (int)floorf(__fadd_rn(py, c.r)));
    const unsigned long long key = ((unsigned long long)__float_as_uint(depth) << 32) | (unsigned long long)i;
    for (int v = v0; v <= v1; ++v) {
      const float dy = __fsub_rn(__fadd_rn((float)v, 0.5f), py);
      for (int u = u0; u <= u1; ++u) {
        const float dx = __fsub_rn(__fadd_rn((float)u, 0.5f), px);
        if (__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)) <= r2) atomicMin(zbuf + (size_t)v * c.W + u, key);
      }
    }
  }
}

__device__ __forceinline__ unsigned char to_u8(float v) {
  const float t = fminf(1.0f, fmaxf(0.0f, v));
  return (unsigned char)(int)__fadd_rn(__fmul_rn(t, 255.0f), 0.5f);
}

__global__ void __launch_bounds__(256)
    k_splat_resolve(const unsigned long long *__restrict__ zbuf, long long npix, const float *__restrict__ col,
                    float3 bg, unsigned char *__restrict__ rgba) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < npix;
       i += (long long)gridDim.x * blockDim.x) {
    const unsigned long long k = zbuf[i];
    float r = bg.x, g = bg.y, b = bg.z;
    if (k != ~0ULL) {
      const long long p = (long long)(k & 0xffffffffULL);
      r = col[3 * p]; g = col[3 * p + 1]; b = col[3 * p + 2];
    }
    rgba[4 * i] = to_u8(r);
    rgba[4 * i + 1] = to_u8(g);
    rgba[4 * i + 2] = to_u8(b);
    rgba[4 * i + 3] = 255;
  }
}

__global__ void k_fill_u64(unsigned long long *__restrict__ a, long long n, unsigned long long v) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    a[i] = v;
}

static unsigned grid_of(long long n) {
  unsigned nb = gc_blocks(n, 256);
  return nb > gc_sms() * 16u ? gc_sms() * 16u : (nb == 0 ? 1u : nb);
}

extern "C" int gc_max_f32(gc_ctx *ctx, const float *a, int64_t n, float *out) {
  if (!ctx) return GC_ERR_ARG;
  GC_REQUIRE(ctx, out && (n == 0 || a) && n >= 0, "gc_max_f32: bad arguments");
  GC_CUDA(ctx, cudaMemsetAsync(out, 0, sizeof(float), ctx->stream));
  if (n == 0) return GC_OK;
  gc_launch(ctx, GK_VIZ, k_max_f32, dim3(grid_of(n)), dim3(256), 0, a, (long long)n, out);
  GC_LAUNCH_CHECK(ctx, "max");
  return GC_OK;
}

extern "C" int gc_colormap_log(gc_ctx *ctx, const float *img, int64_t n, const float *lut, float log_vmin,
                               float inv_logspan, float *rgb) {
  if (!ctx) return GC_ERR_ARG;
  GC_REQUIRE(ctx, n >= 0 && (n == 0 || (img && lut && rgb)), "gc_colormap_log: bad arguments");
  if (n == 0) return GC_OK;
  gc_launch(ctx, GK_VIZ, k_colormap_log, dim3(grid_of(n)), dim3(256), 0, img, (long long)n, lut, log_vmin,
            inv_logspan, rgb);
  GC_LAUNCH_CHECK(ctx, "colormap");
  return GC_OK;
}

extern "C" int gc_pack_positions(gc_ctx *ctx, const float *x, const float *y, const float *z, int64_t stride,
                                 float inv_box, int64_t m, float *out) {
  if (!ctx) return GC_ERR_ARG;
  GC_REQUIRE(ctx, stride >= 1 && m >= 0 && (m == 0 || (x && y && z && out)), "gc_pack_positions: bad arguments");
  if (m == 0) return GC_OK;
  gc_launch(ctx, GK_VIZ, k_pack_positions, dim3(grid_of(m)), dim3(256), 0, x, y, z, (long long)stride, inv_box,
            (long long)m, out);
  GC_LAUNCH_CHECK(ctx, "pack positions");
  return GC_OK;
}

extern "C" int gc_density_color(gc_ctx *ctx, const float *x, const float *y, const float *z, const float *rho,
                                int grid, int64_t stride, int64_t m, float inv_dx, const float *lut, float log_vmin,
                                float inv_logspan, float *col) {
  if (!ctx) return GC_ERR_ARG;
  GC_REQUIRE(ctx, grid >= 1 && stride >= 1 && m >= 0, "gc_density_color: bad sizes");
  if (m == 0) return GC_OK;
  GC_REQUIRE(ctx, x && y && z && rho && lut && col, "gc_density_color: NULL pointer");
  gc_launch(ctx, GK_VIZ, k_density_color, dim3(grid_of(m)), dim3(256), 0, x, y, z, rho, (long long)stride,
            (long long)m, inv_dx, grid, lut, log_vmin, inv_logspan, col);
  GC_LAUNCH_CHECK(ctx, "density colour");
  return GC_OK;
}

extern "C" int gc_splat_points(gc_ctx *ctx, const float *pos, const float *col, int64_t m, const float view_proj[16],
                               int width, int height, float radius_px, const float bg[3],
                               unsigned long long *zbuf, unsigned char *rgba) {
  if (!ctx) return GC_ERR_ARG;
  GC_REQUIRE(ctx, width >= 1 && height >= 1 && (long long)width * height <= (1LL << 30),
             "gc_splat_points: image size %d x %d out of range", width, height);
  GC_REQUIRE(ctx, m >= 0 && m < (1LL << 32), "gc_splat_points: point count out of range");
  GC_REQUIRE(ctx, radius_px >= 0.0f && radius_px <= 64.0f, "gc_splat_points: radius must be in [0, 64] pixels");
  GC_REQUIRE(ctx, view_proj && bg && zbuf && rgba && (m == 0 || (pos && col)), "gc_splat_points: NULL pointer");
  SplatCam c;
  for (int i = 0; i < 16; ++i) c.m[i] = view_proj[i];
  c.W = width;
  c.H = height;
  c.r = radius_px;
  const long long npix = (long long)width * height;
  const float3 bgc = make_float3(bg[0], bg[1], bg[2]);
  gc_launch(ctx, GK_VIZ, k_fill_u64, dim3(grid_of(npix)), dim3(256), 0, zbuf, npix, ~0ULL);
  if (m > 0) gc_launch(ctx, GK_VIZ, k_splat, dim3(grid_of(m)), dim3(256), 0, pos, (long long)m, c, zbuf);
  gc_launch(ctx, GK_VIZ, k_splat_resolve, dim3(grid_of(npix)), dim3(256), 0, (const unsigned long long *)zbuf, npix,
            col, bgc, rgba);
  GC_LAUNCH_CHECK(ctx, "splat");
  return GC_OK;
}
