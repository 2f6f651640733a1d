// Initial conditions sampled on the device (the Plummer sphere and the
// exponential sech^2 disks of the benchmark configurations), with a
// counter-based generator so that particle i's values depend only on (seed, i)
// and not on the launch shape or the particle count.
//
// Generator: Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random
// numbers: as easy as 1, 2, 3", SC 2011): a 4 x 32-bit counter and a 2 x 32-bit
// key, ten rounds of two 32 x 32 -> 64-bit multiplies whose halves are mixed
// with the other counter words and the key, the key bumped by the Weyl
// constants between rounds. The counter is (particle index low, high, attempt,
// stream); the key is the seed.
#include "common.cuh"

#include <math.h>

struct P4 {
  uint32_t x, y, z, w;
};

__host__ __device__ __forceinline__ P4 philox4x32_10(P4 c, uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = (uint64_t)M0 * c.x, p1 = (uint64_t)M1 * c.z;
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    c = P4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
    k0 += W0;
    k1 += W1;
  }
  return c;
}

// Uniform f32 in (0, 1): the top 24 bits, offset by half a step.
__host__ __device__ __forceinline__ float u01(uint32_t b) { return ((float)(b >> 8) + 0.5f) * (1.0f / 16777216.0f); }

__device__ __forceinline__ P4 rng4(uint64_t seed, long long i, uint32_t attempt, uint32_t stream) {
  return philox4x32_10(P4{(uint32_t)i, (uint32_t)((unsigned long long)i >> 32), attempt, stream}, (uint32_t)seed,
                       (uint32_t)(seed >> 32));
}

// Streams (fourth counter word) of the samplers.
enum { RS_UNIFORM = 0, RS_PL_R = 1, RS_PL_DIR = 2, RS_PL_Q = 3, RS_PL_VDIR = 4, RS_DK_A = 5, RS_DK_B = 6 };

__global__ void __launch_bounds__(256) k_rng_uniform(uint64_t seed, uint32_t stream, long long n, float *__restrict__ out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const P4 r = rng4(seed, i, 0, stream);
    out[4 * i] = u01(r.x);
    out[4 * i + 1] = u01(r.y);
    out[4 * i + 2] = u01(r.z);
    out[4 * i + 3] = u01(r.w);
  }
}

__device__ __forceinline__ void unit_vector(const P4 &r, float &ux, float &uy, float &uz) {
  const float ct = 2.0f * u01(r.x) - 1.0f;
  const float st = sqrtf(fmaxf(0.0f, 1.0f - ct * ct));
  float sp, cp;
  sincospif(2.0f * u01(r.y), &sp, &cp);
  ux = st * cp;
  uy = st * sp;
  uz = ct;
}

// Plummer sphere (the benchmark's sampler, restated from its definition):
// r = a / sqrt(u^(-2/3) - 1) kept when r <= rmax a, isotropic directions,
// speed q v_esc with q drawn from g(q) = q^2 (1 - q^2)^(7/2) by rejection
// (0.1 y < g(x)), v_esc = sqrt(2 G M / a) (1 + r^2/a^2)^(-1/4).
__global__ void __launch_bounds__(256)
    k_ic_plummer(long long n, uint64_t seed, float mass, float a, float rmax, float grav, float *__restrict__ pos,
                 float *__restrict__ vel, float *__restrict__ m, int32_t *__restrict__ gid,
                 unsigned *__restrict__ status) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    float r = rmax * a;
    bool ok = false;
    for (uint32_t t = 0; t < 64 && !ok; ++t) {  // acceptance 0.985 per draw at rmax = 10 a
      const P4 q = rng4(seed, i, t, RS_PL_R);
      const float u = u01(q.x);
      const float rr = a / sqrtf(powf(u, -2.0f / 3.0f) - 1.0f);
      if (rr <= rmax * a) { r = rr; ok = true; }
    }
    float qv = 0.0f;
    bool qok = false;
    for (uint32_t t = 0; t < 512 && !qok; ++t) {  // acceptance ~0.19 per draw
      const P4 q = rng4(seed, i, t, RS_PL_Q);
      const float x = u01(q.x), y = u01(q.y);
      const float g = x * x * powf(1.0f - x * x, 3.5f);
      if (0.1f * y < g) { qv = x; qok = true; }
    }
    if (!ok || !qok) atomicOr(status, GC_FLAG_IC_REJECT);
    float ux, uy, uz, vx, vy, vz;
    unit_vector(rng4(seed, i, 0, RS_PL_DIR), ux, uy, uz);
    unit_vector(rng4(seed, i, 0, RS_PL_VDIR), vx, vy, vz);
    const float ra = r / a;
    const float vesc = sqrtf(2.0f * grav * mass / a) * powf(1.0f + ra * ra, -0.25f);
    const float v = qv * vesc;
    pos[3 * i] = r * ux; pos[3 * i + 1] = r * uy; pos[3 * i + 2] = r * uz;
    vel[3 * i] = v * vx; vel[3 * i + 1] = v * vy; vel[3 * i + 2] = v * vz;
    m[i] = mass / (float)n;
    gid[i] = 0;
  }
}

// One exponential sech^2 disk (surface density ~ exp(-R/Rd) cut at 5 Rd, scale
// height 0.1 Rd) with its central point mass (1 % of the disk mass) as the last
// particle. Circular speed from the enclosed disk mass plus the point mass,
// softened by `soft` (Plummer form), with a 10 % Gaussian dispersion in every
// component. The galaxy is then inclined about x, shifted by `off` and given
// the bulk velocity `bulk`.
struct DiskParams {
  long long nd;       // disk particles (the point mass is particle nd)
  uint64_t seed;
  uint32_t stream;    // galaxy index: separates the galaxies' random streams
  float m_disk, rd, grav, soft, cos_i, sin_i;
  float off[3], bulk[3];
  int gid;
};

__device__ __forceinline__ float disk_cdf(float x) { return 1.0f - (1.0f + x) * expf(-x); }  // x = R / Rd

__global__ void __launch_bounds__(256)
    k_ic_disk(DiskParams p, float *__restrict__ pos, float *__restrict__ vel, float *__restrict__ m,
              int32_t *__restrict__ gid) {
  const float c5 = disk_cdf(5.0f);
  const float m_bh = 0.01f * p.m_disk;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i <= p.nd;
       i += (long long)gridDim.x * blockDim.x) {
    float x, y, z, vx, vy, vz, mm;
    if (i == p.nd) {  // the central point mass
      x = y = z = vx = vy = vz = 0.0f;
      mm = m_bh;
    } else {
      const P4 a = rng4(p.seed, i, p.stream, RS_DK_A);
      const P4 b = rng4(p.seed, i, p.stream, RS_DK_B);
      // R: inverse of the truncated cumulative mass by bisection (monotone)
      const float target = u01(a.x) * c5;
      float lo = 0.0f, hi = 5.0f;
#pragma unroll 1
      for (int it = 0; it < 26; ++it) {
        const float mid = 0.5f * (lo + hi);
        if (disk_cdf(mid) < target) lo = mid; else hi = mid;
      }
      const float R = 0.5f * (lo + hi) * p.rd;
      float sp, cp;
      sincospif(2.0f * u01(a.y), &sp, &cp);
      const float s2 = fminf(fmaxf(2.0f * u01(a.z) - 1.0f, -0.9999999f), 0.9999999f);
      z = 0.1f * p.rd * atanhf(s2);
      const float menc = p.m_disk * (disk_cdf(R / p.rd) / c5) + m_bh;
      const float d2 = R * R + p.soft * p.soft;
      const float vc = sqrtf(p.grav * menc * R * R / (d2 * sqrtf(d2)));
      // three Gaussians (Box-Muller on two pairs of uniforms)
      const float r1 = sqrtf(-2.0f * logf(u01(a.w))), r2 = sqrtf(-2.0f * logf(u01(b.x)));
      float s1, c1, s2b, c2b;
      sincospif(2.0f * u01(b.y), &s1, &c1);
      sincospif(2.0f * u01(b.z), &s2b, &c2b);
      const float sig = 0.1f * vc;
      x = R * cp;
      y = R * sp;
      vx = -vc * sp + sig * r1 * c1;
      vy = vc * cp + sig * r1 * s1;
      vz = sig * r2 * c2b;
      mm = p.m_disk / (float)p.nd;
    }
    // incline about x, then shift and boost
    const float y2 = p.cos_i * y - p.sin_i * z, z2 = p.sin_i * y + p.cos_i * z;
    const float vy2 = p.cos_i * vy - p.sin_i * vz, vz2 = p.sin_i * vy + p.cos_i * vz;
    pos[3 * i] = x + p.off[0]; pos[3 * i + 1] = y2 + p.off[1]; pos[3 * i + 2] = z2 + p.off[2];
    vel[3 * i] = vx + p.bulk[0]; vel[3 * i + 1] = vy2 + p.bulk[1]; vel[3 * i + 2] = vz2 + p.bulk[2];
    m[i] = mm;
    gid[i] = p.gid;
  }
}

static unsigned ic_grid(long long n) {
  unsigned nb = gc_blocks(n, 256);
  return nb > gc_sms() * 16u ? gc_sms() * 16u : (nb == 0 ? 1u : nb);
}

extern "C" int gc_rng_uniform(gc_ctx *ctx, uint64_t seed, uint32_t stream, int64_t n, float *out) {
  if (!ctx) return GC_ERR_ARG;
  GC_REQUIRE(ctx, n >= 0 && (n == 0 || out), "gc_rng_uniform: bad arguments");
  if (n == 0) return GC_OK;
  gc_launch(ctx, GK_IC, k_rng_uniform, dim3(ic_grid(n)), dim3(256), 0, seed, stream, (long long)n, out);
  GC_LAUNCH_CHECK(ctx, "rng");
  return GC_OK;
}

extern "C" int gc_ic_plummer(gc_ctx *ctx, int64_t n, uint64_t seed, double mass, double a, double rmax, double grav,
                             float *pos, float *vel, float *m, int32_t *gid) {
  if (!ctx) return GC_ERR_ARG;
  GC_REQUIRE(ctx, n >= 1 && n < (1LL << 31), "gc_ic_plummer: particle count out of range");
  GC_REQUIRE(ctx, mass > 0 && a > 0 && rmax > 0 && grav > 0, "gc_ic_plummer: parameters must be positive");
  GC_REQUIRE(ctx, pos && vel && m && gid, "gc_ic_plummer: NULL output");
  gc_launch(ctx, GK_IC, k_ic_plummer, dim3(ic_grid(n)), dim3(256), 0, (long long)n, seed, (float)mass, (float)a,
            (float)rmax, (float)grav, pos, vel, m, gid, ctx->dstatus);
  GC_LAUNCH_CHECK(ctx, "plummer");
  return GC_OK;
}

extern "C" int gc_ic_disk(gc_ctx *ctx, int64_t n_disk, uint64_t seed, int galaxy, double m_disk, double rd,
                          double grav, double soft, double incline_deg, const double off[3], const double bulk[3],
                          float *pos, float *vel, float *m, int32_t *gid) {
  if (!ctx) return GC_ERR_ARG;
  GC_REQUIRE(ctx, n_disk >= 1 && n_disk < (1LL << 31) - 1, "gc_ic_disk: particle count out of range");
  GC_REQUIRE(ctx, m_disk > 0 && rd > 0 && grav > 0 && soft >= 0, "gc_ic_disk: bad parameters");
  GC_REQUIRE(ctx, off && bulk && pos && vel && m && gid, "gc_ic_disk: NULL pointer");
  DiskParams p;
  p.nd = n_disk;
  p.seed = seed;
  p.stream = (uint32_t)galaxy;
  p.m_disk = (float)m_disk;
  p.rd = (float)rd;
  p.grav = (float)grav;
  p.soft = (float)soft;
  const double ang = incline_deg * M_PI / 180.0;
  p.cos_i = (float)cos(ang);
  p.sin_i = (float)sin(ang);
  for (int c = 0; c < 3; ++c) {
    p.off[c] = (float)off[c];
    p.bulk[c] = (float)bulk[c];
  }
  p.gid = galaxy;
  gc_launch(ctx, GK_IC, k_ic_disk, dim3(ic_grid(n_disk + 1)), dim3(256), 0, p, pos, vel, m, gid);
  GC_LAUNCH_CHECK(ctx, "disk");
  return GC_OK;
}
