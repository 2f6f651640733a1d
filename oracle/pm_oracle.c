/*
 * pm_oracle.c -- CPU restatement of the reference's PM hot path.
 *
 * TEST INFRASTRUCTURE ONLY: this is the oracle the GPU library is checked
 * against (tests/, the smoke check and the CPU-baseline leg of bench.py). It is
 * never part of the product path.
 *
 * It restates, operation by operation in IEEE f32 (built with
 * -ffp-contract=off, no fast-math, so no FMA contraction or reassociation), the
 * Taichi kernels of pouyalj/Galaxy-Collision-with-CUDA-FFT, package
 * src/galaxy_collision:
 *   deposit.py:47-82      _deposit_cic          -> or_deposit_f32 / _f64 / _fixed
 *   deposit.py:85-129     _gather_accel         -> or_gather
 *   deposit.py:132-174    _potential_to_accel   -> or_grad
 *   integrator.py:27-59   kick / drift          -> or_kick / or_drift
 *   solver/multigrid.py:46-130   RB-GS, residual, restriction, prolongation
 *   solver/multigrid.py:133-189  moments, sum of squares (f64)
 *   solver/multigrid.py:261-295  multipole Dirichlet faces (f32)
 *   solver/multigrid.py:330-341, 422-487  hierarchy, V-cycle, adaptive solve
 * Parallel loops use OpenMP where the reference's loop is a Taichi parallel
 * for; the serial deposit gives a deterministic f32 sum (the reference's
 * parallel f32 atomics are order-dependent).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define IDX(i, j, k, n) (((size_t)(i) * (size_t)(n) + (size_t)(j)) * (size_t)(n) + (size_t)(k))

int or_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void or_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

/* ---- cell index (deposit.py:62-70) --------------------------------------- */
typedef struct {
  int ix, iy, iz;
  float fx, fy, fz;
} cellpos;

static int cell_of(float x, float y, float z, float dx, int G, cellpos *c) {
  const float gx = x / dx, gy = y / dx, gz = z / dx;
  if (!(gx >= -1.0f && gx < (float)G && gy >= -1.0f && gy < (float)G && gz >= -1.0f && gz < (float)G)) return 0;
  const float flx = floorf(gx), fly = floorf(gy), flz = floorf(gz);
  c->ix = (int)flx; c->iy = (int)fly; c->iz = (int)flz;
  c->fx = gx - flx; c->fy = gy - fly; c->fz = gz - flz;
  return 1;
}

/* key = ((ix+1)(G+1) + (iy+1))(G+1) + (iz+1); sentinel (G+1)^3 when nothing is deposited */
void or_cell_keys(const float *x, const float *y, const float *z, int64_t n, float dx, int G, uint32_t *keys) {
  const uint32_t g1 = (uint32_t)(G + 1);
  for (int64_t p = 0; p < n; ++p) {
    cellpos c;
    keys[p] = cell_of(x[p], y[p], z[p], dx, G, &c)
                  ? ((uint32_t)(c.ix + 1) * g1 + (uint32_t)(c.iy + 1)) * g1 + (uint32_t)(c.iz + 1)
                  : g1 * g1 * g1;
  }
}

/* ---- deposit (deposit.py:47-82) ------------------------------------------ */
static inline float inv_vol_of(float dx) { return 1.0f / (dx * dx * dx); }

/* The 8 f32 contributions m*wx*wy*wz of one particle in (cx,cy,cz) order. */
static inline void contribs(const cellpos *c, float mm, float w[8]) {
  const float wx[2] = {1.0f - c->fx, c->fx};
  const float wy[2] = {1.0f - c->fy, c->fy};
  const float wz[2] = {1.0f - c->fz, c->fz};
  for (int a = 0; a < 2; ++a)
    for (int b = 0; b < 2; ++b)
      for (int d = 0; d < 2; ++d) w[(a * 2 + b) * 2 + d] = ((mm * wx[a]) * wy[b]) * wz[d];
}

/* Serial f32 accumulation in particle order (one admissible order of the
 * reference's atomics). parallel != 0: OpenMP with f32 atomics, as the
 * reference runs on its CPU backend (order-dependent). */
void or_deposit_f32(const float *x, const float *y, const float *z, const float *m, int64_t n, float dx, int G,
                    float *rho, int parallel) {
  const size_t g3 = (size_t)G * G * G;
  memset(rho, 0, g3 * sizeof(float));
  const float inv_vol = inv_vol_of(dx);
  if (!parallel) {
    for (int64_t p = 0; p < n; ++p) {
      cellpos c;
      if (!cell_of(x[p], y[p], z[p], dx, G, &c)) continue;
      float w[8];
      contribs(&c, m[p] * inv_vol, w);
      for (int t = 0; t < 8; ++t) {
        const int jx = c.ix + (t >> 2), jy = c.iy + ((t >> 1) & 1), jz = c.iz + (t & 1);
        if (jx >= 0 && jx < G && jy >= 0 && jy < G && jz >= 0 && jz < G) rho[IDX(jx, jy, jz, G)] += w[t];
      }
    }
    return;
  }
#pragma omp parallel for schedule(static)
  for (int64_t p = 0; p < n; ++p) {
    cellpos c;
    if (!cell_of(x[p], y[p], z[p], dx, G, &c)) continue;
    float w[8];
    contribs(&c, m[p] * inv_vol, w);
    for (int t = 0; t < 8; ++t) {
      const int jx = c.ix + (t >> 2), jy = c.iy + ((t >> 1) & 1), jz = c.iz + (t & 1);
      if (jx >= 0 && jx < G && jy >= 0 && jy < G && jz >= 0 && jz < G) {
#pragma omp atomic
        rho[IDX(jx, jy, jz, G)] += w[t];
      }
    }
  }
}

/* The same f32 contributions summed in f64 (the FP64 oracle deposit). */
void or_deposit_f64(const float *x, const float *y, const float *z, const float *m, int64_t n, float dx, int G,
                    double *rho) {
  const size_t g3 = (size_t)G * G * G;
  memset(rho, 0, g3 * sizeof(double));
  const float inv_vol = inv_vol_of(dx);
  for (int64_t p = 0; p < n; ++p) {
    cellpos c;
    if (!cell_of(x[p], y[p], z[p], dx, G, &c)) continue;
    float w[8];
    contribs(&c, m[p] * inv_vol, w);
    for (int t = 0; t < 8; ++t) {
      const int jx = c.ix + (t >> 2), jy = c.iy + ((t >> 1) & 1), jz = c.iz + (t & 1);
      if (jx >= 0 && jx < G && jy >= 0 && jy < G && jz >= 0 && jz < G) rho[IDX(jx, jy, jz, G)] += (double)w[t];
    }
  }
}

/* The partial products b = (mm*wx)*wy (f32, the reference's order) of the
 * four (cx,cy) corner columns, and the z weights. */
static inline void contrib_cols(const cellpos *c, float mm, float b[4], float wz[2]) {
  const float wx[2] = {1.0f - c->fx, c->fx};
  const float wy[2] = {1.0f - c->fy, c->fy};
  wz[0] = 1.0f - c->fz;
  wz[1] = c->fz;
  for (int a = 0; a < 2; ++a)
    for (int e = 0; e < 2; ++e) b[a * 2 + e] = (mm * wx[a]) * wy[e];
}

/* Fixed-point deposit with the GPU library's quantum: E = exponent(S) - bits,
 * S = sum of m/dx^3 (frexp exponent). Each corner contribution is the exact
 * product b*wz of the f32 partial product b = (m/dx^3*wx)*wy and the z weight,
 * rounded once to the nearest multiple of 2^E (ties to even; the product of two
 * f32 values is exact in f64, so llrint of it rounds exactly), summed in int64,
 * rho = f32(q) * 2^E. Returns E. */
int or_deposit_fixed(const float *x, const float *y, const float *z, const float *m, int64_t n, float dx, int G,
                     int bits, float *rho, int64_t *q) {
  const size_t g3 = (size_t)G * G * G;
  memset(q, 0, g3 * sizeof(int64_t));
  const float inv_vol = inv_vol_of(dx);
  /* exact, order-independent total: terms truncated to multiples of 2^-s,
   * s from the largest term, integer sum (the GPU library's rule) */
  uint32_t maxbits = 0;
  for (int64_t p = 0; p < n; ++p) {
    const float mm = m[p] * inv_vol;
    if (isfinite(mm) && mm > 0.0f) {
      uint32_t b;
      memcpy(&b, &mm, 4);
      if (b > maxbits) maxbits = b;
    }
  }
  int L = 0;
  while ((1LL << L) < n) ++L;
  double S = 0.0;
  if (maxbits) {
    const int emax = (int)((maxbits >> 23) & 0xffu) - 127;
    const int sh = 62 - L - (emax + 1);
    const double scale = ldexp(1.0, sh);
    uint64_t isum = 0;
    for (int64_t p = 0; p < n; ++p) {
      const float mm = m[p] * inv_vol;
      if (isfinite(mm) && mm > 0.0f) isum += (uint64_t)trunc((double)mm * scale);
    }
    S = ldexp((double)isum, -sh);
  }
  int ex = 0;
  if (S > 0.0) frexp(S, &ex);
  int E = ex - bits;
  if (E < -120) E = -120;
  if (E > 120) E = 120;
  const float qscale = ldexpf(1.0f, -E);
  for (int64_t p = 0; p < n; ++p) {
    cellpos c;
    if (!cell_of(x[p], y[p], z[p], dx, G, &c)) continue;
    float b[4], wz[2];
    contrib_cols(&c, m[p] * inv_vol, b, wz);
    for (int t = 0; t < 8; ++t) {
      const int jx = c.ix + (t >> 2), jy = c.iy + ((t >> 1) & 1), jz = c.iz + (t & 1);
      if (jx >= 0 && jx < G && jy >= 0 && jy < G && jz >= 0 && jz < G)
        q[IDX(jx, jy, jz, G)] += (int64_t)llrint((double)b[t >> 1] * (double)wz[t & 1] * (double)qscale);
    }
  }
  const float qinv = ldexpf(1.0f, E);
  for (size_t i = 0; i < g3; ++i) rho[i] = ((float)q[i]) * qinv;
  return E;
}

/* ---- gradient (deposit.py:132-174) --------------------------------------- */
static inline float gcomp(const float *phi, size_t c, size_t s, int idx, int G, float inv_dx, float inv_2dx) {
  if (idx == 0) return -((phi[c + s] - phi[c]) * inv_dx);
  if (idx == G - 1) return -((phi[c] - phi[c - s]) * inv_dx);
  return -((phi[c + s] - phi[c - s]) * inv_2dx);
}

void or_grad(const float *phi, int G, float dx, float *ax, float *ay, float *az) {
  const float inv_dx = 1.0f / dx;
  const float inv_2dx = 1.0f / (2.0f * dx);
  const size_t sG = (size_t)G;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < G; ++i)
    for (int j = 0; j < G; ++j)
      for (int k = 0; k < G; ++k) {
        const size_t c = IDX(i, j, k, G);
        ax[c] = gcomp(phi, c, sG * sG, i, G, inv_dx, inv_2dx);
        ay[c] = gcomp(phi, c, sG, j, G, inv_dx, inv_2dx);
        az[c] = gcomp(phi, c, 1, k, G, inv_dx, inv_2dx);
      }
}

/* ---- gather (deposit.py:85-129) ------------------------------------------ */
void or_gather(const float *x, const float *y, const float *z, int64_t n, const float *axg, const float *ayg,
               const float *azg, float dx, int G, float *ax, float *ay, float *az) {
#pragma omp parallel for schedule(static)
  for (int64_t p = 0; p < n; ++p) {
    float sx = 0.0f, sy = 0.0f, sz = 0.0f;
    cellpos c;
    if (cell_of(x[p], y[p], z[p], dx, G, &c)) {
      const float wx[2] = {1.0f - c.fx, c.fx};
      const float wy[2] = {1.0f - c.fy, c.fy};
      const float wz[2] = {1.0f - c.fz, c.fz};
      for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b)
          for (int d = 0; d < 2; ++d) {
            const int jx = c.ix + a, jy = c.iy + b, jz = c.iz + d;
            if (jx >= 0 && jx < G && jy >= 0 && jy < G && jz >= 0 && jz < G) {
              const float w = (wx[a] * wy[b]) * wz[d];
              const size_t idx = IDX(jx, jy, jz, G);
              sx += w * axg[idx];
              sy += w * ayg[idx];
              sz += w * azg[idx];
            }
          }
    }
    ax[p] = sx;
    ay[p] = sy;
    az[p] = sz;
  }
}

/* ---- kick / drift (integrator.py:27-59) ---------------------------------- */
void or_axpy3(float *u, float *v, float *w, const float *a, const float *b, const float *c, int64_t n, float dt) {
#pragma omp parallel for schedule(static)
  for (int64_t p = 0; p < n; ++p) {
    u[p] += a[p] * dt;
    v[p] += b[p] * dt;
    w[p] += c[p] * dt;
  }
}

/* ---- multigrid (solver/multigrid.py) -------------------------------------- */
typedef struct {
  int G, nlev;
  float dx;
  double grav;
  int n_cycles, nu1, nu2, coarse_sweeps, min_cycles;
  double tol;
  int sizes[32];
  double dxs[32];
  float *phi[32], *rhs[32], *res[32];
  int last_cycles;
} or_mg;

or_mg *or_mg_create(int G, float dx, double grav, int n_cycles, int nu1, int nu2, int coarse_sweeps, double tol,
                    int min_cycles) {
  or_mg *h = (or_mg *)calloc(1, sizeof(or_mg));
  h->G = G;
  h->dx = dx;
  h->grav = grav;
  h->n_cycles = n_cycles;
  h->nu1 = nu1;
  h->nu2 = nu2;
  h->coarse_sweeps = coarse_sweeps;
  h->tol = tol;
  h->min_cycles = min_cycles < 1 ? 1 : min_cycles;
  /* multigrid.py:330-336 */
  int nl = 0;
  h->sizes[nl++] = G;
  while (h->sizes[nl - 1] % 2 == 0 && h->sizes[nl - 1] / 2 >= 3 && nl < 32) {
    h->sizes[nl] = h->sizes[nl - 1] / 2;
    ++nl;
  }
  h->nlev = nl;
  for (int l = 0; l < nl; ++l) {
    h->dxs[l] = (double)dx * (double)(1 << l);
    const size_t n3 = (size_t)h->sizes[l] * h->sizes[l] * h->sizes[l];
    h->phi[l] = (float *)calloc(n3, sizeof(float));
    h->rhs[l] = (float *)calloc(n3, sizeof(float));
    h->res[l] = (float *)calloc(n3, sizeof(float));
  }
  return h;
}

void or_mg_destroy(or_mg *h) {
  if (!h) return;
  for (int l = 0; l < h->nlev; ++l) {
    free(h->phi[l]);
    free(h->rhs[l]);
    free(h->res[l]);
  }
  free(h);
}

int or_mg_levels(const or_mg *h, int *sizes) {
  for (int l = 0; l < h->nlev; ++l) sizes[l] = h->sizes[l];
  return h->nlev;
}

/* multigrid.py:46-59 */
static void gs_rb(float *phi, const float *rhs, int n, float h2, int color) {
#pragma omp parallel for schedule(static)
  for (int i = 1; i < n - 1; ++i)
    for (int j = 1; j < n - 1; ++j)
      for (int k = 1; k < n - 1; ++k) {
        if (((i + j + k) & 1) != color) continue;
        const size_t c = IDX(i, j, k, n);
        const size_t si = (size_t)n * n, sj = (size_t)n;
        phi[c] = (phi[c + si] + phi[c - si] + phi[c + sj] + phi[c - sj] + phi[c + 1] + phi[c - 1] - h2 * rhs[c]) / 6.0f;
      }
}

/* multigrid.py:62-79 */
static void residual(const float *phi, const float *rhs, float *res, int n, float inv_h2) {
  memset(res, 0, (size_t)n * n * n * sizeof(float));
#pragma omp parallel for schedule(static)
  for (int i = 1; i < n - 1; ++i)
    for (int j = 1; j < n - 1; ++j)
      for (int k = 1; k < n - 1; ++k) {
        const size_t c = IDX(i, j, k, n);
        const size_t si = (size_t)n * n, sj = (size_t)n;
        const float lap = (phi[c + si] + phi[c - si] + phi[c + sj] + phi[c - sj] + phi[c + 1] + phi[c - 1] -
                           6.0f * phi[c]) * inv_h2;
        res[c] = rhs[c] - lap;
      }
}

/* multigrid.py:82-97 */
static void restrict_fw(const float *rf, int nf, float *rc, int nc) {
  memset(rc, 0, (size_t)nc * nc * nc * sizeof(float));
#pragma omp parallel for schedule(static)
  for (int J = 1; J < nc - 1; ++J)
    for (int K = 1; K < nc - 1; ++K)
      for (int L = 1; L < nc - 1; ++L) {
        const int fi = 2 * J, fj = 2 * K, fk = 2 * L;
        float acc = 0.0f;
        for (int a = -1; a <= 1; ++a)
          for (int b = -1; b <= 1; ++b)
            for (int c = -1; c <= 1; ++c) {
              const float wa = a == 0 ? 2.0f : 1.0f, wb = b == 0 ? 2.0f : 1.0f, wc = c == 0 ? 2.0f : 1.0f;
              acc += wa * wb * wc * rf[IDX(fi + a, fj + b, fk + c, nf)];
            }
        rc[IDX(J, K, L, nc)] = acc / 64.0f;
      }
}

/* multigrid.py:100-130 */
static void prolong_add(const float *pc, int nc, float *pf, int nf) {
#pragma omp parallel for schedule(static)
  for (int i = 1; i < nf - 1; ++i)
    for (int j = 1; j < nf - 1; ++j)
      for (int k = 1; k < nf - 1; ++k) {
        const int ci = i / 2, cj = j / 2, ck = k / 2;
        const int oi = i & 1, oj = j & 1, ok = k & 1;
        float val = 0.0f;
        for (int di = 0; di < 2; ++di) {
          const float wi = oi == 1 ? 0.5f : (di == 0 ? 1.0f : 0.0f);
          for (int dj = 0; dj < 2; ++dj) {
            const float wj = oj == 1 ? 0.5f : (dj == 0 ? 1.0f : 0.0f);
            for (int dk = 0; dk < 2; ++dk) {
              const float wk = ok == 1 ? 0.5f : (dk == 0 ? 1.0f : 0.0f);
              const float w = wi * wj * wk;
              if (w > 0.0f) val += w * pc[IDX(ci + di, cj + dj, ck + dk, nc)];
            }
          }
        }
        pf[IDX(i, j, k, nf)] += val;
      }
}

static void smooth(or_mg *h, int l, int sweeps) {
  const int n = h->sizes[l];
  const float h2 = (float)(h->dxs[l] * h->dxs[l]);
  for (int s = 0; s < sweeps; ++s) {
    gs_rb(h->phi[l], h->rhs[l], n, h2, 0);
    gs_rb(h->phi[l], h->rhs[l], n, h2, 1);
  }
}

/* multigrid.py:429-440 */
static void vcycle(or_mg *h, int l) {
  if (l == h->nlev - 1) {
    smooth(h, l, h->coarse_sweeps);
    return;
  }
  smooth(h, l, h->nu1);
  const int n = h->sizes[l];
  residual(h->phi[l], h->rhs[l], h->res[l], n, (float)(1.0 / (h->dxs[l] * h->dxs[l])));
  restrict_fw(h->res[l], n, h->rhs[l + 1], h->sizes[l + 1]);
  memset(h->phi[l + 1], 0, (size_t)h->sizes[l + 1] * h->sizes[l + 1] * h->sizes[l + 1] * sizeof(float));
  vcycle(h, l + 1);
  prolong_add(h->phi[l + 1], h->sizes[l + 1], h->phi[l], n);
  smooth(h, l, h->nu2);
}

void or_mg_vcycle(or_mg *h) { vcycle(h, 0); }

/* multigrid.py:133-178: ten raw moments in f64 (serial order) */
void or_moments(const float *rho, int G, float dx, double out[10]) {
  for (int t = 0; t < 10; ++t) out[t] = 0.0;
  const double ddx = (double)dx;
  const double vol = ddx * ddx * ddx;
  for (int i = 0; i < G; ++i)
    for (int j = 0; j < G; ++j)
      for (int k = 0; k < G; ++k) {
        const double m = (double)rho[IDX(i, j, k, G)] * vol;
        const double x = (double)i * ddx, y = (double)j * ddx, z = (double)k * ddx;
        out[0] += m;
        out[1] += m * x;
        out[2] += m * y;
        out[3] += m * z;
        out[4] += m * x * x;
        out[5] += m * y * y;
        out[6] += m * z * z;
        out[7] += m * x * y;
        out[8] += m * x * z;
        out[9] += m * y * z;
      }
}

static double sumsq(const float *a, size_t n) {
  double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
  for (size_t i = 0; i < n; ++i) s += (double)a[i] * (double)a[i];
  return s;
}

/* multigrid.py:261-295 (all f32, parameters rounded to f32 as Taichi does) */
static void set_faces(float *phi, int n, float dx, float g, float mass, float cmx, float cmy, float cmz, float sxx,
                      float syy, float szz, float sxy, float sxz, float syz) {
  const float tr_s = sxx + syy + szz;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j)
      for (int k = 0; k < n; ++k) {
        if (!(i == 0 || i == n - 1 || j == 0 || j == n - 1 || k == 0 || k == n - 1)) continue;
        const float rx = (float)i * dx - cmx, ry = (float)j * dx - cmy, rz = (float)k * dx - cmz;
        const float d2 = rx * rx + ry * ry + rz * rz + 1e-12f;
        const float d = sqrtf(d2);
        const float nx = rx / d, ny = ry / d, nz = rz / d;
        const float nsn = nx * nx * sxx + ny * ny * syy + nz * nz * szz + 2.0f * (nx * ny * sxy + nx * nz * sxz + ny * nz * syz);
        const float quad = 3.0f * nsn - tr_s;
        phi[IDX(i, j, k, n)] = -g * (mass / d + quad / (2.0f * d2 * d));
      }
}

/* multigrid.py:364-389 + 455-487. Returns the number of V-cycles run;
 * out_norms = [||rhs||, ||res|| after the last check]. */
int or_mg_solve(or_mg *h, const float *rho, float *phi, int warm_start, double *out_norms) {
  const int G = h->G;
  const size_t g3 = (size_t)G * G * G;
  double s[10];
  or_moments(rho, G, h->dx, s);
  double total = s[0], cx = 0, cy = 0, cz = 0, sxx = 0, syy = 0, szz = 0, sxy = 0, sxz = 0, syz = 0;
  if (total > 0.0) {
    cx = s[1] / total;
    cy = s[2] / total;
    cz = s[3] / total;
    sxx = s[4] - total * cx * cx;
    syy = s[5] - total * cy * cy;
    szz = s[6] - total * cz * cz;
    sxy = s[7] - total * cx * cy;
    sxz = s[8] - total * cx * cz;
    syz = s[9] - total * cy * cz;
  } else {
    total = 0.0;
  }
  const float factor = (float)(4.0 * M_PI * h->grav);
  for (size_t i = 0; i < g3; ++i) h->rhs[0][i] = factor * rho[i];
  if (warm_start)
    memcpy(h->phi[0], phi, g3 * sizeof(float));
  else
    memset(h->phi[0], 0, g3 * sizeof(float));
  set_faces(h->phi[0], G, h->dx, (float)h->grav, (float)total, (float)cx, (float)cy, (float)cz, (float)sxx,
            (float)syy, (float)szz, (float)sxy, (float)sxz, (float)syz);
  const float inv_h2 = (float)(1.0 / ((double)h->dx * (double)h->dx));
  const double rhs_norm = sqrt(sumsq(h->rhs[0], g3));
  double rn = NAN;
  h->last_cycles = h->n_cycles;
  for (int c = 0; c < h->n_cycles; ++c) {
    vcycle(h, 0);
    if (c + 1 >= h->min_cycles && rhs_norm > 0.0) {
      residual(h->phi[0], h->rhs[0], h->res[0], G, inv_h2);
      rn = sqrt(sumsq(h->res[0], g3));
      if (rn < h->tol * rhs_norm) {
        h->last_cycles = c + 1;
        break;
      }
    }
  }
  memcpy(phi, h->phi[0], g3 * sizeof(float));
  if (out_norms) {
    out_norms[0] = rhs_norm;
    out_norms[1] = rn;
  }
  return h->last_cycles;
}

/* multigrid.py:489-494 */
double or_mg_residual_norm(or_mg *h) {
  const int G = h->G;
  residual(h->phi[0], h->rhs[0], h->res[0], G, (float)(1.0 / ((double)h->dx * (double)h->dx)));
  return sqrt(sumsq(h->res[0], (size_t)G * G * G));
}

/* FP64 residual of an arbitrary potential against rhs = f32(4 pi G) * rho
 * (interior nodes), for checking any solver's output. */
double or_residual64(const float *rho, const double *phi, int G, float dx, double grav, double *rhs_norm) {
  const float factor = (float)(4.0 * M_PI * grav);
  const double inv_h2 = 1.0 / ((double)dx * (double)dx);
  double rr = 0.0, bb = 0.0;
  const size_t si = (size_t)G * G, sj = (size_t)G;
  for (size_t t = 0; t < (size_t)G * G * G; ++t) {
    const double b = (double)(factor * rho[t]);
    bb += b * b;
  }
#pragma omp parallel for reduction(+ : rr) schedule(static)
  for (int i = 1; i < G - 1; ++i)
    for (int j = 1; j < G - 1; ++j)
      for (int k = 1; k < G - 1; ++k) {
        const size_t c = IDX(i, j, k, G);
        const double lap = ((phi[c + si] - phi[c]) + (phi[c - si] - phi[c]) + (phi[c + sj] - phi[c]) +
                            (phi[c - sj] - phi[c]) + (phi[c + 1] - phi[c]) + (phi[c - 1] - phi[c])) * inv_h2;
        const double r = (double)(factor * rho[c]) - lap;
        rr += r * r;
      }
  if (rhs_norm) *rhs_norm = sqrt(bb);
  return sqrt(rr);
}

/* ---- the same multigrid in FP64 (multigrid.py:46-130, 261-295, 429-487) ----
 * The reference algorithm (vertex-centred coarsening, red-black Gauss-Seidel,
 * full weighting, trilinear prolongation, multipole faces) with every array
 * and every operation in double precision, so that the adaptive loop can be
 * driven below the FP32 floor (to 1e-6 and beyond): the CPU baseline of the
 * mixed-precision GPU solve at the same tolerance. */
typedef struct {
  int G, nlev;
  double dx, grav, tol;
  int n_cycles, nu1, nu2, coarse_sweeps, min_cycles;
  int sizes[32];
  double dxs[32];
  double *phi[32], *rhs[32], *res[32];
  int last_cycles;
} or_mg64;

or_mg64 *or_mg64_create(int G, double dx, double grav, int n_cycles, int nu1, int nu2, int coarse_sweeps, double tol,
                        int min_cycles) {
  or_mg64 *h = (or_mg64 *)calloc(1, sizeof(or_mg64));
  h->G = G;
  h->dx = dx;
  h->grav = grav;
  h->n_cycles = n_cycles;
  h->nu1 = nu1;
  h->nu2 = nu2;
  h->coarse_sweeps = coarse_sweeps;
  h->tol = tol;
  h->min_cycles = min_cycles < 1 ? 1 : min_cycles;
  int nl = 0;
  h->sizes[nl++] = G;
  while (h->sizes[nl - 1] % 2 == 0 && h->sizes[nl - 1] / 2 >= 3 && nl < 32) {
    h->sizes[nl] = h->sizes[nl - 1] / 2;
    ++nl;
  }
  h->nlev = nl;
  for (int l = 0; l < nl; ++l) {
    h->dxs[l] = dx * (double)(1 << l);
    const size_t n3 = (size_t)h->sizes[l] * h->sizes[l] * h->sizes[l];
    h->phi[l] = (double *)calloc(n3, sizeof(double));
    h->rhs[l] = (double *)calloc(n3, sizeof(double));
    h->res[l] = (double *)calloc(n3, sizeof(double));
  }
  return h;
}

void or_mg64_destroy(or_mg64 *h) {
  if (!h) return;
  for (int l = 0; l < h->nlev; ++l) {
    free(h->phi[l]);
    free(h->rhs[l]);
    free(h->res[l]);
  }
  free(h);
}

static void gs_rb64(double *phi, const double *rhs, int n, double h2, int color) {
#pragma omp parallel for schedule(static)
  for (int i = 1; i < n - 1; ++i)
    for (int j = 1; j < n - 1; ++j)
      for (int k = 1 + ((i + j + 1 + color) & 1); k < n - 1; k += 2) {
        const size_t c = IDX(i, j, k, n);
        const size_t si = (size_t)n * n, sj = (size_t)n;
        phi[c] = (phi[c + si] + phi[c - si] + phi[c + sj] + phi[c - sj] + phi[c + 1] + phi[c - 1] - h2 * rhs[c]) / 6.0;
      }
}

static void residual64(const double *phi, const double *rhs, double *res, int n, double inv_h2) {
  memset(res, 0, (size_t)n * n * n * sizeof(double));
#pragma omp parallel for schedule(static)
  for (int i = 1; i < n - 1; ++i)
    for (int j = 1; j < n - 1; ++j)
      for (int k = 1; k < n - 1; ++k) {
        const size_t c = IDX(i, j, k, n);
        const size_t si = (size_t)n * n, sj = (size_t)n;
        const double lap =
            (phi[c + si] + phi[c - si] + phi[c + sj] + phi[c - sj] + phi[c + 1] + phi[c - 1] - 6.0 * phi[c]) * inv_h2;
        res[c] = rhs[c] - lap;
      }
}

static void restrict_fw64(const double *rf, int nf, double *rc, int nc) {
  memset(rc, 0, (size_t)nc * nc * nc * sizeof(double));
#pragma omp parallel for schedule(static)
  for (int J = 1; J < nc - 1; ++J)
    for (int K = 1; K < nc - 1; ++K)
      for (int L = 1; L < nc - 1; ++L) {
        double acc = 0.0;
        for (int a = -1; a <= 1; ++a)
          for (int b = -1; b <= 1; ++b)
            for (int c = -1; c <= 1; ++c)
              acc += (a ? 1.0 : 2.0) * (b ? 1.0 : 2.0) * (c ? 1.0 : 2.0) * rf[IDX(2 * J + a, 2 * K + b, 2 * L + c, nf)];
        rc[IDX(J, K, L, nc)] = acc / 64.0;
      }
}

static void prolong_add64(const double *pc, int nc, double *pf, int nf) {
#pragma omp parallel for schedule(static)
  for (int i = 1; i < nf - 1; ++i)
    for (int j = 1; j < nf - 1; ++j)
      for (int k = 1; k < nf - 1; ++k) {
        const int ci = i / 2, cj = j / 2, ck = k / 2, oi = i & 1, oj = j & 1, ok = k & 1;
        double val = 0.0;
        for (int di = 0; di <= oi; ++di)
          for (int dj = 0; dj <= oj; ++dj)
            for (int dk = 0; dk <= ok; ++dk)
              val += (oi ? 0.5 : 1.0) * (oj ? 0.5 : 1.0) * (ok ? 0.5 : 1.0) * pc[IDX(ci + di, cj + dj, ck + dk, nc)];
        pf[IDX(i, j, k, nf)] += val;
      }
}

static void vcycle64(or_mg64 *h, int l) {
  const int n = h->sizes[l];
  const double h2 = h->dxs[l] * h->dxs[l];
  const int pre = l == h->nlev - 1 ? h->coarse_sweeps : h->nu1;
  for (int s = 0; s < pre; ++s) {
    gs_rb64(h->phi[l], h->rhs[l], n, h2, 0);
    gs_rb64(h->phi[l], h->rhs[l], n, h2, 1);
  }
  if (l == h->nlev - 1) return;
  residual64(h->phi[l], h->rhs[l], h->res[l], n, 1.0 / h2);
  restrict_fw64(h->res[l], n, h->rhs[l + 1], h->sizes[l + 1]);
  memset(h->phi[l + 1], 0, (size_t)h->sizes[l + 1] * h->sizes[l + 1] * h->sizes[l + 1] * sizeof(double));
  vcycle64(h, l + 1);
  prolong_add64(h->phi[l + 1], h->sizes[l + 1], h->phi[l], n);
  for (int s = 0; s < h->nu2; ++s) {
    gs_rb64(h->phi[l], h->rhs[l], n, h2, 0);
    gs_rb64(h->phi[l], h->rhs[l], n, h2, 1);
  }
}

static double sumsq64(const double *a, size_t n) {
  double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
  for (size_t i = 0; i < n; ++i) s += a[i] * a[i];
  return s;
}

/* rho f32 (the deposited density), phi f64 in/out. Returns the V-cycles run;
 * out_norms = [||rhs||, ||res||]. */
int or_mg64_solve(or_mg64 *h, const float *rho, double *phi, int warm_start, double *out_norms) {
  const int G = h->G;
  const size_t g3 = (size_t)G * G * G;
  double s[10];
  or_moments(rho, G, (float)h->dx, s);
  double M = s[0], cx = 0, cy = 0, cz = 0, S[6] = {0, 0, 0, 0, 0, 0};
  if (M > 0.0) {
    cx = s[1] / M; cy = s[2] / M; cz = s[3] / M;
    S[0] = s[4] - M * cx * cx; S[1] = s[5] - M * cy * cy; S[2] = s[6] - M * cz * cz;
    S[3] = s[7] - M * cx * cy; S[4] = s[8] - M * cx * cz; S[5] = s[9] - M * cy * cz;
  }
  const double fpg = 4.0 * M_PI * h->grav;
  for (size_t i = 0; i < g3; ++i) h->rhs[0][i] = fpg * (double)rho[i];
  if (warm_start)
    memcpy(h->phi[0], phi, g3 * sizeof(double));
  else
    memset(h->phi[0], 0, g3 * sizeof(double));
  const double trS = S[0] + S[1] + S[2];
#pragma omp parallel for schedule(static)
  for (int i = 0; i < G; ++i)
    for (int j = 0; j < G; ++j)
      for (int k = 0; k < G; ++k) {
        if (!(i == 0 || i == G - 1 || j == 0 || j == G - 1 || k == 0 || k == G - 1)) continue;
        double v = 0.0;
        if (M > 0.0) {
          const double rx = i * h->dx - cx, ry = j * h->dx - cy, rz = k * h->dx - cz;
          const double d2 = rx * rx + ry * ry + rz * rz + 1e-12, d = sqrt(d2);
          const double nx = rx / d, ny = ry / d, nz = rz / d;
          const double nsn = nx * nx * S[0] + ny * ny * S[1] + nz * nz * S[2] +
                             2.0 * (nx * ny * S[3] + nx * nz * S[4] + ny * nz * S[5]);
          v = -h->grav * (M / d + (3.0 * nsn - trS) / (2.0 * d2 * d));
        }
        h->phi[0][IDX(i, j, k, G)] = v;
      }
  const double inv_h2 = 1.0 / (h->dx * h->dx);
  const double rhs_norm = sqrt(sumsq64(h->rhs[0], g3));
  double rn = NAN;
  h->last_cycles = h->n_cycles;
  for (int c = 0; c < h->n_cycles; ++c) {
    vcycle64(h, 0);
    if (c + 1 >= h->min_cycles && rhs_norm > 0.0) {
      residual64(h->phi[0], h->rhs[0], h->res[0], G, inv_h2);
      rn = sqrt(sumsq64(h->res[0], g3));
      if (rn < h->tol * rhs_norm) {
        h->last_cycles = c + 1;
        break;
      }
    }
  }
  memcpy(phi, h->phi[0], g3 * sizeof(double));
  if (out_norms) {
    out_norms[0] = rhs_norm;
    out_norms[1] = rn;
  }
  return h->last_cycles;
}
