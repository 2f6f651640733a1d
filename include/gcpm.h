/*
 * gcpm.h — C ABI of the GB300 particle-mesh (PM) force chain.
 *
 * This is the drop-in boundary for the reference's PM hot path
 * (pouyalj/Galaxy-Collision-with-CUDA-FFT, package src/galaxy_collision):
 * CIC deposit -> open-boundary multigrid Poisson solve -> -grad(phi) -> CIC
 * gather -> KDK kick/drift. Every entry point takes plain device pointers,
 * element counts and an opaque context; no torch or CUDA types appear in the
 * signatures (streams are passed as `void*` holding a cudaStream_t).
 *
 * Conventions shared with the reference (src/galaxy_collision/deposit.py:16-37):
 *   - node-centred grid: node (i,j,k) sits at physical (i,j,k)*dx, the G nodes
 *     per axis span [0, (G-1)*dx];
 *   - grids are C-order [i][j][k] with k fastest (Taichi field to_numpy order);
 *   - particles are SoA f32 arrays (src/galaxy_collision/data.py:84-113);
 *   - out-of-box CIC weight is dropped, never wrapped (deposit.py:33-37).
 *
 * Error convention: every call returns GC_OK (0) or a negative status; the
 * message of the last failure is returned by gc_last_error(ctx) (ctx may be
 * NULL for failures of gc_ctx_create). Calls are stream-ordered and
 * asynchronous unless their documentation says they return host scalars.
 * No entry point allocates caller-visible memory or frees caller memory.
 */
#ifndef GCPM_H
#define GCPM_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GC_ABI_VERSION 1

enum gc_status_code {
  GC_OK = 0,
  GC_ERR_ARG = -1,           /* bad argument: maps to ValueError, as the reference raises */
  GC_ERR_CUDA = -2,          /* a CUDA runtime call failed */
  GC_ERR_TIMEOUT = -3,       /* a bounded device wait gave up */
  GC_ERR_NOT_CONVERGED = -4, /* reserved: the solvers report convergence in their stats */
  GC_ERR_NONFINITE = -5,     /* non-finite particle or grid values were seen */
  GC_ERR_STATE = -6          /* call made in the wrong state (e.g. step before prime) */
};

/* Device status bits, OR-ed by kernels into a per-context word (gc_status). */
#define GC_FLAG_NONFINITE_POS 0x1u  /* a particle position was NaN/Inf: it deposited nothing */
#define GC_FLAG_NONFINITE_RHO 0x2u  /* the density handed to the solver had NaN/Inf */
#define GC_FLAG_BAD_PID 0x4u        /* gc_pm_export met a pid outside [0, n): that particle was skipped */
#define GC_FLAG_IC_REJECT 0x8u      /* a device IC rejection loop reached its attempt limit */
#define GC_FLAG_TIMEOUT 0x10u       /* a bounded wait inside a kernel ran out; that kernel stopped early */

/* gc_mg_params.flags: run exactly max_cycles V-cycles without reading the
 * residual norm on the host (it is left on the device; gc_pm_last_residual
 * reads it). The engine's step then makes no host synchronisation, so it can be
 * captured in a CUDA graph. Stats report converged = -1 and NaN norms. */
#define GC_MG_FIXED_CYCLES 0x2
/* gc_mg_params.flags: the plain FP32 method. The potential is a single f32
 * array (the lo part is ignored and left alone), the residual is formed in f32
 * with the reference's left-to-right neighbour sum (multigrid.py:62-79) and the
 * corrections are added in f32, so the residual stalls at the FP32 floor (about
 * 1e-5 to 1e-4 of ||rhs||, as the reference's does) and the solve then runs to
 * max_cycles. The comparison baseline for the mixed-precision default. */
#define GC_MG_PLAIN_F32 0x4
/* gc_mg_params.flags: validation path. The finest level's correction and
 * residual are kept in natural (interleaved) layout and relaxed by the generic
 * level kernels instead of the colour-split half-sweeps; the potential is
 * identical bit for bit, it just moves more bytes. */
#define GC_MG_NATURAL_LAYOUT 0x8
/* gc_mg_params.flags (gc_mg_solve): the Dirichlet face values are the boundary
 * nodes of phi as passed, instead of the multipole faces from the moments of
 * rho (multigrid.py:261-295); phi's interior is the initial guess when
 * warm_start, else zero. With faces from a free-space (lattice Green's function)
 * evaluation this is the isolated-boundary solve of James's method. */
#define GC_MG_FACES_GIVEN 0x10
/* gc_mg_params.flags: the coarse levels by one launch per phase instead of the
 * two persistent cooperative launches: slower for one solve alone, but the
 * launches of many small solves running at once on one GPU (an ensemble of
 * runs on separate streams) can interleave. Same potentials bit for bit. */
#define GC_MG_PHASE_LAUNCHES 0x20
/* gc_mg_params.flags: every level below the finest relaxes with one red-black
 * sweep before restriction and one after prolongation; the finest keeps
 * pre_sweeps / post_sweeps. Fewer barrier-separated phases on the latency-bound
 * coarse levels for a slightly weaker V-cycle; the stopping rule is unchanged. */
#define GC_MG_COARSE_ONE_SWEEP 0x40

typedef struct gc_ctx gc_ctx;

/* Multigrid controls. Defaults follow MultigridPoissonSolver.__init__
 * (src/galaxy_collision/solver/multigrid.py:301-312). */
typedef struct gc_mg_params {
  int pre_sweeps;     /* nu1 red-black sweeps before restriction (reference: 2) */
  int post_sweeps;    /* nu2 sweeps after prolongation (reference: 2) */
  int coarse_sweeps;  /* FP64 Gauss-Seidel sweeps on the coarsest level (reference: 40) */
  int max_cycles;     /* V-cycle cap (reference n_cycles: 20) */
  int min_cycles;     /* never fewer V-cycles than this (reference: 1) */
  int flags;          /* GC_MG_* bits; 0 = default */
  double tol;         /* stop when ||r||_2 < tol * ||4 pi G rho||_2 (reference: 1e-3) */
} gc_mg_params;

typedef struct gc_mg_stats {
  int cycles;         /* V-cycles run by the last solve (reference last_cycles) */
  int converged;      /* 1 if ||r|| < tol*||rhs|| was reached within max_cycles */
  double rhs_norm;    /* ||4 pi G rho||_2 over all G^3 nodes */
  double res_norm;    /* ||rhs - L phi||_2 over the interior after the last cycle */
} gc_mg_stats;

/* Particle set for the fused engine: SoA device arrays of length n. */
typedef struct gc_particles {
  float *x, *y, *z;      /* positions, grid-origin coordinates (node i at i*dx) */
  float *vx, *vy, *vz;   /* velocities */
  float *m;              /* masses */
  int32_t *gid;          /* galaxy id (carried through sorts; may be NULL) */
  int32_t *pid;          /* original particle index (carried through sorts; may be NULL) */
  int64_t n;
} gc_particles;

/* Modes of gc_pm_step (the staggered KDK state machine of the fused engine). */
enum gc_step_mode {
  GC_STEP_PRIME = 0, /* a_0 = F(x_0); v += a h; x += v dt            (state -> open)   */
  GC_STEP_ADVANCE = 1,/* a_n = F(x_n); v += a h; v += a h; x += v dt (open -> open)    */
  GC_STEP_CLOSE = 2  /* a_n = F(x_n); v += a h                      (open -> synced)  */
};

typedef struct gc_step_params {
  float dt;          /* full step; the kicks use dt/2 as in kdk_step */
  int mode;          /* gc_step_mode */
  int warm_start;    /* reuse the previous potential (hi+lo) as the initial guess */
  int diagnostics;   /* 1: accumulate the particle diagnostics (as gc_diag_particles) at the synchronised time */
  gc_mg_params mg;
  int fixed_point_bits; /* deposit quantum = 2^-bits of the total mass; 24 <= bits <= 62 - ceil(log2 G) */
  int flags;         /* GC_STEP_* bits */
} gc_step_params;

/* gc_step_params.flags: form g = -grad(phi) once per step as a float4 node grid
 * and gather it with one vector load per corner (same arithmetic as forming it
 * on the fly from phi; costs a G^3 float4 buffer held by the context). */
#define GC_STEP_GRAD_GRID 0x1
/* gc_step_params.flags: split a step in two calls. SOLVE_ONLY runs the deposit
 * and the solve and stops; PUSH_ONLY (the next call, same mode and dt) runs the
 * particle pass on that potential. In between, gc_pm_residual_host reads the
 * residual of a fixed-cycle solve and gc_pm_refine adds V-cycles, so batched
 * fixed-cycle solves can still meet the tolerance. */
#define GC_STEP_SOLVE_ONLY 0x2
#define GC_STEP_PUSH_ONLY 0x4
/* gc_step_params.flags: the particle pass also deposits the drifted positions
 * (the next step's density) into the context's fixed-point grid, and the next
 * step given this flag skips its own deposit. PRIME always deposits; a CLOSE,
 * gc_pm_import or gc_pm_import_sorted drops the pending deposit. Same density,
 * bit for bit, one pass over the particles fewer. */
#define GC_STEP_DEPOSIT_NEXT 0x8

typedef struct gc_step_stats {
  gc_mg_stats mg;
  double diag[11];   /* M, KE, Px,Py,Pz, Lx,Ly,Lz, Sum m x, Sum m y, Sum m z (diagnostics_device.py:32-38) */
  double grid_pe_raw;/* Sum rho*phi over the grid (diagnostics_device.py:78-88) */
} gc_step_stats;

/* ---- context ------------------------------------------------------------ */

/* Create a context for a G^3 grid (2 <= G <= 1024) of node spacing dx and gravitational
 * constant grav. Allocates the multigrid hierarchy, the int64 mass grid and
 * reduction scratch on the current device. Replaces the per-solver state of
 * MultigridPoissonSolver.__init__ (solver/multigrid.py:301-360) and the grid
 * scratch of GridState (data.py:116-138). */
int gc_ctx_create(gc_ctx **out, int grid_size, double dx, double grav_constant);
int gc_ctx_destroy(gc_ctx *ctx);
/* Message of the last failure on ctx (or of the last gc_ctx_create when ctx is NULL). */
const char *gc_last_error(const gc_ctx *ctx);
/* Stream (a cudaStream_t passed as void*) used by all later calls on ctx. NULL = legacy default. */
int gc_set_stream(gc_ctx *ctx, void *stream);
/* Read (and optionally clear) the device status word; synchronises the stream. */
int gc_status(gc_ctx *ctx, uint32_t *flags_out, int clear);
int gc_abi_version(void);
int gc_num_levels(const gc_ctx *ctx);
/* Level geometry of the multigrid hierarchy: nodes per axis and last interior index. */
int gc_level_info(const gc_ctx *ctx, int level, int *n_nodes, int *last_interior, double *far_face);

/* ---- particle <-> grid operators (reference deposit.py / integrator.py) -- */

/* Zero rho, then CIC-deposit m*w/dx^3 onto the G^3 nodes, dropping out-of-box
 * weight. Accumulates in int64 fixed point (quantum 2^-fixed_point_bits of the
 * total), so rho is bit-identical run to run whatever the particle order.
 * fixed_point_bits must be in [24, 62 - ceil(log2 G)] (GC_ERR_ARG otherwise).
 * Replaces _deposit_cic / deposit_density (deposit.py:47-82, 177-182). */
int gc_deposit_cic(gc_ctx *ctx, const float *x, const float *y, const float *z, const float *m,
                   int64_t n, int fixed_point_bits, float *rho);

/* Allocation-free variant of gc_deposit_cic, with no counterpart in the
 * reference. For callers that cannot allocate device memory where they need a
 * density (a memory pool that already owns the device, a loop that must not take
 * cudaMalloc's device-wide synchronisation, or no context object to own
 * scratch): it needs no gc_ctx and calls no allocating routine. Its int64 mass
 * grid and reduction scratch are one file-scope device array (about 2.2 MiB per
 * GPU that loads the library, held until exit), so grid_size is limited to
 * [2, 64]; larger grids are rejected with GC_ERR_ARG. The first call on each
 * device looks the array's address up (make it before any stream capture);
 * every call clears the part it needs. All calls share the array: calls whose
 * work overlaps on the GPU race and must be serialised by the caller. On failure
 * the message is gc_last_error(NULL). The device address of the array is
 * cached per device ordinal: after cudaDeviceReset do not call it again on that
 * device in the same process. flags (device, may be NULL): a NaN/Inf position
 * deposits nothing and GC_FLAG_NONFINITE_POS is OR-ed into *flags (the caller
 * clears it); without flags that status is not reported. Same result, bit for
 * bit, as gc_deposit_cic with the same fixed_point_bits. */
int gc_deposit_cic_noalloc(const float *x, const float *y, const float *z, const float *m, int64_t n,
                           int grid_size, double dx, int fixed_point_bits, float *rho, uint32_t *flags,
                           void *stream);

/* g = -grad(phi) at every node: central differences inside, one-sided on faces.
 * Replaces _potential_to_accel / potential_to_accel (deposit.py:132-174, 204-207). */
int gc_potential_to_accel(gc_ctx *ctx, const float *phi, float *ax, float *ay, float *az);

/* Trilinear gather of the node acceleration field to particles; out-of-box
 * nodes contribute zero. Replaces _gather_accel / gather_acceleration
 * (deposit.py:85-129, 185-201). */
int gc_gather_accel(gc_ctx *ctx, const float *x, const float *y, const float *z, int64_t n,
                    const float *ax_g, const float *ay_g, const float *az_g,
                    float *acc_x, float *acc_y, float *acc_z);

/* v += a*dt. Replaces integrator.kick (integrator.py:27-41). */
int gc_kick(gc_ctx *ctx, float *vx, float *vy, float *vz, const float *ax, const float *ay,
            const float *az, int64_t n, float dt);
/* x += v*dt. Replaces integrator.drift (integrator.py:44-59). */
int gc_drift(gc_ctx *ctx, float *px, float *py, float *pz, const float *vx, const float *vy,
             const float *vz, int64_t n, float dt);

/* Cell key of each particle from the reference's cell index ix=floor(x/dx)
 * (deposit.py:62-67, f32 IEEE division and floor):
 *   key = ((ix+1)*(G+1) + (iy+1))*(G+1) + (iz+1)   for -1 <= ix,iy,iz <= G-1,
 *   key = (G+1)^3 (sentinel) for particles that deposit nothing or are non-finite. */
int gc_cell_keys(gc_ctx *ctx, const float *x, const float *y, const float *z, int64_t n,
                 uint32_t *keys);
/* Stable LSD radix sort of the keys: sorted_keys (may be NULL) and the
 * permutation perm (sorted position -> original index). Equal keys keep their
 * original order, so the permutation is unique. No reference counterpart: it
 * is the cell sort the reference benchmarked as a deposit variant
 * (docs/performance.md:74-82), built here as the locality step of the deposit. */
int gc_sort_keys(gc_ctx *ctx, const uint32_t *keys, int64_t n, uint32_t *sorted_keys,
                 uint32_t *perm);

/* ---- Poisson solve (reference solver/multigrid.py) ---------------------- */

/* Default parameters of MultigridPoissonSolver (solver/multigrid.py:301-312). */
void gc_mg_default_params(gc_mg_params *p);

/* Solve laplacian(phi) = 4 pi G rho with the reference's open boundary:
 * Dirichlet faces from the monopole+quadrupole of rho about its centre of mass
 * (evaluated in FP64), then adaptive V-cycles until ||r|| < tol*||rhs||.
 * Reads rho, overwrites phi; with warm_start the current phi is the initial
 * guess. The finest level relaxes a double-float (hi+lo FP32 pair) potential so
 * the residual can go below the FP32 floor; coarse levels relax FP32
 * corrections; the coarsest level is solved in FP64. Synchronises the stream to
 * read the residual norms. Replaces MultigridPoissonSolver.solve
 * (solver/multigrid.py:455-487). stats may be NULL. */
int gc_mg_solve(gc_ctx *ctx, const float *rho, float *phi, int warm_start,
                const gc_mg_params *params, gc_mg_stats *stats);

/* FP64 L2 norm of the finest residual rhs - L(phi) of the last solve, phi taken
 * as the double-float pair (or as phi_f32 when it is non-NULL). Returns the norm
 * in the reference's units. Replaces MultigridPoissonSolver.residual_norm
 * (solver/multigrid.py:489-494). Synchronises. */
int gc_mg_residual_norm(gc_ctx *ctx, const float *phi_f32, double *out);

/* The ten raw mass moments [M, Smx, Smy, Smz, Smx2, Smy2, Smz2, Smxy, Smxz, Smyz]
 * of rho (m = rho dx^3 at node (i,j,k)dx), FP64. Replaces _accumulate_moments
 * (solver/multigrid.py:133-178). Synchronises. */
int gc_moments(gc_ctx *ctx, const float *rho, double out[10]);

/* ---- diagnostics (reference diagnostics_device.py) ---------------------- */

/* Sums [M, KE, P(3), L about the origin (3), Sum m r (3)] returned as FP64: each
 * thread forms its particles' products exactly or to ~2^-46 and sums them in
 * double-float (FP32 hi + lo), the threads' totals are added in FP64 (relative
 * error ~1e-14 of the sum of magnitudes).
 * Replaces _reduce_particle_scalars (diagnostics_device.py:42-74). Synchronises. */
int gc_diag_particles(gc_ctx *ctx, const float *x, const float *y, const float *z,
                      const float *vx, const float *vy, const float *vz, const float *m,
                      int64_t n, double out[11]);
/* Raw Sum rho*phi in FP64. Replaces _reduce_grid_pe (diagnostics_device.py:78-88). Synchronises. */
int gc_diag_grid_pe(gc_ctx *ctx, const float *rho, const float *phi, double *out);
/* Mass-weighted histogram of radius about (cx,cy,cz), last bin catch-all, FP64
 * (written to a device array of nbins doubles). Replaces _radial_mass_histogram
 * (diagnostics_device.py:153-185). */
int gc_radial_histogram(gc_ctx *ctx, const float *x, const float *y, const float *z,
                        const float *m, int64_t n, double cx, double cy, double cz,
                        double inv_binw, int nbins, double *hist);

/* Nearest-bin 2-D mass histogram of the particles over two in-plane axes
 * (img[ia*bins + ib], ia = floor((a - lo_a)/binw_a) in f32; out-of-range mass
 * dropped), the device projection behind movie frames and the 2-D view.
 * Replaces viz/project.py _project / scatter_density (viz/project.py:26-70). */
int gc_project_ngp(gc_ctx *ctx, const float *pa, const float *pb, const float *m, int64_t n, double lo_a,
                   double lo_b, double binw_a, double binw_b, int bins, float *img);

/* ---- initial conditions on the device (the reference samples on the host:
 * _sample_plummer / _sample_plummer_q, ic.py:296-384, and _sample_disk /
 * build_ic, ic.py:145-285; these follow the benchmark configurations' spec
 * with counter-based random numbers, so particle i depends only on (seed, i)) */

/* out[4i..4i+3]: the four uniforms in (0, 1) of Philox4x32-10 with counter
 * (i, 0, stream) and key seed (24-bit resolution, centred in their bins). */
int gc_rng_uniform(gc_ctx *ctx, uint64_t seed, uint32_t stream, int64_t n, float *out);
/* n-particle Plummer sphere of mass `mass`, scale a, truncated at rmax*a;
 * speeds from the isotropic distribution function (rejection sampling).
 * pos, vel: n x 3 f32; m: n f32 (mass/n); gid: n (0). */
int gc_ic_plummer(gc_ctx *ctx, int64_t n, uint64_t seed, double mass, double a, double rmax, double grav, float *pos,
                  float *vel, float *m, int32_t *gid);
/* One galaxy of the two-disk collision: n_disk particles of an exponential
 * sech^2 disk (scale rd, cut at 5 rd, height 0.1 rd) plus its central point mass
 * (1 % of m_disk) as particle n_disk, circular speeds from the enclosed mass
 * (softened by soft) with 10 % dispersion, inclined about x by incline_deg,
 * shifted by off and boosted by bulk. Writes n_disk + 1 particles (gid = galaxy). */
int gc_ic_disk(gc_ctx *ctx, int64_t n_disk, uint64_t seed, int galaxy, double m_disk, double rd, double grav,
               double soft, double incline_deg, const double off[3], const double bulk[3], float *pos, float *vel,
               float *m, int32_t *gid);

/* ---- headless views (viz/viewer.py; the GGUI window and scene are replaced by
 * device buffers) ------------------------------------------------------------ */

/* *out = max(0, max of a[0..n)) (device scalar; _max_field / _max_grid3,
 * viewer.py:68-73, 98-101). */
int gc_max_f32(gc_ctx *ctx, const float *a, int64_t n, float *out);
/* rgb[3i..3i+2] = lut[idx], idx = int(clamp01((ln img[i] - log_vmin) * inv_logspan)
 * * 255 + 0.5) (0 where img <= 0); lut is 256 x 3 f32 (_colormap_log,
 * viewer.py:76-93). */
int gc_colormap_log(gc_ctx *ctx, const float *img, int64_t n, const float *lut, float log_vmin, float inv_logspan,
                    float *rgb);
/* out[3i+c] = pos_c[i*stride] * inv_box - 0.5 for i < m (_pack_positions, viewer.py:50-65). */
int gc_pack_positions(gc_ctx *ctx, const float *x, const float *y, const float *z, int64_t stride, float inv_box,
                      int64_t m, float *out);
/* col[3i..] = lut colour of rho at the nearest node of particle i*stride
 * (clamp(int(x * inv_dx + 0.5)) per axis), as gc_colormap_log (_density_color,
 * viewer.py:104-121). */
int gc_density_color(gc_ctx *ctx, const float *x, const float *y, const float *z, const float *rho, int grid,
                     int64_t stride, int64_t m, float inv_dx, const float *lut, float log_vmin, float inv_logspan,
                     float *col);
/* Draw m points (unit-cube coordinates pos[3i..], colours col[3i..] in [0,1]) as
 * flat discs of radius_px pixels into rgba (width x height x 4, row 0 at the
 * top), nearest point per pixel (ties to the lower index), bg elsewhere; the 3-D
 * view's scene.particles (viewer.py:258-272) without a graphics API. view_proj
 * is a row-major 4 x 4 matrix to clip space; points with w <= 0 or depth
 * outside [0, 1] are skipped. zbuf is width x height u64 scratch. */
int gc_splat_points(gc_ctx *ctx, const float *pos, const float *col, int64_t m, const float view_proj[16], int width,
                    int height, float radius_px, const float bg[3], unsigned long long *zbuf, unsigned char *rgba);

/* ---- fused engine (callers: bench.py:145-152, sim.py:320-325) ------------ */

/* Stable-sort the particles by cell key and write the permuted set to out
 * (every non-NULL array of in is permuted into the matching array of out). */
int gc_pm_sort(gc_ctx *ctx, const gc_particles *in, const gc_particles *out);

/* gc_pm_sort by the cells of the positions predicted tau ahead, x + v*tau (f32,
 * rounded per operation; the current cell where the predicted position
 * deposits nothing). With tau = half the time to the next sort the deposit and
 * gather passes see the particles drift from their sorted cells by half as
 * much. tau = 0 is gc_pm_sort; tau != 0 needs the velocities. */
int gc_pm_sort_ahead(gc_ctx *ctx, const gc_particles *in, const gc_particles *out, float tau);

/* Allocate the sort scratch of the context for n particles now (keys, values,
 * digit histograms), so that the first gc_pm_sort allocates nothing. Optional. */
int gc_pm_reserve(gc_ctx *ctx, int64_t n);

/* Fill the engine's particle arrays from the reference's interleaved layout:
 * pos and vel are N x 3 f32 in physical coordinates, as ParticleState holds them
 * after from_numpy (data.py:84-113, ic.py:386-405); m is N f32; gid may be NULL
 * (zeros). Writes out->x = f32((double)pos[3i] - origin[0]) (grid-origin
 * coordinates), the velocities and masses as given, out->pid = i. All pointers
 * are device pointers; stream-ordered, no synchronisation. */
int gc_pm_import(gc_ctx *ctx, const float *pos, const float *vel, const float *m, const int32_t *gid,
                 const double origin[3], const gc_particles *out);

/* gc_pm_import followed by gc_pm_sort in one: the cell keys are computed from
 * the interleaved positions and the particles are gathered from the interleaved
 * arrays straight into cell order (out->pid = original index). The result is
 * identical to gc_pm_import + gc_pm_sort. */
int gc_pm_import_sorted(gc_ctx *ctx, const float *pos, const float *vel, const float *m, const int32_t *gid,
                        const double origin[3], const gc_particles *out);
/* gc_pm_import_sorted in two phases, so that the copies of vel, m and gid can
 * still be in flight (on another stream) while the positions are keyed and
 * sorted: gc_pm_import_order reads only pos and keeps the permutation in the
 * context; gc_pm_import_gather (n must match; no other sort in between) then
 * gathers the arrays into cell order. Any of pos, vel, m, gid may be NULL, so
 * that each array can be gathered as soon as its copy has landed: pos writes
 * out->x, y, z and out->pid, vel out->vx, vy, vz, m out->m, gid out->gid (zeros
 * when gid is NULL and pos is given). The permutation stays valid for further
 * gathers until the next call on this context that sorts (gc_pm_import_order,
 * gc_pm_import_sorted, gc_pm_sort, gc_sort_keys) or grows its particle scratch
 * (gc_pm_reserve). */
int gc_pm_import_order(gc_ctx *ctx, const float *pos, const double origin[3], int64_t n);
int gc_pm_import_gather(gc_ctx *ctx, const float *pos, const float *vel, const float *m, const int32_t *gid,
                        const double origin[3], const gc_particles *out);

/* The inverse, in the original particle order: for every i, with q = p->pid[i],
 * pos[3q+c] = f32((double)x_c[i] + origin[c]), vel[3q+c] = v_c[i], m_out[q],
 * gid_out[q] (each output may be NULL; p->pid is required). Replaces
 * ParticleState.to_numpy (data.py:84-113) on the engine's sorted state. A pid
 * outside [0, n) is skipped and raises GC_FLAG_BAD_PID. Device pointers;
 * stream-ordered. */
int gc_pm_export(gc_ctx *ctx, const gc_particles *p, const double origin[3], float *pos, float *vel, float *m_out,
                 int32_t *gid_out);
/* gc_pm_export in two phases, written in the original order (coalesced
 * stores) so that finished ranges can go to the host while later ones are
 * written: gc_pm_export_order inverts p->pid into the context's scratch
 * (a pid outside [0, n) raises GC_FLAG_BAD_PID); gc_pm_export_range then
 * writes the outputs of original indices [q0, q1) exactly as gc_pm_export does
 * (outputs are whole arrays indexed by the original index; an index that no
 * particle claims is left untouched and raises GC_FLAG_BAD_PID). The ranks stay
 * valid until the next call on this context that sorts or grows its particle
 * scratch, or the next gc_pm_import_order; gc_pm_export_range returns
 * GC_ERR_ARG for a particle set whose count or pid array differs from the one
 * the ranks were made from (a pid array rewritten in place in between is not
 * detected). */
int gc_pm_export_order(gc_ctx *ctx, const gc_particles *p);
int gc_pm_export_range(gc_ctx *ctx, const gc_particles *p, const double origin[3], float *pos, float *vel,
                       float *m_out, int32_t *gid_out, int64_t q0, int64_t q1);

/* One force evaluation of the fused chain plus the kicks/drift of the mode:
 * int64 fixed-point deposit, moments and 4 pi G h^2 rho in one pass, FP64
 * boundary faces, adaptive multigrid to params->mg.tol, then one particle pass
 * that gathers -grad(phi) on the fly and applies the kicks and drift.
 * KDK arithmetic is that of kdk_step (integrator.py:100-131). Synchronises to
 * fill stats (may be NULL). */
int gc_pm_step(gc_ctx *ctx, const gc_particles *p, const gc_step_params *sp, gc_step_stats *st);

/* Device pointer of the current finest-level potential (f32 hi part, G^3). */
const float *gc_pm_potential(const gc_ctx *ctx);
/* Stream-ordered copy of the current finest-level potential into phi (G^3 f32). */
int gc_pm_copy_potential(gc_ctx *ctx, float *phi);
/* Relative residual ||r||/||4 pi G rho|| of the engine's last solve (synchronises). */
int gc_pm_last_residual(gc_ctx *ctx, double *rel);
/* Same, for a fixed-cycle solve, from the pinned host copy that solve enqueued:
 * no copy and no synchronisation (the caller has synchronised the stream). */
int gc_pm_residual_host(const gc_ctx *ctx, double *rel);
/* Between a SOLVE_ONLY and a PUSH_ONLY step: more V-cycles on the current
 * potential until ||r|| < tol ||4 pi G rho|| (at least one); *cycles gets how many. */
int gc_pm_refine(gc_ctx *ctx, const gc_mg_params *params, int *cycles);

/* ---- the whole step as one CUDA graph (no reference counterpart: the reference
 * synchronises with the host after every V-cycle, solver/multigrid.py:477-485) */

/* Capture one ADVANCE step of the fused engine (same particles, parameters and
 * flags as sp, without diagnostics) from the context's stream (set one with
 * gc_set_stream) and instantiate it. The adaptive solve keeps the reference's
 * stopping rule, decided on the device: a conditional while node repeats the
 * V-cycle until ||r|| < tol ||b|| (at least max(1, min_cycles), at most
 * max_cycles cycles). A replay (gc_pm_graph_launch) makes no host
 * synchronisation and gives the state an eager gc_pm_step would, bit for bit.
 * Needs an open engine that has taken at least three steps with these flags
 * (the warm-start history must be complete); a graph stays valid while the
 * particle arrays, the stream and the warm-start mode are unchanged (the cell
 * sort swaps particle buffers: keep one graph per buffer set). */
typedef struct gc_graph gc_graph;
int gc_pm_graph_create(gc_ctx *ctx, const gc_particles *p, const gc_step_params *sp, gc_graph **out);
int gc_pm_graph_launch(gc_graph *g);
int gc_pm_graph_destroy(gc_graph *g);
/* Kernels a replay launches: fixed_launches + cycles * body_launches. */
int gc_pm_graph_info(const gc_graph *g, long long *fixed_launches, long long *body_launches);
/* V-cycles, converged flag and relative residual of the last replayed solve,
 * from the pinned mirror the graph writes: synchronise the stream first. */
int gc_pm_graph_stats(const gc_ctx *ctx, int *cycles, int *converged, double *rel);
/* Totals of the solves decided on the device since the last reset: out[0]
 * solves, out[1] V-cycles, out[2] the largest relative residual they ended with.
 * Synchronises; reset != 0 clears the totals afterwards. */
int gc_pm_solve_counters(gc_ctx *ctx, double out[3], int reset);

/* ---- instrumentation (no kernel counterpart in the reference: it replaces the
 * sync-bracketed per-stage wall clock of bench.py:66-73, 176-186) ---------- */

/* Every launch is counted per kernel id; with profiling enabled each launch is
 * also bracketed by CUDA events on the context's stream. */
int gc_profile_enable(gc_ctx *ctx, int enable);
int gc_profile_reset(gc_ctx *ctx);
/* Launches, event-timed launches and their total milliseconds for kernel id kid
 * since the last reset (synchronises when events are pending). */
int gc_profile_read(gc_ctx *ctx, int kid, long long *launches, long long *timed, double *ms);
int gc_num_kernel_ids(void);
const char *gc_kernel_name(int kid);

/* Self-test of the bounded device waits (no reference counterpart): one thread
 * arms an mbarrier for one arrival and waits on it with the library's bounded
 * wait for budget_cycles SM clocks (1 <= budget_cycles <= 2e9, about a second).
 * With arrive = 0 nobody arrives, the wait gives up and GC_FLAG_TIMEOUT is OR-ed
 * into *status (device word); with arrive = 1 the wait succeeds and *status is
 * left alone. Stream-ordered; the context stays usable either way. */
int gc_selftest_wait_timeout(void *stream, uint32_t *status, int64_t budget_cycles, int arrive);

/* ---- learned warm start (new: replaces the previous-step initial guess of the
 * multigrid, solver/multigrid.py:464-467, by a convolutional prediction) ----- */

/* Device check of the tensor-core operand conventions: D (128 x N, f32, row-major)
 * = A (128 x K) * B (N x K)^T with A, B row-major bf16 bits; a_mn / b_mn stage the
 * operand MN-major instead of K-major; swap exchanges the descriptor's two byte
 * offsets of MN-major operands. 16 <= N <= 256, 16 <= K <= 64, both multiples of
 * 16. *status (device) gets bit 0 on a completion timeout. */
int gc_ws_selftest_gemm(const void *A, const void *B, float *D, int N, int K, int a_mn, int b_mn, int swap,
                        void *stream, unsigned *status);

/* The warm-start network: a 3-D convolutional encoder-decoder on an R^3 grid
 * (R = G/2; levels R, R/2, R/4, R/8 with 16, 32, 64, 128 channels; 3x3x3
 * kernels; BF16 weights and activations, FP32 accumulation on the tensor cores).
 * Parameters are one f32 vector: for each of the 11 layers (gc_ws_layer_info)
 * the weights [27][cout][cin] (tap t = (dz+1)*9 + (dy+1)*3 + (dx+1)) then the
 * bias [cout]. All pointers are device pointers; calls are ordered on the
 * object's stream. */
typedef struct gc_ws gc_ws;
int gc_ws_create(gc_ws **out, int R);           /* 16 <= R <= 512, R % 8 == 0 */
int gc_ws_destroy(gc_ws *ws);
const char *gc_ws_last_error(const gc_ws *ws);
int gc_ws_set_stream(gc_ws *ws, void *stream);
int gc_ws_layer_info(int layer, int *cin, int *cout, int *level, int *relu);
int gc_ws_num_params(const gc_ws *ws, int64_t *n);
/* Replace the parameters (resets the Adam moments) / read them / read the last gradient. */
int gc_ws_set_params(gc_ws *ws, const float *params);
int gc_ws_get_params(gc_ws *ws, float *params);
int gc_ws_get_grads(gc_ws *ws, float *grads);
/* Forward pass: feat = f16 [4][R^3] input channels; y_out (nullable) = f32 [R^3]. */
int gc_ws_forward(gc_ws *ws, const void *feat, float *y_out);
/* Backward pass of the last forward for the loss 0.5 * mean((y - target)^2),
 * target f16 [R^3]; the loss goes to *loss_out (device f32, nullable) and the
 * parameter gradient to the object's gradient vector. */
int gc_ws_backward(gc_ws *ws, const void *target, float *loss_out);
/* One Adam step (bias-corrected, step >= 1) with the last gradient. */
int gc_ws_adam(gc_ws *ws, float lr, float beta1, float beta2, float eps, int step);
/* Device status bits (bit 0: a tensor-core completion wait timed out); clear resets them. */
int gc_ws_status(gc_ws *ws, unsigned *flags, int clear);
/* Autotuner: time every feasible tile plan (block of output planes x lines,
 * taps per weight group) of each layer's forward, data-gradient and weight-
 * gradient kernels with CUDA events over `iters` launches and keep the fastest.
 * Overwrites activations. ms_out (host, nullable, 33 floats): best milliseconds
 * per [layer][pass]. Synchronises the stream. */
int gc_ws_autotune(gc_ws *ws, int iters, float *ms_out);
/* Plan in use for (layer, pass 0/1/2): out[5] = {planes, lines, taps per group or
 * pass, CTAs, M tiles per CTA (0 for the weight gradient)}. */
int gc_ws_plan_info(const gc_ws *ws, int layer, int kind, int *out);

/* Initial guess of the engine's solve (gc_pm_step with warm_start != 0):
 *   GC_WS_PLAIN       phi(n-1), the previous potential (the reference's warm start);
 *   GC_WS_EXTRAPOLATE phi(n-1) + (phi(n-1) - phi(n-2)) at full resolution;
 *   GC_WS_LEARNED     the extrapolation + the network's prediction of the next
 *                     second difference of the potential (R = G/2 grid, trilinear).
 * The multigrid always iterates to the same residual: only the start changes.
 * The non-plain modes keep the previous potential; the learned mode, and any
 * mode with track != 0, also keep the coarse (G/2) history and build the
 * network features every solve (gc_pm_record_sample needs track != 0). A
 * change of mode restarts the history. G even. */
#define GC_WS_PLAIN 0
#define GC_WS_LEARNED 1
#define GC_WS_EXTRAPOLATE 2
int gc_pm_set_warmstart(gc_ctx *ctx, gc_ws *ws, int mode, int track);
/* One-shot: the next gc_pm_step writes its network input features and the
 * second difference its solve produced (the training target) to out, f16
 * [5][(G/2)^3]: channels 0..3 the features, 4 the target (see gc_ws_forward). */
int gc_pm_record_sample(gc_ctx *ctx, void *out);

#ifdef __cplusplus
}
#endif

#endif /* GCPM_H */
