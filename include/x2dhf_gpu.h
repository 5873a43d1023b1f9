/*
 * x2dhf_gpu.h -- C ABI of the GB300 (sm_103a) relaxation library for x2dhf.
 *
 * The library replaces the (MC)SOR relaxation hot path of x2dhf 3.0
 * (src/sormcsor.F90, src/relaxOrbs.F90, src/relaxPots.F90, src/inout.F90 and
 * the C backend src/c/*.c) and the Newton-Cotes quadratures the SCF loop
 * calls between sweeps, with hand-written CUDA kernels on one GPU.
 *
 * Two layers are exported:
 *
 *  1. Reference-named entry points with the reference's exact C signatures,
 *     so a PTHREAD build of x2dhf links this library instead of src/c/*.c.
 *     They read the Fortran COMMON blocks c_interface_*_, c_sorptr_,
 *     c_supplptr_, c_orbptr_, c_exchptr_, c_i4b_, c_iadex_ (layouts of
 *     src/c/sorpt.h:58-249), which the library references weakly; without a
 *     Fortran program that defines them these entry points return without
 *     touching memory and set x2g_last_status() to X2G_ERR_NO_COMMON.
 *
 *  2. Explicit entry points (x2g_*) taking plain pointers and sizes.  They
 *     return an int status (0 = success, see X2G_ERR_*) and never abort.
 *
 * All arrays are FP64, column-major as in the reference: nu (N_nu points) is
 * the fastest index, mu (N_mu points) the slowest.  "plain" arrays hold
 * N_nu*N_mu values; "extended" arrays hold (N_nu+8)*(N_mu+8) values with the
 * function at (nu+4, mu+4) and 4-point ghost margins (src/inout.F90:23-82).
 */
#ifndef X2DHF_GPU_H
#define X2DHF_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ */
/* status codes                                                       */
/* ------------------------------------------------------------------ */
#define X2G_OK 0
#define X2G_ERR_ARG 1          /* bad argument (dimension, pointer, range)          */
#define X2G_ERR_CUDA 2         /* CUDA runtime error (message in x2g_last_error)    */
#define X2G_ERR_ALLOC 3        /* device allocation failed                          */
#define X2G_ERR_TIMEOUT 4      /* a device-side barrier wait ran out (no hang)      */
#define X2G_ERR_NAN 5          /* NaN detected in an orbital or potential           */
#define X2G_ERR_SCHEDULE 6     /* colour/level schedule failed its host-side check  */
#define X2G_ERR_NO_COMMON 7    /* reference COMMON blocks not linked                */
#define X2G_ERR_UNSUPPORTED 8  /* case outside the supported scope (open shells)    */
#define X2G_ERR_NO_DEVICE 9    /* no CUDA device                                    */

#define X2G_MAXORB 36          /* src/params.h MAXORB */

/* precision forms */
#define X2G_FP64 0   /* plain: FP64 MCSOR, reference colour order, bit-exact sweeps    */
#define X2G_MIXED 1  /* FP32 sweeps on CUDA cores + FP64 defect correction per call      */
#define X2G_SOR 2    /* FP64 list-order SOR over the reference's "middle" point list (sor,
                        src/sormcsor.F90:20-132, the reference's default): bit-exact */

typedef struct x2g_ctx x2g_ctx;    /* one GPU, one stream, owned device memory */
typedef struct x2g_grid x2g_grid;  /* prolate-spheroidal grid + operator tables + sweep schedule */
typedef struct x2g_scf x2g_scf;    /* device-resident SCF state of one molecule */

/* Last status / message of the calling thread (never NULL). */
int x2g_last_status(void);
const char *x2g_last_error(void);

/* ------------------------------------------------------------------ */
/* context                                                            */
/* ------------------------------------------------------------------ */
/* Create a context on CUDA device `device` with its own non-blocking stream
 * (highest priority; not ordered after the legacy default stream: device
 * inputs written on other streams must be complete before a call). */
int x2g_create(x2g_ctx **ctx, int device);
int x2g_destroy(x2g_ctx *ctx);
/* Wait for all work queued on the context's stream. */
int x2g_synchronize(x2g_ctx *ctx);
/* The context's cudaStream_t, as an opaque pointer. */
void *x2g_stream(x2g_ctx *ctx);
/* Sweep-kernel timing with CUDA events on the context's stream.
 * enable: 1 on, 0 off, 2 reset counters and switch on, -1 query only.
 * precision selects the FP64 sweep kernel (0) or the FP32 sweep kernel of
 * the mixed form (1); outputs are summed over launches resolved at the last
 * x2g_synchronize: milliseconds, point-updates, launches. */
int x2g_profile(x2g_ctx *ctx, int enable, int precision, double *ms, double *points, long *launches);

/* ------------------------------------------------------------------ */
/* grid                                                               */
/* ------------------------------------------------------------------ */
/* Build the grid, every supplementary array of src/initCBAllocArrays.F90
 * initSuppl:1636-2051 (b, d, e, f0..f4, g, wgt1, wgt2, Legendre tables),
 * the "middle" point ordering of mesh:2503-2544 and the colour/level
 * schedule of the GPU sweep.  nnu, nmu must already satisfy the reference's
 * n = 1 (mod 30) rounding (x2g_round_grid). */
int x2g_grid_create(x2g_ctx *ctx, int nnu, int nmu, double r, double rinf, double z1, double z2, int mpole,
                    x2g_grid **grid);
int x2g_grid_destroy(x2g_grid *grid);
/* The reference's grid rounding (src/inputInterface.F90:2961-3095). */
int x2g_round_grid(int n);
/* Number of mu points the reference derives from nnu and R_inf when the grid
 * card gives no mu count (nmucalc with n=0, inputInterface.F90:2983-2992). */
int x2g_nmu_from_rinf(int nnu, double r, double rinf);
/* Default overrelaxation parameters (setOmega, initCBAllocArrays.F90:636-650,
 * 1010-1040): omega_pot and omega_orb = (omega_pot-1)*omega_pot - 0.001*max(Z1,Z2). */
int x2g_default_omega(int nnu, int nmu, double z1, double z2, double *omega_orb, double *omega_pot);
/* Copy a host table of the grid: which = 0 borb 1 bpot 2 d 3 e 4 f0 5 f1 6 f2
 * 7 f3 8 f4 9 g 10 wgt1 11 wgt2 (plain, N_nu*N_mu values). */
int x2g_grid_table(x2g_grid *grid, int which, double *host_out);
/* Host-only (no CUDA call) copies of the same tables and of the sweep
 * schedule, for checking the setup without a GPU.  x2g_host_schedule fills
 * order[k] (extended index, 0-based) with tile[k], colour[k], level[k] of
 * the k-th scheduled point when tile/colour/level are non-NULL, else the
 * reference's list order. */
int x2g_host_table(int nnu, int nmu, double r, double rinf, double z1, double z2, int which, double *out);
int x2g_host_schedule(int nnu, int nmu, int *npoints, int *ntiles, int *nlevels, int *order, int *tile,
                      int *colour, int *level);
/* Cluster plan of the on-chip FP32 sweep of the mixed form (no CUDA call):
 * CTAs per relaxation job (0 = grid too large, persistent-band kernel used),
 * rows of the largest band, shared memory per CTA, band starts row0[C+1]. */
int x2g_host_cluster_plan(int nnu, int nmu, int *csize, int *maxrows, long *smem, int *row0);
/* Chunk lists of the on-chip sweep (host only): chunks of up to 4 points of
 * one row at stride 5, packed (band row << 19) | (ext col << 2) | (count-1),
 * and the offsets of each CTA's 5 colours x (levels + 2) segments (level 0
 * off the shared band edges, level 0 near them, level-0 seam points, levels
 * 1..), plus the end.  Null arrays: counts only. */
int x2g_host_cluster_chunks(int nnu, int nmu, int *nchunks, int *noff, int *chunks, int *off);
/* The same for the seam-free colouring (x2g_set_mixed_colouring 1): per CTA
 * and colour the segments A, B and an empty seam segment. */
int x2g_host_free_chunks(int nnu, int nmu, int *nchunks, int *noff, int *chunks, int *off);
/* Schedule of the persistent-band FP32 sweep (host only): the scheduled
 * points regrouped by colour, level and tile, packed (ext row << 16) | ext
 * col (pts, npoints values); off[(c * nlevels + l) * (ntiles + 1) + t] is
 * the first point of tile t in colour c, level l (5 * nlevels * (ntiles+1)
 * values); rows[G] for G = 0..16 the most rows of G consecutive tiles plus
 * the two 4-row halos (rows[0] unused); tile_row0 / tile_row1 the tiles' ext
 * row ranges (ntiles values each).  Null arrays are skipped. */
int x2g_host_band_schedule(int nnu, int nmu, int *npoints, int *ntiles, int *nlevels, int *pts, int *off, int *rows,
                           int *tile_row0, int *tile_row1);
/* Longest time one block of a persistent sweep waits for the others (its
 * grid barrier or its neighbours' phase counts) before the launch gives up:
 * the block records X2G_ERR_TIMEOUT in the context's error word and every
 * block returns, so a stalled launch never hangs the GPU.  The error word
 * stays set, and later launches on the context leave at their first wait,
 * until x2g_synchronize (or the call's own readback) reports it and clears
 * it.  Default 2 s; 0 makes any wait that is not met at once fail (for
 * testing the error path).  Applies to launches queued after the call.  The
 * reference has no device waits (its threads join, src/c/mcsor_pthread.c:87). */
int x2g_set_wait_limit(x2g_ctx *ctx, double seconds);
/* Schedule of the list-order SOR wavefront (host only, no CUDA call): the
 * interior points grouped by SOR level (1 + the largest level of their
 * stencil neighbours earlier in the "middle" list), packed (ext row << 16) |
 * ext col (pts, npoints values; off, nlev + 1 offsets), the axis points
 * grouped by the level their extrapolation follows (bpts; boff, nblev + 1
 * offsets), and delta, the level shift between successive sweeps: sweep s
 * of a level-l point runs at step l + s * delta.  Null arrays are skipped. */
int x2g_host_sor_schedule(int nnu, int nmu, int *npoints, int *nlev, int *nblev, int *delta, int *pts, int *off,
                          int *bpts, int *boff);
/* Mixed form sweep path: 1 (default) on-chip cluster kernel where the grid
 * fits, 0 the persistent-band kernel, 2 the cluster kernel for batches that
 * fit its co-resident clusters and the persistent-band kernel for larger
 * batches that it holds in one launch. */
int x2g_set_mixed_on_chip(x2g_ctx *ctx, int on);
/* Mixed form, cluster kernel, batches of potentials built from orbitals
 * (lhs = f3 + idel^2 e, separable in mu and nu): a variant that keeps only
 * the residual on chip and forms omega / lhs from a row and a column term,
 * so that two CTAs fit each SM and twice the clusters are co-resident.
 * mode 0 never, 1 always, 2 (default) for batches larger than the clusters
 * of the plain kernel co-resident on the device.  No reference counterpart. */
int x2g_set_potential_clusters(x2g_ctx *ctx, int mode);
/* Batch mode 2, no orbital frozen: the orthonormalisation of an SCF
 * iteration (normOrtho.F90:14-59,103-207 for every orbital in the
 * reference's order) as 0 (default) rounds of independent orbitals with the
 * loop's own sums and operations (bit-identical to the orbital-by-orbital
 * loop), or 1 its Gram-matrix form -- the norms and every inner product of
 * the orbitals of a symmetry block in one pass, the coefficients of the
 * final orbitals from them, one pass applying them: equal in exact
 * arithmetic, faster, the rounding differs (so does the iteration at which
 * an SCF near its noise floor meets the convergence test).  No reference
 * counterpart. */
int x2g_set_gram_orthonormalise(x2g_ctx *ctx, int on);
/* Mixed form, potential batches larger than the co-resident clusters of
 * the potentials' cluster variant: 1 (default) the batch runs in waves of
 * that size and the FP64 residuals of the later waves run on the context's
 * low-priority auxiliary stream beside the earlier waves' sweeps (on the SMs
 * they leave free), 0 every residual before the first sweep.  Same kernels,
 * same results.  No reference counterpart. */
int x2g_set_residual_overlap(x2g_ctx *ctx, int on);
/* Colouring of the mixed form's on-chip cluster sweep: 0 the reference's
 * (colour = position in the "middle" list mod 5, sormcsor.F90:143-386, with
 * its seam points relaxed level by level, so that in exact arithmetic the
 * sweep equals the FP64 one), 1 seam-free (colour (col - row) mod 5 of the
 * extended-array point: no two points of a colour are stencil neighbours, so
 * every colour is one parallel step).  Both converge to the same fixed point;
 * the persistent-band sweep of large grids keeps the reference's colouring.
 * No reference counterpart. */
int x2g_set_mixed_colouring(x2g_ctx *ctx, int free);
/* Co-resident clusters of the mixed form's cluster sweep (plain) and of its
 * potentials' variant (pot) for this grid on the context's device; 0 where
 * that kernel cannot run the grid.  No reference counterpart. */
int x2g_cluster_occupancy(x2g_ctx *ctx, x2g_grid *grid, int *plain, int *pot);
/* Self-check of the mixed form's integer-pipe FP64<->FP32 conversions
 * against the hardware conversions on n values (edge cases, then hashed bit
 * patterns from seed); mismatches outside the documented flush-to-zero
 * range of float subnormals.  No reference counterpart. */
int x2g_convert_selftest(x2g_ctx *ctx, long n, unsigned long long seed, unsigned long long *mismatches);
/* Schedule statistics: tiles (row bands), colour levels, points per sweep. */
int x2g_grid_info(x2g_grid *grid, int *nnu, int *nmu, int *ntiles, int *nlevels, int *npoints);

/* ------------------------------------------------------------------ */
/* relaxation (src/sormcsor.F90 mcsor:143-386)                        */
/* ------------------------------------------------------------------ */
/* One function to relax.  All pointers are DEVICE pointers.
 *   u    extended array, relaxed in place (ghosts are refreshed from the
 *        interior first, as putin does, src/inout.F90:23-82)
 *   lhs  plain diagonal term; NULL for a potential: lhs = f3 + idel^2 e
 *   rhs  plain right-hand side; NULL for a potential: rhs = psa*psb*g
 *        (relaxPots.F90:81-95) built from psa/psb (extended orbitals)
 *   kind 0 orbital (b = borb), 1 potential (b = bpot)              */
typedef struct {
  double *u;
  const double *lhs;
  const double *rhs;
  const double *psa;
  const double *psb;
  double omega;
  int isym;
  int idel;
  int kind;
  int pad;
} x2g_job;

/* Relax `njobs` independent functions on the same grid with `nsweeps`
 * micro-sweeps each, in one persistent launch on the context's stream (jobs
 * beyond 32 in further launches).  `jobs` is a HOST array.  precision:
 * X2G_FP64 or X2G_MIXED (MCSOR forms) or X2G_SOR (list-order SOR, FP64). */
int x2g_relax(x2g_ctx *ctx, x2g_grid *grid, const x2g_job *jobs, int njobs, int nsweeps, int precision);

/* Relaxation that allocates no device memory (this entry point has no
 * counterpart in the reference).  Same contract and FP64 results as
 * x2g_relax with precision X2G_FP64, for callers that must not allocate:
 * x2g_relax grows a context workspace with cudaMalloc, after synchronising
 * the stream, when a larger batch arrives, which a loop admitting work
 * against a fixed HBM budget, or a host driver relaxing inside its inner
 * loop, cannot allow.  Here the scratch is one fixed 32 MiB device array in
 * the library (held by every GPU that loads it until the process exits),
 * looked up with cudaGetSymbolAddress on the first call on each device:
 * make that first call before any stream capture.  A batch needing more
 * than 32 MiB (256 B + a job table of 112 B per job rounded up to 256 B +
 * one nnu*nmu FP64 right-hand side per job, each rounded up to 256 B) is
 * rejected with X2G_ERR_ARG.  Batches above 32 jobs run as several launches;
 * a device wait timeout in any of them is returned as X2G_ERR_TIMEOUT.  Every call shares
 * the array and the call returns only after its kernel has finished; calls
 * that overlap on the GPU (other threads, other contexts on the same
 * device) would race on the shared scratch and must be serialised by the
 * caller. */
int x2g_relax_noalloc(x2g_ctx *ctx, x2g_grid *grid, const x2g_job *jobs, int njobs, int nsweeps);

/* putin / putout on device buffers (src/inout.F90:23-82, 165-183). */
int x2g_putin(x2g_ctx *ctx, x2g_grid *grid, int isym, const double *fun_plain, double *work_ext);
int x2g_putout(x2g_ctx *ctx, x2g_grid *grid, const double *work_ext, double *fun_plain);

/* Host-buffer form of one relaxation call, the unit the reference's
 * mcsor_pthread_ performs (mcsor_pthread.c:32): copies wk2/lhs/rhs to the
 * device, relaxes, copies wk2 back.  kind as in x2g_job. */
int x2g_mcsor_host(x2g_ctx *ctx, x2g_grid *grid, int isym, int kind, double omega, int nsweeps,
                   double *wk2_ext_host, const double *lhs_host, const double *rhs_host);

/* ------------------------------------------------------------------ */
/* quadratures (src/normOrtho.F90, src/integrals.F90)                  */
/* ------------------------------------------------------------------ */
/* sum_i w_i * a_i * b_i * c_i over the plain grid (c may be NULL), with w =
 * wgt1 (which=1) or wgt2 (which=2); a, b, c are EXTENDED device arrays.
 * Deterministic two-pass reduction; result written to host *out. */
int x2g_quadrature(x2g_ctx *ctx, x2g_grid *grid, int which, const double *a_ext, const double *b_ext,
                   const double *c_ext, double *out);

/* ------------------------------------------------------------------ */
/* SCF (src/doSCF.F90 prepSCF:24, scf:211, relaxDriver:943)            */
/* ------------------------------------------------------------------ */
/* A closed-shell HF case, the fields of the reference's input cards. */
typedef struct {
  double z1, z2, r;        /* nuclei card (bohr) */
  int nnu, nmu;            /* grid card after rounding (x2g_round_grid) */
  double rinf;             /* practical infinity (bohr) */
  int norb;                /* config card: orbitals in input order */
  int m[X2G_MAXORB];       /* |lambda|: 0 sigma 1 pi 2 delta 3 phi */
  char gu[X2G_MAXORB];     /* 'g', 'u' or ' ' */
  double occ[X2G_MAXORB];  /* 2 (sigma) or 4 (non-sigma): closed shells only */
  /* lcao card (hydrogenic start, initHyd initOrbitalsPotentials.F90:714) */
  double co1[X2G_MAXORB], co2[X2G_MAXORB], za[X2G_MAXORB], zb[X2G_MAXORB];
  int n1[X2G_MAXORB], l1[X2G_MAXORB], n2[X2G_MAXORB], l2[X2G_MAXORB];
  /* scf / conv / orbpot cards */
  int maxscf, ienterm, inoterm, ienterm4init;
  int nscf2skip, nenlast, nnolast;
  int maxsor_orb, maxsor_pot;   /* micro sweeps per relaxation (10) */
  double omega_orb, omega_pot;  /* <= 0: reference default */
  double recalc_mm;             /* recalcMMfactor (1.15) */
  int mpole;                    /* multipole terms (4) */
  int homonuclear;              /* g/u labels given: enforce C_i (setCi) */
  int precision;                /* X2G_FP64 or X2G_MIXED */
  int start;                    /* 0: hydrogenic LCAO guess (orbpot hydrogen); 1: functions, moments and
                                   Lagrange multipliers loaded by the caller before the first run
                                   (orbpot old: x2g_scf_set_function, x2g_scf_set_start_values) */
  /* relaxation scheme of the orbitals / the potentials (relaxDriver, doSCF.F90:943-1011):
   * 1 MCSOR (the mcsor or mcsor-o card sets it for orbitals, mcsor-ce for
   * potentials, inputInterface.F90:1910-2028), 0 list-order SOR (the
   * reference's default, sormcsor.F90:20-132) */
  int orb_scheme, pot_scheme;
  /* 0: the reference's order, the potentials of orbital i relaxed just
   * before orbital i (relaxDriver, doSCF.F90:943-1011); 1: every Coulomb and
   * exchange potential of an SCF iteration relaxed in one batched launch
   * from the orbitals at the start of the iteration, then the orbitals in
   * the reference's order; 2: as 1, then every orbital relaxed in one
   * batched launch with the Fock operators of the state after the
   * potentials, before the norms, orthogonalisation and energies in the
   * reference's order.  Same fixed point, different trajectory (no
   * reference counterpart). */
  int batch_mode;
} x2g_case;

typedef struct {
  int iterations;          /* SCF iterations performed */
  int converged;           /* 1 energy threshold, 2 norm threshold, 0 limit/other */
  long sweeps;             /* (MC)SOR sweeps: nsor4orb + nsor4pot */
  double total_energy;     /* etot (Eh) */
  double electronic_energy;
  double virial;
  double ee[X2G_MAXORB];   /* orbital energies (diagonal Lagrange multipliers) */
  double norm_error[X2G_MAXORB];
} x2g_result;

int x2g_case_defaults(x2g_case *c);
int x2g_scf_create(x2g_ctx *ctx, const x2g_case *c, x2g_scf **scf);
int x2g_scf_destroy(x2g_scf *scf);
/* Run up to max_iterations SCF iterations (prepSCF on the first call).
 * Returns X2G_OK; result->converged tells why the loop stopped. */
int x2g_scf_run(x2g_scf *scf, int max_iterations, x2g_result *result);
/* Copy orbital iorb (1-based, input order) / its Coulomb potential to a host
 * plain array of N_nu*N_mu values. */
int x2g_scf_get_orbital(x2g_scf *scf, int iorb, double *host_plain);
int x2g_scf_get_coulomb(x2g_scf *scf, int iorb, double *host_plain);
/* Functions of the SCF as plain nnu*nmu host arrays (nu fastest): kind 0
 * orbital i1, 1 Coulomb potential of i1, 2 exchange potential of the pair
 * i1 <= i2 (which = 1: the second potential of two non-sigma orbitals,
 * Delta m = m1 + m2); i2 = which = 0 for kinds 0 and 1.  Setting them before
 * the first x2g_scf_run is the orbpot old start (readFuncs,
 * src/diskInterface.F90:247-779). */
int x2g_scf_set_function(x2g_scf *scf, int kind, int i1, int i2, int which, const double *host_plain);
int x2g_scf_get_function(x2g_scf *scf, int kind, int i1, int i2, int which, double *host_plain);
/* Values an orbpot old start takes from the checkpoint instead of
 * recomputing them (prepSCF runs no initAddData, src/doSCF.F90:73-134), in
 * the checkpoint's layout: diagonal Lagrange multipliers ee[norb], norms
 * orbnorm[norb], Coulomb moments cmulti[iorb-1 + (k-1) norb] (X2G_MAXORB*8
 * entries) and exchange moments exc[(k-1) X2G_MAXORB(X2G_MAXORB+1) +
 * ipc-1] (8 arrays).  The getter returns the current values (for writing a
 * checkpoint). */
int x2g_scf_set_start_values(x2g_scf *scf, const double *ee, const double *orbnorm, const double *cmulti,
                             const double *exc);
int x2g_scf_get_start_values(x2g_scf *scf, double *ee, double *orbnorm, double *cmulti, double *exc);
/* Per-iteration record i (0-based): iscf, iorb, ee, delta ee, 1-norm. */
int x2g_scf_nrecords(x2g_scf *scf);
int x2g_scf_record(x2g_scf *scf, int i, int *iscf, int *iorb, double *ee, double *dee, double *dnorm);
/* Device launches of this library's kernels so far on the scf's context. */
long x2g_kernel_launches(x2g_ctx *ctx);
/* Host-to-device and device-to-host bytes the library has copied so far on
 * the context (grid tables, function uploads and readbacks, per-iteration
 * scalars, error words). */
int x2g_transfer_bytes(x2g_ctx *ctx, long long *h2d, long long *d2h);

/* ------------------------------------------------------------------ */
/* reference-named entry points (link-compatible with src/c/*.c)       */
/* ------------------------------------------------------------------ */
/* src/c/mcsor_pthread.c:32 -- relax the orbital held in wk2 (extended),
 * lhs/rhs plain; nthreads is accepted and ignored (one GPU). */
void mcsor_pthread_(int *isym, int *nthreads, double *wk2, double *lhs, double *rhs);
/* src/c/mcsor_tpool.c:135 -- same contract as mcsor_pthread_. */
void mcsor_tpool_(int *isym, int *nthreads, double *wk2, double *lhs, double *rhs);
/* src/c/coulExch_pthread.c:19 -- relax every Coulomb/exchange potential of
 * orbital c_interface_46_.iorbc in one batched launch. */
void coulExch_pthread_(void);
/* src/c/coulExch_tpool.c:109 -- same contract as coulExch_pthread_. */
void coulExch_tpool_(void);
/* x2dhf.F90:44-55 tpool shutdown hooks: release the GPU context. */
void tpoolStop4mcsor_(int *nthreads);
void tpoolStop4pots_(int *nthreads);

#ifdef __cplusplus
}
#endif
#endif
