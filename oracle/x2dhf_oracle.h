/*
 * x2dhf CPU oracle -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the x2dhf (MC)SOR relaxation path and of the
 * closed-shell HF SCF loop that drives it (reference: x2dhf 3.0, Fortran 90).
 * Only tests/, __graft_entry__.smoke() and bench.py (cpu_baseline leg and the
 * --impl reference arm) may load this code, and only as the checker or as
 * the timed CPU baseline.  The GPU product never links or calls it.
 *
 * Parity of this restatement is pinned against the per-iteration orbital
 * energies printed in the reference's own golden outputs
 * (test-sets/{h2/set-01,he/set-01,he/set-02,ne/set-01,h/set-04}/reference.lst,
 * extracted into tests/golden/ by tests/golden/make_golden.py) and, for the
 * potential sweep, bit-for-bit against the reference's own C kernel sorpt_
 * (src/c/sorpt.c) built by oracle/build_ref.sh.
 *
 * Every function cites the reference file:line it restates.
 */
#ifndef X2DHF_ORACLE_H
#define X2DHF_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

#define X2O_MAXORB 36
#define X2O_MAXMPOLE 8

typedef struct x2o_state x2o_state;

/* Parse a reference input file (cards: title method nuclei config grid orbpot [hydrogen|old]
 * lcao scf conv mcsor mcsor-o mcsor-ce omega multipol altsweeps homo break
 * sor4orb sor4pot stop) -- restates src/inputInterface.F90:681-818 for the HF
 * subset.  Returns NULL and fills err on failure. */
x2o_state *x2o_from_input(const char *text, char *err, int errlen);

/* Build grid, supplementary arrays, index lists, potential tables
 * (src/initCBAllocArrays.F90 initArrays:1472) and the hydrogenic start
 * (src/initOrbitalsPotentials.F90 initHyd:714). */
int x2o_setup(x2o_state *s);

/* prepSCF (src/doSCF.F90:24) + scf (src/doSCF.F90:211).  verbose>0 prints the
 * reference's per-iteration lines on stdout.  Returns the iteration count. */
int x2o_run_scf(x2o_state *s, int verbose);
/* Run at most n SCF iterations (prepSCF is run on the first call); returns 1
 * when the SCF loop has terminated. */
int x2o_scf_steps(x2o_state *s, int n, int verbose);

void x2o_free(x2o_state *s);

/* ---- accessors used by the tests ---- */
int x2o_nni(const x2o_state *s);
int x2o_nmu(const x2o_state *s);
int x2o_norb(const x2o_state *s);
int x2o_iterations(const x2o_state *s);
double x2o_total_energy(const x2o_state *s);
double x2o_orbital_energy(const x2o_state *s, int iorb); /* 1-based */
double x2o_omega_orb(const x2o_state *s);
double x2o_omega_pot(const x2o_state *s);
long x2o_sweeps(const x2o_state *s); /* nsor4orb + nsor4pot */
/* number of energy records (one per orbital per SCF iteration) and record i:
 * iscf, iorb, ee, deltaee, 1-norm */
int x2o_nrecords(const x2o_state *s);
void x2o_record(const x2o_state *s, int i, int *iscf, int *iorb, double *ee,
                double *dee, double *dnorm);

/* Grid tables (copies into caller buffers). */
int x2o_ngrid(const x2o_state *s, int *ngrid1, int *ngrid6a, int *ngrid6b, int *ngrid7);
void x2o_lists(const x2o_state *s, int *indx1, int *indx2, int *indx6a, int *indx6b, int *indx7);
/* which: 0 borb 1 bpot 2 d 3 e 4 f0 5 f1 6 f2 7 f3 8 f4 9 g 10 wjac1 11 wjac2 12 wgt1 13 wgt2 */
void x2o_suppl(const x2o_state *s, int which, double *out);
void x2o_coeffs(const x2o_state *s, double *dmu1, double *dmu2, double *dni1, double *dni2,
                double *exeven, double *diag);
void x2o_get_orbital(const x2o_state *s, int iorb, double *out);      /* plain mxsize */
void x2o_set_orbital(x2o_state *s, int iorb, const double *in);
/* diagonal Lagrange multiplier of iorb (an orbpot old start reads it from
 * the checkpoint, src/diskInterface.F90:335-337) */
void x2o_set_orbital_energy(x2o_state *s, int iorb, double ee);
/* multipole moments stored in a checkpoint: cmulti (MAXORB*MAXMPOLE
 * entries) and the exchange moments excdi..exc8 (8 x MAXORB*(MAXORB+1)) */
void x2o_set_moments(x2o_state *s, const double *cmulti, const double *exc);
/* potential slot k of orbital iorb's relaxation batch (1-based, k<=npots) */
int x2o_npots(const x2o_state *s, int iorb);
void x2o_pot_info(const x2o_state *s, int iorb, int k, int *in1, int *in2, int *idel, int *isym);
void x2o_get_pot(const x2o_state *s, int iorb, int k, double *out);
void x2o_set_pot(x2o_state *s, int iorb, int k, const double *in);

/* ---- free-standing kernels (same arithmetic as the SCF path) ---- */
/* putin / putout: src/inout.F90:23-82, 165-183 */
void x2o_putin(int nni, int nmu, int isym, const double *fun, double *work);
void x2o_putout(int nni, int nmu, double *fun, const double *work);
/* One relaxation call of maxsor2 micro-sweeps on an extended array.
 * mode 0: sor in list order (src/sormcsor.F90:20-132)
 * mode 1: single-thread mcsor, colour classes i = c (mod 5) of the list
 *         (src/sormcsor.F90:143-386)
 * mode 2: not a reference ordering -- the checker of the GPU mixed form's
 *         seam-free colouring: colour (col - row) mod 5 of the extended-array
 *         point, colours in turn, then the axis extrapolation as above. */
void x2o_sweep(const x2o_state *s, int mode, int isym, int maxsor2, double omega,
               double *uext, const double *lhs, const double *rhs,
               const double *b, const double *d, int isstart, int isstop, int isstep);
/* Relax potential k of orbital iorb's batch in place (coulExchSOR body,
 * src/relaxPots.F90:64-104), mode as above. */
void x2o_relax_pot(x2o_state *s, int iorb, int k, int mode);
/* Relax orbital iorb in place (orbSOR / orbMCSOR, src/relaxOrbs.F90:16-241). */
void x2o_relax_orb(x2o_state *s, int iorb, int mode);
/* Fock potential for orbital iorb (src/fock.F90:57-186): fock1, fock2 plain. */
void x2o_fock(x2o_state *s, int iorb, double *fock1, double *fock2);
/* Quadratures */
double x2o_norm_value(x2o_state *s, int iorb);                 /* norm94 */
void x2o_norm(x2o_state *s, int iorb);                          /* norm */
void x2o_ortho(x2o_state *s, int iorb);
void x2o_eahf(x2o_state *s, int iorb);
double x2o_ee(const x2o_state *s, int i, int j);
void x2o_etotal(x2o_state *s, double *etot, double *evt, double *vkt, double *vnt);
void x2o_mpole_moments(x2o_state *s, int all_touched);
void x2o_pot_asympt(x2o_state *s, int iorb);
/* multipole moments: cmulti[(k-1)*norb + iorb-1], exchange moments by pair */
void x2o_cmulti(const x2o_state *s, double *out);

/* Batched modes (no reference counterpart): 1 relaxes every potential of an
 * SCF iteration from the orbitals at the start of the iteration, before the
 * orbital loop; 2 then also relaxes every orbital with the Fock operator of
 * the state after the potentials before the norms, orthogonalisation and
 * energies of the orbital loop; 0 (default) is relaxDriver's order. */
void x2o_set_batch_potentials(x2o_state *s, int on);

/* Replace the relaxations by external kernels (the reference's own C backend
 * in the timed reference run): pot_hook(ud, iorb) relaxes every potential of
 * orbital iorb in the potential block; orb_hook(ud, iorb, isym, wk2, lhs,
 * rhs) sweeps the extended orbital wk2.  Storage: one orbital block (orbital
 * i at (i-1)*mxsize) and one potential block; x2o_pot_offset is the 1-based
 * offset of potential k of orbital iorb (the reference's ibexcp). */
void x2o_set_hooks(x2o_state *s, void (*pot_hook)(void *, int),
                   void (*orb_hook)(void *, int, int, double *, double *, double *), void *ud);
double *x2o_orbital_block(x2o_state *s);
double *x2o_potential_block(x2o_state *s);
long x2o_pot_offset(const x2o_state *s, int iorb, int k);

#ifdef __cplusplus
}
#endif
#endif
