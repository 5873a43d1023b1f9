/*
 * Host shim for the reference's C relaxation kernels -- TEST INFRASTRUCTURE.
 *
 * x2dhf's src/c/*.c read their parameters from Fortran COMMON blocks and
 * call back into Fortran (putinc_/putoutc_).  Without a Fortran compiler
 * this file provides both, so the reference's own sorpt_ and
 * mcsor_pthread_ / mcsor_single_colour_pthread_ run unmodified as a checker
 * and as the timed CPU reference:
 *   - COMMON block instances with the layouts of src/c/sorpt.h:58-249,
 *   - putinc_/putoutc_ restated from src/inout.F90:195-290,
 *   - x2r_* setters that fill the blocks from plain arrays (the values the
 *     Fortran program writes in initCBAllocArrays.F90 initMesh:2053-2370,
 *     initAddr:1339-1466, initSuppl:1636-2051, relaxPots.F90:137-142),
 *   - x2r_coulexch: the thread-per-potential driver of coulExch_pthread.c /
 *     relax_single_pot_pthread.c restated around the reference's sorpt_.
 *     The reference's own driver writes one element past a stack array
 *     (relax_single_pot_pthread.c:47), which is not safe to run on aarch64.
 */
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include "sorpt.h"

/* The reference sources are compiled with -Dpthread_join=x2r_pthread_join:
 * they pass an int* as the void** exit value (mcsor_pthread.c:87,
 * coulExch_pthread.c:120), so the real call would store a pointer into 4
 * bytes of their stack.  The exit value is never used; it is discarded. */
#undef pthread_join
extern int pthread_join(pthread_t, void **);
int x2r_pthread_join(pthread_t t, void **ret) {
  (void)ret;
  return pthread_join(t, NULL);
}

struct commonBlock_1_t c_interface_1_;
struct commonBlock_2_t c_interface_2_;
struct commonBlock_3_t c_interface_3_;
struct commonBlock_4_t c_interface_4_;
struct commonBlock_6_t c_interface_6_;
struct commonBlock_7_t c_interface_7_;
struct commonBlock_8_t c_interface_8_;
struct commonBlock_9_t c_interface_9_;
struct commonBlock_10_t c_interface_10_;
struct commonBlock_11_t c_interface_11_;
struct commonBlock_12_t c_interface_12_;
struct commonBlock_13_t c_interface_13_;
struct commonBlock_14_t c_interface_14_;
struct commonBlock_15_t c_interface_15_;
struct commonBlock_16_t c_interface_16_;
struct commonBlock_17_t c_interface_17_;
struct commonBlock_20_t c_interface_20_;
struct commonBlock_40_t c_interface_40_;
struct commonBlock_41_t c_interface_41_;
struct commonBlock_42_t c_interface_42_;
struct commonBlock_43_t c_interface_43_;
struct commonBlock_44_t c_interface_44_;
struct commonBlock_45_t c_interface_45_;
struct commonBlock_46_t c_interface_46_;
struct commonBlock_47_t c_interface_47_;
struct cb_1_t c_orbptr_;
struct cb_2_t c_exchptr_;
struct cb_3_t c_supplptr_;
struct cb_5_t c_sorptr_;
struct cb_10_t c_i4b_;
struct cb_11_t c_iadex_;

static int *g_sor = NULL; /* [orig ext list | orig plain list | colour ext | colour plain | 6a | 6b | 7] */
static int g_ngrid1 = 0, g_nni = 0, g_nmu = 0, g_n6a = 0, g_n6b = 0, g_n7 = 0;

/* putinc: src/inout.F90:195-260 (also replicates row nmu+4 upwards) */
void putinc_(int *pnni, int *pnmi, int *pisym, double *fun, double *work) {
  int nni = *pnni, nmi = *pnmi, isym = *pisym, n8 = nni + 8;
#define FUN(j, i) fun[((i)-1) * nni + ((j)-1)]
#define WRK(j, i) work[((i)-1) * n8 + ((j)-1)]
  for (int i = 1; i <= nmi; i++)
    for (int j = 1; j <= nni; j++) WRK(4 + j, i + 4) = FUN(j, i);
  for (int i = 2; i <= 5; i++)
    for (int j = 1; j <= nni; j++) WRK(4 + j, 6 - i) = (isym == 1) ? FUN(j, i) : -FUN(j, i);
  for (int j = 2; j <= 5; j++)
    for (int i = 1; i <= nmi; i++) WRK(6 - j, 4 + i) = (isym == 1) ? FUN(j, i) : -FUN(j, i);
  for (int j = 1; j <= 4; j++)
    for (int i = 1; i <= nmi; i++) WRK(nni + 4 + j, 4 + i) = (isym == 1) ? FUN(nni - j, i) : -FUN(nni - j, i);
  for (int i = 1; i <= 4; i++)
    for (int j = 1; j <= n8; j++) WRK(j, nmi + 4 + i) = WRK(j, nmi + 4);
#undef FUN
#undef WRK
}

/* putoutc: src/inout.F90:266-290 */
void putoutc_(int *pnni, int *pnmi, double *fun, double *work) {
  int nni = *pnni, nmi = *pnmi, n8 = nni + 8;
  for (int i = 1; i <= nmi; i++)
    for (int j = 1; j <= nni; j++) fun[(i - 1) * nni + (j - 1)] = work[(i + 3) * n8 + (j + 3)];
}

/* Grid, lists, coefficients and supplementary arrays.  suppl holds the 14
 * supplementary arrays (borb bpot d e f0 f1 f2 f3 f4 g wjac1 wjac2 wgt1
 * wgt2) of mxsize values each, as initSuppl lays out cw_suppl. */
int x2r_setup(int nni, int nmu, const int *indx1, const int *indx2, int ngrid1, const int *i6a, int n6a,
              const int *i6b, int n6b, const int *i7, int n7, const double *dmu1, const double *dmu2,
              const double *dnu1, const double *dnu2, const double *exeven, double *suppl, int maxsor2) {
  free(g_sor);
  g_sor = (int *)malloc(sizeof(int) * (4 * (size_t)ngrid1 + n6a + n6b + n7));
  if (!g_sor) return 1;
  g_ngrid1 = ngrid1; g_nni = nni; g_nmu = nmu; g_n6a = n6a; g_n6b = n6b; g_n7 = n7;
  int *o1 = g_sor, *o2 = g_sor + ngrid1, *c1 = g_sor + 2 * ngrid1, *c2 = g_sor + 3 * ngrid1;
  memcpy(o1, indx1, sizeof(int) * ngrid1);
  memcpy(o2, indx2, sizeof(int) * ngrid1);
  /* colour reorder (initMesh:2226-2240): stable partition by i mod 5 */
  int j = 0;
  for (int col = 1; col <= 5; col++)
    for (int i = col; i <= ngrid1; i += 5) { c1[j] = indx1[i - 1]; c2[j] = indx2[i - 1]; j++; }
  int *b6a = g_sor + 4 * ngrid1, *b6b = b6a + n6a, *b7 = b6b + n6b;
  memcpy(b6a, i6a, sizeof(int) * n6a);
  memcpy(b6b, i6b, sizeof(int) * n6b);
  memcpy(b7, i7, sizeof(int) * n7);
  c_sorptr_.cw_sor = g_sor;
  c_iadex_.iadex1c = 4 * ngrid1 + 1;
  c_iadex_.iadex2c = 4 * ngrid1 + n6a + 1;
  c_iadex_.iadex3c = 4 * ngrid1 + n6a + n6b + 1;
  c_iadex_.iadextc = 1;
  c_iadex_.iadnorc = ngrid1 + 1;
  int n1 = nni + 8;
  c_interface_17_.mxnmuc = nmu;
  c_interface_17_.mxsizec = nni * nmu;
  c_interface_17_.ngrd6ac = n6a;
  c_interface_17_.ngrd6bc = n6b;
  c_interface_17_.ngrd7c = n7;
  c_interface_17_.nnu1c = n1; c_interface_17_.nnu2c = 2 * n1; c_interface_17_.nnu3c = 3 * n1;
  c_interface_17_.nnu4c = 4 * n1; c_interface_17_.nnu5c = 5 * n1;
  c_interface_17_.isstartc = 1; c_interface_17_.isstopc = ngrid1;
  c_interface_17_.maxsor1c = 1; c_interface_17_.maxsor2c = maxsor2;
  memcpy(c_interface_40_.dmu1c, dmu1, 32);
  memcpy(c_interface_41_.dmu2c, dmu2, 32);
  memcpy(c_interface_42_.dnu1c, dnu1, 32);
  memcpy(c_interface_43_.dnu2c, dnu2, 32);
  memcpy(c_interface_44_.exevenc, exeven, 40);
  c_supplptr_.cw_suppl = suppl;
  for (int i = 0; i < 20; i++) c_i4b_.i4barr[i] = i * nni * nmu + 1;
  return 0;
}

/* list order seen by the kernels: 0 the "middle" order (SOR), 1 the colour
 * reordered list (what a PT build with the mcsor card holds in cw_sor) */
void x2r_use_colour_lists(int colour) {
  c_iadex_.iadextc = colour ? 2 * g_ngrid1 + 1 : 1;
  c_iadex_.iadnorc = colour ? 3 * g_ngrid1 + 1 : g_ngrid1 + 1;
}

void x2r_set_omega(double omega) {
  c_interface_45_.omegac = omega;
  c_interface_45_.omega1c = 1.0 - omega;
}

/* thread slices of every colour and of the boundary lists (initMesh:2242-2370) */
static void slices(int nthreads) {
  int icol_start[6];
  int j = 0;
  for (int col = 1; col <= 5; col++) { icol_start[col - 1] = j + 1; for (int i = col; i <= g_ngrid1; i += 5) j++; }
  icol_start[5] = g_ngrid1 + 1;
  for (int icol = 0; icol <= 4; icol++) {
    int start = icol_start[icol], stop = icol_start[icol + 1] - 1, step = (stop - start + 1) / nthreads;
    for (int t = 0; t < nthreads; t++) {
      int a, b;
      if (nthreads == 1) { a = start; b = stop; }
      else if (t + 1 == nthreads) { a = start + t * step; b = stop; }
      else { a = start + t * step; b = a + step - 1; }
      c_interface_9_.nstartc[icol + 5 * t] = a;
      c_interface_10_.nstopc[icol + 5 * t] = b;
    }
  }
  int n[3] = {g_n6a, g_n6b, g_n7};
  int *st[3] = {c_interface_11_.nstart6ac, c_interface_13_.nstart6bc, c_interface_15_.nstart7c};
  int *sp[3] = {c_interface_12_.nstop6ac, c_interface_14_.nstop6bc, c_interface_16_.nstop7c};
  for (int q = 0; q < 3; q++) {
    int step = n[q] / nthreads;
    for (int t = 0; t < nthreads; t++) {
      if (nthreads == 1) { st[q][t] = 1; sp[q][t] = n[q]; }
      else if (t + 1 == nthreads) { st[q][t] = 1 + t * step; sp[q][t] = n[q]; }
      else { st[q][t] = 1 + t * step; sp[q][t] = st[q][t] + step - 1; }
    }
  }
}

/* sorpt_ on one extended function: e = lhs, g = rhs (src/c/sorpt.c:11) */
void x2r_sorpt(int isym, double *uext, double *lhs, double *rhs) {
  struct sor_t p;
  memset(&p, 0, sizeof p);
  p.threadsNum = 1; p.threadNum = 0; p.isym = isym;
  p.indxex = &c_sorptr_.cw_sor[c_iadex_.iadextc - 1];
  p.indx = &c_sorptr_.cw_sor[c_iadex_.iadnorc - 1];
  p.indx6a = &c_sorptr_.cw_sor[c_iadex_.iadex1c - 1];
  p.indx6b = &c_sorptr_.cw_sor[c_iadex_.iadex2c - 1];
  p.indx7 = &c_sorptr_.cw_sor[c_iadex_.iadex3c - 1];
  p.e = lhs; p.g = rhs; p.uext = uext;
  c_interface_17_.isstartc = 1;
  c_interface_17_.isstopc = g_ngrid1;
  sorpt_((void *)&p);
}

/* mcsor_pthread_ with nthreads threads on the colour-reordered lists
 * (src/c/mcsor_pthread.c:32) */
void x2r_mcsor(int isym, int nthreads, double *uext, double *lhs, double *rhs) {
  if (nthreads < 1) nthreads = 1;
  if (nthreads > MAXTHREADS4MCSOR) nthreads = MAXTHREADS4MCSOR;
  slices(nthreads);
  x2r_use_colour_lists(1);
  mcsor_pthread_(&isym, &nthreads, uext, lhs, rhs);
}

/* Orbitals and potentials for coulExch_pthread_: cw_orb/cw_exch blocks and
 * the batch of orbital iorb (relaxPots.F90:137-142, initAddr:1456-1465). */
void x2r_set_functions(double *cw_orb, const int *i1b, int norb, double *cw_exch) {
  c_orbptr_.cw_orb = cw_orb;
  c_exchptr_.cw_exch = cw_exch;
  for (int i = 0; i < norb && i < MAXORB; i++) c_interface_7_.i1bc[i] = i1b[i];
}
void x2r_set_batch(int iorb, int npots, const int *ins1, const int *ins2, const int *ibexcp, const int *idel,
                   const int *isym) {
  for (int k = 0; k < npots; k++) {
    c_interface_1_.ins1[k][iorb - 1] = ins1[k];
    c_interface_2_.ins2[k][iorb - 1] = ins2[k];
    c_interface_3_.ibexcpc[k][iorb - 1] = ibexcp[k];
    c_interface_4_.deltam4potc[k][iorb - 1] = idel[k];
    c_interface_6_.isymsc[k][iorb - 1] = isym[k];
  }
  c_interface_8_.nexchpotsc[iorb - 1] = npots;
}
/* One potential k of orbital iorb's batch: relax_single_pot_pthread.c:15-110
 * (rhs = psi_in1 psi_in2 g, lhs = f3 + idel^2 e, maxsor1 x putinc_, sorpt_,
 * putoutc_) with its own, correctly sized sor_t. */
struct x2r_pot { int k, iorb; };
static void *x2r_relax_pot(void *arg) {
  const struct x2r_pot *a = (const struct x2r_pot *)arg;
  const int k = a->k, iorb = a->iorb;
  int nnu = c_interface_17_.nnu1c - 8, mxnmu = c_interface_17_.mxnmuc;
  const int mxsize = c_interface_17_.mxsizec, maxsor1 = c_interface_17_.maxsor1c;
  const int in1 = c_interface_1_.ins1[k][iorb - 1], in2 = c_interface_2_.ins2[k][iorb - 1];
  const int ib1 = c_interface_7_.i1bc[in1 - 1], ib2 = c_interface_7_.i1bc[in2 - 1];
  const int ibexc = c_interface_3_.ibexcpc[k][iorb - 1], idel = c_interface_4_.deltam4potc[k][iorb - 1];
  int isym = c_interface_6_.isymsc[k][iorb - 1];
  const double deltam2 = (double)idel * idel;
  double *psi = c_orbptr_.cw_orb, *excp = c_exchptr_.cw_exch;
  double *suppl = c_supplptr_.cw_suppl;
  const double *ef = &suppl[c_i4b_.i4barr[3] - 1], *f3 = &suppl[c_i4b_.i4barr[7] - 1];
  const double *gf = &suppl[c_i4b_.i4barr[9] - 1];
  struct sor_t p;
  memset(&p, 0, sizeof p);
  p.threadsNum = 1;
  p.threadNum = 0;
  p.indxex = &c_sorptr_.cw_sor[c_iadex_.iadextc - 1];
  p.indx = &c_sorptr_.cw_sor[c_iadex_.iadnorc - 1];
  p.indx6a = &c_sorptr_.cw_sor[c_iadex_.iadex1c - 1];
  p.indx6b = &c_sorptr_.cw_sor[c_iadex_.iadex2c - 1];
  p.indx7 = &c_sorptr_.cw_sor[c_iadex_.iadex3c - 1];
  p.b = &suppl[c_i4b_.i4barr[1] - 1];
  p.d = &suppl[c_i4b_.i4barr[2] - 1];
  p.isym = isym;
  double *lhs = (double *)malloc(mxsize * sizeof(double));
  double *rhs = (double *)malloc(mxsize * sizeof(double));
  double *wk2 = (double *)malloc((size_t)(nnu + 8) * (mxnmu + 8) * sizeof(double));
  for (int i = 0; i < mxsize; i++) rhs[i] = psi[ib1 + i - 1] * psi[ib2 + i - 1] * gf[i];
  if (deltam2 == 0.0)
    for (int i = 0; i < mxsize; i++) lhs[i] = f3[i];
  else
    for (int i = 0; i < mxsize; i++) lhs[i] = f3[i] + ef[i] * deltam2;
  p.g = rhs;
  p.e = lhs;
  for (int it = 1; it <= maxsor1; it++) {
    putinc_(&nnu, &mxnmu, &isym, &excp[ibexc - 1], wk2);
    p.uext = wk2;
    sorpt_((void *)&p);
    putoutc_(&nnu, &mxnmu, &excp[ibexc - 1], wk2);
  }
  free(lhs);
  free(rhs);
  free(wk2);
  return NULL;
}

/* coulExch_pthread.c:19-125: every potential of orbital iorb's batch, one
 * thread each (a single potential runs on the calling thread). */
void x2r_coulexch(int iorb) {
  c_interface_46_.iorbc = iorb;
  c_interface_17_.isstartc = 1;
  c_interface_17_.isstopc = g_ngrid1;
  const int n = c_interface_8_.nexchpotsc[iorb - 1];
  if (n <= 0) return;
  struct x2r_pot *args = (struct x2r_pot *)malloc(sizeof(struct x2r_pot) * n);
  pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * n);
  for (int k = 0; k < n; k++) {
    args[k].k = k;
    args[k].iorb = iorb;
  }
  if (n == 1) {
    x2r_relax_pot(&args[0]);
  } else {
    for (int k = 0; k < n; k++) pthread_create(&th[k], NULL, x2r_relax_pot, &args[k]);
    for (int k = 0; k < n; k++) pthread_join(th[k], NULL);
  }
  free(args);
  free(th);
}
