/*
 * x2dhf CPU oracle -- TEST INFRASTRUCTURE ONLY (see x2dhf_oracle.h).
 *
 * Plain-C restatement of the reference's closed-shell HF path:
 *   grid / operator setup      src/initCBAllocArrays.F90
 *   hydrogenic start           src/initOrbitalsPotentials.F90, src/coulombExchangePotentials.f90
 *   (MC)SOR sweeps             src/sormcsor.F90
 *   ghost embedding            src/inout.F90
 *   orbital / potential relax  src/relaxOrbs.F90, src/relaxPots.F90
 *   Fock potential             src/fock.F90
 *   quadratures                src/normOrtho.F90, src/integrals.F90,
 *                              src/lagrangeMultipliers.F90, src/totalEnergy.F90
 *   multipole asymptotics      src/scfUtils.F90
 *   SCF driver                 src/doSCF.F90
 * Arithmetic follows the reference's expression order (no FMA contraction:
 * build with -ffp-contract=off).  Sums are plain left-to-right loops as in the
 * reference's internal BLAS (src/blas.F90:16-26).
 */
#include "x2dhf_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <ctype.h>

#define MAXORB X2O_MAXORB
#define MAXMPOLE X2O_MAXMPOLE
#define PII 3.14159265358979323846264338327950
#define PRECIS 2.220446049250313080847263336181640625e-16 /* epsilon(1d0) */

typedef struct {
  int iscf, iorb;
  double ee, dee, dnorm;
} rec_t;

struct x2o_state {
  /* ---------------- input ---------------- */
  char title[96];
  double z1, z2, r, r2;
  int norb;
  int m[MAXORB + 1];         /* mgx(3,i)=mgx(6,i): |lambda| */
  char bond[MAXORB + 1][8];  /* sigma pi delta phi */
  char gusym[MAXORB + 1];    /* 'g' 'u' ' ' */
  double occ[MAXORB + 1];
  int n1[MAXORB + 1], l1[MAXORB + 1], n2[MAXORB + 1], l2[MAXORB + 1];
  double co1[MAXORB + 1], co2[MAXORB + 1], eza1[MAXORB + 1], eza2[MAXORB + 1];
  int inhyd[MAXORB + 1];
  int nni, nmu;
  double rgrid;
  int maxscf, saveScfData, ienterm, inoterm, verboseLevel;
  int nscf2skip, nenlast, nnolast, maxresets, nscfExtra;
  int ienterm4init, lfixorb4init, lfixorb, lfixexch;
  int ifixorb[MAXORB + 1];
  int lorbmcsor, lpotmcsor, altSweeps, lomegaz;
  double ovforb, ovfcoul, ovfexch;
  int mpole;
  double recalcMMfactor, orbEnergyIncThld;
  int lhomonucl, lbreakCi;
  int maxsororb[2], maxsorpot[2];
  int hydrogen_start, old_start;
  int batch_pots; /* 1: all potentials of an iteration from its starting orbitals; 2: and then all orbitals
                     from the state after the potentials (no reference counterpart) */

  /* ---------------- grid ---------------- */
  int mxnmu, mxsize, nni8, mxsize8;
  double hni, hmu, rinf;
  double *vmu, *vxi, *vxisq, *vxi1, *vxi2; /* 1..mxnmu */
  double *vni, *veta, *vetasq, *veta1, *veta2; /* 1..nni */
  double *wmu, *wni;
  double dmu1[4], dmu2[4], dni1[4], dni2[4], exeven[5];
  double *dmu9, *dni9; /* (9,mxnmu) (9,nni) */
  double diag;
  double *sup[14]; /* borb bpot d e f0 f1 f2 f3 f4 g wjac1 wjac2 wgt1 wgt2 */
  double *leg[MAXMPOLE];
  int ngrid1, ngrid6a, ngrid6b, ngrid7;
  int *indx1, *indx2, *indx6a, *indx6b, *indx7;
  int nni1, nni2, nni3, nni4, nni5;

  /* ---------------- orbitals, potentials ---------------- */
  int mm[MAXORB + 1], isymOrb[MAXORB + 1], ihomo[MAXORB + 1], ige[MAXORB + 1];
  int iorn[MAXORB + 1], lock[MAXORB + 1], iloop[MAXORB + 1], iqm[4 * MAXORB + 1];
  char spin[4 * MAXORB + 1];
  double *orbblock, *potblock; /* contiguous storage (reference orbptr / exchptr) */
  void (*pot_hook)(void *, int);
  void (*orb_hook)(void *, int, int, double *, double *, double *);
  void *hook_ud;
  double **psi;  /* [1..norb] plain */
  double **coul; /* [1..norb] plain Coulomb potential (exchptr(i2b)) */
  /* exchange potential storage by pair index k=k2(i,j), two slots each */
  double **exch; /* [k*2+slot] */
  int k2[MAXORB + 1][MAXORB + 1], ilc2[MAXORB + 1][MAXORB + 1];
  int ilc[MAXORB * (MAXORB + 1) / 2 + 2];
  int nexchpots[MAXORB + 1];
  int ins1[MAXORB + 1][2 * MAXORB + 2], ins2[MAXORB + 1][2 * MAXORB + 2];
  int deltam4pot[MAXORB + 1][2 * MAXORB + 2], isyms[MAXORB + 1][2 * MAXORB + 2];
  double *pottarget[MAXORB + 1][2 * MAXORB + 2];
  double gec[2 * MAXORB * MAXORB + 1];
  int offDiagLM[MAXORB + 1][MAXORB + 1], loffDiagLM;
  int nexchmm, iorb1mm[MAXORB * MAXORB + 1], iorb2mm[MAXORB * MAXORB + 1];
  int idelmm[MAXORB * MAXORB + 1], ipcmm[MAXORB * MAXORB + 1];
  double ee[MAXORB + 1][MAXORB + 1];
  double cmulti[MAXMPOLE * MAXORB + 1];
  double excm[MAXMPOLE][MAXORB * (MAXORB + 1) + 2]; /* excdi..exc8 by ipc */
  double **coulombptr, **exchangeptr;
  double orbNorm[MAXORB + 1], wstorthog[MAXORB + 1], vk[MAXORB + 1], vn[MAXORB + 1];
  int itouch[MAXORB + 1];
  int isstart, isstop, isstep;
  long nsor4orb, nsor4pot;
  double etot, evt, vkt, vnt, virrat;
  int nel;

  /* scratch */
  double *w[8];

  /* SCF control (doSCF.F90:211-886 locals kept across calls) */
  int scf_started, scf_done, iscf;
  double eeOld[MAXORB + 1], deltaee[MAXORB + 1], deltaNorm[MAXORB + 1], demax1;
  double deltaeeMax, deltaNormMax, eeconv, eeconvprev, dnmaxprev;
  double orbEnergyThld, orbNormThld, thren4init;
  int nresets, nresets4no, nOrbEnergyThld, nOrbNormThld, noenergydec, nonormdec;
  int lenergyThld, lnormThld, lmpoleInit, ldemax0;
  /* records */
  rec_t *rec;
  int nrec, caprec;
  int verbose;
};

/* ======================================================================== */
/* small utilities (src/utils.f90)                                         */
/* ======================================================================== */

/* factor: src/utils.f90:230-241 */
static double factor(int n) {
  double f = 1.0;
  for (int i = 1; i <= n; i++) f = (double)i * f;
  return f;
}

/* hypg1f1: src/utils.f90:265-282 */
static double hypg1f1(int np, int lp, double x) {
  double h = 1.0, t;
  if (-np == 0) return h;
  t = (double)np * x / (double)lp;
  h = h + t;
  if (-np == 1) return h;
  for (int i = 2; i <= -np; i++) {
    t = t * x * (double)(np + i - 1) / (double)(lp + i - 1) / (double)i;
    h = h + t;
  }
  return h;
}

/* hypg2f1: src/utils.f90:289-309 */
static double hypg2f1(int na, int nb, int nc, double x) {
  double h = 1.0, a, b, c, t;
  if (na == 0) return h;
  a = (double)na; b = (double)nb; c = (double)nc;
  t = a * b * x / c;
  h = h + t;
  if (-na == 1) return h;
  for (int i = 2; i <= -na; i++) {
    t = t * x * (a + (double)(i - 1)) * (b + (double)(i - 1)) / (c + (double)(i - 1)) / (double)i;
    h = h + t;
  }
  return h;
}

/* plegendg: src/utils.f90:315-335.  Note the reference writes (-one**m),
 * which Fortran evaluates as -(1**m) = -1. */
static double plegendg(int l, int m, double costh) {
  double ct = fabs(1.0 - costh * costh);
  if (m == 0) return hypg2f1(-l, l + 1, 1, (1.0 - costh) / 2.0);
  if (ct < PRECIS) return 0.0;
  double fn0 = (-pow(1.0, (double)m)) * factor(l + m) / factor(l - m) / factor(m) / pow(2.0, (double)m);
  double ct1 = fn0 * pow(ct, (double)m / 2.0);
  return hypg2f1(m - l, m + l + 1, m + 1, (1.0 - costh) / 2.0) * ct1;
}

static double ddot(int n, const double *x, const double *y) {
  double s = 0.0;
  for (int i = 0; i < n; i++) s = s + x[i] * y[i];
  return s;
}

/* ======================================================================== */
/* input (src/inputInterface.F90)                                          */
/* ======================================================================== */

typedef struct {
  char **tok;
  int ntok, pos;
} card_t;

static void card_free(card_t *c) {
  for (int i = 0; i < c->ntok; i++) free(c->tok[i]);
  free(c->tok);
  c->tok = NULL; c->ntok = 0; c->pos = 0;
}

/* split one input line into lower-case tokens; '!' starts a comment */
static void card_split(const char *line, card_t *c) {
  card_free(c);
  int cap = 16;
  c->tok = (char **)malloc(sizeof(char *) * cap);
  const char *p = line;
  while (*p) {
    while (*p && (isspace((unsigned char)*p) || *p == ',')) p++;
    if (!*p || *p == '!') break;
    const char *q = p;
    while (*q && !isspace((unsigned char)*q) && *q != ',' && *q != '!') q++;
    int n = (int)(q - p);
    char *t = (char *)malloc(n + 1);
    for (int i = 0; i < n; i++) t[i] = (char)tolower((unsigned char)p[i]);
    t[n] = 0;
    if (c->ntok == cap) { cap *= 2; c->tok = (char **)realloc(c->tok, sizeof(char *) * cap); }
    c->tok[c->ntok++] = t;
    p = q;
  }
  c->pos = 0;
}

static int tok_int(card_t *c, int *v) {
  if (c->pos >= c->ntok) return 0;
  char *e;
  long x = strtol(c->tok[c->pos], &e, 10);
  if (*e) return 0;
  *v = (int)x; c->pos++;
  return 1;
}
static int tok_float(card_t *c, double *v) {
  if (c->pos >= c->ntok) return 0;
  char buf[64]; strncpy(buf, c->tok[c->pos], 63); buf[63] = 0;
  for (char *q = buf; *q; q++) if (*q == 'd') *q = 'e';
  char *e;
  double x = strtod(buf, &e);
  if (*e) return 0;
  *v = x; c->pos++;
  return 1;
}
static const char *tok_str(card_t *c) {
  if (c->pos >= c->ntok) return "";
  return c->tok[c->pos++];
}

/* nnucalc / nmucalc grid rounding: src/inputInterface.F90:2961-3095.
 * The mesh-ordering test there is always true, so n = 1 (mod 6) and
 * n - 6 = 0 (mod 5) are enforced alternately until both hold. */
static int round_grid(int n) {
  for (;;) {
    while ((n - 1) % 6 != 0) n--;
    int ntemp = n;
    while (((n - 6) / 5) * 5 != n - 6) n--;
    if (n > 1 && n != ntemp) continue;
    return n;
  }
}

static void set_defaults(x2o_state *s) {
  /* src/initVariables.F90:13-364 (HF subset) */
  s->lomegaz = 1;
  s->mpole = 4;
  s->maxscf = 1000; s->saveScfData = 20; s->ienterm = 10; s->inoterm = 10; s->verboseLevel = 2;
  s->ienterm4init = 1; s->lfixorb4init = 0; s->lfixorb = 0; s->lfixexch = 0;
  s->maxsororb[0] = 1; s->maxsororb[1] = 10; s->maxsorpot[0] = 1; s->maxsorpot[1] = 10;
  s->ovforb = -1.0; s->ovfcoul = -1.0; s->ovfexch = -1.0;
  s->nscf2skip = 600; s->nenlast = 20; s->nnolast = 20; s->maxresets = 5; s->nscfExtra = 3;
  s->recalcMMfactor = 1.150; s->orbEnergyIncThld = 1.0e4;
  for (int i = 0; i <= MAXORB; i++) { s->gusym[i] = ' '; }
  for (int i = 0; i <= 4 * MAXORB; i++) s->spin[i] = ' ';
}

x2o_state *x2o_from_input(const char *text, char *err, int errlen) {
  x2o_state *s = (x2o_state *)calloc(1, sizeof(x2o_state));
  set_defaults(s);
  card_t c = {0};
  const char *p = text;
  char line[512];
  int have_grid = 0, have_lcao = 0, grid_nmu = 0;
  double grid_rinf = 0.0;
  int grid_nnu_raw = 0;
  /* read lines */
  char **lines = NULL; int nl = 0, capl = 0;
  while (*p) {
    const char *q = strchr(p, '\n');
    int n = q ? (int)(q - p) : (int)strlen(p);
    if (n > 511) n = 511;
    memcpy(line, p, n); line[n] = 0;
    if (nl == capl) { capl = capl ? 2 * capl : 64; lines = (char **)realloc(lines, sizeof(char *) * capl); }
    lines[nl++] = strdup(line);
    p = q ? q + 1 : p + strlen(p);
  }
  int li = 0;
#define NEXTCARD() do { while (li < nl) { card_split(lines[li++], &c); if (c.ntok) break; } } while (0)
  int ok = 1;
  while (li < nl && ok) {
    NEXTCARD();
    if (!c.ntok) break;
    const char *lab = tok_str(&c);
    char label[9]; strncpy(label, lab, 8); label[8] = 0;
    if (!strcmp(label, "title")) {
      strncpy(s->title, lines[li - 1], 95);
    } else if (!strcmp(label, "method")) {
      const char *mth = tok_str(&c);
      if (strcmp(mth, "hf")) { snprintf(err, errlen, "only method hf is supported"); ok = 0; }
    } else if (!strcmp(label, "nuclei")) {
      tok_float(&c, &s->z1); tok_float(&c, &s->z2); tok_float(&c, &s->r);
      const char *u = tok_str(&c);
      if (!strcmp(u, "angstrom")) s->r = s->r / 0.52917721067121204;
      s->r2 = s->r / 2.0;
    } else if (!strcmp(label, "config")) {
      /* src/inputInterface.F90:862-1077 (closed and '+-.' spin shells) */
      int itotq = 0; tok_int(&c, &itotq);
      int isum = 0;
      for (;;) {
        NEXTCARD();
        int nbsym = 0;
        if (!tok_int(&c, &nbsym)) { snprintf(err, errlen, "bad config card"); ok = 0; break; }
        const char *sym = tok_str(&c);
        int mt = -1;
        if (!strcmp(sym, "sigma")) mt = 0; else if (!strcmp(sym, "pi")) mt = 1;
        else if (!strcmp(sym, "delta")) mt = 2; else if (!strcmp(sym, "phi")) mt = 3;
        if (mt < 0) { snprintf(err, errlen, "bad symmetry %s", sym); ok = 0; break; }
        int isum0 = isum;
        for (int i = 0; i < nbsym; i++) {
          isum++;
          s->m[isum] = mt;
          strcpy(s->bond[isum], sym);
          s->gusym[isum] = ' ';
        }
        const char *t = tok_str(&c);
        if (!strcmp(t, "g") || !strcmp(t, "u")) {
          s->lhomonucl = 1;
          for (int i = isum0 + 1; i <= isum; i++) s->gusym[i] = t[0];
          t = tok_str(&c);
        }
        double cloe = (mt == 0) ? 2.0 : 4.0;
        int iput = 4 * (isum - 1);
        int k = 0;
        char sp[4] = {' ', ' ', ' ', ' '};
        while (strcmp(t, "end") && t[0] && k < 4) { sp[k++] = t[0]; t = tok_str(&c); }
        if (sp[0] != '+' && sp[0] != '-' && sp[0] != '.') {
          for (int i = isum0 + 1; i <= isum; i++) s->occ[i] = cloe;
        } else {
          for (int i = 0; i < 4; i++) {
            s->spin[1 + i + iput] = sp[i];
            if (sp[i] == '+' || sp[i] == '-') {
              for (int j = isum0 + 1; j <= isum; j++) {
                s->occ[j] += 1.0;
                s->spin[1 + i + 4 * (j - 1)] = sp[i];
              }
            }
          }
        }
        if (!strcmp(t, "end")) break;
      }
      s->norb = isum;
      for (int i = 1; i <= s->norb; i++) {
        s->ifixorb[i] = 0; s->inhyd[i] = 1;
        s->co1[i] = (s->z1 > PRECIS) ? 1.0 : 0.0;
        s->co2[i] = (s->z2 > PRECIS) ? 1.0 : 0.0;
        double clo = (s->m[i] == 0) ? 2.0 : 4.0;
        s->lock[i] = (fabs(s->occ[i] / clo - 1.0) > 1e-6) ? 1 : 0;
      }
    } else if (!strcmp(label, "grid")) {
      /* src/inputInterface.F90:1491-1556 */
      tok_int(&c, &grid_nnu_raw);
      double t1 = 0, t2 = 0;
      tok_float(&c, &t1); tok_float(&c, &t2);
      if (fabs(t2) > PRECIS) { grid_nmu = (int)lround(t1); grid_rinf = t2; }
      else { grid_nmu = 0; grid_rinf = t1; }
      have_grid = 1;
    } else if (!strcmp(label, "orbpot")) {
      /* src/inputInterface.F90:2257-2360 */
      const char *src = tok_str(&c);
      if (!strcmp(src, "old")) {
        /* linitFuncsOld (:2311-2313): functions, Lagrange multipliers and
         * moments come from a checkpoint (readFromDisk), no frozen start;
         * the caller loads them with x2o_set_orbital/x2o_set_pot/
         * x2o_set_orbital_energy after x2o_setup */
        s->hydrogen_start = 0;
        s->old_start = 1;
        s->lfixorb4init = 0; s->lfixorb = 0;
        for (int i = 1; i <= s->norb; i++) s->ifixorb[i] = 0;
        continue;
      }
      if (strcmp(src, "hydrogen")) { snprintf(err, errlen, "only orbpot hydrogen and old are supported"); ok = 0; break; }
      int itmp;
      if (tok_int(&c, &itmp)) s->ienterm4init = itmp;
      if (s->ienterm4init > 0) {
        s->lfixorb4init = 1; s->lfixorb = 1;
        for (int i = 1; i <= s->norb; i++) s->ifixorb[i] = 1;
      }
      s->hydrogen_start = 1;
      if (s->ienterm4init == 0) {
        s->lfixorb4init = 0; s->lfixorb = 0;
        for (int i = 1; i <= s->norb; i++) s->ifixorb[i] = 0;
      }
    } else if (!strcmp(label, "lcao")) {
      /* src/inputInterface.F90:1749-1881 */
      int inclorb = 1, itmp;
      if (tok_int(&c, &itmp)) inclorb = itmp;
      for (int i = 1; i <= s->norb; i++) {
        NEXTCARD();
        tok_float(&c, &s->co1[i]); tok_int(&c, &s->n1[i]); tok_int(&c, &s->l1[i]); tok_float(&c, &s->eza1[i]);
        tok_float(&c, &s->co2[i]); tok_int(&c, &s->n2[i]); tok_int(&c, &s->l2[i]); tok_float(&c, &s->eza2[i]);
        if (inclorb == 2) { s->eza1[i] = s->z1 - s->eza1[i]; s->eza2[i] = s->z2 - s->eza2[i]; }
        int ih;
        if (tok_int(&c, &ih)) s->inhyd[i] = ih; else s->inhyd[i] = 1;
      }
      for (int i = 1; i <= s->norb; i++) {
        double co12 = fabs(s->co1[i]) + fabs(s->co2[i]);
        if (fabs(co12) > PRECIS) { s->co1[i] = s->co1[i] / co12; s->co2[i] = s->co2[i] / co12; }
      }
      have_lcao = 1;
    } else if (!strcmp(label, "scf")) {
      int v;
      if (tok_int(&c, &v)) { s->maxscf = v;
        if (tok_int(&c, &v)) { s->saveScfData = v;
          if (tok_int(&c, &v)) { s->ienterm = v;
            if (tok_int(&c, &v)) { s->inoterm = v;
              if (tok_int(&c, &v)) s->verboseLevel = v; } } } }
    } else if (!strcmp(label, "conv")) {
      int v;
      if (tok_int(&c, &v)) { s->nscf2skip = v;
        if (tok_int(&c, &v)) { s->nenlast = v;
          if (tok_int(&c, &v)) s->nnolast = v; } }
    } else if (!strcmp(label, "mcsor")) {
      int v;
      s->lorbmcsor = 1; s->lpotmcsor = 0;
      if (tok_int(&c, &v)) { /* nthreads: irrelevant to single-thread order */ }
      if (tok_int(&c, &v)) { s->maxsororb[1] = v; if (tok_int(&c, &v)) s->maxsorpot[1] = v; }
    } else if (!strcmp(label, "mcsor-o")) {
      int v; s->lorbmcsor = 1;
      if (tok_int(&c, &v) && tok_int(&c, &v)) { s->maxsororb[1] = v; if (tok_int(&c, &v)) s->maxsororb[0] = v; }
    } else if (!strcmp(label, "mcsor-ce")) {
      int v; s->lpotmcsor = 1;
      if (tok_int(&c, &v) && tok_int(&c, &v)) { s->maxsorpot[1] = v; if (tok_int(&c, &v)) s->maxsorpot[0] = v; }
    } else if (!strcmp(label, "omega")) {
      double a = 0, b = 0; tok_float(&c, &a); tok_float(&c, &b);
      if (fabs(a) > PRECIS) s->ovforb = a;
      if (fabs(b) > PRECIS) s->ovfcoul = b;
      s->ovfexch = s->ovfcoul;
    } else if (!strcmp(label, "multipol")) {
      double f = 0; tok_float(&c, &f);
      s->recalcMMfactor = (f < PRECIS) ? 1e15 : f;
      int v; if (tok_int(&c, &v)) s->mpole = v;
    } else if (!strcmp(label, "altsweep")) {
      s->altSweeps = 1;
    } else if (!strcmp(label, "break")) {
      s->lbreakCi = 1;
    } else if (!strcmp(label, "sor4orb")) {
      int v; if (tok_int(&c, &v)) { s->maxsororb[1] = v; if (tok_int(&c, &v)) s->maxsororb[0] = v; }
    } else if (!strcmp(label, "sor4pot")) {
      int v; if (tok_int(&c, &v)) { s->maxsorpot[1] = v; if (tok_int(&c, &v)) s->maxsorpot[0] = v; }
    } else if (!strcmp(label, "stop")) {
      break;
    } else {
      /* cards with no effect on the closed-shell HF path (mmoments, print, ...) */
    }
  }
  card_free(&c);
  for (int i = 0; i < nl; i++) free(lines[i]);
  free(lines);
  if (ok && (!have_grid || s->norb < 1 || s->r <= 0)) { snprintf(err, errlen, "incomplete input"); ok = 0; }
  if (ok && s->hydrogen_start && !have_lcao) { snprintf(err, errlen, "lcao card missing"); ok = 0; }
  if (!ok) { free(s); return NULL; }
  /* grid rounding (read_grid): nnu first, then nmu from R_inf if absent */
  s->nni = round_grid(grid_nnu_raw);
  s->rgrid = grid_rinf;
  if (grid_nmu > 0) {
    s->nmu = round_grid(grid_nmu);
  } else {
    double hnu = PII / (double)(s->nni - 1);
    double xmi0 = 2.0 * s->rgrid / s->r;
    xmi0 = log(xmi0 + sqrt(xmi0 * xmi0 - 1.0));
    int n = (int)lround(xmi0 / hnu + 1.0);
    s->nmu = round_grid(n);
  }
  for (int i = 1; i <= s->norb; i++) {
    /* read_stop normalises the mixing coefficients again */
    double co12 = fabs(s->co1[i]) + fabs(s->co2[i]);
    if (fabs(co12) > PRECIS) { s->co1[i] = s->co1[i] / co12; s->co2[i] = s->co2[i] / co12; }
  }
  return s;
}

/* ======================================================================== */
/* setup (src/initCBAllocArrays.F90)                                       */
/* ======================================================================== */

static double *dalloc(long n) { return (double *)calloc((size_t)n, sizeof(double)); }

/* setOmega: src/initCBAllocArrays.F90:636-650 */
static double set_omega(const x2o_state *s) {
  double rho = 0.5 * (cos(PII / (double)s->mxnmu) + cos(PII / (double)s->nni));
  return 2.0 * 0.603 / (1.0 + sqrt(1.0 - rho * rho)) + 0.79;
}

/* initCBlocks: src/initCBAllocArrays.F90:726-1070 */
static void init_cblocks(x2o_state *s) {
  int nni = s->nni;
  s->mxnmu = s->nmu;
  s->mxsize = nni * s->mxnmu;
  s->nel = 0;
  for (int i = 1; i <= s->norb; i++) {
    s->mm[i] = s->m[i];
    int iocc = (int)lround(s->occ[i] + 0.000001);
    s->nel += iocc;
    s->isymOrb[i] = (s->m[i] % 2 == 0) ? 1 : -1;
  }
  if (s->mm[1] == 2 && s->mpole < 4) s->mpole = 4;
  if (s->mm[1] == 3 && s->mpole <= 4) s->mpole = 8;
  s->hni = PII / (double)(nni - 1);
  double xmi0 = 2.0 * s->rgrid / s->r;
  xmi0 = log(xmi0 + sqrt(xmi0 * xmi0 - 1.0));
  s->hmu = xmi0 / (double)(s->mxnmu - 1);
  int nm = s->mxnmu;
  s->vmu = dalloc(nm + 1); s->vxi = dalloc(nm + 1); s->vxisq = dalloc(nm + 1);
  s->vxi1 = dalloc(nm + 1); s->vxi2 = dalloc(nm + 1);
  s->vmu[1] = 0.0; s->vxi[1] = cosh(s->vmu[1]); s->vxisq[1] = s->vxi[1] * s->vxi[1];
  s->vxi1[1] = sqrt(s->vxi[1] * s->vxi[1] - 1.0); s->vxi2[1] = 0.0;
  for (int i = 2; i <= nm; i++) {
    s->vmu[i] = s->vmu[i - 1] + s->hmu;
    s->vxi[i] = cosh(s->vmu[i]);
    s->vxisq[i] = s->vxi[i] * s->vxi[i];
    s->vxi1[i] = sqrt(s->vxi[i] * s->vxi[i] - 1.0);
    s->vxi2[i] = s->vxi[i] / s->vxi1[i];
  }
  s->vni = dalloc(nni + 1); s->veta = dalloc(nni + 1); s->vetasq = dalloc(nni + 1);
  s->veta1 = dalloc(nni + 1); s->veta2 = dalloc(nni + 1);
  for (int i = 1; i <= nni; i++) {
    s->vni[i] = (double)(i - 1) * s->hni;
    s->veta[i] = cos(s->vni[i]);
    s->vetasq[i] = s->veta[i] * s->veta[i];
    s->veta1[i] = sqrt(1.0 - s->veta[i] * s->veta[i]);
    s->veta2[i] = (s->veta1[i] < PRECIS) ? 0.0 : s->veta[i] / s->veta1[i];
  }
  s->rinf = s->r * s->vxi[nm] / 2.0;
  if (s->lbreakCi) for (int i = 1; i <= s->norb; i++) s->gusym[i] = ' ';
  /* numbering within symmetry (orbitals listed in reverse) */
  int cnt[4][3] = {{0}};
  for (int ibo = 1; ibo <= s->norb; ibo++) {
    int iba = s->norb + 1 - ibo;
    int g = (s->gusym[iba] == 'u') ? 1 : 0;
    s->iorn[iba] = ++cnt[s->m[iba]][g];
  }
  for (int i = 1; i <= s->norb; i++) {
    s->ihomo[i] = 1;
    if (s->gusym[i] == 'u' && s->m[i] == 0) s->ihomo[i] = -1;
    if (s->gusym[i] == 'u' && s->m[i] == 2) s->ihomo[i] = -1;
    if (s->gusym[i] == 'g' && s->m[i] == 1) s->ihomo[i] = -1;
    if (s->gusym[i] == 'g' && s->m[i] == 3) s->ihomo[i] = -1;
    s->ige[i] = (s->gusym[i] == 'u') ? 1 : 2;
  }
  if (s->ovfcoul < 0.0) { s->ovfcoul = set_omega(s); s->ovfexch = s->ovfcoul; }
  if (s->ovforb < 0.0) {
    double ovf = set_omega(s);
    s->ovforb = (ovf - 1.0) * ovf;
    if (s->lomegaz) s->ovforb = s->ovforb - 0.001 * (s->z1 > s->z2 ? s->z1 : s->z2);
  }
}

/* initAddr: src/initCBAllocArrays.F90:1147-1466 (lfastexch, lcoulexch) */
static void init_addr(x2o_state *s) {
  int norb = s->norb, mx = s->mxsize;
  s->psi = (double **)calloc(norb + 1, sizeof(double *));
  s->coul = (double **)calloc(norb + 1, sizeof(double *));
  s->coulombptr = (double **)calloc(norb + 1, sizeof(double *));
  s->exchangeptr = (double **)calloc(norb + 1, sizeof(double *));
  int nk = norb * (norb + 1) / 2 + 1;
  /* one block per kind, like the reference's orbptr / exchptr */
  s->orbblock = dalloc((long)norb * mx);
  s->potblock = dalloc((long)(norb + 2 * nk + 2) * mx);
  for (int i = 1; i <= norb; i++) {
    s->psi[i] = s->orbblock + (long)(i - 1) * mx;
    s->coul[i] = s->potblock + (long)(i - 1) * mx;
    s->coulombptr[i] = dalloc(mx); s->exchangeptr[i] = dalloc(mx);
  }
  s->exch = (double **)calloc(2 * nk + 2, sizeof(double *));
  for (int i1 = 1; i1 <= norb; i1++)
    for (int i2 = i1; i2 <= norb; i2++) {
      int k = i1 + i2 * (i2 - 1) / 2;
      s->ilc[k] = 0; s->ilc2[i1][i2] = 0; s->ilc2[i2][i1] = 0;
      if (i1 == i2 && s->m[i1] == 0) continue;
      s->ilc[k] = 1; s->ilc2[i1][i2] = 1; s->ilc2[i2][i1] = 1;
      s->k2[i1][i2] = k; s->k2[i2][i1] = k;
      s->exch[2 * k] = s->potblock + (long)(norb + 2 * k) * mx;
      s->exch[2 * k + 1] = s->potblock + (long)(norb + 2 * k + 1) * mx;
      if (i1 == i2) continue;
      if (s->m[i1] == 0 || s->m[i2] == 0) continue;
      s->ilc[k] = 2; s->ilc2[i1][i2] = 2; s->ilc2[i2][i1] = 2;
    }
  for (int iorb = 1; iorb <= norb; iorb++) {
    int n = 0;
    for (int iorb1 = iorb; iorb1 <= norb; iorb1++) {
      if (iorb == iorb1 && s->m[iorb] == 0) continue;
      if (iorb == iorb1 && s->ilc2[iorb][iorb] == 0) continue;
      n++;
      int in1 = (iorb < iorb1) ? iorb : iorb1, in2 = (iorb < iorb1) ? iorb1 : iorb;
      s->ins1[iorb][n] = in1; s->ins2[iorb][n] = in2;
      int idel = abs(s->m[in1] - s->m[in2]);
      if (in1 == in2) idel = 2 * s->m[in1];
      s->deltam4pot[iorb][n] = idel;
      s->isyms[iorb][n] = (idel % 2 == 0) ? 1 : -1;
      int ipc = in1 + in2 * (in2 - 1) / 2;
      s->pottarget[iorb][n] = s->exch[2 * ipc];
      if (s->ilc2[in1][in2] == 2) {
        n++;
        s->deltam4pot[iorb][n] = s->m[in1] + s->m[in2];
        s->ins1[iorb][n] = in1; s->ins2[iorb][n] = in2;
        s->pottarget[iorb][n] = s->exch[2 * ipc + 1];
        idel = s->deltam4pot[iorb][n];
        s->isyms[iorb][n] = (idel % 2 == 0) ? 1 : -1;
      }
    }
    /* lcoulexch: the Coulomb potential closes the batch */
    n++;
    s->ins1[iorb][n] = iorb; s->ins2[iorb][n] = iorb;
    s->deltam4pot[iorb][n] = 0; s->isyms[iorb][n] = 1;
    s->pottarget[iorb][n] = s->coul[iorb];
    s->nexchpots[iorb] = n;
  }
}

/* initSuppl: src/initCBAllocArrays.F90:1636-2051 (Coulomb nuclei) */
static void init_suppl(x2o_state *s) {
  int nni = s->nni, nm = s->mxnmu, mx = s->mxsize;
  double r = s->r;
  for (int k = 0; k < 14; k++) s->sup[k] = dalloc(mx);
  double *borb = s->sup[0], *bpot = s->sup[1], *d = s->sup[2], *e = s->sup[3], *f0 = s->sup[4],
         *f1 = s->sup[5], *f2 = s->sup[6], *f3 = s->sup[7], *f4 = s->sup[8], *g = s->sup[9],
         *wjac1 = s->sup[10], *wjac2 = s->sup[11], *wgt1 = s->sup[12], *wgt2 = s->sup[13];
  double wj1 = -r * PII / 2.0, wj2 = r * r * PII / 2.0, xrr = 0.5 * r;
  s->diag = -14350.0 / (5040.0) * (1.0 / (s->hmu * s->hmu) + 1.0 / (s->hni * s->hni));
  for (int i = 1; i <= nm; i++) {
    double w1 = s->vxi1[i], w2 = s->vxi[i] * s->vxi[i], w9 = xrr * s->vxi[i], w4 = s->vxi2[i], w5, w6;
    if (i == 1) { w5 = 0.0; w6 = 0.0; }
    else { w5 = s->vxi[i] / s->vxi1[i] - 2.0 * s->vxi1[i] / s->vxi[i]; w6 = 1.0 / (s->vxi1[i] * s->vxi1[i]); }
    double w8 = -r * r * r * PII * s->vxi[i] / 2.0;
    for (int j = 1; j <= nni; j++) {
      int ij = (i - 1) * nni + (j - 1);
      double w10 = s->veta1[j];
      borb[ij] = w4; bpot[ij] = w5; d[ij] = s->veta2[j];
      e[ij] = (w10 < PRECIS) ? 0.0 : (-w6 - 1.0 / (w10 * w10));
      double w7 = w2 - s->veta[j] * s->veta[j];
      f1[ij] = r * r * w7 / 2.0;
      f0[ij] = r * (s->vxi[i] * (s->z1 + s->z2) + s->veta[j] * (s->z2 - s->z1));
      f2[ij] = (i == 1) ? 0.0 : -r * w7 / s->vxi[i];
      f3[ij] = -2.0 / w2 + s->diag;
      g[ij] = w8 * w7;
      f4[ij] = w9;
      wjac1[ij] = wj1 * w1 * w10;
      wjac2[ij] = wj2 * w1 * w10 * (w1 * w1 + w10 * w10) / s->vxi[i];
    }
  }
  /* 7-point Newton-Cotes weights (Abramowitz 25.4.16) */
  s->wmu = dalloc(nm + 7); s->wni = dalloc(nni + 7);
  {
    double w1 = s->hmu / 140.0;
    s->wmu[1] = 0.0 + w1 * 41.0;
    for (int i = 2; i <= nm; i += 6) {
      s->wmu[i] = w1 * 216.0; s->wmu[i + 1] = w1 * 27.0; s->wmu[i + 2] = w1 * 272.0;
      s->wmu[i + 3] = w1 * 27.0; s->wmu[i + 4] = w1 * 216.0;
      s->wmu[i + 5] = (i + 5 == nm) ? w1 * 41.0 : 2.0 * w1 * 41.0;
    }
  }
  {
    double w1 = s->hni / 140.0;
    s->wni[1] = w1 * 41.0;
    for (int i = 2; i <= nni; i += 6) {
      s->wni[i] = w1 * 216.0; s->wni[i + 1] = w1 * 27.0; s->wni[i + 2] = w1 * 272.0;
      s->wni[i + 3] = w1 * 27.0; s->wni[i + 4] = w1 * 216.0;
      s->wni[i + 5] = (i + 5 == nni) ? w1 * 41.0 : 2.0 * w1 * 41.0;
    }
  }
  for (int i = 1; i <= nm; i++)
    for (int j = 1; j <= nni; j++) {
      int ij = (i - 1) * nni + (j - 1);
      wjac1[ij] = s->wmu[i] * wjac1[ij];
      wjac2[ij] = s->wmu[i] * wjac2[ij];
    }
  for (int i = 1; i <= nm; i++)
    for (int j = 1; j <= nni; j++) {
      int ij = (i - 1) * nni + (j - 1);
      wgt1[ij] = s->wni[j] * wjac1[ij];
      wgt2[ij] = s->wni[j] * wjac2[ij];
    }
  static const double aa1[9] = {3.0, -32.0, 168.0, -672.0, 0.0, 672.0, -168.0, 32.0, -3.0};
  static const double aa2[9] = {-9.0, 128.0, -1008.0, 8064.0, -14350.0, 8064.0, -1008.0, 128.0, -9.0};
  double w1 = 1.0 / (840.0), w2 = 1.0 / (5040.0);
  for (int i = 0; i < 4; i++) {
    s->dmu2[i] = w2 * aa2[i] / (s->hmu * s->hmu);
    s->dmu1[i] = w1 * aa1[i] / s->hmu;
    s->dni2[i] = w2 * aa2[i] / (s->hni * s->hni);
    s->dni1[i] = w1 * aa1[i] / s->hni;
  }
  /* 9-point derivative matrices for diffmu / diffnu (:1979-2030) */
  s->dmu9 = dalloc(9 * (nm + 1));
  s->dni9 = dalloc(9 * (nni + 1));
  double a1[9], a2[9];
  for (int k = 0; k < 9; k++) { a2[k] = w2 * aa2[k] / (s->hmu * s->hmu); a1[k] = w1 * aa1[k] / s->hmu; }
  for (int i = 1; i <= nm; i++)
    for (int k = 0; k < 9; k++) s->dmu9[9 * i + k] = a2[k] + borb[(i - 1) * nni + 0] * a1[k];
  for (int k = 0; k < 9; k++) { a2[k] = w2 * aa2[k] / (s->hni * s->hni); a1[k] = w1 * aa1[k] / s->hni; }
  for (int i = 1; i <= nni; i++)
    for (int k = 0; k < 9; k++) s->dni9[9 * i + k] = a2[k] + d[(2 - 1) * nni + (i - 1)] * a1[k];
  s->exeven[0] = 210.0 / 126.0; s->exeven[1] = -120.0 / 126.0; s->exeven[2] = 45.0 / 126.0;
  s->exeven[3] = -10.0 / 126.0; s->exeven[4] = 1.0 / 126.0;
  /* initLP: Legendre polynomials times r^k (:1517-1628) */
  for (int k = 0; k < MAXMPOLE; k++) s->leg[k] = dalloc(mx);
  for (int mu = 1; mu <= nm; mu++)
    for (int ni = 1; ni <= nni; ni++) {
      int i = (mu - 1) * nni + (ni - 1);
      double rr = sqrt(s->vxisq[mu] + s->vetasq[ni] - 1.0);
      double xr = s->r2 * rr;
      double costh = (fabs(rr) < PRECIS) ? 0.0 : s->vxi[mu] * s->veta[ni] / rr;
      double dome[10];
      dome[1] = costh;
      dome[2] = (3.0 * costh * costh - 1.0) * 0.50;
      for (int n = 2; n <= s->mpole - 1; n++)
        dome[n + 1] = ((double)(2 * n + 1) * costh * dome[n] - (double)n * dome[n - 1]) / (double)(n + 1);
      double xw = xr;
      s->leg[0][i] = dome[1] * xw;
      for (int k = 2; k <= s->mpole; k++) { xw = xw * xr; s->leg[k - 1][i] = dome[k] * xw; }
    }
  s->nexchmm = 0;
  for (int i1 = 1; i1 <= s->norb; i1++)
    for (int i2 = i1; i2 <= s->norb; i2++) {
      if (i1 == i2 && s->m[i2] == 0) continue;
      int n = ++s->nexchmm;
      s->iorb1mm[n] = i1; s->iorb2mm[n] = i2;
      int idel = abs(s->m[i2] - s->m[i1]);
      if (i1 == i2) idel = 2 * s->m[i2];
      s->idelmm[n] = idel;
      int ipc = s->k2[i1][i2];
      if (ipc == 0) continue;
      s->ipcmm[n] = ipc;
      if (s->ilc2[i1][i2] == 2) {
        n = ++s->nexchmm;
        s->idelmm[n] = s->m[i2] + s->m[i1];
        s->iorb1mm[n] = i1; s->iorb2mm[n] = i2;
        s->ipcmm[n] = ipc + s->norb * (s->norb + 1) / 2;
      }
    }
}

/* mesh ("middle" ordering) + boundary lists: src/initCBAllocArrays.F90:2408-2847 */
static void init_mesh(x2o_state *s) {
  int nni = s->nni, nmut = s->mxnmu;
  int nni8 = nni + 8, nmu8 = nmut + 8;
  s->nni8 = nni8; s->mxsize8 = nni8 * nmu8;
  s->nni1 = nni8; s->nni2 = 2 * nni8; s->nni3 = 3 * nni8; s->nni4 = 4 * nni8; s->nni5 = 5 * nni8;
  int iend1 = nmut;
  int ng = (nni - 2) * (nmut - 5);
  s->indx1 = (int *)calloc(ng + 1, sizeof(int));
  s->indx2 = (int *)calloc(ng + 1, sizeof(int));
  int nmux = (nmu8 - 1) / 2, nnix = (nni8 - 1) / 2, i0 = 0;
  for (int i = 6; i <= iend1; i++) {
    int ii = (i <= nmux) ? nmux - i + 6 : i;
    int i2 = ii - 4;
    for (int j = 6; j <= nni + 3; j++) {
      int jj = (j <= nnix) ? nnix - j + 6 : j;
      int j2 = jj - 4;
      i0++;
      s->indx2[i0 - 1] = (i2 - 1) * nni + j2;
      s->indx1[i0 - 1] = (ii - 1) * nni8 + jj;
    }
  }
  s->ngrid1 = i0;
  s->indx6a = (int *)calloc(nmut + 8, sizeof(int));
  s->indx6b = (int *)calloc(nmut + 8, sizeof(int));
  s->indx7 = (int *)calloc(nni + 8, sizeof(int));
  i0 = 0;
  for (int i = 5; i <= iend1; i++) s->indx6a[i0++] = (i - 1) * nni8 + 5;
  s->ngrid6a = i0;
  i0 = 0;
  for (int i = 5; i <= iend1; i++) s->indx6b[i0++] = (i - 1) * nni8 + nni + 4;
  s->ngrid6b = i0;
  i0 = 0;
  for (int j = 6; j <= nni + 3; j++) s->indx7[i0++] = 4 * nni8 + j;
  s->ngrid7 = i0;
}

/* initExWeights: src/initCBAllocArrays.F90:3303-3499 */
static void init_exweights(x2o_state *s) {
  int norb = s->norb;
  for (int i = 0; i <= 2 * MAXORB * MAXORB; i++) s->gec[i] = 0.0;
  char spn[4 * MAXORB + 1];
  for (int i = 1; i <= 4 * norb; i++) spn[i] = s->spin[i];
  for (int i = 1; i <= norb; i++) {
    int is = 4 * (i - 1);
    s->iloop[i] = 2; s->iqm[1 + is] = 1; s->iqm[2 + is] = 1;
    if (s->m[i] > 0) { s->iloop[i] = 4; s->iqm[3 + is] = -1; s->iqm[4 + is] = -1; }
  }
  for (int i = 1; i <= norb; i++)
    if (s->lock[i] == 0) {
      int jj = 4 * (i - 1);
      spn[jj + 1] = '+'; spn[jj + 2] = '-';
      if (s->m[i] > 0) { spn[jj + 3] = '+'; spn[jj + 4] = '-'; }
    }
  for (int i = 1; i <= 4 * norb; i++) s->spin[i] = spn[i];
  int isu2 = norb * norb;
  for (int i = 1; i <= norb; i++) {
    int ixx = 4 * (i - 1);
    double div = 0.0;
    for (int ii = 1; ii <= s->iloop[i]; ii++) {
      int ix = ii + ixx;
      if (spn[ix] != '+' && spn[ix] != '-') continue;
      div = div + 1.0;
      for (int j = 1; j <= norb; j++) {
        int jxx = 4 * (j - 1), kk = i + norb * (j - 1);
        int mpl = abs(s->m[i] - s->m[j]), mmi = abs(s->m[i] + s->m[j]);
        for (int jj = 1; jj <= s->iloop[j]; jj++) {
          int jx = jxx + jj;
          if (spn[jx] != '+' && spn[jx] != '-') continue;
          if (mpl == mmi && spn[ix] == spn[jx] && i != j) s->gec[kk] += 1.0;
          if (mpl != mmi && spn[ix] == spn[jx]) {
            if (i == j && s->iqm[ix] != s->iqm[jx]) s->gec[kk] += 1.0;
            if (i != j && s->iqm[ix] == s->iqm[jx]) s->gec[kk] += 1.0;
            if (i != j && s->iqm[ix] != s->iqm[jx]) s->gec[kk + isu2] += 1.0;
          }
        }
      }
    }
    for (int idiv = 1; idiv <= norb; idiv++) {
      int kk = i + norb * (idiv - 1);
      if (fabs(div) > PRECIS) { s->gec[kk] = s->gec[kk] / div; s->gec[kk + isu2] = s->gec[kk + isu2] / div; }
      else { s->gec[kk] = 0.0; s->gec[kk + isu2] = 0.0; }
    }
  }
  s->loffDiagLM = 0;
  for (int j = 1; j <= norb - 1; j++)
    for (int i = j + 1; i <= norb; i++) {
      if (s->m[j] != s->m[i] || s->gusym[j] != s->gusym[i] || s->iloop[j] != s->iloop[i]) continue;
      int match = 0;
      for (int ii = 1; ii <= s->iloop[i]; ii++)
        if (spn[ii + 4 * (i - 1)] == spn[ii + 4 * (j - 1)]) match++;
      if (match != s->iloop[i]) { s->offDiagLM[j][i] = s->offDiagLM[i][j] = 1; s->loffDiagLM = 1; }
    }
}

/* ======================================================================== */
/* initial guess                                                           */
/* ======================================================================== */

/* laguerre_normalization / sphharm_normalization / plaguer:
 * src/initOrbitalsPotentials.F90:878-934 */
static double lag_norm(double z, int n, int l) {
  return pow(2.0 * z / (double)n, 3.0 / 2.0 + (double)l) *
         sqrt(factor(n + l) / (2.0 * (double)n * factor(n - l - 1))) / factor(2 * l + 1);
}
static double sph_norm(int l, int m) {
  if (m == 0) return 1.0 / sqrt(4.0 * PII) * sqrt((2.0 * l + 1.0) * factor(l - m) / factor(l + m));
  return pow(-1.0, (double)m) / sqrt(4.0 * PII) * sqrt((2.0 * l + 1.0) * factor(l - m) / factor(l + m));
}
static double plaguer(int n, int l, double cz, double cr) {
  int np = n - l - 1, lp = 2 * l + 2;
  double x = cz * cr / (double)n;
  return pow(cr, (double)l) * exp(-x) * hypg1f1(-np, lp, x + x);
}

/* hydrogenOrbA / hydrogenOrbB: src/initOrbitalsPotentials.F90:782-876 */
static void hydrogen_orb(const x2o_state *s, double *orb, int n, int l, int m, double ez, int centreB) {
  double fn = lag_norm(ez, n, l), shn = sph_norm(l, m);
  double r = s->r;
  for (int in = 1; in <= s->nni; in++)
    for (int imu = 1; imu <= s->mxnmu; imu++) {
      int igp = (imu - 1) * s->nni + (in - 1);
      double z = (r / 2.0) * s->vxi[imu] * s->veta[in];
      double rt, costh;
      if (!centreB) {
        rt = (r / 2.0) * (s->vxi[imu] + s->veta[in]);
        if (rt < PRECIS) costh = -1.0;
        else { costh = (z + r / 2.0) / rt; if (costh < -1.0) costh = -1.0; if (costh > 1.0) costh = 1.0; }
      } else {
        rt = (r / 2.0) * (s->vxi[imu] - s->veta[in]);
        if (rt < PRECIS) costh = -1.0;
        else { costh = -(z - r / 2.0) / rt; if (costh < -1.0) costh = -1.0; if (costh > 1.0) costh = 1.0; }
      }
      orb[igp] = fn * plaguer(n, l, ez, rt) * shn * plegendg(l, m, costh);
    }
}

/* pottf: src/coulombExchangePotentials.f90:222-239 */
static double pottf(double r, double veta, double vxi) {
  if (fabs(vxi + veta) < PRECIS) return 0.0;
  double rab = r * (vxi + veta) / 2.0;
  double w = sqrt(rab / 0.885340);
  double t = w * (0.6011200 * w + 1.8106100) + 1.0;
  w = w * (w * (w * (w * (0.0479300 * w + 0.2146500) + 0.7711200) + 1.3951500) + 1.8106100) + 1.0;
  return (1.0 - (t / w) * (t / w)) / rab;
}

/* initHyd + initCoulomb + initExchange:
 * src/initOrbitalsPotentials.F90:714-775, src/coulombExchangePotentials.f90:14-147 */
static void init_hyd(x2o_state *s) {
  int mx = s->mxsize, nni = s->nni;
  double *tmp = dalloc(mx);
  double *f4 = s->sup[8];
  for (int iorb = 1; iorb <= s->norb; iorb++) {
    if (s->inhyd[iorb] == 0) continue;
    double *psi = s->psi[iorb];
    memset(psi, 0, sizeof(double) * mx);
    if (fabs(s->co1[iorb]) > PRECIS) {
      hydrogen_orb(s, tmp, s->n1[iorb], s->l1[iorb], s->m[iorb], s->eza1[iorb], 0);
      for (int i = 0; i < mx; i++) psi[i] = s->co1[iorb] * tmp[i] + psi[i];
    }
    if (fabs(s->co2[iorb]) > PRECIS) {
      hydrogen_orb(s, tmp, s->n2[iorb], s->l2[iorb], s->m[iorb], s->eza2[iorb], 1);
      for (int i = 0; i < mx; i++) psi[i] = s->co2[iorb] * tmp[i] + psi[i];
    }
  }
  free(tmp);
  int iz1 = (int)lround(s->z1), iz2 = (int)lround(s->z2);
  for (int iorb = 1; iorb <= s->norb; iorb++) {
    if (s->inhyd[iorb] == 0) continue;
    double *ex = s->coul[iorb];
    double crt1 = fabs(s->co1[iorb]), crt2 = fabs(s->co2[iorb]);
    for (int in = 1; in <= nni; in++) {
      double vetat = s->veta[in];
      for (int imu = 1; imu <= s->mxnmu; imu++) {
        double vxit = s->vxi[imu];
        int igp = (imu - 1) * nni + (in - 1);
        if (imu == 1 && (in == 1 || in == nni)) ex[igp] = 0.0;
        else if (iz1 != 0 && iz2 != 0)
          ex[igp] = -1.0 * pottf(s->r, vetat, vxit) * crt1 + -1.0 * pottf(s->r, -vetat, vxit) * crt2;
        else
          ex[igp] = -1.0 * pottf(s->r, vetat, vxit) * crt1;
      }
    }
    for (int i = 0; i < mx; i++) ex[i] = ex[i] * f4[i];
  }
  for (int i1 = 1; i1 <= s->norb; i1++)
    for (int i2 = i1; i2 <= s->norb; i2++) {
      if (i1 == i2 && s->m[i2] == 0) continue;
      int k = s->k2[i1][i2];
      double *ex = s->exch[2 * k];
      for (int imu = 2; imu <= s->mxnmu; imu++) {
        double vxit = s->vxi[imu];
        for (int in = 2; in <= nni - 1; in++) {
          int igp = (imu - 1) * nni + (in - 1);
          double vetat = s->veta[in];
          double ra1 = (s->r / 2.0) * (vxit + vetat), ra2 = (s->r / 2.0) * (vxit - vetat);
          ex[igp] = (ra1 > 1.0e-8) ? s->co1[i1] / ra1 : 0.0;
          if (ra2 > 1.0e-8) ex[igp] = ex[igp] + s->co2[i1] / ra2;
        }
      }
      for (int i = 0; i < mx; i++) ex[i] = ex[i] * f4[i];
      if (i1 != i2 && s->m[i1] != 0 && s->m[i2] != 0) memcpy(s->exch[2 * k + 1], ex, sizeof(double) * mx);
    }
}

int x2o_setup(x2o_state *s) {
  init_cblocks(s);
  init_addr(s);
  init_suppl(s);
  init_mesh(s);
  init_exweights(s);
  for (int k = 0; k < 8; k++) s->w[k] = dalloc(s->mxsize8 + 16);
  for (int i = 0; i <= MAXORB; i++) for (int j = 0; j <= MAXORB; j++) s->ee[i][j] = 0.0;
  if (s->hydrogen_start) init_hyd(s);
  s->isstart = 1; s->isstop = s->ngrid1; s->isstep = 1;
  return 0;
}

/* ======================================================================== */
/* putin / putout (src/inout.F90:23-183)                                   */
/* ======================================================================== */

void x2o_putin(int nni, int nmi, int isym, const double *fun, double *work) {
  int n8 = nni + 8;
#define FUN(j, i) fun[((i)-1) * nni + ((j)-1)]
#define WRK(j, i) work[((i)-1) * n8 + ((j)-1)]
  for (int i = 1; i <= nmi; i++)
    for (int j = 1; j <= nni; j++) WRK(4 + j, i + 4) = FUN(j, i);
  double sg = (isym == 1) ? 1.0 : -1.0;
  for (int i = 2; i <= 5; i++)
    for (int j = 1; j <= nni; j++) WRK(4 + j, 6 - i) = (isym == 1) ? FUN(j, i) : -FUN(j, i);
  for (int j = 2; j <= 5; j++)
    for (int i = 1; i <= nmi; i++) WRK(6 - j, 4 + i) = (isym == 1) ? FUN(j, i) : -FUN(j, i);
  for (int j = 1; j <= 4; j++)
    for (int i = 1; i <= nmi; i++) WRK(nni + 4 + j, 4 + i) = (isym == 1) ? FUN(nni - j, i) : -FUN(nni - j, i);
  (void)sg;
#undef FUN
#undef WRK
}

void x2o_putout(int nni, int nmi, double *fun, const double *work) {
  int n8 = nni + 8;
  for (int i = 1; i <= nmi; i++)
    for (int j = 1; j <= nni; j++) fun[(i - 1) * nni + (j - 1)] = work[(i + 3) * n8 + (j + 3)];
}

/* ======================================================================== */
/* sweeps (src/sormcsor.F90)                                               */
/* ======================================================================== */

static inline void relax_point(const x2o_state *s, double *fun, int ij, int ik, const double *lhs,
                               const double *rhs, const double *b, const double *d, double omega,
                               double omega1) {
  const int n1 = s->nni1, n2 = s->nni2, n3 = s->nni3, n4 = s->nni4;
  const double *dmu1 = s->dmu1, *dmu2 = s->dmu2, *dni1 = s->dni1, *dni2 = s->dni2;
  double ddmi2 = dmu2[0] * (fun[ij - n4] + fun[ij + n4]) + dmu2[1] * (fun[ij - n3] + fun[ij + n3]) +
                 dmu2[2] * (fun[ij - n2] + fun[ij + n2]) + dmu2[3] * (fun[ij - n1] + fun[ij + n1]);
  double ddmi1 = dmu1[0] * (fun[ij - n4] - fun[ij + n4]) + dmu1[1] * (fun[ij - n3] - fun[ij + n3]) +
                 dmu1[2] * (fun[ij - n2] - fun[ij + n2]) + dmu1[3] * (fun[ij - n1] - fun[ij + n1]);
  double ddni2 = dni2[0] * (fun[ij - 4] + fun[ij + 4]) + dni2[1] * (fun[ij - 3] + fun[ij + 3]) +
                 dni2[2] * (fun[ij - 2] + fun[ij + 2]) + dni2[3] * (fun[ij - 1] + fun[ij + 1]);
  double ddni1 = dni1[0] * (fun[ij - 4] - fun[ij + 4]) + dni1[1] * (fun[ij - 3] - fun[ij + 3]) +
                 dni1[2] * (fun[ij - 2] - fun[ij + 2]) + dni1[3] * (fun[ij - 1] - fun[ij + 1]);
  double cc = ddmi2 + b[ik] * ddmi1 + ddni2 + d[ik] * ddni1;
  fun[ij] = omega * (rhs[ik] - cc) / lhs[ik] + omega1 * fun[ij];
}

/* boundary extrapolation after each micro-sweep: src/sormcsor.F90:94-129 */
static void sweep_boundary(const x2o_state *s, int isym, double *fun) {
  const double *ex = s->exeven;
  const int n1 = s->nni1, n2 = s->nni2, n3 = s->nni3, n4 = s->nni4, n5 = s->nni5;
  if (isym == 1) {
    for (int i = 0; i < s->ngrid7; i++) {
      int ij = s->indx7[i] - 1;
      fun[ij] = ex[0] * fun[ij + n1] + ex[1] * fun[ij + n2] + ex[2] * fun[ij + n3] + ex[3] * fun[ij + n4] +
                ex[4] * fun[ij + n5];
    }
    for (int i = 0; i < s->ngrid6a; i++) {
      int ij = s->indx6a[i] - 1;
      fun[ij] = ex[0] * fun[ij + 1] + ex[1] * fun[ij + 2] + ex[2] * fun[ij + 3] + ex[3] * fun[ij + 4] +
                ex[4] * fun[ij + 5];
    }
    for (int i = 0; i < s->ngrid6b; i++) {
      int ij = s->indx6b[i] - 1;
      fun[ij] = ex[0] * fun[ij - 1] + ex[1] * fun[ij - 2] + ex[2] * fun[ij - 3] + ex[3] * fun[ij - 4] +
                ex[4] * fun[ij - 5];
    }
  } else {
    for (int i = 0; i < s->ngrid7; i++) fun[s->indx7[i] - 1] = 0.0;
    for (int i = 0; i < s->ngrid6a; i++) fun[s->indx6a[i] - 1] = 0.0;
    for (int i = 0; i < s->ngrid6b; i++) fun[s->indx6b[i] - 1] = 0.0;
  }
}

void x2o_sweep(const x2o_state *s, int mode, int isym, int maxsor2, double omega, double *fun,
               const double *lhs, const double *rhs, const double *b, const double *d, int isstart,
               int isstop, int isstep) {
  double omega1 = 1.0 - omega;
  for (int itr2 = 1; itr2 <= maxsor2; itr2++) {
    if (mode == 0) {
      /* Fortran DO i=isstart,isstop,isstep */
      if (isstep > 0) {
        for (int i = isstart; i <= isstop; i += isstep)
          relax_point(s, fun, s->indx1[i - 1] - 1, s->indx2[i - 1] - 1, lhs, rhs, b, d, omega, omega1);
      } else {
        for (int i = isstart; i >= isstop; i += isstep)
          relax_point(s, fun, s->indx1[i - 1] - 1, s->indx2[i - 1] - 1, lhs, rhs, b, d, omega, omega1);
      }
    } else if (mode == 1) {
      for (int c = 1; c <= 5; c++)
        for (int i = c; i <= s->ngrid1; i += 5)
          relax_point(s, fun, s->indx1[i - 1] - 1, s->indx2[i - 1] - 1, lhs, rhs, b, d, omega, omega1);
    } else {
      /* Not a reference ordering: the GPU mixed form's seam-free colouring,
       * colour (col - row) mod 5 of the extended-array point, the colours in
       * turn (its points are independent; taken in list order) */
      for (int c = 0; c < 5; c++)
        for (int i = 1; i <= s->ngrid1; i++) {
          const int ij = s->indx1[i - 1] - 1, row = ij / s->nni8, col = ij % s->nni8;
          if (((col - row) % 5 + 5) % 5 != c) continue;
          relax_point(s, fun, ij, s->indx2[i - 1] - 1, lhs, rhs, b, d, omega, omega1);
        }
    }
    sweep_boundary(s, isym, fun);
  }
}

/* ======================================================================== */
/* Fock potential (src/fock.F90:57-186)                                    */
/* ======================================================================== */

void x2o_fock(x2o_state *s, int iorb, double *fock1, double *fock2) {
  int mx = s->mxsize, norb = s->norb;
  double *e = s->sup[3], *f0 = s->sup[4], *f1 = s->sup[5], *f2 = s->sup[6], *f4 = s->sup[8];
  double *wk1 = s->w[6], *wk2 = s->w[7];
  for (int i = 0; i < mx; i++) fock1[i] = f0[i];
  for (int i = 0; i < mx; i++) fock1[i] = s->ee[iorb][iorb] * f1[i] + fock1[i];
  if (s->mm[iorb] != 0) {
    double w = (double)(s->mm[iorb] * s->mm[iorb]);
    for (int i = 0; i < mx; i++) fock1[i] = w * e[i] + fock1[i];
  }
  memset(fock2, 0, sizeof(double) * mx);
  if (s->nel == 1) return;
  memset(wk1, 0, sizeof(double) * mx);
  for (int iorb1 = 1; iorb1 <= norb; iorb1++) {
    int kex = iorb + (iorb1 - 1) * norb;
    double coo = s->occ[iorb1];
    if (iorb == iorb1) coo = coo - 1.0;
    const double *pot1 = s->coul[iorb1];
    for (int i = 0; i < mx; i++) wk1[i] = coo * pot1[i] + wk1[i];
    int idexp = s->k2[iorb][iorb1];
    if (iorb1 != iorb) {
      const double *ex = s->exch[2 * idexp];
      for (int i = 0; i < mx; i++) wk2[i] = ex[i];
      for (int i = 0; i < mx; i++) wk2[i] = s->gec[kex] * wk2[i];
      if (s->ilc2[iorb][iorb1] == 2) {
        const double *ex2 = s->exch[2 * idexp + 1];
        double g2 = s->gec[kex + norb * norb];
        for (int i = 0; i < mx; i++) wk2[i] = g2 * ex2[i] + wk2[i];
      }
      if (fabs(s->ee[iorb1][iorb]) > PRECIS) {
        double eab = s->ee[iorb1][iorb];
        for (int i = 0; i < mx; i++) wk2[i] = eab * f4[i] + wk2[i];
      }
      const double *p1 = s->psi[iorb1];
      for (int i = 0; i < mx; i++) wk2[i] = wk2[i] * p1[i];
      for (int i = 0; i < mx; i++) fock2[i] = fock2[i] + wk2[i];
    } else {
      if (s->mm[iorb] > 0 && s->ilc2[iorb][iorb1] > 0) {
        const double *ex = s->exch[2 * idexp];
        const double *p1 = s->psi[iorb1];
        for (int i = 0; i < mx; i++) wk2[i] = ex[i];
        for (int i = 0; i < mx; i++) wk2[i] = wk2[i] * p1[i];
        for (int i = 0; i < mx; i++) fock2[i] = s->gec[kex] * wk2[i] + fock2[i];
      }
    }
  }
  memcpy(s->coulombptr[iorb], wk1, sizeof(double) * mx);
  memcpy(s->exchangeptr[iorb], fock2, sizeof(double) * mx);
  for (int i = 0; i < mx; i++) wk1[i] = wk1[i] * f2[i];
  for (int i = 0; i < mx; i++) fock2[i] = fock2[i] * f2[i];
  for (int i = 0; i < mx; i++) fock1[i] = fock1[i] + wk1[i];
}

/* ======================================================================== */
/* relaxation drivers                                                      */
/* ======================================================================== */

/* orbAsymptGet / orbAsymptSet: src/relaxOrbs.F90:415-462 */
static void orb_asympt_get(const x2o_state *s, double *edecay, const double *fa) {
  int nni = s->nni, jj = 0;
  for (int j = s->mxnmu - 3; j <= s->mxnmu; j++) {
    jj++;
    for (int i = 1; i <= nni; i++) {
      double raiq1 = sqrt(s->vxisq[j - 1] + s->vetasq[i] - 1.0);
      double raiq = sqrt(s->vxisq[j] + s->vetasq[i] - 1.0);
      int k = i + (j - 1) * nni - 1;
      edecay[(jj - 1) * nni + (i - 1)] =
          pow(fabs(fa[k] / fa[k - nni]), 0.250) * exp(sqrt(fabs(fa[k - nni])) * (raiq1 - raiq));
    }
  }
}
static void orb_asympt_set(const x2o_state *s, double *psi, const double *edecay) {
  int nni = s->nni, jj = 0;
  for (int j = s->mxnmu - 3; j <= s->mxnmu; j++) {
    jj++;
    for (int i = 1; i <= nni; i++) {
      int k = i + (j - 1) * nni - 1;
      psi[k] = psi[k - nni] * edecay[(jj - 1) * nni + (i - 1)];
    }
  }
}

/* orbSOR / orbMCSOR: src/relaxOrbs.F90:16-241 (serial variant: wk1=fock1/f1) */
void x2o_relax_orb(x2o_state *s, int iorb, int mode) {
  int mx = s->mxsize, nni = s->nni;
  double *fock1 = s->w[0], *rhs = s->w[1], *wk1 = s->w[2], *wk2 = s->w[3], *wk3 = s->w[4], *lhs = s->w[5];
  double *f1 = s->sup[5];
  x2o_fock(s, iorb, fock1, rhs);
  double omega = s->ovforb;
  int isym = s->isymOrb[iorb];
  s->nsor4orb += (long)s->maxsororb[0] * s->maxsororb[1];
  for (int itr1 = 1; itr1 <= s->maxsororb[0]; itr1++) {
    for (int i = 0; i < mx; i++) lhs[i] = fock1[i] + s->diag;
    for (int i = s->mxnmu - 4; i <= s->mxnmu; i++)
      for (int j = 1; j <= nni; j++) {
        int ij = (i - 1) * nni + (j - 1);
        wk1[ij] = (fabs(f1[ij]) <= PRECIS) ? 0.0 : fock1[ij] / f1[ij];
      }
    orb_asympt_get(s, wk3, wk1);
    x2o_putin(nni, s->mxnmu, isym, s->psi[iorb], wk2);
    if (s->orb_hook)
      s->orb_hook(s->hook_ud, iorb, isym, wk2, lhs, rhs);
    else
      x2o_sweep(s, mode, isym, s->maxsororb[1], omega, wk2, lhs, rhs, s->sup[0], s->sup[2], s->isstart,
                s->isstop, s->isstep);
    x2o_putout(nni, s->mxnmu, s->psi[iorb], wk2);
    orb_asympt_set(s, s->psi[iorb], wk3);
  }
}

/* coulExchSOR body for one potential: src/relaxPots.F90:64-104 */
void x2o_relax_pot(x2o_state *s, int iorb, int k, int mode) {
  int mx = s->mxsize, nni = s->nni;
  double *lhs = s->w[5], *rhs = s->w[1], *wk2 = s->w[3];
  double *e = s->sup[3], *f3 = s->sup[7], *g = s->sup[9];
  int in1 = s->ins1[iorb][k], in2 = s->ins2[iorb][k];
  int idel = s->deltam4pot[iorb][k], isym = s->isyms[iorb][k];
  double *excp = s->pottarget[iorb][k];
  s->nsor4pot += (long)s->maxsorpot[0] * s->maxsorpot[1];
  const double *p1 = s->psi[in1], *p2 = s->psi[in2];
  for (int i = 0; i < mx; i++) wk2[i] = p1[i] * p2[i];
  for (int i = 0; i < mx; i++) rhs[i] = wk2[i] * g[i];
  if (idel == 0) for (int i = 0; i < mx; i++) lhs[i] = f3[i];
  else {
    double dd = (double)(idel * idel);
    for (int i = 0; i < mx; i++) lhs[i] = f3[i] + dd * e[i];
  }
  for (int itr1 = 1; itr1 <= s->maxsorpot[0]; itr1++) {
    x2o_putin(nni, s->mxnmu, isym, excp, wk2);
    x2o_sweep(s, mode, isym, s->maxsorpot[1], s->ovfexch, wk2, lhs, rhs, s->sup[1], s->sup[2], s->isstart,
              s->isstop, s->isstep);
    x2o_putout(nni, s->mxnmu, excp, wk2);
  }
}

/* ======================================================================== */
/* quadratures                                                             */
/* ======================================================================== */

/* norm: src/normOrtho.F90:14-59 */
double x2o_norm_value(x2o_state *s, int iorb) {
  int mx = s->mxsize;
  double *wk0 = s->w[0], *f4 = s->sup[8], *psi = s->psi[iorb];
  for (int i = 0; i < mx; i++) wk0[i] = psi[i] * psi[i];
  for (int i = 0; i < mx; i++) wk0[i] = wk0[i] * f4[i];
  return ddot(mx, s->sup[13], wk0);
}
void x2o_norm(x2o_state *s, int iorb) {
  double xnorm = x2o_norm_value(s, iorb);
  s->orbNorm[iorb] = xnorm;
  double zarea = 1.0 / sqrt(xnorm);
  double *psi = s->psi[iorb];
  for (int i = 0; i < s->mxsize; i++) psi[i] = zarea * psi[i];
}

/* ortho: src/normOrtho.F90:103-207 */
void x2o_ortho(x2o_state *s, int iorb1) {
  int mx = s->mxsize, norb = s->norb, jor = 0;
  int istp[MAXORB + 1];
  double ovla[MAXORB + 1];
  double *wk0 = s->w[0], *f4 = s->sup[8], *psi1 = s->psi[iorb1];
  if (s->ifixorb[iorb1] != 0) return;
  for (int iorb2 = 1; iorb2 <= norb; iorb2++) {
    int iorb3 = norb - iorb2 + 1;
    if (iorb3 <= iorb1) continue;
    if (s->m[iorb3] != s->m[iorb1]) continue;
    if (s->ige[iorb3] != s->ige[iorb1] && !s->lbreakCi) continue;
    jor++;
    istp[jor] = iorb3;
    const double *psi3 = s->psi[iorb3];
    for (int i = 0; i < mx; i++) wk0[i] = psi1[i] * psi3[i];
    for (int i = 0; i < mx; i++) wk0[i] = wk0[i] * f4[i];
    ovla[jor] = ddot(mx, s->sup[13], wk0);
  }
  if (jor > 0) {
    double wmax = 0.0;
    for (int i = 1; i <= jor; i++) if (fabs(ovla[i]) > wmax) wmax = fabs(ovla[i]);
    s->wstorthog[iorb1] = wmax;
  }
  if (jor == 0) return;
  double ano = 0.0;
  for (int ira = 1; ira <= jor; ira++) {
    ano = ano + ovla[ira] * ovla[ira];
    const double *psi3 = s->psi[istp[ira]];
    double a = -ovla[ira];
    for (int i = 0; i < mx; i++) psi1[i] = a * psi3[i] + psi1[i];
  }
  ano = sqrt(1.0 + ano) / (1.0 - ano * ano);
  for (int i = 0; i < mx; i++) psi1[i] = ano * psi1[i];
}

/* setCi / setCiOrb: src/scfUtils.F90:337-434 */
static void setci_orb(const x2o_state *s, int iorb) {
  int nni = s->nni, n2 = nni / 2 + 1;
  double *orb = s->psi[iorb];
  if (s->ihomo[iorb] == 1) {
    for (int ni = 1; ni <= n2 - 1; ni++)
      for (int mi = 1; mi <= s->mxnmu; mi++) orb[(mi - 1) * nni + (nni - ni)] = orb[(mi - 1) * nni + (ni - 1)];
  } else {
    for (int ni = 1; ni <= n2 - 1; ni++)
      for (int mi = 1; mi <= s->mxnmu; mi++) orb[(mi - 1) * nni + (nni - ni)] = -orb[(mi - 1) * nni + (ni - 1)];
    for (int mi = 1; mi <= s->mxnmu; mi++) orb[(mi - 1) * nni + (n2 - 1)] = 0.0;
  }
}
static void setci(x2o_state *s, int iorb) {
  if (iorb == 0) { for (int i = 1; i <= s->norb; i++) setci_orb(s, i); }
  else setci_orb(s, iorb);
}

/* diffnu + diffmu on a putin-extended function (src/utils.f90:599-695):
 * out(plain) = d2/dnu2 + d(nu) d/dnu + d2/dmu2 + b(mu) d/dmu.
 * The ext rows nmu+5..nmu+8 are never written by putin; they read as zero. */
static void laplace_terms(x2o_state *s, const double *wext, double *out) {
  int nni = s->nni, n8 = s->nni8, nm = s->mxnmu;
  /* diffnu: fd(nu=j+4, row) = sum_k f(j+k-1,row) dni(k,j), dgemv order */
  for (int i = 1; i <= nm; i++) {
    int row = i + 4;
    for (int j = 1; j <= nni; j++) {
      double sn = 0.0;
      for (int k = 1; k <= 9; k++) sn = sn + wext[(row - 1) * n8 + (j + k - 2)] * s->dni9[9 * j + k - 1];
      double sm = 0.0;
      for (int k = 1; k <= 9; k++) sm = sm + wext[(i + k - 2) * n8 + (j + 3)] * s->dmu9[9 * i + k - 1];
      /* add(mxsize, wk0(mu part), wk1(nu part)): wk1 = wk1 + wk0 */
      out[(i - 1) * nni + (j - 1)] = sn + sm;
    }
  }
}

/* oneelij with iorb1 == iorb2 (integrals.F90:406-480); returns <a|T+V|a>
 * and stores the kinetic and nuclear parts (oneelii, integrals.F90:37-165). */
static double oneel_ii(x2o_state *s, int iorb, double *wkin, double *wnucl) {
  int mx = s->mxsize;
  double *wk3 = s->w[3], *wk1 = s->w[1], *wk2 = s->w[2], *wk0 = s->w[0];
  double *psi = s->psi[iorb], *e = s->sup[3], *f0 = s->sup[4], *wgt1 = s->sup[12];
  memset(wk3, 0, sizeof(double) * s->mxsize8);
  x2o_putin(s->nni, s->mxnmu, s->isymOrb[iorb], psi, wk3);
  laplace_terms(s, wk3, wk1);
  if (s->mm[iorb] != 0) {
    double w = (double)(s->mm[iorb] * s->mm[iorb]);
    for (int i = 0; i < mx; i++) wk1[i] = w * e[i] * psi[i] + wk1[i];
  }
  if (wkin) {
    for (int i = 0; i < mx; i++) wk2[i] = wk1[i] * psi[i];
    *wkin = ddot(mx, wgt1, wk2);
  }
  for (int i = 0; i < mx; i++) wk0[i] = f0[i];
  if (wnucl) {
    for (int i = 0; i < mx; i++) wk2[i] = psi[i] * wk0[i];
    for (int i = 0; i < mx; i++) wk2[i] = wk2[i] * psi[i];
    *wnucl = ddot(mx, wgt1, wk2);
  }
  for (int i = 0; i < mx; i++) wk1[i] = psi[i] * wk0[i] + wk1[i];
  for (int i = 0; i < mx; i++) wk1[i] = wk1[i] * psi[i];
  return ddot(mx, wgt1, wk1);
}

/* EaHF: src/lagrangeMultipliers.F90:21-107 */
void x2o_eahf(x2o_state *s, int iorb) {
  int mx = s->mxsize;
  double woneel = oneel_ii(s, iorb, NULL, NULL);
  double *wk0 = s->w[0], *psi = s->psi[iorb], *wgt2 = s->sup[13];
  const double *cp = s->coulombptr[iorb], *xp = s->exchangeptr[iorb];
  for (int i = 0; i < mx; i++) wk0[i] = psi[i] * cp[i];
  for (int i = 0; i < mx; i++) wk0[i] = wk0[i] * psi[i];
  double wc = ddot(mx, wgt2, wk0);
  for (int i = 0; i < mx; i++) wk0[i] = psi[i] * xp[i];
  double wx = -ddot(mx, wgt2, wk0);
  s->ee[iorb][iorb] = woneel + (wc + wx);
}

double x2o_ee(const x2o_state *s, int i, int j) { return s->ee[i][j]; }

/* EabHF: src/lagrangeMultipliers.F90:335-409.  For closed shells
 * offDiagLM is never set (initExWeights), so the loop body never runs;
 * open shells are rejected by the input reader of this oracle. */
static void eabhf(x2o_state *s, int iorb) {
  (void)s; (void)iorb;
}

static double coulij(x2o_state *s, int iorb1, int iorb2) {
  int mx = s->mxsize;
  double *wk0 = s->w[0];
  const double *p = s->psi[iorb2], *pot = s->coul[iorb1];
  for (int i = 0; i < mx; i++) wk0[i] = p[i] * pot[i];
  for (int i = 0; i < mx; i++) wk0[i] = wk0[i] * p[i];
  return ddot(mx, s->sup[13], wk0);
}
static double exchij(x2o_state *s, int type, int iorb1, int iorb2) {
  int mx = s->mxsize;
  double *wk0 = s->w[0];
  int ihc = s->k2[iorb1][iorb2];
  const double *ex = s->exch[2 * ihc + (type ? 1 : 0)];
  const double *p1 = s->psi[iorb1], *p2 = s->psi[iorb2];
  for (int i = 0; i < mx; i++) wk0[i] = p1[i] * ex[i];
  for (int i = 0; i < mx; i++) wk0[i] = wk0[i] * p2[i];
  return ddot(mx, s->sup[13], wk0);
}

/* excont / exint: src/exchContribs.f90:11-154 */
static void excont(const x2o_state *s, int iorb1, int iorb2, double *ox1, double *ox2) {
  int ipe1 = s->m[iorb1], ipe2 = s->m[iorb2], ip1 = 4 * (iorb1 - 1), ip2 = 4 * (iorb2 - 1);
  int icase, i1end, i2end = 2;
  const char *sp = s->spin;
#define OK(c) ((c) == '+' || (c) == '-')
  *ox1 = 0.0; *ox2 = 0.0;
  if (ipe1 == 0) { icase = 1; i1end = 2; i2end = (ipe2 == 0) ? 2 : 4; }
  else { i1end = 4; if (ipe2 == 0) { icase = 1; i2end = 2; } else icase = 2; }
  if (icase == 1) {
    for (int i1 = 1; i1 <= i1end; i1++) {
      if (!OK(sp[ip1 + i1])) continue;
      for (int i2 = 1; i2 <= i2end; i2++) {
        if (!OK(sp[ip2 + i2])) continue;
        if (sp[ip1 + i1] == sp[ip2 + i2]) *ox1 += 1.0;
      }
    }
  } else {
    for (int i1 = 1; i1 <= 2; i1++) { if (!OK(sp[ip1 + i1])) continue;
      for (int i2 = 1; i2 <= 2; i2++) { if (!OK(sp[ip2 + i2])) continue; if (sp[ip1 + i1] == sp[ip2 + i2]) *ox1 += 1.0; } }
    for (int i1 = 3; i1 <= 4; i1++) { if (!OK(sp[ip1 + i1])) continue;
      for (int i2 = 3; i2 <= 4; i2++) { if (!OK(sp[ip2 + i2])) continue; if (sp[ip1 + i1] == sp[ip2 + i2]) *ox1 += 1.0; } }
    for (int i1 = 1; i1 <= 2; i1++) { if (!OK(sp[ip1 + i1])) continue;
      for (int i2 = 3; i2 <= 4; i2++) { if (!OK(sp[ip2 + i2])) continue; if (sp[ip1 + i1] == sp[ip2 + i2]) *ox2 += 1.0; } }
    for (int i1 = 3; i1 <= 4; i1++) { if (!OK(sp[ip1 + i1])) continue;
      for (int i2 = 1; i2 <= 2; i2++) { if (!OK(sp[ip2 + i2])) continue; if (sp[ip1 + i1] == sp[ip2 + i2]) *ox2 += 1.0; } }
  }
}
static void exint(const x2o_state *s, int iorb1, double *ox1) {
  int ip1 = 4 * (iorb1 - 1);
  const char *sp = s->spin;
  *ox1 = 0.0;
  for (int i1 = 1; i1 <= 2; i1++) { if (!OK(sp[ip1 + i1])) continue;
    for (int i2 = 3; i2 <= 4; i2++) { if (!OK(sp[ip1 + i2])) continue; if (sp[ip1 + i1] == sp[ip1 + i2]) *ox1 += 1.0; } }
#undef OK
}

/* etotalHF: src/totalEnergy.F90:13-245 */
void x2o_etotal(x2o_state *s, double *etot, double *evt, double *vkt, double *vnt) {
  double woneel = 0, wdcoul = 0, wndc = 0, wex1 = 0, wex2 = 0;
  s->vkt = 0; s->vnt = 0;
  for (int iorb = 1; iorb <= s->norb; iorb++) {
    double wk, wn;
    double o = oneel_ii(s, iorb, &wk, &wn);
    s->vk[iorb] = wk; s->vn[iorb] = wn;
    woneel = woneel + s->occ[iorb] * o;
    s->vkt = s->vkt + s->occ[iorb] * wk;
    s->vnt = s->vnt + s->occ[iorb] * wn;
    if (s->occ[iorb] > 1.0) {
      double w = coulij(s, iorb, iorb);
      wdcoul = wdcoul + s->occ[iorb] * (s->occ[iorb] - 1.0) * w / 2.0;
    }
  }
  for (int i1 = 1; i1 <= s->norb; i1++) {
    if (s->mm[i1] > 0 && fabs(s->occ[i1] - 1.0) > 1.e-7) {
      double ocx1;
      exint(s, i1, &ocx1);
      double w = exchij(s, 0, i1, i1);
      wex1 = wex1 + ocx1 * w;
    }
    for (int i2 = i1 + 1; i2 <= s->norb; i2++) {
      double w = coulij(s, i2, i1);
      wndc = wndc + s->occ[i1] * s->occ[i2] * w;
      double ocx1, ocx2;
      excont(s, i1, i2, &ocx1, &ocx2);
      w = exchij(s, 0, i1, i2);
      wex1 = wex1 + ocx1 * w;
      if (s->ilc2[i1][i2] == 2) {
        w = exchij(s, 1, i1, i2);
        wex2 = wex2 + ocx2 * w;
      }
    }
  }
  s->evt = woneel + wdcoul + wndc - wex1 - wex2;
  double epott = s->vnt + wdcoul + wndc - wex1 - wex2;
  s->virrat = (epott + s->z1 * s->z2 / s->r) / s->vkt;
  s->etot = s->evt + s->z1 * s->z2 / s->r;
  if (etot) *etot = s->etot;
  if (evt) *evt = s->evt;
  if (vkt) *vkt = s->vkt;
  if (vnt) *vnt = s->vnt;
}

/* ======================================================================== */
/* multipole moments and potential asymptotics (src/scfUtils.F90)          */
/* ======================================================================== */

/* mulex: src/scfUtils.F90:856-1032 (normalised associated Legendre) */
static void mulex(const x2o_state *s, int i, int j, int mt, double *dome) {
  int mpole = s->mpole;
  dome[1] = 0.0;
  if (mt > 4) return;
  double rr = sqrt(s->vxisq[j] + s->vetasq[i] - 1.0);
  double costh = 0.0;
  if (fabs(rr) > PRECIS) costh = s->veta[i] * s->vxi[j] / rr;
  double c2, c4, c6, c8, si, si2, si3;
  if (mt == 0) {
    dome[1] = costh;
    dome[2] = (3.0 * costh * costh - 1.0) * 0.50;
    for (int n = 2; n <= mpole - 1; n++)
      dome[n + 1] = ((double)(2 * n + 1) * costh * dome[n] - (double)n * dome[n - 1]) / (double)(n + 1);
  } else if (mt == 1) {
    c2 = costh * costh; si2 = fabs(1.0 - c2); si = sqrt(si2);
    dome[1] = -si / sqrt(2.0);
    dome[2] = -3.0 * si * costh / sqrt(6.0);
    if (mpole < 3) return;
    dome[3] = (3.0 / 2.0) * si * (1.0 - 5.0 * c2) / sqrt(12.0);
    if (mpole < 4) return;
    dome[4] = (5.0 / 2.0) * si * costh * (3.0 - 7.0 * c2) / sqrt(20.0);
    if (mpole < 5) return;
    c4 = c2 * c2;
    dome[5] = (15.0 / 8.0) * si * (-1.0 + 14.0 * c2 - 21.0 * c4) / sqrt(30.0);
    if (mpole < 6) return;
    dome[6] = (21.0 / 8.0) * si * costh * (-5.0 + 30.0 * c2 - 33.0 * c4) / sqrt(42.0);
    if (mpole < 7) return;
    c6 = c4 * c2;
    dome[7] = (7.0 / 16.0) * si * (5.0 - 135.0 * c2 + 495.0 * c4 - 429.0 * c6) / sqrt(56.0);
    if (mpole < 8) return;
    dome[8] = (9.0 / 16.0) * si * costh * (35.0 - 385.0 * c2 + 1001.0 * c4 - 715.0 * c6) / sqrt(72.0);
  } else if (mt == 2) {
    c2 = costh * costh; si2 = fabs(1.0 - c2);
    dome[1] = 0.0;
    dome[2] = 3.0 * si2 / sqrt(24.0);
    if (mpole < 3) return;
    dome[3] = 15.0 * costh * si2 / sqrt(120.0);
    if (mpole < 4) return;
    c4 = c2 * c2;
    dome[4] = (15.0 / 2.0) * (-1.0 + 8.0 * c2 - 7.0 * c4) / sqrt(360.0);
    if (mpole < 5) return;
    dome[5] = (105.0 / 2.0) * costh * (-1.0 + 4.0 * c2 - 3.0 * c4) / sqrt(840.0);
    if (mpole < 6) return;
    c6 = c4 * c2;
    dome[6] = (105.0 / 8.0) * (1.0 - 19.0 * c2 + 51.0 * c4 - 33.0 * c6) / sqrt(1680.0);
    if (mpole < 7) return;
    dome[7] = (63.0 / 8.0) * costh * (15.0 - 125.0 * c2 + 253.0 * c4 - 143.0 * c6) / sqrt(3024.0);
    if (mpole < 8) return;
    c8 = c6 * c2;
    dome[8] = (315.0 / 8.0) * (-1.0 + 34.0 * c2 - 176.0 * c4 + 286.0 * c6 - 143.0 * c8) / sqrt(5040.0);
  } else if (mt == 3) {
    c2 = costh * costh; si2 = fabs(1.0 - c2); si = sqrt(si2); si3 = si2 * si;
    dome[1] = 0.0; dome[2] = 0.0;
    if (mpole < 3) return;
    dome[3] = -15.0 * si3 / sqrt(720.0);
    if (mpole < 4) return;
    dome[4] = -105.0 * si3 * costh / sqrt(5040.0);
    if (mpole < 5) return;
    dome[5] = -(105.0 / 2.0) * si3 * (-1.0 + 9.0 * c2) / sqrt(20160.0);
    if (mpole < 6) return;
    dome[6] = -(315.0 / 2.0) * si3 * costh * (-3.0 + 11.0 * c2) / sqrt(60480.0);
    if (mpole < 7) return;
    c4 = c2 * c2;
    dome[7] = -(315.0 / 8.0) * si3 * (3.0 - 66.0 * c2 + 143.0 * c4) / sqrt(151200.0);
    if (mpole < 8) return;
    dome[8] = -(3465.0 / 8.0) * si3 * costh * (3.0 - 26.0 * c2 + 39.0 * c4) / sqrt(332640.0);
  } else if (mt == 4) {
    dome[1] = 0.0; dome[2] = 0.0; dome[3] = 0.0;
    if (mpole < 4) return;
    c2 = costh * costh; c4 = c2 * c2;
    dome[4] = 105.0 * (1.0 - 2.0 * c2 + c4) / sqrt(40320.0);
    if (mpole < 5) return;
    dome[5] = 945.0 * costh * (1.0 - 2.0 * c2 + c4) / sqrt(362880.0);
    if (mpole < 6) return;
    c6 = c4 * c2;
    dome[6] = (945.0 / 2.0) * (-1.0 + 13 * c2 - 23.0 * c4 + 11.0 * c6) / sqrt(1814400.0);
    if (mpole < 7) return;
    dome[7] = (3465.0 / 2.0) * costh * (-3.0 + 19 * c2 - 29.0 * c4 + 13.0 * c6) / sqrt(6652800.0);
    if (mpole < 8) return;
    c8 = c6 * c2;
    dome[8] = (10395.0 / 8.0) * (1.0 - 28.0 * c2 + 118.0 * c4 - 156.0 * c6 + 65.0 * c8) / sqrt(19958400.0);
  }
}

/* vexch associated Legendre block: the reference's m=3 branch uses
 * sini = sini2 (not its square root), src/scfUtils.F90:1200-1203. */
static void vexch_dome(const x2o_state *s, int mt, double costh, double *dome) {
  if (mt != 3) {
    /* identical to mulex for mt != 3; mulex recomputes costh from (i,j) */
    int mpole = s->mpole;
    double c2, c4, c6, c8, si, si2;
    if (mt == 0) {
      dome[1] = costh;
      dome[2] = (3.0 * costh * costh - 1.0) * 0.50;
      for (int n = 2; n <= mpole - 1; n++)
        dome[n + 1] = ((double)(2 * n + 1) * costh * dome[n] - (double)n * dome[n - 1]) / (double)(n + 1);
    } else if (mt == 1) {
      c2 = costh * costh; si2 = fabs(1.0 - c2); si = sqrt(si2);
      dome[1] = -si / sqrt(2.0);
      dome[2] = -3.0 * si * costh / sqrt(6.0);
      if (mpole < 3) return;
      dome[3] = (3.0 / 2.0) * si * (1.0 - 5.0 * c2) / sqrt(12.0);
      if (mpole < 4) return;
      dome[4] = (5.0 / 2.0) * si * costh * (3.0 - 7.0 * c2) / sqrt(20.0);
      if (mpole < 5) return;
      c4 = c2 * c2;
      dome[5] = (15.0 / 8.0) * si * (-1.0 + 14.0 * c2 - 21.0 * c4) / sqrt(30.0);
      if (mpole < 6) return;
      dome[6] = (21.0 / 8.0) * si * costh * (-5.0 + 30.0 * c2 - 33.0 * c4) / sqrt(42.0);
      if (mpole < 7) return;
      c6 = c4 * c2;
      dome[7] = (7.0 / 16.0) * si * (5.0 - 135.0 * c2 + 495.0 * c4 - 429.0 * c6) / sqrt(56.0);
      if (mpole < 8) return;
      dome[8] = (9.0 / 16.0) * si * costh * (35.0 - 385.0 * c2 + 1001.0 * c4 - 715.0 * c6) / sqrt(72.0);
    } else if (mt == 2) {
      c2 = costh * costh; si2 = fabs(1.0 - c2);
      dome[1] = 0.0;
      dome[2] = 3.0 * si2 / sqrt(24.0);
      if (mpole < 3) return;
      dome[3] = 15.0 * costh * si2 / sqrt(120.0);
      if (mpole < 4) return;
      c4 = c2 * c2;
      dome[4] = (15.0 / 2.0) * (-1.0 + 8.0 * c2 - 7.0 * c4) / sqrt(360.0);
      if (mpole < 5) return;
      dome[5] = (105.0 / 2.0) * costh * (-1.0 + 4.0 * c2 - 3.0 * c4) / sqrt(840.0);
      if (mpole < 6) return;
      c6 = c4 * c2;
      dome[6] = (105.0 / 8.0) * (1.0 - 19.0 * c2 + 51.0 * c4 - 33.0 * c6) / sqrt(1680.0);
      if (mpole < 7) return;
      dome[7] = (63.0 / 8.0) * costh * (15.0 - 125.0 * c2 + 253.0 * c4 - 143.0 * c6) / sqrt(3024.0);
      if (mpole < 8) return;
      c8 = c6 * c2;
      dome[8] = (315.0 / 8.0) * (-1.0 + 34.0 * c2 - 176.0 * c4 + 286.0 * c6 - 143.0 * c8) / sqrt(5040.0);
    } else if (mt == 4) {
      dome[1] = 0.0; dome[2] = 0.0; dome[3] = 0.0;
      if (mpole < 4) return;
      c2 = costh * costh; c4 = c2 * c2;
      dome[4] = 105.0 * (1.0 - 2.0 * c2 + c4) / sqrt(40320.0);
      if (mpole < 5) return;
      dome[5] = 945.0 * costh * (1.0 - 2.0 * c2 + c4) / sqrt(362880.0);
      if (mpole < 6) return;
      c6 = c4 * c2;
      dome[6] = (945.0 / 2.0) * (-1.0 + 13 * c2 - 23.0 * c4 + 11.0 * c6) / sqrt(1814400.0);
      if (mpole < 7) return;
      dome[7] = (3465.0 / 2.0) * costh * (-3.0 + 19 * c2 - 29.0 * c4 + 13.0 * c6) / sqrt(6652800.0);
      if (mpole < 8) return;
      c8 = c6 * c2;
      dome[8] = (10395.0 / 8.0) * (1.0 - 28.0 * c2 + 118.0 * c4 - 156.0 * c6 + 65.0 * c8) / sqrt(19958400.0);
    }
    return;
  }
  int mpole = s->mpole;
  double c2 = costh * costh, si2 = fabs(1.0 - c2), si = si2, si3 = si2 * si, c4;
  dome[1] = 0.0; dome[2] = 0.0;
  if (mpole < 3) return;
  dome[3] = -15.0 * si3 / sqrt(720.0);
  if (mpole < 4) return;
  dome[4] = -105.0 * si3 * costh / sqrt(5040.0);
  if (mpole < 5) return;
  dome[5] = -(105.0 / 2.0) * si3 * (-1.0 + 9.0 * c2) / sqrt(20160.0);
  if (mpole < 6) return;
  dome[6] = -(315.0 / 2.0) * si3 * costh * (-3.0 + 11.0 * c2) / sqrt(60480.0);
  if (mpole < 7) return;
  c4 = c2 * c2;
  dome[7] = -(315.0 / 8.0) * si3 * (3.0 - 66.0 * c2 + 143.0 * c4) / sqrt(151200.0);
  if (mpole < 8) return;
  dome[8] = -(3465.0 / 8.0) * si3 * costh * (3.0 - 26.0 * c2 + 39.0 * c4) / sqrt(332640.0);
}

/* coulMom: src/scfUtils.F90:490-603 */
static void coul_mom(x2o_state *s) {
  int mx = s->mxsize, norb = s->norb;
  double *wk1 = s->w[1], *wk2 = s->w[2], *f4 = s->sup[8], *wgt2 = s->sup[13];
  int homo = s->lhomonucl && !s->lbreakCi;
  for (int iorb = 1; iorb <= norb; iorb++) {
    if (s->itouch[iorb] == 0) continue;
    const double *psi = s->psi[iorb];
    for (int i = 0; i < mx; i++) wk1[i] = psi[i] * psi[i];
    for (int i = 0; i < mx; i++) wk1[i] = wk1[i] * f4[i];
    for (int k = 1; k <= s->mpole; k++) {
      double v;
      if (homo && (k % 2 == 1)) v = 0.0;
      else {
        const double *dd = s->leg[k - 1];
        for (int i = 0; i < mx; i++) wk2[i] = dd[i] * wk1[i];
        v = ddot(mx, wgt2, wk2);
      }
      s->cmulti[iorb + (k - 1) * norb] = v;
    }
  }
}

/* exchMom: src/scfUtils.F90:615-844 */
static void exch_mom(x2o_state *s) {
  int mx = s->mxsize, nni = s->nni;
  double *wk1 = s->w[1], *wk2 = s->w[2], *f4 = s->sup[8], *wgt2 = s->sup[13];
  double *dd[MAXMPOLE];
  for (int k = 0; k < s->mpole; k++) dd[k] = dalloc(mx);
  for (int i = 1; i <= s->nexchmm; i++) {
    int idel = s->idelmm[i], iorb1 = s->iorb1mm[i], iorb2 = s->iorb2mm[i], ipc = s->ipcmm[i];
    for (int mu = 1; mu <= s->mxnmu; mu++)
      for (int ni = 1; ni <= nni; ni++) {
        double xrr = s->r2 * sqrt(s->vxisq[mu] + s->vetasq[ni] - 1.0);
        double dome[10];
        mulex(s, ni, mu, idel, dome);
        double xw = xrr;
        int ij = (mu - 1) * nni + (ni - 1);
        dd[0][ij] = dome[1] * xw;
        for (int k = 2; k <= s->mpole; k++) { xw = xw * xrr; dd[k - 1][ij] = dome[k] * xw; }
      }
    const double *p1 = s->psi[iorb1], *p2 = s->psi[iorb2];
    for (int j = 0; j < mx; j++) wk1[j] = p1[j] * p2[j];
    for (int j = 0; j < mx; j++) wk1[j] = wk1[j] * f4[j];
    for (int k = 0; k < s->mpole; k++) {
      for (int j = 0; j < mx; j++) wk2[j] = dd[k][j] * wk1[j];
      s->excm[k][ipc] = ddot(mx, wgt2, wk2);
    }
  }
  for (int k = 0; k < s->mpole; k++) free(dd[k]);
}

void x2o_mpole_moments(x2o_state *s, int all_touched) {
  if (all_touched) for (int i = 1; i <= s->norb; i++) s->itouch[i] = 1;
  if (s->nel == 1) return;
  coul_mom(s);
  if (s->nel > 1) exch_mom(s);
}

/* vcoul: src/scfUtils.F90:1039-1068 */
static double vcoul(const x2o_state *s, int iorb, int i, int j, double costh) {
  double rr = sqrt(s->vxisq[j] + s->vetasq[i] - 1.0);
  double rr1 = 1.0 / (rr * s->r2);
  double dome[10];
  dome[1] = costh;
  dome[2] = (3.0 * costh * costh - 1.0) * 0.5;
  for (int n = 2; n <= s->mpole - 1; n++)
    dome[n + 1] = ((double)(2 * n + 1) * costh * dome[n] - (double)n * dome[n - 1]) / (double)(n + 1);
  double pe = 0.0;
  for (int m = 1; m <= s->mpole; m++)
    pe = pe + s->cmulti[iorb + (m - 1) * s->norb] * dome[m] * pow(rr1, (double)(m + 1));
  return pe;
}

/* coulAsympt: src/scfUtils.F90:275-296 */
static void coul_asympt(const x2o_state *s, int iorb, double *pot) {
  int nni = s->nni;
  for (int j = s->mxnmu - 3; j <= s->mxnmu; j++)
    for (int i = 1; i <= nni; i++) {
      int kk = i + (j - 1) * nni - 1;
      double rr = sqrt(s->vxisq[j] + s->vetasq[i] - 1.0);
      double rr1 = 1.0 / (rr * s->r2);
      double costh = s->veta[i] * s->vxi[j] / rr;
      pot[kk] = s->r2 * s->vxi[j] * (rr1 + vcoul(s, iorb, i, j, costh));
    }
}

/* vexch + exchAsympt: src/scfUtils.F90:1075-1270, 310-329 */
static void exch_asympt(const x2o_state *s, int idel, int ipc, double *excp) {
  int nni = s->nni, mpole = s->mpole;
  for (int j = s->mxnmu - 3; j <= s->mxnmu; j++)
    for (int i = 1; i <= nni; i++) {
      int kk = i + (j - 1) * nni - 1;
      double pe[10] = {0};
      if (idel <= 4) {
        double rr = sqrt(s->vxisq[j] + s->vetasq[i] - 1.0);
        double costh = 0.0;
        if (fabs(rr) > PRECIS) costh = s->veta[i] * s->vxi[j] / rr;
        rr = rr * s->r2;
        double dome[10] = {0};
        vexch_dome(s, idel, costh, dome);
        double xrn = rr * rr;
        pe[1] = dome[1] * s->excm[0][ipc] / xrn;
        for (int k = 2; k <= mpole; k++) {
          xrn = xrn * rr;
          pe[k] = pe[k - 1] + dome[k] * s->excm[k - 1][ipc] / xrn;
        }
      }
      excp[kk] = s->r2 * s->vxi[j] * pe[mpole];
    }
}

/* potAsympt: src/scfUtils.F90:179-222 */
void x2o_pot_asympt(x2o_state *s, int iorb1) {
  if (s->itouch[iorb1] == 1) coul_asympt(s, iorb1, s->coul[iorb1]);
  for (int iorb2 = 1; iorb2 <= s->norb; iorb2++) {
    if (s->itouch[iorb1] == 0 && s->itouch[iorb2] == 0) continue;
    int k = s->k2[iorb1][iorb2];
    if (k == 0) continue;
    if (s->ilc[k] != 0) {
      int idel = abs(s->m[iorb1] - s->m[iorb2]);
      if (iorb1 == iorb2) idel = 2 * s->m[iorb1];
      exch_asympt(s, idel, k, s->exch[2 * k]);
      if (s->ilc[k] == 2) {
        idel = s->m[iorb2] + s->m[iorb1];
        exch_asympt(s, idel, k + s->norb * (s->norb + 1) / 2, s->exch[2 * k + 1]);
      }
    }
  }
}

/* ======================================================================== */
/* SCF driver (src/doSCF.F90)                                              */
/* ======================================================================== */

static void add_record(x2o_state *s, int iscf, int iorb) {
  if (s->nrec == s->caprec) {
    s->caprec = s->caprec ? 2 * s->caprec : 1024;
    s->rec = (rec_t *)realloc(s->rec, sizeof(rec_t) * s->caprec);
  }
  rec_t *r = &s->rec[s->nrec++];
  r->iscf = iscf; r->iorb = iorb; r->ee = s->ee[iorb][iorb]; r->dee = s->deltaee[iorb];
  r->dnorm = s->orbNorm[iorb] - 1.0;
}

static const char *bondname(const x2o_state *s, int i) { return s->bond[i]; }

/* the potentials of orbital iorb's batch (relaxDriver's first half) */
static void relax_pots_of(x2o_state *s, int iorb) {
  if (s->nexchpots[iorb] != 0 && !s->lfixexch) {
    if (s->pot_hook) {
      s->nsor4pot += (long)s->nexchpots[iorb] * s->maxsorpot[0] * s->maxsorpot[1];
      s->pot_hook(s->hook_ud, iorb);
    } else {
      for (int k = 1; k <= s->nexchpots[iorb]; k++) x2o_relax_pot(s, iorb, k, s->lpotmcsor ? 1 : 0);
    }
  }
}

/* relaxDriver: src/doSCF.F90:943-1011 (serial build); in the batched mode
 * the potentials were relaxed before the orbital loop */
static void relax_driver(x2o_state *s, int iorb) {
  if (!s->batch_pots) relax_pots_of(s, iorb);
  if (!s->lfixorb && s->batch_pots != 2) x2o_relax_orb(s, iorb, s->lorbmcsor ? 1 : 0);
}

/* batched orbitals (mode 2): every orbital relaxed with the Fock operator
 * of the state after the potentials, i.e. from the other orbitals' values at
 * that point; the relaxed orbitals replace the old ones together */
static void relax_all_orbitals(x2o_state *s) {
  const int norb = s->norb;
  double *keep[MAXORB + 1], *fresh[MAXORB + 1];
  for (int i = 1; i <= norb; i++) {
    const int iorb = norb - i + 1;
    keep[iorb] = s->psi[iorb];
    fresh[iorb] = dalloc(s->mxsize);
    memcpy(fresh[iorb], keep[iorb], sizeof(double) * s->mxsize);
    s->psi[iorb] = fresh[iorb];
    x2o_relax_orb(s, iorb, s->lorbmcsor ? 1 : 0);
    s->psi[iorb] = keep[iorb];
  }
  for (int iorb = 1; iorb <= norb; iorb++) {
    memcpy(keep[iorb], fresh[iorb], sizeof(double) * s->mxsize);
    free(fresh[iorb]);
  }
}

/* prepSCF: src/doSCF.F90:24-174 */
static void prep_scf(x2o_state *s) {
  double *fk1 = dalloc(s->mxsize), *fk2 = dalloc(s->mxsize);
  for (int iorb = 1; iorb <= s->norb; iorb++) x2o_fock(s, iorb, fk1, fk2);
  free(fk1); free(fk2);
  /* initAddData (hydrogenic start, doSCF.F90:73-134); a checkpoint start
   * keeps the stored norms, moments and Lagrange multipliers */
  if (!s->old_start) {
    for (int iorb = 1; iorb <= s->norb; iorb++) {
      int jorb = s->norb + 1 - iorb;
      x2o_norm(s, jorb);
      x2o_ortho(s, jorb);
    }
    for (int iorb = 1; iorb <= s->norb; iorb++) s->itouch[iorb] = 1;
    s->lmpoleInit = 1;
    x2o_mpole_moments(s, 0);
    for (int iorb = s->norb; iorb >= 1; iorb--) {
      x2o_eahf(s, iorb);
      s->eeOld[iorb] = s->ee[iorb][iorb];
      eabhf(s, iorb);
    }
  }
  x2o_etotal(s, NULL, NULL, NULL, NULL);
  if (s->verbose) {
    printf("     total energy:            %28.16E\n", s->etot);
    printf("     total electronic energy: %28.16E\n", s->evt);
    printf("     virial ratio:            %28.16E\n", s->virrat);
  }
}

static void scf_init(x2o_state *s) {
  s->orbEnergyThld = pow(10.0, (double)(-s->ienterm));
  s->orbNormThld = pow(10.0, (double)(-s->inoterm));
  s->thren4init = pow(10.0, (double)(-s->ienterm4init));
  s->nresets = 0; s->nresets4no = 0; s->nOrbEnergyThld = 0; s->nOrbNormThld = 0;
  s->eeconv = 10.0;
  for (int i = 1; i <= s->norb; i++) {
    s->itouch[i] = 0; s->deltaee[i] = 0.0; s->eeOld[i] = s->ee[i][i]; s->deltaNorm[i] = 0.0;
  }
  s->demax1 = 100.0; s->deltaeeMax = 100.0; s->deltaNormMax = 100.0;
  s->lenergyThld = 0; s->lnormThld = 0; s->lmpoleInit = 0; s->ldemax0 = 1;
  s->eeconvprev = 1.e35; s->dnmaxprev = 1.e35; s->noenergydec = 0; s->nonormdec = 0;
  if (s->lhomonucl && !s->lbreakCi) setci(s, 0);
  s->iscf = 0;
}

/* one SCF iteration; returns 1 when the SCF loop terminates */
static int scf_iteration(x2o_state *s) {
  int norb = s->norb;
  int iscf = ++s->iscf;
  int iasympt = norb;
  if (s->batch_pots) {
    /* batched mode (no reference counterpart): every potential's boundary
     * values, then every orbital's potential batch, all from the orbitals at
     * the start of the iteration; the orbitals follow in relaxDriver order */
    for (int i = 1; i <= norb; i++) {
      int iorb = norb - i + 1;
      s->itouch[iorb] = 1;
      if (iasympt != 0 && s->ifixorb[iorb] == 0) { x2o_pot_asympt(s, iorb); iasympt--; }
    }
    s->isstart = 1; s->isstop = s->ngrid1; s->isstep = 1;
    for (int i = 1; i <= norb; i++) relax_pots_of(s, norb - i + 1);
    if (s->batch_pots == 2 && !s->lfixorb) relax_all_orbitals(s);
  }
  for (int i = 1; i <= norb; i++) {
    int iorb = norb - i + 1;
    s->itouch[iorb] = 1;
    if (!s->batch_pots && iasympt != 0 && s->ifixorb[iorb] == 0) { x2o_pot_asympt(s, iorb); iasympt--; }
    s->isstart = 1; s->isstop = s->ngrid1; s->isstep = 1;
    if (s->altSweeps && (iorb % 2 != 0)) { s->isstart = s->ngrid1; s->isstop = 1; s->isstep = -1; }
    relax_driver(s, iorb);
    if (s->ifixorb[iorb] == 0) x2o_norm(s, iorb);
    if (s->lhomonucl && !s->lbreakCi) setci(s, iorb);
    if (norb > 1 && s->ifixorb[iorb] == 0) x2o_ortho(s, iorb);
    if (s->ifixorb[iorb] != 0) {
      double *fk1 = s->w[6], *fk2 = dalloc(s->mxsize);
      double *tmp = dalloc(s->mxsize);
      x2o_fock(s, iorb, tmp, fk2);
      free(tmp); free(fk2); (void)fk1;
    }
    x2o_eahf(s, iorb);
    s->deltaee[iorb] = s->ee[iorb][iorb] - s->eeOld[iorb];
    if (fabs(s->deltaee[iorb]) < PRECIS) s->deltaee[iorb] = 2.0 * s->orbEnergyThld;
    s->eeOld[iorb] = s->ee[iorb][iorb];
    eabhf(s, iorb);
    add_record(s, iscf, iorb);
    if (s->verbose && s->verboseLevel >= 3)
      printf("%5d%4d %-8s%c  %23.16E%16.2E%16.2E%16.2E\n", iscf, s->iorn[iorb], bondname(s, iorb),
             s->gusym[iorb], s->ee[iorb][iorb], s->deltaee[iorb], s->orbNorm[iorb] - 1.0, s->wstorthog[iorb]);
  }
  s->deltaeeMax = 0.0; s->deltaNormMax = 0.0;
  for (int nei = 1; nei <= norb; nei++)
    if (fabs(s->deltaee[nei]) >= fabs(s->deltaeeMax)) s->deltaeeMax = s->deltaee[nei];
  for (int nei = 1; nei <= norb; nei++) {
    s->deltaNorm[nei] = fabs(s->orbNorm[nei] - 1.0);
    if (s->ifixorb[nei] == 0 && s->deltaNorm[nei] >= s->deltaNormMax) {
      s->deltaNormMax = s->deltaNorm[nei];
      if (fabs(s->deltaNormMax) < PRECIS) s->deltaNormMax = PRECIS;
    }
  }
  if (fabs(s->eeconv) < PRECIS) s->eeconv = s->deltaeeMax;
  if (iscf > s->nscf2skip) {
    if (fabs(s->deltaeeMax) >= fabs(s->eeconvprev)) s->noenergydec++;
    else { s->eeconvprev = s->deltaeeMax; s->noenergydec = 0; }
    if (fabs(s->deltaNormMax) >= fabs(s->dnmaxprev)) s->nonormdec++;
    else { s->dnmaxprev = s->deltaNormMax; s->nonormdec = 0; }
    if (s->noenergydec > s->nenlast || s->nonormdec > s->nnolast) {
      if (s->verbose) printf(" ... solution cannot be further improved ...\n");
      return 1;
    }
  } else {
    s->eeconvprev = s->demax1;
    s->dnmaxprev = s->deltaNormMax;
  }
  if (fabs(s->demax1) > s->orbEnergyIncThld) return 1;
  if (iscf == s->maxscf) {
    if (s->verbose) printf(" ... scf iteration limit reached ... \n");
    return 1;
  }
  if (s->lfixorb4init && fabs(s->deltaeeMax) < s->thren4init) {
    if (s->nOrbEnergyThld == s->nscfExtra) {
      if (s->verbose) printf(" ... initial relaxation of potentials with fixed orbitals reached the threshold ...\n");
      for (int i = 1; i <= norb; i++) s->ifixorb[i] = 0;
      s->lfixorb = 0; s->lfixorb4init = 0;
      s->eeconv = 10.0; s->deltaeeMax = 100.0;
    } else s->nOrbEnergyThld++;
  }
  if (!s->lenergyThld) {
    if (fabs(s->deltaeeMax) < s->orbEnergyThld) {
      s->lenergyThld = 1; s->eeconv = s->deltaeeMax;
      for (int i = 1; i <= norb; i++) s->itouch[i] = 0;
      s->nOrbEnergyThld = 0;
    }
  } else {
    if (fabs(s->deltaeeMax) < s->orbEnergyThld) {
      if (s->nOrbEnergyThld == s->nscfExtra) {
        if (s->verbose) printf(" ... orbital energy threshold reached ...\n");
        return 1;
      }
      s->nOrbEnergyThld++;
    } else if (fabs(s->deltaNormMax) < s->orbNormThld) {
      if (s->nOrbNormThld == s->nscfExtra) {
        if (s->verbose) printf(" ... orbital normalization threshold reached ...\n");
        return 1;
      }
      s->nOrbNormThld++;
    } else {
      s->lenergyThld = 0;
      if (s->nresets > s->maxresets) return 1;
      s->nresets++;
    }
  }
  if (!s->lfixorb) {
    if (!s->lnormThld) {
      if (fabs(s->deltaNormMax) < s->orbNormThld) {
        s->lnormThld = 1;
        for (int i = 1; i <= norb; i++) s->itouch[i] = 0;
        s->nOrbNormThld = 0;
      }
    } else {
      if (fabs(s->deltaNormMax) < s->orbNormThld) {
        if (s->nOrbNormThld == s->nscfExtra) {
          if (s->verbose) printf(" ... orbital normalization threshold reached ...\n");
          return 1;
        }
        s->nOrbNormThld++;
      } else {
        s->lnormThld = 0;
        if (s->nresets4no > s->maxresets) return 1;
        s->nresets4no++;
      }
    }
  }
  if (fabs(s->eeconv / s->deltaeeMax) > s->recalcMMfactor) {
    s->eeconv = s->deltaeeMax;
    x2o_mpole_moments(s, 0);
    if (s->verbose && s->verboseLevel > 2) printf(" ... multipole moment expansion coefficients recalculated ...\n");
  }
  for (int i = 1; i <= norb; i++) s->itouch[i] = 0;
  if (s->saveScfData > 0 && iscf % s->saveScfData == 0) {
    x2o_etotal(s, NULL, NULL, NULL, NULL);
    if (s->verbose) printf("\n       total energy: %23.16E\n\n", s->etot);
  }
  return 0;
}

/* end of scf(): src/doSCF.F90:790-860 */
static void scf_finish(x2o_state *s) {
  if (s->norb > 1) {
    double keep[MAXORB + 1];
    for (int i = 1; i <= s->norb; i++) keep[i] = s->orbNorm[i];
    for (int iorb = 1; iorb <= s->norb; iorb++) {
      int jorb = s->norb + 1 - iorb;
      x2o_norm(s, jorb);
      x2o_ortho(s, jorb);
    }
    for (int i = 1; i <= s->norb; i++) s->orbNorm[i] = keep[i];
  }
  for (int iorb = s->norb; iorb >= 1; iorb--) { x2o_eahf(s, iorb); eabhf(s, iorb); }
  x2o_mpole_moments(s, 0);
  x2o_etotal(s, NULL, NULL, NULL, NULL);
  if (s->verbose) {
    printf("     total energy:            %28.16E\n", s->etot);
    printf("     total electronic energy: %28.16E\n", s->evt);
    printf("     virial ratio:            %28.16E\n", s->virrat);
    printf("     (MC)SOR iterations:            %8ld\n", s->nsor4orb + s->nsor4pot);
  }
}

int x2o_scf_steps(x2o_state *s, int n, int verbose) {
  s->verbose = verbose;
  if (!s->scf_started) {
    prep_scf(s);
    scf_init(s);
    s->scf_started = 1;
  }
  for (int k = 0; k < n && !s->scf_done; k++) {
    if (scf_iteration(s)) {
      s->scf_done = 1;
      scf_finish(s);
    }
  }
  return s->scf_done;
}

int x2o_run_scf(x2o_state *s, int verbose) {
  while (!x2o_scf_steps(s, 1 << 30, verbose)) {}
  return s->iscf;
}

/* ======================================================================== */
/* accessors                                                               */
/* ======================================================================== */

int x2o_nni(const x2o_state *s) { return s->nni; }
int x2o_nmu(const x2o_state *s) { return s->mxnmu ? s->mxnmu : s->nmu; }
int x2o_norb(const x2o_state *s) { return s->norb; }
int x2o_iterations(const x2o_state *s) { return s->iscf; }
double x2o_total_energy(const x2o_state *s) { return s->etot; }
double x2o_orbital_energy(const x2o_state *s, int iorb) { return s->ee[iorb][iorb]; }
double x2o_omega_orb(const x2o_state *s) { return s->ovforb; }
double x2o_omega_pot(const x2o_state *s) { return s->ovfexch; }
long x2o_sweeps(const x2o_state *s) { return s->nsor4orb + s->nsor4pot; }
int x2o_nrecords(const x2o_state *s) { return s->nrec; }
void x2o_record(const x2o_state *s, int i, int *iscf, int *iorb, double *ee, double *dee, double *dnorm) {
  const rec_t *r = &s->rec[i];
  *iscf = r->iscf; *iorb = r->iorb; *ee = r->ee; *dee = r->dee; *dnorm = r->dnorm;
}
int x2o_ngrid(const x2o_state *s, int *g1, int *g6a, int *g6b, int *g7) {
  *g1 = s->ngrid1; *g6a = s->ngrid6a; *g6b = s->ngrid6b; *g7 = s->ngrid7;
  return s->mxsize8;
}
void x2o_lists(const x2o_state *s, int *i1, int *i2, int *i6a, int *i6b, int *i7) {
  memcpy(i1, s->indx1, sizeof(int) * s->ngrid1);
  memcpy(i2, s->indx2, sizeof(int) * s->ngrid1);
  memcpy(i6a, s->indx6a, sizeof(int) * s->ngrid6a);
  memcpy(i6b, s->indx6b, sizeof(int) * s->ngrid6b);
  memcpy(i7, s->indx7, sizeof(int) * s->ngrid7);
}
void x2o_suppl(const x2o_state *s, int which, double *out) { memcpy(out, s->sup[which], sizeof(double) * s->mxsize); }
void x2o_coeffs(const x2o_state *s, double *dmu1, double *dmu2, double *dni1, double *dni2, double *exeven,
                double *diag) {
  memcpy(dmu1, s->dmu1, 32); memcpy(dmu2, s->dmu2, 32); memcpy(dni1, s->dni1, 32); memcpy(dni2, s->dni2, 32);
  memcpy(exeven, s->exeven, 40); *diag = s->diag;
}
void x2o_get_orbital(const x2o_state *s, int iorb, double *out) { memcpy(out, s->psi[iorb], sizeof(double) * s->mxsize); }
/* multipole moments of an orbpot old start, as the checkpoint stores them
 * (readFuncs, diskInterface.F90:350-390): cmulti(iorb + (k-1) norb) for
 * MAXORB*MAXMPOLE entries, then excdi, excqu, ..., exc8 by pair index ipc,
 * MAXORB*(MAXORB+1) entries each */
void x2o_set_moments(x2o_state *s, const double *cmulti, const double *exc) {
  for (int i = 1; i <= MAXMPOLE * MAXORB; i++) s->cmulti[i] = cmulti[i - 1];
  for (int k = 0; k < MAXMPOLE; k++)
    for (int i = 1; i <= MAXORB * (MAXORB + 1); i++) s->excm[k][i] = exc[k * MAXORB * (MAXORB + 1) + i - 1];
}

/* ee(iorb,iorb) of an orbpot old start (readFuncs, diskInterface.F90:335-337) */
void x2o_set_orbital_energy(x2o_state *s, int iorb, double ee) { s->ee[iorb][iorb] = ee; }

void x2o_set_orbital(x2o_state *s, int iorb, const double *in) { memcpy(s->psi[iorb], in, sizeof(double) * s->mxsize); }
int x2o_npots(const x2o_state *s, int iorb) { return s->nexchpots[iorb]; }
void x2o_pot_info(const x2o_state *s, int iorb, int k, int *in1, int *in2, int *idel, int *isym) {
  *in1 = s->ins1[iorb][k]; *in2 = s->ins2[iorb][k]; *idel = s->deltam4pot[iorb][k]; *isym = s->isyms[iorb][k];
}
void x2o_get_pot(const x2o_state *s, int iorb, int k, double *out) {
  memcpy(out, s->pottarget[iorb][k], sizeof(double) * s->mxsize);
}
void x2o_set_pot(x2o_state *s, int iorb, int k, const double *in) {
  memcpy(s->pottarget[iorb][k], in, sizeof(double) * s->mxsize);
}
void x2o_cmulti(const x2o_state *s, double *out) {
  for (int k = 1; k <= s->mpole; k++)
    for (int i = 1; i <= s->norb; i++) out[(k - 1) * s->norb + (i - 1)] = s->cmulti[i + (k - 1) * s->norb];
}

/* batched-potential mode on (1) or off (0, the reference's order) */
void x2o_set_batch_potentials(x2o_state *s, int on) { s->batch_pots = (on >= 0 && on <= 2) ? on : 0; }

void x2o_set_hooks(x2o_state *s, void (*pot_hook)(void *, int),
                   void (*orb_hook)(void *, int, int, double *, double *, double *), void *ud) {
  s->pot_hook = pot_hook;
  s->orb_hook = orb_hook;
  s->hook_ud = ud;
}
double *x2o_orbital_block(x2o_state *s) { return s->orbblock; }
double *x2o_potential_block(x2o_state *s) { return s->potblock; }
long x2o_pot_offset(const x2o_state *s, int iorb, int k) { return (long)(s->pottarget[iorb][k] - s->potblock) + 1; }

void x2o_free(x2o_state *s) {
  if (!s) return;
  if (s->psi) {
    for (int i = 1; i <= s->norb; i++) {
      free(s->coulombptr[i]); free(s->exchangeptr[i]);
    }
    free(s->psi); free(s->coul); free(s->coulombptr); free(s->exchangeptr);
    free(s->exch);
    free(s->orbblock); free(s->potblock);
  }
  double *arrs[] = {s->vmu, s->vxi, s->vxisq, s->vxi1, s->vxi2, s->vni, s->veta, s->vetasq, s->veta1, s->veta2,
                    s->wmu, s->wni, s->dmu9, s->dni9};
  for (unsigned i = 0; i < sizeof(arrs) / sizeof(arrs[0]); i++) free(arrs[i]);
  for (int k = 0; k < 14; k++) free(s->sup[k]);
  for (int k = 0; k < MAXMPOLE; k++) free(s->leg[k]);
  for (int k = 0; k < 8; k++) free(s->w[k]);
  free(s->indx1); free(s->indx2); free(s->indx6a); free(s->indx6b); free(s->indx7);
  free(s->rec);
  free(s);
}
