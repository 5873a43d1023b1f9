// Device-resident closed-shell HF SCF of x2dhf (src/doSCF.F90 prepSCF:24,
// scf:211, relaxDriver:943).  Orbitals, Coulomb and exchange potentials live
// on the GPU in the extended layout for the whole run; the host keeps only
// the scalar control of the reference's SCF loop and reads back a few
// scalars (orbital energies, norms, overlaps) once per SCF iteration.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "x2g_kernels.cuh"

using namespace x2g;

namespace {

constexpr int MAXO = X2G_MAXORB;

struct Rec {
  int iscf, iorb;
  double ee, dee, dnorm;
};

// one potential of an orbital's relaxation batch (initAddr:1339-1461)
struct PotSlot {
  int in1, in2, idel, isym;
  double *target;  // ext array
};

}  // namespace

struct x2g_scf {
  x2g_ctx *ctx = nullptr;
  x2g_grid *grid = nullptr;
  x2g_case cs{};
  int norb = 0, nel = 0, mpole = 4, nslots = 0;
  int m[MAXO + 1]{}, isymOrb[MAXO + 1]{}, ihomo[MAXO + 1]{}, ige[MAXO + 1]{};
  double occ[MAXO + 1]{};
  double gec[2 * MAXO * MAXO + 1]{};
  int k2[MAXO + 1][MAXO + 1]{}, ilc2[MAXO + 1][MAXO + 1]{};
  std::vector<int> ilc;
  std::vector<double *> orb, coul, coulp, exchp, exch;  // device arrays
  double *lhs = nullptr, *rhs = nullptr, *fa = nullptr, *edecay = nullptr;
  // batch_mode 2: per-orbital Fock outputs (lhs, rhs, fock1/f1 tail, decay)
  std::vector<double *> blhs, brhs, bfa, bedecay;
  double *sc = nullptr;  // device scalars
  // scalar block offsets (doubles)
  enum { O_EE = 0, O_NORM = 64, O_OVL = 128, O_CM = 128 + 64 * 64, O_EX = O_CM + 64 * 8 };
  size_t sc_count = 0;
  double *hsc = nullptr;  // pinned host copy of the first O_CM scalars
  std::vector<std::vector<PotSlot>> pots;
  // exchange-moment list (initLP:1592-1626)
  std::vector<int> mm_i1, mm_i2, mm_idel, mm_ipc;
  std::vector<void *> allocs;
  double omega_orb = 0, omega_pot = 0;
  // SCF control (doSCF.F90:211-886)
  int started = 0, done = 0, iscf = 0, converged = 0;
  int ifixorb[MAXO + 1]{}, itouch[MAXO + 1]{};
  int lfixorb = 0, lfixorb4init = 0;
  double ee[MAXO + 1]{}, eeOld[MAXO + 1]{}, deltaee[MAXO + 1]{}, orbNorm[MAXO + 1]{}, wst[MAXO + 1]{};
  double deltaeeMax = 100, deltaNormMax = 100, eeconv = 10, eeconvprev = 1e35, dnmaxprev = 1e35, demax1 = 100;
  double orbEnergyThld = 0, orbNormThld = 0, thren4init = 0;
  int nresets = 0, nresets4no = 0, nOrbEnergyThld = 0, nOrbNormThld = 0, noenergydec = 0, nonormdec = 0;
  int lenergyThld = 0, lnormThld = 0;
  long nsor4orb = 0, nsor4pot = 0;
  double etot = 0, evt = 0, virial = 0;
  std::vector<Rec> recs;
  int last_error = 0;
};

namespace {

double *dalloc(x2g_scf *s, size_t n) {
  void *p = nullptr;
  if (cudaMalloc(&p, n * sizeof(double)) != cudaSuccess) return nullptr;
  // on the context's stream: its kernels are not ordered after the legacy
  // default stream (the stream is non-blocking)
  cudaMemsetAsync(p, 0, n * sizeof(double), s->ctx->stream);
  s->allocs.push_back(p);
  return static_cast<double *>(p);
}

// ---------------------------------------------------------------------
// hydrogenic start (initOrbitalsPotentials.F90:714-934) and initial
// potentials (coulombExchangePotentials.f90:14-239), evaluated on the
// device, one elementwise launch per function; the orbital-constant
// prefactors are formed on the host
// ---------------------------------------------------------------------
// unfused product and sum on both sides: the device compiler would
// otherwise contract a*b+c into one rounding, unlike the host build
__host__ __device__ inline double mul_rn(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dmul_rn(a, b);
#else
  return a * b;
#endif
}
__host__ __device__ inline double add_rn(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dadd_rn(a, b);
#else
  return a + b;
#endif
}

__host__ __device__ inline double factorial(int n) {
  double f = 1.0;
  for (int i = 1; i <= n; i++) f = double(i) * f;
  return f;
}

__host__ __device__ inline double hyp1f1(int np, int lp, double x) {  // utils.f90:265-282
  double h = 1.0;
  if (-np == 0) return h;
  double t = double(np) * x / double(lp);
  h = h + t;
  for (int i = 2; i <= -np; i++) {
    t = t * x * double(np + i - 1) / double(lp + i - 1) / double(i);
    h = h + t;
  }
  return h;
}

__host__ __device__ inline double hyp2f1(int na, int nb, int nc, double x) {  // utils.f90:289-309
  double h = 1.0;
  if (na == 0) return h;
  double a = na, b = nb, c = nc;
  double t = a * b * x / c;
  h = h + t;
  for (int i = 2; i <= -na; i++) {
    t = t * x * (a + double(i - 1)) * (b + double(i - 1)) / (c + double(i - 1)) / double(i);
    h = h + t;
  }
  return h;
}

// associated Legendre as evaluated by plegendg (utils.f90:315-335); its
// prefactor is written (-one**m), i.e. always -1 in Fortran precedence
__host__ __device__ inline double plegendre(int l, int m, double c) {
  double ct = fabs(add_rn(1.0, -mul_rn(c, c)));
  if (m == 0) return hyp2f1(-l, l + 1, 1, (1.0 - c) / 2.0);
  if (ct < kPrecis) return 0.0;
  double fn0 = -pow(1.0, double(m)) * factorial(l + m) / factorial(l - m) / factorial(m) / pow(2.0, double(m));
  return hyp2f1(m - l, m + l + 1, m + 1, (1.0 - c) / 2.0) * (fn0 * pow(ct, double(m) / 2.0));
}

// one hydrogenic function |n l m> of charge z on centre A or B
struct HydroTerm {
  int n, l, use, centre_b;
  double z, co, fn, shn;
};
struct GuessOrbital {
  HydroTerm t[2];
  int m;
};

HydroTerm hydro_term(int n, int l, int m, double z, double co, bool centre_b) {
  HydroTerm t{};
  t.n = n;
  t.l = l;
  t.z = z;
  t.co = co;
  t.centre_b = centre_b;
  t.use = std::fabs(co) > kPrecis;
  t.fn = std::pow(2.0 * z / double(n), 3.0 / 2.0 + double(l)) *
         std::sqrt(factorial(n + l) / (2.0 * double(n) * factorial(n - l - 1))) / factorial(2 * l + 1);
  t.shn = (m == 0 ? 1.0 : std::pow(-1.0, double(m))) / std::sqrt(4.0 * kPi) *
          std::sqrt((2.0 * l + 1.0) * factorial(l - m) / factorial(l + m));
  return t;
}

__device__ double hydro_value(const HydroTerm &t, int m, double r, double xi, double eta) {
  const double z0 = (r / 2.0) * xi * eta;
  double rt, c;
  if (!t.centre_b) {
    rt = (r / 2.0) * (xi + eta);
    c = (rt < kPrecis) ? -1.0 : fmin(1.0, fmax(-1.0, (z0 + r / 2.0) / rt));
  } else {
    rt = (r / 2.0) * (xi - eta);
    c = (rt < kPrecis) ? -1.0 : fmin(1.0, fmax(-1.0, -(z0 - r / 2.0) / rt));
  }
  const int np = t.n - t.l - 1, lp = 2 * t.l + 2;
  const double x = t.z * rt / double(t.n);
  const double lag = __dmul_rn(__dmul_rn(pow(rt, double(t.l)), exp(-x)), hyp1f1(-np, lp, x + x));
  return __dmul_rn(__dmul_rn(__dmul_rn(t.fn, lag), t.shn), plegendre(t.l, m, c));
}

// pottf, coulombExchangePotentials.f90:222-239
__host__ __device__ inline double thomas_fermi(double r, double veta, double vxi) {
  if (fabs(vxi + veta) < kPrecis) return 0.0;
  double rab = r * (vxi + veta) / 2.0;
  double w = sqrt(rab / 0.885340);
  double t = add_rn(mul_rn(w, add_rn(mul_rn(0.6011200, w), 1.8106100)), 1.0);
  double p = add_rn(mul_rn(0.0479300, w), 0.2146500);
  p = add_rn(mul_rn(w, p), 0.7711200);
  p = add_rn(mul_rn(w, p), 1.3951500);
  p = add_rn(mul_rn(w, p), 1.8106100);
  w = add_rn(mul_rn(w, p), 1.0);
  return add_rn(1.0, -mul_rn(t / w, t / w)) / rab;
}

// orbital: co1 |n1 l1 m>_A + co2 |n2 l2 m>_B on the interior of ext
__global__ void k_guess_orbital(GridDev g, double r, GuessOrbital a, double *ext) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < g.mxsize; k += gridDim.x * blockDim.x) {
    const int i = k / g.nni, j = k - i * g.nni;
    double psi = 0.0;
    for (int p = 0; p < 2; p++)
      if (a.t[p].use) psi = __dadd_rn(__dmul_rn(a.t[p].co, hydro_value(a.t[p], a.m, r, g.vxi[i], g.veta[j])), psi);
    ext[(i + 4) * g.n8 + j + 4] = psi;
  }
}

// Coulomb potential: -(TF_A crt1 + TF_B crt2) f4 (initCoulomb)
__global__ void k_guess_coulomb(GridDev g, double r, double crt1, double crt2, int both, double *ext) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < g.mxsize; k += gridDim.x * blockDim.x) {
    const int i = k / g.nni, j = k - i * g.nni;
    double v;
    if (i == 0 && (j == 0 || j == g.nni - 1))
      v = 0.0;
    else if (both)
      v = __dadd_rn(__dmul_rn(-1.0 * thomas_fermi(r, g.veta[j], g.vxi[i]), crt1),
                    __dmul_rn(-1.0 * thomas_fermi(r, -g.veta[j], g.vxi[i]), crt2));
    else
      v = __dmul_rn(-1.0 * thomas_fermi(r, g.veta[j], g.vxi[i]), crt1);
    ext[(i + 4) * g.n8 + j + 4] = __dmul_rn(v, g.f4[k]);
  }
}

// exchange potential: (co1/r_A + co2/r_B) f4 off the axis rows/columns
// (initExchange); ext2, when set, receives the same values
__global__ void k_guess_exchange(GridDev g, double r, double co1, double co2, double *ext, double *ext2) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < g.mxsize; k += gridDim.x * blockDim.x) {
    const int i = k / g.nni, j = k - i * g.nni;
    double v = 0.0;
    if (i >= 1 && j >= 1 && j < g.nni - 1) {
      const double ra1 = (r / 2.0) * (g.vxi[i] + g.veta[j]), ra2 = (r / 2.0) * (g.vxi[i] - g.veta[j]);
      v = (ra1 > 1.0e-8) ? co1 / ra1 : 0.0;
      if (ra2 > 1.0e-8) v = __dadd_rn(v, co2 / ra2);
    }
    v = __dmul_rn(v, g.f4[k]);
    ext[(i + 4) * g.n8 + j + 4] = v;
    if (ext2) ext2[(i + 4) * g.n8 + j + 4] = v;
  }
}

int upload_ext(x2g_scf *s, double *dst, const std::vector<double> &plain) {
  const HostGrid &g = s->grid->h;
  std::vector<double> ext(g.next, 0.0);
  for (int i = 0; i < g.nmu; i++)
    for (int j = 0; j < g.nni; j++) ext[(i + 4) * g.n8 + j + 4] = plain[i * g.nni + j];
  cudaError_t e =
      cudaMemcpyAsync(dst, ext.data(), ext.size() * sizeof(double), cudaMemcpyHostToDevice, s->ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->ctx->stream);  // ext is freed on return
  count_copy(s->ctx, ext.size() * sizeof(double), 0);
  return e == cudaSuccess ? X2G_OK : cuda_status(e, "function upload");
}

int initial_guess(x2g_scf *s) {
  const HostGrid &h = s->grid->h;
  const GridDev &g = s->grid->d;
  const x2g_case &c = s->cs;
  const int blocks = (h.mxsize + 255) / 256 < 1184 ? (h.mxsize + 255) / 256 : 1184;
  cudaStream_t st = s->ctx->stream;
  for (int o = 1; o <= s->norb; o++) {
    const int k = o - 1;
    GuessOrbital a{};
    a.m = s->m[o];
    a.t[0] = hydro_term(c.n1[k], c.l1[k], s->m[o], c.za[k], c.co1[k], false);
    a.t[1] = hydro_term(c.n2[k], c.l2[k], s->m[o], c.zb[k], c.co2[k], true);
    k_guess_orbital<<<blocks, 256, 0, st>>>(g, h.r, a, s->orb[o]);
  }
  const int iz1 = int(std::lround(h.z1)), iz2 = int(std::lround(h.z2));
  for (int o = 1; o <= s->norb; o++) {
    const int k = o - 1;
    k_guess_coulomb<<<blocks, 256, 0, st>>>(g, h.r, std::fabs(c.co1[k]), std::fabs(c.co2[k]),
                                            (iz1 != 0 && iz2 != 0) ? 1 : 0, s->coul[o]);
  }
  for (int i1 = 1; i1 <= s->norb; i1++)
    for (int i2 = i1; i2 <= s->norb; i2++) {
      if (i1 == i2 && s->m[i2] == 0) continue;
      const int kk = s->k2[i1][i2];
      double *second = (i1 != i2 && s->m[i1] != 0 && s->m[i2] != 0) ? s->exch[2 * kk + 1] : nullptr;
      k_guess_exchange<<<blocks, 256, 0, st>>>(g, h.r, c.co1[i1 - 1], c.co2[i1 - 1], s->exch[2 * kk], second);
      s->ctx->launches += 1;
    }
  s->ctx->launches += 2 * s->norb;  // orbitals and Coulomb potentials
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return e == cudaSuccess ? X2G_OK : cuda_status(e, "initial guess");
}

// exchange weights of a closed-shell configuration (initExWeights:3303-3436)
void exchange_weights(x2g_scf *s) {
  const int norb = s->norb, isu2 = norb * norb;
  char spn[4 * MAXO + 1];
  int iloop[MAXO + 1], iqm[4 * MAXO + 1];
  for (int i = 1; i <= norb; i++) {
    int is = 4 * (i - 1);
    iloop[i] = 2;
    iqm[1 + is] = 1;
    iqm[2 + is] = 1;
    spn[is + 1] = '+';
    spn[is + 2] = '-';
    spn[is + 3] = ' ';
    spn[is + 4] = ' ';
    if (s->m[i] > 0) {
      iloop[i] = 4;
      iqm[3 + is] = -1;
      iqm[4 + is] = -1;
      spn[is + 3] = '+';
      spn[is + 4] = '-';
    }
  }
  std::fill(std::begin(s->gec), std::end(s->gec), 0.0);
  for (int i = 1; i <= norb; i++) {
    int ixx = 4 * (i - 1);
    double div = 0.0;
    for (int ii = 1; ii <= iloop[i]; ii++) {
      int ix = ii + ixx;
      div += 1.0;
      for (int j = 1; j <= norb; j++) {
        int jxx = 4 * (j - 1), kk = i + norb * (j - 1);
        int mpl = std::abs(s->m[i] - s->m[j]), mmi = std::abs(s->m[i] + s->m[j]);
        for (int jj = 1; jj <= iloop[j]; jj++) {
          int jx = jxx + jj;
          if (mpl == mmi && spn[ix] == spn[jx] && i != j) s->gec[kk] += 1.0;
          if (mpl != mmi && spn[ix] == spn[jx]) {
            if (i == j && iqm[ix] != iqm[jx]) s->gec[kk] += 1.0;
            if (i != j && iqm[ix] == iqm[jx]) s->gec[kk] += 1.0;
            if (i != j && iqm[ix] != iqm[jx]) s->gec[kk + isu2] += 1.0;
          }
        }
      }
    }
    for (int idiv = 1; idiv <= norb; idiv++) {
      int kk = i + norb * (idiv - 1);
      s->gec[kk] = s->gec[kk] / div;
      s->gec[kk + isu2] = s->gec[kk + isu2] / div;
    }
  }
}

// ---------------------------------------------------------------------
// device operations of one SCF step
// ---------------------------------------------------------------------
// fockHF of orbital iorb into lhs (fock1 + diag), rhs (fock2) and fa
// (fock1/f1 on the last 5 mu rows)
FockArgs fock_args(x2g_scf *s, int iorb, double *lhs, double *rhs, double *fa) {
  FockArgs a{};
  a.m = s->m[iorb];
  a.nel1 = (s->nel == 1);
  a.exact = (s->cs.precision == X2G_FP64);
  a.ee = s->sc + x2g_scf::O_EE + iorb;
  a.lhs = lhs;
  a.rhs = rhs;
  a.coulp = s->coulp[iorb];
  a.exchp = s->exchp[iorb];
  a.fa = fa;
  int n = 0;
  for (int j = 1; j <= s->norb; j++) {
    FockTerm &t = a.t[n++];
    t.coul = s->coul[j];
    t.coo = s->occ[j] - (j == iorb ? 1.0 : 0.0);
    const int kex = iorb + (j - 1) * s->norb;
    t.psi = s->orb[j];
    t.gec = s->gec[kex];
    t.gec2 = s->gec[kex + s->norb * s->norb];
    const int kp = s->k2[iorb][j];
    if (j != iorb) {
      t.mode = 0;
      t.ex = s->exch[2 * kp];
      t.ex2 = (s->ilc2[iorb][j] == 2) ? s->exch[2 * kp + 1] : nullptr;
    } else if (s->m[iorb] > 0 && s->ilc2[iorb][j] > 0) {
      t.mode = 1;
      t.ex = s->exch[2 * kp];
      t.ex2 = nullptr;
    } else {
      t.mode = 2;
      t.ex = t.ex2 = nullptr;
    }
  }
  a.nterms = n;
  return a;
}

int fock(x2g_scf *s, int iorb) {
  launch_fock(s->ctx, s->grid->d, fock_args(s, iorb, s->lhs, s->rhs, s->fa));
  return X2G_OK;
}

// relaxation form of a kind of function: list-order SOR (always FP64) or
// MCSOR in the case's precision (relaxDriver, doSCF.F90:960-1004)
int pot_form(const x2g_scf *s) { return s->cs.pot_scheme == 0 ? X2G_SOR : s->cs.precision; }
int orb_form(const x2g_scf *s) { return s->cs.orb_scheme == 0 ? X2G_SOR : s->cs.precision; }

void potential_jobs(x2g_scf *s, int iorb, std::vector<x2g_job> &jobs) {
  for (const PotSlot &P : s->pots[iorb]) {
    x2g_job j{};
    j.u = P.target;
    j.psa = s->orb[P.in1];
    j.psb = s->orb[P.in2];
    j.omega = s->omega_pot;
    j.isym = P.isym;
    j.idel = P.idel;
    j.kind = 1;
    jobs.push_back(j);
  }
}

// coulExchSOR/MCSOR of one orbital's batch (relaxPots.F90:8-114)
int relax_potentials(x2g_scf *s, int iorb) {
  std::vector<x2g_job> jobs;
  potential_jobs(s, iorb, jobs);
  s->nsor4pot += long(jobs.size()) * s->cs.maxsor_pot;
  return launch_relax(s->ctx, s->grid, jobs.data(), int(jobs.size()), s->cs.maxsor_pot, pot_form(s));
}

// Batched mode: every orbital's batch (each Coulomb and exchange potential
// of the iteration once) in one launch, all from the orbitals at the start
// of the iteration, in relaxDriver's orbital order
int relax_all_potentials(x2g_scf *s) {
  std::vector<x2g_job> jobs;
  for (int i = 1; i <= s->norb; i++) potential_jobs(s, s->norb - i + 1, jobs);
  s->nsor4pot += long(jobs.size()) * s->cs.maxsor_pot;
  return launch_relax(s->ctx, s->grid, jobs.data(), int(jobs.size()), s->cs.maxsor_pot, pot_form(s));
}

int relax_orbital(x2g_scf *s, int iorb) {
  const GridDev &g = s->grid->d;
  fock(s, iorb);
  launch_asympt_get(s->ctx, g, s->fa, s->edecay);
  x2g_job j{};
  j.u = s->orb[iorb];
  j.lhs = s->lhs;
  j.rhs = s->rhs;
  j.omega = s->omega_orb;
  j.isym = s->isymOrb[iorb];
  j.kind = 0;
  s->nsor4orb += s->cs.maxsor_orb;
  int rc = launch_relax(s->ctx, s->grid, &j, 1, s->cs.maxsor_orb, orb_form(s));
  if (rc) return rc;
  launch_asympt_set(s->ctx, g, s->orb[iorb], s->edecay);
  return X2G_OK;
}

// batch_mode 2: the Fock operators of every orbital from the state after
// the potentials (no orbital has changed yet), then all orbitals relaxed in
// one launch, each with its own lhs, rhs and asymptotic decay
int relax_all_orbitals(x2g_scf *s) {
  const GridDev &g = s->grid->d;
  std::vector<x2g_job> jobs;
  std::vector<FockArgs> fa;
  OrbDecayList dl{};
  for (int i = 1; i <= s->norb; i++) {
    const int iorb = s->norb - i + 1;
    fa.push_back(fock_args(s, iorb, s->blhs[iorb], s->brhs[iorb], s->bfa[iorb]));
    dl.fa[i - 1] = s->bfa[iorb];
    dl.edecay[i - 1] = s->bedecay[iorb];
    dl.psi[i - 1] = s->orb[iorb];
    x2g_job j{};
    j.u = s->orb[iorb];
    j.lhs = s->blhs[iorb];
    j.rhs = s->brhs[iorb];
    j.omega = s->omega_orb;
    j.isym = s->isymOrb[iorb];
    j.kind = 0;
    jobs.push_back(j);
  }
  launch_fock_batch(s->ctx, g, fa.data(), int(fa.size()));
  launch_asympt_get_batch(s->ctx, g, dl, s->norb);
  s->nsor4orb += long(jobs.size()) * s->cs.maxsor_orb;
  int rc = launch_relax(s->ctx, s->grid, jobs.data(), int(jobs.size()), s->cs.maxsor_orb, orb_form(s));
  if (rc) return rc;
  launch_asympt_set_batch(s->ctx, g, dl, s->norb);
  return X2G_OK;
}

void norm(x2g_scf *s, int iorb) {
  double *out = s->sc + x2g_scf::O_NORM + iorb;
  launch_norm(s->ctx, s->grid->d, s->orb[iorb], out);
  launch_scale(s->ctx, s->grid->d, s->orb[iorb], out);
}

// lower orbitals of the same symmetry (normOrtho.F90:124-131)
std::vector<int> ortho_partners(x2g_scf *s, int iorb1) {
  std::vector<int> v;
  for (int iorb2 = 1; iorb2 <= s->norb; iorb2++) {
    int iorb3 = s->norb - iorb2 + 1;
    if (iorb3 <= iorb1) continue;
    if (s->m[iorb3] != s->m[iorb1]) continue;
    if (s->ige[iorb3] != s->ige[iorb1]) continue;
    v.push_back(iorb3);
  }
  return v;
}

// Batch mode 2, no orbital frozen: the norms and Gram-Schmidt steps of the
// iteration in rounds.  Orbital i is orthogonalised only against the higher
// orbitals of its own symmetry, which the reference's loop has finished by
// then, so an orbital's round is 1 + the latest round of its partners; the
// orbitals of one round are independent and each goes through the same
// operations as in the loop.  N2: 3 rounds instead of 6 orbitals, all in
// one cooperative launch.  false: an orbital has more partners than one
// round item holds.
bool orthonormalise_in_rounds(x2g_scf *s) {
  const int norb = s->norb;
  std::vector<int> depth(norb + 1, 0);
  std::vector<std::vector<int>> partners(norb + 1);
  int maxd = 0;
  for (int iorb = norb; iorb >= 1; iorb--) {
    partners[iorb] = ortho_partners(s, iorb);
    if (partners[iorb].size() > 16) return false;
    for (int q : partners[iorb]) depth[iorb] = std::max(depth[iorb], depth[q] + 1);
    maxd = std::max(maxd, depth[iorb]);
  }
  if (s->ctx->gram_ortho) {
    // the Gram-matrix form, orbitals in the reference's order
    std::vector<OrthoOrbital> w;
    std::vector<int> index(norb + 1, -1), pidx;
    for (int iorb = norb; iorb >= 1; iorb--) {
      OrthoOrbital x{};
      x.psi = s->orb[iorb];
      x.n = int(partners[iorb].size());
      for (int k = 0; k < x.n; k++) x.partners[k] = s->orb[partners[iorb][k]];
      x.ihomo = s->cs.homonuclear ? s->ihomo[iorb] : 0;
      x.norm_out = s->sc + x2g_scf::O_NORM + iorb;
      x.ovl_out = s->sc + x2g_scf::O_OVL + 64 * iorb;
      index[iorb] = int(w.size());
      w.push_back(x);
    }
    pidx.assign(w.size() * 16, -1);
    for (int iorb = norb; iorb >= 1; iorb--)
      for (size_t k = 0; k < partners[iorb].size(); k++) pidx[size_t(index[iorb]) * 16 + k] = index[partners[iorb][k]];
    if (launch_orthonormalise_gram(s->ctx, s->grid->d, w.data(), int(w.size()), pidx.data())) return true;
  }
  std::vector<OrthoOrbital> v;
  std::vector<int> off(1, 0);
  for (int r = 0; r <= maxd; r++) {
    for (int iorb = norb; iorb >= 1; iorb--) {
      if (depth[iorb] != r) continue;
      OrthoOrbital x{};
      x.psi = s->orb[iorb];
      x.n = int(partners[iorb].size());
      for (int k = 0; k < x.n; k++) x.partners[k] = s->orb[partners[iorb][k]];
      x.ihomo = s->cs.homonuclear ? s->ihomo[iorb] : 0;
      x.norm_out = s->sc + x2g_scf::O_NORM + iorb;
      x.ovl_out = s->sc + x2g_scf::O_OVL + 64 * iorb;
      v.push_back(x);
    }
    off.push_back(int(v.size()));
  }
  // every round in one launch where the plan fits it, else round by round
  if (!launch_orthonormalise(s->ctx, s->grid->d, v.data(), off.data(), maxd + 1))
    for (int r = 0; r <= maxd; r++) launch_ortho_round(s->ctx, s->grid->d, v.data() + off[r], off[r + 1] - off[r]);
  return true;
}

void ortho(x2g_scf *s, int iorb) {
  if (s->ifixorb[iorb] != 0) return;  // normOrtho.F90:143
  std::vector<int> p = ortho_partners(s, iorb);
  if (p.empty()) return;
  std::vector<const double *> o;
  for (int q : p) o.push_back(s->orb[q]);
  double *ovl = s->sc + x2g_scf::O_OVL + 64 * iorb;
  launch_overlaps(s->ctx, s->grid->d, s->orb[iorb], o.data(), int(o.size()), ovl);
  launch_ortho_apply(s->ctx, s->grid->d, s->orb[iorb], o.data(), int(o.size()), ovl);
}

void eahf(x2g_scf *s, int iorb, double *ee_out, double *parts) {
  launch_eahf(s->ctx, s->grid->d, s->orb[iorb], s->isymOrb[iorb], s->m[iorb], s->coulp[iorb], s->exchp[iorb], ee_out,
              parts, s->cs.precision == X2G_FP64);
}

// EaHF of the listed orbitals in one launch: the same sums in the same
// order as one launch per orbital.  parts: 5 values per orbital (index
// iorb) or null.
void eahf_batch(x2g_scf *s, const std::vector<int> &orbs, double *ee_base, double *parts) {
  std::vector<EahfItem> items;
  for (int iorb : orbs)
    items.push_back(EahfItem{s->orb[iorb], s->coulp[iorb], s->exchp[iorb], ee_base + iorb,
                             parts ? parts + 5 * iorb : nullptr, s->isymOrb[iorb], s->m[iorb]});
  if (!items.empty())
    launch_eahf_batch(s->ctx, s->grid->d, items.data(), int(items.size()), s->cs.precision == X2G_FP64);
}

std::vector<int> orbitals_descending(const x2g_scf *s) {
  std::vector<int> v;
  for (int i = s->norb; i >= 1; i--) v.push_back(i);
  return v;
}

void mpole_moments(x2g_scf *s) {
  if (s->nel == 1) return;
  const GridDev &g = s->grid->d;
  const int homo = s->cs.homonuclear;
  // all moments of the iteration in one batched launch
  std::vector<MomentItem> items;
  for (int i = 1; i <= s->norb; i++) {
    if (!s->itouch[i]) continue;
    items.push_back(MomentItem{s->orb[i], s->orb[i], s->sc + x2g_scf::O_CM + 8 * (i - 1), 0, 1});
  }
  for (size_t q = 0; q < s->mm_i1.size(); q++)
    items.push_back(MomentItem{s->orb[s->mm_i1[q]], s->orb[s->mm_i2[q]], s->sc + x2g_scf::O_EX + 8 * s->mm_ipc[q],
                               s->mm_idel[q], 0});
  if (!items.empty()) launch_moments(s->ctx, g, items.data(), int(items.size()), homo);
}

// the boundary rows of orbital iorb1's potentials (potAsympt) as items
void pot_asympt_items(x2g_scf *s, int iorb1, std::vector<AsymptItem> &items) {
  if (s->itouch[iorb1] == 1) items.push_back(AsymptItem{s->coul[iorb1], 0, iorb1 - 1, 0, 0});
  for (int iorb2 = 1; iorb2 <= s->norb; iorb2++) {
    if (!s->itouch[iorb1] && !s->itouch[iorb2]) continue;
    int k = s->k2[iorb1][iorb2];
    if (k == 0 || s->ilc[k] == 0) continue;
    int idel = std::abs(s->m[iorb1] - s->m[iorb2]);
    if (iorb1 == iorb2) idel = 2 * s->m[iorb1];
    items.push_back(AsymptItem{s->exch[2 * k], 1, k, idel, 0});
    if (s->ilc[k] == 2)
      items.push_back(AsymptItem{s->exch[2 * k + 1], 1, k + s->norb * (s->norb + 1) / 2, s->m[iorb2] + s->m[iorb1], 0});
  }
}

// potAsympt items in launches of kMaxAsympt; an item repeated for the same
// potential (the same values) is written once
void launch_asympt_items(x2g_scf *s, const std::vector<AsymptItem> &all) {
  std::vector<AsymptItem> items;
  for (const AsymptItem &it : all) {
    bool dup = false;
    for (const AsymptItem &x : items) dup = dup || (x.pot == it.pot);
    if (!dup) items.push_back(it);
  }
  for (size_t b = 0; b < items.size(); b += kMaxAsympt) {
    AsymptArgs a{};
    a.norb = s->norb;
    a.cmulti = s->sc + x2g_scf::O_CM;
    a.excm = s->sc + x2g_scf::O_EX;
    a.nslots = s->nslots;
    a.n = int(std::min(items.size() - b, size_t(kMaxAsympt)));
    for (int q = 0; q < a.n; q++) a.it[q] = items[b + q];
    launch_asympt(s->ctx, s->grid->d, a);
  }
}

void pot_asympt(x2g_scf *s, int iorb1) {
  AsymptArgs a{};
  a.norb = s->norb;
  a.cmulti = s->sc + x2g_scf::O_CM;
  a.excm = s->sc + x2g_scf::O_EX;
  a.nslots = s->nslots;
  int n = 0;
  if (s->itouch[iorb1] == 1) a.it[n++] = AsymptItem{s->coul[iorb1], 0, iorb1 - 1, 0, 0};
  for (int iorb2 = 1; iorb2 <= s->norb; iorb2++) {
    if (!s->itouch[iorb1] && !s->itouch[iorb2]) continue;
    int k = s->k2[iorb1][iorb2];
    if (k == 0 || s->ilc[k] == 0) continue;
    int idel = std::abs(s->m[iorb1] - s->m[iorb2]);
    if (iorb1 == iorb2) idel = 2 * s->m[iorb1];
    a.it[n++] = AsymptItem{s->exch[2 * k], 1, k, idel, 0};
    if (s->ilc[k] == 2)
      a.it[n++] = AsymptItem{s->exch[2 * k + 1], 1, k + s->norb * (s->norb + 1) / 2,
                             s->m[iorb2] + s->m[iorb1], 0};
  }
  a.n = n;
  launch_asympt(s->ctx, s->grid->d, a);
}

// total energy (totalEnergy.F90:13-245)
int etotal(x2g_scf *s) {
  const GridDev &g = s->grid->d;
  const int norb = s->norb;
  double *parts = s->sc + x2g_scf::O_OVL + 64 * 40;  // scratch region after the overlaps
  double *eedummy = parts + 5 * (MAXO + 1);           // MAXO + 1 discarded orbital energies
  eahf_batch(s, orbitals_descending(s), eedummy, parts);
  std::vector<TripleItem> items;
  std::vector<int> kind;  // 0 coulij(i,i) 1 coulij(i2,i1) 2 exch self 3 exch type0 4 exch type1
  std::vector<std::pair<int, int>> who;
  for (int i = 1; i <= norb; i++)
    if (s->occ[i] > 1.0) {
      items.push_back({s->orb[i], s->coul[i], s->orb[i]});
      kind.push_back(0);
      who.push_back({i, i});
    }
  for (int i1 = 1; i1 <= norb; i1++) {
    if (s->m[i1] > 0 && std::fabs(s->occ[i1] - 1.0) > 1e-7) {
      int k = s->k2[i1][i1];
      items.push_back({s->orb[i1], s->exch[2 * k], s->orb[i1]});
      kind.push_back(2);
      who.push_back({i1, i1});
    }
    for (int i2 = i1 + 1; i2 <= norb; i2++) {
      items.push_back({s->orb[i1], s->coul[i2], s->orb[i1]});
      kind.push_back(1);
      who.push_back({i1, i2});
      int k = s->k2[i1][i2];
      items.push_back({s->orb[i1], s->exch[2 * k], s->orb[i2]});
      kind.push_back(3);
      who.push_back({i1, i2});
      if (s->ilc2[i1][i2] == 2) {
        items.push_back({s->orb[i1], s->exch[2 * k + 1], s->orb[i2]});
        kind.push_back(4);
        who.push_back({i1, i2});
      }
    }
  }
  double *out = s->sc + s->sc_count - 1024;
  if (!items.empty()) launch_triples(s->ctx, g, items.data(), int(items.size()), out);
  std::vector<double> hp(5 * (MAXO + 1)), ho(items.size() + 1);
  cudaMemcpyAsync(hp.data(), parts, hp.size() * sizeof(double), cudaMemcpyDeviceToHost, s->ctx->stream);
  if (!items.empty())
    cudaMemcpyAsync(ho.data(), out, items.size() * sizeof(double), cudaMemcpyDeviceToHost, s->ctx->stream);
  count_copy(s->ctx, 0, (hp.size() + items.size()) * sizeof(double));
  int rc = x2g_synchronize(s->ctx);
  if (rc) return rc;
  // spin-pair counts for closed shells (exchContribs.f90 excont/exint)
  auto excont = [&](int a, int b, double &ox1, double &ox2) {
    int pa = s->m[a], pb = s->m[b];
    ox1 = ox2 = 0;
    if (pa == 0 || pb == 0) {
      ox1 = (pa == 0 && pb == 0) ? 2.0 : 4.0;
    } else {
      ox1 = 2.0 + 2.0;
      ox2 = 2.0 + 2.0;
    }
  };
  double woneel = 0, vkt = 0, vnt = 0, wdcoul = 0, wndc = 0, wex1 = 0, wex2 = 0;
  for (int i = 1; i <= norb; i++) {
    woneel = woneel + s->occ[i] * hp[5 * i + 2];
    vkt = vkt + s->occ[i] * hp[5 * i + 0];
    vnt = vnt + s->occ[i] * hp[5 * i + 1];
  }
  size_t q = 0;
  for (int i = 1; i <= norb; i++)
    if (s->occ[i] > 1.0) {
      wdcoul = wdcoul + s->occ[i] * (s->occ[i] - 1.0) * ho[q] / 2.0;
      q++;
    }
  for (; q < items.size(); q++) {
    int i1 = who[q].first, i2 = who[q].second;
    if (kind[q] == 2) {
      wex1 = wex1 + 2.0 * ho[q];  // exint: 2 same-spin pairs in a closed non-sigma shell
    } else if (kind[q] == 1) {
      wndc = wndc + s->occ[i1] * s->occ[i2] * ho[q];
    } else if (kind[q] == 3) {
      double ox1, ox2;
      excont(i1, i2, ox1, ox2);
      wex1 = wex1 + ox1 * ho[q];
    } else if (kind[q] == 4) {
      double ox1, ox2;
      excont(i1, i2, ox1, ox2);
      wex2 = wex2 + ox2 * ho[q];
    }
  }
  const double z1 = s->grid->h.z1, z2 = s->grid->h.z2, r = s->grid->h.r;
  s->evt = woneel + wdcoul + wndc - wex1 - wex2;
  double epott = vnt + wdcoul + wndc - wex1 - wex2;
  s->virial = (epott + z1 * z2 / r) / vkt;
  s->etot = s->evt + z1 * z2 / r;
  return X2G_OK;
}

// the energies, norms and overlap rows of the iteration (orbitals 0..norb),
// into pinned memory
int read_scalars(x2g_scf *s) {
  const size_t n = size_t(x2g_scf::O_OVL) + 64 * size_t(s->norb + 1);
  cudaError_t e = cudaMemcpyAsync(s->hsc, s->sc, n * sizeof(double), cudaMemcpyDeviceToHost, s->ctx->stream);
  if (e != cudaSuccess) return cuda_status(e, "scalar readback");
  count_copy(s->ctx, 0, n * sizeof(double));
  int rc = x2g_synchronize(s->ctx);
  if (rc) return rc;
  for (int i = 1; i <= s->norb; i++) {
    s->ee[i] = s->hsc[x2g_scf::O_EE + i];
    s->orbNorm[i] = s->hsc[x2g_scf::O_NORM + i];
    if (std::isnan(s->ee[i]) || std::isnan(s->orbNorm[i])) return set_status(X2G_ERR_NAN, "NaN in orbital energy");
  }
  return X2G_OK;
}

void update_wst(x2g_scf *s, int iorb) {
  std::vector<int> p = ortho_partners(s, iorb);
  double w = 0;
  for (size_t q = 0; q < p.size(); q++) w = std::max(w, std::fabs(s->hsc[x2g_scf::O_OVL + 64 * iorb + q]));
  if (!p.empty()) s->wst[iorb] = w;
}

int prep_scf(x2g_scf *s) {
  // prepSCF (doSCF.F90:24-174)
  for (int i = 1; i <= s->norb; i++) fock(s, i);
  if (s->cs.start == 1) {
    // orbpot old: no initAddData, the checkpoint's norms, moments and
    // Lagrange multipliers stand (doSCF.F90:73-134)
    int rc = read_scalars(s);
    if (rc) return rc;
    for (int i = 1; i <= s->norb; i++) s->eeOld[i] = s->ee[i];
    return etotal(s);
  }
  for (int i = 1; i <= s->norb; i++) {
    int j = s->norb + 1 - i;
    norm(s, j);
    ortho(s, j);
  }
  for (int i = 1; i <= s->norb; i++) s->itouch[i] = 1;
  mpole_moments(s);
  eahf_batch(s, orbitals_descending(s), s->sc + x2g_scf::O_EE, nullptr);
  int rc = read_scalars(s);
  if (rc) return rc;
  for (int i = 1; i <= s->norb; i++) s->eeOld[i] = s->ee[i];
  return etotal(s);
}

// one SCF iteration (doSCF.F90:342-786); returns 1 when the loop ends
int scf_iteration(x2g_scf *s, int *rc) {
  const int norb = s->norb;
  const int iscf = ++s->iscf;
  int iasympt = norb;
  *rc = X2G_OK;
  const bool batched = (s->cs.batch_mode >= 1);
  bool frozen = false;
  for (int i = 1; i <= norb; i++) frozen = frozen || (s->ifixorb[i] != 0);
  if (batched) {
    // the boundary values of every potential first (they depend only on the
    // multipole moments, which change only between iterations), then all
    // potentials of the iteration in one relaxation launch
    for (int i = 1; i <= norb; i++) s->itouch[norb - i + 1] = 1;
    std::vector<AsymptItem> items;
    for (int i = 1; i <= norb; i++) {
      const int iorb = norb - i + 1;
      if (iasympt != 0 && s->ifixorb[iorb] == 0) {
        pot_asympt_items(s, iorb, items);
        iasympt--;
      }
    }
    launch_asympt_items(s, items);
    if ((*rc = relax_all_potentials(s))) return 1;
    if (s->cs.batch_mode == 2 && !s->lfixorb)
      if ((*rc = relax_all_orbitals(s))) return 1;
  }
  const bool rounds = s->cs.batch_mode == 2 && !frozen && !s->lfixorb && norb > 1 && orthonormalise_in_rounds(s);
  for (int i = 1; i <= norb; i++) {
    const int iorb = norb - i + 1;
    if (!batched) {
      s->itouch[iorb] = 1;
      if (iasympt != 0 && s->ifixorb[iorb] == 0) {
        pot_asympt(s, iorb);
        iasympt--;
      }
      // relaxDriver (doSCF.F90:943-1011)
      if ((*rc = relax_potentials(s, iorb))) return 1;
    }
    if (!s->lfixorb && s->cs.batch_mode != 2)
      if ((*rc = relax_orbital(s, iorb))) return 1;
    if (rounds) {
      // normalised and orthogonalised above
    } else if (s->ifixorb[iorb] == 0 && s->cs.homonuclear) {
      // norm scaling and setCiOrb in one pass
      double *out = s->sc + x2g_scf::O_NORM + iorb;
      launch_norm(s->ctx, s->grid->d, s->orb[iorb], out);
      launch_scale_setci(s->ctx, s->grid->d, s->orb[iorb], out, s->ihomo[iorb]);
    } else {
      if (s->ifixorb[iorb] == 0) norm(s, iorb);
      if (s->cs.homonuclear) launch_setci(s->ctx, s->grid->d, s->orb[iorb], s->ihomo[iorb]);
    }
    if (!rounds && norb > 1 && s->ifixorb[iorb] == 0) ortho(s, iorb);
    if (s->ifixorb[iorb] != 0) fock(s, iorb);
    // EaHF of iorb reads only iorb and its own Fock sums, which nothing
    // later in the iteration changes: deferred and batched unless an
    // orbital is frozen (its Fock build above reads the current potentials)
    if (frozen) eahf(s, iorb, s->sc + x2g_scf::O_EE + iorb, nullptr);
  }
  if (!frozen) eahf_batch(s, orbitals_descending(s), s->sc + x2g_scf::O_EE, nullptr);
  if ((*rc = read_scalars(s))) return 1;
  for (int i = 1; i <= norb; i++) {
    const int iorb = norb - i + 1;
    if (norb > 1 && s->ifixorb[iorb] == 0) update_wst(s, iorb);
    s->deltaee[iorb] = s->ee[iorb] - s->eeOld[iorb];
    if (std::fabs(s->deltaee[iorb]) < kPrecis) s->deltaee[iorb] = 2.0 * s->orbEnergyThld;
    s->eeOld[iorb] = s->ee[iorb];
    s->recs.push_back({iscf, iorb, s->ee[iorb], s->deltaee[iorb], s->orbNorm[iorb] - 1.0});
  }
  // convergence logic (doSCF.F90:540-723)
  s->deltaeeMax = 0.0;
  s->deltaNormMax = 0.0;
  for (int n = 1; n <= norb; n++)
    if (std::fabs(s->deltaee[n]) >= std::fabs(s->deltaeeMax)) s->deltaeeMax = s->deltaee[n];
  for (int n = 1; n <= norb; n++) {
    double dn = std::fabs(s->orbNorm[n] - 1.0);
    if (s->ifixorb[n] == 0 && dn >= s->deltaNormMax) {
      s->deltaNormMax = dn;
      if (std::fabs(s->deltaNormMax) < kPrecis) s->deltaNormMax = kPrecis;
    }
  }
  if (std::fabs(s->eeconv) < kPrecis) s->eeconv = s->deltaeeMax;
  if (iscf > s->cs.nscf2skip) {
    if (std::fabs(s->deltaeeMax) >= std::fabs(s->eeconvprev)) s->noenergydec++;
    else {
      s->eeconvprev = s->deltaeeMax;
      s->noenergydec = 0;
    }
    if (std::fabs(s->deltaNormMax) >= std::fabs(s->dnmaxprev)) s->nonormdec++;
    else {
      s->dnmaxprev = s->deltaNormMax;
      s->nonormdec = 0;
    }
    if (s->noenergydec > s->cs.nenlast || s->nonormdec > s->cs.nnolast) return 1;
  } else {
    s->eeconvprev = s->demax1;
    s->dnmaxprev = s->deltaNormMax;
  }
  if (iscf == s->cs.maxscf) return 1;
  if (s->lfixorb4init && std::fabs(s->deltaeeMax) < s->thren4init) {
    if (s->nOrbEnergyThld == 3) {
      for (int i = 1; i <= norb; i++) s->ifixorb[i] = 0;
      s->lfixorb = 0;
      s->lfixorb4init = 0;
      s->eeconv = 10.0;
      s->deltaeeMax = 100.0;
    } else
      s->nOrbEnergyThld++;
  }
  if (!s->lenergyThld) {
    if (std::fabs(s->deltaeeMax) < s->orbEnergyThld) {
      s->lenergyThld = 1;
      s->eeconv = s->deltaeeMax;
      for (int i = 1; i <= norb; i++) s->itouch[i] = 0;
      s->nOrbEnergyThld = 0;
    }
  } else {
    if (std::fabs(s->deltaeeMax) < s->orbEnergyThld) {
      if (s->nOrbEnergyThld == 3) {
        s->converged = 1;
        return 1;
      }
      s->nOrbEnergyThld++;
    } else if (std::fabs(s->deltaNormMax) < s->orbNormThld) {
      if (s->nOrbNormThld == 3) {
        s->converged = 2;
        return 1;
      }
      s->nOrbNormThld++;
    } else {
      s->lenergyThld = 0;
      if (s->nresets > 5) return 1;
      s->nresets++;
    }
  }
  if (!s->lfixorb) {
    if (!s->lnormThld) {
      if (std::fabs(s->deltaNormMax) < s->orbNormThld) {
        s->lnormThld = 1;
        for (int i = 1; i <= norb; i++) s->itouch[i] = 0;
        s->nOrbNormThld = 0;
      }
    } else {
      if (std::fabs(s->deltaNormMax) < s->orbNormThld) {
        if (s->nOrbNormThld == 3) {
          s->converged = 2;
          return 1;
        }
        s->nOrbNormThld++;
      } else {
        s->lnormThld = 0;
        if (s->nresets4no > 5) return 1;
        s->nresets4no++;
      }
    }
  }
  if (std::fabs(s->eeconv / s->deltaeeMax) > s->cs.recalc_mm) {
    s->eeconv = s->deltaeeMax;
    mpole_moments(s);
  }
  for (int i = 1; i <= norb; i++) s->itouch[i] = 0;
  return 0;
}

int scf_finish(x2g_scf *s) {
  // end of scf (doSCF.F90:790-860)
  if (s->norb > 1) {
    for (int i = 1; i <= s->norb; i++) {
      int j = s->norb + 1 - i;
      double *keep = s->sc + x2g_scf::O_OVL + 64 * 50 + j;  // norm kept for the report
      launch_norm(s->ctx, s->grid->d, s->orb[j], keep);
      launch_scale(s->ctx, s->grid->d, s->orb[j], keep);
      ortho(s, j);
    }
  }
  eahf_batch(s, orbitals_descending(s), s->sc + x2g_scf::O_EE, nullptr);
  mpole_moments(s);
  int rc = read_scalars(s);
  if (rc) return rc;
  return etotal(s);
}

}  // namespace

extern "C" {

int x2g_case_defaults(x2g_case *c) {
  if (!c) return set_status(X2G_ERR_ARG, "null case");
  std::memset(c, 0, sizeof *c);
  c->maxscf = 1000;
  c->ienterm = 10;
  c->inoterm = 10;
  c->ienterm4init = 1;
  c->nscf2skip = 600;
  c->nenlast = 20;
  c->nnolast = 20;
  c->maxsor_orb = 10;
  c->maxsor_pot = 10;
  c->omega_orb = -1;
  c->omega_pot = -1;
  c->recalc_mm = 1.15;
  c->mpole = 4;
  c->precision = X2G_FP64;
  for (int i = 0; i < X2G_MAXORB; i++) c->gu[i] = ' ';
  return X2G_OK;
}

int x2g_scf_destroy(x2g_scf *s) {
  if (!s) return X2G_OK;
  if (s->ctx) cudaStreamSynchronize(s->ctx->stream);
  for (void *p : s->allocs) cudaFree(p);
  if (s->hsc) cudaFreeHost(s->hsc);
  if (s->grid) x2g_grid_destroy(s->grid);
  delete s;
  return X2G_OK;
}

int x2g_scf_create(x2g_ctx *ctx, const x2g_case *c, x2g_scf **out) {
  if (!ctx || !c || !out) return set_status(X2G_ERR_ARG, "null argument");
  *out = nullptr;
  if (c->norb < 1 || c->norb > X2G_MAXORB) return set_status(X2G_ERR_ARG, "norb out of range");
  for (int i = 0; i < c->norb; i++) {
    double full = (c->m[i] == 0) ? 2.0 : 4.0;
    if (c->m[i] < 0 || c->m[i] > 3) return set_status(X2G_ERR_ARG, "orbital |lambda| must be 0..3");
    if (!(c->occ[i] > 0) || c->occ[i] > full + 1e-6) return set_status(X2G_ERR_ARG, "bad occupation");
    // one open orbital has neither exchange nor off-diagonal multipliers;
    // several orbitals must form closed shells
    if (c->norb > 1 && std::fabs(c->occ[i] - full) > 1e-6)
      return set_status(X2G_ERR_UNSUPPORTED, "open-shell configurations with several orbitals are not supported");
  }
  if (c->precision != X2G_FP64 && c->precision != X2G_MIXED) return set_status(X2G_ERR_ARG, "unknown precision");
  if (c->orb_scheme < 0 || c->orb_scheme > 1 || c->pot_scheme < 0 || c->pot_scheme > 1)
    return set_status(X2G_ERR_ARG, "orb_scheme and pot_scheme must be 0 (SOR) or 1 (MCSOR)");
  if (c->batch_mode < 0 || c->batch_mode > 2) return set_status(X2G_ERR_ARG, "batch_mode must be 0, 1 or 2");
  if (c->maxsor_orb < 1 || c->maxsor_pot < 1) return set_status(X2G_ERR_ARG, "sweep counts must be positive");
  auto *s = new x2g_scf();
  s->ctx = ctx;
  s->cs = *c;
  int mpole = c->mpole > 0 ? c->mpole : 4;
  // initCBlocks:781-806: mpole raised for delta/phi orbitals listed first
  if (c->m[0] == 2 && mpole < 4) mpole = 4;
  if (c->m[0] == 3 && mpole <= 4) mpole = 8;
  s->mpole = mpole;
  int rc = x2g_grid_create(ctx, c->nnu, c->nmu, c->r, c->rinf, c->z1, c->z2, mpole, &s->grid);
  if (rc) {
    delete s;
    return rc;
  }
  const int norb = c->norb;
  s->norb = norb;
  for (int i = 1; i <= norb; i++) {
    s->m[i] = c->m[i - 1];
    s->occ[i] = c->occ[i - 1];
    s->nel += int(std::lround(s->occ[i]));
    s->isymOrb[i] = (s->m[i] % 2 == 0) ? 1 : -1;
    char gu = c->gu[i - 1];
    s->ihomo[i] = 1;
    if (gu == 'u' && (s->m[i] == 0 || s->m[i] == 2)) s->ihomo[i] = -1;
    if (gu == 'g' && (s->m[i] == 1 || s->m[i] == 3)) s->ihomo[i] = -1;
    s->ige[i] = (gu == 'u') ? 1 : 2;
  }
  x2g_default_omega(c->nnu, c->nmu, c->z1, c->z2, &s->omega_orb, &s->omega_pot);
  if (c->omega_orb > 0) s->omega_orb = c->omega_orb;
  if (c->omega_pot > 0) s->omega_pot = c->omega_pot;
  exchange_weights(s);
  // storage (initAddr:1189-1296)
  const size_t next = size_t(s->grid->h.next), mx = size_t(s->grid->h.mxsize);
  s->orb.assign(norb + 1, nullptr);
  s->coul.assign(norb + 1, nullptr);
  s->coulp.assign(norb + 1, nullptr);
  s->exchp.assign(norb + 1, nullptr);
  const int nk = norb * (norb + 1) / 2 + 1;
  s->exch.assign(2 * nk + 2, nullptr);
  s->ilc.assign(nk + 1, 0);
  bool ok = true;
  for (int i = 1; i <= norb; i++) {
    ok &= (s->orb[i] = dalloc(s, next)) != nullptr;
    ok &= (s->coul[i] = dalloc(s, next)) != nullptr;
    ok &= (s->coulp[i] = dalloc(s, mx)) != nullptr;
    ok &= (s->exchp[i] = dalloc(s, mx)) != nullptr;
  }
  for (int i1 = 1; i1 <= norb; i1++)
    for (int i2 = i1; i2 <= norb; i2++) {
      int k = i1 + i2 * (i2 - 1) / 2;
      if (i1 == i2 && s->m[i1] == 0) continue;
      s->ilc[k] = 1;
      s->ilc2[i1][i2] = s->ilc2[i2][i1] = 1;
      s->k2[i1][i2] = s->k2[i2][i1] = k;
      ok &= (s->exch[2 * k] = dalloc(s, next)) != nullptr;
      if (i1 != i2 && s->m[i1] != 0 && s->m[i2] != 0) {
        s->ilc[k] = 2;
        s->ilc2[i1][i2] = s->ilc2[i2][i1] = 2;
        ok &= (s->exch[2 * k + 1] = dalloc(s, next)) != nullptr;
      }
    }
  ok &= (s->lhs = dalloc(s, mx)) != nullptr;
  ok &= (s->rhs = dalloc(s, mx)) != nullptr;
  ok &= (s->fa = dalloc(s, 5 * size_t(s->grid->h.nni))) != nullptr;
  ok &= (s->edecay = dalloc(s, 4 * size_t(s->grid->h.nni))) != nullptr;
  if (c->batch_mode == 2) {
    s->blhs.assign(s->norb + 1, nullptr);
    s->brhs.assign(s->norb + 1, nullptr);
    s->bfa.assign(s->norb + 1, nullptr);
    s->bedecay.assign(s->norb + 1, nullptr);
    for (int i = 1; i <= s->norb; i++) {
      ok &= (s->blhs[i] = dalloc(s, mx)) != nullptr;
      ok &= (s->brhs[i] = dalloc(s, mx)) != nullptr;
      ok &= (s->bfa[i] = dalloc(s, 5 * size_t(s->grid->h.nni))) != nullptr;
      ok &= (s->bedecay[i] = dalloc(s, 4 * size_t(s->grid->h.nni))) != nullptr;
    }
  }
  s->nslots = norb * (norb + 1) + 2;
  s->sc_count = size_t(x2g_scf::O_EX) + 8 * size_t(s->nslots) + 2048;
  ok &= (s->sc = dalloc(s, s->sc_count)) != nullptr;
  if (cudaHostAlloc(reinterpret_cast<void **>(&s->hsc), size_t(x2g_scf::O_CM) * sizeof(double),
                    cudaHostAllocDefault) == cudaSuccess)
    std::fill(s->hsc, s->hsc + x2g_scf::O_CM, 0.0);
  else
    ok = false;
  if (!ok) {
    x2g_scf_destroy(s);
    return set_status(X2G_ERR_ALLOC, "device allocation failed");
  }
  // relaxation batches: exchange potentials K(iorb, j>=iorb) then J(iorb)
  s->pots.assign(norb + 1, {});
  for (int iorb = 1; iorb <= norb; iorb++) {
    auto &P = s->pots[iorb];
    for (int j = iorb; j <= norb; j++) {
      if (iorb == j && s->m[iorb] == 0) continue;
      if (iorb == j && s->ilc2[iorb][iorb] == 0) continue;
      int in1 = std::min(iorb, j), in2 = std::max(iorb, j);
      int idel = std::abs(s->m[in1] - s->m[in2]);
      if (in1 == in2) idel = 2 * s->m[in1];
      int ipc = in1 + in2 * (in2 - 1) / 2;
      P.push_back({in1, in2, idel, (idel % 2 == 0) ? 1 : -1, s->exch[2 * ipc]});
      if (s->ilc2[in1][in2] == 2) {
        int id2 = s->m[in1] + s->m[in2];
        P.push_back({in1, in2, id2, (id2 % 2 == 0) ? 1 : -1, s->exch[2 * ipc + 1]});
      }
    }
    P.push_back({iorb, iorb, 0, 1, s->coul[iorb]});
  }
  for (int i1 = 1; i1 <= norb; i1++)
    for (int i2 = i1; i2 <= norb; i2++) {
      if (i1 == i2 && s->m[i2] == 0) continue;
      int idel = std::abs(s->m[i2] - s->m[i1]);
      if (i1 == i2) idel = 2 * s->m[i2];
      int ipc = s->k2[i1][i2];
      s->mm_i1.push_back(i1);
      s->mm_i2.push_back(i2);
      s->mm_idel.push_back(idel);
      s->mm_ipc.push_back(ipc);
      if (s->ilc2[i1][i2] == 2) {
        s->mm_i1.push_back(i1);
        s->mm_i2.push_back(i2);
        s->mm_idel.push_back(s->m[i2] + s->m[i1]);
        s->mm_ipc.push_back(ipc + norb * (norb + 1) / 2);
      }
    }
  if (c->start != 0 && c->start != 1) {
    x2g_scf_destroy(s);
    return set_status(X2G_ERR_ARG, "start must be 0 (hydrogenic) or 1 (loaded by the caller)");
  }
  if (c->start == 0 && (rc = initial_guess(s))) {
    x2g_scf_destroy(s);
    return rc;
  }
  // orbpot hydrogen [ienterm4init] (inputInterface.F90:2257-2305); an
  // orbpot old start has no frozen phase
  if (c->start == 0 && c->ienterm4init > 0) {
    s->lfixorb4init = s->lfixorb = 1;
    for (int i = 1; i <= norb; i++) s->ifixorb[i] = 1;
  }
  *out = s;
  return set_status(X2G_OK, "");
}

int x2g_scf_run(x2g_scf *s, int max_iterations, x2g_result *res) {
  if (!s) return set_status(X2G_ERR_ARG, "null scf");
  cudaSetDevice(s->ctx->device);
  int rc = X2G_OK;
  if (!s->started) {
    if ((rc = prep_scf(s))) return rc;
    s->orbEnergyThld = std::pow(10.0, double(-s->cs.ienterm));
    s->orbNormThld = std::pow(10.0, double(-s->cs.inoterm));
    s->thren4init = std::pow(10.0, double(-s->cs.ienterm4init));
    for (int i = 1; i <= s->norb; i++) {
      s->itouch[i] = 0;
      s->deltaee[i] = 0;
      s->eeOld[i] = s->ee[i];
    }
    if (s->cs.homonuclear)
      for (int i = 1; i <= s->norb; i++) launch_setci(s->ctx, s->grid->d, s->orb[i], s->ihomo[i]);
    s->started = 1;
  }
  for (int k = 0; k < max_iterations && !s->done; k++) {
    if (scf_iteration(s, &rc)) {
      if (rc) return rc;
      s->done = 1;
      if ((rc = scf_finish(s))) return rc;
    }
  }
  if (res) {
    std::memset(res, 0, sizeof *res);
    res->iterations = s->iscf;
    res->converged = s->converged;
    res->sweeps = s->nsor4orb + s->nsor4pot;
    res->total_energy = s->etot;
    res->electronic_energy = s->evt;
    res->virial = s->virial;
    for (int i = 1; i <= s->norb; i++) {
      res->ee[i - 1] = s->ee[i];
      res->norm_error[i - 1] = s->orbNorm[i] - 1.0;
    }
  }
  return set_status(X2G_OK, "");
}

int x2g_scf_get_orbital(x2g_scf *s, int iorb, double *host) {
  if (!s || !host || iorb < 1 || iorb > s->norb) return set_status(X2G_ERR_ARG, "bad argument");
  const HostGrid &g = s->grid->h;
  std::vector<double> ext(g.next);
  cudaError_t e = cudaMemcpyAsync(ext.data(), s->orb[iorb], ext.size() * sizeof(double), cudaMemcpyDeviceToHost,
                                  s->ctx->stream);
  if (e != cudaSuccess) return cuda_status(e, "orbital readback");
  count_copy(s->ctx, 0, ext.size() * sizeof(double));
  int rc = x2g_synchronize(s->ctx);
  if (rc) return rc;
  for (int i = 0; i < g.nmu; i++)
    for (int j = 0; j < g.nni; j++) host[i * g.nni + j] = ext[(i + 4) * g.n8 + j + 4];
  return X2G_OK;
}

int x2g_scf_get_coulomb(x2g_scf *s, int iorb, double *host) {
  if (!s || !host || iorb < 1 || iorb > s->norb) return set_status(X2G_ERR_ARG, "bad argument");
  const HostGrid &g = s->grid->h;
  std::vector<double> ext(g.next);
  cudaError_t e = cudaMemcpyAsync(ext.data(), s->coul[iorb], ext.size() * sizeof(double), cudaMemcpyDeviceToHost,
                                  s->ctx->stream);
  if (e != cudaSuccess) return cuda_status(e, "potential readback");
  count_copy(s->ctx, 0, ext.size() * sizeof(double));
  int rc = x2g_synchronize(s->ctx);
  if (rc) return rc;
  for (int i = 0; i < g.nmu; i++)
    for (int j = 0; j < g.nni; j++) host[i * g.nni + j] = ext[(i + 4) * g.n8 + j + 4];
  return X2G_OK;
}

// device array of (kind, i1, i2, which), or null when it names no function
static double *function_ptr(x2g_scf *s, int kind, int i1, int i2, int which) {
  if (i1 < 1 || i1 > s->norb) return nullptr;
  if (kind == 0 && i2 == 0 && which == 0) return s->orb[i1];
  if (kind == 1 && i2 == 0 && which == 0) return s->coul[i1];
  if (kind != 2 || i2 < i1 || i2 > s->norb || (which != 0 && which != 1)) return nullptr;
  if (i1 == i2 && s->m[i1] == 0) return nullptr;  // no sigma self-exchange
  const int k = s->k2[i1][i2];
  if (which == 0) return s->exch[2 * k];
  return (i1 != i2 && s->ilc2[i1][i2] == 2) ? s->exch[2 * k + 1] : nullptr;
}

int x2g_scf_set_function(x2g_scf *s, int kind, int i1, int i2, int which, const double *host) {
  if (!s || !host) return set_status(X2G_ERR_ARG, "null argument");
  double *d = function_ptr(s, kind, i1, i2, which);
  if (!d) return set_status(X2G_ERR_ARG, "no such function");
  cudaSetDevice(s->ctx->device);
  int rc = x2g_synchronize(s->ctx);
  if (rc) return rc;
  std::vector<double> plain(host, host + s->grid->h.mxsize);
  return upload_ext(s, d, plain);
}

int x2g_scf_get_function(x2g_scf *s, int kind, int i1, int i2, int which, double *host) {
  if (!s || !host) return set_status(X2G_ERR_ARG, "null argument");
  double *d = function_ptr(s, kind, i1, i2, which);
  if (!d) return set_status(X2G_ERR_ARG, "no such function");
  cudaSetDevice(s->ctx->device);
  const HostGrid &g = s->grid->h;
  std::vector<double> ext(g.next);
  cudaError_t e = cudaMemcpyAsync(ext.data(), d, ext.size() * sizeof(double), cudaMemcpyDeviceToHost, s->ctx->stream);
  if (e != cudaSuccess) return cuda_status(e, "function readback");
  count_copy(s->ctx, 0, ext.size() * sizeof(double));
  int rc = x2g_synchronize(s->ctx);
  if (rc) return rc;
  for (int i = 0; i < g.nmu; i++)
    for (int j = 0; j < g.nni; j++) host[i * g.nni + j] = ext[(i + 4) * g.n8 + j + 4];
  return X2G_OK;
}

// checkpoint layout <-> device scalars: cmulti(iorb + (k-1) norb) <->
// O_CM + 8 (iorb-1) + k-1; exc_k(ipc) <-> O_EX + 8 ipc + k-1
static constexpr size_t kExcLen = size_t(X2G_MAXORB) * (X2G_MAXORB + 1);

int x2g_scf_set_start_values(x2g_scf *s, const double *ee, const double *orbnorm, const double *cmulti,
                             const double *exc) {
  if (!s || !ee || !orbnorm || !cmulti || !exc) return set_status(X2G_ERR_ARG, "null argument");
  if (s->started) return set_status(X2G_ERR_ARG, "start values must be set before the first run");
  cudaSetDevice(s->ctx->device);
  int rc = x2g_synchronize(s->ctx);
  if (rc) return rc;
  std::vector<double> h(s->sc_count);
  cudaError_t e = cudaMemcpyAsync(h.data(), s->sc, h.size() * sizeof(double), cudaMemcpyDeviceToHost, s->ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->ctx->stream);
  if (e != cudaSuccess) return cuda_status(e, "start values");
  const int norb = s->norb;
  for (int i = 1; i <= norb; i++) {
    h[x2g_scf::O_EE + i] = s->ee[i] = ee[i - 1];
    h[x2g_scf::O_NORM + i] = s->orbNorm[i] = orbnorm[i - 1];
    for (int k = 1; k <= 8; k++) h[x2g_scf::O_CM + 8 * (i - 1) + (k - 1)] = cmulti[(i - 1) + (k - 1) * norb];
  }
  for (int ipc = 1; ipc < s->nslots && size_t(ipc) <= kExcLen; ipc++)
    for (int k = 1; k <= 8; k++) h[x2g_scf::O_EX + 8 * size_t(ipc) + (k - 1)] = exc[(k - 1) * kExcLen + ipc - 1];
  e = cudaMemcpyAsync(s->sc, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, s->ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->ctx->stream);  // h is freed on return
  count_copy(s->ctx, h.size() * sizeof(double), h.size() * sizeof(double));
  return e == cudaSuccess ? X2G_OK : cuda_status(e, "start values");
}

int x2g_scf_get_start_values(x2g_scf *s, double *ee, double *orbnorm, double *cmulti, double *exc) {
  if (!s || !ee || !orbnorm || !cmulti || !exc) return set_status(X2G_ERR_ARG, "null argument");
  cudaSetDevice(s->ctx->device);
  int rc = x2g_synchronize(s->ctx);
  if (rc) return rc;
  std::vector<double> h(s->sc_count);
  cudaError_t e = cudaMemcpyAsync(h.data(), s->sc, h.size() * sizeof(double), cudaMemcpyDeviceToHost, s->ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->ctx->stream);
  if (e != cudaSuccess) return cuda_status(e, "start values");
  count_copy(s->ctx, 0, h.size() * sizeof(double));
  const int norb = s->norb;
  std::fill(cmulti, cmulti + size_t(X2G_MAXORB) * 8, 0.0);
  std::fill(exc, exc + 8 * kExcLen, 0.0);
  for (int i = 1; i <= norb; i++) {
    ee[i - 1] = h[x2g_scf::O_EE + i];
    orbnorm[i - 1] = h[x2g_scf::O_NORM + i];
    for (int k = 1; k <= 8; k++) cmulti[(i - 1) + (k - 1) * norb] = h[x2g_scf::O_CM + 8 * (i - 1) + (k - 1)];
  }
  for (int ipc = 1; ipc < s->nslots && size_t(ipc) <= kExcLen; ipc++)
    for (int k = 1; k <= 8; k++) exc[(k - 1) * kExcLen + ipc - 1] = h[x2g_scf::O_EX + 8 * size_t(ipc) + (k - 1)];
  return X2G_OK;
}

int x2g_scf_nrecords(x2g_scf *s) { return s ? int(s->recs.size()) : 0; }

int x2g_scf_record(x2g_scf *s, int i, int *iscf, int *iorb, double *ee, double *dee, double *dnorm) {
  if (!s || i < 0 || i >= int(s->recs.size())) return set_status(X2G_ERR_ARG, "record index out of range");
  const Rec &r = s->recs[i];
  if (iscf) *iscf = r.iscf;
  if (iorb) *iorb = r.iorb;
  if (ee) *ee = r.ee;
  if (dee) *dee = r.dee;
  if (dnorm) *dnorm = r.dnorm;
  return X2G_OK;
}

}  // extern "C"
