// Reference-named, link-compatible entry points (src/c/mcsor_pthread.c:32,
// src/c/coulExch_pthread.c:19, src/c/mcsor_tpool.c:135,
// src/c/coulExch_tpool.c:109).  They read the Fortran COMMON blocks whose C
// layouts are given in src/c/sorpt.h:58-249; the blocks are referenced
// weakly so the library also loads in programs without them.
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "x2g_kernels.cuh"

#define MAXORB X2G_MAXORB
#define MAXTHREADS4MCSOR 16

extern "C" {
struct x2g_cb1 { int v[2 * MAXORB][MAXORB]; };
struct x2g_cb7 { int i1bc[MAXORB]; };
struct x2g_cb8 { int nexchpotsc[MAXORB]; int maxpotsc; };
struct x2g_cb17 {
  int mxnmuc, mxsizec, ngrd6ac, ngrd6bc, ngrd7c, nnu1c, nnu2c, nnu3c, nnu4c, nnu5c, isstartc, isstopc, maxsor1c,
      maxsor2c;
};
struct x2g_cb4d { double v[4]; };
struct x2g_cb5d { double v[5]; };
struct x2g_cb45 { double omegac, omega1c; };
struct x2g_cb46 { int iorbc, isymc, nthreadsc; };
struct x2g_cbptrd { double *p; };
struct x2g_cbi4b { int i4barr[20]; };
struct x2g_cbptri { int *p; };
struct x2g_cbiadex { int iadex1c, iadex2c, iadex3c, iadextc, iadnorc; };

extern struct x2g_cb1 c_interface_1_ __attribute__((weak));   // ins1
extern struct x2g_cb1 c_interface_2_ __attribute__((weak));   // ins2
extern struct x2g_cb1 c_interface_3_ __attribute__((weak));   // ibexcpc
extern struct x2g_cb1 c_interface_4_ __attribute__((weak));   // deltam4potc
extern struct x2g_cb1 c_interface_6_ __attribute__((weak));   // isymsc
extern struct x2g_cb7 c_interface_7_ __attribute__((weak));   // i1bc
extern struct x2g_cb8 c_interface_8_ __attribute__((weak));   // nexchpotsc
extern struct x2g_cb17 c_interface_17_ __attribute__((weak));
extern struct x2g_cb4d c_interface_40_ __attribute__((weak));  // dmu1
extern struct x2g_cb4d c_interface_41_ __attribute__((weak));  // dmu2
extern struct x2g_cb4d c_interface_42_ __attribute__((weak));  // dnu1
extern struct x2g_cb4d c_interface_43_ __attribute__((weak));  // dnu2
extern struct x2g_cb5d c_interface_44_ __attribute__((weak));  // exeven
extern struct x2g_cb45 c_interface_45_ __attribute__((weak));
extern struct x2g_cb46 c_interface_46_ __attribute__((weak));
extern struct x2g_cbptrd c_orbptr_ __attribute__((weak));
extern struct x2g_cbptrd c_exchptr_ __attribute__((weak));
extern struct x2g_cbptrd c_supplptr_ __attribute__((weak));
extern struct x2g_cbi4b c_i4b_ __attribute__((weak));
extern struct x2g_cbptri c_sorptr_ __attribute__((weak));    // cw_sor: index lists
extern struct x2g_cbiadex c_iadex_ __attribute__((weak));    // offsets of the lists in cw_sor
}

using namespace x2g;

namespace {

std::mutex g_mu;
x2g_ctx *g_ctx = nullptr;
x2g_grid *g_grid = nullptr;
int g_nni = 0, g_nmu = 0;

bool have_common() {
  return &c_interface_17_ && &c_interface_40_ && &c_interface_41_ && &c_interface_42_ && &c_interface_43_ &&
         &c_interface_44_ && &c_interface_45_ && &c_supplptr_ && &c_i4b_;
}

// Grid for the COMMON-block dimensions; operator coefficients and the
// b/d tables are taken from the Fortran program's own arrays.
int ensure_grid() {
  const int nni = c_interface_17_.nnu1c - 8, nmu = c_interface_17_.mxnmuc;
  if (!g_ctx) {
    int rc = x2g_create(&g_ctx, 0);
    if (rc) return rc;
  }
  if (g_grid && g_nni == nni && g_nmu == nmu) goto apply_common;
  if (g_grid) x2g_grid_destroy(g_grid);
  g_grid = nullptr;
  {
    // a nominal geometry only fills tables that the sweep then overrides
    int rc = x2g_grid_create(g_ctx, nni, nmu, 1.0, 40.0, 1.0, 1.0, 4, &g_grid);
    if (rc) return rc;
  }
  g_nni = nni;
  g_nmu = nmu;
apply_common : {
  GridDev &d = g_grid->d;
  std::memcpy(d.dmu1, c_interface_40_.v, sizeof d.dmu1);
  std::memcpy(d.dmu2, c_interface_41_.v, sizeof d.dmu2);
  std::memcpy(d.dni1, c_interface_42_.v, sizeof d.dni1);
  std::memcpy(d.dni2, c_interface_43_.v, sizeof d.dni2);
  std::memcpy(d.exeven, c_interface_44_.v, sizeof d.exeven);
  const double *sup = c_supplptr_.p;
  const int *i4 = c_i4b_.i4barr;
  std::vector<double> borb(nmu), bpot(nmu), dnu(nni);
  for (int i = 0; i < nmu; i++) {
    borb[i] = sup[i4[0] - 1 + i * nni];
    bpot[i] = sup[i4[1] - 1 + i * nni];
  }
  for (int j = 0; j < nni; j++) dnu[j] = sup[i4[2] - 1 + nni + j];
  cudaStream_t st = g_ctx->stream;
  cudaMemcpyAsync(const_cast<double *>(d.borb_mu), borb.data(), nmu * sizeof(double), cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(const_cast<double *>(d.bpot_mu), bpot.data(), nmu * sizeof(double), cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(const_cast<double *>(d.d_nu), dnu.data(), nni * sizeof(double), cudaMemcpyHostToDevice, st);
  cudaStreamSynchronize(st);  // the host vectors are freed on return
  count_copy(g_ctx, (2 * size_t(nmu) + nni) * sizeof(double), 0);
}
  return X2G_OK;
}

void mcsor_common(int *isym, double *wk2, double *lhs, double *rhs) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!have_common()) {
    set_status(X2G_ERR_NO_COMMON, "x2dhf COMMON blocks are not linked");
    return;
  }
  if (ensure_grid()) return;
  // maxsor2 sweeps (mcsor_single_colour_pthread.c:54-72); the Fortran
  // caller runs the macro iterations with putin/putout around each call
  if (x2g_mcsor_host(g_ctx, g_grid, *isym, 0, c_interface_45_.omegac, c_interface_17_.maxsor2c, wk2, lhs, rhs))
    return;
  set_status(X2G_OK, "");
}

// Which order the extended index list in cw_sor holds (the list sorpt_
// sweeps, coulExch_pthread.c:42-46): 1 the colour-reordered list of a PT
// build with the mcsor-ce card (initCBAllocArrays.F90:2221-2240: stable
// partition of the "middle" list by position mod 5), i.e. single-thread
// MCSOR; 0 the "middle" list itself, i.e. list-order SOR; -1 neither.
int sor_list_order() {
  const std::vector<int> &mid = g_grid->h.order;  // 0-based ext indices, middle order
  const int n = int(mid.size());
  const int *lst = c_sorptr_.p + (c_iadex_.iadextc - 1);
  bool is_mid = true, is_col = true;
  int j = 0;
  for (int c = 0; c < 5; c++)
    for (int i = c; i < n; i += 5, j++) {
      if (lst[j] != mid[i] + 1) is_col = false;
      if (lst[j] != mid[j] + 1) is_mid = false;
    }
  return is_col ? 1 : (is_mid ? 0 : -1);
}

// device and pinned host staging of coulExch_pthread_, kept across calls
double *g_dev = nullptr, *g_pin = nullptr;
size_t g_dev_n = 0, g_pin_n = 0;

bool stage_buffers(size_t dev_n, size_t pin_n) {
  if (g_dev_n < dev_n) {
    if (g_dev) cudaFree(g_dev);
    g_dev = nullptr;
    g_dev_n = 0;
    if (cudaMalloc(&g_dev, dev_n * sizeof(double)) != cudaSuccess) return false;
    g_dev_n = dev_n;
  }
  if (g_pin_n < pin_n) {
    if (g_pin) cudaFreeHost(g_pin);
    g_pin = nullptr;
    g_pin_n = 0;
    if (cudaMallocHost(&g_pin, pin_n * sizeof(double)) != cudaSuccess) return false;
    g_pin_n = pin_n;
  }
  return true;
}

// coulExch_pthread_: every potential of orbital iorbc in one launch, with
// relax_single_pot_pthread.c:74-92's lhs/rhs and putinc/putoutc embedding,
// staged in one host-to-device copy and read back in one copy
void coulexch_common() {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!have_common() || !&c_interface_46_ || !&c_interface_8_ || !&c_orbptr_ || !&c_exchptr_ ||
      !&c_interface_1_ || !&c_interface_7_ || !&c_sorptr_ || !&c_iadex_) {
    set_status(X2G_ERR_NO_COMMON, "x2dhf COMMON blocks are not linked");
    return;
  }
  if (ensure_grid()) return;
  // sorpt_ sweeps whichever list cw_sor holds: colour-reordered = MCSOR in
  // colour order, middle = list-order SOR
  const int order = sor_list_order();
  if (order < 0) {
    set_status(X2G_ERR_UNSUPPORTED, "cw_sor holds an unrecognised list order; potentials left unchanged");
    return;
  }
  const int form = (order == 1) ? X2G_FP64 : X2G_SOR;
  const int iorb = c_interface_46_.iorbc;
  const int n = c_interface_8_.nexchpotsc[iorb - 1];
  const int nni = g_nni, nmu = g_nmu, mx = nni * nmu;
  const GridDev &g = g_grid->d;
  const double *sup = c_supplptr_.p;
  const int *i4 = c_i4b_.i4barr;
  const double *f3 = sup + i4[7] - 1, *ef = sup + i4[3] - 1, *gf = sup + i4[9] - 1;
  const double *psi = c_orbptr_.p;
  double *excp = c_exchptr_.p;
  const int maxsor1 = c_interface_17_.maxsor1c, maxsor2 = c_interface_17_.maxsor2c;
  const double omega = c_interface_45_.omegac;
  const size_t per = size_t(g.next) + 3 * size_t(mx);
  if (n <= 0) {
    set_status(X2G_OK, "");
    return;
  }
  if (!stage_buffers(per * n, 3 * size_t(mx) * n)) {
    set_status(X2G_ERR_ALLOC, "coulExch buffers");
    return;
  }
  std::vector<x2g_job> jobs(n);
  for (int k = 0; k < n; k++) {
    const int in1 = c_interface_1_.v[k][iorb - 1], in2 = c_interface_2_.v[k][iorb - 1];
    const int ib1 = c_interface_7_.i1bc[in1 - 1], ib2 = c_interface_7_.i1bc[in2 - 1];
    const int ibexc = c_interface_3_.v[k][iorb - 1];
    const int idel = c_interface_4_.v[k][iorb - 1];
    const int isym = c_interface_6_.v[k][iorb - 1];
    const double deltam2 = double(idel * idel);
    double *rhsh = g_pin + 3 * size_t(mx) * k, *lhsh = rhsh + mx, *funh = rhsh + 2 * size_t(mx);
    for (int i = 0; i < mx; i++) rhsh[i] = psi[ib1 + i - 1] * psi[ib2 + i - 1] * gf[i];
    for (int i = 0; i < mx; i++) lhsh[i] = (deltam2 == 0.0) ? f3[i] : f3[i] + ef[i] * deltam2;
    std::memcpy(funh, excp + ibexc - 1, mx * sizeof(double));
    double *base = g_dev + per * k;
    cudaMemcpyAsync(base + g.next, rhsh, 3 * size_t(mx) * sizeof(double), cudaMemcpyHostToDevice, g_ctx->stream);
    count_copy(g_ctx, 3 * size_t(mx) * sizeof(double), 0);
    launch_putin(g_ctx, g, isym, base + g.next + 2 * size_t(mx), base);
    x2g_job &j = jobs[k];
    j.u = base;
    j.rhs = base + g.next;
    j.lhs = base + g.next + mx;
    j.omega = omega;
    j.isym = isym;
    j.idel = idel;
    j.kind = 1;
  }
  for (int it = 0; it < maxsor1; it++)
    if (launch_relax(g_ctx, g_grid, jobs.data(), n, maxsor2, form)) return;
  for (int k = 0; k < n; k++) {
    double *base = g_dev + per * k;
    launch_putout(g_ctx, g, base, base + g.next + 2 * size_t(mx));
    cudaMemcpyAsync(g_pin + 3 * size_t(mx) * k, base + g.next + 2 * size_t(mx), mx * sizeof(double),
                    cudaMemcpyDeviceToHost, g_ctx->stream);
    count_copy(g_ctx, 0, mx * sizeof(double));
  }
  if (x2g_synchronize(g_ctx)) return;
  for (int k = 0; k < n; k++)
    std::memcpy(excp + c_interface_3_.v[k][iorb - 1] - 1, g_pin + 3 * size_t(mx) * k, mx * sizeof(double));
  set_status(X2G_OK, "");
}

}  // namespace

extern "C" {

void mcsor_pthread_(int *isym, int *nthreads, double *wk2, double *lhs, double *rhs) {
  (void)nthreads;
  mcsor_common(isym, wk2, lhs, rhs);
}

void mcsor_tpool_(int *isym, int *nthreads, double *wk2, double *lhs, double *rhs) {
  (void)nthreads;
  mcsor_common(isym, wk2, lhs, rhs);
}

void coulExch_pthread_(void) { coulexch_common(); }

void coulExch_tpool_(void) { coulexch_common(); }

static void release() {
  std::lock_guard<std::mutex> lk(g_mu);
  if (g_dev) cudaFree(g_dev);
  if (g_pin) cudaFreeHost(g_pin);
  g_dev = g_pin = nullptr;
  g_dev_n = g_pin_n = 0;
  if (g_grid) x2g_grid_destroy(g_grid);
  if (g_ctx) x2g_destroy(g_ctx);
  g_grid = nullptr;
  g_ctx = nullptr;
}

void tpoolStop4mcsor_(int *nthreads) {
  (void)nthreads;
  release();
}

void tpoolStop4pots_(int *nthreads) {
  (void)nthreads;
  release();
}

}  // extern "C"
