// Internal structures of the x2dhf GB300 relaxation library.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/x2dhf_gpu.h"

namespace x2g {

constexpr double kPrecis = 2.220446049250313080847263336181640625e-16;  // epsilon(1d0), initVariables.F90:397
constexpr double kPi = 3.14159265358979323846264338327950;                // params.F90:94
constexpr int kMaxLevels = 8;
// device words of a context's barrier state: [0] arrivals, [1] generation,
// [2] error word, [3] reduction ticket, then the tickets of the batched
// moment reductions from word 288 (kMomentItems), then the persistent
// sweep's per-block phase counts from word kPhaseWords (kPhaseBlocks, one
// 128-byte line each)
constexpr int kMomentTickets = 288;
// most warps per CTA of the potentials' cluster variant (two CTAs per SM:
// the register file holds 2 x 32 x warps threads at <= 65536 / that
// registers each): 16 with the reference colouring (measured faster than 20
// at 48 registers), 20 with the seam-free one, whose two segments then take
// every chunk of a colour in one pass
constexpr int kPotWarpsRef = 16, kPotWarpsFree = 20;
constexpr int kPhaseWords = 352, kPhaseBlocks = 320, kPhaseStride = 32;
constexpr int kBarWords = kPhaseWords + kPhaseBlocks * kPhaseStride;

// ----------------------------------------------------------------------
// Host-side grid: every table the relaxation path reads, built with the
// reference's formulas (initCBAllocArrays.F90 initCBlocks:813-858,
// initSuppl:1636-2051).  Indices are 0-based: nu j in [0,nni), mu i in
// [0,nmu); plain index i*nni+j; extended index (i+4)*n8+(j+4).
// ----------------------------------------------------------------------
struct HostGrid {
  int nni = 0, nmu = 0, n8 = 0, m8 = 0, next = 0, mxsize = 0, mpole = 4;
  double r = 0, r2 = 0, z1 = 0, z2 = 0, rinf = 0, hni = 0, hmu = 0, diag = 0;
  std::vector<double> vxi, vxisq, vxi1, vxi2, veta, vetasq, veta1, veta2, wmu, wni;
  double dmu1[4], dmu2[4], dni1[4], dni2[4], exeven[5];
  std::vector<double> dmu9, dni9;              // 9-point derivative weights (diffmu/diffnu)
  std::vector<double> borb_mu, bpot_mu, f3_mu;  // mu-only coefficient tables
  // the two axis terms of e = e_mu(mu) - e_nu(nu) (e_mu = -1/(xi^2-1),
  // e_nu = 1/(1-eta^2), 0 on the nu axis points, where e is 0)
  std::vector<double> e_mu, e_nu;
  std::vector<double> d_nu;                     // nu-only
  std::vector<double> e, f0, f1, f2, f4, g, wgt1, wgt2;  // plain 2-D tables
  std::vector<double> leg;                      // mpole tables P_k(cos th) r^k, plain
  // "middle" ordering of interior points (ext indices, reference list order)
  std::vector<int> order;
  // sweep schedule: tiles = bands of ext rows [row0,row1)
  int ntiles = 0, nlev = 0;
  std::vector<int> tile_row0, tile_row1;
  std::vector<int> pts;  // ext indices grouped [tile][colour][level]
  std::vector<int> off;  // (ntiles*5*nlev + 1) offsets into pts
  std::vector<int> pts_rc;  // same points as (ext row << 16) | ext col
  // cluster plan of the on-chip FP32 sweep: cl_size CTAs per job, CTA k
  // owns tiles [cl_tile0[k], cl_tile0[k+1]) = ext rows [cl_row0[k], cl_row0[k+1])
  int cl_size = 0, cl_maxrows = 0, cl_maxchunks = 0, cl_wa = 1, cl_wb = 1, cl_ws = 1;
  // warps per role of the potentials' variant (two CTAs per SM, at most kPotWarpsRef)
  int cl_pa = 1, cl_pb = 1, cl_ps = 1;
  // the same CTA bands with the seam-free colouring of the mixed form,
  // colour (col - row) mod 5 in ext coordinates (no two points of a colour
  // within 4 rows or columns of each other on the stencil's cross): per
  // (CTA, colour) the segments A (off the shared band edges), B (within 4
  // rows of one) and an empty seam segment, chunks packed as in cl_pts
  int cf_maxchunks = 0, cf_wa = 1, cf_wb = 1, cf_ws = 0, cf_pa = 1, cf_pb = 1, cf_ps = 0;
  std::vector<int> cf_pts, cf_off;
  size_t cl_smem = 0;
  std::vector<int> cl_tile0, cl_row0;
  // the CTAs' points regrouped [cta][colour][segment] as chunks of up to 4
  // points of one row at stride 5, packed (band row << 19) | (col << 2) |
  // (count - 1); segments: level-0 points off the band edges, level-0 points
  // within 4 rows of an edge shared with another CTA, level-0 seam points
  // (same-colour neighbours of higher levels), then levels 1..nlev-1; cl_off
  // has cl_size * 5 * (nlev + 2) + 1 chunk offsets; cl_wa/wb/ws warps per
  // CTA work on the three kinds
  std::vector<int> cl_pts, cl_off;
  // persistent-band FP32 sweep of grids beyond one cluster: the same points
  // regrouped [colour][level][tile] (st_pts, packed (ext row << 16) | ext
  // col), so that the points of one colour and level in any run of
  // consecutive tiles are one contiguous range; st_off[(c * nlev + l) *
  // (ntiles + 1) + t] is the start of tile t.  st_rows[G] = most rows of any
  // run of G consecutive tiles plus the 4-row halos on both sides (G =
  // 1..kBandRuns)
  static constexpr int kBandRuns = 16;
  std::vector<int> st_pts, st_off;
  int st_rows[kBandRuns + 1] = {};
  // list-order SOR (sor, sormcsor.F90:20-132) as a pipelined wavefront: an
  // interior point's SOR level is 1 + the largest level of its stencil
  // neighbours earlier in the list (their new values are read), an axis
  // point's level 1 + the largest level of the points its extrapolation
  // reads (the corners read the mu=1 row); sweep s of a point runs at step
  // level + s * sor_delta.  sor_pts / sor_bpts hold the interior / axis
  // points by level, packed (ext row << 16) | ext col, with offsets
  // sor_off[sor_nlev + 1] / sor_boff[sor_nblev + 1]
  int sor_nlev = 0, sor_nblev = 0, sor_delta = 0;
  std::vector<int> sor_pts, sor_off, sor_bpts, sor_boff;
};

std::string build_host_grid(HostGrid &g, int nni, int nmu, double r, double rinf, double z1, double z2, int mpole);

// ----------------------------------------------------------------------
// Device view of a grid, passed by value to kernels.
// ----------------------------------------------------------------------
struct GridDev {
  int nni, nmu, n8, m8, next, mxsize, ntiles, nlev, mpole;
  double r2;
  double dmu1[4], dmu2[4], dni1[4], dni2[4], exeven[5], diag;
  const double *borb_mu, *bpot_mu, *f3_mu, *d_nu;
  const double *e, *f0, *f1, *f2, *f4, *g, *wgt1, *wgt2, *leg;
  const double *wf;  // wgt2 f4: the weight of the orbital inner products (Gram-matrix orthonormalisation)
  const double *dmu9, *dni9;
  const double *vxi, *vxisq, *veta, *vetasq;
  const int *tile_row0, *tile_row1, *pts, *off, *pts_rc;
  int cl_size, cl_maxrows, cl_maxchunks, cl_wa, cl_wb, cl_ws, cl_pa, cl_pb, cl_ps;
  int cf_maxchunks, cf_wa, cf_wb, cf_ws, cf_pa, cf_pb, cf_ps;
  const int *cf_pts, *cf_off;
  const int *cl_tile0, *cl_row0, *cl_pts, *cl_off;
  const int *st_pts, *st_off;
  int st_rows[17];
  const int *sor_pts, *sor_off, *sor_bpts, *sor_boff;
  int sor_nlev, sor_nblev, sor_delta;
  // FP32 copies of the coefficient tables for the mixed form
  const float *borb_mu32, *bpot_mu32, *d_nu32;
  const double *e_mu, *e_nu;
  // separable stencil weights of the mixed form's FP64 residual: for the
  // neighbours at distance 4,3,2,1 before and after the point, cmu_*[mu * 8 +
  // q] = dmu2 + b dmu1 (q < 4, before) and dmu2 - b dmu1 (q >= 4, after) with
  // b = borb or bpot; cnu[nu * 8 + q] likewise with dni2, d(nu), dni1
  const double *cmu_orb, *cmu_pot, *cnu;
  // per-grid moment tables (built on the device at grid creation):
  // exm[(idel * 8 + q) * mxsize + k] = wgt2 f4 P_{q+1}^idel(cos th) (r2 r)^(q+1)
  // for idel 0..4, q < mpole; asy[slot * 4 nni + p] on the 4 boundary rows
  // (p = row * nni + nu): slot 0 r2 xi, 1 1/(r2 r), 2+m-1 P_m(cos th)
  // (r2 r)^-(m+1) for m = 1..8, 10 + idel * 8 + m-1 the exchange functions
  // P_m^idel(cos th) (r2 r)^-(m+1), 50 orbAsymptGet's raiq(mu-1) - raiq(mu)
  const double *exm, *asy;
  // FP32 stencil weights, rounded on the host: GB300 issues double->float
  // conversions on its narrow FP64 pipe, so the FP32 kernels never convert
  float dmu1f[4], dmu2f[4], dni1f[4], dni2f[4], exevenf[5];
};

// Device job (one function to relax), built from x2g_job.
struct JobDev {
  double *u;
  const double *lhs;
  const double *rhs;
  const double *psa, *psb;
  double *rhs_buf;  // materialised rhs for potentials
  float *e32;       // mixed: FP32 extended correction
  float *r32, *w32; // mixed: FP32 residual and omega / diagonal
  float2 *rw;       // mixed, persistent-band sweep: (residual, omega / diagonal) in st_pts order
  double omega;
  double idel2;
  float omegaf, omega1f;  // omega and 1 - omega rounded to FP32 on the host
  int isym, kind;
};

// Jobs of one relaxation launch, passed by value as a kernel parameter
// (__grid_constant__): no host-to-device copy per call.  Larger batches are
// split into launches of kParamJobs.
constexpr int kParamJobs = 32;
struct JobTable {
  JobDev j[kParamJobs];
};

// Grid barrier state in device memory.  The error word is sticky: a
// launch that finds it set leaves at its first wait, and only the host's
// readback (x2g_synchronize) clears it, so an error of one launch of a
// multi-launch call survives the launches after it.
struct BarrierDev {
  unsigned int *count;
  unsigned int *gen;
  int *err;                     // first error code (0 = none)
  unsigned long long limit_ns;  // longest wait of one block; 0: a wait not met at its first check fails
};

constexpr unsigned long long kDefaultWaitLimitNs = 2000000000ull;  // 2 s

}  // namespace x2g

struct x2g_ctx {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;  // highest priority
  cudaStream_t aux = nullptr;     // lowest priority, joined back into stream by events
  cudaEvent_t ev_split[2] = {nullptr, nullptr};
  int residual_overlap = 1;       // potential batches in two waves: the second wave's residual under the first's sweep
  // barrier words + error flag (4 ints)
  unsigned int *bar = nullptr;
  // reusable device workspace
  void *work = nullptr;
  size_t work_bytes = 0;
  void *red = nullptr;  // reduction partials
  size_t red_bytes = 0;
  double *host_red = nullptr;  // pinned host buffer for small readbacks
  long long h2d_bytes = 0, d2h_bytes = 0;  // host<->device bytes copied by the library
  long launches = 0;
  size_t cluster_smem_set = 0;  // dynamic shared memory granted to the cluster kernel
  int no_cluster = 0;           // 1: mixed form uses the persistent-band FP32 kernel
  int auto_band = 0;            // 1: batches beyond the co-resident clusters take the persistent-band kernel
  int pot_clusters = 2;         // potentials' cluster variant: 0 never, 1 always, 2 batches above cluster_active[0]
  int mixed_free = 0;           // cluster sweep colouring: 0 the reference's list order mod 5, 1 seam-free
  // [0] the cluster kernel, [1] its potentials' variant:
  int cluster_active[2] = {0, 0};       // clusters co-resident on the device (last shape checked)
  long cluster_checked_key[2] = {-1, -1};  // (shared bytes, cluster size, warps) last checked
  int cluster_ok[2] = {0, 0};             // that cluster shape is schedulable here
  int cluster_nonportable = 0;  // cluster kernels allowed more than 8 CTAs
  int band_attr = 0;            // shared memory cap granted to the persistent-band sweep
  long band_key = -1;           // shared bytes of its last occupancy query
  int band_blocks = 0;          // co-resident blocks for that size
  int band_sm_smem = 0;         // shared memory per SM
  int f64_blocks = -1;          // co-resident blocks of the cooperative FP64 sweep on this device
  int sor_blocks = -1;          // co-resident blocks of the cooperative list-order SOR sweep
  int ortho_blocks = -1;        // co-resident blocks of the one-launch orthonormalisation
  int gram_blocks = -1;         // co-resident blocks of its Gram-matrix form
  int gram_ortho = 0;           // batch mode 2: orthonormalise in rounds (0) or through the Gram matrix (1)
  unsigned long long wait_limit_ns = x2g::kDefaultWaitLimitNs;  // device-side wait limit (x2g_set_wait_limit)
  // optional per-launch timing of the sweep kernels (CUDA events on stream)
  int profiling = 0;
  struct Pending {
    cudaEvent_t a, b;
    int precision;
    double points;  // point-updates performed by the launch
  };
  std::vector<Pending> pending;
  std::vector<cudaEvent_t> event_pool;
  double prof_ms[2] = {0, 0};      // FP64, mixed (FP32 sweep kernel only)
  double prof_points[2] = {0, 0};
  long prof_launches[2] = {0, 0};
};

struct x2g_grid {
  x2g_ctx *ctx = nullptr;
  x2g::HostGrid h;
  x2g::GridDev d{};
  std::vector<void *> allocs;
};

namespace x2g {
// status helpers (x2g_capi.cu)
int set_status(int code, const std::string &msg);
int cuda_status(cudaError_t e, const char *where);
void *ctx_workspace(x2g_ctx *ctx, size_t bytes);
inline void count_copy(x2g_ctx *ctx, size_t h2d, size_t d2h) {
  if (ctx) {
    ctx->h2d_bytes += (long long)h2d;
    ctx->d2h_bytes += (long long)d2h;
  }
}
}  // namespace x2g
