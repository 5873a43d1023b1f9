// Host-side construction of the grid, operator tables and the GPU sweep
// schedule.  The formulas are those of x2dhf's src/initCBAllocArrays.F90
// (initCBlocks:813-858, initSuppl:1636-2051, initLP:1517-1560, mesh:2503-2544)
// written out in 0-based C++; the schedule (row bands, colour levels) is this
// library's own.
#include <algorithm>
#include <memory>
#include <mutex>
#include <cmath>
#include <cstdio>
#include <numeric>

#include "x2g_internal.h"

namespace x2g {

namespace {

// 7-point Newton-Cotes weights on n = 1 (mod 6) points (initSuppl:1917-1955)
std::vector<double> newton_cotes(int n, double h) {
  std::vector<double> w(n + 6, 0.0);
  double w1 = h / 140.0;
  w[0] = 0.0 + w1 * 41.0;
  for (int i = 1; i < n; i += 6) {
    w[i] = w1 * 216.0;
    w[i + 1] = w1 * 27.0;
    w[i + 2] = w1 * 272.0;
    w[i + 3] = w1 * 27.0;
    w[i + 4] = w1 * 216.0;
    w[i + 5] = (i + 5 == n - 1) ? w1 * 41.0 : 2.0 * w1 * 41.0;
  }
  w.resize(n);
  return w;
}

// List-order SOR as a pipelined wavefront.  Sequential SOR over the
// "middle" list (sormcsor.F90:41-74) followed by the axis extrapolation
// (:94-129) after every sweep is reproduced exactly when every point update
// and every axis extrapolation of sweep s runs at step level + s * delta and
// the updates of one step run in any order: a point reads the new values of
// its neighbours earlier in the list (lower levels, this sweep), the previous
// sweep's values of those later in the list and of the axis, and delta makes
// every such previous-sweep value final before it is read and not yet
// overwritten.  The ghost cells and the mu >= nmu-3 rows stay fixed during a
// relaxation call.  Every dependency is checked here; a violation refuses
// the grid.
std::string build_sor_schedule(HostGrid &g, const std::vector<int> &pos, const int *offs) {
  const int npts = int(g.order.size()), n8 = g.n8, nni = g.nni, nmu = g.nmu;
  std::vector<int> L(npts, 0);
  int nlev = 0;
  for (int p = 0; p < npts; ++p) {
    const int ij = g.order[p];
    int l = 0;
    for (int k = 0; k < 16; ++k) {
      const int q = ij + offs[k];
      if (q < 0 || q >= g.next || pos[q] < 0 || pos[q] >= p) continue;
      l = std::max(l, L[pos[q]] + 1);
    }
    L[p] = l;
    nlev = std::max(nlev, l + 1);
  }
  // axis points (sormcsor.F90:94-129, lists of mesh:2823-2842): the mu=1
  // row (ext row 4, cols 5..nni+2) from rows 5..9, then the nu=1 and nu=nni
  // columns (ext rows 4..nmu-1, cols 4 and nni+3) from the 5 columns inward;
  // their row-4 corners read the mu=1 row
  struct Axis {
    int ij, st;
  };
  std::vector<Axis> ax;
  for (int c = 5; c <= nni + 2; ++c) ax.push_back({4 * n8 + c, n8});
  for (int r = 4; r < nmu; ++r) {
    ax.push_back({r * n8 + 4, 1});
    ax.push_back({r * n8 + nni + 3, -1});
  }
  std::vector<int> B(g.next, -1);  // axis level by ext index
  int nblev = 0;
  for (const Axis &a : ax) {
    int b = 0;
    for (int k = 1; k <= 5; ++k) {
      const int q = a.ij + k * a.st;
      const int lq = (pos[q] >= 0) ? L[pos[q]] : B[q];
      if (lq < 0) return "SOR schedule: an axis point reads neither an interior nor an axis point";
      b = std::max(b, lq + 1);
    }
    B[a.ij] = b;
    nblev = std::max(nblev, b + 1);
  }
  // delta: every value a step reads from the previous sweep is final and
  // not yet overwritten by the next
  int delta = 1;
  for (int p = 0; p < npts; ++p) {
    const int ij = g.order[p];
    for (int k = 0; k < 16; ++k) {
      const int q = ij + offs[k];
      if (q < 0 || q >= g.next) continue;
      if (pos[q] > p) delta = std::max(delta, L[pos[q]] - L[p] + 1);  // a later point's old value
      if (B[q] >= 0) delta = std::max(delta, B[q] - L[p] + 1);        // an axis value
    }
  }
  for (const Axis &a : ax)
    for (int k = 1; k <= 5; ++k) {
      const int q = a.ij + k * a.st;
      const int lq = (pos[q] >= 0) ? L[pos[q]] : B[q];
      delta = std::max(delta, B[a.ij] - lq + 1);  // read before the next sweep overwrites it
    }
  // check every dependency at sweeps s and s+1 (step = level + s * delta)
  for (int p = 0; p < npts; ++p) {
    const int ij = g.order[p];
    for (int k = 0; k < 16; ++k) {
      const int q = ij + offs[k];
      if (q < 0 || q >= g.next) continue;
      if (pos[q] >= 0 && pos[q] < p && !(L[pos[q]] < L[p])) return "SOR schedule: new value read too early";
      if (pos[q] > p && !(L[pos[q]] > L[p] && L[pos[q]] < L[p] + delta))
        return "SOR schedule: old value of a later point not preserved";
      if (B[q] >= 0 && !(B[q] > L[p] && B[q] < L[p] + delta)) return "SOR schedule: axis value out of order";
    }
  }
  for (const Axis &a : ax)
    for (int k = 1; k <= 5; ++k) {
      const int q = a.ij + k * a.st;
      const int lq = (pos[q] >= 0) ? L[pos[q]] : B[q];
      if (!(lq < B[a.ij] && B[a.ij] < lq + delta)) return "SOR schedule: extrapolation out of order";
    }
  g.sor_nlev = nlev;
  g.sor_nblev = nblev;
  g.sor_delta = delta;
  g.sor_off.assign(nlev + 1, 0);
  for (int p = 0; p < npts; ++p) g.sor_off[L[p] + 1]++;
  for (int l = 0; l < nlev; ++l) g.sor_off[l + 1] += g.sor_off[l];
  g.sor_pts.assign(npts, 0);
  {
    std::vector<int> fill(g.sor_off.begin(), g.sor_off.end() - 1);
    for (int p = 0; p < npts; ++p) g.sor_pts[fill[L[p]]++] = ((g.order[p] / n8) << 16) | (g.order[p] % n8);
  }
  g.sor_boff.assign(nblev + 1, 0);
  for (const Axis &a : ax) g.sor_boff[B[a.ij] + 1]++;
  for (int l = 0; l < nblev; ++l) g.sor_boff[l + 1] += g.sor_boff[l];
  g.sor_bpts.assign(ax.size(), 0);
  {
    std::vector<int> fill(g.sor_boff.begin(), g.sor_boff.end() - 1);
    for (const Axis &a : ax) g.sor_bpts[fill[B[a.ij]]++] = ((a.ij / n8) << 16) | (a.ij % n8);
  }
  return "";
}

}  // namespace

// Chunks of one segment appended to `chunks`: the segment's points (ext
// row, col) of one CTA band starting at ext row r0 grouped into runs of up to
// 4 points of one row at stride 5, packed (band row << 19) | (col << 2) |
// (count - 1), and dealt round-robin over buckets of the shared-memory bank
// of their first correction value, so that a warp's 32 chunks start on
// distinct banks where the buckets allow.
static void append_chunks(std::vector<std::pair<int, int>> &pts, int r0, int n8, std::vector<int> &chunks) {
  std::sort(pts.begin(), pts.end());
  std::vector<std::vector<int>> bank(32);
  for (size_t i = 0; i < pts.size();) {
    size_t n = 1;
    while (n < 4 && i + n < pts.size() && pts[i + n].first == pts[i].first &&
           pts[i + n].second == pts[i + n - 1].second + 5)
      ++n;
    const int lr = pts[i].first - r0;
    bank[((lr + 4) * n8 + pts[i].second) % 32].push_back(
        int((unsigned(lr) << 19) | (unsigned(pts[i].second) << 2) | unsigned(n - 1)));
    i += n;
  }
  for (size_t depth = 0, left = 1; left;) {
    left = 0;
    for (auto &bk : bank)
      if (depth < bk.size()) {
        chunks.push_back(bk[depth]);
        left = 1;
      }
    ++depth;
  }
}

// Seam-free colouring of the mixed form's cluster sweep on the CTA bands r0:
// colour (col - row) mod 5 of the ext point, so the stencil's neighbours at
// distance 1..4 along a row or a column always have another colour and the
// points of one colour are independent.  No level chain: per (CTA, colour)
// segment A (no halo read or write), B (within 4 rows of a shared band
// edge), and an empty seam segment.
template <class Fit>
static void build_free_plan(HostGrid &g, const std::vector<int> &r0, Fit fit) {
  const int C = int(r0.size()) - 1, S = 3;
  g.cf_pts.clear();
  g.cf_off.assign(size_t(C) * 5 * S + 1, 0);
  int maxchunks = 0, maxa = 0, maxb = 0;
  for (int k = 0; k < C; ++k) {
    const int first = int(g.cf_pts.size());
    auto edge = [&](int row) { return (k > 0 && row < r0[k] + 4) || (k < C - 1 && row >= r0[k + 1] - 4); };
    const int ra = std::max(r0[k], 5), rb = std::min(r0[k + 1], g.nmu);
    for (int c = 0; c < 5; ++c)
      for (int seg = 0; seg < S; ++seg) {
        const int seg0 = int(g.cf_pts.size());
        g.cf_off[(size_t(k) * 5 + c) * S + seg] = seg0;
        if (seg == 2) continue;
        std::vector<std::pair<int, int>> pts;
        for (int row = ra; row < rb; ++row) {
          if (edge(row) != (seg == 1)) continue;
          for (int col = 5; col <= g.nni + 2; ++col)
            if (((col - row) % 5 + 5) % 5 == c) pts.push_back({row, col});
        }
        append_chunks(pts, r0[k], g.n8, g.cf_pts);
        const int n = int(g.cf_pts.size()) - seg0;
        if (seg == 0) maxa = std::max(maxa, n);
        else maxb = std::max(maxb, n);
      }
    maxchunks = std::max(maxchunks, int(g.cf_pts.size()) - first);
  }
  g.cf_off[size_t(C) * 5 * S] = int(g.cf_pts.size());
  g.cf_maxchunks = maxchunks;
  g.cf_wa = std::max(1, (maxa + 31) / 32);
  g.cf_wb = std::max(1, (maxb + 31) / 32);
  g.cf_ws = 0;
  g.cf_pa = g.cf_wa;
  g.cf_pb = g.cf_wb;
  g.cf_ps = 0;
  fit(g.cf_wa, g.cf_wb, g.cf_ws, 24);
  fit(g.cf_pa, g.cf_pb, g.cf_ps, kPotWarpsFree);
}

std::string attach_schedule(HostGrid &g);

std::string build_host_grid(HostGrid &g, int nni, int nmu, double r, double rinf, double z1, double z2,
                            int mpole) {
  if (nni < 13 || nmu < 13 || (nni - 1) % 6 || (nmu - 1) % 6 || (nni - 6) % 5 || (nmu - 6) % 5)
    return "grid sizes must be >= 13 and satisfy n = 1 (mod 6), n - 6 = 0 (mod 5)";
  if (!(r > 0) || !(rinf > r / 2)) return "bond length must be > 0 and R_inf > R/2";
  if (mpole < 2 || mpole > 8) return "mpole must be in [2,8]";
  g.nni = nni;
  g.nmu = nmu;
  g.n8 = nni + 8;
  g.m8 = nmu + 8;
  g.next = g.n8 * g.m8;
  g.mxsize = nni * nmu;
  g.r = r;
  g.r2 = r / 2.0;
  g.z1 = z1;
  g.z2 = z2;
  g.mpole = mpole;
  // grid steps (initCBlocks:813-858)
  g.hni = kPi / double(nni - 1);
  double xmi0 = 2.0 * rinf / r;
  xmi0 = std::log(xmi0 + std::sqrt(xmi0 * xmi0 - 1.0));
  g.hmu = xmi0 / double(nmu - 1);
  g.vxi.assign(nmu, 0);
  g.vxisq.assign(nmu, 0);
  g.vxi1.assign(nmu, 0);
  g.vxi2.assign(nmu, 0);
  double vmu = 0.0;
  for (int i = 0; i < nmu; i++) {
    if (i > 0) vmu = vmu + g.hmu;
    g.vxi[i] = std::cosh(vmu);
    g.vxisq[i] = g.vxi[i] * g.vxi[i];
    g.vxi1[i] = std::sqrt(g.vxi[i] * g.vxi[i] - 1.0);
    g.vxi2[i] = (i == 0) ? 0.0 : g.vxi[i] / g.vxi1[i];
  }
  g.veta.assign(nni, 0);
  g.vetasq.assign(nni, 0);
  g.veta1.assign(nni, 0);
  g.veta2.assign(nni, 0);
  for (int j = 0; j < nni; j++) {
    double vni = double(j) * g.hni;
    g.veta[j] = std::cos(vni);
    g.vetasq[j] = g.veta[j] * g.veta[j];
    g.veta1[j] = std::sqrt(1.0 - g.veta[j] * g.veta[j]);
    g.veta2[j] = (g.veta1[j] < kPrecis) ? 0.0 : g.veta[j] / g.veta1[j];
  }
  g.rinf = r * g.vxi[nmu - 1] / 2.0;
  // supplementary arrays (initSuppl:1759-1911), Coulomb nuclei
  const int mx = g.mxsize;
  g.e.assign(mx, 0);
  g.f0.assign(mx, 0);
  g.f1.assign(mx, 0);
  g.f2.assign(mx, 0);
  g.f4.assign(mx, 0);
  g.g.assign(mx, 0);
  g.wgt1.assign(mx, 0);
  g.wgt2.assign(mx, 0);
  g.borb_mu.assign(nmu, 0);
  g.bpot_mu.assign(nmu, 0);
  g.f3_mu.assign(nmu, 0);
  g.e_mu.assign(nmu, 0);
  g.e_nu.assign(nni, 0);
  g.d_nu = g.veta2;
  g.diag = -14350.0 / (5040.0) * (1.0 / (g.hmu * g.hmu) + 1.0 / (g.hni * g.hni));
  std::vector<double> wjac1(mx), wjac2(mx);
  const double wj1 = -r * kPi / 2.0, wj2 = r * r * kPi / 2.0, xrr = 0.5 * r;
  for (int i = 0; i < nmu; i++) {
    double w1 = g.vxi1[i], w2 = g.vxi[i] * g.vxi[i], w9 = xrr * g.vxi[i], w4 = g.vxi2[i];
    double w5 = 0.0, w6 = 0.0;
    if (i > 0) {
      w5 = g.vxi[i] / g.vxi1[i] - 2.0 * g.vxi1[i] / g.vxi[i];
      w6 = 1.0 / (g.vxi1[i] * g.vxi1[i]);
    }
    double w8 = -r * r * r * kPi * g.vxi[i] / 2.0;
    g.borb_mu[i] = w4;
    g.bpot_mu[i] = w5;
    g.f3_mu[i] = -2.0 / w2 + g.diag;
    g.e_mu[i] = -w6;
    for (int j = 0; j < nni; j++) {
      int ij = i * nni + j;
      double w10 = g.veta1[j];
      g.e[ij] = (w10 < kPrecis) ? 0.0 : (-w6 - 1.0 / (w10 * w10));
      if (i == 0) g.e_nu[j] = (w10 < kPrecis) ? 0.0 : 1.0 / (w10 * w10);
      double w7 = w2 - g.veta[j] * g.veta[j];
      g.f1[ij] = r * r * w7 / 2.0;
      g.f0[ij] = r * (g.vxi[i] * (z1 + z2) + g.veta[j] * (z2 - z1));
      g.f2[ij] = (i == 0) ? 0.0 : -r * w7 / g.vxi[i];
      g.g[ij] = w8 * w7;
      g.f4[ij] = w9;
      wjac1[ij] = wj1 * w1 * w10;
      wjac2[ij] = wj2 * w1 * w10 * (w1 * w1 + w10 * w10) / g.vxi[i];
    }
  }
  g.wmu = newton_cotes(nmu, g.hmu);
  g.wni = newton_cotes(nni, g.hni);
  for (int i = 0; i < nmu; i++)
    for (int j = 0; j < nni; j++) {
      int ij = i * nni + j;
      wjac1[ij] = g.wmu[i] * wjac1[ij];
      wjac2[ij] = g.wmu[i] * wjac2[ij];
      g.wgt1[ij] = g.wni[j] * wjac1[ij];
      g.wgt2[ij] = g.wni[j] * wjac2[ij];
    }
  // 8th-order Stirling coefficients (initSuppl:1680-1683, 1979-2001)
  static const double aa1[9] = {3.0, -32.0, 168.0, -672.0, 0.0, 672.0, -168.0, 32.0, -3.0};
  static const double aa2[9] = {-9.0, 128.0, -1008.0, 8064.0, -14350.0, 8064.0, -1008.0, 128.0, -9.0};
  const double c1 = 1.0 / (840.0), c2 = 1.0 / (5040.0);
  for (int k = 0; k < 4; k++) {
    g.dmu2[k] = c2 * aa2[k] / (g.hmu * g.hmu);
    g.dmu1[k] = c1 * aa1[k] / g.hmu;
    g.dni2[k] = c2 * aa2[k] / (g.hni * g.hni);
    g.dni1[k] = c1 * aa1[k] / g.hni;
  }
  g.dmu9.assign(9 * nmu, 0);
  g.dni9.assign(9 * nni, 0);
  for (int i = 0; i < nmu; i++)
    for (int k = 0; k < 9; k++) {
      double a2 = c2 * aa2[k] / (g.hmu * g.hmu), a1 = c1 * aa1[k] / g.hmu;
      g.dmu9[9 * i + k] = a2 + g.borb_mu[i] * a1;
    }
  for (int j = 0; j < nni; j++)
    for (int k = 0; k < 9; k++) {
      double a2 = c2 * aa2[k] / (g.hni * g.hni), a1 = c1 * aa1[k] / g.hni;
      g.dni9[9 * j + k] = a2 + g.d_nu[j] * a1;
    }
  g.exeven[0] = 210.0 / 126.0;
  g.exeven[1] = -120.0 / 126.0;
  g.exeven[2] = 45.0 / 126.0;
  g.exeven[3] = -10.0 / 126.0;
  g.exeven[4] = 1.0 / 126.0;
  // Legendre polynomials times (R/2 r)^k (initLP:1531-1589)
  g.leg.assign(size_t(mpole) * mx, 0.0);
  for (int i = 0; i < nmu; i++)
    for (int j = 0; j < nni; j++) {
      int ij = i * nni + j;
      double rr = std::sqrt(g.vxisq[i] + g.vetasq[j] - 1.0);
      double xr = g.r2 * rr;
      double costh = (std::fabs(rr) < kPrecis) ? 0.0 : g.vxi[i] * g.veta[j] / rr;
      double dome[10];
      dome[1] = costh;
      dome[2] = (3.0 * costh * costh - 1.0) * 0.50;
      for (int n = 2; n <= mpole - 1; n++)
        dome[n + 1] = (double(2 * n + 1) * costh * dome[n] - double(n) * dome[n - 1]) / double(n + 1);
      double xw = xr;
      g.leg[ij] = dome[1] * xw;
      for (int k = 2; k <= mpole; k++) {
        xw = xw * xr;
        g.leg[size_t(k - 1) * mx + ij] = dome[k] * xw;
      }
    }

  return attach_schedule(g);
}

// The sweep schedules of a grid -- "middle" ordering, colour levels, tiles,
// cluster plans, persistent-band and SOR schedules -- depend on N_nu and
// N_mu only.  build_schedule makes them; attach_schedule copies them from a
// process-wide cache of the most recent grid sizes (they take tens of
// milliseconds to build; a serving loop or repeated solves on one grid size
// build them once).
static std::string build_schedule(HostGrid &g) {
  const int nni = g.nni, nmu = g.nmu;
  // ------------------------------------------------------------------
  // "middle" ordering of the interior points (mesh:2503-2544), 1-based
  // ext rows ii in 6..nmu, cols jj in 6..nni+3, middle-outward.
  // ------------------------------------------------------------------
  const int nmux = (g.m8 - 1) / 2, nnix = (g.n8 - 1) / 2;
  g.order.clear();
  g.order.reserve(size_t(nni - 2) * (nmu - 5));
  for (int i = 6; i <= nmu; i++) {
    int ii = (i <= nmux) ? nmux - i + 6 : i;
    for (int j = 6; j <= nni + 3; j++) {
      int jj = (j <= nnix) ? nnix - j + 6 : j;
      g.order.push_back((ii - 1) * g.n8 + (jj - 1));
    }
  }
  const int npts = int(g.order.size());
  // colour = list position mod 5 (mcsor loops i=c,ngrid1,5)
  std::vector<int> pos(g.next, -1);
  for (int p = 0; p < npts; p++) pos[g.order[p]] = p;
  // colour level: a point waits for every same-colour stencil neighbour
  // earlier in the list (new value read) and, by symmetry, is waited on by
  // every same-colour neighbour later in the list (old value read).
  std::vector<int> lev(npts, 0);
  std::vector<std::pair<int, int>> deps;
  int offs[16];
  for (int k = 1; k <= 4; k++) {
    offs[4 * (k - 1) + 0] = -k;
    offs[4 * (k - 1) + 1] = k;
    offs[4 * (k - 1) + 2] = -k * g.n8;
    offs[4 * (k - 1) + 3] = k * g.n8;
  }
  int maxlev = 0;
  for (int p = 0; p < npts; p++) {
    int ij = g.order[p], L = 0;
    for (int o : offs) {
      int q = ij + o;
      if (q < 0 || q >= g.next) continue;
      int pq = pos[q];
      if (pq < 0 || pq % 5 != p % 5) continue;
      if (pq < p) {
        L = std::max(L, lev[pq] + 1);
        deps.push_back({pq, p});
      }
    }
    lev[p] = L;
    maxlev = std::max(maxlev, L);
  }
  if (maxlev + 1 > kMaxLevels) return "colour level depth exceeds the schedule limit";
  g.nlev = maxlev + 1;
  // row bands: 0-based ext rows [4, nmu); band 0 must hold rows 4..9 (the
  // mu=1 extrapolation reads rows 5..9), ~4 rows each, merged until every
  // same-colour dependency lies inside one band.
  const int H = 4;
  std::vector<int> bounds;
  bounds.push_back(4);
  int b = 10;
  while (b < nmu) {
    bounds.push_back(b);
    b += H;
  }
  bounds.push_back(nmu);
  // a band narrower than 2 rows at the end is merged into its neighbour
  if (bounds.size() > 2 && bounds[bounds.size() - 1] - bounds[bounds.size() - 2] < 2)
    bounds.erase(bounds.end() - 2);
  auto band_of = [&](int row) {
    return int(std::upper_bound(bounds.begin(), bounds.end(), row) - bounds.begin()) - 1;
  };
  for (bool changed = true; changed;) {
    changed = false;
    for (auto &d : deps) {
      int ra = g.order[d.first] / g.n8, rb = g.order[d.second] / g.n8;
      int ta = band_of(ra), tb = band_of(rb);
      if (ta != tb) {
        int lo = std::min(ta, tb), hi = std::max(ta, tb);
        bounds.erase(bounds.begin() + lo + 1, bounds.begin() + hi + 1);
        changed = true;
        break;
      }
    }
  }
  g.ntiles = int(bounds.size()) - 1;
  g.tile_row0.assign(bounds.begin(), bounds.end() - 1);
  g.tile_row1.assign(bounds.begin() + 1, bounds.end());
  // bucket points by (tile, colour, level), list order inside each bucket
  const int nb = g.ntiles * 5 * g.nlev;
  std::vector<int> cnt(nb + 1, 0);
  for (int p = 0; p < npts; p++) {
    int t = band_of(g.order[p] / g.n8);
    cnt[(t * 5 + p % 5) * g.nlev + lev[p] + 1]++;
  }
  for (int k = 0; k < nb; k++) cnt[k + 1] += cnt[k];
  g.off = cnt;
  g.pts.assign(npts, 0);
  std::vector<int> fill(cnt.begin(), cnt.end() - 1);
  for (int p = 0; p < npts; p++) {
    int t = band_of(g.order[p] / g.n8);
    g.pts[fill[(t * 5 + p % 5) * g.nlev + lev[p]]++] = g.order[p];
  }
  g.st_pts.clear();
  g.st_pts.reserve(g.pts.size());
  g.st_off.assign(size_t(5) * g.nlev * (g.ntiles + 1), 0);
  for (int c = 0; c < 5; ++c)
    for (int l = 0; l < g.nlev; ++l) {
      int *so = &g.st_off[size_t(c * g.nlev + l) * (g.ntiles + 1)];
      for (int t = 0; t < g.ntiles; ++t) {
        so[t] = int(g.st_pts.size());
        const int o = (t * 5 + c) * g.nlev + l;
        for (int k = g.off[o]; k < g.off[o + 1]; ++k) g.st_pts.push_back(((g.pts[k] / g.n8) << 16) | (g.pts[k] % g.n8));
      }
      so[g.ntiles] = int(g.st_pts.size());
    }
  for (int G = 1; G <= HostGrid::kBandRuns; ++G) {
    int most = 0;
    for (int t0 = 0; t0 < g.ntiles; t0 += G) {
      const int t1 = std::min(t0 + G, g.ntiles);
      most = std::max(most, g.tile_row1[t1 - 1] - g.tile_row0[t0]);
    }
    g.st_rows[G] = most + 8;
  }
  g.pts_rc.resize(g.pts.size());
  for (size_t k = 0; k < g.pts.size(); ++k) g.pts_rc[k] = ((g.pts[k] / g.n8) << 16) | (g.pts[k] % g.n8);
  // cluster plan for the on-chip FP32 sweep: contiguous tile ranges, ~30
  // rows per CTA, 2..16 CTAs; each CTA keeps its FP32 band with 4-row halos
  // plus the band's residual, omega/lhs, coefficient rows and point list in
  // shared memory
  g.cl_size = 0;
  {
    const int rows = nmu - 4;
    int C = std::max(2, std::min(16, (rows + 29) / 30));
    C = std::min(C, g.ntiles);
    if (C >= 2) {
      std::vector<int> t0(C + 1), r0(C + 1);
      int t = 0;
      t0[0] = 0;
      for (int k = 1; k < C; ++k) {
        const int target = 4 + (rows * k + C / 2) / C;
        while (t < g.ntiles - (C - k) && g.tile_row1[t] <= target) ++t;
        if (t <= t0[k - 1]) t = t0[k - 1] + 1;
        t0[k] = t;
      }
      t0[C] = g.ntiles;
      bool ok = true;
      int maxrows = 0;
      for (int k = 0; k < C; ++k) {
        if (t0[k + 1] <= t0[k]) ok = false;
        r0[k] = g.tile_row0[t0[k]];
        maxrows = std::max(maxrows, g.tile_row1[t0[k + 1] - 1] - g.tile_row0[t0[k]]);
      }
      r0[C] = nmu;
      // Per (CTA, colour) nlev+2 segments, each processed by its own warps:
      //   A  level-0 points off the band edges (no halo read or write),
      //   B  level-0 points within 4 rows of an edge shared with another CTA,
      //   S0 level-0 points with a same-colour stencil neighbour of a higher
      //      level (seam points), S1.. the levels 1..nlev-1.
      // A and B points have no same-colour neighbour at all, so A, B and S0
      // run concurrently and only the seam warps step through the levels.
      // Each segment is stored as chunks of up to 4 of its points on one row
      // at stride 5 (same-colour points of a row are 5 columns apart),
      // packed (band row << 19) | (col << 2) | (count - 1).
      const int S = g.nlev + 2;
      std::vector<char> seam0(g.next, 0);
      for (auto &d : deps)
        if (lev[d.first] == 0) seam0[g.order[d.first]] = 1;
      std::vector<int> chunks, coff(size_t(C) * 5 * S + 1, 0);
      int maxchunks = 0, maxa = 0, maxb = 0, maxs = 0;
      for (int k = 0; k < C; ++k) {
        const int first = int(chunks.size());
        auto edge = [&](int row) { return (k > 0 && row < r0[k] + 4) || (k < C - 1 && row >= r0[k + 1] - 4); };
        for (int c = 0; c < 5; ++c)
          for (int seg = 0; seg < S; ++seg) {
            const int seg0 = int(chunks.size());
            coff[(size_t(k) * 5 + c) * S + seg] = seg0;
            const int l = (seg < 2) ? 0 : seg - 2;
            std::vector<std::pair<int, int>> pts;
            for (int t = t0[k]; t < t0[k + 1]; ++t) {
              const int o = (t * 5 + c) * g.nlev + l;
              for (int q = g.off[o]; q < g.off[o + 1]; ++q) {
                const int row = g.pts_rc[q] >> 16, col = g.pts_rc[q] & 0xffff;
                const bool s0 = seam0[row * g.n8 + col] != 0;
                if (seg == 0 && (s0 || edge(row))) continue;
                if (seg == 1 && (s0 || !edge(row))) continue;
                if (seg == 2 && !s0) continue;
                pts.push_back({row, col});
              }
            }
            append_chunks(pts, r0[k], g.n8, chunks);
            const int n = int(chunks.size()) - seg0;
            if (seg == 0) maxa = std::max(maxa, n);
            else if (seg == 1) maxb = std::max(maxb, n);
            else maxs = std::max(maxs, n);
          }
        maxchunks = std::max(maxchunks, int(chunks.size()) - first);
      }
      coff[size_t(C) * 5 * S] = int(chunks.size());
      // shared memory: (residual, omega/lhs) pairs, correction band with
      // 4-row halos, b(mu) of the band's rows, d(nu) by column, the segment
      // offsets, then the CTA's chunk list
      const size_t smem = 2 * size_t(maxrows) * g.n8 * sizeof(float) + size_t(maxrows + 8) * g.n8 * sizeof(float) +
                          size_t(maxrows + g.n8) * sizeof(float) + size_t(5 * S + 1) * sizeof(int) +
                          size_t(maxchunks) * sizeof(int);
      // a band must be at least 4 rows (halo pushes go to the next CTA only)
      for (int k = 0; k < C; ++k)
        if (r0[k + 1] - r0[k] < 4) ok = false;
      if (ok && maxrows < 4096 && g.n8 < (1 << 17) && smem <= 200 * 1024) {
        g.cl_size = C;
        g.cl_maxrows = maxrows;
        g.cl_maxchunks = maxchunks;
        // warps per role: enough for one pass over the largest segment, at
        // most 24 warps in all (the roles loop when a segment is larger)
        g.cl_wa = std::max(1, (maxa + 31) / 32);
        g.cl_wb = std::max(1, (maxb + 31) / 32);
        g.cl_ws = std::max(1, (maxs + 31) / 32);
        auto fit = [](int &a, int &b, int &c, int most) {
          while (a + b + c > most) {
            if (a >= b && a >= c) --a;
            else if (b >= c) --b;
            else --c;
          }
        };
        g.cl_pa = g.cl_wa;
        g.cl_pb = g.cl_wb;
        g.cl_ps = g.cl_ws;
        fit(g.cl_wa, g.cl_wb, g.cl_ws, 24);
        fit(g.cl_pa, g.cl_pb, g.cl_ps, kPotWarpsRef);
        g.cl_smem = smem;
        g.cl_tile0 = t0;
        g.cl_row0 = r0;
        g.cl_pts = chunks;
        g.cl_off = coff;
        build_free_plan(g, r0, fit);
      }
    }
  }
  // final check: no two points of one (tile,colour,level) bucket interact,
  // and every dependency is inside a tile with a strictly larger level
  for (auto &d : deps) {
    int ra = g.order[d.first] / g.n8, rb = g.order[d.second] / g.n8;
    if (band_of(ra) != band_of(rb)) return "schedule check: dependency crosses a tile";
    if (!(lev[d.second] > lev[d.first])) return "schedule check: level order violated";
  }
  return build_sor_schedule(g, pos, offs);
}


namespace {
struct ScheduleCache {
  std::mutex m;
  std::vector<std::shared_ptr<const HostGrid>> entries;  // most recent last
};
ScheduleCache &schedule_cache() {
  static ScheduleCache c;
  return c;
}
void copy_schedule(HostGrid &to, const HostGrid &from) {
  to.order = from.order;
  to.ntiles = from.ntiles;
  to.nlev = from.nlev;
  to.tile_row0 = from.tile_row0;
  to.tile_row1 = from.tile_row1;
  to.pts = from.pts;
  to.off = from.off;
  to.pts_rc = from.pts_rc;
  to.cl_size = from.cl_size;
  to.cl_maxrows = from.cl_maxrows;
  to.cl_maxchunks = from.cl_maxchunks;
  to.cl_wa = from.cl_wa;
  to.cl_wb = from.cl_wb;
  to.cl_ws = from.cl_ws;
  to.cl_pa = from.cl_pa;
  to.cl_pb = from.cl_pb;
  to.cl_ps = from.cl_ps;
  to.cl_smem = from.cl_smem;
  to.cl_tile0 = from.cl_tile0;
  to.cl_row0 = from.cl_row0;
  to.cl_pts = from.cl_pts;
  to.cl_off = from.cl_off;
  to.cf_maxchunks = from.cf_maxchunks;
  to.cf_wa = from.cf_wa;
  to.cf_wb = from.cf_wb;
  to.cf_ws = from.cf_ws;
  to.cf_pa = from.cf_pa;
  to.cf_pb = from.cf_pb;
  to.cf_ps = from.cf_ps;
  to.cf_pts = from.cf_pts;
  to.cf_off = from.cf_off;
  to.st_pts = from.st_pts;
  to.st_off = from.st_off;
  for (int k = 0; k <= HostGrid::kBandRuns; ++k) to.st_rows[k] = from.st_rows[k];
  to.sor_nlev = from.sor_nlev;
  to.sor_nblev = from.sor_nblev;
  to.sor_delta = from.sor_delta;
  to.sor_pts = from.sor_pts;
  to.sor_off = from.sor_off;
  to.sor_bpts = from.sor_bpts;
  to.sor_boff = from.sor_boff;
}
constexpr size_t kScheduleCacheEntries = 8;
}  // namespace

std::string attach_schedule(HostGrid &g) {
  ScheduleCache &c = schedule_cache();
  {
    std::lock_guard<std::mutex> lock(c.m);
    for (auto &e : c.entries)
      if (e->nni == g.nni && e->nmu == g.nmu) {
        copy_schedule(g, *e);
        return "";
      }
  }
  std::string msg = build_schedule(g);
  if (!msg.empty()) return msg;
  auto keep = std::make_shared<HostGrid>();
  keep->nni = g.nni;
  keep->nmu = g.nmu;
  copy_schedule(*keep, g);
  std::lock_guard<std::mutex> lock(c.m);
  c.entries.push_back(std::move(keep));
  if (c.entries.size() > kScheduleCacheEntries) c.entries.erase(c.entries.begin());
  return "";
}

}  // namespace x2g

// ---------------------------------------------------------------------
// CUDA-free access to the host-side tables (used by CPU tests)
// ---------------------------------------------------------------------
extern "C" int x2g_host_table(int nnu, int nmu, double r, double rinf, double z1, double z2, int which,
                              double *out) {
  x2g::HostGrid g;
  std::string msg = x2g::build_host_grid(g, nnu, nmu, r, rinf, z1, z2, 4);
  if (!msg.empty()) return X2G_ERR_ARG;
  for (int i = 0; i < nmu; ++i)
    for (int j = 0; j < nnu; ++j) {
      const int k = i * nnu + j;
      double v;
      switch (which) {
        case 0: v = g.borb_mu[i]; break;
        case 1: v = g.bpot_mu[i]; break;
        case 2: v = g.d_nu[j]; break;
        case 3: v = g.e[k]; break;
        case 4: v = g.f0[k]; break;
        case 5: v = g.f1[k]; break;
        case 6: v = g.f2[k]; break;
        case 7: v = g.f3_mu[i]; break;
        case 8: v = g.f4[k]; break;
        case 9: v = g.g[k]; break;
        case 10: v = g.wgt1[k]; break;
        case 11: v = g.wgt2[k]; break;
        default: return X2G_ERR_ARG;
      }
      out[k] = v;
    }
  return X2G_OK;
}

// Sweep order and schedule of the host grid: order[npoints] (ext indices,
// 0-based, reference list order), tile/colour/level of every point.
extern "C" int x2g_host_schedule(int nnu, int nmu, int *npoints, int *ntiles, int *nlevels, int *order,
                                 int *tile, int *colour, int *level) {
  x2g::HostGrid g;
  std::string msg = x2g::build_host_grid(g, nnu, nmu, 2.0, 40.0, 1.0, 1.0, 4);
  if (!msg.empty()) return X2G_ERR_SCHEDULE;
  if (npoints) *npoints = int(g.order.size());
  if (ntiles) *ntiles = g.ntiles;
  if (nlevels) *nlevels = g.nlev;
  if (order) std::copy(g.order.begin(), g.order.end(), order);
  if (tile && colour && level) {
    for (int t = 0; t < g.ntiles; ++t)
      for (int c = 0; c < 5; ++c)
        for (int l = 0; l < g.nlev; ++l) {
          const int o = (t * 5 + c) * g.nlev + l;
          for (int k = g.off[o]; k < g.off[o + 1]; ++k) {
            tile[k] = t;
            colour[k] = c;
            level[k] = l;
            order[k] = g.pts[k];
          }
        }
  }
  return X2G_OK;
}

// Cluster plan of the on-chip FP32 sweep (no CUDA call): CTAs per job,
// rows per CTA, shared memory bytes; row0[C+1] when non-NULL.
extern "C" int x2g_host_cluster_plan(int nnu, int nmu, int *csize, int *maxrows, long *smem, int *row0) {
  x2g::HostGrid g;
  std::string msg = x2g::build_host_grid(g, nnu, nmu, 2.0, 40.0, 1.0, 1.0, 4);
  if (!msg.empty()) return X2G_ERR_SCHEDULE;
  if (csize) *csize = g.cl_size;
  if (maxrows) *maxrows = g.cl_maxrows;
  if (smem) *smem = long(g.cl_smem);
  if (row0 && g.cl_size > 0) std::copy(g.cl_row0.begin(), g.cl_row0.end(), row0);
  return X2G_OK;
}

// Chunk lists of the on-chip sweep: nchunks packed chunks and noff segment
// offsets (CTA-major, 5 colours x (nlevels + 1) segments per CTA, plus the
// end).  Call with null arrays for the counts.
extern "C" int x2g_host_band_schedule(int nnu, int nmu, int *npoints, int *ntiles, int *nlevels, int *pts, int *off,
                                      int *rows, int *tile_row0, int *tile_row1) {
  x2g::HostGrid g;
  std::string msg = x2g::build_host_grid(g, nnu, nmu, 2.0, 40.0, 1.0, 1.0, 4);
  if (!msg.empty()) return X2G_ERR_SCHEDULE;
  if (npoints) *npoints = int(g.st_pts.size());
  if (ntiles) *ntiles = g.ntiles;
  if (nlevels) *nlevels = g.nlev;
  if (pts) std::copy(g.st_pts.begin(), g.st_pts.end(), pts);
  if (off) std::copy(g.st_off.begin(), g.st_off.end(), off);
  if (rows) std::copy(g.st_rows, g.st_rows + x2g::HostGrid::kBandRuns + 1, rows);
  if (tile_row0) std::copy(g.tile_row0.begin(), g.tile_row0.end(), tile_row0);
  if (tile_row1) std::copy(g.tile_row1.begin(), g.tile_row1.end(), tile_row1);
  return X2G_OK;
}

extern "C" int x2g_host_cluster_chunks(int nnu, int nmu, int *nchunks, int *noff, int *chunks, int *off) {
  x2g::HostGrid g;
  std::string msg = x2g::build_host_grid(g, nnu, nmu, 2.0, 40.0, 1.0, 1.0, 4);
  if (!msg.empty()) return X2G_ERR_SCHEDULE;
  if (nchunks) *nchunks = int(g.cl_pts.size());
  if (noff) *noff = int(g.cl_off.size());
  if (chunks) std::copy(g.cl_pts.begin(), g.cl_pts.end(), chunks);
  if (off) std::copy(g.cl_off.begin(), g.cl_off.end(), off);
  return X2G_OK;
}

// The same for the seam-free colouring of the mixed form (colour (col - row)
// mod 5; per CTA and colour the segments A, B and an empty seam segment).
extern "C" int x2g_host_free_chunks(int nnu, int nmu, int *nchunks, int *noff, int *chunks, int *off) {
  x2g::HostGrid g;
  std::string msg = x2g::build_host_grid(g, nnu, nmu, 2.0, 40.0, 1.0, 1.0, 4);
  if (!msg.empty()) return X2G_ERR_SCHEDULE;
  if (nchunks) *nchunks = int(g.cf_pts.size());
  if (noff) *noff = int(g.cf_off.size());
  if (chunks) std::copy(g.cf_pts.begin(), g.cf_pts.end(), chunks);
  if (off) std::copy(g.cf_off.begin(), g.cf_off.end(), off);
  return X2G_OK;
}

// Schedule of the list-order SOR wavefront (host only): interior points by
// SOR level, packed (ext row << 16) | ext col (pts, npoints values; off,
// nlev + 1 offsets), axis points by the level their extrapolation follows
// (bpts; boff, nblev + 1 offsets), and the level shift between sweeps.
// Null arrays: counts only.
extern "C" int x2g_host_sor_schedule(int nnu, int nmu, int *npoints, int *nlev, int *nblev, int *delta, int *pts,
                                     int *off, int *bpts, int *boff) {
  x2g::HostGrid g;
  std::string msg = x2g::build_host_grid(g, nnu, nmu, 2.0, 40.0, 1.0, 1.0, 4);
  if (!msg.empty()) return X2G_ERR_SCHEDULE;
  if (npoints) *npoints = int(g.sor_pts.size());
  if (nlev) *nlev = g.sor_nlev;
  if (nblev) *nblev = g.sor_nblev;
  if (delta) *delta = g.sor_delta;
  if (pts) std::copy(g.sor_pts.begin(), g.sor_pts.end(), pts);
  if (off) std::copy(g.sor_off.begin(), g.sor_off.end(), off);
  if (bpts) std::copy(g.sor_bpts.begin(), g.sor_bpts.end(), bpts);
  if (boff) std::copy(g.sor_boff.begin(), g.sor_boff.end(), boff);
  return X2G_OK;
}
