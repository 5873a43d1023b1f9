// CUDA kernels of the x2dhf GB300 relaxation library (sm_103a).
//
// Layout: every function lives in the reference's extended layout
// ((nni+8) x (nmu+8) doubles, nu fastest), so putin reduces to a ghost
// refresh and putout to nothing.  Plain 2-D tables are nni x nmu.
//
// FP64 arithmetic that must reproduce the reference bit for bit is written
// with __dadd_rn/__dmul_rn/__ddiv_rn, which the compiler never contracts
// into FMAs (the reference was built without FMA contraction).
#include <algorithm>
#include <cooperative_groups.h>
#include <cstdio>
#include <vector>

#include "x2g_kernels.cuh"

namespace x2g {

namespace {

constexpr int kThreads = 256;
constexpr int kBandThreads = 512;

__device__ __forceinline__ double A(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double S(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double M(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double D(double a, double b) { return __ddiv_rn(a, b); }

template <typename T>
__device__ __forceinline__ T ldcg(const T *p) {
  return __ldcg(p);
}

__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Whether a wait that started at t0 has run out: checked every 256 spins,
// or at every spin when the limit is 0 (a wait not met at once fails).
__device__ __forceinline__ bool wait_expired(const BarrierDev &b, unsigned spins, unsigned long long t0) {
  return (b.limit_ns == 0 || (spins & 255u) == 0) && globaltimer() - t0 >= b.limit_ns;
}

// Grid-wide barrier for a cooperative launch.  Every wait is bounded: after
// b.limit_ns the block records X2G_ERR_TIMEOUT and all blocks leave the
// kernel at their next barrier; a launch that finds the error word already
// set leaves at its first barrier.  Returns false when the kernel must stop.
__device__ bool grid_barrier(const BarrierDev &b, unsigned nblocks) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    volatile unsigned *vgen = b.gen;
    volatile int *verr = b.err;
    const unsigned g0 = *vgen;
    __threadfence();
    const unsigned arrived = atomicAdd(b.count, 1u);
    if (arrived == nblocks - 1) {
      atomicExch(b.count, 0u);
      __threadfence();
      atomicAdd(b.gen, 1u);
    } else {
      const unsigned long long t0 = globaltimer();
      unsigned spins = 0;
      while (*vgen == g0) {
        if (*verr) {
          ok = 0;
          break;
        }
        if (wait_expired(b, ++spins, t0)) {
          atomicCAS(b.err, 0, X2G_ERR_TIMEOUT);
          ok = 0;
          break;
        }
        __nanosleep(32);
      }
    }
    __threadfence();
    if (*verr) ok = 0;
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

__device__ __forceinline__ unsigned ld_acquire(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Neighbour wait of the persistent-band sweep: block b publishes in
// phase[b] how many colour phases it has finished (release store after its
// writes), and before reloading its halos for phase k waits until every
// block whose rows lie within 4 rows of its band (nb[0..5], -1 = none) has
// finished k phases (acquire loads by lanes 0..5 of warp 0), while lane 6
// reads the error word once, so that a launch started after an error leaves
// at its first wait.  The wait is bounded as in grid_barrier.
__device__ __forceinline__ void st_release(unsigned *p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ bool wait_neighbours(const BarrierDev &b, const unsigned *phase, int nbq, unsigned k) {
  __shared__ int s_ok;
  if (threadIdx.x < 32) {
    int ok = 1;
    volatile int *verr = b.err;
    if (threadIdx.x == 6) {
      if (*verr) ok = 0;
    } else if (nbq >= 0) {
      const unsigned long long t0 = globaltimer();
      unsigned spins = 0;
      while (ld_acquire(phase + size_t(nbq) * kPhaseStride) < k) {
        if (*verr) {
          ok = 0;
          break;
        }
        if (wait_expired(b, ++spins, t0)) {
          atomicCAS(b.err, 0, X2G_ERR_TIMEOUT);
          ok = 0;
          break;
        }
        __nanosleep(20);
      }
      __threadfence();
    }
    ok = __all_sync(0xffffffffu, ok);
    if (threadIdx.x == 0) s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// ----------------------------------------------------------------------
// One point update, FP64, reference arithmetic order (sormcsor.F90:46-71).
// ----------------------------------------------------------------------
__device__ __forceinline__ void relax_f64(double *__restrict__ u, int ij, const GridDev &g, double b, double d,
                                          double lhs, double rhs, double omega, double omega1) {
  const int n1 = g.n8, n2 = 2 * g.n8, n3 = 3 * g.n8, n4 = 4 * g.n8;
  const double m4 = ldcg(u + ij - n4), p4 = ldcg(u + ij + n4);
  const double m3 = ldcg(u + ij - n3), p3 = ldcg(u + ij + n3);
  const double m2 = ldcg(u + ij - n2), p2 = ldcg(u + ij + n2);
  const double m1 = ldcg(u + ij - n1), p1 = ldcg(u + ij + n1);
  const double l4 = ldcg(u + ij - 4), r4 = ldcg(u + ij + 4);
  const double l3 = ldcg(u + ij - 3), r3 = ldcg(u + ij + 3);
  const double l2 = ldcg(u + ij - 2), r2 = ldcg(u + ij + 2);
  const double l1 = ldcg(u + ij - 1), r1 = ldcg(u + ij + 1);
  const double uc = ldcg(u + ij);
  const double ddmi2 =
      A(A(A(M(g.dmu2[0], A(m4, p4)), M(g.dmu2[1], A(m3, p3))), M(g.dmu2[2], A(m2, p2))), M(g.dmu2[3], A(m1, p1)));
  const double ddmi1 =
      A(A(A(M(g.dmu1[0], S(m4, p4)), M(g.dmu1[1], S(m3, p3))), M(g.dmu1[2], S(m2, p2))), M(g.dmu1[3], S(m1, p1)));
  const double ddni2 =
      A(A(A(M(g.dni2[0], A(l4, r4)), M(g.dni2[1], A(l3, r3))), M(g.dni2[2], A(l2, r2))), M(g.dni2[3], A(l1, r1)));
  const double ddni1 =
      A(A(A(M(g.dni1[0], S(l4, r4)), M(g.dni1[1], S(l3, r3))), M(g.dni1[2], S(l2, r2))), M(g.dni1[3], S(l1, r1)));
  const double cc = A(A(A(ddmi2, M(b, ddmi1)), ddni2), M(d, ddni1));
  u[ij] = A(D(M(omega, S(rhs, cc)), lhs), M(omega1, uc));
}

struct CoefF {
  float dmu1[4], dmu2[4], dni1[4], dni2[4];
};

// FP32 correction sweep point update (same operator, FMA allowed) on a band
// of the correction held in shared memory; w is omega / lhs of the point,
// formed once per relaxation call.  Returns the new value.
__device__ __forceinline__ float relax_f32(const float *__restrict__ e, int ij, int n8, const CoefF &c, float b,
                                           float d, float w, float r, float omega1) {
  const int n1 = n8, n2 = 2 * n8, n3 = 3 * n8, n4 = 4 * n8;
  const float m4 = e[ij - n4], p4 = e[ij + n4];
  const float m3 = e[ij - n3], p3 = e[ij + n3];
  const float m2 = e[ij - n2], p2 = e[ij + n2];
  const float m1 = e[ij - n1], p1 = e[ij + n1];
  const float l4 = e[ij - 4], r4 = e[ij + 4];
  const float l3 = e[ij - 3], r3 = e[ij + 3];
  const float l2 = e[ij - 2], r2 = e[ij + 2];
  const float l1 = e[ij - 1], r1 = e[ij + 1];
  const float ec = e[ij];
  float dm2 = c.dmu2[0] * (m4 + p4);
  dm2 = __fmaf_rn(c.dmu2[1], m3 + p3, dm2);
  dm2 = __fmaf_rn(c.dmu2[2], m2 + p2, dm2);
  dm2 = __fmaf_rn(c.dmu2[3], m1 + p1, dm2);
  float dm1 = c.dmu1[0] * (m4 - p4);
  dm1 = __fmaf_rn(c.dmu1[1], m3 - p3, dm1);
  dm1 = __fmaf_rn(c.dmu1[2], m2 - p2, dm1);
  dm1 = __fmaf_rn(c.dmu1[3], m1 - p1, dm1);
  float dn2 = c.dni2[0] * (l4 + r4);
  dn2 = __fmaf_rn(c.dni2[1], l3 + r3, dn2);
  dn2 = __fmaf_rn(c.dni2[2], l2 + r2, dn2);
  dn2 = __fmaf_rn(c.dni2[3], l1 + r1, dn2);
  float dn1 = c.dni1[0] * (l4 - r4);
  dn1 = __fmaf_rn(c.dni1[1], l3 - r3, dn1);
  dn1 = __fmaf_rn(c.dni1[2], l2 - r2, dn1);
  dn1 = __fmaf_rn(c.dni1[3], l1 - r1, dn1);
  const float cc = __fmaf_rn(d, dn1, __fmaf_rn(b, dm1, dm2) + dn2);
  return __fmaf_rn(omega1, ec, w * (r - cc));
}

// ----------------------------------------------------------------------
// Tile-local pieces of one relaxation call.  A tile is a band of ext rows
// [row0,row1) over the full nu width.
// ----------------------------------------------------------------------

// putin ghosts for the tile's rows (src/inout.F90:47-80): ghost columns copy
// nu = 2..5 / nni-1..nni-4, tile 0 also fills the mu ghost rows.
__device__ void tile_ghosts(const GridDev &g, double *u, int t, int isym) {
  const int row0 = g.tile_row0[t], row1 = g.tile_row1[t], n8 = g.n8, nni = g.nni;
  const bool neg = (isym != 1);
  const int nr = row1 - row0;
  for (int k = threadIdx.x; k < nr * 8; k += blockDim.x) {
    const int r = row0 + k / 8, q = k % 8;
    const int base = r * n8;
    if (q < 4) {
      const int j = q + 1;  // ghost col 4-j <- col 4+j
      const double v = ldcg(u + base + 4 + j);
      u[base + 4 - j] = neg ? -v : v;
    } else {
      const int j = q - 3;  // ghost col nni+3+j <- col nni+3-j
      const double v = ldcg(u + base + nni + 3 - j);
      u[base + nni + 3 + j] = neg ? -v : v;
    }
  }
  if (t == 0) {
    for (int k = threadIdx.x; k < 4 * nni; k += blockDim.x) {
      const int i = k / nni + 1, col = 4 + k % nni;  // ghost row 4-i <- row 4+i
      const double v = ldcg(u + (4 + i) * n8 + col);
      u[(4 - i) * n8 + col] = neg ? -v : v;
    }
  }
}

// Axis extrapolation after a micro-sweep (sormcsor.F90:94-129): mu=1 row
// (tile 0), nu=1 and nu=nni columns of the tile's rows; the two corners at
// mu=1 read the freshly extrapolated mu=1 row, so they follow a sync.
template <typename T>
__device__ void tile_boundary(const GridDev &g, T *u, int t, int isym) {
  const int row0 = g.tile_row0[t], row1 = g.tile_row1[t], n8 = g.n8, nni = g.nni;
  const int n1 = n8, n2 = 2 * n8, n3 = 3 * n8, n4 = 4 * n8, n5 = 5 * n8;
  const bool even = (isym == 1);
  const int nrow7 = (t == 0) ? nni - 2 : 0;
  const int r0 = (t == 0) ? 5 : row0;
  const int nside = 2 * (row1 - r0);
  for (int k = threadIdx.x; k < nrow7 + nside; k += blockDim.x) {
    if (k < nrow7) {
      const int ij = 4 * n8 + 5 + k;
      T v = T(0);
      if (even) {
        if constexpr (sizeof(T) == 8) {
          v = A(A(A(A(M(g.exeven[0], ldcg(u + ij + n1)), M(g.exeven[1], ldcg(u + ij + n2))),
                    M(g.exeven[2], ldcg(u + ij + n3))),
                  M(g.exeven[3], ldcg(u + ij + n4))),
                M(g.exeven[4], ldcg(u + ij + n5)));
        } else {
          v = g.exevenf[0] * ldcg(u + ij + n1) + g.exevenf[1] * ldcg(u + ij + n2) +
              g.exevenf[2] * ldcg(u + ij + n3) + g.exevenf[3] * ldcg(u + ij + n4) +
              g.exevenf[4] * ldcg(u + ij + n5);
        }
      }
      u[ij] = v;
    } else {
      const int q = k - nrow7;
      const int r = r0 + q / 2;
      const int side = q % 2;
      const int ij = r * n8 + (side == 0 ? 4 : nni + 3);
      const int s = (side == 0) ? 1 : -1;
      T v = T(0);
      if (even) {
        if constexpr (sizeof(T) == 8) {
          v = A(A(A(A(M(g.exeven[0], ldcg(u + ij + s)), M(g.exeven[1], ldcg(u + ij + 2 * s))),
                    M(g.exeven[2], ldcg(u + ij + 3 * s))),
                  M(g.exeven[3], ldcg(u + ij + 4 * s))),
                M(g.exeven[4], ldcg(u + ij + 5 * s)));
        } else {
          v = g.exevenf[0] * ldcg(u + ij + s) + g.exevenf[1] * ldcg(u + ij + 2 * s) +
              g.exevenf[2] * ldcg(u + ij + 3 * s) + g.exevenf[3] * ldcg(u + ij + 4 * s) +
              g.exevenf[4] * ldcg(u + ij + 5 * s);
        }
      }
      u[ij] = v;
    }
  }
  if (t == 0) {
    __syncthreads();
    if (threadIdx.x < 2) {
      const int ij = 4 * n8 + (threadIdx.x == 0 ? 4 : nni + 3);
      const int s = (threadIdx.x == 0) ? 1 : -1;
      T v = T(0);
      if (even) {
        if constexpr (sizeof(T) == 8) {
          v = A(A(A(A(M(g.exeven[0], ldcg(u + ij + s)), M(g.exeven[1], ldcg(u + ij + 2 * s))),
                    M(g.exeven[2], ldcg(u + ij + 3 * s))),
                  M(g.exeven[3], ldcg(u + ij + 4 * s))),
                M(g.exeven[4], ldcg(u + ij + 5 * s)));
        } else {
          v = g.exevenf[0] * ldcg(u + ij + s) + g.exevenf[1] * ldcg(u + ij + 2 * s) +
              g.exevenf[2] * ldcg(u + ij + 3 * s) + g.exevenf[3] * ldcg(u + ij + 4 * s) +
              g.exevenf[4] * ldcg(u + ij + 5 * s);
        }
      }
      u[ij] = v;
    }
  }
}

// Potential right-hand side for the tile's interior points
// (relaxPots.F90:81-82: rhs = psi_a psi_b g, two successive products).
__device__ void tile_rhs(const GridDev &g, const JobDev &J, int t) {
  const int b0 = g.off[(t * 5) * g.nlev], b1 = g.off[(t * 5 + 5) * g.nlev];
  for (int k = b0 + threadIdx.x; k < b1; k += blockDim.x) {
    const int ij = g.pts[k];
    const int row = ij / g.n8, col = ij - row * g.n8;
    const int ik = (row - 4) * g.nni + (col - 4);
    J.rhs_buf[ik] = M(M(J.psa[ij], J.psb[ij]), g.g[ik]);
  }
}

// ----------------------------------------------------------------------
// Persistent cooperative MCSOR kernel: all jobs x tiles, 5 colour phases
// per micro-sweep, grid barrier between phases.
// ----------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads) k_mcsor_f64(GridDev g, const __grid_constant__ JobTable jobs, int njobs,
                                                        int nsweeps, BarrierDev bar, unsigned nblocks) {
  const int nitems = njobs * g.ntiles;
  for (int s = 0; s < nsweeps; ++s) {
    for (int c = 0; c < 5; ++c) {
      for (int item = blockIdx.x; item < nitems; item += gridDim.x) {
        const int jb = item / g.ntiles, t = item - jb * g.ntiles;
        const JobDev &J = jobs.j[jb];
        double *u = J.u;
        if (c == 0) {
          if (s == 0) {
            tile_ghosts(g, u, t, J.isym);
            if (J.kind == 1) tile_rhs(g, J, t);  // kind 2: explicit rhs
          } else {
            tile_boundary<double>(g, u, t, J.isym);
          }
          __syncthreads();
        }
        const double omega = J.omega, omega1 = 1.0 - J.omega;  // omega1 = 1 - omega (relaxOrbs.F90:83)
        const double *bt = (J.kind >= 1) ? g.bpot_mu : g.borb_mu;
        const double *rhsv = (J.kind == 1) ? J.rhs_buf : J.rhs;
        for (int l = 0; l < g.nlev; ++l) {
          const int o = (t * 5 + c) * g.nlev + l;
          const int b0 = g.off[o], b1 = g.off[o + 1];
          if (b0 == b1) continue;
          for (int k = b0 + threadIdx.x; k < b1; k += blockDim.x) {
            const int ij = g.pts[k];
            const int row = ij / g.n8, col = ij - row * g.n8;
            const int mu = row - 4, nu = col - 4, ik = mu * g.nni + nu;
            double lhs;
            if (J.kind == 1)
              lhs = (J.idel2 == 0.0) ? g.f3_mu[mu] : A(g.f3_mu[mu], M(J.idel2, g.e[ik]));
            else
              lhs = J.lhs[ik];
            relax_f64(u, ij, g, bt[mu], g.d_nu[nu], lhs, rhsv[ik], omega, omega1);
          }
          __syncthreads();
        }
      }
      if (!(s == nsweeps - 1 && c == 4)) {
        if (!grid_barrier(bar, nblocks)) return;
      }
    }
  }
  for (int item = blockIdx.x; item < nitems; item += gridDim.x) {
    const int jb = item / g.ntiles, t = item - jb * g.ntiles;
    tile_boundary<double>(g, jobs.j[jb].u, t, jobs.j[jb].isym);
    __syncthreads();
  }
}

// ----------------------------------------------------------------------
// List-order SOR (sormcsor.F90:20-132) as a pipelined wavefront over all
// jobs of the launch: step t updates, for every sweep s still running, the
// interior points of SOR level t - s * delta and the axis points whose
// extrapolation after sweep s belongs to that level (the host schedule,
// build_sor_schedule, proves these updates independent and every read
// value current), then all blocks meet at the grid barrier.  Reference
// arithmetic order (relax_f64); a potential's rhs = psa psb g and lhs = f3
// (+ idel^2 e) are formed per point with the same roundings as
// relaxPots.F90:81-95.  Ghost cells are refreshed once before the first
// sweep (putin) and stay fixed, as in the reference.
// ----------------------------------------------------------------------
__device__ __forceinline__ void sor_point(const GridDev &g, const JobDev &J, int rc) {
  const int row = rc >> 16, col = rc & 0xffff, ij = row * g.n8 + col;
  const int mu = row - 4, nu = col - 4, ik = mu * g.nni + nu;
  double lhs, rhs;
  if (J.kind == 1) {
    lhs = (J.idel2 == 0.0) ? g.f3_mu[mu] : A(g.f3_mu[mu], M(J.idel2, g.e[ik]));
    rhs = M(M(ldcg(J.psa + ij), ldcg(J.psb + ij)), g.g[ik]);
  } else {
    lhs = J.lhs[ik];
    rhs = J.rhs[ik];
  }
  const double *bt = (J.kind >= 1) ? g.bpot_mu : g.borb_mu;
  relax_f64(J.u, ij, g, bt[mu], g.d_nu[nu], lhs, rhs, J.omega, 1.0 - J.omega);
}

__device__ __forceinline__ void sor_axis(const GridDev &g, const JobDev &J, int rc) {
  const int row = rc >> 16, col = rc & 0xffff, ij = row * g.n8 + col;
  // the mu=1 row extrapolates along mu, the nu=1 / nu=nni columns along nu
  const int st = (col == 4) ? 1 : (col == g.nni + 3) ? -1 : g.n8;
  double *u = J.u;
  double v = 0.0;
  if (J.isym == 1)
    v = A(A(A(A(M(g.exeven[0], ldcg(u + ij + st)), M(g.exeven[1], ldcg(u + ij + 2 * st))),
              M(g.exeven[2], ldcg(u + ij + 3 * st))),
            M(g.exeven[3], ldcg(u + ij + 4 * st))),
          M(g.exeven[4], ldcg(u + ij + 5 * st)));
  u[ij] = v;
}

__global__ void __launch_bounds__(kThreads) k_sor_f64(GridDev g, const __grid_constant__ JobTable jobs, int njobs,
                                                      int nsweeps, BarrierDev bar, unsigned nblocks) {
  for (int item = blockIdx.x; item < njobs * g.ntiles; item += gridDim.x) {
    const int jb = item / g.ntiles;
    tile_ghosts(g, jobs.j[jb].u, item - jb * g.ntiles, jobs.j[jb].isym);
  }
  if (!grid_barrier(bar, nblocks)) return;
  const int D = g.sor_delta, NL = g.sor_nlev, NB = g.sor_nblev;
  const int T = (nsweeps - 1) * D + (NL > NB ? NL : NB);
  const int gt = int(blockIdx.x * blockDim.x + threadIdx.x), gs = int(gridDim.x * blockDim.x);
  for (int t = 0; t < T; ++t) {
    // the (sweep, level) pairs of this step as one index space over all jobs
    for (int s = 0; s < nsweeps; ++s) {
      const int l = t - s * D;
      if (l < 0) break;
      if (l < NL) {
        const int b0 = g.sor_off[l], n = g.sor_off[l + 1] - b0;
        for (int k = gt; k < n * njobs; k += gs) {
          const int jb = k / n;
          sor_point(g, jobs.j[jb], g.sor_pts[b0 + k - jb * n]);
        }
      }
      if (l < NB) {
        const int b0 = g.sor_boff[l], n = g.sor_boff[l + 1] - b0;
        for (int k = gt; k < n * njobs; k += gs) {
          const int jb = k / n;
          sor_axis(g, jobs.j[jb], g.sor_bpts[b0 + k - jb * n]);
        }
      }
    }
    if (t + 1 < T && !grid_barrier(bar, nblocks)) return;
  }
}

// double -> float with round to nearest even, on the integer pipes (GB300
// issues conversion instructions on its narrow FP64 pipe); values beyond the
// float range become infinities, values below its normal range signed zero
__device__ __forceinline__ float narrow_f64(double x) {
  const unsigned hi = unsigned(__double2hiint(x)), lo = unsigned(__double2loint(x));
  const unsigned sign = hi & 0x80000000u;
  const int dex = int((hi >> 20) & 0x7ffu);
  if (dex == 0x7ff) return __uint_as_float(sign | 0x7f800000u | ((hi & 0xfffffu) ? 0x400000u : 0u));
  const int fex = dex - 896;
  if (fex >= 255) return __uint_as_float(sign | 0x7f800000u);
  if (fex <= 0) return __uint_as_float(sign);
  // 23 mantissa bits: 20 from hi, 3 from lo; the remaining 29 bits round
  unsigned bits = (unsigned(fex) << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29);
  const unsigned rest = lo & 0x1fffffffu;
  if (rest > 0x10000000u || (rest == 0x10000000u && (bits & 1u))) ++bits;  // may carry into the exponent
  return __uint_as_float(sign | bits);
}

// float -> double by bit manipulation on the integer pipes (GB300 issues
// conversion instructions on its narrow FP64 pipe); exact for normal floats,
// infinities and NaNs; float subnormals (|e| < 1.2e-38, far below any
// correction that matters) become signed zero
__device__ __forceinline__ double widen_f32(float f) {
  const unsigned b = __float_as_uint(f), ex = (b >> 23) & 0xffu, m = b & 0x7fffffu;
  const unsigned sign = b & 0x80000000u;
  if (ex == 0) return __hiloint2double(int(sign), 0);
  const unsigned dex = (ex == 0xffu) ? 0x7ffu : ex + 896u;
  return __hiloint2double(int(sign | (dex << 20) | (m >> 3)), int(m << 29));
}

// FP64 axis extrapolation of one point from its 5 neighbours at stride st
// (sormcsor.F90:94-129 order)
__device__ __forceinline__ double extrap64(const GridDev &g, const double *u, int ij, int st) {
  return A(A(A(A(M(g.exeven[0], u[ij + st]), M(g.exeven[1], u[ij + 2 * st])), M(g.exeven[2], u[ij + 3 * st])),
             M(g.exeven[3], u[ij + 4 * st])),
           M(g.exeven[4], u[ij + 5 * st]));
}

// Axis extrapolation of the correction (tile_boundary<float>) for tiles
// [t0, t1) computed in the band sb held in shared memory (indexed by ext
// index).
__device__ void band_boundary(const GridDev &g, float *sb, int t0, int t1, bool even) {
  const int n8 = g.n8, nni = g.nni;
  const int nrow7 = (t0 == 0) ? nni - 2 : 0;
  const int r0 = (t0 == 0) ? 5 : g.tile_row0[t0];
  const int nside = 2 * (g.tile_row1[t1 - 1] - r0);
  for (int k = threadIdx.x; k < nrow7 + nside; k += blockDim.x) {
    int ij, st;
    if (k < nrow7) {
      ij = 4 * n8 + 5 + k;
      st = n8;
    } else {
      const int q = k - nrow7, r = r0 + q / 2, side = q % 2;
      ij = r * n8 + (side == 0 ? 4 : nni + 3);
      st = (side == 0) ? 1 : -1;
    }
    float v = 0.0f;
    if (even)
      v = g.exevenf[0] * sb[ij + st] + g.exevenf[1] * sb[ij + 2 * st] + g.exevenf[2] * sb[ij + 3 * st] +
          g.exevenf[3] * sb[ij + 4 * st] + g.exevenf[4] * sb[ij + 5 * st];
    sb[ij] = v;
  }
  if (t0 == 0) {
    __syncthreads();
    if (threadIdx.x < 2) {
      const int ij = 4 * n8 + (threadIdx.x == 0 ? 4 : nni + 3);
      const int st = (threadIdx.x == 0) ? 1 : -1;
      float v = 0.0f;
      if (even)
        v = g.exevenf[0] * sb[ij + st] + g.exevenf[1] * sb[ij + 2 * st] + g.exevenf[2] * sb[ij + 3 * st] +
            g.exevenf[3] * sb[ij + 4 * st] + g.exevenf[4] * sb[ij + 5 * st];
      sb[ij] = v;
    }
  }
}

// Shared memory of the band of a run of G tiles with its 4-row halos, as
// whole 16-byte pieces.
__host__ __device__ inline size_t band_smem_bytes(const GridDev &g, int G) {
  return ((size_t(g.st_rows[G]) * g.n8 + 8) * sizeof(float) + 15) / 16 * 16;
}

// Persistent-band FP32 sweep for grids whose bands do not fit one cluster's
// shared memory.  Block b owns, for the whole launch, one run of G
// consecutive tiles of one job (rows [row0, row1)) and keeps the
// correction on those rows, with 4-row halos, in shared memory, as whole
// 16-byte pieces: piece f holds ext indices 4f..4f+3 at sband[4 (f - f0)].
// Every colour phase waits until the blocks within halo reach have
// finished the previous phase (wait_neighbours; this also means they are
// done reading this band's edge rows), refreshes the two halos from the
// correction in global memory (L2), updates the phase's points level by
// level in shared memory, writes to global memory only the new values
// within 4 rows of a band edge shared with another block (that block's
// halo), and publishes its finished phase count.  No grid-wide barrier.
// Same-colour
// stencil neighbours never lie in different tiles, so the values a phase
// changes in a neighbour's rows are never read by this block in that phase,
// and a halo piece that reaches into an own row covers only ghost columns
// (zero throughout).  The kernel ends with u += e and the FP64 axis values
// of u on the band's rows, so the correction never returns to global memory.
__global__ void __launch_bounds__(kBandThreads) k_mcsor_f32p(GridDev g, const __grid_constant__ JobTable jobs,
                                                               int nsweeps, int G, BarrierDev bar,
                                                               unsigned *phase) {
  extern __shared__ __align__(16) float sband[];
  const int nrun = (g.ntiles + G - 1) / G;
  const int jb = int(blockIdx.x) / nrun, t0 = (int(blockIdx.x) - jb * nrun) * G;
  const int t1 = (t0 + G < g.ntiles) ? t0 + G : g.ntiles;
  const JobDev &J = jobs.j[jb];
  float *e = J.e32;
  const int n8 = g.n8, nlev = g.nlev;
  const int row0 = g.tile_row0[t0], row1 = g.tile_row1[t1 - 1];
  const int f0 = ((row0 - 4) * n8) >> 2, f1 = ((row1 + 4) * n8 + 3) >> 2;
  const int fa = (row0 * n8 + 3) >> 2, fb = (row1 * n8) >> 2;  // top halo [f0, fa), bottom [fb, f1)
  const int edge_lo = (t0 > 0) ? row0 + 4 : row0, edge_hi = (t1 < g.ntiles) ? row1 - 4 : row1;
  const float4 *src = reinterpret_cast<const float4 *>(e);
  float4 *dst = reinterpret_cast<float4 *>(sband);
  float *sb = sband - 4 * f0;  // indexed by ext index
  // lanes 0..2 watch the runs above, 3..5 the runs below, whose rows reach
  // into this band's halos
  int nbq = -1;
  {
    const int lane = int(threadIdx.x), run = int(blockIdx.x) - jb * nrun;
    if (lane < 6) {
      const int q = (lane < 3) ? run - 1 - lane : run + 1 + (lane - 3);
      if (q >= 0 && q < nrun) {
        const int q0 = q * G, q1 = (q0 + G < g.ntiles) ? q0 + G : g.ntiles;
        const int r0q = g.tile_row0[q0], r1q = g.tile_row1[q1 - 1];
        if ((lane < 3 && r1q > row0 - 4) || (lane >= 3 && r0q < row1 + 4)) nbq = jb * nrun + q;
      }
    }
  }
  const float omega1 = J.omega1f;
  const float *bt = (J.kind >= 1) ? g.bpot_mu32 : g.borb_mu32;
  CoefF cf;
  for (int k = 0; k < 4; ++k) {
    cf.dmu1[k] = g.dmu1f[k];
    cf.dmu2[k] = g.dmu2f[k];
    cf.dni1[k] = g.dni1f[k];
    cf.dni2[k] = g.dni2f[k];
  }
  for (int f = f0 + int(threadIdx.x); f < f1; f += blockDim.x) dst[f - f0] = __ldcg(src + f);
  __syncthreads();
  unsigned done = 0;  // colour phases finished
  for (int s = 0; s < nsweeps; ++s) {
    for (int c = 0; c < 5; ++c) {
      if (s > 0 || c > 0) {
        if (!wait_neighbours(bar, phase, nbq, done)) return;
        for (int f = f0 + int(threadIdx.x); f < fa; f += blockDim.x) dst[f - f0] = __ldcg(src + f);
        for (int f = fb + int(threadIdx.x); f < f1; f += blockDim.x) dst[f - f0] = __ldcg(src + f);
        if (c == 0) {
          __syncthreads();
          band_boundary(g, sb, t0, t1, J.isym == 1);
        }
        __syncthreads();
      }
#pragma unroll 1
      for (int l = 0; l < nlev; ++l) {
        const int *so = g.st_off + (c * nlev + l) * (g.ntiles + 1);
        const int b0 = so[t0], b1 = so[t1];
        if (b0 == b1) continue;
        // four points per thread and pass, their list entries loaded
        // together (points of one colour and level are independent)
        for (int k0 = b0 + int(threadIdx.x); k0 < b1; k0 += 4 * int(blockDim.x)) {
          int rc[4];
          float2 p[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const int k = k0 + u * int(blockDim.x);
            if (k < b1) {
              rc[u] = __ldg(g.st_pts + k);
              p[u] = __ldg(J.rw + k);
            }
          }
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            if (k0 + u * int(blockDim.x) < b1) {
              const int row = rc[u] >> 16, col = rc[u] & 0xffff, ij = row * n8 + col;
              const float v =
                  relax_f32(sb, ij, n8, cf, bt[row - 4], g.d_nu32[col - 4], p[u].y, p[u].x, omega1);
              sb[ij] = v;
              if (row < edge_lo || row >= edge_hi) e[ij] = v;
            }
          }
        }
        __syncthreads();
      }
      // publish the finished phase (the level loop ended with a block barrier)
      ++done;
      if (threadIdx.x == 0) {
        __threadfence();
        st_release(phase + size_t(blockIdx.x) * kPhaseStride, done);
      }
    }
  }
  // u += e on the band's interior rows, then the FP64 axis values of u on
  // the band's rows (sormcsor.F90:94-129; the axis points read only the
  // band's own rows)
  double *u = J.u;
  const int ra = (row0 > 5) ? row0 : 5, ncol = g.nni - 2, total = (row1 - ra) * ncol;
  for (int k0 = threadIdx.x; k0 < total; k0 += 8 * int(blockDim.x)) {
    // eight loads of u in flight per thread before the adds
    int ij[8];
    double uv[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int k = k0 + q * int(blockDim.x);
      ij[q] = -1;
      if (k < total) {
        ij[q] = (ra + k / ncol) * n8 + 5 + k % ncol;
        uv[q] = __ldcg(u + ij[q]);
      }
    }
#pragma unroll
    for (int q = 0; q < 8; ++q)
      if (ij[q] >= 0) u[ij[q]] = uv[q] + widen_f32(sb[ij[q]]);
  }
  __syncthreads();
  const bool even = (J.isym == 1);
  const int nrow7 = (t0 == 0) ? g.nni - 2 : 0, nside = 2 * (row1 - ra);
  for (int k = threadIdx.x; k < nrow7 + nside; k += blockDim.x) {
    if (k < nrow7) {
      const int ij = 4 * n8 + 5 + k;
      u[ij] = even ? extrap64(g, u, ij, n8) : 0.0;
    } else {
      const int q = k - nrow7, r = ra + q / 2, side = q % 2;
      const int ij = r * n8 + (side == 0 ? 4 : g.nni + 3);
      u[ij] = even ? extrap64(g, u, ij, side == 0 ? 1 : -1) : 0.0;
    }
  }
  if (t0 == 0) {
    __syncthreads();
    if (threadIdx.x < 2) {
      const int ij = 4 * n8 + (threadIdx.x == 0 ? 4 : g.nni + 3);
      u[ij] = even ? extrap64(g, u, ij, threadIdx.x == 0 ? 1 : -1) : 0.0;
    }
  }
}

// ----------------------------------------------------------------------
// On-chip FP32 correction sweep of the mixed form: one relaxation job per
// thread-block cluster.  CTA k of the cluster keeps ext rows
// [cl_row0[k]-4, cl_row0[k+1]+4) of the correction e in shared memory for
// all micro-sweeps, together with the band's residual, omega/lhs, the
// coefficient rows and its point list; after updating a point within 4 rows
// of its band edge it also stores the value into the neighbouring CTA's halo
// through distributed shared memory, and the colour phases are separated by
// the cluster's hardware barrier.  Ends with u += e (FP64) on the band's
// interior points and the FP64 axis re-extrapolation of u.
// ----------------------------------------------------------------------
constexpr int kClusterMaxThreads = 768;  // 24 warps: interior + edge + seam roles

__device__ __forceinline__ float ex5f(const float *ex, const float *p, int s) {
  return ex[0] * p[s] + ex[1] * p[2 * s] + ex[2] * p[3 * s] + ex[3] * p[4 * s] + ex[4] * p[5 * s];
}

// axis extrapolation of e in shared memory for the CTA's rows
__device__ void smem_boundary(const GridDev &g, float *E, int R0, int R1, int rank, bool even, const float *ex) {
  const int n8 = g.n8, nni = g.nni;
  const int nrow7 = (rank == 0) ? nni - 2 : 0;
  const int r0 = (rank == 0) ? 5 : R0;
  const int nside = 2 * (R1 - r0);
  for (int k = threadIdx.x; k < nrow7 + nside; k += blockDim.x) {
    if (k < nrow7) {
      float *p = E + (4 - R0 + 4) * n8 + 5 + k;
      *p = even ? ex5f(ex, p, n8) : 0.0f;
    } else {
      const int q = k - nrow7, r = r0 + q / 2, side = q % 2;
      float *p = E + (r - R0 + 4) * n8 + (side == 0 ? 4 : nni + 3);
      *p = even ? ex5f(ex, p, side == 0 ? 1 : -1) : 0.0f;
    }
  }
  __syncthreads();
  if (rank == 0 && threadIdx.x < 2) {
    float *p = E + (4 - R0 + 4) * n8 + (threadIdx.x == 0 ? 4 : nni + 3);
    *p = even ? ex5f(ex, p, threadIdx.x == 0 ? 1 : -1) : 0.0f;
  }
}

// dynamic shared memory of k_mixed_cluster: (residual, omega/lhs) pairs of
// the band's points, correction band with 4-row halos, b(mu) of the band's
// rows, d(nu) by ext column, the CTA's segment offsets, then its chunk list.
// k_mixed_cluster_pot (potentials, lhs = f3(mu) + idel^2 (e_mu(mu) -
// e_nu(nu))) keeps the residual alone and the lhs as a row term of the
// band's rows and a column term by ext column, after d(nu).
// free: the seam-free colouring's plan (one level, cf_*), else the
// reference colouring's (cl_*)
size_t cluster_smem_bytes(const GridDev &g, bool sep, bool free) {
  const size_t band = size_t(g.cl_maxrows) * g.n8 * sizeof(float);
  const int S = (free ? 1 : g.nlev) + 2, chunks = free ? g.cf_maxchunks : g.cl_maxchunks;
  return (sep ? band : 2 * band) + size_t(g.cl_maxrows + 8) * g.n8 * sizeof(float) +
         size_t(g.cl_maxrows + g.n8) * sizeof(float) * (sep ? 2 : 1) + size_t(5 * S + 1) * sizeof(int) +
         size_t(chunks) * sizeof(int);
}


// split cluster barrier: arrive releases this thread's earlier shared and
// distributed-shared writes, wait acquires every CTA's released writes
__device__ __forceinline__ void cluster_arrive() { asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory"); }
__device__ __forceinline__ void cluster_wait() { asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory"); }

// (row, col) of the points k, k+T, k+2T, ... of a band's interior listed
// row by row from (ra, 5) with ncols columns per row, advanced without
// division
struct BandWalk {
  int row, col, step_r, step_c, col_end, ncols;
  __device__ BandWalk(int k, int T, int ra, int nc) : ncols(nc) {
    row = ra + k / nc;
    col = 5 + k % nc;
    step_r = T / nc;
    step_c = T % nc;
    col_end = 5 + nc;
  }
  __device__ __forceinline__ void next() {
    row += step_r;
    col += step_c;
    if (col >= col_end) {
      col -= ncols;
      ++row;
    }
  }
};

struct ClusterBand {
  float *E;               // correction rows [R0-4, R1+4) of the band
  const float2 *RW;       // (residual, omega/lhs) by band row * n8 + col
  const float *R;         // potentials' variant: residual by band row * n8 + col
  const float *BT, *DN;   // b(mu) by band row, d(nu) by ext column
  const float *LP, *LQ;   // potentials' variant: lhs = LP[band row] - LQ[ext column]
  const unsigned *PL;     // chunks (band row << 19) | (col << 2) | (count-1)
  float *up, *dn;         // neighbours' halos addressed like E, or null
  int n8, hdn;            // band rows >= hdn feed the lower neighbour
  float omega, omega1;
  CoefF cf;
};

// One chunk: up to 4 same-colour points of one band row at columns col,
// col+5, col+10, col+15.  The row values col-4..col+19 are read once (a
// point's left neighbours are the previous point's right ones); every read
// precedes every write.  Positions past the chunk's count are computed but
// not stored: their reads stay inside the CTA's shared allocation (at most
// 10 elements past the correction band, the pairs, the residual, d(nu) or
// the lhs column term, each followed by a larger array).  kSep: omega / lhs
// from the row and column terms (fast reciprocal: the correction sweep is
// the inner solver of the FP64 defect correction, whose fixed point does
// not depend on it).
template <bool halo, bool kSep>
__device__ __forceinline__ void cluster_chunk(const ClusterBand &B, unsigned q) {
  const int n8 = B.n8;
  const int lr = int(q >> 19), col = int((q >> 2) & 0x1ffffu), n = int(q & 3u) + 1;
  const int ls = lr * n8 + col;
  float *const p = B.E + ls + 4 * n8;
  const CoefF &cf = B.cf;
  float rv[24];
#pragma unroll
  for (int i = 0; i < 24; ++i) rv[i] = p[i - 4];
  const float b = B.BT[lr];
  float out[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const float *pj = p + 5 * j;
    const float m4 = pj[-4 * n8], p4 = pj[4 * n8], m3 = pj[-3 * n8], p3 = pj[3 * n8];
    const float m2 = pj[-2 * n8], p2 = pj[2 * n8], m1 = pj[-n8], p1 = pj[n8];
    const float l4 = rv[5 * j], l3 = rv[5 * j + 1], l2 = rv[5 * j + 2], l1 = rv[5 * j + 3], ec = rv[5 * j + 4];
    const float r1 = rv[5 * j + 5], r2 = rv[5 * j + 6], r3 = rv[5 * j + 7], r4 = rv[5 * j + 8];
    float2 rw;
    if (kSep)
      rw = make_float2(B.R[ls + 5 * j], __fdividef(B.omega, B.LP[lr] - B.LQ[col + 5 * j]));
    else
      rw = B.RW[ls + 5 * j];
    const float d = B.DN[col + 5 * j];
    float dm2 = cf.dmu2[0] * (m4 + p4);
    dm2 = __fmaf_rn(cf.dmu2[1], m3 + p3, dm2);
    dm2 = __fmaf_rn(cf.dmu2[2], m2 + p2, dm2);
    dm2 = __fmaf_rn(cf.dmu2[3], m1 + p1, dm2);
    float dm1 = cf.dmu1[0] * (m4 - p4);
    dm1 = __fmaf_rn(cf.dmu1[1], m3 - p3, dm1);
    dm1 = __fmaf_rn(cf.dmu1[2], m2 - p2, dm1);
    dm1 = __fmaf_rn(cf.dmu1[3], m1 - p1, dm1);
    float dn2 = cf.dni2[0] * (l4 + r4);
    dn2 = __fmaf_rn(cf.dni2[1], l3 + r3, dn2);
    dn2 = __fmaf_rn(cf.dni2[2], l2 + r2, dn2);
    dn2 = __fmaf_rn(cf.dni2[3], l1 + r1, dn2);
    float dn1 = cf.dni1[0] * (l4 - r4);
    dn1 = __fmaf_rn(cf.dni1[1], l3 - r3, dn1);
    dn1 = __fmaf_rn(cf.dni1[2], l2 - r2, dn1);
    dn1 = __fmaf_rn(cf.dni1[3], l1 - r1, dn1);
    const float cc = __fmaf_rn(d, dn1, __fmaf_rn(b, dm1, dm2) + dn2);
    out[j] = __fmaf_rn(B.omega1, ec, rw.y * (rw.x - cc));
  }
#pragma unroll
  for (int j = 0; j < 4; ++j)
    if (j < n) p[5 * j] = out[j];
  if (halo) {
    if (B.up && lr < 4) {
#pragma unroll
      for (int j = 0; j < 4; ++j)
        if (j < n) B.up[ls + 4 * n8 + 5 * j] = out[j];
    }
    if (B.dn && lr >= B.hdn) {
#pragma unroll
      for (int j = 0; j < 4; ++j)
        if (j < n) B.dn[ls + 4 * n8 + 5 * j] = out[j];
    }
  }
}

// update chunks [b0, b1) of the CTA's list (their points are independent),
// thread t of the n threads of a warp role taking chunks t, t+n, ...
template <bool halo, bool kSep>
__device__ __forceinline__ void cluster_chunks(const ClusterBand &B, int b0, int b1, int t, int n) {
  for (int k = b0 + t; k < b1; k += n) cluster_chunk<halo, kSep>(B, B.PL[k]);
}

// barrier among the seam warps only (named barrier 1)
__device__ __forceinline__ void seam_barrier(int nthreads) {
  asm volatile("bar.sync 1, %0;" ::"r"(nthreads) : "memory");
}

template <bool kSep>
__device__ __forceinline__ void mixed_cluster_body(const GridDev &g, const JobTable &jobs, int nsweeps, int free) {
  namespace cg = cooperative_groups;
  cg::cluster_group cl = cg::this_cluster();
  const int C = int(cl.num_blocks()), rank = int(cl.block_rank());
  const JobDev &J = jobs.j[blockIdx.x / C];
  const float *const r32 = J.r32, *const w32 = J.w32;
  const bool even = (J.isym == 1);
  const float *const bt = (J.kind >= 1) ? g.bpot_mu32 : g.borb_mu32;
  extern __shared__ float2 smem2[];
  const int n8 = g.n8, nni = g.nni, nlev = free ? 1 : g.nlev, S = nlev + 2;
  const int R0 = g.cl_row0[rank], R1 = g.cl_row0[rank + 1];
  const int nloc = (g.cl_maxrows + 8) * n8;
  const int *const plan_off = free ? g.cf_off : g.cl_off, *const plan_pts = free ? g.cf_pts : g.cl_pts;
  float2 *const RW = smem2;
  float *const RR = reinterpret_cast<float *>(smem2);
  float *const E = kSep ? RR + g.cl_maxrows * n8 : reinterpret_cast<float *>(RW + g.cl_maxrows * n8);
  float *const BT = E + nloc;
  float *const DN = BT + g.cl_maxrows;
  float *const LP = DN + n8;                   // kSep only
  float *const LQ = LP + g.cl_maxrows;         // kSep only
  int *const SO = reinterpret_cast<int *>(kSep ? LQ + n8 : DN + n8);  // segment offsets into PL
  unsigned *const PL = reinterpret_cast<unsigned *>(SO + 5 * S + 1);
  const int *const coff = plan_off + size_t(rank) * 5 * S;
  const int pbase = coff[0], npl = coff[5 * S] - pbase;
  for (int k = threadIdx.x; k <= 5 * S; k += blockDim.x) SO[k] = coff[k] - pbase;
  for (int k = threadIdx.x; k < nloc; k += blockDim.x) E[k] = 0.0f;
  for (int k = threadIdx.x; k < R1 - R0; k += blockDim.x) BT[k] = bt[R0 + k - 4];
  for (int k = threadIdx.x; k < n8; k += blockDim.x) DN[k] = (k >= 4 && k < nni + 4) ? g.d_nu32[k - 4] : 0.0f;
  if (kSep) {
    // lhs = f3 + idel^2 e with e = e_mu - e_nu: the row term in FP64, then
    // both terms in FP32 (the nu axis columns, never updated, get 0)
    for (int k = threadIdx.x; k < R1 - R0; k += blockDim.x) {
      const int mu = R0 + k - 4;
      LP[k] = narrow_f64(fma(J.idel2, g.e_mu[mu], g.f3_mu[mu]));
    }
    for (int k = threadIdx.x; k < n8; k += blockDim.x)
      LQ[k] = (k >= 4 && k < nni + 4) ? narrow_f64(J.idel2 * g.e_nu[k - 4]) : 0.0f;
  }
  for (int k = threadIdx.x; k < npl; k += blockDim.x) PL[k] = unsigned(plan_pts[pbase + k]);
  const int ra = (R0 < 5) ? 5 : R0, ncols = nni - 2, nband = (R1 - ra) * ncols;
  {
    // four points per thread in flight: all loads before the stores
    BandWalk w(threadIdx.x, blockDim.x, ra, ncols);
    for (int k = threadIdx.x; k < nband; k += 4 * blockDim.x) {
      float rv[4], wv[4];
      int ls[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        ls[j] = -1;
        if (k + j * int(blockDim.x) < nband) {
          const int ik = (w.row - 4) * nni + (w.col - 4);
          ls[j] = (w.row - R0) * n8 + w.col;
          rv[j] = r32[ik];
          if (!kSep) wv[j] = w32[ik];
        }
        w.next();
      }
#pragma unroll
      for (int j = 0; j < 4; ++j)
        if (ls[j] >= 0) {
          if (kSep)
            RR[ls[j]] = rv[j];
          else
            RW[ls[j]] = make_float2(rv[j], wv[j]);
        }
    }
  }
  ClusterBand B;
  B.E = E;
  B.RW = RW;
  B.R = RR;
  B.BT = BT;
  B.DN = DN;
  B.LP = LP;
  B.LQ = LQ;
  B.PL = PL;
  B.n8 = n8;
  B.hdn = R1 - R0 - 4;
  B.omega = J.omegaf;
  B.omega1 = J.omega1f;
  for (int k = 0; k < 4; ++k) {
    B.cf.dmu1[k] = g.dmu1f[k];
    B.cf.dmu2[k] = g.dmu2f[k];
    B.cf.dni1[k] = g.dni1f[k];
    B.cf.dni2[k] = g.dni2f[k];
  }
  float ex[5];
  for (int k = 0; k < 5; ++k) ex[k] = g.exevenf[k];
  // neighbours' halo rows, addressed by this CTA's band offsets
  B.up = (rank > 0) ? cl.map_shared_rank(E, rank - 1) + (R0 - g.cl_row0[rank - 1]) * n8 : nullptr;
  B.dn = (rank < C - 1) ? cl.map_shared_rank(E, rank + 1) + (R0 - R1) * n8 : nullptr;
  // warp roles: interior, edge, seam
  const int wa = free ? (kSep ? g.cf_pa : g.cf_wa) : (kSep ? g.cl_pa : g.cl_wa);
  const int wb = free ? (kSep ? g.cf_pb : g.cf_wb) : (kSep ? g.cl_pb : g.cl_wb);
  const int ws = free ? (kSep ? g.cf_ps : g.cf_ws) : (kSep ? g.cl_ps : g.cl_ws);
  const int warp = threadIdx.x >> 5;
  const int role = (warp < wa) ? 0 : (warp < wa + wb) ? 1 : 2;
  const int rbase = (role == 0) ? 0 : (role == 1) ? wa : wa + wb;
  const int rt = threadIdx.x - 32 * rbase;
  const int rn = 32 * ((role == 0) ? wa : (role == 1) ? wb : ws);
  __syncthreads();
  cluster_arrive();  // this band is zeroed: neighbours may push into its halos
  for (int s = 0; s < nsweeps; ++s) {
    for (int c = 0; c < 5; ++c) {
      if (c == 0 && s > 0) {
        smem_boundary(g, E, R0, R1, rank, even, ex);
        __syncthreads();
      }
      const int *o = SO + c * S;
      // After the cluster wait the halos hold the neighbours' previous
      // colour, and the neighbours no longer read the halo values this colour
      // overwrites.  Interior points need only this CTA's values; seam points
      // go level by level among the seam warps.
      if (role == 0) {
        cluster_chunks<false, kSep>(B, o[0], o[1], rt, rn);
        cluster_wait();
      } else if (role == 1) {
        cluster_wait();
        cluster_chunks<true, kSep>(B, o[1], o[2], rt, rn);
      } else {
        cluster_wait();
        cluster_chunks<true, kSep>(B, o[2], o[3], rt, rn);
        for (int l = 1; l < nlev; ++l) {
          if (o[2 + l] == o[3 + l]) continue;
          seam_barrier(rn);
          cluster_chunks<true, kSep>(B, o[2 + l], o[3 + l], rt, rn);
        }
      }
      __syncthreads();
      cluster_arrive();
    }
  }
  cluster_wait();  // no CTA leaves while a neighbour may still write its halo
  // u += e on the band's interior points, then the FP64 axis of u for the
  // band's rows (the mu=1 row and corners by the first CTA, whose band holds
  // rows 4..9)
  double *const u = J.u;
  {
    BandWalk w(threadIdx.x, blockDim.x, ra, ncols);
    for (int k = threadIdx.x; k < nband; k += 4 * blockDim.x) {
      double uv[4];
      int ij[4], le[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        ij[j] = -1;
        if (k + j * int(blockDim.x) < nband) {
          ij[j] = w.row * n8 + w.col;
          le[j] = (w.row - R0 + 4) * n8 + w.col;
          uv[j] = u[ij[j]];
        }
        w.next();
      }
#pragma unroll
      for (int j = 0; j < 4; ++j)
        if (ij[j] >= 0) u[ij[j]] = uv[j] + widen_f32(E[le[j]]);
    }
  }
  __syncthreads();
  const int nrow7 = (rank == 0) ? nni - 2 : 0, nside = 2 * (R1 - ra);
  for (int k = threadIdx.x; k < nrow7 + nside; k += blockDim.x) {
    if (k < nrow7) {
      const int ij = 4 * n8 + 5 + k;
      u[ij] = even ? extrap64(g, u, ij, n8) : 0.0;
    } else {
      const int q = k - nrow7, r = ra + q / 2, side = q % 2;
      const int ij = r * n8 + (side == 0 ? 4 : nni + 3);
      u[ij] = even ? extrap64(g, u, ij, side == 0 ? 1 : -1) : 0.0;
    }
  }
  __syncthreads();
  if (rank == 0 && threadIdx.x < 2) {
    const int ij = 4 * n8 + (threadIdx.x == 0 ? 4 : nni + 3);
    u[ij] = even ? extrap64(g, u, ij, threadIdx.x == 0 ? 1 : -1) : 0.0;
  }
}

__global__ void __launch_bounds__(kClusterMaxThreads, 1) k_mixed_cluster(GridDev g, const __grid_constant__ JobTable jobs,
                                                                        int nsweeps, int free) {
  mixed_cluster_body<false>(g, jobs, nsweeps, free);
}

// Potentials only (job kind 1): two CTAs per SM, so that twice the clusters
// are co-resident for the batches of an SCF iteration's potentials; at most
// kWarps warps per CTA (kPotWarpsRef for the reference colouring,
// kPotWarpsFree for the seam-free one)
template <int kWarps>
__global__ void __launch_bounds__(32 * kWarps, 2) k_mixed_cluster_pot(GridDev g, const __grid_constant__ JobTable jobs,
                                                                     int nsweeps, int free) {
  mixed_cluster_body<true>(g, jobs, nsweeps, free);
}

// the potentials' variant for a colouring
static const void *pot_kernel(bool free) {
  return free ? (const void *)k_mixed_cluster_pot<kPotWarpsFree> : (const void *)k_mixed_cluster_pot<kPotWarpsRef>;
}

// ----------------------------------------------------------------------
// Mixed form: ghost refresh, FP64 residual, FP32 correction, FP64 update.
// ----------------------------------------------------------------------
__device__ __forceinline__ void ghost_point(const GridDev &g, double *u, int k, int isym) {
  // k indexes (rows 4..nmu+3) x 8 ghost columns, then 4 ghost rows x nni
  const int nrows = g.nmu;
  const bool neg = (isym != 1);
  if (k < nrows * 8) {
    const int r = 4 + k / 8, q = k % 8, base = r * g.n8;
    if (q < 4) {
      const int j = q + 1;
      const double v = u[base + 4 + j];
      u[base + 4 - j] = neg ? -v : v;
    } else {
      const int j = q - 3;
      const double v = u[base + g.nni + 3 - j];
      u[base + g.nni + 3 + j] = neg ? -v : v;
    }
  } else {
    k -= nrows * 8;
    const int i = k / g.nni + 1, col = 4 + k % g.nni;
    const double v = u[(4 + i) * g.n8 + col];
    u[(4 - i) * g.n8 + col] = neg ? -v : v;
  }
}

// u at ext (row, col) with the putin ghost cells (inout.F90:47-80) read as
// the mirrored interior value, negated for odd functions (a sign-bit flip);
// the corner ghosts, never filled by putin, are not reachable by the cross
// stencil
__device__ __forceinline__ double ghost_read(const GridDev &g, const double *u, int row, int col, int isym) {
  bool m = false;
  if (col < 4) {
    col = 8 - col;
    m = true;
  } else if (col > g.nni + 3) {
    col = 2 * g.nni + 6 - col;
    m = true;
  }
  if (row < 4) {
    row = 8 - row;
    m = true;
  }
  const double v = u[row * g.n8 + col];
  return (m && isym != 1) ? __longlong_as_double(__double_as_longlong(v) ^ (1ll << 63)) : v;
}

// Mixed form residual r = rhs - A u in FP64 over the interior, stored as
// FP32 with omega / lhs; the stencil uses the grid's separable weights (one
// FMA per neighbour) and reads the ghost cells as mirrored interior values,
// so u needs no ghost refresh first.  kPacked: the points are taken in
// st_pts order and stored as (r, w) pairs in that order (persistent-band
// sweep);
// otherwise r32 / w32 are plain nni x nmu arrays (cluster sweep; need_w 0:
// the potentials' cluster sweep forms omega / lhs itself, only r32 is
// stored).
template <bool kPacked>
__global__ void k_residual(GridDev g, const __grid_constant__ JobTable jobs, int zero_e, int need_w) {
  const JobDev &J = jobs.j[blockIdx.y];
  const int nint = (g.nni - 2) * (g.nmu - 5);
  const int n8 = g.n8;
  if (zero_e)
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < g.next; k += gridDim.x * blockDim.x) J.e32[k] = 0.0f;
  const double *cmu = (J.kind == 0) ? g.cmu_orb : g.cmu_pot;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nint; k += gridDim.x * blockDim.x) {
    int mu, nu;
    if (kPacked) {
      const int rc = g.st_pts[k];
      mu = (rc >> 16) - 4;
      nu = (rc & 0xffff) - 4;
    } else {
      mu = 1 + k / (g.nni - 2);
      nu = 1 + k % (g.nni - 2);
    }
    const int ik = mu * g.nni + nu, ij = (mu + 4) * n8 + nu + 4;
    const double *u = J.u;
    double rhs, lhs;
    if (J.kind == 1) {
      rhs = (J.psa[ij] * J.psb[ij]) * g.g[ik];
      lhs = (J.idel2 == 0.0) ? g.f3_mu[mu] : fma(J.idel2, g.e[ik], g.f3_mu[mu]);
    } else {
      rhs = J.rhs[ik];
      lhs = J.lhs[ik];
    }
    const double *cm = cmu + mu * 8, *cn = g.cnu + nu * 8;
    double cc = lhs * u[ij];
    if (mu >= 4 && nu >= 4 && nu <= g.nni - 5) {
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int dm = (4 - q) * n8, dn = 4 - q;
        cc = fma(cm[q], u[ij - dm], cc);
        cc = fma(cm[4 + q], u[ij + dm], cc);
        cc = fma(cn[q], u[ij - dn], cc);
        cc = fma(cn[4 + q], u[ij + dn], cc);
      }
    } else {
      // the stencil reaches the putin ghosts: read them as mirrored interior
      // values
      const int row = mu + 4, col = nu + 4;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int d = 4 - q;
        cc = fma(cm[q], ghost_read(g, u, row - d, col, J.isym), cc);
        cc = fma(cm[4 + q], u[ij + d * n8], cc);
        cc = fma(cn[q], ghost_read(g, u, row, col - d, J.isym), cc);
        cc = fma(cn[4 + q], ghost_read(g, u, row, col + d, J.isym), cc);
      }
    }
    if (kPacked) {
      J.rw[k] = make_float2(narrow_f64(rhs - cc), J.omegaf / narrow_f64(lhs));
    } else {
      J.r32[ik] = narrow_f64(rhs - cc);
      if (need_w) J.w32[ik] = J.omegaf / narrow_f64(lhs);
    }
  }
}


// ----------------------------------------------------------------------
// Elementwise kernels of the SCF path
// ----------------------------------------------------------------------
__global__ void k_ghost(GridDev g, double *u, int isym) {
  const int n = g.nmu * 8 + 4 * g.nni;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) ghost_point(g, u, k, isym);
}

__global__ void k_putin_interior(GridDev g, const double *plain, double *ext) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < g.mxsize; k += gridDim.x * blockDim.x) {
    const int mu = k / g.nni, nu = k - mu * g.nni;
    ext[(mu + 4) * g.n8 + nu + 4] = plain[k];
  }
}

__global__ void k_putout(GridDev g, const double *ext, double *plain) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < g.mxsize; k += gridDim.x * blockDim.x) {
    const int mu = k / g.nni, nu = k - mu * g.nni;
    plain[k] = ext[(mu + 4) * g.n8 + nu + 4];
  }
}

// fockHF (src/fock.F90:57-186), per grid point: exact keeps the reference's
// unfused order, otherwise (mixed form) products are fused into FMAs.
template <bool exact>
__device__ __forceinline__ double madd(double a, double b, double c) {  // a*b + c
  if (exact) return A(M(a, b), c);
  return fma(a, b, c);
}

template <bool exact>
__device__ __forceinline__ void fock_point(const GridDev &g, const FockArgs &a, double ee, int k) {
  const int mu = k / g.nni, nu = k - mu * g.nni;
  const int ij = (mu + 4) * g.n8 + nu + 4;
  double fock1 = g.f0[k];
  fock1 = madd<exact>(ee, g.f1[k], fock1);
  if (a.m != 0) fock1 = madd<exact>(double(a.m * a.m), g.e[k], fock1);
  double fock2 = 0.0;
  if (!a.nel1) {
    double wk1 = 0.0;
    for (int q = 0; q < a.nterms; ++q) {
      const FockTerm &T = a.t[q];
      wk1 = madd<exact>(T.coo, T.coul[ij], wk1);
      if (T.mode == 0) {
        double wk2 = M(T.gec, T.ex[ij]);
        if (T.ex2) wk2 = madd<exact>(T.gec2, T.ex2[ij], wk2);
        fock2 = madd<exact>(wk2, T.psi[ij], fock2);
      } else if (T.mode == 1) {
        const double wk2 = M(T.ex[ij], T.psi[ij]);
        fock2 = madd<exact>(T.gec, wk2, fock2);
      }
    }
    a.coulp[k] = wk1;
    a.exchp[k] = fock2;
    fock2 = M(fock2, g.f2[k]);
    fock1 = madd<exact>(wk1, g.f2[k], fock1);
  }
  a.lhs[k] = A(fock1, g.diag);
  a.rhs[k] = fock2;
  if (mu >= g.nmu - 5) {
    const double f1 = g.f1[k];
    a.fa[(mu - (g.nmu - 5)) * g.nni + nu] = (fabs(f1) <= kPrecis) ? 0.0 : D(fock1, f1);
  }
}

template <bool exact>
__global__ void k_fock(GridDev g, FockArgs a) {
  const double ee = *a.ee;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < g.mxsize; k += gridDim.x * blockDim.x)
    fock_point<exact>(g, a, ee, k);
}

// the Fock builds of several orbitals from the same state, orbital blockIdx.y
constexpr int kFockBatch = 8;
struct FockBatch {
  FockArgs a[kFockBatch];
};
template <bool exact>
__global__ void k_fock_batch(GridDev g, const __grid_constant__ FockBatch B) {
  const FockArgs &a = B.a[blockIdx.y];
  const double ee = *a.ee;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < g.mxsize; k += gridDim.x * blockDim.x)
    fock_point<exact>(g, a, ee, k);
}

// orbAsymptGet (relaxOrbs.F90:415-437): edecay for mu = nmu-4..nmu-1 (0-based)
__global__ void k_asympt_get(GridDev g, const double *fa, double *edecay) {
  const int n = 4 * g.nni;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const int jj = k / g.nni, i = k - jj * g.nni;
    const int j = g.nmu - 4 + jj;  // 0-based mu
    (void)j;
    // raiq1 - raiq from the grid's table; x**0.25 as sqrt(sqrt(x))
    const double dr = g.asy[size_t(50) * n + k];
    const double fj = fa[(jj + 1) * g.nni + i], fjm = fa[jj * g.nni + i];
    edecay[k] = sqrt(sqrt(fabs(fj / fjm))) * exp(sqrt(fabs(fjm)) * dr);
  }
}

// orbAsymptSet (relaxOrbs.F90:444-462), rows in order
__global__ void k_asympt_set(GridDev g, double *psi, const double *edecay) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < g.nni; i += gridDim.x * blockDim.x) {
    for (int jj = 0; jj < 4; ++jj) {
      const int j = g.nmu - 4 + jj;
      const int ij = (j + 4) * g.n8 + i + 4;
      psi[ij] = M(psi[ij - g.n8], edecay[jj * g.nni + i]);
    }
  }
}

// orbAsymptGet / orbAsymptSet of several orbitals, orbital blockIdx.y
__global__ void k_asympt_get_batch(GridDev g, const __grid_constant__ OrbDecayList L) {
  const int n = 4 * g.nni, o = blockIdx.y;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const int jj = k / g.nni, i = k - jj * g.nni;
    const double dr = g.asy[size_t(50) * n + k];
    const double fj = L.fa[o][(jj + 1) * g.nni + i], fjm = L.fa[o][jj * g.nni + i];
    L.edecay[o][k] = sqrt(sqrt(fabs(fj / fjm))) * exp(sqrt(fabs(fjm)) * dr);
  }
}
__global__ void k_asympt_set_batch(GridDev g, const __grid_constant__ OrbDecayList L) {
  const int o = blockIdx.y;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < g.nni; i += gridDim.x * blockDim.x)
    for (int jj = 0; jj < 4; ++jj) {
      const int j = g.nmu - 4 + jj;
      const int ij = (j + 4) * g.n8 + i + 4;
      L.psi[o][ij] = M(L.psi[o][ij - g.n8], L.edecay[o][jj * g.nni + i]);
    }
}

// setCiOrb (scfUtils.F90:380-434)
__global__ void k_setci(GridDev g, double *psi, int ihomo) {
  const int n2 = g.nni / 2 + 1;
  const int n = (n2 - 1) * g.nmu;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const int mu = k / (n2 - 1), ni = k - mu * (n2 - 1);  // ni 0-based = reference ni-1
    const int row = (mu + 4) * g.n8 + 4;
    const double v = psi[row + ni];
    psi[row + (g.nni - 1 - ni)] = (ihomo == 1) ? v : -v;
  }
  if (ihomo != 1) {
    for (int mu = blockIdx.x * blockDim.x + threadIdx.x; mu < g.nmu; mu += gridDim.x * blockDim.x)
      psi[(mu + 4) * g.n8 + 4 + (n2 - 1)] = 0.0;
  }
}

// norm scaling: psi = (1/sqrt(xnorm)) psi over the plain region (normOrtho.F90:50-52)
__global__ void k_scale(GridDev g, double *psi, const double *xnorm) {
  const double zarea = D(1.0, sqrt(*xnorm));
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < g.mxsize; k += gridDim.x * blockDim.x) {
    const int mu = k / g.nni, nu = k - mu * g.nni;
    const int ij = (mu + 4) * g.n8 + nu + 4;
    psi[ij] = M(zarea, psi[ij]);
  }
}

// norm scaling followed by setCiOrb (normOrtho.F90:50-52, scfUtils.F90:380-
// 434) in one pass: the left half of each row is scaled and mirrored, the
// middle column scaled (gerade) or zeroed (ungerade)
__global__ void k_scale_setci(GridDev g, double *psi, const double *xnorm, int ihomo) {
  const double zarea = D(1.0, sqrt(*xnorm));
  const int n2 = g.nni / 2 + 1;
  const int n = n2 * g.nmu;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const int mu = k / n2, ni = k - mu * n2;
    const int row = (mu + 4) * g.n8 + 4;
    if (ni < n2 - 1) {
      const double v = M(zarea, psi[row + ni]);
      psi[row + ni] = v;
      psi[row + (g.nni - 1 - ni)] = (ihomo == 1) ? v : -v;
    } else {
      psi[row + ni] = (ihomo == 1) ? M(zarea, psi[row + ni]) : 0.0;
    }
  }
}

struct PtrList {
  const double *p[kMaxTerms];
};

// Gram-Schmidt step of ortho (normOrtho.F90:175-188)
__global__ void k_ortho_apply(GridDev g, double *psi, PtrList others, int n, const double *ovl) {
  double ano = 0.0;
  for (int q = 0; q < n; ++q) ano = A(ano, M(ovl[q], ovl[q]));
  ano = D(sqrt(A(1.0, ano)), S(1.0, M(ano, ano)));
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < g.mxsize; k += gridDim.x * blockDim.x) {
    const int mu = k / g.nni, nu = k - mu * g.nni;
    const int ij = (mu + 4) * g.n8 + nu + 4;
    double v = psi[ij];
    for (int q = 0; q < n; ++q) v = A(M(-ovl[q], others.p[q][ij]), v);
    psi[ij] = M(ano, v);
  }
}

// vexch/mulex normalised associated Legendre functions P_k^q(cos th) for
// k = 1..mpole (scfUtils.F90:856-1270).  legacy_m3 reproduces vexch's m=3
// branch, which uses sin^2 in place of sin.
__device__ void assoc_legendre(int mt, int mpole, double costh, double *dome, bool legacy_m3) {
  for (int k = 0; k < 10; ++k) dome[k] = 0.0;
  if (mt > 4) return;
  double c2, c4, c6, c8, si, si2, si3;
  if (mt == 0) {
    dome[1] = costh;
    dome[2] = (3.0 * costh * costh - 1.0) * 0.50;
    for (int n = 2; n <= mpole - 1; n++)
      dome[n + 1] = (double(2 * n + 1) * costh * dome[n] - double(n) * dome[n - 1]) / double(n + 1);
  } else if (mt == 1) {
    c2 = costh * costh;
    si2 = fabs(1.0 - c2);
    si = sqrt(si2);
    c4 = c2 * c2;
    c6 = c4 * c2;
    dome[1] = -si / sqrt(2.0);
    dome[2] = -3.0 * si * costh / sqrt(6.0);
    dome[3] = (3.0 / 2.0) * si * (1.0 - 5.0 * c2) / sqrt(12.0);
    dome[4] = (5.0 / 2.0) * si * costh * (3.0 - 7.0 * c2) / sqrt(20.0);
    dome[5] = (15.0 / 8.0) * si * (-1.0 + 14.0 * c2 - 21.0 * c4) / sqrt(30.0);
    dome[6] = (21.0 / 8.0) * si * costh * (-5.0 + 30.0 * c2 - 33.0 * c4) / sqrt(42.0);
    dome[7] = (7.0 / 16.0) * si * (5.0 - 135.0 * c2 + 495.0 * c4 - 429.0 * c6) / sqrt(56.0);
    dome[8] = (9.0 / 16.0) * si * costh * (35.0 - 385.0 * c2 + 1001.0 * c4 - 715.0 * c6) / sqrt(72.0);
  } else if (mt == 2) {
    c2 = costh * costh;
    si2 = fabs(1.0 - c2);
    c4 = c2 * c2;
    c6 = c4 * c2;
    c8 = c6 * c2;
    dome[2] = 3.0 * si2 / sqrt(24.0);
    dome[3] = 15.0 * costh * si2 / sqrt(120.0);
    dome[4] = (15.0 / 2.0) * (-1.0 + 8.0 * c2 - 7.0 * c4) / sqrt(360.0);
    dome[5] = (105.0 / 2.0) * costh * (-1.0 + 4.0 * c2 - 3.0 * c4) / sqrt(840.0);
    dome[6] = (105.0 / 8.0) * (1.0 - 19.0 * c2 + 51.0 * c4 - 33.0 * c6) / sqrt(1680.0);
    dome[7] = (63.0 / 8.0) * costh * (15.0 - 125.0 * c2 + 253.0 * c4 - 143.0 * c6) / sqrt(3024.0);
    dome[8] = (315.0 / 8.0) * (-1.0 + 34.0 * c2 - 176.0 * c4 + 286.0 * c6 - 143.0 * c8) / sqrt(5040.0);
  } else if (mt == 3) {
    c2 = costh * costh;
    si2 = fabs(1.0 - c2);
    si = legacy_m3 ? si2 : sqrt(si2);
    si3 = si2 * si;
    c4 = c2 * c2;
    dome[3] = -15.0 * si3 / sqrt(720.0);
    dome[4] = -105.0 * si3 * costh / sqrt(5040.0);
    dome[5] = -(105.0 / 2.0) * si3 * (-1.0 + 9.0 * c2) / sqrt(20160.0);
    dome[6] = -(315.0 / 2.0) * si3 * costh * (-3.0 + 11.0 * c2) / sqrt(60480.0);
    dome[7] = -(315.0 / 8.0) * si3 * (3.0 - 66.0 * c2 + 143.0 * c4) / sqrt(151200.0);
    dome[8] = -(3465.0 / 8.0) * si3 * costh * (3.0 - 26.0 * c2 + 39.0 * c4) / sqrt(332640.0);
  } else if (mt == 4) {
    c2 = costh * costh;
    c4 = c2 * c2;
    c6 = c4 * c2;
    c8 = c6 * c2;
    dome[4] = 105.0 * (1.0 - 2.0 * c2 + c4) / sqrt(40320.0);
    dome[5] = 945.0 * costh * (1.0 - 2.0 * c2 + c4) / sqrt(362880.0);
    dome[6] = (945.0 / 2.0) * (-1.0 + 13 * c2 - 23.0 * c4 + 11.0 * c6) / sqrt(1814400.0);
    dome[7] = (3465.0 / 2.0) * costh * (-3.0 + 19 * c2 - 29.0 * c4 + 13.0 * c6) / sqrt(6652800.0);
    dome[8] = (10395.0 / 8.0) * (1.0 - 28.0 * c2 + 118.0 * c4 - 156.0 * c6 + 65.0 * c8) / sqrt(19958400.0);
  }
  for (int k = mpole + 1; k <= 8; ++k) dome[k] = 0.0;
}

// Moment tables of a grid: exchange moment weights over the plain grid and
// the boundary functions of potAsympt on mu = nmu-4..nmu-1 (0-based),
// evaluated once per grid with the formulas of coulAsympt/vcoul,
// exchAsympt/vexch and exchMom (scfUtils.F90:615-1270).
__global__ void k_moment_tables(GridDev g, double *exm, double *asy) {
  const int stride = gridDim.x * blockDim.x;
  double dome[10];
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < g.mxsize; k += stride) {
    const int mu = k / g.nni, nu = k - mu * g.nni;
    const double rr = sqrt(g.vxisq[mu] + g.vetasq[nu] - 1.0);
    const double xrr = g.r2 * rr;
    const double costh = (fabs(rr) > kPrecis) ? g.veta[nu] * g.vxi[mu] / rr : 0.0;
    const double wk = g.wgt2[k] * g.f4[k];
    for (int idel = 0; idel <= 4; ++idel) {
      assoc_legendre(idel, g.mpole, costh, dome, false);
      double xw = xrr;
      for (int q = 0; q < g.mpole; ++q) {
        if (q > 0) xw = xw * xrr;
        exm[(size_t(idel) * 8 + q) * g.mxsize + k] = wk * (dome[q + 1] * xw);
      }
    }
  }
  const int P = 4 * g.nni;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < P; p += stride) {
    const int jj = p / g.nni, i = p - jj * g.nni, j = g.nmu - 4 + jj;
    const double rr = sqrt(g.vxisq[j] + g.vetasq[i] - 1.0);
    asy[p] = g.r2 * g.vxi[j];
    asy[size_t(50) * P + p] = sqrt(g.vxisq[j - 1] + g.vetasq[i] - 1.0) - rr;  // orbAsymptGet's raiq1 - raiq
    const double rr1 = 1.0 / (rr * g.r2);
    asy[P + p] = rr1;
    const double costh = g.veta[i] * g.vxi[j] / rr;
    dome[1] = costh;
    dome[2] = (3.0 * costh * costh - 1.0) * 0.5;
    for (int m = 2; m <= g.mpole - 1; m++)
      dome[m + 1] = (double(2 * m + 1) * costh * dome[m] - double(m) * dome[m - 1]) / double(m + 1);
    double rp = rr1;
    for (int m = 1; m <= 8; m++) {
      rp = rp * rr1;
      asy[size_t(2 + m - 1) * P + p] = (m <= g.mpole) ? dome[m] * rp : 0.0;
    }
    const double costx = (fabs(rr) > kPrecis) ? costh : 0.0;
    const double rs = rr * g.r2;
    for (int idel = 0; idel <= 4; ++idel) {
      assoc_legendre(idel, g.mpole, costx, dome, true);  // vexch's m=3 branch
      double xrn = rs;
      for (int m = 1; m <= 8; m++) {
        xrn = xrn * rs;
        asy[size_t(10 + idel * 8 + m - 1) * P + p] = (m <= g.mpole) ? dome[m] / xrn : 0.0;
      }
    }
  }
}

// potAsympt: Coulomb (coulAsympt/vcoul) and exchange (exchAsympt/vexch)
// boundary values on mu = nmu-4..nmu-1 (0-based) from the grid's tables.
__global__ void k_asympt(GridDev g, AsymptArgs a) {
  const AsymptItem &it = a.it[blockIdx.y];
  const int P = 4 * g.nni;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < P; p += gridDim.x * blockDim.x) {
    const int jj = p / g.nni, i = p - jj * g.nni;
    const int ij = (g.nmu + jj) * g.n8 + i + 4;
    double pe = 0.0;
    if (it.type == 0) {
      const double *cm = a.cmulti + it.idx * 8;
      for (int m = 1; m <= g.mpole; m++) pe = fma(cm[m - 1], g.asy[size_t(1 + m) * P + p], pe);
      pe = g.asy[P + p] + pe;
    } else if (it.idel <= 4) {
      const double *xm = a.excm + it.idx * 8;
      const double *X = g.asy + size_t(10 + it.idel * 8) * P + p;
      for (int m = 1; m <= g.mpole; m++) pe = fma(X[size_t(m - 1) * P], xm[m - 1], pe);
    }
    it.pot[ij] = g.asy[p] * pe;
  }
}

__global__ void k_zero(double *p, size_t n) {
  for (size_t k = blockIdx.x * size_t(blockDim.x) + threadIdx.x; k < n; k += size_t(gridDim.x) * blockDim.x) p[k] = 0.0;
}

// ----------------------------------------------------------------------
// Deterministic reductions: fixed grid -> per-block partials -> the last
// block to finish sums the partials in block order.
// ----------------------------------------------------------------------
constexpr int kRedBlocks = 160, kRedBlocksMax = 608;
// blocks of a single-launch reduction over the grid: 160 up to ~160k
// points, one per 1024 points above that (more loads in flight on large
// grids), at most 608; fixed per grid, so every sum runs in the same order
// on every call
inline int red_blocks(const GridDev &g) {
  const int b = g.mxsize / 1024;
  return b < kRedBlocks ? kRedBlocks : (b > kRedBlocksMax ? kRedBlocksMax : b);
}
constexpr int kMaxK = 16;

template <int K>
__device__ void block_sum_store(double (&v)[K], double *partials) {
  __shared__ double sh[kThreads / 32][K];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < K; ++q) {
    double x = v[q];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) sh[w][q] = x;
  }
  __syncthreads();
  if (threadIdx.x < K) {
    double s = 0.0;
    for (int i = 0; i < kThreads / 32; ++i) s += sh[i][threadIdx.x];
    partials[blockIdx.x * K + threadIdx.x] = s;
  }
}

// Every block stores its K partial sums; the block that finishes last (an
// atomic ticket, reset by that block) sums the partials of all blocks in
// block order -- the same order on every run -- and
// writes out[0..nout).  Returns true in that block.  No block waits for
// another.
// Sum of partial q of nblocks blocks' stores (K per block), in block order:
// thread t adds blocks t, t + blockDim, ..., then a warp tree, then the warp
// totals in warp order.  Every thread of the block gets the total.
__device__ double sum_partials(const double *partials, int K, int q, int nblocks) {
  __shared__ double sh[kThreads / 32];
  __shared__ double tot;
  double s = 0.0;
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x) s += __ldcg(partials + size_t(b) * K + q);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int i = 0; i < kThreads / 32; ++i) t += sh[i];
    tot = t;
  }
  __syncthreads();
  const double r = tot;
  __syncthreads();
  return r;
}

// sum_partials of nq <= kMaxK slots at once, slot q of block b at
// base[b * bstride + q * qstride]: the same sums in the same order, with one
// pass over the partials and two block barriers for all of them; out[] in
// shared memory, valid in every thread on return
__device__ void sum_partials_multi(const double *base, int bstride, int qstride, int nq, int nblocks, double *out) {
  __shared__ double sh[kThreads / 32][kMaxK];
  double s[kMaxK];
#pragma unroll
  for (int q = 0; q < kMaxK; ++q) s[q] = 0.0;
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
#pragma unroll
    for (int q = 0; q < kMaxK; ++q)
      if (q < nq) s[q] += __ldcg(base + size_t(b) * bstride + size_t(q) * qstride);
  }
#pragma unroll
  for (int q = 0; q < kMaxK; ++q) {
    if (q >= nq) break;
    double x = s[q];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5][q] = x;
  }
  __syncthreads();
  if (threadIdx.x < nq) {
    double t = 0.0;
    for (int i = 0; i < kThreads / 32; ++i) t += sh[i][threadIdx.x];
    out[threadIdx.x] = t;
  }
  __syncthreads();
}

template <int K>
__device__ bool block_sum_finish(double (&v)[K], double *partials, double *out, int nout, unsigned *ticket) {
  __shared__ bool s_last;
  block_sum_store<K>(v, partials);
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = (atomicAdd(ticket, 1u) == gridDim.x - 1);
  __syncthreads();
  if (!s_last) return false;
  __threadfence();
  for (int q = 0; q < nout; ++q) {
    const double t = sum_partials(partials, K, q, int(gridDim.x));
    if (threadIdx.x == 0) out[q] = t;
  }
  if (threadIdx.x == 0) *ticket = 0u;
  return true;
}

__global__ void k_norm(GridDev g, const double *psi, double *partials, double *out, unsigned *ticket) {
  double v[1] = {0.0};
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < g.mxsize; k += gridDim.x * blockDim.x) {
    const int mu = k / g.nni, nu = k - mu * g.nni;
    const double p = psi[(mu + 4) * g.n8 + nu + 4];
    v[0] += g.wgt2[k] * M(M(p, p), g.f4[k]);
  }
  block_sum_finish<1>(v, partials, out, 1, ticket);
}

__global__ void k_overlaps(GridDev g, const double *psi, PtrList o, int n, double *partials, double *out,
                           unsigned *ticket) {
  double v[kMaxK];
  for (int q = 0; q < kMaxK; ++q) v[q] = 0.0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < g.mxsize; k += gridDim.x * blockDim.x) {
    const int mu = k / g.nni, nu = k - mu * g.nni;
    const int ij = (mu + 4) * g.n8 + nu + 4;
    const double p = psi[ij], w = g.wgt2[k], f4 = g.f4[k];
    for (int q = 0; q < n; ++q) v[q] += w * M(M(p, o.p[q][ij]), f4);
  }
  block_sum_finish<kMaxK>(v, partials, out, n, ticket);
}

// One round of the orthonormalisation of several orbitals (normOrtho.F90:
// 14-59, 103-207, scfUtils.F90:380-434): orbital blockIdx.y of the round's
// list.  Each orbital's sums run over the same blocks in the same order as
// k_norm / k_overlaps, so the results equal the one-orbital launches.
constexpr int kRoundItems = 12;
struct OrthoItem {
  double *psi;
  const double *o[kMaxK];  // orthogonalisation partners (normalised earlier)
  int n;                   // number of partners
  int ihomo;               // 0: scale only; +-1: scale and setCiOrb
  double *norm_out;        // sum wgt2 psi psi f4
  double *ovl_out;         // overlaps with the partners
};
struct OrthoRound {
  OrthoItem it[kRoundItems];
};

__global__ void k_norm_round(GridDev g, const __grid_constant__ OrthoRound R, double *partials, unsigned *tickets) {
  const OrthoItem &I = R.it[blockIdx.y];
  double v[1] = {0.0};
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < g.mxsize; k += gridDim.x * blockDim.x) {
    const int mu = k / g.nni, nu = k - mu * g.nni;
    const double p = I.psi[(mu + 4) * g.n8 + nu + 4];
    v[0] += g.wgt2[k] * M(M(p, p), g.f4[k]);
  }
  block_sum_finish<1>(v, partials + size_t(blockIdx.y) * gridDim.x, I.norm_out, 1, tickets + blockIdx.y);
}

__global__ void k_scale_round(GridDev g, const __grid_constant__ OrthoRound R) {
  const OrthoItem &I = R.it[blockIdx.y];
  const double zarea = D(1.0, sqrt(*I.norm_out));
  if (I.ihomo == 0) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < g.mxsize; k += gridDim.x * blockDim.x) {
      const int mu = k / g.nni, nu = k - mu * g.nni;
      const int ij = (mu + 4) * g.n8 + nu + 4;
      I.psi[ij] = M(zarea, I.psi[ij]);
    }
    return;
  }
  const int n2 = g.nni / 2 + 1;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n2 * g.nmu; k += gridDim.x * blockDim.x) {
    const int mu = k / n2, ni = k - mu * n2;
    const int row = (mu + 4) * g.n8 + 4;
    if (ni < n2 - 1) {
      const double v = M(zarea, I.psi[row + ni]);
      I.psi[row + ni] = v;
      I.psi[row + (g.nni - 1 - ni)] = (I.ihomo == 1) ? v : -v;
    } else {
      I.psi[row + ni] = (I.ihomo == 1) ? M(zarea, I.psi[row + ni]) : 0.0;
    }
  }
}

__global__ void k_overlaps_round(GridDev g, const __grid_constant__ OrthoRound R, double *partials,
                                 unsigned *tickets) {
  const OrthoItem &I = R.it[blockIdx.y];
  double v[kMaxK];
  for (int q = 0; q < kMaxK; ++q) v[q] = 0.0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < g.mxsize; k += gridDim.x * blockDim.x) {
    const int mu = k / g.nni, nu = k - mu * g.nni;
    const int ij = (mu + 4) * g.n8 + nu + 4;
    const double p = I.psi[ij], w = g.wgt2[k], f4 = g.f4[k];
    for (int q = 0; q < I.n; ++q) v[q] += w * M(M(p, I.o[q][ij]), f4);
  }
  block_sum_finish<kMaxK>(v, partials + size_t(blockIdx.y) * gridDim.x * kMaxK, I.ovl_out, I.n,
                          tickets + blockIdx.y);
}

__global__ void k_ortho_round(GridDev g, const __grid_constant__ OrthoRound R) {
  const OrthoItem &I = R.it[blockIdx.y];
  const double *ovl = I.ovl_out;
  double ano = 0.0;
  for (int q = 0; q < I.n; ++q) ano = A(ano, M(ovl[q], ovl[q]));
  ano = D(sqrt(A(1.0, ano)), S(1.0, M(ano, ano)));
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < g.mxsize; k += gridDim.x * blockDim.x) {
    const int mu = k / g.nni, nu = k - mu * g.nni;
    const int ij = (mu + 4) * g.n8 + nu + 4;
    double v = I.psi[ij];
    for (int q = 0; q < I.n; ++q) v = A(M(-ovl[q], I.o[q][ij]), v);
    I.psi[ij] = M(ano, v);
  }
}

// Every round of an iteration's orthonormalisation in one cooperative
// launch: the norms and scalings (and setCiOrb) of every orbital, then per
// round the overlaps with the partners and the Gram-Schmidt step of each of
// its orbitals, separated by grid barriers.  Each block stores the same per-block partial
// sums as k_norm_round / k_overlaps_round (same blocks, same points, same
// order) and every block adds them up in the order of block_sum_finish, so
// the results equal the per-round launches bit for bit.
constexpr int kOrthoItems = 32, kOrthoRounds = 16;
struct OrthoPlan {
  OrthoItem it[kOrthoItems];
  int round_off[kOrthoRounds + 1];
  int nrounds;
};

// The phases below take up to kGroup orbitals (or orbital-partner pairs) of
// a round in one pass over the points, so that their loads are in flight
// together; each orbital's (pair's) per-thread sum still runs over the same
// points in the same order, and block_sum_store reduces every slot the same
// way whatever the number of slots stored, so the sums are those of the
// one-orbital kernels.
constexpr int kGroup = 8;

// scaling (and setCiOrb) of items [a, b) of the plan with zarea[j]
__device__ void scale_items(const GridDev &g, const OrthoPlan &P, int a, int b, const double *zarea) {
  const int stride = gridDim.x * blockDim.x, n2 = g.nni / 2 + 1;
  const int homo = P.it[a].ihomo != 0;  // one kind per call (the caller groups them)
  const int n = homo ? n2 * g.nmu : g.mxsize;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride) {
#pragma unroll
    for (int j = 0; j < kGroup; ++j) {
      if (a + j >= b) break;
      const OrthoItem &I = P.it[a + j];
      if (!homo) {
        const int mu = k / g.nni, nu = k - mu * g.nni;
        const int ij = (mu + 4) * g.n8 + nu + 4;
        I.psi[ij] = M(zarea[j], I.psi[ij]);
      } else {
        const int mu = k / n2, ni = k - mu * n2;
        const int row = (mu + 4) * g.n8 + 4;
        if (ni < n2 - 1) {
          const double v = M(zarea[j], I.psi[row + ni]);
          I.psi[row + ni] = v;
          I.psi[row + (g.nni - 1 - ni)] = (I.ihomo == 1) ? v : -v;
        } else {
          I.psi[row + ni] = (I.ihomo == 1) ? M(zarea[j], I.psi[row + ni]) : 0.0;
        }
      }
    }
  }
}

__global__ void __launch_bounds__(kThreads) k_orthonormalise(GridDev g, const __grid_constant__ OrthoPlan P,
                                                             double *partials, BarrierDev bar) {
  __shared__ double s_val[kGroup * kMaxK];
  __shared__ int s_item[kMaxK], s_q[kMaxK];
  const int nb = int(gridDim.x);
  // An orbital is changed only in its own round, after its partners'
  // rounds: its norm and scaling read nothing another round writes, so the
  // norms and scalings of every round run first, in one pass, and the rounds
  // keep only their overlaps and Gram-Schmidt steps.
  const int n = P.round_off[P.nrounds];
  for (int a = 0; a < n; a += kGroup) {
    double v[kGroup];
#pragma unroll
    for (int j = 0; j < kGroup; ++j) v[j] = 0.0;
#pragma unroll 4
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < g.mxsize; k += gridDim.x * blockDim.x) {
      const int mu = k / g.nni, nu = k - mu * g.nni;
      const int ij = (mu + 4) * g.n8 + nu + 4;
      const double w2 = g.wgt2[k], f4 = g.f4[k];
#pragma unroll
      for (int j = 0; j < kGroup; ++j) {
        if (a + j >= n) break;
        const double p = P.it[a + j].psi[ij];
        v[j] += w2 * M(M(p, p), f4);
      }
    }
#pragma unroll
    for (int j = 0; j < kGroup; ++j) {
      if (a + j >= n) break;
      double w[1] = {v[j]};
      block_sum_store<1>(w, partials + size_t(a + j) * nb);
      __syncthreads();
    }
  }
  __threadfence();
  if (!grid_barrier(bar, unsigned(nb))) return;
  // totals (every block, in block order), then the scaling, grouped by kind
  for (int a = 0; a < n;) {
    int b = a;
    while (b < n && b - a < kGroup && (P.it[b].ihomo != 0) == (P.it[a].ihomo != 0)) ++b;
    double zarea[kGroup];
    sum_partials_multi(partials + size_t(a) * nb, 1, nb, b - a, nb, s_val);
    for (int j = 0; j < b - a; ++j) {
      const double norm = s_val[j];
      if (blockIdx.x == 0 && threadIdx.x == 0) *P.it[a + j].norm_out = norm;
      zarea[j] = D(1.0, sqrt(norm));
    }
    __syncthreads();  // s_val is reused below
    scale_items(g, P, a, b, zarea);
    a = b;
  }
  for (int r = 0; r < P.nrounds; ++r) {
    const int i0 = P.round_off[r], i1 = P.round_off[r + 1];
    bool partners = false;
    for (int i = i0; i < i1; ++i) partners = partners || P.it[i].n > 0;
    if (!partners) continue;
    // the scalings and the earlier rounds' Gram-Schmidt steps done
    // everywhere before this round's overlaps
    __threadfence();
    if (!grid_barrier(bar, unsigned(nb))) return;
    // overlaps: (item, partner) slots of the round, kMaxK at a time; values
    // other blocks wrote in this launch are read through L2
    int slot0 = 0;
    for (int i = i0; i < i1;) {
      // a slot group: at most kGroup items and kMaxK (item, partner) slots
      int nslot = 0, iend = i;
      while (iend < i1 && iend - i < kGroup && nslot + P.it[iend].n <= kMaxK) nslot += P.it[iend++].n;
      if (iend == i) break;  // an item alone has at most kMaxK partners
      if (threadIdx.x == 0) {
        int t = 0;
        for (int x = i; x < iend; ++x)
          for (int q = 0; q < P.it[x].n; ++q, ++t) {
            s_item[t] = x;
            s_q[t] = q;
          }
      }
      __syncthreads();
      double v[kMaxK];
#pragma unroll
      for (int t = 0; t < kMaxK; ++t) v[t] = 0.0;
      for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < g.mxsize; k += gridDim.x * blockDim.x) {
        const int mu = k / g.nni, nu = k - mu * g.nni;
        const int ij = (mu + 4) * g.n8 + nu + 4;
        const double w = g.wgt2[k], f4 = g.f4[k];
#pragma unroll
        for (int t = 0; t < kMaxK; ++t) {
          if (t >= nslot) break;
          const OrthoItem &I = P.it[s_item[t]];
          const double p = __ldcg(I.psi + ij);
          v[t] += w * M(M(p, __ldcg(I.o[s_q[t]] + ij)), f4);
        }
      }
      block_sum_store<kMaxK>(v, partials + size_t(slot0) * nb);
      __syncthreads();
      slot0 += kMaxK;
      i = iend;
    }
    __threadfence();
    if (!grid_barrier(bar, unsigned(nb))) return;
    // totals, then the Gram-Schmidt step of up to kGroup items at a time
    slot0 = 0;
    for (int i = i0; i < i1;) {
      int nslot = 0, iend = i;
      while (iend < i1 && iend - i < kGroup && nslot + P.it[iend].n <= kMaxK) nslot += P.it[iend++].n;
      if (iend == i) break;
      {
        __shared__ double tot[kMaxK];
        sum_partials_multi(partials + size_t(slot0) * nb, kMaxK, 1, nslot, nb, tot);
        if (threadIdx.x == 0)
          for (int x = i, t = 0; x < iend; ++x)
            for (int q = 0; q < P.it[x].n; ++q, ++t) {
              s_val[(x - i) * kMaxK + q] = tot[t];
              if (blockIdx.x == 0) P.it[x].ovl_out[q] = tot[t];
            }
      }
      __syncthreads();
      {
        const int a = i, b = iend;
        double ano[kGroup];
        for (int j = 0; j < b - a; ++j) {
          const OrthoItem &I = P.it[a + j];
          const double *ovl = s_val + j * kMaxK;
          double x = 0.0;
          for (int q = 0; q < I.n; ++q) x = A(x, M(ovl[q], ovl[q]));
          ano[j] = D(sqrt(A(1.0, x)), S(1.0, M(x, x)));
        }
        for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < g.mxsize; k += gridDim.x * blockDim.x) {
          const int mu = k / g.nni, nu = k - mu * g.nni;
          const int ij = (mu + 4) * g.n8 + nu + 4;
#pragma unroll
          for (int j = 0; j < kGroup; ++j) {
            if (a + j >= b) break;
            const OrthoItem &I = P.it[a + j];
            if (I.n == 0) continue;
            const double *ovl = s_val + j * kMaxK;
            double v = __ldcg(I.psi + ij);
            for (int q = 0; q < I.n; ++q) v = A(M(-ovl[q], __ldcg(I.o[q] + ij)), v);
            I.psi[ij] = M(ano[j], v);
          }
        }
      }
      __syncthreads();
      slot0 += kMaxK;
      i = iend;
    }
  }
}

// The same orthonormalisation through the inner products of the orbitals
// (one pass over the points, one grid barrier, one pass applying the
// result).  With Z_j the orbital after setCiOrb (homonuclear: the first half
// of each row mirrored onto the second, the sign by g/u) and <a,b> = sum
// wgt2 f4 a b, the loop "scale orbital j by 1/sqrt(<X_j,X_j>) (then setCiOrb),
// then Gram-Schmidt against its partners Y_q" (normOrtho.F90:14-59,
// 103-207) makes every final orbital a combination Y_j = sum_m C_jm Z_m of
// the orbitals of its symmetry block, and the loop's overlaps are
//   ovl_q = zarea_j sum_m C_qm <Z_j, Z_m>,
// so C, the norms and the overlaps follow exactly from the Gram matrix, in
// the reference's orbital order.  Equal to the loop in exact arithmetic; the
// rounding differs (the loop's sums of the scaled, partly orthogonalised
// orbitals become sums of products of inner products).
constexpr int kGramOrbs = 16, kGramSlots = 64;
struct GramPlan {
  double *psi[kGramOrbs];
  double *norm_out[kGramOrbs], *ovl_out[kGramOrbs];
  int ihomo[kGramOrbs];               // 0 heteronuclear; +-1 setCiOrb parity
  int npart[kGramOrbs];
  signed char part[kGramOrbs][kGramOrbs];  // partners (plan indices, earlier in the order)
  signed char slot_of[kGramOrbs][kGramOrbs];  // slot of <Z_a, Z_b> (a != b), of <X_a, X_a> (a == b)
  signed char sa[kGramSlots], sb[kGramSlots];
  int n, nslots, homo;
};

__global__ void __launch_bounds__(kThreads) k_orthonormalise_gram(GridDev g, const __grid_constant__ GramPlan P,
                                                                  double *partials, BarrierDev bar) {
  __shared__ double s_h[kGramSlots];
  __shared__ double s_z[kGramOrbs];
  __shared__ double s_c[kGramOrbs][kGramOrbs];
  const int nb = int(gridDim.x), n = P.n, n2 = g.nni / 2 + 1;
  // inner products, kMaxK slots per pass; the values are read where the
  // slot needs them (L1 serves the repeats), so nothing is indexed at run
  // time in registers
  for (int s0 = 0; s0 < P.nslots; s0 += kMaxK) {
    double v[kMaxK];
#pragma unroll
    for (int t = 0; t < kMaxK; ++t) v[t] = 0.0;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < g.mxsize; k += gridDim.x * blockDim.x) {
      const int mu = k / g.nni, nu = k - mu * g.nni;
      const int row = (mu + 4) * g.n8 + 4;
      // Z at this point: the orbital itself, or its mirrored first-half value
      int src = nu, middle = 0, second = 0;
      if (P.homo) {
        if (nu > n2 - 1) {
          src = g.nni - 1 - nu;
          second = 1;
        } else if (nu == n2 - 1) {
          middle = 1;
        }
      }
      const double w = g.wf[k];
#pragma unroll
      for (int t = 0; t < kMaxK; ++t) {
        if (s0 + t >= P.nslots) break;
        const int a = P.sa[s0 + t], b = P.sb[s0 + t];
        double pr;
        if (a == b) {
          const double x = P.psi[a][row + nu];
          pr = M(x, x);
        } else {
          double za = P.psi[a][row + src], zb = P.psi[b][row + src];
          if (middle) {
            za = (P.ihomo[a] == 1) ? za : 0.0;
            zb = (P.ihomo[b] == 1) ? zb : 0.0;
          } else if (second) {
            za = (P.ihomo[a] == -1) ? -za : za;
            zb = (P.ihomo[b] == -1) ? -zb : zb;
          }
          pr = M(za, zb);
        }
        v[t] = fma(w, pr, v[t]);
      }
    }
    block_sum_store<kMaxK>(v, partials + size_t(s0) * nb);
    __syncthreads();
  }
  __threadfence();
  if (!grid_barrier(bar, unsigned(nb))) return;
  // totals, one slot per warp at a time, in block order
  {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int t = warp; t < P.nslots; t += kThreads / 32) {
      const double *base = partials + size_t(t / kMaxK * kMaxK) * nb + (t % kMaxK);
      double x = 0.0;
      for (int b = lane; b < nb; b += 32) x += __ldcg(base + size_t(b) * kMaxK);
      for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
      if (lane == 0) s_h[t] = x;
    }
  }
  __syncthreads();
  if (threadIdx.x < n) s_z[threadIdx.x] = D(1.0, sqrt(s_h[P.slot_of[threadIdx.x][threadIdx.x]]));
  __syncthreads();
  // the coefficients, in the reference's orbital order (every block alike)
  if (threadIdx.x == 0) {
    for (int j = 0; j < n; ++j)
      for (int m = 0; m < n; ++m) s_c[j][m] = 0.0;
    for (int j = 0; j < n; ++j) {
      const double zarea = s_z[j];
      double ovl[kGramOrbs];
      double x = 0.0;
      for (int p = 0; p < P.npart[j]; ++p) {
        const int q = P.part[j][p];
        double sum = 0.0;
        for (int m = 0; m < n; ++m) {
          const int sl = P.slot_of[j][m];
          if (s_c[q][m] != 0.0 && sl >= 0) sum = A(sum, M(s_c[q][m], s_h[sl]));
        }
        ovl[p] = M(zarea, sum);
        x = A(x, M(ovl[p], ovl[p]));
      }
      if (P.npart[j] == 0) {
        s_c[j][j] = zarea;
      } else {
        const double ano = D(sqrt(A(1.0, x)), S(1.0, M(x, x)));
        double row[kGramOrbs];
        for (int m = 0; m < n; ++m) row[m] = (m == j) ? zarea : 0.0;
        for (int p = 0; p < P.npart[j]; ++p) {
          const int q = P.part[j][p];
          for (int m = 0; m < n; ++m) row[m] = A(row[m], M(-ovl[p], s_c[q][m]));
        }
        for (int m = 0; m < n; ++m) s_c[j][m] = M(ano, row[m]);
      }
      if (blockIdx.x == 0) {
        *P.norm_out[j] = s_h[P.slot_of[j][j]];
        for (int p = 0; p < P.npart[j]; ++p) P.ovl_out[j][p] = ovl[p];
      }
    }
  }
  __syncthreads();
  // Y = C Z, each thread owning its points (homonuclear: a first-half point
  // and its mirror, read once, written both)
  const int npts = P.homo ? n2 * g.nmu : g.mxsize;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < npts; k += gridDim.x * blockDim.x) {
    int mu, nu;
    if (P.homo) {
      mu = k / n2;
      nu = k - mu * n2;
    } else {
      mu = k / g.nni;
      nu = k - mu * g.nni;
    }
    const int row = (mu + 4) * g.n8 + 4;
    const bool middle = P.homo && nu == n2 - 1;
    double z[kGramOrbs];
#pragma unroll
    for (int j = 0; j < kGramOrbs; ++j) {
      if (j >= n) break;
      const double x = __ldcg(P.psi[j] + row + nu);
      z[j] = (middle && P.ihomo[j] != 1) ? 0.0 : x;
    }
#pragma unroll
    for (int j = 0; j < kGramOrbs; ++j) {
      if (j >= n) break;
      double y = 0.0;
#pragma unroll
      for (int m = 0; m < kGramOrbs; ++m) {
        if (m > j) break;
        if (s_c[j][m] != 0.0) y = A(y, M(s_c[j][m], z[m]));
      }
      P.psi[j][row + nu] = y;
      if (P.homo && !middle) P.psi[j][row + (g.nni - 1 - nu)] = (P.ihomo[j] == 1) ? y : -y;
    }
  }
}

// EaHF = oneelij(i,i) + (J + K): per point terms of integrals.F90:406-480
// and lagrangeMultipliers.F90:67-72.  psi's ghost cells are read as the
// mirrored interior values (identical to a putin ghost refresh); exact keeps
// the reference's unfused order, otherwise products are fused (mixed form).
// EaHF of one orbital (lagrangeMultipliers.F90:21-107 with the kinetic
// term of integrals.F90:406-480): the per-thread partial sums of one block
template <bool exact>
__device__ __forceinline__ void eahf_partials(const GridDev &g, const double *psi, int isym, int m,
                                              const double *coulp, const double *exchp, double (&v)[5]) {
  const int n8 = g.n8;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < g.mxsize; k += gridDim.x * blockDim.x) {
    const int mu = k / g.nni, nu = k - mu * g.nni;
    const int ij = (mu + 4) * n8 + nu + 4;
    // diffnu: sum_k f(nu+k-4) dni(k,nu); diffmu: sum_k f(mu+k-4) dmu(k,mu) (dgemv order)
    double sn = 0.0, sm = 0.0;
    const double *dn = g.dni9 + 9 * nu, *dm = g.dmu9 + 9 * mu;
    if (mu >= 4 && nu >= 4 && nu <= g.nni - 5) {
#pragma unroll
      for (int q = 0; q < 9; ++q) sn = madd<exact>(psi[ij + q - 4], dn[q], sn);
#pragma unroll
      for (int q = 0; q < 9; ++q) sm = madd<exact>(psi[ij + (q - 4) * n8], dm[q], sm);
    } else {
#pragma unroll
      for (int q = 0; q < 9; ++q) sn = madd<exact>(ghost_read(g, psi, mu + 4, nu + q, isym), dn[q], sn);
#pragma unroll
      for (int q = 0; q < 9; ++q) sm = madd<exact>(ghost_read(g, psi, mu + q, nu + 4, isym), dm[q], sm);
    }
    double kin = A(sn, sm);
    const double p = psi[ij];
    if (m != 0) kin = madd<exact>(M(double(m * m), g.e[k]), p, kin);
    const double pf0 = M(p, g.f0[k]);
    const double w1 = g.wgt1[k], w2 = g.wgt2[k];
    if (exact) {
      const double t = M(A(pf0, kin), p);
      v[0] += w1 * t;                   // oneel
      v[1] += w1 * M(kin, p);           // kinetic (+ m^2 e term)
      v[2] += w1 * M(pf0, p);           // nuclear
      v[3] += w2 * M(M(p, coulp[k]), p);
      v[4] += w2 * M(p, exchp[k]);
    } else {
      const double kp = kin * p, np = pf0 * p;
      v[1] = fma(w1, kp, v[1]);
      v[2] = fma(w1, np, v[2]);
      v[3] = fma(w2, (p * coulp[k]) * p, v[3]);
      v[4] = fma(w2, p * exchp[k], v[4]);
    }
  }
  if (!exact) v[0] = v[1] + v[2];  // oneel = kinetic + nuclear, summed per block
}

// EaHF and its parts from the summed quadratures (lagrangeMultipliers.F90:67-72)
__device__ __forceinline__ void eahf_store(const double *sums, double *ee_out, double *parts) {
  const double woneel = sums[0], wc = sums[3], wx = -sums[4];
  *ee_out = woneel + (wc + wx);
  if (parts) {
    parts[0] = sums[1];
    parts[1] = sums[2];
    parts[2] = woneel;
    parts[3] = wc;
    parts[4] = wx;
  }
}

template <bool exact>
__global__ void k_eahf(GridDev g, const double *psi, int isym, int m, const double *coulp, const double *exchp,
                       double *partials, double *sums, double *ee_out, double *parts, unsigned *ticket) {
  double v[5] = {0, 0, 0, 0, 0};
  eahf_partials<exact>(g, psi, isym, m, coulp, exchp, v);
  if (block_sum_finish<5>(v, partials, sums, 5, ticket) && threadIdx.x == 0) eahf_store(sums, ee_out, parts);
}

// EaHF of several orbitals in one launch: orbital blockIdx.y with its own
// partials, sums and ticket, reduced in the same block order as k_eahf
constexpr int kEahfItems = 36;
struct EahfList {
  EahfItem it[kEahfItems];
};
template <bool exact>
__global__ void k_eahf_batch(GridDev g, const __grid_constant__ EahfList L, double *partials, unsigned *tickets) {
  const EahfItem &I = L.it[blockIdx.y];
  double v[5] = {0, 0, 0, 0, 0};
  eahf_partials<exact>(g, I.psi, I.isym, I.m, I.coulp, I.exchp, v);
  double *part = partials + size_t(blockIdx.y) * (gridDim.x * 5 + 5);
  if (block_sum_finish<5>(v, part, part + size_t(gridDim.x) * 5, 5, tickets + blockIdx.y) && threadIdx.x == 0)
    eahf_store(part + size_t(gridDim.x) * 5, I.ee_out, I.parts);
}

struct TripleList {
  TripleItem it[kMaxK];
};

__global__ void k_triples(GridDev g, TripleList L, int n, double *partials, double *out, unsigned *ticket) {
  double v[kMaxK];
  for (int q = 0; q < kMaxK; ++q) v[q] = 0.0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < g.mxsize; k += gridDim.x * blockDim.x) {
    const int mu = k / g.nni, nu = k - mu * g.nni;
    const int ij = (mu + 4) * g.n8 + nu + 4;
    const double w = g.wgt2[k];
    for (int q = 0; q < n; ++q) {
      double t = M(L.it[q].a[ij], L.it[q].b[ij]);
      if (L.it[q].c) t = M(t, L.it[q].c[ij]);
      v[q] += w * t;
    }
  }
  block_sum_finish<kMaxK>(v, partials, out, n, ticket);
}

// coulMom (scfUtils.F90:490-603) and exchMom (scfUtils.F90:615-844, with
// the grid's weighted P_k^q r^k tables) of a batch of items (blockIdx.y =
// item), each with its own gridDim.x partial sums and ticket, so every
// item's sum runs in a fixed order
constexpr int kMomentItems = 64;
struct MomentList {
  MomentItem it[kMomentItems];
};
__global__ void k_moments(GridDev g, const __grid_constant__ MomentList L, int homo, double *partials,
                          unsigned *tickets) {
  const MomentItem &m = L.it[blockIdx.y];
  double v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  if (m.coul) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < g.mxsize; k += gridDim.x * blockDim.x) {
      const int mu = k / g.nni, nu = k - mu * g.nni;
      const double p = m.psa[(mu + 4) * g.n8 + nu + 4];
      const double wk1 = M(M(p, p), g.f4[k]);
      for (int q = 0; q < g.mpole; ++q) {
        if (homo && (q % 2 == 0)) continue;
        v[q] += g.wgt2[k] * M(g.leg[size_t(q) * g.mxsize + k], wk1);
      }
    }
  } else if (m.idel <= 4) {
    const double *T = g.exm + size_t(m.idel) * 8 * g.mxsize;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < g.mxsize; k += gridDim.x * blockDim.x) {
      const int mu = k / g.nni, nu = k - mu * g.nni;
      const int ij = (mu + 4) * g.n8 + nu + 4;
      const double wk1 = m.psa[ij] * m.psb[ij];
#pragma unroll
      for (int q = 0; q < 8; ++q)
        if (q < g.mpole) v[q] = fma(T[size_t(q) * g.mxsize + k], wk1, v[q]);
    }
  }
  block_sum_finish<8>(v, partials + size_t(blockIdx.y) * gridDim.x * 8, m.out, g.mpole, tickets + blockIdx.y);
}

// Checks narrow_f64 / widen_f32 against the hardware conversions on n
// values: edge cases, then bit patterns from a counter hash.  Counts
// mismatches outside the documented flush ranges (float subnormals); NaNs
// must map to NaNs.
__global__ void k_convert_selftest(long n, unsigned long long seed, unsigned long long *bad) {
  unsigned long long nb = 0;
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < n; i += long(gridDim.x) * blockDim.x) {
    unsigned long long h = (unsigned long long)i * 0x9E3779B97F4A7C15ull + seed;
    h ^= h >> 31;
    h *= 0xBF58476D1CE4E5B9ull;
    h ^= h >> 29;
    double x = __longlong_as_double((long long)h);
    if (i < 16) {
      const double edge[16] = {0.0, -0.0, 1.0, -1.0, 3.4028234663852886e38, 3.4028235677973366e38, 1e39, -1e39,
                               1.1754943508222875e-38, 1.1754942e-38, 1e-300, 0.1, 1.0 + 0x1p-24, 1.0 + 0x1p-23 + 0x1p-24,
                               __longlong_as_double(0x7ff0000000000000ll), __longlong_as_double(0x7ff8000000000001ll)};
      x = edge[i];
    }
    // narrowing
    const float a = narrow_f64(x), b = __double2float_rn(x);
    const bool sub = fabs(x) < 1.1754943508222875e-38 && x != 0.0;
    if (!sub) {
      if (isnan(b)) nb += isnan(a) ? 0 : 1;
      else nb += (__float_as_uint(a) == __float_as_uint(b)) ? 0 : 1;
    }
    // widening of a float pattern
    const float f = __uint_as_float(unsigned(h >> 32));
    const double wa = widen_f32(f), wb = double(f);
    const bool fsub = (__float_as_uint(f) & 0x7f800000u) == 0 && (__float_as_uint(f) & 0x7fffffu) != 0;
    if (!fsub) {
      if (isnan(wb)) nb += isnan(wa) ? 0 : 1;
      else nb += (__double_as_longlong(wa) == __double_as_longlong(wb)) ? 0 : 1;
    }
  }
  if (nb) atomicAdd(bad, nb);
}

inline int grid_blocks(int n) {
  int b = (n + kThreads - 1) / kThreads;
  return b < 1 ? 1 : (b > 1184 ? 1184 : b);
}

}  // namespace

// ======================================================================
// launchers
// ======================================================================

static double *reduction_partials(x2g_ctx *ctx, int K) {
  size_t need = size_t(kRedBlocksMax) * K * sizeof(double) + 64 * sizeof(double);
  if (ctx->red_bytes < need) {
    if (ctx->red) cudaFree(ctx->red);
    ctx->red = nullptr;
    ctx->red_bytes = 0;
    if (cudaMalloc(&ctx->red, need) != cudaSuccess) return nullptr;
    ctx->red_bytes = need;
  }
  return static_cast<double *>(ctx->red);
}

// Job-table entry of one x2g_job (kind 0 orbital with borb; 1 potential
// built from psa/psb; 2 potential given explicit lhs/rhs arrays, bpot).
static bool make_job(const x2g_job &x, JobDev &d) {
  const bool explicit_lr = (x.lhs && x.rhs);
  if (!x.u || (x.kind != 0 && x.kind != 1) || (x.kind == 0 && !explicit_lr) ||
      (x.kind == 1 && !explicit_lr && (!x.psa || !x.psb)) || (x.isym != 1 && x.isym != -1))
    return false;
  d = JobDev{};
  d.u = x.u;
  d.lhs = x.lhs;
  d.rhs = x.rhs;
  d.psa = x.psa;
  d.psb = x.psb;
  d.omega = x.omega;
  d.omegaf = float(x.omega);
  d.omega1f = float(1.0 - x.omega);
  d.idel2 = double(x.idel * x.idel);
  d.isym = x.isym;
  d.kind = (x.kind == 1 && explicit_lr) ? 2 : x.kind;
  return true;
}

static int take_event(x2g_ctx *ctx, cudaEvent_t *ev) {
  if (!ctx->event_pool.empty()) {
    *ev = ctx->event_pool.back();
    ctx->event_pool.pop_back();
    return X2G_OK;
  }
  cudaError_t err = cudaEventCreate(ev);
  return (err == cudaSuccess) ? X2G_OK : cuda_status(err, "profiling event");
}

// The cluster kernel's function attributes are shared by every context and
// thread of the process: the dynamic shared memory cap is set once to the
// device's opt-in maximum (never lowered, so concurrent contexts with
// different grids cannot undercut each other) and clusters above 8 CTAs are
// allowed.  Idempotent.
static bool cluster_attributes(x2g_ctx *ctx) {
  if (ctx->cluster_smem_set > 0 && ctx->cluster_nonportable) return true;
  int optin = 0;
  if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device) != cudaSuccess ||
      cudaFuncSetAttribute((const void *)k_mixed_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize, optin) !=
          cudaSuccess ||
      cudaFuncSetAttribute((const void *)k_mixed_cluster, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) !=
          cudaSuccess ||
      cudaFuncSetAttribute(pot_kernel(false), cudaFuncAttributeMaxDynamicSharedMemorySize, optin) != cudaSuccess ||
      cudaFuncSetAttribute(pot_kernel(false), cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess ||
      cudaFuncSetAttribute(pot_kernel(true), cudaFuncAttributeMaxDynamicSharedMemorySize, optin) != cudaSuccess ||
      cudaFuncSetAttribute(pot_kernel(true), cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
    (void)cudaGetLastError();
    return false;
  }
  ctx->cluster_smem_set = size_t(optin);
  ctx->cluster_nonportable = 1;
  return true;
}

// block size of the cluster sweep (pot: the potentials' variant; free: the
// seam-free colouring's plan)
static int cluster_threads(const GridDev &g, bool pot, bool free) {
  if (free) return 32 * (pot ? g.cf_pa + g.cf_pb + g.cf_ps : g.cf_wa + g.cf_wb + g.cf_ws);
  return 32 * (pot ? g.cl_pa + g.cl_pb + g.cl_ps : g.cl_wa + g.cl_wb + g.cl_ws);
}

// whether the on-chip cluster sweep (pot: its potentials' variant) can run
// this grid here, and how many of its clusters are co-resident (asked once
// per shape: shared memory per CTA, cluster size, block size)
static bool cluster_usable(x2g_ctx *ctx, const GridDev &g, bool pot = false) {
  if (g.cl_size < 2 || ctx->no_cluster) return false;
  const bool free = ctx->mixed_free != 0;
  const size_t smem = cluster_smem_bytes(g, pot, free);
  const long key = (long(smem) * 64 + g.cl_size) * 32 + cluster_threads(g, pot, free) / 32;
  const int v = pot ? 1 : 0;
  if (ctx->cluster_checked_key[v] != key) {
    ctx->cluster_checked_key[v] = key;
    ctx->cluster_ok[v] = 0;
    const bool attr_ok = cluster_attributes(ctx) && smem <= ctx->cluster_smem_set;
    if (attr_ok) {
      cudaLaunchConfig_t q = {};
      q.gridDim = dim3(unsigned(g.cl_size));
      q.blockDim = dim3(unsigned(cluster_threads(g, pot, free)));
      q.dynamicSmemBytes = smem;
      cudaLaunchAttribute qa[1];
      qa[0].id = cudaLaunchAttributeClusterDimension;
      qa[0].val.clusterDim.x = unsigned(g.cl_size);
      qa[0].val.clusterDim.y = 1;
      qa[0].val.clusterDim.z = 1;
      q.attrs = qa;
      q.numAttrs = 1;
      int nclusters = 0;
      const void *fn = pot ? pot_kernel(free) : (const void *)k_mixed_cluster;
      if (cudaOccupancyMaxActiveClusters(&nclusters, fn, &q) == cudaSuccess && nclusters > 0) {
        ctx->cluster_ok[v] = 1;
        ctx->cluster_active[v] = nclusters;
      }
    }
    (void)cudaGetLastError();
  }
  return ctx->cluster_ok[v] != 0;
}

// Launch shape of the persistent-band sweep: the most jobs per launch (at
// most `most`) and the shortest tile runs G for which every (job, run) gets
// its own co-resident block at two 512-thread blocks per SM (the band's
// shared memory must fit twice per SM).  The function's shared memory cap
// is raised once to the device's opt-in maximum, as for the cluster kernel.
static int persistent_shape(x2g_ctx *ctx, const GridDev &g, int most, int *nj, int *G, size_t *smem) {
  if (!ctx->band_attr) {
    // the cap counts dynamic bytes only: the opt-in maximum less the
    // kernel's static shared memory (the neighbour wait's flag)
    int optin = 0;
    cudaFuncAttributes fa{};
    if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device) != cudaSuccess ||
        cudaFuncGetAttributes(&fa, (const void *)k_mcsor_f32p) != cudaSuccess ||
        cudaFuncSetAttribute((const void *)k_mcsor_f32p, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             optin - int(fa.sharedSizeBytes)) != cudaSuccess) {
      (void)cudaGetLastError();
      return set_status(X2G_ERR_CUDA, "persistent sweep attributes could not be set");
    }
    ctx->band_attr = optin - int(fa.sharedSizeBytes);
    int per_sm = 0;
    if (cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, ctx->device) != cudaSuccess)
      return set_status(X2G_ERR_CUDA, "device attribute query failed");
    ctx->band_sm_smem = per_sm;
  }
  for (int n = most; n >= 1; --n)
    for (int r = 1; r <= HostGrid::kBandRuns; ++r) {
      const size_t sm = band_smem_bytes(g, r);
      if (sm > size_t(ctx->band_attr)) break;
      // two blocks per SM (1024 threads) hide more latency than one block
      // with twice the band
      int bpsm = int(size_t(ctx->band_sm_smem) / (sm + 1024));
      if (bpsm < 2) break;
      bpsm = 2;
      const int items = n * ((g.ntiles + r - 1) / r);
      if (bpsm >= 1 && items <= bpsm * ctx->num_sms) {
        // confirm with the occupancy calculator (once per shared size)
        if (ctx->band_key != long(sm)) {
          int per = 0;
          cudaError_t err =
              cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, (const void *)k_mcsor_f32p, kBandThreads, sm);
          if (err != cudaSuccess) return cuda_status(err, "occupancy query");
          ctx->band_key = long(sm);
          ctx->band_blocks = per * ctx->num_sms;
        }
        if (items > ctx->band_blocks) continue;
        *nj = n;
        *G = r;
        *smem = sm;
        return X2G_OK;
      }
    }
  return set_status(X2G_ERR_ARG, "grid too large for the persistent FP32 sweep");
}

// Co-resident blocks of the cooperative FP64 sweep on the context's device
// (asked once per context).
static int f64_block_limit(x2g_ctx *ctx) {
  if (ctx->f64_blocks > 0) return X2G_OK;
  int per_sm = 0;
  cudaError_t err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void *)k_mcsor_f64, kThreads, 0);
  if (err != cudaSuccess) return cuda_status(err, "occupancy query");
  if (per_sm < 1) return set_status(X2G_ERR_CUDA, "cooperative FP64 sweep cannot be resident");
  ctx->f64_blocks = per_sm * ctx->num_sms;
  return X2G_OK;
}

// One launch batch (at most kParamJobs jobs) of launch_relax.
// One launch of the on-chip cluster sweep over the jobs of jt, timed with the
// context's events when profiling.
static int cluster_sweep(x2g_ctx *ctx, const GridDev &g, JobTable &jt, int njobs, int nsweeps, bool pot) {
  x2g_ctx::Pending pe{};
  if (ctx->profiling) {
    int rc;
    if ((rc = take_event(ctx, &pe.a)) || (rc = take_event(ctx, &pe.b))) return rc;
    pe.precision = 1;
    pe.points = double(njobs) * double(g.nni - 2) * double(g.nmu - 5) * double(nsweeps);
    cudaEventRecord(pe.a, ctx->stream);
  }
  const int free = ctx->mixed_free;
  const size_t smem = cluster_smem_bytes(g, pot, free != 0);
  if (!cluster_attributes(ctx) || smem > ctx->cluster_smem_set)
    return set_status(X2G_ERR_CUDA, "cluster kernel attributes could not be set");
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(unsigned(njobs * g.cl_size));
  cfg.blockDim = dim3(unsigned(cluster_threads(g, pot, free != 0)));
  cfg.dynamicSmemBytes = smem;
  cfg.stream = ctx->stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = unsigned(g.cl_size);
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  GridDev gd = g;
  cudaError_t err = !pot ? cudaLaunchKernelEx(&cfg, k_mixed_cluster, gd, jt, nsweeps, free)
                    : free ? cudaLaunchKernelEx(&cfg, k_mixed_cluster_pot<kPotWarpsFree>, gd, jt, nsweeps, free)
                           : cudaLaunchKernelEx(&cfg, k_mixed_cluster_pot<kPotWarpsRef>, gd, jt, nsweeps, free);
  if (err != cudaSuccess) return cuda_status(err, "cluster MCSOR launch");
  ctx->launches += 1;
  if (ctx->profiling) {
    cudaEventRecord(pe.b, ctx->stream);
    ctx->pending.push_back(pe);
  }
  return X2G_OK;
}

// One launch batch (at most kParamJobs jobs) of launch_relax.
static int relax_batch(x2g_ctx *ctx, const GridDev &g, JobTable &jt, int njobs, int nsweeps, bool mixed,
                       bool on_chip, bool pot, int G, size_t smem) {
  cudaError_t err;
  x2g_ctx::Pending pe{};
  const double points = double(njobs) * double(g.nni - 2) * double(g.nmu - 5) * double(nsweeps);
  const int wave = ctx->cluster_active[1];
  if (mixed && on_chip && pot && ctx->residual_overlap && wave > 0 && njobs > wave) {
    // waves of the potentials' cluster variant: the first wave's FP64
    // residual, then the later waves' residuals on the low-priority
    // auxiliary stream, beside the sweeps (on the SMs they leave free);
    // each sweep waits for its own wave's residual.  The short wave (the
    // remainder) goes first: its residual is the only one on the critical
    // path, the full waves' residuals run beside sweeps
    const int nw = (njobs + wave - 1) / wave;
    std::vector<JobTable> w(size_t(nw), JobTable{});
    std::vector<int> sz(size_t(nw), wave);
    if (njobs % wave) sz[0] = njobs % wave;
    const unsigned nblk = unsigned(grid_blocks((g.nni - 2) * (g.nmu - 5)));
    for (int c = 0, i0 = 0; c < nw; i0 += sz[size_t(c)], ++c)
      for (int i = 0; i < sz[size_t(c)]; ++i) w[size_t(c)].j[i] = jt.j[i0 + i];
    auto size = [&](int c) { return sz[size_t(c)]; };
    k_residual<false><<<dim3(nblk, size(0)), kThreads, 0, ctx->stream>>>(g, w[0], 0, 0);
    ctx->launches += 1;
    if ((err = cudaEventRecord(ctx->ev_split[0], ctx->stream)) != cudaSuccess ||
        (err = cudaStreamWaitEvent(ctx->aux, ctx->ev_split[0], 0)) != cudaSuccess)
      return cuda_status(err, "residual overlap");
    for (int c = 0; c < nw; ++c) {
      cudaEvent_t ev = ctx->ev_split[(c + 1) & 1];
      if (c + 1 < nw) {
        k_residual<false><<<dim3(nblk, size(c + 1)), kThreads, 0, ctx->aux>>>(g, w[c + 1], 0, 0);
        ctx->launches += 1;
        if ((err = cudaEventRecord(ev, ctx->aux)) != cudaSuccess) return cuda_status(err, "residual overlap");
      }
      int rc = cluster_sweep(ctx, g, w[c], size(c), nsweeps, true);
      if (rc) return rc;
      if (c + 1 < nw && (err = cudaStreamWaitEvent(ctx->stream, ev, 0)) != cudaSuccess)
        return cuda_status(err, "residual overlap");
    }
    return X2G_OK;
  }
  if (mixed) {
    dim3 gr(grid_blocks((g.nni - 2) * (g.nmu - 5)), njobs);
    if (on_chip)
      k_residual<false><<<gr, kThreads, 0, ctx->stream>>>(g, jt, 0, pot ? 0 : 1);
    else
      k_residual<true><<<gr, kThreads, 0, ctx->stream>>>(g, jt, 1, 1);
    ctx->launches += 1;
  }
  if (on_chip) return cluster_sweep(ctx, g, jt, njobs, nsweeps, pot);
  if (ctx->profiling) {
    int rc;
    if ((rc = take_event(ctx, &pe.a)) || (rc = take_event(ctx, &pe.b))) return rc;
    pe.precision = mixed ? 1 : 0;
    pe.points = points;
    cudaEventRecord(pe.a, ctx->stream);
  }
  {
    // persistent cooperative kernels: the FP64 sweep with grid barriers,
    // the mixed form's persistent-band sweep with neighbour waits.  Only the
    // arrival count and generation are reset: the error word keeps an
    // earlier launch's timeout until x2g_synchronize reports it
    err = cudaMemsetAsync(ctx->bar, 0, 2 * sizeof(unsigned), ctx->stream);
    if (err != cudaSuccess) return cuda_status(err, "barrier reset");
    BarrierDev bar{ctx->bar, ctx->bar + 1, reinterpret_cast<int *>(ctx->bar + 2), ctx->wait_limit_ns};
    int nj = njobs, ns = nsweeps;
    GridDev gd = g;
    if (mixed) {
      // one block per (job, run of G tiles); phase counts zeroed
      const unsigned nb = unsigned(njobs * ((g.ntiles + G - 1) / G));
      if (nb > unsigned(kPhaseBlocks)) return set_status(X2G_ERR_ARG, "too many blocks for the phase counts");
      err = cudaMemsetAsync(ctx->bar + kPhaseWords, 0, size_t(kPhaseBlocks) * kPhaseStride * sizeof(unsigned),
                            ctx->stream);
      if (err != cudaSuccess) return cuda_status(err, "barrier reset");
      unsigned *phase = ctx->bar + kPhaseWords;
      void *args[] = {&gd, &jt, &ns, &G, &bar, &phase};
      err = cudaLaunchCooperativeKernel((const void *)k_mcsor_f32p, dim3(nb), dim3(kBandThreads), args, smem,
                                        ctx->stream);
    } else {
      int rc = f64_block_limit(ctx);
      if (rc) return rc;
      const int nitems = njobs * g.ntiles;
      unsigned nblocks = unsigned(nitems < ctx->f64_blocks ? nitems : ctx->f64_blocks);
      if (nblocks < 1) nblocks = 1;
      void *args[] = {&gd, &jt, &nj, &ns, &bar, &nblocks};
      err = cudaLaunchCooperativeKernel((const void *)k_mcsor_f64, dim3(nblocks), dim3(kThreads), args, 0,
                                        ctx->stream);
    }
    if (err != cudaSuccess) return cuda_status(err, "cooperative MCSOR launch");
    ctx->launches += 1;
    if (ctx->profiling) {
      cudaEventRecord(pe.b, ctx->stream);
      ctx->pending.push_back(pe);
    }
    // the mixed form's update u += e and the axis of u are the
    // persistent-band sweep's epilogue
  }
  return X2G_OK;
}

// List-order SOR: jobs in launches of kParamJobs, each one cooperative
// wavefront launch; the grid holds as many blocks as the widest step needs.
static int relax_sor(x2g_ctx *ctx, const x2g_grid *grid, const x2g_job *jobs, int njobs, int nsweeps) {
  const GridDev &g = grid->d;
  if (ctx->sor_blocks < 0) {
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void *)k_sor_f64, kThreads, 0);
    if (e != cudaSuccess) return cuda_status(e, "occupancy query");
    if (per_sm < 1) return set_status(X2G_ERR_CUDA, "cooperative SOR sweep cannot be resident");
    ctx->sor_blocks = per_sm * ctx->num_sms;
  }
  int widest = 0;
  for (int l = 0; l < g.sor_nlev; ++l) widest = std::max(widest, grid->h.sor_off[l + 1] - grid->h.sor_off[l]);
  for (int b0 = 0; b0 < njobs; b0 += kParamJobs) {
    const int nb = (njobs - b0 < kParamJobs) ? njobs - b0 : kParamJobs;
    JobTable jt{};
    for (int i = 0; i < nb; ++i)
      if (!make_job(jobs[b0 + i], jt.j[i])) return set_status(X2G_ERR_ARG, "bad relaxation job");
    cudaError_t err = cudaMemsetAsync(ctx->bar, 0, 2 * sizeof(unsigned), ctx->stream);
    if (err != cudaSuccess) return cuda_status(err, "barrier reset");
    BarrierDev bar{ctx->bar, ctx->bar + 1, reinterpret_cast<int *>(ctx->bar + 2), ctx->wait_limit_ns};
    const int inflight = std::min(nsweeps, (std::max(g.sor_nlev, g.sor_nblev) + g.sor_delta - 1) / g.sor_delta + 1);
    const long items = long(nb) * widest * inflight;
    long want = (items + kThreads - 1) / kThreads;
    want = std::max(want, long(std::min(nb * g.ntiles, ctx->sor_blocks)));  // the ghost prologue's tiles
    unsigned nblocks = unsigned(std::min(want, long(ctx->sor_blocks)));
    if (nblocks < 1) nblocks = 1;
    int nj = nb, ns = nsweeps;
    GridDev gd = g;
    void *args[] = {&gd, &jt, &nj, &ns, &bar, &nblocks};
    err = cudaLaunchCooperativeKernel((const void *)k_sor_f64, dim3(nblocks), dim3(kThreads), args, 0, ctx->stream);
    if (err != cudaSuccess) return cuda_status(err, "cooperative SOR launch");
    ctx->launches += 1;
  }
  return X2G_OK;
}

// co-resident clusters of the cluster sweep and of its potentials' variant
// for this grid on the context's device (0: that kernel cannot run it)
int cluster_occupancy(x2g_ctx *ctx, x2g_grid *grid, int *plain, int *pot) {
  const GridDev &g = grid->d;
  const int a = cluster_usable(ctx, g, false) ? ctx->cluster_active[0] : 0;
  const int b = cluster_usable(ctx, g, true) ? ctx->cluster_active[1] : 0;
  if (plain) *plain = a;
  if (pot) *pot = b;
  return set_status(X2G_OK, "");
}

int launch_relax(x2g_ctx *ctx, x2g_grid *grid, const x2g_job *jobs, int njobs, int nsweeps, int precision) {
  if (njobs <= 0) return X2G_OK;
  if (nsweeps <= 0) return set_status(X2G_ERR_ARG, "nsweeps must be positive");
  if (precision == X2G_SOR) return relax_sor(ctx, grid, jobs, njobs, nsweeps);
  if (precision != X2G_FP64 && precision != X2G_MIXED) return set_status(X2G_ERR_ARG, "unknown relaxation form");
  const GridDev &g = grid->d;
  const bool mixed = (precision == X2G_MIXED);
  bool on_chip = mixed && cluster_usable(ctx, g);
  // potentials built from orbitals (separable lhs): the variant at two CTAs
  // per SM when the batch is larger than the clusters co-resident at one
  bool pot = false;
  if (on_chip && ctx->pot_clusters != 0) {
    pot = true;
    for (int i = 0; i < njobs && pot; ++i) pot = (jobs[i].kind == 1 && !(jobs[i].lhs && jobs[i].rhs));
    if (pot && ctx->pot_clusters == 2) pot = njobs > ctx->cluster_active[0];
    pot = pot && cluster_usable(ctx, g, true);
  }
  if (on_chip && !pot && ctx->auto_band && njobs > ctx->cluster_active[0]) {
    // more jobs than co-resident clusters: the cluster kernel would run in
    // waves, while the persistent-band kernel may hold the whole batch
    int nj = 0, G1 = 0;
    size_t sm1 = 0;
    const int want = njobs < kParamJobs ? njobs : kParamJobs;
    if (persistent_shape(ctx, g, want, &nj, &G1, &sm1) == X2G_OK && nj >= want) on_chip = false;
    set_status(X2G_OK, "");
  }
  // per-job scratch: FP64 rhs of potentials, or the mixed form's FP32
  // correction, residual and omega/lhs
  const size_t per_job =
      (mixed ? (size_t(g.next) * sizeof(float) + 2 * size_t(g.mxsize) * sizeof(float) + 256)
             : (size_t(g.mxsize) * sizeof(double) + 256)) / 256 * 256 + 256;
  char *scratch = static_cast<char *>(ctx_workspace(ctx, per_job * njobs + 256));
  if (!scratch) return set_status(X2G_ERR_ALLOC, "workspace allocation failed");
  // the persistent-band sweep takes as many jobs per launch as give every
  // (job, run of tiles) its own co-resident block
  int per_launch = kParamJobs, G = 0;
  size_t smem = 0;
  if (mixed && !on_chip) {
    int rc = persistent_shape(ctx, g, njobs < kParamJobs ? njobs : kParamJobs, &per_launch, &G, &smem);
    if (rc) return rc;
  }
  for (int b0 = 0; b0 < njobs; b0 += per_launch) {
    const int nb = (njobs - b0 < per_launch) ? njobs - b0 : per_launch;
    JobTable jt{};
    for (int i = 0; i < nb; ++i) {
      JobDev &d = jt.j[i];
      if (!make_job(jobs[b0 + i], d)) return set_status(X2G_ERR_ARG, "bad relaxation job");
      char *p = scratch + per_job * size_t(b0 + i);
      if (mixed) {
        d.e32 = reinterpret_cast<float *>(p);
        d.r32 = reinterpret_cast<float *>(p + (size_t(g.next) * sizeof(float) + 127) / 128 * 128);
        d.w32 = d.r32 + g.mxsize;
        d.rw = reinterpret_cast<float2 *>(d.r32);  // persistent-band sweep: pairs over r32 and w32
      } else {
        d.rhs_buf = reinterpret_cast<double *>(p);
      }
    }
    int rc = relax_batch(ctx, g, jt, nb, nsweeps, mixed, on_chip, pot, G, smem);
    if (rc) return rc;
  }
  // barrier error word: checked by the caller at its next synchronisation
  return X2G_OK;
}

// Scratch layout of launch_relax_in_scratch: 4 barrier words, a reserved
// region the size of a job table, then one plain right-hand-side buffer per
// job (256-byte aligned).  The job-table size is part of the documented
// limit of x2g_relax_noalloc.
static_assert(sizeof(JobDev) == 112, "x2g_relax_noalloc documents 112-byte job-table entries");
size_t relax_scratch_bytes(const GridDev &g, int njobs) {
  const size_t head = 256;
  const size_t table = (sizeof(JobDev) * size_t(njobs) + 255) / 256 * 256;
  const size_t plain = (size_t(g.mxsize) * sizeof(double) + 255) / 256 * 256;
  return head + table + plain * size_t(njobs);
}

int launch_relax_in_scratch(x2g_ctx *ctx, x2g_grid *grid, const x2g_job *jobs, int njobs, int nsweeps,
                            void *scratch, size_t scratch_bytes) {
  const GridDev &g = grid->d;
  if (njobs <= 0 || nsweeps <= 0) return set_status(X2G_ERR_ARG, "njobs and nsweeps must be positive");
  const size_t need = relax_scratch_bytes(g, njobs);
  if (need > scratch_bytes) return set_status(X2G_ERR_ARG, "batch does not fit the scratch");
  char *base = static_cast<char *>(scratch);
  unsigned *barw = reinterpret_cast<unsigned *>(base);
  char *rhs0 = base + 256 + (sizeof(JobDev) * size_t(njobs) + 255) / 256 * 256;
  const size_t plain = (size_t(g.mxsize) * sizeof(double) + 255) / 256 * 256;
  for (int b0 = 0; b0 < njobs; b0 += kParamJobs) {
    const int nb = (njobs - b0 < kParamJobs) ? njobs - b0 : kParamJobs;
    JobTable jt{};
    for (int i = 0; i < nb; ++i)
      if (!make_job(jobs[b0 + i], jt.j[i])) return set_status(X2G_ERR_ARG, "bad relaxation job");
  }
  int rc = f64_block_limit(ctx);
  if (rc) return rc;
  // the error word is cleared once per call; between launches only the
  // arrival count and generation, so that a timeout of one launch is still
  // there when the caller reads it after the last
  cudaError_t err = cudaMemsetAsync(barw, 0, 4 * sizeof(unsigned), ctx->stream);
  if (err != cudaSuccess) return cuda_status(err, "scratch barrier reset");
  for (int b0 = 0; b0 < njobs; b0 += kParamJobs) {
    const int nb = (njobs - b0 < kParamJobs) ? njobs - b0 : kParamJobs;
    JobTable jt{};
    for (int i = 0; i < nb; ++i) {
      make_job(jobs[b0 + i], jt.j[i]);
      jt.j[i].rhs_buf = reinterpret_cast<double *>(rhs0 + plain * size_t(b0 + i));
    }
    if (b0 > 0) {
      err = cudaMemsetAsync(barw, 0, 2 * sizeof(unsigned), ctx->stream);
      if (err != cudaSuccess) return cuda_status(err, "scratch barrier reset");
    }
    BarrierDev bar{barw, barw + 1, reinterpret_cast<int *>(barw + 2), ctx->wait_limit_ns};
    const int nitems = nb * g.ntiles, cap = ctx->f64_blocks;
    unsigned nblocks = unsigned(nitems < cap ? nitems : cap);
    if (nblocks < 1) nblocks = 1;
    int nj = nb, ns = nsweeps;
    GridDev gd = g;
    void *args[] = {&gd, &jt, &nj, &ns, &bar, &nblocks};
    err = cudaLaunchCooperativeKernel((const void *)k_mcsor_f64, dim3(nblocks), dim3(kThreads), args, 0, ctx->stream);
    if (err != cudaSuccess) return cuda_status(err, "cooperative MCSOR launch");
    ctx->launches += 1;
  }
  return X2G_OK;
}

void launch_ghost_fill(x2g_ctx *ctx, const GridDev &g, double *u, int isym) {
  k_ghost<<<grid_blocks(g.nmu * 8 + 4 * g.nni), kThreads, 0, ctx->stream>>>(g, u, isym);
  ctx->launches++;
}

void launch_putin(x2g_ctx *ctx, const GridDev &g, int isym, const double *plain, double *ext) {
  k_putin_interior<<<grid_blocks(g.mxsize), kThreads, 0, ctx->stream>>>(g, plain, ext);
  k_ghost<<<grid_blocks(g.nmu * 8 + 4 * g.nni), kThreads, 0, ctx->stream>>>(g, ext, isym);
  ctx->launches += 2;
}

void launch_putout(x2g_ctx *ctx, const GridDev &g, const double *ext, double *plain) {
  k_putout<<<grid_blocks(g.mxsize), kThreads, 0, ctx->stream>>>(g, ext, plain);
  ctx->launches++;
}

void launch_fock(x2g_ctx *ctx, const GridDev &g, const FockArgs &a) {
  if (a.exact)
    k_fock<true><<<grid_blocks(g.mxsize), kThreads, 0, ctx->stream>>>(g, a);
  else
    k_fock<false><<<grid_blocks(g.mxsize), kThreads, 0, ctx->stream>>>(g, a);
  ctx->launches++;
}

void launch_fock_batch(x2g_ctx *ctx, const GridDev &g, const FockArgs *a, int n) {
  for (int b = 0; b < n; b += kFockBatch) {
    const int m = (n - b < kFockBatch) ? n - b : kFockBatch;
    FockBatch B{};
    for (int q = 0; q < m; ++q) B.a[q] = a[b + q];
    const dim3 gg(grid_blocks(g.mxsize), m);
    if (a[0].exact)
      k_fock_batch<true><<<gg, kThreads, 0, ctx->stream>>>(g, B);
    else
      k_fock_batch<false><<<gg, kThreads, 0, ctx->stream>>>(g, B);
    ctx->launches++;
  }
}

void launch_asympt_get_batch(x2g_ctx *ctx, const GridDev &g, const OrbDecayList &L, int n) {
  if (n <= 0) return;
  k_asympt_get_batch<<<dim3(grid_blocks(4 * g.nni), n), kThreads, 0, ctx->stream>>>(g, L);
  ctx->launches++;
}

void launch_asympt_set_batch(x2g_ctx *ctx, const GridDev &g, const OrbDecayList &L, int n) {
  if (n <= 0) return;
  k_asympt_set_batch<<<dim3(grid_blocks(g.nni), n), kThreads, 0, ctx->stream>>>(g, L);
  ctx->launches++;
}

void launch_asympt_get(x2g_ctx *ctx, const GridDev &g, const double *fa, double *edecay) {
  k_asympt_get<<<grid_blocks(4 * g.nni), kThreads, 0, ctx->stream>>>(g, fa, edecay);
  ctx->launches++;
}

void launch_asympt_set(x2g_ctx *ctx, const GridDev &g, double *psi, const double *edecay) {
  k_asympt_set<<<grid_blocks(g.nni), kThreads, 0, ctx->stream>>>(g, psi, edecay);
  ctx->launches++;
}

void launch_setci(x2g_ctx *ctx, const GridDev &g, double *psi, int ihomo) {
  k_setci<<<grid_blocks((g.nni / 2) * g.nmu), kThreads, 0, ctx->stream>>>(g, psi, ihomo);
  ctx->launches++;
}

void launch_scale(x2g_ctx *ctx, const GridDev &g, double *psi, const double *norm_dev) {
  k_scale<<<grid_blocks(g.mxsize), kThreads, 0, ctx->stream>>>(g, psi, norm_dev);
  ctx->launches++;
}

void launch_scale_setci(x2g_ctx *ctx, const GridDev &g, double *psi, const double *norm_dev, int ihomo) {
  k_scale_setci<<<grid_blocks((g.nni / 2 + 1) * g.nmu), kThreads, 0, ctx->stream>>>(g, psi, norm_dev, ihomo);
  ctx->launches++;
}

void launch_ortho_apply(x2g_ctx *ctx, const GridDev &g, double *psi, const double *const *others, int n,
                        const double *ovl_dev) {
  PtrList L{};
  for (int q = 0; q < n && q < kMaxTerms; ++q) L.p[q] = others[q];
  k_ortho_apply<<<grid_blocks(g.mxsize), kThreads, 0, ctx->stream>>>(g, psi, L, n, ovl_dev);
  ctx->launches++;
}

int convert_selftest(x2g_ctx *ctx, long n, unsigned long long seed, unsigned long long *mismatches) {
  unsigned long long *d = nullptr;
  cudaError_t e = cudaMallocAsync(&d, sizeof(unsigned long long), ctx->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(d, 0, sizeof(unsigned long long), ctx->stream);
  if (e == cudaSuccess) {
    k_convert_selftest<<<4 * ctx->num_sms, kThreads, 0, ctx->stream>>>(n, seed, d);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(mismatches, d, sizeof(unsigned long long), cudaMemcpyDeviceToHost, ctx->stream);
  if (d) cudaFreeAsync(d, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  return (e == cudaSuccess) ? X2G_OK : cuda_status(e, "conversion self-test");
}

int build_moment_tables(x2g_ctx *ctx, const GridDev &g, double *exm, double *asy) {
  k_moment_tables<<<grid_blocks(g.mxsize), kThreads, 0, ctx->stream>>>(g, exm, asy);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  return (e == cudaSuccess) ? X2G_OK : cuda_status(e, "moment tables");
}

void launch_asympt(x2g_ctx *ctx, const GridDev &g, const AsymptArgs &a) {
  if (a.n <= 0) return;
  dim3 gg(grid_blocks(4 * g.nni), a.n);
  k_asympt<<<gg, kThreads, 0, ctx->stream>>>(g, a);
  ctx->launches++;
}

void launch_zero(x2g_ctx *ctx, double *p, size_t n) {
  k_zero<<<grid_blocks(int(n < (1u << 30) ? n : (1u << 30))), kThreads, 0, ctx->stream>>>(p, n);
  ctx->launches++;
}

void launch_norm(x2g_ctx *ctx, const GridDev &g, const double *psi, double *out) {
  double *part = reduction_partials(ctx, 1);
  k_norm<<<red_blocks(g), kThreads, 0, ctx->stream>>>(g, psi, part, out, ctx->bar + 3);
  ctx->launches += 1;
}

void launch_overlaps(x2g_ctx *ctx, const GridDev &g, const double *psi, const double *const *others, int n,
                     double *out) {
  double *part = reduction_partials(ctx, kMaxK);
  for (int b = 0; b < n; b += kMaxK) {
    const int m = (n - b < kMaxK) ? n - b : kMaxK;
    PtrList L{};
    for (int q = 0; q < m; ++q) L.p[q] = others[b + q];
    k_overlaps<<<red_blocks(g), kThreads, 0, ctx->stream>>>(g, psi, L, m, part, out + b, ctx->bar + 3);
    ctx->launches += 1;
  }
}

// one orthonormalisation round: norms, scaling (and setCiOrb), overlaps
// with the partners, Gram-Schmidt, each over all orbitals of the round
void launch_ortho_round(x2g_ctx *ctx, const GridDev &g, const OrthoOrbital *orbs, int n) {
  const int nb = red_blocks(g);
  for (int b = 0; b < n; b += kRoundItems) {
    const int m = (n - b < kRoundItems) ? n - b : kRoundItems;
    OrthoRound R{};
    bool any_partner = false;
    for (int q = 0; q < m; ++q) {
      const OrthoOrbital &x = orbs[b + q];
      OrthoItem &I = R.it[q];
      I.psi = x.psi;
      I.n = x.n;
      for (int k = 0; k < x.n; ++k) I.o[k] = x.partners[k];
      I.ihomo = x.ihomo;
      I.norm_out = x.norm_out;
      I.ovl_out = x.ovl_out;
      any_partner = any_partner || x.n > 0;
    }
    double *part = reduction_partials(ctx, kMaxK * kRoundItems);
    k_norm_round<<<dim3(nb, m), kThreads, 0, ctx->stream>>>(g, R, part, ctx->bar + kMomentTickets);
    k_scale_round<<<dim3(grid_blocks(g.mxsize), m), kThreads, 0, ctx->stream>>>(g, R);
    ctx->launches += 2;
    if (any_partner) {
      k_overlaps_round<<<dim3(nb, m), kThreads, 0, ctx->stream>>>(g, R, part, ctx->bar + kMomentTickets);
      k_ortho_round<<<dim3(grid_blocks(g.mxsize), m), kThreads, 0, ctx->stream>>>(g, R);
      ctx->launches += 2;
    }
  }
}

// the Gram-matrix form of one iteration's orthonormalisation; false: the
// plan does not fit it (more orbitals or inner products than it holds, too
// few co-resident blocks), the caller takes the round-by-round form
bool launch_orthonormalise_gram(x2g_ctx *ctx, const GridDev &g, const OrthoOrbital *orbs, int n,
                                const int *partner_index) {
  if (n < 1 || n > kGramOrbs) return false;
  GramPlan P{};
  P.n = n;
  P.homo = orbs[0].ihomo != 0;
  for (int j = 0; j < n; ++j) {
    P.psi[j] = orbs[j].psi;
    P.norm_out[j] = orbs[j].norm_out;
    P.ovl_out[j] = orbs[j].ovl_out;
    P.ihomo[j] = orbs[j].ihomo;
    if ((orbs[j].ihomo != 0) != (P.homo != 0)) return false;
    P.npart[j] = orbs[j].n;
    for (int p = 0; p < orbs[j].n; ++p) P.part[j][p] = (signed char)partner_index[j * kGramOrbs + p];
    for (int m = 0; m < kGramOrbs; ++m) P.slot_of[j][m] = -1;
  }
  // slots: every norm, then <Z_a, Z_b> of every pair of a symmetry block
  // (the orbitals a partner chain connects)
  std::vector<int> blk(size_t(n), -1);
  int nblk = 0;
  for (int j = 0; j < n; ++j) {
    if (blk[size_t(j)] < 0) blk[size_t(j)] = nblk++;
    for (int p = 0; p < orbs[j].n; ++p) {
      const int q = partner_index[j * kGramOrbs + p];
      if (q < 0 || q >= j) return false;
      if (blk[size_t(q)] != blk[size_t(j)]) {
        const int from = blk[size_t(q)], to = blk[size_t(j)];
        for (auto &b : blk)
          if (b == from) b = to;
      }
    }
  }
  int ns = 0;
  for (int j = 0; j < n; ++j) {
    P.slot_of[j][j] = (signed char)ns;
    P.sa[ns] = P.sb[ns] = (signed char)j;
    ++ns;
  }
  for (int a = 0; a < n; ++a)
    for (int b = a + 1; b < n; ++b)
      if (blk[size_t(a)] == blk[size_t(b)]) {
        if (ns >= kGramSlots) return false;
        P.slot_of[a][b] = P.slot_of[b][a] = (signed char)ns;
        P.sa[ns] = (signed char)a;
        P.sb[ns] = (signed char)b;
        ++ns;
      }
  P.nslots = ns;
  if (ctx->gram_blocks < 0) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void *)k_orthonormalise_gram, kThreads, 0) !=
        cudaSuccess)
      per_sm = 0;
    (void)cudaGetLastError();
    ctx->gram_blocks = per_sm * ctx->num_sms;
  }
  // two blocks per SM (the passes are latency bound), at most the partials' room
  const int nb = std::min(std::min(2 * ctx->num_sms, ctx->gram_blocks), kRedBlocksMax);
  if (nb < 1) return false;
  double *part = reduction_partials(ctx, ((ns + kMaxK - 1) / kMaxK) * kMaxK);
  if (!part) return false;
  if (cudaMemsetAsync(ctx->bar, 0, 2 * sizeof(unsigned), ctx->stream) != cudaSuccess) return false;
  BarrierDev bar{ctx->bar, ctx->bar + 1, reinterpret_cast<int *>(ctx->bar + 2), ctx->wait_limit_ns};
  GridDev gd = g;
  void *args[] = {&gd, &P, &part, &bar};
  if (cudaLaunchCooperativeKernel((const void *)k_orthonormalise_gram, dim3(nb), dim3(kThreads), args, 0,
                                  ctx->stream) != cudaSuccess) {
    (void)cudaGetLastError();
    return false;
  }
  ctx->launches += 1;
  return true;
}

// every round in one cooperative launch; false: the plan does not fit it
// (more orbitals or rounds than its table holds, or too few co-resident
// blocks), the caller then launches round by round
bool launch_orthonormalise(x2g_ctx *ctx, const GridDev &g, const OrthoOrbital *orbs, const int *round_off,
                           int nrounds) {
  const int n = round_off[nrounds];
  if (n > kOrthoItems || nrounds > kOrthoRounds || nrounds < 1) return false;
  const int nb = red_blocks(g);
  if (ctx->ortho_blocks < 0) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void *)k_orthonormalise, kThreads, 0) !=
        cudaSuccess)
      per_sm = 0;
    (void)cudaGetLastError();
    ctx->ortho_blocks = per_sm * ctx->num_sms;
  }
  if (nb > ctx->ortho_blocks) return false;
  OrthoPlan P{};
  for (int q = 0; q < n; ++q) {
    const OrthoOrbital &x = orbs[q];
    OrthoItem &I = P.it[q];
    I.psi = x.psi;
    I.n = x.n;
    for (int k = 0; k < x.n; ++k) I.o[k] = x.partners[k];
    I.ihomo = x.ihomo;
    I.norm_out = x.norm_out;
    I.ovl_out = x.ovl_out;
  }
  int most = n;  // the norms of every item, or a round's overlap slot groups (kMaxK slots each)
  for (int r = 0; r <= nrounds; ++r) P.round_off[r] = round_off[r];
  for (int r = 0; r < nrounds; ++r) most = std::max(most, kMaxK * (round_off[r + 1] - round_off[r]));
  P.nrounds = nrounds;
  double *part = reduction_partials(ctx, most);
  if (!part) return false;
  if (cudaMemsetAsync(ctx->bar, 0, 2 * sizeof(unsigned), ctx->stream) != cudaSuccess) return false;
  BarrierDev bar{ctx->bar, ctx->bar + 1, reinterpret_cast<int *>(ctx->bar + 2), ctx->wait_limit_ns};
  GridDev gd = g;
  void *args[] = {&gd, &P, &part, &bar};
  if (cudaLaunchCooperativeKernel((const void *)k_orthonormalise, dim3(nb), dim3(kThreads), args, 0, ctx->stream) !=
      cudaSuccess) {
    (void)cudaGetLastError();
    return false;
  }
  ctx->launches += 1;
  return true;
}

void launch_eahf(x2g_ctx *ctx, const GridDev &g, const double *psi, int isym, int m, const double *coulp,
                 const double *exchp, double *ee_out, double *parts, bool exact) {
  double *part = reduction_partials(ctx, 5);
  const int nb = red_blocks(g);
  double *sums = part + size_t(nb) * 5;
  if (exact)
    k_eahf<true><<<nb, kThreads, 0, ctx->stream>>>(g, psi, isym, m, coulp, exchp, part, sums, ee_out, parts,
                                                   ctx->bar + 3);
  else
    k_eahf<false><<<nb, kThreads, 0, ctx->stream>>>(g, psi, isym, m, coulp, exchp, part, sums, ee_out, parts,
                                                    ctx->bar + 3);
  ctx->launches += 1;
}

void launch_eahf_batch(x2g_ctx *ctx, const GridDev &g, const EahfItem *items, int n, bool exact) {
  const int nb = red_blocks(g);
  for (int b = 0; b < n; b += kEahfItems) {
    const int m = (n - b < kEahfItems) ? n - b : kEahfItems;
    EahfList L{};
    for (int q = 0; q < m; ++q) L.it[q] = items[b + q];
    double *part = reduction_partials(ctx, 5 * kEahfItems + 5 * kEahfItems / 4);
    if (exact)
      k_eahf_batch<true><<<dim3(nb, m), kThreads, 0, ctx->stream>>>(g, L, part, ctx->bar + kMomentTickets);
    else
      k_eahf_batch<false><<<dim3(nb, m), kThreads, 0, ctx->stream>>>(g, L, part, ctx->bar + kMomentTickets);
    ctx->launches += 1;
  }
}

void launch_triples(x2g_ctx *ctx, const GridDev &g, const TripleItem *items, int n, double *out) {
  double *part = reduction_partials(ctx, kMaxK);
  for (int b = 0; b < n; b += kMaxK) {
    const int m = (n - b < kMaxK) ? n - b : kMaxK;
    TripleList L{};
    for (int q = 0; q < m; ++q) L.it[q] = items[b + q];
    k_triples<<<red_blocks(g), kThreads, 0, ctx->stream>>>(g, L, m, part, out + b, ctx->bar + 3);
    ctx->launches += 1;
  }
}

void launch_moments(x2g_ctx *ctx, const GridDev &g, const MomentItem *items, int n, int homo) {
  for (int b = 0; b < n; b += kMomentItems) {
    const int m = (n - b < kMomentItems) ? n - b : kMomentItems;
    double *part = reduction_partials(ctx, 8 * m);
    MomentList L{};
    for (int q = 0; q < m; ++q) L.it[q] = items[b + q];
    k_moments<<<dim3(red_blocks(g), m), kThreads, 0, ctx->stream>>>(g, L, homo, part, ctx->bar + kMomentTickets);
    ctx->launches += 1;
  }
}


}  // namespace x2g
