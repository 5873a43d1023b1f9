// C ABI of the x2dhf GB300 library: context, grid, relaxation, quadrature
// entry points and the reference-named link-compatible symbols.
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

#include "x2g_kernels.cuh"

namespace {
thread_local int g_status = 0;
thread_local std::string g_msg;
}  // namespace

namespace x2g {

int set_status(int code, const std::string &msg) {
  g_status = code;
  g_msg = msg;
  return code;
}

int cuda_status(cudaError_t e, const char *where) {
  std::string m = std::string(where) + ": " + cudaGetErrorString(e);
  (void)cudaGetLastError();
  return set_status(X2G_ERR_CUDA, m);
}

void *ctx_workspace(x2g_ctx *ctx, size_t bytes) {
  if (ctx->work_bytes < bytes) {
    if (ctx->work) {
      cudaStreamSynchronize(ctx->stream);
      cudaFree(ctx->work);
    }
    ctx->work = nullptr;
    ctx->work_bytes = 0;
    size_t want = bytes + bytes / 4;
    if (cudaMalloc(&ctx->work, want) != cudaSuccess) {
      (void)cudaGetLastError();
      return nullptr;
    }
    ctx->work_bytes = want;
  }
  return ctx->work;
}

}  // namespace x2g

using namespace x2g;

extern "C" {

int x2g_last_status(void) { return g_status; }
const char *x2g_last_error(void) { return g_msg.c_str(); }

int x2g_create(x2g_ctx **out, int device) {
  if (!out) return set_status(X2G_ERR_ARG, "null context pointer");
  *out = nullptr;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) {
    (void)cudaGetLastError();
    return set_status(X2G_ERR_NO_DEVICE, "no CUDA device available");
  }
  if (device < 0 || device >= ndev) return set_status(X2G_ERR_ARG, "device index out of range");
  if ((e = cudaSetDevice(device)) != cudaSuccess) return cuda_status(e, "cudaSetDevice");
  auto *c = new x2g_ctx();
  c->device = device;
  cudaDeviceProp prop;
  if ((e = cudaGetDeviceProperties(&prop, device)) != cudaSuccess) {
    delete c;
    return cuda_status(e, "cudaGetDeviceProperties");
  }
  if (!prop.cooperativeLaunch) {
    delete c;
    return set_status(X2G_ERR_UNSUPPORTED, "device lacks cooperative launch");
  }
  c->num_sms = prop.multiProcessorCount;
  // the context's stream at the highest priority, an auxiliary stream at
  // the lowest: work queued on the auxiliary stream fills the SMs the main
  // stream's kernels leave free (the FP64 residual of a second group of
  // potentials while the first group sweeps)
  int least = 0, greatest = 0;
  if ((e = cudaDeviceGetStreamPriorityRange(&least, &greatest)) != cudaSuccess ||
      (e = cudaStreamCreateWithPriority(&c->stream, cudaStreamNonBlocking, greatest)) != cudaSuccess) {
    delete c;
    return cuda_status(e, "cudaStreamCreate");
  }
  if ((e = cudaStreamCreateWithPriority(&c->aux, cudaStreamNonBlocking, least)) != cudaSuccess ||
      (e = cudaEventCreateWithFlags(&c->ev_split[0], cudaEventDisableTiming)) != cudaSuccess ||
      (e = cudaEventCreateWithFlags(&c->ev_split[1], cudaEventDisableTiming)) != cudaSuccess) {
    cudaStreamDestroy(c->stream);
    if (c->aux) cudaStreamDestroy(c->aux);
    if (c->ev_split[0]) cudaEventDestroy(c->ev_split[0]);
    delete c;
    return cuda_status(e, "auxiliary stream");
  }
  if ((e = cudaMalloc(&c->bar, kBarWords * sizeof(unsigned))) != cudaSuccess ||
      (e = cudaMemsetAsync(c->bar, 0, kBarWords * sizeof(unsigned), c->stream)) != cudaSuccess ||
      (e = cudaStreamSynchronize(c->stream)) != cudaSuccess) {
    cudaStreamDestroy(c->stream);
    cudaStreamDestroy(c->aux);
    cudaEventDestroy(c->ev_split[0]);
    cudaEventDestroy(c->ev_split[1]);
    delete c;
    return cuda_status(e, "barrier allocation");
  }
  c->red_bytes = size_t(608) * 16 * sizeof(double) + 64 * sizeof(double);  // most reduction blocks x partials
  if ((e = cudaMalloc(&c->red, c->red_bytes)) != cudaSuccess ||
      (e = cudaMallocHost(&c->host_red, 1024 * sizeof(double))) != cudaSuccess) {
    cudaFree(c->bar);
    cudaStreamDestroy(c->stream);
    delete c;
    return cuda_status(e, "reduction buffers");
  }
  *out = c;
  return set_status(X2G_OK, "");
}

int x2g_destroy(x2g_ctx *c) {
  if (!c) return X2G_OK;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  for (auto &p : c->pending) {
    cudaEventDestroy(p.a);
    cudaEventDestroy(p.b);
  }
  for (cudaEvent_t ev : c->event_pool) cudaEventDestroy(ev);
  if (c->work) cudaFree(c->work);
  if (c->red) cudaFree(c->red);
  if (c->bar) cudaFree(c->bar);
  if (c->host_red) cudaFreeHost(c->host_red);
  cudaStreamSynchronize(c->aux);
  cudaEventDestroy(c->ev_split[0]);
  cudaEventDestroy(c->ev_split[1]);
  cudaStreamDestroy(c->aux);
  cudaStreamDestroy(c->stream);
  delete c;
  return X2G_OK;
}

int x2g_synchronize(x2g_ctx *c) {
  if (!c) return set_status(X2G_ERR_ARG, "null context");
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_status(e, "stream synchronize");
  for (auto &p : c->pending) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
      c->prof_ms[p.precision] += ms;
      c->prof_points[p.precision] += p.points;
      c->prof_launches[p.precision] += 1;
    }
    c->event_pool.push_back(p.a);
    c->event_pool.push_back(p.b);
  }
  c->pending.clear();
  int err = 0;
  e = cudaMemcpyAsync(&err, c->bar + 2, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_status(e, "error word readback");
  count_copy(c, 0, sizeof(int));
  if (err) {
    cudaMemsetAsync(c->bar, 0, kBarWords * sizeof(unsigned), c->stream);
    return set_status(err, "device-side barrier wait timed out (kernel returned early)");
  }
  return X2G_OK;
}

void *x2g_stream(x2g_ctx *c) { return c ? (void *)c->stream : nullptr; }

int x2g_profile(x2g_ctx *c, int enable, int precision, double *ms, double *points, long *launches) {
  if (!c || precision < 0 || precision > 1) return set_status(X2G_ERR_ARG, "bad argument");
  if (enable >= 0) {
    c->profiling = enable;
    if (enable == 2) {  // reset counters
      c->prof_ms[0] = c->prof_ms[1] = 0;
      c->prof_points[0] = c->prof_points[1] = 0;
      c->prof_launches[0] = c->prof_launches[1] = 0;
      c->profiling = 1;
    }
  }
  if (ms) *ms = c->prof_ms[precision];
  if (points) *points = c->prof_points[precision];
  if (launches) *launches = c->prof_launches[precision];
  return X2G_OK;
}

long x2g_kernel_launches(x2g_ctx *c) { return c ? c->launches : 0; }

int x2g_transfer_bytes(x2g_ctx *c, long long *h2d, long long *d2h) {
  if (!c || !h2d || !d2h) return set_status(X2G_ERR_ARG, "null argument");
  *h2d = c->h2d_bytes;
  *d2h = c->d2h_bytes;
  return X2G_OK;
}

int x2g_convert_selftest(x2g_ctx *c, long n, unsigned long long seed, unsigned long long *mismatches) {
  if (!c || !mismatches || n < 0) return set_status(X2G_ERR_ARG, "bad argument");
  return convert_selftest(c, n, seed, mismatches);
}

int x2g_set_wait_limit(x2g_ctx *c, double seconds) {
  if (!c || !(seconds >= 0.0) || seconds > 3600.0) return set_status(X2G_ERR_ARG, "wait limit must be in [0, 3600] s");
  c->wait_limit_ns = (unsigned long long)(seconds * 1e9);
  return set_status(X2G_OK, "");
}

int x2g_set_mixed_on_chip(x2g_ctx *c, int on) {
  if (!c || on < 0 || on > 2) return set_status(X2G_ERR_ARG, "on must be 0, 1 or 2");
  c->no_cluster = (on == 0) ? 1 : 0;
  c->auto_band = (on == 2) ? 1 : 0;
  return X2G_OK;
}

int x2g_set_potential_clusters(x2g_ctx *c, int mode) {
  if (!c || mode < 0 || mode > 2) return set_status(X2G_ERR_ARG, "mode must be 0, 1 or 2");
  c->pot_clusters = mode;
  return X2G_OK;
}

int x2g_set_gram_orthonormalise(x2g_ctx *c, int on) {
  if (!c || on < 0 || on > 1) return set_status(X2G_ERR_ARG, "on must be 0 or 1");
  c->gram_ortho = on;
  return X2G_OK;
}

int x2g_set_residual_overlap(x2g_ctx *c, int on) {
  if (!c || on < 0 || on > 1) return set_status(X2G_ERR_ARG, "on must be 0 or 1");
  c->residual_overlap = on;
  return X2G_OK;
}

int x2g_set_mixed_colouring(x2g_ctx *c, int free) {
  if (!c || free < 0 || free > 1) return set_status(X2G_ERR_ARG, "colouring must be 0 or 1");
  c->mixed_free = free;
  return X2G_OK;
}

int x2g_round_grid(int n) {
  // nnucalc/nmucalc (inputInterface.F90:2961-3095): n = 1 (mod 6) and
  // n - 6 = 0 (mod 5) enforced alternately, always rounding down.
  if (n < 7) return 0;
  for (;;) {
    while ((n - 1) % 6 != 0) n--;
    int nt = n;
    while (((n - 6) / 5) * 5 != n - 6) n--;
    if (n > 1 && n != nt) continue;
    return n;
  }
}

int x2g_nmu_from_rinf(int nnu, double r, double rinf) {
  double hnu = kPi / double(nnu - 1);
  double x = 2.0 * rinf / r;
  x = std::log(x + std::sqrt(x * x - 1.0));
  long n = lround(x / hnu + 1.0);
  return x2g_round_grid(int(n));
}

int x2g_default_omega(int nnu, int nmu, double z1, double z2, double *oorb, double *opot) {
  double rho = 0.5 * (std::cos(kPi / double(nmu)) + std::cos(kPi / double(nnu)));
  double w = 2.0 * 0.603 / (1.0 + std::sqrt(1.0 - rho * rho)) + 0.79;
  if (opot) *opot = w;
  if (oorb) *oorb = (w - 1.0) * w - 0.001 * (z1 > z2 ? z1 : z2);
  return X2G_OK;
}

static int upload(x2g_grid *gr, const void *src, size_t bytes, const void **dst) {
  void *p = nullptr;
  cudaError_t e = cudaMalloc(&p, bytes < 16 ? 16 : bytes);
  if (e != cudaSuccess) return cuda_status(e, "grid table allocation");
  gr->allocs.push_back(p);
  // on the context's stream, whose kernels read the table (a legacy-stream
  // copy from pageable memory may return before its DMA lands, and the
  // non-blocking stream is not ordered after it); synchronised because src
  // may be freed on return
  e = cudaMemcpyAsync(p, src, bytes, cudaMemcpyHostToDevice, gr->ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(gr->ctx->stream);
  if (e != cudaSuccess) return cuda_status(e, "grid table upload");
  count_copy(gr->ctx, bytes, 0);
  *dst = p;
  return X2G_OK;
}

int x2g_grid_create(x2g_ctx *ctx, int nnu, int nmu, double r, double rinf, double z1, double z2, int mpole,
                    x2g_grid **out) {
  if (!ctx || !out) return set_status(X2G_ERR_ARG, "null argument");
  *out = nullptr;
  auto *gr = new x2g_grid();
  gr->ctx = ctx;
  std::string msg = build_host_grid(gr->h, nnu, nmu, r, rinf, z1, z2, mpole);
  if (!msg.empty()) {
    delete gr;
    return set_status(msg.rfind("schedule", 0) == 0 ? X2G_ERR_SCHEDULE : X2G_ERR_ARG, msg);
  }
  cudaSetDevice(ctx->device);
  const HostGrid &h = gr->h;
  GridDev &d = gr->d;
  d.nni = h.nni;
  d.nmu = h.nmu;
  d.n8 = h.n8;
  d.m8 = h.m8;
  d.next = h.next;
  d.mxsize = h.mxsize;
  d.ntiles = h.ntiles;
  d.nlev = h.nlev;
  d.mpole = h.mpole;
  d.r2 = h.r2;
  std::memcpy(d.dmu1, h.dmu1, sizeof d.dmu1);
  std::memcpy(d.dmu2, h.dmu2, sizeof d.dmu2);
  std::memcpy(d.dni1, h.dni1, sizeof d.dni1);
  std::memcpy(d.dni2, h.dni2, sizeof d.dni2);
  std::memcpy(d.exeven, h.exeven, sizeof d.exeven);
  for (int k = 0; k < 4; ++k) {
    d.dmu1f[k] = float(h.dmu1[k]);
    d.dmu2f[k] = float(h.dmu2[k]);
    d.dni1f[k] = float(h.dni1[k]);
    d.dni2f[k] = float(h.dni2[k]);
  }
  for (int k = 0; k < 5; ++k) d.exevenf[k] = float(h.exeven[k]);
  d.diag = h.diag;
  std::vector<float> b32(h.borb_mu.begin(), h.borb_mu.end()), p32(h.bpot_mu.begin(), h.bpot_mu.end()),
      d32(h.d_nu.begin(), h.d_nu.end());
  std::vector<double> cmo(size_t(h.nmu) * 8), cmp(size_t(h.nmu) * 8), cnu(size_t(h.nni) * 8);
  for (int mu = 0; mu < h.nmu; ++mu)
    for (int q = 0; q < 4; ++q) {
      cmo[mu * 8 + q] = h.dmu2[q] + h.borb_mu[mu] * h.dmu1[q];
      cmo[mu * 8 + 4 + q] = h.dmu2[q] - h.borb_mu[mu] * h.dmu1[q];
      cmp[mu * 8 + q] = h.dmu2[q] + h.bpot_mu[mu] * h.dmu1[q];
      cmp[mu * 8 + 4 + q] = h.dmu2[q] - h.bpot_mu[mu] * h.dmu1[q];
    }
  for (int nu = 0; nu < h.nni; ++nu)
    for (int q = 0; q < 4; ++q) {
      cnu[nu * 8 + q] = h.dni2[q] + h.d_nu[nu] * h.dni1[q];
      cnu[nu * 8 + 4 + q] = h.dni2[q] - h.d_nu[nu] * h.dni1[q];
    }
  const void *tmp;
  int rc = X2G_OK;
#define UP(vec, field)                                                                  \
  do {                                                                                  \
    if ((rc = upload(gr, vec.data(), vec.size() * sizeof(vec[0]), &tmp)) != X2G_OK) { \
      x2g_grid_destroy(gr);                                                             \
      return rc;                                                                        \
    }                                                                                   \
    d.field = static_cast<decltype(d.field)>(tmp);                                     \
  } while (0)
  UP(h.borb_mu, borb_mu);
  UP(h.bpot_mu, bpot_mu);
  UP(h.f3_mu, f3_mu);
  UP(h.e_mu, e_mu);
  UP(h.e_nu, e_nu);
  UP(h.d_nu, d_nu);
  UP(h.e, e);
  UP(h.f0, f0);
  UP(h.f1, f1);
  UP(h.f2, f2);
  UP(h.f4, f4);
  UP(h.g, g);
  UP(h.wgt1, wgt1);
  UP(h.wgt2, wgt2);
  {
    std::vector<double> wf(h.wgt2.size());
    for (size_t k = 0; k < wf.size(); ++k) wf[k] = h.wgt2[k] * h.f4[k];
    UP(wf, wf);
  }
  UP(h.leg, leg);
  UP(h.dmu9, dmu9);
  UP(h.dni9, dni9);
  UP(h.vxi, vxi);
  UP(h.vxisq, vxisq);
  UP(h.veta, veta);
  UP(h.vetasq, vetasq);
  UP(h.tile_row0, tile_row0);
  UP(h.tile_row1, tile_row1);
  UP(h.pts, pts);
  UP(h.off, off);
  UP(h.pts_rc, pts_rc);
  UP(h.st_pts, st_pts);
  UP(h.st_off, st_off);
  UP(h.sor_pts, sor_pts);
  UP(h.sor_off, sor_off);
  UP(h.sor_bpts, sor_bpts);
  UP(h.sor_boff, sor_boff);
  d.sor_nlev = h.sor_nlev;
  d.sor_nblev = h.sor_nblev;
  d.sor_delta = h.sor_delta;
  for (int k = 0; k <= HostGrid::kBandRuns; ++k) d.st_rows[k] = h.st_rows[k];
  d.cl_size = h.cl_size;
  d.cl_maxrows = h.cl_maxrows;
  d.cl_maxchunks = h.cl_maxchunks;
  d.cl_wa = h.cl_wa;
  d.cl_wb = h.cl_wb;
  d.cl_ws = h.cl_ws;
  d.cl_pa = h.cl_pa;
  d.cf_maxchunks = h.cf_maxchunks;
  d.cf_wa = h.cf_wa;
  d.cf_wb = h.cf_wb;
  d.cf_ws = h.cf_ws;
  d.cf_pa = h.cf_pa;
  d.cf_pb = h.cf_pb;
  d.cf_ps = h.cf_ps;
  d.cl_pb = h.cl_pb;
  d.cl_ps = h.cl_ps;
  if (h.cl_size > 0) {
    UP(h.cl_tile0, cl_tile0);
    UP(h.cl_row0, cl_row0);
    UP(h.cl_pts, cl_pts);
    UP(h.cl_off, cl_off);
    UP(h.cf_pts, cf_pts);
    UP(h.cf_off, cf_off);
  } else {
    d.cl_tile0 = d.cl_row0 = d.cl_pts = d.cl_off = d.cf_pts = d.cf_off = nullptr;
  }
  UP(b32, borb_mu32);
  UP(p32, bpot_mu32);
  UP(d32, d_nu32);
  UP(cmo, cmu_orb);
  UP(cmp, cmu_pot);
  UP(cnu, cnu);
#undef UP
  {
    double *exm = nullptr, *asy = nullptr;
    cudaError_t e = cudaMalloc(&exm, size_t(40) * h.mxsize * sizeof(double));
    if (e == cudaSuccess) gr->allocs.push_back(exm);
    if (e == cudaSuccess) e = cudaMalloc(&asy, size_t(51) * 4 * h.nni * sizeof(double));
    if (e == cudaSuccess) gr->allocs.push_back(asy);
    if (e != cudaSuccess) {
      rc = cuda_status(e, "moment tables");
      x2g_grid_destroy(gr);
      return rc;
    }
    d.exm = exm;
    d.asy = asy;
    if ((rc = build_moment_tables(ctx, d, exm, asy)) != X2G_OK) {
      x2g_grid_destroy(gr);
      return rc;
    }
  }
  *out = gr;
  return set_status(X2G_OK, "");
}

int x2g_grid_destroy(x2g_grid *gr) {
  if (!gr) return X2G_OK;
  cudaDeviceSynchronize();
  for (void *p : gr->allocs) cudaFree(p);
  delete gr;
  return X2G_OK;
}

int x2g_grid_table(x2g_grid *gr, int which, double *out) {
  if (!gr || !out) return set_status(X2G_ERR_ARG, "null argument");
  const HostGrid &h = gr->h;
  const int nni = h.nni, nmu = h.nmu;
  for (int i = 0; i < nmu; ++i)
    for (int j = 0; j < nni; ++j) {
      const int k = i * nni + j;
      double v;
      switch (which) {
        case 0: v = h.borb_mu[i]; break;
        case 1: v = h.bpot_mu[i]; break;
        case 2: v = h.d_nu[j]; break;
        case 3: v = h.e[k]; break;
        case 4: v = h.f0[k]; break;
        case 5: v = h.f1[k]; break;
        case 6: v = h.f2[k]; break;
        case 7: v = h.f3_mu[i]; break;
        case 8: v = h.f4[k]; break;
        case 9: v = h.g[k]; break;
        case 10: v = h.wgt1[k]; break;
        case 11: v = h.wgt2[k]; break;
        default: return set_status(X2G_ERR_ARG, "unknown table");
      }
      out[k] = v;
    }
  return X2G_OK;
}

int x2g_grid_info(x2g_grid *gr, int *nnu, int *nmu, int *ntiles, int *nlevels, int *npoints) {
  if (!gr) return set_status(X2G_ERR_ARG, "null grid");
  if (nnu) *nnu = gr->h.nni;
  if (nmu) *nmu = gr->h.nmu;
  if (ntiles) *ntiles = gr->h.ntiles;
  if (nlevels) *nlevels = gr->h.nlev;
  if (npoints) *npoints = int(gr->h.order.size());
  return X2G_OK;
}

int x2g_cluster_occupancy(x2g_ctx *ctx, x2g_grid *grid, int *plain, int *pot) {
  if (!ctx || !grid) return set_status(X2G_ERR_ARG, "null argument");
  return cluster_occupancy(ctx, grid, plain, pot);
}

int x2g_relax(x2g_ctx *ctx, x2g_grid *grid, const x2g_job *jobs, int njobs, int nsweeps, int precision) {
  if (!ctx || !grid || (!jobs && njobs > 0) || njobs < 0) return set_status(X2G_ERR_ARG, "null argument");
  if (precision != X2G_FP64 && precision != X2G_MIXED && precision != X2G_SOR)
    return set_status(X2G_ERR_ARG, "unknown precision");
  return launch_relax(ctx, grid, jobs, njobs, nsweeps, precision);
}

int x2g_putin(x2g_ctx *ctx, x2g_grid *grid, int isym, const double *fun, double *work) {
  if (!ctx || !grid || !fun || !work || (isym != 1 && isym != -1)) return set_status(X2G_ERR_ARG, "bad argument");
  launch_putin(ctx, grid->d, isym, fun, work);
  return X2G_OK;
}

int x2g_putout(x2g_ctx *ctx, x2g_grid *grid, const double *work, double *fun) {
  if (!ctx || !grid || !fun || !work) return set_status(X2G_ERR_ARG, "bad argument");
  launch_putout(ctx, grid->d, work, fun);
  return X2G_OK;
}

int x2g_mcsor_host(x2g_ctx *ctx, x2g_grid *grid, int isym, int kind, double omega, int nsweeps, double *wk2,
                   const double *lhs, const double *rhs) {
  if (!ctx || !grid || !wk2 || !lhs || !rhs) return set_status(X2G_ERR_ARG, "null argument");
  if (kind != 0 && kind != 1) return set_status(X2G_ERR_ARG, "kind must be 0 or 1");
  const GridDev &g = grid->d;
  const size_t eb = size_t(g.next) * sizeof(double), pb = size_t(g.mxsize) * sizeof(double);
  double *buf = nullptr;
  cudaError_t e = cudaMallocAsync(&buf, eb + 2 * pb, ctx->stream);
  if (e != cudaSuccess) return cuda_status(e, "mcsor buffers");
  double *du = buf, *dl = buf + g.next, *dr = dl + g.mxsize;
  cudaMemcpyAsync(du, wk2, eb, cudaMemcpyHostToDevice, ctx->stream);
  cudaMemcpyAsync(dl, lhs, pb, cudaMemcpyHostToDevice, ctx->stream);
  cudaMemcpyAsync(dr, rhs, pb, cudaMemcpyHostToDevice, ctx->stream);
  count_copy(ctx, eb + 2 * pb, eb);
  x2g_job j{};
  j.u = du;
  j.lhs = dl;
  j.rhs = dr;
  j.omega = omega;
  j.isym = isym;
  j.kind = kind;
  int rc = launch_relax(ctx, grid, &j, 1, nsweeps, X2G_FP64);
  cudaMemcpyAsync(wk2, du, eb, cudaMemcpyDeviceToHost, ctx->stream);
  cudaFreeAsync(buf, ctx->stream);
  int s = x2g_synchronize(ctx);
  return rc != X2G_OK ? rc : s;
}

int x2g_quadrature(x2g_ctx *ctx, x2g_grid *grid, int which, const double *a, const double *b, const double *c,
                   double *out) {
  if (!ctx || !grid || !a || !b || !out || (which != 2)) return set_status(X2G_ERR_ARG, "bad argument");
  TripleItem it{a, b, c};
  double *dout = static_cast<double *>(ctx->red) + size_t(160) * 16;
  launch_triples(ctx, grid->d, &it, 1, dout);
  cudaError_t e = cudaMemcpyAsync(ctx->host_red, dout, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
  if (e != cudaSuccess) return cuda_status(e, "quadrature readback");
  count_copy(ctx, 0, sizeof(double));
  int s = x2g_synchronize(ctx);
  if (s != X2G_OK) return s;
  *out = ctx->host_red[0];
  return X2G_OK;
}

}  // extern "C"
