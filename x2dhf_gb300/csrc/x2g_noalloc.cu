// Relaxation entry point that allocates no device memory.
//
// x2g_relax draws its job table and right-hand-side buffers from a context
// workspace that grows with cudaMalloc (after a full stream synchronisation)
// the first time a larger batch arrives.  Some callers cannot accept that:
// an SCF or serving loop that admits work against a fixed HBM budget and
// must keep its device footprint constant, or a host program (such as the
// Fortran SCF driver calling through the C ABI) that relaxes inside its
// inner loop and must not have a call stall the device or change the memory
// pool under it.  x2g_relax_noalloc serves them: its scratch is one
// file-scope device array of fixed size, reserved when the library is loaded
// on a GPU and held until the process exits.
#include <cstdio>
#include <mutex>

#include "x2g_kernels.cuh"

namespace {

// 32 MiB: barrier words, a job table and one right-hand side per
// potential, e.g. 25 potentials of a 331 x 481 grid per call.
constexpr size_t kNoAllocScratchBytes = size_t(32) << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void *g_scratch_addr[kMaxDevices] = {};

// Device address of the array for `device`, looked up once per device with
// that device current (the host-side symbol is not a device address).
int scratch_address(int device, void **out) {
  if (device < 0 || device >= kMaxDevices) return x2g::set_status(X2G_ERR_ARG, "device index out of range");
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_scratch_addr[device]) {
    int prev = 0;
    cudaError_t e = cudaGetDevice(&prev);
    if (e != cudaSuccess) return x2g::cuda_status(e, "cudaGetDevice");
    if (prev != device && (e = cudaSetDevice(device)) != cudaSuccess) return x2g::cuda_status(e, "cudaSetDevice");
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (prev != device) cudaSetDevice(prev);
    if (e != cudaSuccess) return x2g::cuda_status(e, "cudaGetSymbolAddress(no-allocation scratch)");
    g_scratch_addr[device] = p;
  }
  *out = g_scratch_addr[device];
  return X2G_OK;
}

}  // namespace

extern "C" int x2g_relax_noalloc(x2g_ctx *ctx, x2g_grid *grid, const x2g_job *jobs, int njobs, int nsweeps) {
  using namespace x2g;
  if (!ctx || !grid || !jobs) return set_status(X2G_ERR_ARG, "null argument");
  if (njobs <= 0 || nsweeps <= 0) return set_status(X2G_ERR_ARG, "njobs and nsweeps must be positive");
  const size_t need = relax_scratch_bytes(grid->d, njobs);
  if (need > kNoAllocScratchBytes) {
    char msg[200];
    std::snprintf(msg, sizeof msg,
                  "x2g_relax_noalloc: %d jobs on this grid need %zu bytes of scratch, more than its fixed %zu bytes; "
                  "split the batch or use x2g_relax",
                  njobs, need, kNoAllocScratchBytes);
    return set_status(X2G_ERR_ARG, msg);
  }
  void *scratch = nullptr;
  int rc = scratch_address(ctx->device, &scratch);
  if (rc) return rc;
  rc = launch_relax_in_scratch(ctx, grid, jobs, njobs, nsweeps, scratch, kNoAllocScratchBytes);
  if (rc) return rc;
  // wait for this call so that its barrier word can be checked and the
  // shared scratch is free for the next call
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_status(e, "stream synchronize");
  int err = 0;
  e = cudaMemcpyAsync(&err, static_cast<char *>(scratch) + 2 * sizeof(unsigned), sizeof(int), cudaMemcpyDeviceToHost,
                      ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_status(e, "scratch error word readback");
  count_copy(ctx, 0, sizeof(int));
  if (err) return set_status(err, "device-side barrier wait timed out (kernel returned early)");
  return set_status(X2G_OK, "");
}
