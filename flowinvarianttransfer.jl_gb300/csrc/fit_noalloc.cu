// Allocation-free resolved mode-to-mode transfer (fit_mode_to_mode_noalloc).
//
// Some callers cannot allocate device memory at the point where they need S(k|p): code running
// under a caller-owned memory budget or a custom allocator that forbids cudaMalloc, callers in
// the middle of latency-critical loops where an allocation would synchronise the device, and
// embedding runtimes that hand this library only the buffers they own. This entry point takes
// every input and output as a device pointer and keeps its intermediate tables (advecting
// velocity, masked giver field, effective carrier, per-chunk net sums) in one file-scope device
// array of fixed size. It never calls cudaMalloc, cudaFree, or any allocating library routine.
//
// Limits and sharing: grids of at most FIT_NOALLOC_MAX_MODES modes (32^3). The array is
// FIT_NOALLOC_SCRATCH_BYTES (6.5 MiB); every GPU that loads the library holds it until the
// process exits. All calls share it, and it keeps the previous call's contents: every entry a
// call reads is written earlier in the same call, so nothing needs clearing, but two calls that
// overlap on the GPU (different streams, or different host threads) race on the same array.
// Serialise calls per device. The array's device address is looked up once per device and kept
// for the life of the process: after cudaDeviceReset (or anything else that destroys and
// re-creates the device's primary context) the kept address is stale, so such a caller must not
// use this entry point again in that process.
#include <mutex>

#include "fit_gb300.h"
#include "fit_plan.cuh"

#define FIT_NOALLOC_MAX_MODES 32768
#define FIT_NOALLOC_CHUNKS 8
// A, F, C tables: 9 complex128 per mode; net partials: FIT_NOALLOC_CHUNKS doubles per mode.
#define FIT_NOALLOC_SCRATCH_BYTES ((size_t)FIT_NOALLOC_MAX_MODES * (9 * 16 + FIT_NOALLOC_CHUNKS * 8))

static __device__ __align__(256) unsigned char g_noalloc_scratch[FIT_NOALLOC_SCRATCH_BYTES];

namespace fit {
int triad_run_scratch(const GridDesc& g, const KTab& kt, int M, int two_thirds, int io_f64, const void* u,
                      const void* adv, int inv, int fp64, void* scratch, int nchunk, double* S, double* net,
                      cudaStream_t st);
}

// 1 when p is device (or managed) memory: the kernels dereference every array argument on the GPU.
static bool noalloc_is_device(const void* p) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();   // clear the error the call records for an unknown pointer
    return false;
  }
  return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

// Device address of the array, looked up once per device (with that device current). In host
// code the symbol itself is only a host-side stand-in, never a device address.
static int noalloc_scratch_ptr(void** out) {
  static std::mutex mu;
  static void* ptrs[64] = {nullptr};
  int dev = 0;
  FIT_CUDA_CHECK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) {
    fit_set_error("device ordinal %d out of range", dev);
    return FIT_ERR_ARG;
  }
  std::lock_guard<std::mutex> lk(mu);
  if (!ptrs[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) {
      fit_set_error("cudaGetSymbolAddress(scratch) failed: %s", cudaGetErrorString(e));
      return FIT_ERR_CUDA;
    }
    ptrs[dev] = p;
  }
  *out = ptrs[dev];
  return FIT_OK;
}

extern "C" int fit_mode_to_mode_noalloc(int nd, const int64_t* ns, int n_advected, int n_advecting, int dealias,
                                        const double* const* ks_dev, int invariant, int fp64_products, int io_f64,
                                        const void* u_hat, const void* adv_hat, double* S, double* net,
                                        void* stream) {
  if (nd < 1 || nd > 3 || ns == nullptr || ks_dev == nullptr) {
    fit_set_error("nd must be 1..3 with ns and ks given");
    return FIT_ERR_ARG;
  }
  if (n_advected < 1 || n_advected > 3 || n_advecting < nd) {
    fit_set_error("advected field needs 1..3 components and the advecting velocity >= nd components");
    return FIT_ERR_ARG;
  }
  if (dealias != 0 && dealias != 1) {
    fit_set_error("mode-to-mode triads support NoDealiasing and OrszagTwoThirds");
    return FIT_ERR_ARG;
  }
  if (invariant < 0 || invariant > 3 || (invariant == 2 && !(nd == 3 && n_advected == 3)) ||
      (invariant == 3 && !((nd == 2 || nd == 3) && n_advected == nd))) {
    fit_set_error("invariant %d is not defined for nd=%d with %d components", invariant, nd, n_advected);
    return FIT_ERR_ARG;
  }
  if (u_hat == nullptr || S == nullptr || net == nullptr) {
    fit_set_error("u_hat, S and net must be device pointers");
    return FIT_ERR_ARG;
  }
  if (adv_hat == nullptr && n_advected < nd) {
    fit_set_error("self-advection needs >= nd components (pass adv_hat)");
    return FIT_ERR_ARG;
  }
  long nm = 1;
  for (int d = 0; d < nd; ++d) {
    if (ns[d] < 1) {
      fit_set_error("grid size must be positive");
      return FIT_ERR_ARG;
    }
    nm *= (long)ns[d];
    if (nm > FIT_NOALLOC_MAX_MODES) break;
  }
  if (nm > FIT_NOALLOC_MAX_MODES) {
    fit_set_error("fit_mode_to_mode_noalloc: grid has more than %d modes (the fixed scratch limit); "
                  "use fit_mode_to_mode", FIT_NOALLOC_MAX_MODES);
    return FIT_ERR_SIZE;
  }
  // every array is read or written by the kernels: reject NULL tables and host memory up front,
  // before anything is launched
  for (int d = 0; d < nd; ++d) {
    if (ks_dev[d] == nullptr || !noalloc_is_device(ks_dev[d])) {
      fit_set_error("ks_dev[%d] must be a device pointer to the axis-%d wavenumbers", d, d);
      return FIT_ERR_ARG;
    }
  }
  const void* arrays[4] = {u_hat, adv_hat, S, net};
  const char* names[4] = {"u_hat", "adv_hat", "S", "net"};
  for (int i = 0; i < 4; ++i) {
    if (arrays[i] != nullptr && !noalloc_is_device(arrays[i])) {
      fit_set_error("%s must be a device pointer (device or managed memory)", names[i]);
      return FIT_ERR_ARG;
    }
  }
  void* scratch = nullptr;
  FIT_TRY(noalloc_scratch_ptr(&scratch));
  GridDesc g;
  g.nd = nd;
  g.padded = 0;
  for (int d = 0; d < 3; ++d) {
    g.N[d] = d < nd ? (int)ns[d] : 1;
    g.M[d] = g.N[d];
  }
  g.Mh0 = g.M[0] / 2 + 1;
  g.Ntot = nm;
  g.Mtot = nm;
  g.Mhalf = (long)g.Mh0 * g.M[1] * g.M[2];
  fit::KTab kt;
  for (int d = 0; d < 3; ++d) kt.k[d] = d < nd ? ks_dev[d] : nullptr;
  cudaStream_t st = (cudaStream_t)stream;
  FIT_TRY(fit::triad_run_scratch(g, kt, n_advected, dealias == 1, io_f64 ? 1 : 0, u_hat,
                                 adv_hat ? adv_hat : u_hat, invariant, fp64_products ? 1 : 0, scratch,
                                 FIT_NOALLOC_CHUNKS, S, net, st));
  // a stream that is being captured cannot be synchronised: then the call returns after enqueuing
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  FIT_CUDA_CHECK(cudaStreamIsCapturing(st, &cs));
  if (cs == cudaStreamCaptureStatusNone) FIT_CUDA_CHECK(cudaStreamSynchronize(st));
  return FIT_OK;
}
