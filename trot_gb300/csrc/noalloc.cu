// Allocation-free local energy.
//
// Some callers of this library cannot allocate device memory for scratch:
// an XLA/JAX custom call runs inside a process where XLA has already
// pre-allocated most of the GPU for its own pool (trot's own configuration
// sets XLA_PYTHON_CLIENT_MEM_FRACTION), so a cudaMalloc issued behind XLA's
// back can fail or starve it, and a handler that has no scratch-allocator
// plumbing has nowhere else to get memory from; other callers run under a
// fixed memory budget or must not call the CUDA allocator at all on their hot
// path.  trot_local_energy_noalloc serves them: the caller passes only its
// inputs and outputs, and the scratch the energy kernels need (half Green's
// functions, force bias, exchange partial sums) lives in one file-scope
// device array of fixed size, reserved once per GPU when the library's
// device code is loaded and held until the process exits.
//
// Contract:
//  * at most kNoAllocScratchBytes (32 MiB) of scratch; larger systems are
//    rejected with TROT_ERR_WORKSPACE_TOO_SMALL (use trot_local_energy with a
//    caller workspace instead);
//  * a call outside stream capture looks up the array's device address with
//    cudaGetSymbolAddress on the current device and caches it; a call under
//    capture uses the cached address, so the first call on each device must
//    come before any stream capture begins.  Under CUDA's lazy module loading
//    (the default) that first lookup also loads the library's device code and
//    so reserves the 32 MiB on that device: make it before a framework
//    pre-allocates the GPU's memory, or set CUDA_MODULE_LOADING=EAGER.  After
//    cudaDeviceReset (or any destruction of the primary context) the next call
//    outside capture resolves the address again;
//  * every call on a device shares the same array and leaves its contents
//    behind.  The array starts zero-filled; each call writes every scratch
//    value it reads, except the status block at its start: int 0 is reset by
//    each call and int 3 keeps a sticky record of device timeouts, which
//    trot_local_energy_noalloc_status reads (and clears).  A mixed-precision
//    call whose tensor-core kernel timed out returns NaN energies, never stale
//    numbers.  Calls whose kernels overlap on the GPU (different streams, or
//    different host threads without ordering) race on the array: order them
//    on one stream;
//  * nothing here calls cudaMalloc, cudaFree or any allocating routine.
#include <mutex>

#include "kernels.h"

namespace trot {
namespace {

constexpr size_t kNoAllocScratchBytes = size_t(32) << 20;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_setup_mu;
void* g_scratch_addr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device: looked up again
// whenever `stream` is not capturing (so a re-created context is followed), the
// cached value under capture.
int scratch_for_current_device(cudaStream_t stream, void** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_status(e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) {
    set_error("device ordinal %d outside the %d devices the no-alloc scratch table covers", dev, kMaxDevices);
    return TROT_ERR_UNSUPPORTED;
  }
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  e = cudaStreamIsCapturing(stream, &cap);
  if (e != cudaSuccess) return cuda_status(e, "cudaStreamIsCapturing");
  std::lock_guard<std::mutex> lk(g_setup_mu);
  if (cap == cudaStreamCaptureStatusNone) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_status(e, "cudaGetSymbolAddress(no-alloc scratch)");
    g_scratch_addr[dev] = p;
  } else if (g_scratch_addr[dev] == nullptr) {
    set_error("trot_local_energy_noalloc: first call on device %d is under stream capture; make one call "
              "before capturing", dev);
    return TROT_ERR_UNSUPPORTED;
  }
  *out = g_scratch_addr[dev];
  return TROT_OK;
}

}  // namespace
}  // namespace trot

extern "C" int trot_local_energy_noalloc(const trot_system* sys, const double* walkers_a, const double* walkers_b,
                                         double* energy_out, void* stream) {
  using namespace trot;
  const size_t need = trot_workspace_size(sys, TROT_OP_LOCAL_ENERGY);
  // need == 0 means the system failed validation: let the workspace entry point
  // report the precise status and message (it validates before launching anything)
  if (need == 0) return trot_local_energy(sys, walkers_a, walkers_b, energy_out, nullptr, 0, stream);
  if (need > kNoAllocScratchBytes) {
    set_error("trot_local_energy_noalloc: this system needs %zu bytes of scratch but the built-in scratch "
              "array holds %zu bytes; call trot_local_energy with a caller workspace",
              need, kNoAllocScratchBytes);
    return TROT_ERR_WORKSPACE_TOO_SMALL;
  }
  void* scratch = nullptr;
  int rc = scratch_for_current_device((cudaStream_t)stream, &scratch);
  if (rc != TROT_OK) return rc;
  return trot_local_energy(sys, walkers_a, walkers_b, energy_out, scratch, kNoAllocScratchBytes, stream);
}

extern "C" int trot_local_energy_noalloc_status(int clear, int* status_out) {
  using namespace trot;
  if (!status_out) { set_error("null pointer"); return TROT_ERR_NULL_PTR; }
  void* scratch = nullptr;
  int rc = scratch_for_current_device((cudaStream_t)0, &scratch);
  if (rc != TROT_OK) return rc;
  return trot_workspace_timeouts(scratch, clear, status_out);
}
