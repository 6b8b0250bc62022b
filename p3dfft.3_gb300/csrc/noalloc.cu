// Allocation-free variant of the 3D transform executor.
//
// Some callers cannot call cudaMalloc: applications that hand all device memory to their own
// allocator at start-up, real-time loops that may not take cudaMalloc's implicit device
// synchronisation, or plugin hosts that forbid device allocations by their plugins.  For them,
// p3dfft_gb300_exec3d_noalloc runs a 3D plan with the intermediate fields and the twiddle tables
// held in the file-scope device array below instead of library-allocated buffers.
//
// The array is P3DFFT_GB300_NOALLOC_BYTES long and every GPU that loads the library holds it
// until the process exits.  All calls share it and it keeps the last call's contents; calls
// that overlap on the GPU (different streams, or several host threads) race on it.  The twiddle
// tables reach it through the static host array g_tw_host, which the next call overwrites, so
// calls on a capturing stream are refused (a replayed graph would copy the host array as it is
// at replay time).
#include <cuda_runtime.h>

#include <cstddef>
#include <mutex>

#include "kernels.h"
#include "p3dfft_gb300.h"

namespace p3d {
int exec_plan_given_memory(int plan, const void *in, void *out, int idir, void *scratch0, void *scratch1,
                           size_t scratch_bytes, void *tw_dev, size_t tw_bytes, void *tw_host);
void record_error(int code, const char *msg);
}  // namespace p3d

namespace {

constexpr size_t kTwBytes = size_t(1) << 20;                              // twiddle-table region
constexpr size_t kScratchBytes = (P3DFFT_GB300_NOALLOC_BYTES - kTwBytes) / 2;  // per intermediate field

__device__ __align__(256) unsigned char g_noalloc_scratch[P3DFFT_GB300_NOALLOC_BYTES];

// Device address of g_noalloc_scratch, looked up once per device with that device current.
constexpr int kMaxDevices = 64;
void *g_scratch_ptr[kMaxDevices] = {nullptr};
std::mutex g_setup_mu;

// Host staging for the twiddle tables (static storage: no heap use on this path)
unsigned char g_tw_host[kTwBytes];
std::mutex g_call_mu;

int scratch_for_current_device(void **ptr) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return p3d::E_NO_DEVICE;
  }
  std::lock_guard<std::mutex> g(g_setup_mu);
  if (!g_scratch_ptr[dev]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      return p3d::E_CUDA;
    }
    g_scratch_ptr[dev] = p;
  }
  *ptr = g_scratch_ptr[dev];
  return p3d::E_OK;
}

}  // namespace

extern "C" int p3dfft_gb300_exec3d_noalloc(int plan, const void *in, void *out, int idir) {
  void *base = nullptr;
  int rc = scratch_for_current_device(&base);
  if (rc != p3d::E_OK) {
    p3d::record_error(rc, "exec3d_noalloc: cannot resolve the static scratch array on the current device");
    return rc;
  }
  unsigned char *b = static_cast<unsigned char *>(base);
  std::lock_guard<std::mutex> g(g_call_mu);  // one host thread at a time uses the host staging area
  return p3d::exec_plan_given_memory(plan, in, out, idir, b + kTwBytes, b + kTwBytes + kScratchBytes, kScratchBytes,
                                     b, kTwBytes, g_tw_host);
}

extern "C" long long p3dfft_gb300_noalloc_max_field_bytes(void) { return (long long)kScratchBytes; }
