// Allocation-free variant of the Davidson multi-dot reduction.
//
// Who needs it: host code that cannot call cudaMalloc while it runs — a solver
// embedded in a host application that has claimed the device memory for its own
// pool allocator and hands its plugins only buffers it allocated itself, or a
// latency-sensitive loop that cannot afford the device-wide synchronisation that
// cudaMalloc/cudaFree may cause (or an allocation that fails half-way through a
// step once the environments have filled the device).  The regular path keeps its
// reduction partials in a context-owned buffer that grows with cudaMalloc; this
// entry point takes them from a fixed array compiled into the library instead.
//
// The array is a file-scope __device__ variable: every GPU that loads the library
// holds it (kNoAllocPartials doubles) until the process exits, and all calls on a
// device share it.  Each call overwrites the partials it uses before reading them,
// so nothing has to start at zero, but two calls whose kernels overlap on the GPU
// (different streams, or concurrent host threads) race on the array.  The first
// call on a device looks up the array's device address for that device (with it
// current); a caller that captures streams makes that first call before any
// capture.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <string>

#include "../../include/mpsxx_gb300.h"
#include "kernels.hpp"

namespace mpsxx {
void set_last_error(const std::string& msg);  // message returned by mpsxx_last_error()
}

namespace {

// The multi-dot kernel writes one slot of kPartialStride doubles per CTA and uses
// at most kMaxBlocks CTAs (see multidot_blocks), so this bounds every call.
constexpr int kMaxBlocks = mpsxx::kMultidotMaxBlocks;
constexpr int kPartialStride = 100;  // up to 10 x 10 dot products per CTA
constexpr int kNoAllocPartials = kMaxBlocks * kPartialStride;
constexpr int kMaxVectors = 10;
// the slot stride and vector limit the multi-dot kernel writes and accepts
static_assert(kPartialStride == mpsxx::kMaxDot * mpsxx::kMaxDot, "partial slot stride of the multi-dot kernel");
static_assert(kMaxVectors == mpsxx::kMaxDot, "vector limit of the multi-dot kernel");

static __device__ __align__(256) double g_noalloc_partials[kNoAllocPartials];

// Device addresses of the array, one per device, found once with that device current.
constexpr int kMaxDevices = 64;
std::mutex g_mu;
double* g_addr[kMaxDevices] = {nullptr};

int fail(int code, const char* msg) {
  mpsxx::set_last_error(msg);
  return code;
}

}  // namespace

extern "C" int mpsxx_multidot_noalloc(const double* X, int nx, const double* Y, int ny, int64_t n, int64_t stride,
                                      double* out, void* stream) {
  mpsxx::set_last_error("");
  if (nx < 1 || ny < 1 || nx > kMaxVectors || ny > kMaxVectors)
    return fail(MPSXX_INVALID_ARGUMENT, "mpsxx_multidot_noalloc: at most 10 x 10 dot products per call");
  if (n < 0 || stride < n) return fail(MPSXX_INVALID_ARGUMENT, "mpsxx_multidot_noalloc: need 0 <= n <= stride");
  if (!X || !Y || !out) return fail(MPSXX_INVALID_ARGUMENT, "mpsxx_multidot_noalloc: null pointer");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return fail(MPSXX_CUDA, "mpsxx_multidot_noalloc: no usable current device");
  double* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_addr[dev]) {
      // first call on this device: resolve the array's device address (host code
      // cannot use the symbol itself as a pointer)
      void* p = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_partials);
      if (e != cudaSuccess || p == nullptr) {
        cudaGetLastError();
        return fail(MPSXX_CUDA, "mpsxx_multidot_noalloc: cudaGetSymbolAddress failed");
      }
      g_addr[dev] = static_cast<double*>(p);
    }
    scratch = g_addr[dev];
  }
  const int nblocks = mpsxx::multidot_blocks(n);
  if (nblocks > kMaxBlocks) return fail(MPSXX_INVALID_ARGUMENT, "mpsxx_multidot_noalloc: scratch too small");
  mpsxx::launch_multidot(X, nx, Y, ny, n, stride, out, scratch, nblocks, static_cast<cudaStream_t>(stream));
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(MPSXX_CUDA, "mpsxx_multidot_noalloc: kernel launch failed");
  return MPSXX_OK;
}
