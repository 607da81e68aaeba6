// Allocation-free shell spectrum of a caller-owned device state.
//
// Some callers cannot call cudaMalloc: code that records a CUDA graph (an
// allocation inside stream capture invalidates the capture), code running
// under a framework's caching allocator that owns all device memory, and
// latency-critical loops where the implicit synchronisation of an allocation
// is not acceptable.  vk_spectrum_noalloc serves them: the caller passes the
// state and the output buffer, and the per-block partial histograms live in
// the fixed device array below, which every GPU that loads this library holds
// until the process exits (256 x 448 doubles = 896 KiB).
#include <math.h>

#include <mutex>

#include "vk_host.h"
#include "vonkarman_gpu.h"

namespace vk {
void set_global_error(const char* msg);
}

namespace {

constexpr int kNoallocBlocks = 256;     // partial histograms (one per CTA)
constexpr int kNoallocMaxShells = 448;  // ceil(sqrt(3) * 512 / 2) + 1 = 445 fits

static __device__ __align__(256) double g_spectrum_scratch[kNoallocBlocks * kNoallocMaxShells];

// Device address of the scratch per device ordinal, valid for the CUDA
// context it was looked up in: a context torn down and created again (a
// device reset) loads the module again, possibly elsewhere, so the address is
// looked up again whenever the current context's unique id has changed.
struct ScratchAddr {
  unsigned long long ctx_id = 0;
  double* ptr = nullptr;
};
std::mutex g_scratch_mu;
ScratchAddr g_scratch_addr[64];

using CtxGetIdFn = int (*)(void* ctx, unsigned long long* id);   // cuCtxGetId

// Unique id of the current context (cuCtxGetId, reached through the runtime's
// driver entry point so that the library links only the CUDA runtime); 0 when
// no context is current yet or the driver lacks the call.
unsigned long long current_ctx_id() {
  static const CtxGetIdFn fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return reinterpret_cast<CtxGetIdFn>(p);
  }();
  unsigned long long id = 0;
  if (!fn || fn(nullptr, &id) != 0) return 0;
  return id;
}

// Set-up of the current device: the scratch's device address in the current
// context.  cudaGetSymbolAddress also loads the module into the context when
// it is not loaded yet, which is why the first call on a device should come
// before any stream capture.
cudaError_t scratch_address(int dev, double** out) {
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  ScratchAddr& a = g_scratch_addr[dev];
  const unsigned long long id = current_ctx_id();
  if (a.ptr && id != 0 && id == a.ctx_id) {
    *out = a.ptr;
    return cudaSuccess;
  }
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_spectrum_scratch);
  if (e != cudaSuccess) return e;
  if (!p) return cudaErrorInvalidSymbol;
  a.ptr = static_cast<double*>(p);
  a.ctx_id = current_ctx_id();   // the lookup made the primary context current if none was
  *out = a.ptr;
  return cudaSuccess;
}

}  // namespace

extern "C" int vk_spectrum_noalloc(const void* u_hat, int32_t n, double l, int32_t precision,
                                   double* spectrum_out, void* stream) {
  if (!u_hat || !spectrum_out) {
    vk::set_global_error("vk_spectrum_noalloc: null pointer");
    return VK_ERR_INVALID;
  }
  if (n < 8 || (n & (n - 1)) != 0 || !(l > 0.0)) {
    vk::set_global_error("vk_spectrum_noalloc: n must be a power of 2 >= 8 and l > 0");
    return VK_ERR_INVALID;
  }
  if (precision != VK_PRECISION_FP64 && precision != VK_PRECISION_FP32BULK) {
    vk::set_global_error("vk_spectrum_noalloc: bad precision");
    return VK_ERR_INVALID;
  }
  const double kmx = (double)(n / 2);
  const int nsh = (int)ceil(sqrt(kmx * kmx + kmx * kmx + kmx * kmx)) + 1;
  if (n > 512 || nsh > kNoallocMaxShells) {
    vk::set_global_error("vk_spectrum_noalloc: n > 512 exceeds the fixed scratch (448 shells)");
    return VK_ERR_UNSUPPORTED;
  }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= 64) {
    vk::set_global_error("vk_spectrum_noalloc: no usable current device");
    return VK_ERR_CUDA;
  }
  double* scratch = nullptr;
  e = scratch_address(dev, &scratch);
  if (e != cudaSuccess) {
    vk::set_global_error(cudaGetErrorString(e));
    return VK_ERR_CUDA;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t cs = (size_t)n * n * (n / 2 + 1);
  const double ks = 2.0 * 3.14159265358979323846 / l;
  e = precision == VK_PRECISION_FP64
          ? vk::Engine<double>::spectrum_partial(static_cast<const double2*>(u_hat), cs, n, ks, nsh, scratch,
                                                 kNoallocBlocks, s)
          : vk::Engine<float>::spectrum_partial(static_cast<const float2*>(u_hat), cs, n, ks, nsh, scratch,
                                                kNoallocBlocks, s);
  if (e != cudaSuccess) {
    vk::set_global_error(cudaGetErrorString(e));
    return VK_ERR_CUDA;
  }
  // the Neumaier-compensated column sum of vk_spectrum with the 1/2 and 1/N^6
  // of spectrum.rs:53 folded in; every partial row is rewritten by each call,
  // so the shared scratch needs no clearing between calls
  const double ntot = (double)n * (double)n * (double)n;
  e = vk::launch_reduce_columns(scratch, kNoallocBlocks, nsh, spectrum_out, s, 0.5 / (ntot * ntot));
  if (e != cudaSuccess) {
    vk::set_global_error(cudaGetErrorString(e));
    return VK_ERR_CUDA;
  }
  return VK_OK;
}
