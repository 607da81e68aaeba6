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

std::mutex g_scratch_mu;
double* g_scratch_addr[64] = {};  // device address of the scratch, per device ordinal

// One CTA per shell: fixed-order sum of the nblk partials of that shell, then
// the 1/2 and 1/N^6 of spectrum.rs:53.  Every partial is rewritten by each
// call, so the shared scratch needs no clearing between calls.
__global__ void __launch_bounds__(256)
k_noalloc_spectrum_finish(const double* __restrict__ part, int nblk, int nsh, double scale,
                          double* __restrict__ out) {
  __shared__ double sm[256];
  const int col = blockIdx.x;
  double s = 0.0;
  for (int b = threadIdx.x; b < nblk; b += 256) s += part[(size_t)b * nsh + col];
  sm[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) sm[threadIdx.x] += sm[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[col] = scale * sm[0];
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
  {
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_addr[dev]) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_spectrum_scratch);
      if (e != cudaSuccess || !p) {
        vk::set_global_error(cudaGetErrorString(e));
        return VK_ERR_CUDA;
      }
      g_scratch_addr[dev] = static_cast<double*>(p);
    }
    scratch = g_scratch_addr[dev];
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
  const double ntot = (double)n * (double)n * (double)n;
  k_noalloc_spectrum_finish<<<nsh, 256, 0, s>>>(scratch, kNoallocBlocks, nsh, 0.5 / (ntot * ntot), spectrum_out);
  e = cudaGetLastError();
  if (e != cudaSuccess) {
    vk::set_global_error(cudaGetErrorString(e));
    return VK_ERR_CUDA;
  }
  return VK_OK;
}
