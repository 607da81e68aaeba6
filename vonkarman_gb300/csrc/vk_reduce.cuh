// Reductions over the spectral state that are instantiated per precision:
// Tier-1 sums and shell-spectrum partials.
#pragma once

#include "vk_kernels.cuh"

namespace vk {

// ---------------------------------------------------------------------------
// Tier-1 sums (solver.rs:412-535) with the R2C weights w(iz) = 1 at iz in
// {0, N/2}, else 2.  Per-thread Neumaier-compensated accumulation, then a
// fixed-order pairwise tree in the CTA and a fixed-order final reduction, so
// results are deterministic for a given launch shape.
// ---------------------------------------------------------------------------
struct Neu {
  double s, c;
  __device__ __forceinline__ void add(double x) {
    const double t = s + x;
    c += fabs(s) >= fabs(x) ? (s - t) + x : (x - t) + s;
    s = t;
  }
  __device__ __forceinline__ double val() const { return s + c; }
};

template <typename R>
__global__ void __launch_bounds__(RED_THREADS)
k_tier1_partial(const C2<R>* __restrict__ u, size_t cs, int N, int H, double ks, double* __restrict__ part) {
  Neu acc[4] = {{0, 0}, {0, 0}, {0, 0}, {0, 0}};
  const size_t total = (size_t)N * N * H;
  for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (size_t)gridDim.x * blockDim.x) {
    const int z = (int)(idx % H);
    const int iy = (int)((idx / H) % N);
    const int ix = (int)(idx / ((size_t)H * N));
    const double kx = (double)signed_k(ix, N) * ks, ky = (double)signed_k(iy, N) * ks, kz = (double)z * ks;
    const double w = (z == 0 || z == N / 2) ? 1.0 : 2.0;
    double ur[3], ui[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) { const C2<R> v = u[c * cs + idx]; ur[c] = v.x; ui[c] = v.y; }
    // omega = i k x u  (spectral_ops.rs:92-104)
    const double o_r[3] = {-(ky * ui[2] - kz * ui[1]), -(kz * ui[0] - kx * ui[2]), -(kx * ui[1] - ky * ui[0])};
    const double o_i[3] = {ky * ur[2] - kz * ur[1], kz * ur[0] - kx * ur[2], kx * ur[1] - ky * ur[0]};
    const double c_r[3] = {-(ky * o_i[2] - kz * o_i[1]), -(kz * o_i[0] - kx * o_i[2]), -(kx * o_i[1] - ky * o_i[0])};
    const double c_i[3] = {ky * o_r[2] - kz * o_r[1], kz * o_r[0] - kx * o_r[2], kx * o_r[1] - ky * o_r[0]};
    double e = 0, en = 0, he = 0, sh = 0;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      e += ur[c] * ur[c] + ui[c] * ui[c];
      en += o_r[c] * o_r[c] + o_i[c] * o_i[c];
      he += ur[c] * o_r[c] + ui[c] * o_i[c];
      sh += o_r[c] * c_r[c] + o_i[c] * c_i[c];
    }
    acc[0].add(w * e); acc[1].add(w * en); acc[2].add(w * he); acc[3].add(w * sh);
  }
  __shared__ double sm[4][RED_THREADS];
#pragma unroll
  for (int j = 0; j < 4; ++j) sm[j][threadIdx.x] = acc[j].val();
  __syncthreads();
  for (int s = RED_THREADS / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
#pragma unroll
      for (int j = 0; j < 4; ++j) sm[j][threadIdx.x] += sm[j][threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x < 4) part[(size_t)blockIdx.x * 4 + threadIdx.x] = sm[threadIdx.x][0];
}

// Shell spectrum partials (vonkarman-diag/src/spectrum.rs:13-60): shell =
// round(|k|) with |k| evaluated without contraction, as the reference does.
template <typename R>
__global__ void __launch_bounds__(RED_THREADS)
k_spectrum_partial(const C2<R>* __restrict__ u, size_t cs, int N, int H, double ks, int nsh,
                   double* __restrict__ part) {
  extern __shared__ __align__(16) unsigned char vk_smem[];
  double* hist = reinterpret_cast<double*>(vk_smem);
  for (int i = threadIdx.x; i < nsh; i += blockDim.x) hist[i] = 0.0;
  __syncthreads();
  const size_t total = (size_t)N * N * H;
  for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (size_t)gridDim.x * blockDim.x) {
    const int z = (int)(idx % H);
    const int iy = (int)((idx / H) % N);
    const int ix = (int)(idx / ((size_t)H * N));
    const double kx = __dmul_rn((double)signed_k(ix, N), ks);
    const double ky = __dmul_rn((double)signed_k(iy, N), ks);
    const double kz = __dmul_rn((double)z, ks);
    const double kk = __dadd_rn(__dadd_rn(__dmul_rn(kx, kx), __dmul_rn(ky, ky)), __dmul_rn(kz, kz));
    const int shell = (int)round(sqrt(kk));
    if (shell >= nsh) continue;
    double m2 = 0.0;
#pragma unroll
    for (int c = 0; c < 3; ++c) { const C2<R> v = u[c * cs + idx]; m2 += (double)v.x * v.x + (double)v.y * v.y; }
    const double w = (z == 0 || z == N / 2) ? 1.0 : 2.0;
    atomicAdd(&hist[shell], w * m2);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nsh; i += blockDim.x) part[(size_t)blockIdx.x * nsh + i] = hist[i];
}

}  // namespace vk
