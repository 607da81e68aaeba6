// Reductions over the spectral state that are instantiated per precision:
// Tier-1 sums and shell-spectrum partials.
#pragma once

#include "vk_kernels.cuh"

namespace vk {

// ---------------------------------------------------------------------------
// Tier-1 sums (solver.rs:412-535) with the R2C weights w(iz) = 1 at iz in
// {0, N/2}, else 2.  Per-mode quantities in the working precision R (the
// FP32-bulk form evaluates its products in FP32, the FP64 form in FP64); every
// thread sums its modes in FP64 (at most a few hundred terms at the launch
// sizes used), the CTA adds its threads in a fixed pairwise tree and the
// column reduction adds the CTAs with Neumaier compensation, so results are
// deterministic for a given launch shape.  Grid sizes are template constants
// (index decomposition without runtime division; N^2 (N/2 + 1) < 2^31).
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

// Per-mode Tier-1 terms of one mode in the working precision R: |u|^2,
// |omega|^2, Re(u . conj omega), Re(omega . conj(i k x omega)) with
// omega = i k x u (spectral_ops.rs:92-104, solver.rs:412-535).  Shared by the
// separate reduction pass and the one fused into the final stage epilogue.
template <typename R>
__device__ __forceinline__ void tier1_terms(R kx, R ky, R kz, const C2<R>* uv, R& e, R& en, R& he, R& sh) {
  R ur[3], ui[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) { ur[c] = uv[c].x; ui[c] = uv[c].y; }
  const R o_r[3] = {-(ky * ui[2] - kz * ui[1]), -(kz * ui[0] - kx * ui[2]), -(kx * ui[1] - ky * ui[0])};
  const R o_i[3] = {ky * ur[2] - kz * ur[1], kz * ur[0] - kx * ur[2], kx * ur[1] - ky * ur[0]};
  const R c_r[3] = {-(ky * o_i[2] - kz * o_i[1]), -(kz * o_i[0] - kx * o_i[2]), -(kx * o_i[1] - ky * o_i[0])};
  const R c_i[3] = {ky * o_r[2] - kz * o_r[1], kz * o_r[0] - kx * o_r[2], kx * o_r[1] - ky * o_r[0]};
  e = 0; en = 0; he = 0; sh = 0;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    e += ur[c] * ur[c] + ui[c] * ui[c];
    en += o_r[c] * o_r[c] + o_i[c] * o_i[c];
    he += ur[c] * o_r[c] + ui[c] * o_i[c];
    sh += o_r[c] * c_r[c] + o_i[c] * c_i[c];
  }
}

// |u|^2 of one mode for the shell spectrum, in R.
template <typename R>
__device__ __forceinline__ R spectrum_term(const C2<R>* uv) {
  R m2 = 0;
#pragma unroll
  for (int c = 0; c < 3; ++c) m2 += uv[c].x * uv[c].x + uv[c].y * uv[c].y;
  return m2;
}

template <typename R, int N>
__global__ void __launch_bounds__(RED_THREADS)
k_tier1_partial(const C2<R>* __restrict__ u, size_t cs, double ks, double* __restrict__ part) {
  constexpr int H = N / 2 + 1;
  constexpr int TOTAL = N * N * H;
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  const R kr = (R)ks;
  for (int idx = blockIdx.x * RED_THREADS + threadIdx.x; idx < TOTAL; idx += gridDim.x * RED_THREADS) {
    const int z = idx % H;
    const int row = idx / H;
    const int iy = row % N, ix = row / N;
    const R kx = (R)signed_k(ix, N) * kr, ky = (R)signed_k(iy, N) * kr, kz = (R)z * kr;
    C2<R> uv[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) uv[c] = u[c * cs + idx];
    R e, en, he, sh;
    tier1_terms<R>(kx, ky, kz, uv, e, en, he, sh);
    const R w = (z == 0 || z == N / 2) ? R(1) : R(2);   // exact in R
    acc[0] += (double)(w * e); acc[1] += (double)(w * en); acc[2] += (double)(w * he); acc[3] += (double)(w * sh);
  }
  __shared__ double sm[4][RED_THREADS];
#pragma unroll
  for (int j = 0; j < 4; ++j) sm[j][threadIdx.x] = acc[j];
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

// Shell of a mode (vonkarman-diag/src/spectrum.rs:13-60): round(|k|) with
// |k| evaluated in FP64 without contraction, as the reference does.  With
// ks == 1 (box length 2 pi) |k|^2 is the integer m = kx^2 + ky^2 + kz^2
// exactly, sqrt(m) is never a half-integer, and round(sqrt(m)) = s is decided
// by the integer test (2s - 1)^2 <= 4m < (2s + 1)^2 around an FP32 estimate.
__device__ __forceinline__ int shell_of(int kxi, int kyi, int z, double ks, bool ks_one) {
  if (ks_one) {
    const int m = kxi * kxi + kyi * kyi + z * z;
    int s = (int)(sqrtf((float)m) + 0.5f);
    if ((2 * s + 1) * (2 * s + 1) <= 4 * m) ++s;
    if (s > 0 && (2 * s - 1) * (2 * s - 1) > 4 * m) --s;
    return s;
  }
  const double kx = __dmul_rn((double)kxi, ks);
  const double ky = __dmul_rn((double)kyi, ks);
  const double kz = __dmul_rn((double)z, ks);
  const double kk = __dadd_rn(__dadd_rn(__dmul_rn(kx, kx), __dmul_rn(ky, ky)), __dmul_rn(kz, kz));
  return (int)round(sqrt(kk));
}

// Shell spectrum partials: per-mode |u|^2 in R, per-CTA FP64 histograms in
// shared memory, one partial row per CTA.
template <typename R, int N>
__global__ void __launch_bounds__(RED_THREADS)
k_spectrum_partial(const C2<R>* __restrict__ u, size_t cs, double ks, int nsh, double* __restrict__ part) {
  constexpr int H = N / 2 + 1;
  constexpr int TOTAL = N * N * H;
  extern __shared__ __align__(16) unsigned char vk_smem[];
  double* hist = reinterpret_cast<double*>(vk_smem);
  for (int i = threadIdx.x; i < nsh; i += blockDim.x) hist[i] = 0.0;
  __syncthreads();
  const bool ks_one = ks == 1.0;
  for (int idx = blockIdx.x * RED_THREADS + threadIdx.x; idx < TOTAL; idx += gridDim.x * RED_THREADS) {
    const int z = idx % H;
    const int row = idx / H;
    const int iy = row % N, ix = row / N;
    const int shell = shell_of(signed_k(ix, N), signed_k(iy, N), z, ks, ks_one);
    if (shell >= nsh) continue;
    C2<R> uv[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) uv[c] = u[c * cs + idx];
    const R m2 = spectrum_term<R>(uv);
    const R w = (z == 0 || z == N / 2) ? R(1) : R(2);   // exact in R
    atomicAdd(&hist[shell], (double)(w * m2));
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nsh; i += blockDim.x) part[(size_t)blockIdx.x * nsh + i] = hist[i];
}

}  // namespace vk
