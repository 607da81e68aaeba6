// Non-template kernels of a solver context and their launchers: ETD
// coefficient table, CFL update, scalar bookkeeping, column reductions and
// precision conversion.
#include "vk_reduce.cuh"

namespace vk {

// One entry of EtdCoeffs::new (etd.rs:113-135) per integer |k|^2 index m:
// lambda = -nu k^2, z = lambda dt.  The phi functions are the contour means
// of etd.rs:15-84; exp(z + cos theta_j) is evaluated as exp(z) exp(cos theta_j)
// (the second factor precomputed), shared by phi1, phi2 and phi3.  The
// denominators of phi1(z), phi2 and phi3 at a contour point w are |w|^2,
// |w^2|^2 = |w|^4 and |w^3|^2 = |w|^6, so one reciprocal serves all three
// (VK_ETD_SHARED_RCP; the FP64 pipe bounds this kernel and a division costs
// several FP64 instructions): two divisions per point instead of four, each
// term within a few ulp of the separately divided one.
#ifndef VK_ETD_SHARED_RCP
#define VK_ETD_SHARED_RCP 1
#endif
__global__ void k_etd_table(double* __restrict__ tab, int nent, double nu, double ks2,
                            const DevScalars* __restrict__ d, int force, ContourConsts cc) {
  if (!force && d->etd_recompute == 0) return;
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= nent) return;
  const double dt = d->dt;
  const double k2 = ks2 * (double)m;
  const double lambda = -nu * k2;
  const double z = lambda * dt;
  const double zh = z / 2.0;
  double p1h = 0.0, p1 = 0.0, p2 = 0.0, p3 = 0.0;
  const double ez = exp(z), ezh = exp(zh);
  for (int j = 0; j < 32; ++j) {
    const double wim = cc.sth[j];
    // phi1(z/2)
    {
      const double wre = zh + cc.cth[j];
      const double e = ezh * cc.exp_cth[j];
      const double ere = e * cc.cos_sth[j], eim = e * cc.sin_sth[j];
      const double nre = ere - 1.0, nim = eim;
      const double den = wre * wre + wim * wim;
      p1h += (nre * wre + nim * wim) / den;
    }
    const double wre = z + cc.cth[j];
    const double e = ez * cc.exp_cth[j];
    const double ere = e * cc.cos_sth[j], eim = e * cc.sin_sth[j];
    const double w2re = wre * wre - wim * wim;
    const double w2im = 2.0 * wre * wim;
#if VK_ETD_SHARED_RCP
    const double inv = 1.0 / (wre * wre + wim * wim);
    const double inv2 = inv * inv;
    {  // phi1(z)
      const double nre = ere - 1.0, nim = eim;
      p1 += (nre * wre + nim * wim) * inv;
    }
    {  // phi2(z)
      const double nre = ere - 1.0 - wre, nim = eim - wim;
      p2 += (nre * w2re + nim * w2im) * inv2;
    }
    {  // phi3(z)
      const double nre = ere - 1.0 - wre - 0.5 * w2re;
      const double nim = eim - wim - 0.5 * w2im;
      const double w3re = wre * w2re - wim * w2im;
      const double w3im = wre * w2im + wim * w2re;
      p3 += (nre * w3re + nim * w3im) * (inv2 * inv);
    }
#else
    {  // phi1(z)
      const double nre = ere - 1.0, nim = eim;
      const double den = wre * wre + wim * wim;
      p1 += (nre * wre + nim * wim) / den;
    }
    {  // phi2(z)
      const double nre = ere - 1.0 - wre, nim = eim - wim;
      const double den = w2re * w2re + w2im * w2im;
      p2 += (nre * w2re + nim * w2im) / den;
    }
    {  // phi3(z)
      const double nre = ere - 1.0 - wre - 0.5 * w2re;
      const double nim = eim - wim - 0.5 * w2im;
      const double w3re = wre * w2re - wim * w2im;
      const double w3im = wre * w2im + wim * w2re;
      const double den = w3re * w3re + w3im * w3im;
      p3 += (nre * w3re + nim * w3im) / den;
    }
#endif
  }
  p1h /= 32.0; p1 /= 32.0; p2 /= 32.0; p3 /= 32.0;
  if (fabs(zh) < 1e-300) p1h = 1.0;
  if (fabs(z) < 1e-300) { p1 = 1.0; p2 = 0.5; p3 = 1.0 / 6.0; }
  double* t = tab + (size_t)m * ETD_STRIDE;
  t[E_FULL] = ez;
  t[E_HALF] = ezh;
  t[E_A21] = p1h;
  t[E_A41] = p1;
  t[E_B1] = p1 - 3.0 * p2 + 4.0 * p3;
  t[E_B23] = 2.0 * p2 - 4.0 * p3;
  t[E_B4] = -p2 + 4.0 * p3;
  t[7] = 0.0;
}

// CFL step size on the N grid (solver.rs:180-218) and the 1% re-tabulation
// rule of Domain::step (solver.rs:383-396).  mode: 0 = step rule,
// 1 = initialise (Periodic3D::new, solver.rs:88-93), 2 = estimate only.
__global__ void k_cfl_update(DevScalars* d, double dx, double nu, double safety, int mode) {
  const double umax = sqrt(__longlong_as_double((long long)d->mx.umax2));
  // a NaN never wins the maxima (fmax drops it; the pass raises nan_flag) and
  // an infinity does: either marks the state non-finite for the host
  if (d->mx.nan_flag || !isfinite(umax)) d->nonfinite = 1;
  const double adv = umax > 1e-30 ? dx / umax : 1.0;
  const double visc = nu > 1e-30 ? dx * dx / nu : INFINITY;
  const double nd = safety * fmin(fmin(adv, visc), 0.1);
  d->cfl_dt = nd;
  if (mode == 2) return;
  if (mode == 1 || fabs(nd - d->dt) / fmax(d->dt, 1e-30) > 0.01) {
    d->dt = nd;
    d->etd_recompute = 1;
  } else {
    d->etd_recompute = 0;
  }
}

__global__ void k_reset_max(DevScalars* d) {
  d->mx.umax2 = 0ull;
  d->mx.wmax2 = 0ull;
  d->mx.nan_flag = 0;
}

__global__ void k_time_advance(DevScalars* d) { d->time += d->dt; }

// Reduce the first width columns of part[nblk][ld] column-wise in a fixed
// order into out[width] = scale * sum (Neumaier-compensated per thread, then
// a fixed pairwise tree).
__global__ void __launch_bounds__(RED_THREADS)
k_reduce_columns(const double* __restrict__ part, int nblk, int width, int ld, double scale,
                 double* __restrict__ out) {
  __shared__ double sm[RED_THREADS];
  for (int col = blockIdx.x; col < width; col += gridDim.x) {
    Neu a = {0, 0};
    for (int b = threadIdx.x; b < nblk; b += RED_THREADS) a.add(part[(size_t)b * ld + col]);
    sm[threadIdx.x] = a.val();
    __syncthreads();
    for (int s = RED_THREADS / 2; s > 0; s >>= 1) {
      if (threadIdx.x < s) sm[threadIdx.x] += sm[threadIdx.x + s];
      __syncthreads();
    }
    if (threadIdx.x == 0) out[col] = scale * sm[0];
    __syncthreads();
  }
}

// |k|^2 of mode (ix, iy, iz) as SpectralOps::new forms it
// (vonkarman-core/src/spectral_ops.rs:26-44, 51-74): k = index * (2 pi / L)
// with index n/2 mapped to -n/2, kx^2 + ky^2 + kz^2 summed left to right,
// every operation rounded once (no contraction), so the FP64 values are the
// reference's bit for bit.
__device__ __forceinline__ double k_mag_sq_of(int ix, int iy, int iz, int n, double ks) {
  const double kx = __dmul_rn((double)signed_k(ix, n), ks);
  const double ky = __dmul_rn((double)signed_k(iy, n), ks);
  const double kz = __dmul_rn((double)iz, ks);
  return __dadd_rn(__dadd_rn(__dmul_rn(kx, kx), __dmul_rn(ky, ky)), __dmul_rn(kz, kz));
}

__global__ void k_k_mag_sq(double* __restrict__ out, int n, double ks) {
  const int h = n / 2 + 1;
  const size_t total = (size_t)n * n * h;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const int iz = (int)(i % h);
    const size_t row = i / h;
    out[i] = k_mag_sq_of((int)(row / n), (int)(row % n), iz, n, ks);
  }
}

// SpectralOps::apply_viscous (spectral_ops.rs:154-175): out_c = -(nu |k|^2) u_c
// for the three components (component stride cs).
template <typename R>
__global__ void k_apply_viscous(C2<R>* __restrict__ out, const C2<R>* __restrict__ in, int n, size_t cs, double ks,
                                double nu) {
  const int h = n / 2 + 1;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < cs; i += (size_t)gridDim.x * blockDim.x) {
    const int iz = (int)(i % h);
    const size_t row = i / h;
    const R f = (R)(-__dmul_rn(nu, k_mag_sq_of((int)(row / n), (int)(row % n), iz, n, ks)));
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const C2<R> v = in[c * cs + i];
      out[c * cs + i] = cmk<R>(f * v.x, f * v.y);
    }
  }
}

// complex precision conversion (host state is always f64)
template <typename RO, typename RI>
__global__ void k_convert(C2<RO>* __restrict__ out, const C2<RI>* __restrict__ in, size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const C2<RI> v = in[i];
    out[i] = cmk<RO>((RO)v.x, (RO)v.y);
  }
}

template <typename RO, typename RI>
__global__ void k_convert_real(RO* __restrict__ out, const RI* __restrict__ in, size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    out[i] = (RO)in[i];
}


cudaError_t launch_etd_table(double* tab, int nent, double nu, double ks2, const DevScalars* d, int force,
                             const ContourConsts& cc, cudaStream_t s) {
  const int nt = 128;
  k_etd_table<<<(nent + nt - 1) / nt, nt, 0, s>>>(tab, nent, nu, ks2, d, force, cc);
  return cudaGetLastError();
}

cudaError_t launch_cfl_update(DevScalars* d, double dx, double nu, double safety, int mode, cudaStream_t s) {
  k_cfl_update<<<1, 1, 0, s>>>(d, dx, nu, safety, mode);
  return cudaGetLastError();
}

cudaError_t launch_reset_max(DevScalars* d, cudaStream_t s) {
  k_reset_max<<<1, 1, 0, s>>>(d);
  return cudaGetLastError();
}

cudaError_t launch_time_advance(DevScalars* d, cudaStream_t s) {
  k_time_advance<<<1, 1, 0, s>>>(d);
  return cudaGetLastError();
}

cudaError_t launch_reduce_columns(const double* part, int nblk, int width, double* out, cudaStream_t s,
                                  double scale, int ld) {
  const int nb = width < 1024 ? width : 1024;
  k_reduce_columns<<<nb, RED_THREADS, 0, s>>>(part, nblk, width, ld > 0 ? ld : width, scale, out);
  return cudaGetLastError();
}

static int conv_blocks(size_t n) {
  const size_t nb = (n + 255) / 256;
  return (int)(nb < 65536 ? nb : 65536);
}

cudaError_t launch_k_mag_sq(double* out, int n, double ks, cudaStream_t s) {
  k_k_mag_sq<<<conv_blocks((size_t)n * n * (n / 2 + 1)), 256, 0, s>>>(out, n, ks);
  return cudaGetLastError();
}

cudaError_t launch_apply_viscous(void* out, const void* in, int fp32, int n, size_t cs, double ks, double nu,
                                 cudaStream_t s) {
  if (fp32)
    k_apply_viscous<float><<<conv_blocks(cs), 256, 0, s>>>((float2*)out, (const float2*)in, n, cs, ks, nu);
  else
    k_apply_viscous<double><<<conv_blocks(cs), 256, 0, s>>>((double2*)out, (const double2*)in, n, cs, ks, nu);
  return cudaGetLastError();
}

cudaError_t launch_convert_c(void* out, int out_fp32, const void* in, int in_fp32, size_t n, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  const int nb = conv_blocks(n);
  if (out_fp32 && !in_fp32)
    k_convert<float, double><<<nb, 256, 0, s>>>((float2*)out, (const double2*)in, n);
  else if (!out_fp32 && in_fp32)
    k_convert<double, float><<<nb, 256, 0, s>>>((double2*)out, (const float2*)in, n);
  else
    return cudaMemcpyAsync(out, in, n * (out_fp32 ? sizeof(float2) : sizeof(double2)), cudaMemcpyDeviceToDevice, s);
  return cudaGetLastError();
}

cudaError_t launch_convert_r(void* out, int out_fp32, const void* in, int in_fp32, size_t n, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  const int nb = conv_blocks(n);
  if (out_fp32 && !in_fp32)
    k_convert_real<float, double><<<nb, 256, 0, s>>>((float*)out, (const double*)in, n);
  else if (!out_fp32 && in_fp32)
    k_convert_real<double, float><<<nb, 256, 0, s>>>((double*)out, (const float*)in, n);
  else
    return cudaMemcpyAsync(out, in, n * (out_fp32 ? sizeof(float) : sizeof(double)), cudaMemcpyDeviceToDevice, s);
  return cudaGetLastError();
}

template <typename T>
__global__ void k_fma_probe(T* out, int iters, T a, T b) {
  T x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = x0 * a + b; x1 = x1 * a + b; x2 = x2 * a + b; x3 = x3 * a + b;
    x4 = x4 * a + b; x5 = x5 * a + b; x6 = x6 * a + b; x7 = x7 * a + b;
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

template <typename T>
static cudaError_t fma_peak(double* gflops) {
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
  const int blocks = sms * 8, threads = 256, iters = sizeof(T) == 8 ? 2048 : 32768;
  T* out = nullptr;
  if ((e = cudaMalloc(&out, sizeof(T) * blocks * threads)) != cudaSuccess) return e;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_fma_probe<T><<<blocks, threads>>>(out, 64, (T)0.999, (T)0.001);
  float best = 1e30f;
  for (int r = 0; r < 5; ++r) {
    cudaEventRecord(e0);
    k_fma_probe<T><<<blocks, threads>>>(out, iters, (T)0.999, (T)0.001);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  e = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  *gflops = 2.0 * 8.0 * (double)iters * blocks * threads / (best * 1e6);
  return e;
}

cudaError_t probe_fma_peak(int fp64, double* gflops) {
  return fp64 ? fma_peak<double>(gflops) : fma_peak<float>(gflops);
}

}  // namespace vk
