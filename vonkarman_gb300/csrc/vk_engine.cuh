// Host-side launchers: map runtime grid sizes onto the compile-time kernel
// instances.  Instantiated once per precision (vk_engine_f64.cu,
// vk_engine_f32.cu) so the two compile in parallel.
#pragma once

#include <algorithm>
#include <atomic>
#include <type_traits>

#include "vk_adjoint.cuh"
#include "vk_lines.cuh"
#include "vk_p3f.cuh"
#include "vk_tma.cuh"

// P1 with its input tiles staged in shared memory by the tensor-memory
// accelerator (k_lines_tma) instead of direct loads (k_lines)
#ifndef VK_P1_TMA
#define VK_P1_TMA 0
#endif
// L2 prefetch of the inputs one residency wave ahead in the x-inverse passes
// (P1, NX: the op supplies prefetch_row) and in the FP32 z passes (k_p3f,
// k_p3, k_nz_max)
#ifndef VK_LINES_PREFETCH
#define VK_LINES_PREFETCH 1
#endif
#ifndef VK_P3F_PREFETCH
#define VK_P3F_PREFETCH 1
#endif
#include "vk_reduce.cuh"

namespace vk {

// column pairs per CTA of the fused FP32 P3 (k_p3f; 2 measured faster than 4)
constexpr int P3F_CP = 2;


// Per-device cache of the dynamic shared memory opt-in (one bit per device
// below 64, one cache per kernel instance).  Kernels with static shared
// memory as well need the opt-in below 48 KB of dynamic memory too, so any
// sizeable request opts in.
// The mask is atomic: contexts on several host threads (and the
// allocation-free entry point, from any thread) share these instances.
template <auto KERN>
inline cudaError_t prepare_kernel(size_t smem) {
  static std::atomic<unsigned long long> done_mask{0ull};
  if (smem <= 16 * 1024) return cudaSuccess;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const unsigned long long bit = dev < 64 ? (1ull << dev) : 0ull;
  if (bit && (done_mask.load(std::memory_order_acquire) & bit)) return cudaSuccess;
  e = cudaFuncSetAttribute(KERN, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess) done_mask.fetch_or(bit, std::memory_order_acq_rel);
  return e;
}


// Register-resident strided pass (k_lines): nouter * hz lines per field in
// tiles of NLINES.
// Lines per CTA: 8 (row segments of 64 bytes in FP32, 128 in FP64), and 16
// for FP32 passes up to Op::MAX_L16 points (default 512; 384 for the x
// passes and for ops with paired raw loads, beyond which the 16-line kernels
// spill; 0 for ops that always take 8).
template <class Op, class = void> struct OpMaxL16 { static constexpr int value = 512; };
template <class Op> struct OpMaxL16<Op, std::void_t<decltype(Op::MAX_L16)>> {
  static constexpr int value = Op::MAX_L16;
};
template <typename R, int L, bool XAXIS, class Op> struct NLof {
  static constexpr int LMAX = XAXIS ? cmin(384, OpMaxL16<Op>::value) : OpMaxL16<Op>::value;
  static constexpr int value = (sizeof(R) == 4 && L <= LMAX) ? 16 : 8;
};

// One residency wave of kernel instance KERN on the current device (resident
// CTAs per SM at nt threads and smem bytes, times the SMs): the L2 prefetch
// distance of the passes that hint a later CTA's inputs.  Cached per device,
// as prepare_kernel's opt-in is (0 when a query fails).
template <auto KERN>
inline int wave_blocks(int nt, size_t smem) {
  static std::atomic<int> cache[64];   // wave + 1 once known
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (dev < 64) {
    const int v = cache[dev].load(std::memory_order_relaxed);
    if (v > 0) return v - 1;
  }
  int per_sm = 0, sms = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, KERN, nt, smem) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return 0;
  const int w = per_sm * sms;
  if (dev < 64) cache[dev].store(w + 1, std::memory_order_relaxed);
  return w;
}

// L2 prefetch distance of the FP32 column-pair z passes (k_p3, k_nz_max,
// k_adj_z): one residency wave (0 = off, and for FP64, whose passes the FP64
// pipe bounds)
template <typename R, auto KERN>
inline int zpass_prefetch_distance(int nt, size_t smem) {
  return sizeof(R) == 4 && VK_P3F_PREFETCH ? wave_blocks<KERN>(nt, smem) : 0;
}

template <typename R, int L, bool INV, bool XAXIS = false, class Op>
inline cudaError_t launch_lines(const Op& op, int nouter, const C2<R>* tw, cudaStream_t s) {
  constexpr int NLINES = NLof<R, L, XAXIS, Op>::value;
  constexpr int NT = cmin(rthreads<R, L, NLINES>(), 384);
  const size_t smem = (size_t)rsmem_elems<R, L, NLINES>() * sizeof(C2<R>);
  constexpr auto kern = k_lines<R, L, INV, NLINES, NT, Op>;
  cudaError_t e = prepare_kernel<kern>(smem);
  if (e != cudaSuccess) return e;
  const int nlines = nouter * op.hz;
  const int ntiles = (nlines + NLINES - 1) / NLINES;
  // L2 prefetch one residency wave ahead
  const int pf = VK_LINES_PREFETCH ? wave_blocks<kern>(NT, smem) : 0;
  kern<<<op.nfields * ntiles, NT, smem, s>>>(op, tw, nlines, pf);
  return cudaGetLastError();
}


// P1 through k_lines_tma: N x (N H) lines of 3 components at component
// stride cs (complex values), NLINES lines per CTA.
template <int L, int NLINES, class Op>
inline cudaError_t launch_lines_tma(const Op& op, int nouter, const float2* tw, const float2* in, size_t cs,
                                    int* err, cudaStream_t s) {
  constexpr int NSRC = 2 * L / 3;
  constexpr int NT = cmin(rthreads<float, L, NLINES>(), 384);
  const int nlines = nouter * op.hz;
  if (nlines % NLINES != 0 || (reinterpret_cast<uintptr_t>(in) & 15u) != 0 || ((cs * sizeof(float2)) & 15u) != 0)
    return cudaErrorInvalidValue;
  const TensorMapEncodeTiledFn enc = tensor_map_encoder();
  if (!enc) return cudaErrorNotSupported;
  CUtensorMap map;
  const cuuint64_t dims[3] = {(cuuint64_t)2 * nlines, (cuuint64_t)NSRC, 3};
  const cuuint64_t strides[2] = {(cuuint64_t)nlines * sizeof(float2), (cuuint64_t)cs * sizeof(float2)};
  const cuuint32_t box[3] = {2 * NLINES, NSRC, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  if (enc(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float2*>(in), dims, strides, box, estr,
          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return cudaErrorInvalidValue;
  const size_t smem = (size_t)(NSRC * NLINES + rsmem_elems<float, L, NLINES>()) * sizeof(float2) + 128;
  constexpr auto kern = k_lines_tma<L, NLINES, NT, Op>;
  cudaError_t e = prepare_kernel<kern>(smem);
  if (e != cudaSuccess) return e;
  kern<<<op.nfields * (nlines / NLINES), NT, smem, s>>>(op, tw, map, err);
  return cudaGetLastError();
}


template <typename R, int N>
inline cudaError_t nle_n(const NleParams<R>& p, cudaStream_t s) {
  constexpr int M = 3 * N / 2;
  constexpr int H = N / 2 + 1;
  const size_t fsA1 = (size_t)M * N * H;   // P1 out field stride
  const size_t fsB2 = (size_t)M * M * H;   // P2 out field stride
  const size_t fsA3 = (size_t)M * M * H;   // P3 out field stride
  const size_t fsB4 = (size_t)M * N * H;   // P4 out field stride
  const R ks = (R)p.ks;
  cudaError_t e;
  // P1
  {
    TimerScope ts(p.timer, PASS_P1, s);
    OpXInv<R, N, M> o{5, H, N, M, (R)(1.0 / ((double)N * N * N)), ks, p.in, p.cs, p.bufA, fsA1};
#if VK_P1_TMA
    if constexpr (sizeof(R) == 4 && M == 384 && (N * H) % 16 == 0)
      e = launch_lines_tma<M, 16>(o, N, p.twM, p.in, p.cs, p.async_err, s);
    else
#endif
      e = launch_lines<R, M, true, true>(o, N, p.twM, s);
    if (e != cudaSuccess) return e;
  }
  // P2
  {
    TimerScope ts(p.timer, PASS_P2, s);
    OpYInv<R, N, M> o{6, H, N, M, 0, ks, p.bufA, fsA1, p.bufB, fsB2};
    e = launch_lines<R, M, true>(o, M, p.twM, s);
    if (e != cudaSuccess) return e;
  }
  // P3 (FP32 at M = 384: the fused inverse-last / cross / forward-first kernel)
  if constexpr (sizeof(R) == 4 && M == 384) {
    TimerScope ts(p.timer, PASS_P3, s);
    constexpr int CP = P3F_CP;
    static_assert((M * M) % (2 * CP) == 0, "whole tiles");
    P3Args<R> a{M * M, p.bufB, fsB2, p.bufA, fsA3};
    const int ntiles = M * M / (2 * CP);
    const size_t smem = (size_t)P3F<CP>::SMEM_ELEMS * sizeof(float2);
    constexpr auto kern = k_p3f<CP>;
    e = prepare_kernel<kern>(smem);
    if (e != cudaSuccess) return e;
    const int pf = VK_P3F_PREFETCH ? wave_blocks<kern>(P3F<CP>::NT, smem) : 0;
    kern<<<ntiles, P3F<CP>::NT, smem, s>>>(a, p.twM, pf);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  } else {
    TimerScope ts(p.timer, PASS_P3, s);
    constexpr int CP = zpairs<M, 384>();
    constexpr int NT = p3_threads<R, M, CP>();
    const size_t smem = (size_t)p3_smem_lines<R, M, CP>() * zpad_len<R>(M) * sizeof(C2<R>);
    constexpr auto kern = k_p3<R, M, CP, NT>;
    e = prepare_kernel<kern>(smem);
    if (e != cudaSuccess) return e;
    P3Args<R> a{M * M, p.bufB, fsB2, p.bufA, fsA3};
    const int nb = (M * M + 2 * CP - 1) / (2 * CP);
    kern<<<nb, NT, smem, s>>>(a, p.twM, zpass_prefetch_distance<R, kern>(NT, smem));
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  // P4
  {
    TimerScope ts(p.timer, PASS_P4, s);
    OpYFwdTrunc<R, N, M> o{3, H, N, M, p.bufA, fsA3, p.bufB, fsB4};
    e = launch_lines<R, M, false>(o, M, p.twM, s);
    if (e != cudaSuccess) return e;
  }
  // P5 (the DIAG instance when the stage also feeds fused diagnostics)
  if (p.wait_p5) {
    e = cudaStreamWaitEvent(s, p.wait_p5, 0);
    if (e != cudaSuccess) return e;
  }
  {
    TimerScope ts(p.timer, PASS_P5, s);
    constexpr int NL = P5Lines<R, M>::value;
    constexpr int NT = p5_threads<R, M, NL>();
    const int nlines = N * H;
    const bool diag = p.st.diag != 0;
    const size_t smem = (size_t)(rsmem_elems<R, M, NL>() + 3 * N * NL) * sizeof(C2<R>) +
                        (diag ? (size_t)p.st.nsh * sizeof(double) : 0);
    const double scale = (double)M * M * M / ((double)N * N * N);
    P5Args<R> a{N, M, H, nlines, (R)(1.0 / scale), ks, p.bufB, fsB4, p.st};
    const int ntiles = (nlines + NL - 1) / NL;
    if (diag) {
      constexpr auto kern = k_p5<R, M, NL, NT, true>;
      e = prepare_kernel<kern>(smem);
      if (e != cudaSuccess) return e;
      kern<<<ntiles, NT, smem, s>>>(a, p.twM);
    } else {
      constexpr auto kern = k_p5<R, M, NL, NT, false>;
      e = prepare_kernel<kern>(smem);
      if (e != cudaSuccess) return e;
      kern<<<ntiles, NT, smem, s>>>(a, p.twM);
    }
    e = cudaGetLastError();
  }
  return e;
}

template <typename R, int N>
inline cudaError_t nla_n(const NlaParams<R>& p, cudaStream_t s) {
  constexpr int M = 3 * N / 2;
  constexpr int H = N / 2 + 1;
  const size_t fsA1 = (size_t)M * N * H;   // A1 out: 8 fields (M, N, H)
  const size_t fsB2 = (size_t)M * M * H;   // A2 out: 9 fields (M, M, H)
  const size_t fsA3 = (size_t)M * M * H;   // A3 out: 6 fields (M, M, H)
  const size_t fsB4 = (size_t)M * N * H;   // A4 out: 6 fields (M, N, H)
  const R ks = (R)p.ks;
  const double scale = (double)M * M * M / ((double)N * N * N);
  cudaError_t e;
  {
    TimerScope ts(p.timer, PASS_A1, s);
    // c_bar source into bufB (free until A2 writes it)
    CbarArgs<R> ca{N, H, (R)(1.0 / scale), ks, p.nb, p.cs, p.etd, p.slot, p.fac, p.dt, p.bufB};
    const size_t nm = (size_t)N * N * H;
    k_adj_cbar<R><<<(unsigned)((nm + 255) / 256), 256, 0, s>>>(ca);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    OpAdjXInv<R, N, M> o{8, H, N, M, (R)(1.0 / ((double)N * N * N)), ks, p.x, p.cs, p.bufB, p.bufA, fsA1};
    e = launch_lines<R, M, true, true>(o, N, p.twM, s);
    if (e != cudaSuccess) return e;
  }
  {
    TimerScope ts(p.timer, PASS_A2, s);
    OpAdjYInv<R, N, M> o{OpYInv<R, N, M>{6, H, N, M, 0, ks, p.bufA, fsA1, p.bufB, fsB2}, 9, H};
    e = launch_lines<R, M, true>(o, M, p.twM, s);
    if (e != cudaSuccess) return e;
  }
  {
    TimerScope ts(p.timer, PASS_A3, s);
    constexpr int CP = zpairs<M, 384>();
    constexpr int NT = adj_z_threads<R, M, CP>();
    const size_t smem = (size_t)adj_z_smem_elems<R, M, CP>() * sizeof(C2<R>);
    constexpr auto kern = k_adj_z<R, M, CP, NT>;
    e = prepare_kernel<kern>(smem);
    if (e != cudaSuccess) return e;
    A3Args<R> a{M * M, p.bufB, fsB2, p.bufA, fsA3};
    const int nb = (M * M + 2 * CP - 1) / (2 * CP);
    kern<<<nb, NT, smem, s>>>(a, p.twM, zpass_prefetch_distance<R, kern>(NT, smem));
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  {
    TimerScope ts(p.timer, PASS_A4, s);
    OpYFwdTrunc<R, N, M> o{6, H, N, M, p.bufA, fsA3, p.bufB, fsB4};
    e = launch_lines<R, M, false>(o, M, p.twM, s);
    if (e != cudaSuccess) return e;
  }
  {
    TimerScope ts(p.timer, PASS_A5, s);
    constexpr int NL = A5Lines<R>::value;
    constexpr int NT = cmin(rthreads<R, M, NL>(), 384);
    const int nlines = N * H;
    const size_t smem = (size_t)(rsmem_elems<R, M, NL>() + 3 * N * NL) * sizeof(C2<R>);
    constexpr auto kern = k_adj_p5<R, M, NL, NT>;
    e = prepare_kernel<kern>(smem);
    if (e != cudaSuccess) return e;
    A5Args<R> a{N, M, H, nlines, (R)(1.0 / ((double)N * N * N)), ks, p.bufB, fsB4, p.st};
    const int ntiles = (nlines + NL - 1) / NL;
    kern<<<ntiles, NT, smem, s>>>(a, p.twM);
    e = cudaGetLastError();
  }
  return e;
}

template <typename R, int N>
inline cudaError_t ngrid_n(const NgridParams<R>& p, cudaStream_t s) {
  constexpr int H = N / 2 + 1;
  const size_t fs = (size_t)N * N * H;
  const R ks = (R)p.ks;
  const bool both = p.which == 3;
  const bool need_w = p.which != 1;
  cudaError_t e;
  {
    TimerScope ts(p.timer, PASS_NX, s);
    const int nf = need_w ? 5 : 3;
    OpXInv<R, N, N> o{nf, H, N, N, (R)(1.0 / ((double)N * N * N)), ks, p.in, p.cs, p.bufA, fs};
    e = launch_lines<R, N, true, true>(o, N, p.twN, s);
    if (e != cudaSuccess) return e;
  }
  {
    TimerScope ts(p.timer, PASS_NY, s);
    const int nf = both ? 6 : 3;
    const int gbase = p.which == 2 ? 3 : 0;
    OpYInv<R, N, N> o{nf, H, N, N, gbase, ks, p.bufA, fs, p.bufB, fs};
    e = launch_lines<R, N, true>(o, N, p.twN, s);
    if (e != cudaSuccess) return e;
  }
  TimerScope ts(p.timer, PASS_NZ, s);
  constexpr int CP = zpairs<N, 512>();
  NZArgs<R> a{N * N, p.bufB, fs, p.out, p.which};
  const int nb = (N * N + 2 * CP - 1) / (2 * CP);
  if (both) {
    constexpr int NT = nz_threads<R, N, CP, true>();
    const size_t smem = (size_t)6 * CP * zpad_len<R>(N) * sizeof(C2<R>);
    constexpr auto kern = k_nz_max<R, N, CP, true, NT>;
    e = prepare_kernel<kern>(smem);
    if (e != cudaSuccess) return e;
    kern<<<nb, NT, smem, s>>>(a, p.twN, zpass_prefetch_distance<R, kern>(NT, smem));
  } else {
    constexpr int NT = nz_threads<R, N, CP, false>();
    const size_t smem = (size_t)3 * CP * zpad_len<R>(N) * sizeof(C2<R>);
    constexpr auto kern = k_nz_max<R, N, CP, false, NT>;
    e = prepare_kernel<kern>(smem);
    if (e != cudaSuccess) return e;
    kern<<<nb, NT, smem, s>>>(a, p.twN, zpass_prefetch_distance<R, kern>(NT, smem));
  }
  return cudaGetLastError();
}

// Standalone backend: one pass per axis with its own length.
template <typename R, int L>
inline cudaError_t fz_pass(const FftParams<R>& p, bool inverse, R scale, cudaStream_t s) {
  constexpr int CP = zpairs<L, 4096>();
  constexpr int NT = zthreads<R, CP, L>();
  const size_t smem = (size_t)CP * zpad_len<R>(L) * sizeof(C2<R>);
  const int ncols = p.nx * p.ny;
  const int nb = (ncols + 2 * CP - 1) / (2 * CP);
  FZArgs<R> a{ncols, p.real, p.cplx, scale};
  cudaError_t e;
  if (inverse) {
    constexpr auto kern = k_fz_c2r<R, L, CP, NT>;
    e = prepare_kernel<kern>(smem);
    if (e != cudaSuccess) return e;
    kern<<<nb, NT, smem, s>>>(a, p.twz);
  } else {
    constexpr auto kern = k_fz_r2c<R, L, CP, NT>;
    e = prepare_kernel<kern>(smem);
    if (e != cudaSuccess) return e;
    kern<<<nb, NT, smem, s>>>(a, p.twz);
  }
  return cudaGetLastError();
}

template <typename R, int L, int AXIS>
inline cudaError_t fxy_pass(const FftParams<R>& p, bool inverse, cudaStream_t s) {
  const int hz = p.nz / 2 + 1;
  OpPlainC2C<R, AXIS> o{1, hz, p.nx, p.ny, p.cplx};
  const int nouter = AXIS == 0 ? p.ny : p.nx;
  const C2<R>* tw = AXIS == 0 ? p.twx : p.twy;
  if (inverse) return launch_lines<R, L, true, AXIS == 0>(o, nouter, tw, s);
  return launch_lines<R, L, false, AXIS == 0>(o, nouter, tw, s);
}

#define VK_FOR_LENGTHS(X) X(8) X(16) X(32) X(64) X(128) X(256) X(512) X(12) X(24) X(48) X(96) X(192) X(384) X(768)

template <typename R>
inline cudaError_t fz_dispatch(const FftParams<R>& p, bool inverse, R scale, cudaStream_t s) {
  switch (p.nz) {
#define VK_CASE(L) case L: return fz_pass<R, L>(p, inverse, scale, s);
    VK_FOR_LENGTHS(VK_CASE)
#undef VK_CASE
    default: return cudaErrorInvalidValue;
  }
}

template <typename R, int AXIS>
inline cudaError_t fxy_dispatch(const FftParams<R>& p, bool inverse, cudaStream_t s) {
  const int L = AXIS == 0 ? p.nx : p.ny;
  switch (L) {
#define VK_CASE(LL) case LL: return fxy_pass<R, LL, AXIS>(p, inverse, s);
    VK_FOR_LENGTHS(VK_CASE)
#undef VK_CASE
    default: return cudaErrorInvalidValue;
  }
}

#define VK_FOR_GRIDS(X) X(8) X(16) X(32) X(64) X(128) X(256) X(512)

template <typename R>
cudaError_t Engine<R>::nle(const NleParams<R>& p, cudaStream_t s) {
  switch (p.N) {
#define VK_CASE(NN) case NN: return nle_n<R, NN>(p, s);
    VK_FOR_GRIDS(VK_CASE)
#undef VK_CASE
    default: return cudaErrorInvalidValue;
  }
}

template <typename R>
cudaError_t Engine<R>::nle_adjoint(const NlaParams<R>& p, cudaStream_t s) {
  switch (p.N) {
#define VK_CASE(NN) case NN: return nla_n<R, NN>(p, s);
    VK_FOR_GRIDS(VK_CASE)
#undef VK_CASE
    default: return cudaErrorInvalidValue;
  }
}

template <typename R>
cudaError_t Engine<R>::adj_mode(int N, double ks, size_t cs, const C2<R>* in, C2<R>* out, int mode,
                                cudaStream_t s) {
  ModeArgs<R> a{N, N / 2 + 1, ks, cs, in, out, mode};
  const size_t total = (size_t)N * N * (N / 2 + 1);
  const int nb = (int)std::min<size_t>((total + 255) / 256, 65536);
  k_adj_mode<R><<<nb, 256, 0, s>>>(a);
  return cudaGetLastError();
}

template <typename R>
cudaError_t Engine<R>::hermitian_avg(int N, size_t cs, const C2<R>* in, C2<R>* out, cudaStream_t s) {
  const size_t total = (size_t)N * N * (N / 2 + 1);
  const int nb = (int)std::min<size_t>((total + 255) / 256, 65536);
  k_hermitian_avg<R><<<nb, 256, 0, s>>>(N, N / 2 + 1, cs, in, out);
  return cudaGetLastError();
}

template <typename R>
cudaError_t Engine<R>::ngrid_max(const NgridParams<R>& p, cudaStream_t s) {
  switch (p.N) {
#define VK_CASE(NN) case NN: return ngrid_n<R, NN>(p, s);
    VK_FOR_GRIDS(VK_CASE)
#undef VK_CASE
    default: return cudaErrorInvalidValue;
  }
}

template <typename R>
cudaError_t Engine<R>::fft_r2c(const FftParams<R>& p, cudaStream_t s) {
  cudaError_t e;
  {
    TimerScope ts(p.timer, PASS_FFT_Z, s);
    e = fz_dispatch<R>(p, false, R(1), s);
  }
  if (e != cudaSuccess) return e;
  {
    TimerScope ts(p.timer, PASS_FFT_Y, s);
    e = fxy_dispatch<R, 1>(p, false, s);
  }
  if (e != cudaSuccess) return e;
  TimerScope ts(p.timer, PASS_FFT_X, s);
  return fxy_dispatch<R, 0>(p, false, s);
}

template <typename R>
cudaError_t Engine<R>::fft_c2r(const FftParams<R>& p, cudaStream_t s) {
  cudaError_t e;
  {
    TimerScope ts(p.timer, PASS_FFT_X, s);
    e = fxy_dispatch<R, 0>(p, true, s);
  }
  if (e != cudaSuccess) return e;
  {
    TimerScope ts(p.timer, PASS_FFT_Y, s);
    e = fxy_dispatch<R, 1>(p, true, s);
  }
  if (e != cudaSuccess) return e;
  const R scale = (R)(1.0 / ((double)p.nx * p.ny * p.nz));
  TimerScope ts(p.timer, PASS_FFT_Z, s);
  return fz_dispatch<R>(p, true, scale, s);
}

#define VK_FOR_GRIDS(X) X(8) X(16) X(32) X(64) X(128) X(256) X(512)

template <typename R>
cudaError_t Engine<R>::tier1_partial(const C2<R>* u, size_t cs, int N, double ks, double* part, int nblk,
                                     cudaStream_t s) {
  switch (N) {
#define VK_CASE(G) \
  case G: k_tier1_partial<R, G><<<nblk, RED_THREADS, 0, s>>>(u, cs, ks, part); break;
    VK_FOR_GRIDS(VK_CASE)
#undef VK_CASE
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

template <typename R, int G>
inline cudaError_t spectrum_partial_n(const C2<R>* u, size_t cs, double ks, int nsh, double* part, int nblk,
                                      cudaStream_t s) {
  const size_t smem = (size_t)nsh * sizeof(double);
  constexpr auto kern = k_spectrum_partial<R, G>;
  cudaError_t e = prepare_kernel<kern>(smem);
  if (e != cudaSuccess) return e;
  kern<<<nblk, RED_THREADS, smem, s>>>(u, cs, ks, nsh, part);
  return cudaGetLastError();
}

template <typename R>
cudaError_t Engine<R>::spectrum_partial(const C2<R>* u, size_t cs, int N, double ks, int nsh, double* part,
                                        int nblk, cudaStream_t s) {
  switch (N) {
#define VK_CASE(G) \
  case G: return spectrum_partial_n<R, G>(u, cs, ks, nsh, part, nblk, s);
    VK_FOR_GRIDS(VK_CASE)
#undef VK_CASE
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace vk
