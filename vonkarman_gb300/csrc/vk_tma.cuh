// P1 (x-inverse with the zero-pad) with its input tile staged in shared
// memory by the tensor-memory accelerator: one cp.async.bulk.tensor copy per
// CTA brings the CTA's NLINES consecutive (iy, z) lines of one velocity
// component, all N rows of x (N x NLINES complex values, rows of
// NLINES * 8 bytes), into shared memory; an mbarrier with the copy's byte
// count signals its arrival, and the first FFT stage reads its butterfly
// inputs from there instead of from global memory.  The rest of the pass is
// k_lines's.
//
// Tensor map (3-D, FP32 elements, no swizzle, no interleave): dimension 0 the
// flattened (iy, z) index in floats (2 N H, contiguous), dimension 1 x (N
// rows, stride N H complex), dimension 2 the component (3, stride cs complex);
// box {2 NLINES, N, 1}.  The box's x coordinate is 2 NLINES tile floats, a
// multiple of 16 bytes, as every tiled bulk copy needs.
//
// The wait on the mbarrier is bounded (about a second of clock cycles); a
// CTA whose copy has not arrived by then sets *err, waits once more with the
// same bound and leaves without touching the tile (every thread of the CTA
// takes the same branch).
#pragma once

#include <cuda.h>

#include "vk_lines.cuh"

namespace vk {

__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
  unsigned done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return done != 0u;
}

// Wait for phase `parity` of the mbarrier for at most `limit` clock cycles.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, unsigned parity, long long limit) {
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity))
    if (clock64() - t0 > limit) return false;
  return true;
}

// 3-D tiled bulk copy global -> shared memory, completion counted on bar.
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int c0, int c1, int c2,
                                            unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
      ::"r"(smem_u32(dst)), "l"(reinterpret_cast<unsigned long long>(map)), "r"(c0), "r"(c1), "r"(c2),
        "r"(smem_u32(bar))
      : "memory");
}

constexpr long long kMbarWaitCycles = 2000000000ll;   // about one second at 2 GHz

// k_lines for OpXInv with the input tile staged by the tensor copy.  Whole
// tiles only (nlines a multiple of NLINES).
template <int L, int NLINES, int NT, class Op>
__global__ void __launch_bounds__(NT, lines_min_blocks<float, L, NT>())
k_lines_tma(Op op, const float2* __restrict__ tw, const __grid_constant__ CUtensorMap tmap, int* err) {
  using R = float;
  constexpr int NSRC = 2 * L / 3;   // source rows (the unpadded x length)
  extern __shared__ __align__(128) unsigned char vk_smem[];
  __shared__ C2<R> tw_s[twtab_elems<R, false>(L)];
  __shared__ __align__(8) unsigned long long bar;
  // the copy's destination on a 128-byte boundary (the launch adds 128 bytes
  // of slack to the dynamic shared memory)
  const unsigned mis = smem_u32(vk_smem) & 127u;
  C2<R>* stage = reinterpret_cast<C2<R>*>(vk_smem + (mis ? 128u - mis : 0u));   // NSRC x NLINES
  C2<R>* xb = stage + NSRC * NLINES;
  const int f = blockIdx.x % op.nfields;
  const int tile = blockIdx.x / op.nfields;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    mbar_arrive_expect_tx(&bar, (unsigned)(NSRC * NLINES * sizeof(C2<R>)));
    tma_load_3d(stage, &tmap, 2 * NLINES * tile, 0, op.src_component(f), &bar);
  }
  load_twtab<R, L, false, NT>(tw_s, tw);   // overlaps the copy
  bool arrived = mbar_wait_bounded(&bar, 0, kMbarWaitCycles);
  if (__syncthreads_or(!arrived)) {
    if (threadIdx.x == 0) {
      if (err) atomicExch(err, 1);
      mbar_wait_bounded(&bar, 0, kMbarWaitCycles);
    }
    return;
  }
  const int l0 = (int)(threadIdx.x % NLINES);
  const int lam = tile * NLINES + l0;
  const int outer = lam / op.h_();
  const int z = lam - outer * op.h_();
  const int kd = op.kind(f);
  auto st = [&](int, int p, C2<R> v) {
    const int i = op.out_index(p);
    if (i >= 0) op.store(f, outer, z, i, v);
  };
  sfor<Op::NKIND>([&](auto kc) {
    constexpr int K = decltype(kc)::value;
    if (kd != K) return;   // uniform over the CTA
    fft_lines<R, L, true, NT, NLINES, MapInterleaved<R, L, NLINES>, false, true, OpZeroRange<Op>::lo,
              OpZeroRange<Op>::hi>(
        xb, tw_s,
        [&](int l, int p) {
          const int ix = unpad_pos(p, NSRC, L);
          return ix < 0 ? czero<R>() : stage[ix * NLINES + l];
        },
        [&](int, int p, const auto& raw) { return op.template prep<K>(f, outer, z, p, raw); }, st);
  });
}

using TensorMapEncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                            const cuuint64_t*, const cuuint32_t*, const cuuint32_t*,
                                            CUtensorMapInterleave, CUtensorMapSwizzle, CUtensorMapL2promotion,
                                            CUtensorMapFloatOOBfill);

inline TensorMapEncodeTiledFn tensor_map_encoder() {
  static const TensorMapEncodeTiledFn fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return reinterpret_cast<TensorMapEncodeTiledFn>(p);
  }();
  return fn;
}

}  // namespace vk
