// P3 for the FP32-bulk form at M = 384 (N = 256) with the inverse's last
// stage, the cross product and the forward's first stage fused in registers.
//
// Per CTA CP column pairs; six real fields ride in three packed lines per
// column, (u_x + i u_y), (u_z + i w_x), (w_y + i w_z), the three real cross
// product fields of a column pair in three forward lines, F0 = c_x^A + i c_y^A,
// F1 = c_z^A + i c_z^B, F2 = c_x^B + i c_y^B (the layout k_p3 unpacks).
// Plans: inverse {24, 16}, forward {16, 24}.  Butterfly j' of the inverse's
// radix-16 last stage (stride NS = 24) yields positions j' + 24 r, r < 16 --
// exactly the inputs of butterfly j' of the forward's radix-16 first stage.
// So one thread per (column, j') transforms the three packed lines of its
// column at j', forms u x omega at those 16 positions and runs the forward
// first stage there; the partner column's c_z (the other half of F1) comes
// from the neighbouring lane by shuffle, and both lanes of a pair evaluate F1
// (each stores half of its outputs).  Shared-memory traffic per column pair
// drops from about 41 to 23 line transfers against the unfused k_p3.
//
//   phase A  inverse stage 0, radix 24 (untwiddled): inputs packed from
//            global with the Hermitian extension, 7 of 24 inputs zero padding
//   phase B  inverse stage 1 (radix 16) + cross product + forward stage 0
//            (radix 16), registers; writes the forward exchange
//   phase C  forward stage 1, radix 24
//   phase D  unpack the kept H modes of every real field and store
//
// Exchange layouts (complex floats; 64-bit accesses, served per half-warp):
//   XA (inverse): line (2 pair + cc) * 3 + t at stride LPA = 408, position p
//     at p + p / 24.  Phase A writes positions 24 j + r (index 25 j + r: 9 j
//     mod 16 distinct over a half-warp); phase B reads j' + 24 r (index
//     j' + 25 r) with lanes (j', cc) interleaved, and 3 LPA = 8 (mod 16)
//     separates the two columns' banks.
//   XF (forward, aliases XA after a barrier): line 3 pair + f at stride
//     LPF = 412, position p at p + p / 16; 2 LPF = 8 (mod 16) separates the
//     F0 and F2 writes of a half-warp.
#pragma once

#include "vk_lines.cuh"
#include "vk_pair.cuh"

// phase D from the registers of phase C with a shuffle for the Hermitian
// partner (1), or through shared memory after a barrier (0)
#ifndef VK_P3F_UNPACK_REGS
#define VK_P3F_UNPACK_REGS 1
#endif

namespace vk {

template <int CP>
struct P3F {
  static constexpr int M = 384;
  static constexpr int N = 256;
  static constexpr int H = N / 2 + 1;   // 129 kept modes
  static constexpr int NT = 48 * CP;    // one thread per (column, j') of the fused phase
  static constexpr int LPA = 408;
  static constexpr int LPF = 412;
  static constexpr int NI = 6 * CP;     // inverse lines
  static constexpr int NF = 3 * CP;     // forward lines
  static constexpr int SMEM_ELEMS = NI * LPA;   // >= NF * LPF
  static_assert(NF * LPF <= NI * LPA, "forward exchange must fit in the inverse one");
  static_assert((3 * LPA) % 16 == 8 && (2 * LPF) % 16 == 8, "bank-spreading strides");
  __device__ __forceinline__ static int ia(int p) { return p + p / 24; }
  __device__ __forceinline__ static int iff(int p) { return p + p / 16; }
};

// stage twiddles of both radix-16 / radix-24 twiddled stages, conflict-free
// per-stage tables: inverse stage 1 at (r - 1) 24 + j', forward stage 1 at
// (r - 1) 16 + j''
constexpr int P3F_TWI = 15 * 24;
constexpr int P3F_TWF = 23 * 16;

// Source of the phase-A inputs: field f (0..5) of column col, mode k,
// straight from global memory.
struct P3SrcGlobal {
  const float2* in;
  size_t fs;
  __device__ __forceinline__ float2 operator()(int f, int col, int k) const {
    return in[(size_t)f * fs + (size_t)col * 129 + k];
  }
};

// One tile of 2 CP columns (col0 ...): phases A..D.  X is the exchange
// buffer (P3F<CP>::SMEM_ELEMS); all NT threads call it; it returns after
// phase D's stores with no barrier after them.
template <int CP, class SRC>
__device__ __forceinline__ void p3f_tile(const P3Args<float>& a, int col0, float2* X, const float2* twi,
                                         const float2* twf, const SRC& src) {
  using G = P3F<CP>;
  constexpr int M = G::M, H = G::H, NT = G::NT;

  // ---- phase A: inverse stage 0, radix 24 over the 6 CP packed lines -------
  // butterflies (line la, j) and (line la + 3 CP, j), la = tid / 16, j = tid % 16,
  // as one lane pair.  Inputs at p = j + 16 r: r <= 7 are kept modes k = p, r = 8
  // is the mode k = 128 for j = 0 and padding otherwise, r in [9, 15] padding,
  // r >= 16 the Hermitian mirror k = M - p (tiles are always full: 2 CP divides
  // M^2, so no column bound is checked).
  {
    const int j = threadIdx.x & 15;
    int lines[2], cols[2], fld[2];
    lines[0] = threadIdx.x >> 4;
    lines[1] = lines[0] + 3 * CP;
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int l = lines[q];
      const int pair = l / 6, cc = (l / 3) & 1, t = l % 3;
      cols[q] = col0 + 2 * pair + cc;
      fld[q] = 2 * t;
    }
    C2f2 v[24], w0[24];
#pragma unroll
    for (int r = 0; r < 24; ++r) {
      float2 z[2];
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        float2 Xv = make_float2(0.f, 0.f), Yv = make_float2(0.f, 0.f);
        if (r <= 7 || (r == 8 && j == 0)) {
          Xv = src(fld[q], cols[q], j + 16 * r);
          Yv = src(fld[q] + 1, cols[q], j + 16 * r);
        } else if (r >= 16) {
          Xv = src(fld[q], cols[q], M - j - 16 * r);
          Yv = src(fld[q] + 1, cols[q], M - j - 16 * r);
        }
        // Z = X + i Y with the Hermitian extension; the DC's imaginary parts
        // are dropped (the reference backend's c2r convention)
        if (r <= 8) {
          z[q] = (r == 0 && j == 0) ? make_float2(Xv.x, Yv.x) : make_float2(Xv.x - Yv.y, Xv.y + Yv.x);
        } else {
          z[q] = make_float2(Xv.x + Yv.y, Yv.x - Xv.y);
        }
      }
      v[r] = cpack(z[0], z[1]);
    }
    dft<f2, true, 24, false>(v, w0);
    // outputs at positions 24 j + r, index 25 j + r
    float2* la = X + lines[0] * G::LPA + 25 * j;
    float2* lb = X + lines[1] * G::LPA + 25 * j;
#pragma unroll
    for (int r = 0; r < 24; ++r) {
      la[r] = clane0(v[r]);
      lb[r] = clane1(v[r]);
    }
  }
  __syncthreads();

  // ---- phase B: inverse stage 1 + cross product + forward stage 0 ----------
  const int pair = threadIdx.x / 48;
  const int rem = threadIdx.x - 48 * pair;
  const int jp = rem >> 1, cc = rem & 1;
  float cx[16], cy[16], cz[16];
  {
    float2 z[3][16];
    const float2* lines = X + ((2 * pair + cc) * 3) * G::LPA;
#pragma unroll
    for (int t = 0; t < 3; ++t) {
#pragma unroll
      for (int r = 0; r < 16; ++r) z[t][r] = lines[t * G::LPA + jp + 25 * r];   // position jp + 24 r
    }
    __syncthreads();   // XA is reused for the forward exchange below
    float2 w[16];
#pragma unroll
    for (int r = 1; r < 16; ++r) w[r] = twi[(r - 1) * 24 + jp];
    {
      // lines 0 and 1 as one lane pair (same twiddles), line 2 alone
      C2f2 P[16], W[16];
#pragma unroll
      for (int r = 0; r < 16; ++r) P[r] = cpack(z[0][r], z[1][r]);
#pragma unroll
      for (int r = 1; r < 16; ++r) W[r] = cbcast(w[r]);
      dft<f2, true, 16, true>(P, W);
      dft<float, true, 16, true>(z[2], w);
#pragma unroll
      for (int r = 0; r < 16; ++r) {
        z[0][r] = clane0(P[r]);
        z[1][r] = clane1(P[r]);
      }
    }
    // physical values at positions jp + 24 r: (u_x, u_y), (u_z, w_x), (w_y, w_z)
#pragma unroll
    for (int r = 0; r < 16; ++r) {
      const float ux = z[0][r].x, uy = z[0][r].y, uz = z[1][r].x, wx = z[1][r].y, wy = z[2][r].x, wz = z[2][r].y;
      cx[r] = uy * wz - uz * wy;
      cy[r] = uz * wx - ux * wz;
      cz[r] = ux * wy - uy * wx;
    }
  }
  {
    float2 fo[16], f1[16];
#pragma unroll
    for (int r = 0; r < 16; ++r) {
      const float other = __shfl_xor_sync(0xffffffffu, cz[r], 1);
      fo[r] = make_float2(cx[r], cy[r]);
      f1[r] = cc == 0 ? make_float2(cz[r], other) : make_float2(other, cz[r]);
    }
    {
      C2f2 F[16], W0[16];
#pragma unroll
      for (int r = 0; r < 16; ++r) F[r] = cpack(fo[r], f1[r]);
      dft<f2, false, 16, false>(F, W0);
#pragma unroll
      for (int r = 0; r < 16; ++r) {
        fo[r] = clane0(F[r]);
        f1[r] = clane1(F[r]);
      }
    }
    // stage-0 outputs at positions 16 jp + r
    float2* lo = X + (3 * pair + (cc == 0 ? 0 : 2)) * G::LPF;
    float2* l1 = X + (3 * pair + 1) * G::LPF;
#pragma unroll
    for (int r = 0; r < 16; ++r) lo[G::iff(16 * jp + r)] = fo[r];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int r = cc == 0 ? i : 8 + i;
      l1[G::iff(16 * jp + r)] = cc == 0 ? f1[i] : f1[8 + i];
    }
  }
  __syncthreads();

  // ---- phase C: forward stage 1, radix 24 -----------------------------------
  {
    const int f = rem >> 4, j = rem & 15;
    float2* line = X + (3 * pair + f) * G::LPF;
    float2 v[24], w[24];
#pragma unroll
    for (int r = 0; r < 24; ++r) v[r] = line[G::iff(j + 16 * r)];
#pragma unroll
    for (int r = 1; r < 24; ++r) w[r] = twf[(r - 1) * 16 + j];
#if VK_P3F_UNPACK_REGS
    dft<float, false, 24, true>(v, w);
    // ---- phase D: unpack the kept modes k = j + 16 r <= 128 from registers.
    // Z(M - k) is output 23 - r of lane 16 - j of this 16-lane group (the
    // line's), or, for j = 0, output (24 - r) mod 24 of this lane.
    const int lane = threadIdx.x & 31;
    const int src = (lane & 16) | ((16 - j) & 15);
    const int ca = col0 + 2 * pair, cb = ca + 1;
    float2* o0 = a.out + (size_t)(f == 2 ? cb : ca) * H;
#pragma unroll
    for (int r = 0; r <= 8; ++r) {
      const float2 zs = make_float2(__shfl_sync(0xffffffffu, v[23 - r].x, src),
                                    __shfl_sync(0xffffffffu, v[23 - r].y, src));
      const float2 zk = v[r];
      const float2 zm = j == 0 ? v[(24 - r) % 24] : zs;
      if (r == 8 && j != 0) continue;   // k = 128 only at j = 0
      const int k = j + 16 * r;
      const float2 Xv = make_float2(0.5f * (zk.x + zm.x), 0.5f * (zk.y - zm.y));
      const float2 Yv = make_float2(0.5f * (zk.y + zm.y), 0.5f * (zm.x - zk.x));
      if (f == 1) {
        o0[2 * a.fsout + k] = Xv;                       // c_z of column A
        a.out[2 * a.fsout + (size_t)cb * H + k] = Yv;   // c_z of column B
      } else {
        o0[k] = Xv;                                     // c_x of column A (f = 0) / B (f = 2)
        o0[a.fsout + k] = Yv;                           // c_y
      }
    }
  }
#else
    __syncthreads();   // outputs go back into the same line positions' buffer
    dft<float, false, 24, true>(v, w);
#pragma unroll
    for (int r = 0; r < 24; ++r) line[G::iff(j + 16 * r)] = v[r];
  }
  __syncthreads();

  // ---- phase D: unpack the kept H modes of each real field and store --------
#pragma unroll 1
  for (int row = 0; row < CP * 3; ++row) {
    const int pr = row / 3, f = row - 3 * pr;
    const float2* line = X + (3 * pr + f) * G::LPF;
    const int ca = col0 + 2 * pr, cb = ca + 1;
    float2* o0 = a.out + (size_t)(f == 0 ? ca : f == 1 ? ca : cb) * H;
    for (int k = threadIdx.x; k < H; k += NT) {
      const float2 zk = line[G::iff(k)];
      const float2 zm = line[G::iff(k == 0 ? 0 : M - k)];
      const float2 Xv = make_float2(0.5f * (zk.x + zm.x), 0.5f * (zk.y - zm.y));
      const float2 Yv = make_float2(0.5f * (zk.y + zm.y), 0.5f * (zm.x - zk.x));
      if (f == 0) {
        o0[k] = Xv;                                     // c_x of column A
        o0[a.fsout + k] = Yv;                           // c_y of column A
      } else if (f == 1) {
        o0[2 * a.fsout + k] = Xv;                       // c_z of column A
        a.out[2 * a.fsout + (size_t)cb * H + k] = Yv;   // c_z of column B
      } else {
        o0[k] = Xv;                                     // c_x of column B
        o0[a.fsout + k] = Yv;                           // c_y of column B
      }
    }
  }
#endif
}

template <int CP>
__device__ __forceinline__ void p3f_twiddles(float2* twi, float2* twf, const float2* __restrict__ tw) {
  for (int i = threadIdx.x; i < P3F_TWI; i += P3F<CP>::NT) {
    const int r = i / 24 + 1, j = i - (r - 1) * 24;
    twi[i] = tw[r * j];   // W_384^(r j), stride TWS = 384 / (24 * 16) = 1
  }
  for (int i = threadIdx.x; i < P3F_TWF; i += P3F<CP>::NT) {
    const int r = i / 16 + 1, j = i - (r - 1) * 16;
    twf[i] = tw[r * j];   // TWS = 384 / (16 * 24) = 1
  }
}

// One tile per CTA, inputs straight from global memory.
template <int CP>
__global__ void __launch_bounds__(P3F<CP>::NT, 384 / P3F<CP>::NT)
k_p3f(P3Args<float> a, const float2* __restrict__ tw, int pf) {
  extern __shared__ __align__(16) unsigned char vk_smem[];
  __shared__ float2 twi[P3F_TWI];
  __shared__ float2 twf[P3F_TWF];
  // L2 prefetch of the six input ranges of the CTA pf blocks ahead: per field
  // its 2 CP consecutive columns, 2 CP x 129 complex values (16-byte multiples)
  if (pf > 0 && threadIdx.x < 6 && blockIdx.x + pf < gridDim.x)
    prefetch_l2_bulk(a.in + (size_t)threadIdx.x * a.fsin + (size_t)(blockIdx.x + pf) * (2 * CP * 129),
                     2 * CP * 129 * sizeof(float2));
  p3f_twiddles<CP>(twi, twf, tw);
  float2* X = reinterpret_cast<float2*>(vk_smem);
  // the first barrier of the tile orders the twiddle loads before their use
  p3f_tile<CP>(a, blockIdx.x * 2 * CP, X, twi, twf, P3SrcGlobal{a.in, a.fsin});
}

}  // namespace vk
