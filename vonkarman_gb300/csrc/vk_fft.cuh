// Shared-memory batched FFT engine for sm_103a.
//
// Lines of length L = 2^a or 3*2^a (8 <= L <= 1536) are transformed in shared
// memory by a mixed-radix Stockham auto-sort (radix 8/4/3/2, natural-order
// output, no bit reversal).  All threads of a CTA cooperate on NLINES lines:
// in each stage every thread loads the inputs of its butterflies into
// registers, the CTA synchronises, then every thread twiddles, runs the radix
// kernel and stores.  Twiddles W_L^m = exp(-2 pi i m / L) come from a table
// computed on the host in extended precision (no device trigonometry).
//
// Forward = exp(-i...), unnormalised; inverse = exp(+i...), unnormalised.  The
// callers fold the 1/N normalisations of the reference's c2r_3d
// (vonkarman-fft/src/ndrustfft_backend.rs:46-57) into their load/store steps.
#pragma once

#include "vk_host.h"

namespace vk {

template <typename R>
__device__ __forceinline__ C2<R> cmk(R x, R y) { C2<R> c; c.x = x; c.y = y; return c; }
template <typename R>
__device__ __forceinline__ C2<R> cadd(C2<R> a, C2<R> b) { return cmk<R>(a.x + b.x, a.y + b.y); }
template <typename R>
__device__ __forceinline__ C2<R> csub(C2<R> a, C2<R> b) { return cmk<R>(a.x - b.x, a.y - b.y); }
template <typename R>
__device__ __forceinline__ C2<R> cscale(C2<R> a, R s) { return cmk<R>(a.x * s, a.y * s); }
template <typename R>
__device__ __forceinline__ C2<R> cconj(C2<R> a) { return cmk<R>(a.x, -a.y); }
// a * (+i)
template <typename R>
__device__ __forceinline__ C2<R> cmul_i(C2<R> a) { return cmk<R>(-a.y, a.x); }
// a * (-i)
template <typename R>
__device__ __forceinline__ C2<R> cmul_mi(C2<R> a) { return cmk<R>(a.y, -a.x); }
template <typename R>
__device__ __forceinline__ C2<R> cmul(C2<R> a, C2<R> b) {
  return cmk<R>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
template <typename R>
__device__ __forceinline__ C2<R> cmulc(C2<R> a, C2<R> b) {
  return cmk<R>(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
template <typename R>
__device__ __forceinline__ C2<R> czero() { return cmk<R>(R(0), R(0)); }

// ---------------------------------------------------------------------------
// Radix plans.  The first stage carries no twiddles, so the largest radix goes
// first.
// ---------------------------------------------------------------------------
__host__ __device__ constexpr int plan_stages(int L) {
  return L == 8 ? 1 : L == 16 ? 2 : L == 32 ? 2 : L == 64 ? 2 : L == 128 ? 3 : L == 256 ? 3
       : L == 512 ? 3 : L == 1024 ? 4 : L == 12 ? 2 : L == 24 ? 2 : L == 48 ? 3 : L == 96 ? 3
       : L == 192 ? 3 : L == 384 ? 4 : L == 768 ? 4 : L == 1536 ? 4 : -1;
}

__host__ __device__ constexpr int plan_radix(int L, int s) {
  return L == 8 ? 8
       : L == 16 ? 4
       : L == 32 ? (s == 0 ? 8 : 4)
       : L == 64 ? 8
       : L == 128 ? (s == 0 ? 8 : 4)
       : L == 256 ? (s < 2 ? 8 : 4)
       : L == 512 ? 8
       : L == 1024 ? (s < 2 ? 8 : 4)
       : L == 12 ? (s == 0 ? 4 : 3)
       : L == 24 ? (s == 0 ? 8 : 3)
       : L == 48 ? (s < 2 ? 4 : 3)
       : L == 96 ? (s == 0 ? 8 : s == 1 ? 4 : 3)
       : L == 192 ? (s < 2 ? 8 : 3)
       : L == 384 ? (s == 0 ? 8 : s < 3 ? 4 : 3)
       : L == 768 ? (s < 2 ? 8 : s == 2 ? 4 : 3)
       : L == 1536 ? (s < 3 ? 8 : 3)
       : 1;
}

__host__ __device__ constexpr bool fft_len_supported(int L) { return plan_stages(L) > 0; }

// ---------------------------------------------------------------------------
// Radix kernels (in registers).  INV selects exp(+i...).
// ---------------------------------------------------------------------------
template <typename R, bool INV>
__device__ __forceinline__ void dft2(C2<R>* v) {
  C2<R> a = v[0], b = v[1];
  v[0] = cadd<R>(a, b);
  v[1] = csub<R>(a, b);
}

template <typename R, bool INV>
__device__ __forceinline__ void dft4(C2<R>& a0, C2<R>& a1, C2<R>& a2, C2<R>& a3) {
  C2<R> t0 = cadd<R>(a0, a2), t1 = csub<R>(a0, a2);
  C2<R> t2 = cadd<R>(a1, a3), t3 = csub<R>(a1, a3);
  t3 = INV ? cmul_i<R>(t3) : cmul_mi<R>(t3);
  a0 = cadd<R>(t0, t2);
  a2 = csub<R>(t0, t2);
  a1 = cadd<R>(t1, t3);
  a3 = csub<R>(t1, t3);
}

template <typename R, bool INV>
__device__ __forceinline__ void dft3(C2<R>* v) {
  const R c = R(0.86602540378443864676372317075293618);  // sqrt(3)/2
  C2<R> a0 = v[0], a1 = v[1], a2 = v[2];
  C2<R> t = cadd<R>(a1, a2);
  C2<R> d = csub<R>(a1, a2);
  C2<R> m = cmk<R>(a0.x - R(0.5) * t.x, a0.y - R(0.5) * t.y);
  // forward: d * (-i c); inverse: d * (+i c)
  C2<R> e = INV ? cmk<R>(-c * d.y, c * d.x) : cmk<R>(c * d.y, -c * d.x);
  v[0] = cadd<R>(a0, t);
  v[1] = cadd<R>(m, e);
  v[2] = csub<R>(m, e);
}

template <typename R, bool INV>
__device__ __forceinline__ void dft8(C2<R>* v) {
  const R h = R(0.70710678118654752440084436210484904);  // sqrt(2)/2
  C2<R> e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
  C2<R> o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
  dft4<R, INV>(e0, e1, e2, e3);
  dft4<R, INV>(o0, o1, o2, o3);
  // o_q *= W8^q  (forward W8 = h(1 - i), inverse h(1 + i))
  C2<R> w1, w3;
  if (INV) {
    w1 = cmk<R>(h * (o1.x - o1.y), h * (o1.x + o1.y));
    w3 = cmk<R>(-h * (o3.x + o3.y), h * (o3.x - o3.y));
    o2 = cmul_i<R>(o2);
  } else {
    w1 = cmk<R>(h * (o1.x + o1.y), h * (o1.y - o1.x));
    w3 = cmk<R>(h * (o3.y - o3.x), -h * (o3.x + o3.y));
    o2 = cmul_mi<R>(o2);
  }
  v[0] = cadd<R>(e0, o0);
  v[4] = csub<R>(e0, o0);
  v[1] = cadd<R>(e1, w1);
  v[5] = csub<R>(e1, w1);
  v[2] = cadd<R>(e2, o2);
  v[6] = csub<R>(e2, o2);
  v[3] = cadd<R>(e3, w3);
  v[7] = csub<R>(e3, w3);
}

template <typename R, bool INV, int RAD>
__device__ __forceinline__ void dft(C2<R>* v) {
  if constexpr (RAD == 8) {
    dft8<R, INV>(v);
  } else if constexpr (RAD == 4) {
    dft4<R, INV>(v[0], v[1], v[2], v[3]);
  } else if constexpr (RAD == 3) {
    dft3<R, INV>(v);
  } else {
    dft2<R, INV>(v);
  }
}

// ---------------------------------------------------------------------------
// Stockham stages.  Element p of line l lives at buf[l*ld_line + p*ld_elem].
// LINE_FAST: consecutive threads take consecutive lines (use when lines are
// interleaved, ld_line == 1); otherwise consecutive butterflies of a line.
// ---------------------------------------------------------------------------
template <typename R, int L, bool INV, int NT, int NLINES, bool LINE_FAST, int S, int NS>
struct StockhamStage {
  __device__ __forceinline__ static void run(C2<R>* buf, int ld_line, int ld_elem,
                                             const C2<R>* __restrict__ tw) {
    constexpr int RAD = plan_radix(L, S);
    constexpr int NB = L / RAD;          // butterflies per line
    constexpr int TOTAL = NB * NLINES;   // butterflies per stage
    constexpr int Q = (TOTAL + NT - 1) / NT;
    constexpr int TWS = L / (NS * RAD);  // twiddle table stride
    const int tid = threadIdx.x;
    C2<R> v[Q][RAD];
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      const int g = tid + q * NT;
      if (TOTAL % NT == 0 || g < TOTAL) {
        const int l = LINE_FAST ? (g % NLINES) : (g / NB);
        const int j = LINE_FAST ? (g / NLINES) : (g % NB);
        const C2<R>* src = buf + l * ld_line;
#pragma unroll
        for (int r = 0; r < RAD; ++r) v[q][r] = src[(j + r * NB) * ld_elem];
      }
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      const int g = tid + q * NT;
      if (TOTAL % NT == 0 || g < TOTAL) {
        const int l = LINE_FAST ? (g % NLINES) : (g / NB);
        const int j = LINE_FAST ? (g / NLINES) : (g % NB);
        const int k = j % NS;
        if (S > 0) {
#pragma unroll
          for (int r = 1; r < RAD; ++r) {
            const C2<R> w = tw[r * k * TWS];
            v[q][r] = INV ? cmulc<R>(v[q][r], w) : cmul<R>(v[q][r], w);
          }
        }
        dft<R, INV, RAD>(v[q]);
        C2<R>* dst = buf + l * ld_line;
        const int base = (j - k) * RAD + k;
#pragma unroll
        for (int r = 0; r < RAD; ++r) dst[(base + r * NS) * ld_elem] = v[q][r];
      }
    }
    __syncthreads();
    if constexpr (S + 1 < plan_stages(L)) {
      StockhamStage<R, L, INV, NT, NLINES, LINE_FAST, S + 1, NS * RAD>::run(buf, ld_line, ld_elem, tw);
    }
  }
};

// Transform NLINES lines held in shared memory.  Must be called by all NT
// threads of the CTA; begins and ends with the data synchronised.
template <typename R, int L, bool INV, int NT, int NLINES, bool LINE_FAST>
__device__ __forceinline__ void fft_smem(C2<R>* buf, int ld_line, int ld_elem,
                                         const C2<R>* __restrict__ tw) {
  static_assert(plan_stages(L) > 0, "unsupported FFT length");
  StockhamStage<R, L, INV, NT, NLINES, LINE_FAST, 0, 1>::run(buf, ld_line, ld_elem, tw);
}

}  // namespace vk
