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

#include <type_traits>
#include <utility>

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
// two loaded complex values (raw inputs that a later step combines)
template <typename R> struct C2x2 { C2<R> a, b; };

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

// FP32 plans use in-register radix-16 stages: fewer shared-memory passes for
// the bandwidth-bound FP32 form.  FP64 keeps radix <= 8 (registers; the FP64
// form is bound by the FP64 pipe, where radix 16 saves no instructions).
__host__ __device__ constexpr int plan_stages_f(int L) {
  return L == 8 ? 1 : L == 16 ? 1 : L == 32 ? 2 : L == 64 ? 2 : L == 128 ? 2 : L == 256 ? 2
       : L == 512 ? 3 : L == 1024 ? 3 : L == 12 ? 2 : L == 24 ? 2 : L == 48 ? 2 : L == 96 ? 3
       : L == 192 ? 3 : L == 384 ? 3 : L == 768 ? 3 : L == 1536 ? 4 : -1;
}

__host__ __device__ constexpr int plan_radix_f(int L, int s) {
  return L == 8 ? 8
       : L == 16 ? 16
       : L == 32 ? (s == 0 ? 16 : 2)
       : L == 64 ? (s == 0 ? 16 : 4)
       : L == 128 ? (s == 0 ? 16 : 8)
       : L == 256 ? 16
       : L == 512 ? (s < 2 ? 8 : 8)
       : L == 1024 ? (s < 2 ? 16 : 4)
       : L == 12 ? (s == 0 ? 4 : 3)
       : L == 24 ? (s == 0 ? 8 : 3)
       : L == 48 ? (s == 0 ? 16 : 3)
       : L == 96 ? (s == 0 ? 16 : s == 1 ? 2 : 3)
       : L == 192 ? (s == 0 ? 16 : s == 1 ? 4 : 3)
       : L == 384 ? (s == 0 ? 16 : s == 1 ? 8 : 3)
       : L == 768 ? (s < 2 ? 16 : 3)
       : L == 1536 ? (s < 2 ? 16 : s == 2 ? 2 : 3)
       : 1;
}

template <typename R> __host__ __device__ constexpr int stages_of(int L) {
  return sizeof(R) == 4 ? plan_stages_f(L) : plan_stages(L);
}
template <typename R> __host__ __device__ constexpr int radix_of(int L, int s) {
  return sizeof(R) == 4 ? plan_radix_f(L, s) : plan_radix(L, s);
}
// widest butterfly of a plan (threads per line = L / widest)
template <typename R> __host__ __device__ constexpr int max_radix(int L) {
  return sizeof(R) == 4 ? ((L % 16 == 0 && L >= 16 && L != 512) ? 16 : 8) : 8;
}

__host__ __device__ constexpr bool fft_len_supported(int L) { return plan_stages(L) > 0; }

// ---------------------------------------------------------------------------
// Radix kernels (in registers), with the stage twiddles fused into the first
// butterfly layer: a + w b costs 4 FMAs and a - w b = 2a - (a + w b) costs 2,
// instead of a complex multiply (4) plus two complex adds (4).  INV selects
// exp(+i...) and conjugated twiddles.  TW = false: first stage, no twiddles.
// ---------------------------------------------------------------------------
template <typename R, bool INV>
__device__ __forceinline__ C2<R> tw_mul(C2<R> w, C2<R> b) {  // w b (conj(w) b if INV)
  return INV ? cmk<R>(fma(w.x, b.x, w.y * b.y), fma(w.x, b.y, -(w.y * b.x)))
             : cmk<R>(fma(w.x, b.x, -(w.y * b.y)), fma(w.x, b.y, w.y * b.x));
}
template <typename R, bool INV>
__device__ __forceinline__ C2<R> tw_fma(C2<R> a, C2<R> w, C2<R> b) {  // a + w b (a + conj(w) b if INV)
  return INV ? cmk<R>(fma(w.y, b.y, fma(w.x, b.x, a.x)), fma(-w.y, b.x, fma(w.x, b.y, a.y)))
             : cmk<R>(fma(-w.y, b.y, fma(w.x, b.x, a.x)), fma(w.y, b.x, fma(w.x, b.y, a.y)));
}
template <typename R>
__device__ __forceinline__ C2<R> twice_minus(C2<R> a, C2<R> t) {  // 2a - t
  return cmk<R>(fma(R(2), a.x, -t.x), fma(R(2), a.y, -t.y));
}
// multiply by -i (forward) or +i (inverse)
template <typename R, bool INV>
__device__ __forceinline__ C2<R> rot(C2<R> a) { return INV ? cmul_i<R>(a) : cmul_mi<R>(a); }

// (s, d) pair: a + (x, y) and a - (x, y)
template <typename R>
__device__ __forceinline__ void bfly(C2<R> a, C2<R> b, C2<R>& p, C2<R>& m) {
  p = cadd<R>(a, b);
  m = csub<R>(a, b);
}

// radix-2: v[1] carries twiddle w[1]
template <typename R, bool INV, bool TW>
__device__ __forceinline__ void rad2(C2<R>* v, const C2<R>* w) {
  C2<R> p, m;
  if (TW) {
    p = tw_fma<R, INV>(v[0], w[1], v[1]);
    m = twice_minus<R>(v[0], p);
  } else {
    bfly<R>(v[0], v[1], p, m);
  }
  v[0] = p;
  v[1] = m;
}

// 4-point DFT of (a0, w_a a1, w_b a2, w_c a3) where the pairs (a0, a2) and
// (a1, a3) form the first butterfly layer.  Outputs in natural order.
// Z (untwiddled only): bit i set = input a_i is known to be zero (a
// zero-padded position), so its first-layer additions are skipped.
template <typename R, bool INV, bool TW, unsigned Z = 0u>
__device__ __forceinline__ void rad4_core(C2<R> a0, C2<R> a1, C2<R> a2, C2<R> a3, C2<R> w1, C2<R> w2, C2<R> w3,
                                          C2<R>& y0, C2<R>& y1, C2<R>& y2, C2<R>& y3) {
  static_assert(!TW || Z == 0u, "known-zero inputs only in untwiddled stages");
  C2<R> t0, t1, t2, t3;
  if constexpr (!TW && (Z & 5u) != 0u) {
    if constexpr (Z & 4u) { t0 = a0; t1 = a0; } else { t0 = a2; t1 = cmk<R>(-a2.x, -a2.y); }
    if constexpr (Z & 10u) {
      if constexpr (Z & 8u) { t2 = a1; t3 = a1; } else { t2 = a3; t3 = cmk<R>(-a3.x, -a3.y); }
    } else {
      bfly<R>(a1, a3, t2, t3);
    }
  } else if constexpr (!TW && (Z & 10u) != 0u) {
    bfly<R>(a0, a2, t0, t1);
    if constexpr (Z & 8u) { t2 = a1; t3 = a1; } else { t2 = a3; t3 = cmk<R>(-a3.x, -a3.y); }
  } else if (TW) {
    t0 = tw_fma<R, INV>(a0, w2, a2);
    t1 = twice_minus<R>(a0, t0);
    const C2<R> b1 = tw_mul<R, INV>(w1, a1);
    t2 = tw_fma<R, INV>(b1, w3, a3);
    t3 = twice_minus<R>(b1, t2);
  } else {
    bfly<R>(a0, a2, t0, t1);
    bfly<R>(a1, a3, t2, t3);
  }
  t3 = rot<R, INV>(t3);
  bfly<R>(t0, t2, y0, y2);
  bfly<R>(t1, t3, y1, y3);
}

template <typename R, bool INV, bool TW, unsigned Z = 0u>
__device__ __forceinline__ void rad4(C2<R>* v, const C2<R>* w) {
  rad4_core<R, INV, TW, Z>(v[0], v[1], v[2], v[3], w[1], w[2], w[3], v[0], v[1], v[2], v[3]);
}

template <typename R, bool INV, bool TW>
__device__ __forceinline__ void rad3(C2<R>* v, const C2<R>* w) {
  const R c = R(0.86602540378443864676372317075293618);  // sqrt(3)/2
  C2<R> t, d;
  if (TW) {
    const C2<R> b1 = tw_mul<R, INV>(w[1], v[1]);
    t = tw_fma<R, INV>(b1, w[2], v[2]);   // v1 + v2
    d = twice_minus<R>(b1, t);            // v1 - v2
  } else {
    bfly<R>(v[1], v[2], t, d);
  }
  const C2<R> a0 = v[0];
  const C2<R> m = cmk<R>(fma(R(-0.5), t.x, a0.x), fma(R(-0.5), t.y, a0.y));
  v[0] = cadd<R>(a0, t);
  if (INV) {
    v[1] = cmk<R>(fma(-c, d.y, m.x), fma(c, d.x, m.y));
    v[2] = cmk<R>(fma(c, d.y, m.x), fma(-c, d.x, m.y));
  } else {
    v[1] = cmk<R>(fma(c, d.y, m.x), fma(-c, d.x, m.y));
    v[2] = cmk<R>(fma(-c, d.y, m.x), fma(c, d.x, m.y));
  }
}

// radix-8 = two 4-point DFTs (even / odd inputs) and a W8 layer.  Z: known-zero
// inputs (bit r for v[r]) of an untwiddled stage.
template <int B0, int B1, int B2, int B3>
__host__ __device__ constexpr unsigned zbits4(unsigned z) {
  return ((z >> B0) & 1u) | (((z >> B1) & 1u) << 1) | (((z >> B2) & 1u) << 2) | (((z >> B3) & 1u) << 3);
}
template <typename R, bool INV, bool TW, unsigned Z = 0u>
__device__ __forceinline__ void rad8(C2<R>* v, const C2<R>* w) {
  const R h = R(0.70710678118654752440084436210484904);  // sqrt(2)/2
  const C2<R> one = cmk<R>(R(1), R(0));
  C2<R> e0, e1, e2, e3, o0, o1, o2, o3;
  // even inputs v0, v2, v4, v6 (twiddles w0 = 1, w2, w4, w6)
  rad4_core<R, INV, TW, zbits4<0, 2, 4, 6>(Z)>(v[0], v[2], v[4], v[6], TW ? w[2] : one, TW ? w[4] : one,
                                              TW ? w[6] : one, e0, e1, e2, e3);
  // odd inputs v1, v3, v5, v7: fold w1 into the first pair's base
  if (TW) {
    const C2<R> b1 = tw_mul<R, INV>(w[1], v[1]);
    const C2<R> b3 = tw_mul<R, INV>(w[3], v[3]);
    C2<R> t0 = tw_fma<R, INV>(b1, w[5], v[5]);
    C2<R> t1 = twice_minus<R>(b1, t0);
    C2<R> t2 = tw_fma<R, INV>(b3, w[7], v[7]);
    C2<R> t3 = twice_minus<R>(b3, t2);
    t3 = rot<R, INV>(t3);
    bfly<R>(t0, t2, o0, o2);
    bfly<R>(t1, t3, o1, o3);
  } else {
    rad4_core<R, INV, false, zbits4<1, 3, 5, 7>(Z)>(v[1], v[3], v[5], v[7], one, one, one, o0, o1, o2, o3);
  }
  // W8 layer
  bfly<R>(e0, o0, v[0], v[4]);
  const C2<R> r2 = rot<R, INV>(o2);
  bfly<R>(e2, r2, v[2], v[6]);
  // W8^1 o1 = h (s + i d)
  R s1, d1, s3, d3;
  if (INV) {
    s1 = o1.x - o1.y; d1 = o1.x + o1.y;
    s3 = -(o3.x + o3.y); d3 = o3.x - o3.y;
  } else {
    s1 = o1.x + o1.y; d1 = o1.y - o1.x;
    s3 = o3.y - o3.x; d3 = -(o3.x + o3.y);
  }
  v[1] = cmk<R>(fma(h, s1, e1.x), fma(h, d1, e1.y));
  v[5] = cmk<R>(fma(-h, s1, e1.x), fma(-h, d1, e1.y));
  v[3] = cmk<R>(fma(h, s3, e3.x), fma(h, d3, e3.y));
  v[7] = cmk<R>(fma(-h, s3, e3.x), fma(-h, d3, e3.y));
}

// radix-16 = 4 x 4: 4-point DFTs over n1 of x[n1 + 4 n2] (stage twiddles fused),
// internal twiddles W16^(n1 k2) fused into the second layer, output
// X[4 k1 + k2] from the k2-th second-layer DFT.
template <typename R, bool INV, bool TW>
__device__ __forceinline__ void rad16(C2<R>* v, const C2<R>* w) {
  const R c1 = R(0.92387953251128675612818318939678829);   // cos(pi/8)
  const R s1 = R(0.38268343236508977172845998403039887);   // sin(pi/8)
  const R h = R(0.70710678118654752440084436210484904);
  const C2<R> one = cmk<R>(R(1), R(0));
  C2<R> y[4][4];
#pragma unroll
  for (int n1 = 0; n1 < 4; ++n1) {
    C2<R> a0 = v[n1];
    if (TW && n1 > 0) a0 = tw_mul<R, INV>(w[n1], a0);
    rad4_core<R, INV, TW>(a0, v[n1 + 4], v[n1 + 8], v[n1 + 12], TW ? w[n1 + 4] : one, TW ? w[n1 + 8] : one,
                          TW ? w[n1 + 12] : one, y[n1][0], y[n1][1], y[n1][2], y[n1][3]);
  }
  // forward W16^m (m = n1 k2): conjugated for the inverse by tw_fma/tw_mul<INV>
  const C2<R> W1 = cmk<R>(c1, -s1), W2 = cmk<R>(h, -h), W3 = cmk<R>(s1, -c1), W4 = cmk<R>(R(0), R(-1));
  const C2<R> W6 = cmk<R>(-h, -h), W9 = cmk<R>(-c1, s1);
  C2<R> x[4];
  rad4_core<R, INV, false>(y[0][0], y[1][0], y[2][0], y[3][0], one, one, one, x[0], x[1], x[2], x[3]);
  v[0] = x[0]; v[4] = x[1]; v[8] = x[2]; v[12] = x[3];
  rad4_core<R, INV, true>(y[0][1], y[1][1], y[2][1], y[3][1], W1, W2, W3, x[0], x[1], x[2], x[3]);
  v[1] = x[0]; v[5] = x[1]; v[9] = x[2]; v[13] = x[3];
  rad4_core<R, INV, true>(y[0][2], y[1][2], y[2][2], y[3][2], W2, W4, W6, x[0], x[1], x[2], x[3]);
  v[2] = x[0]; v[6] = x[1]; v[10] = x[2]; v[14] = x[3];
  rad4_core<R, INV, true>(y[0][3], y[1][3], y[2][3], y[3][3], W3, W6, W9, x[0], x[1], x[2], x[3]);
  v[3] = x[0]; v[7] = x[1]; v[11] = x[2]; v[15] = x[3];
}

// ---------------------------------------------------------------------------
// Compile-time twiddles for the composite radices: cos and sin of 2 pi m / n
// from Taylor series on [0, pi/4] after an exact octant reduction in integers.
// ---------------------------------------------------------------------------
__host__ __device__ constexpr double ct_sin_red(double x) {
  double term = x, sum = x;
  for (int k = 1; k < 14; ++k) {
    term *= -x * x / (double)((2 * k) * (2 * k + 1));
    sum += term;
  }
  return sum;
}
__host__ __device__ constexpr double ct_cos_red(double x) {
  double term = 1.0, sum = 1.0;
  for (int k = 1; k < 14; ++k) {
    term *= -x * x / (double)((2 * k - 1) * (2 * k));
    sum += term;
  }
  return sum;
}
// (cos, sin)(2 pi m / n): angle = (pi/4) (oct + rem/n) with oct = 8m div n
__host__ __device__ constexpr double ct_trig(int m, int n, bool want_sin) {
  const double quarter_pi = 0.78539816339744830961566084581987572;
  m %= n;
  if (m < 0) m += n;
  const long long t = 8LL * m;
  int oct = (int)(t / n);
  const long long rem = t - (long long)oct * n;
  double c = 0.0, s = 0.0;
  int q = 0;
  if (oct % 2 == 0) {           // q quarter turns + phi, phi in [0, pi/4)
    const double phi = quarter_pi * (double)rem / (double)n;
    c = ct_cos_red(phi);
    s = ct_sin_red(phi);
    q = oct / 2;
  } else {                      // q quarter turns - psi, psi in (0, pi/4]
    const double psi = quarter_pi * (double)(n - rem) / (double)n;
    c = ct_cos_red(psi);
    s = -ct_sin_red(psi);
    q = (oct + 1) / 2;
  }
  double rc = c, rs = s;        // rotate (c, s) by q quarter turns
  if (q % 4 == 1) { rc = -s; rs = c; }
  if (q % 4 == 2) { rc = -c; rs = -s; }
  if (q % 4 == 3) { rc = s; rs = -c; }
  return want_sin ? rs : rc;
}
// forward twiddle W_n^m = exp(-2 pi i m / n) as a compile-time constant
template <int M, int NN> struct CTw {
  static constexpr double c = ct_trig(M, NN, false);
  static constexpr double s = -ct_trig(M, NN, true);
};

// Compile-time loop: f(std::integral_constant<int, i>) for i = 0..N-1.
template <class F, int... I>
__device__ __forceinline__ void sfor_impl(F&& f, std::integer_sequence<int, I...>) {
  (f(std::integral_constant<int, I>{}), ...);
}
template <int N, class F>
__device__ __forceinline__ void sfor(F&& f) {
  sfor_impl(f, std::make_integer_sequence<int, N>{});
}

// Z: bit r set = input v[r] is known to be zero (untwiddled radix-8/4 stages
// skip its first-layer additions; other radices ignore it).
template <typename R, bool INV, int RAD, bool TW, unsigned Z = 0u>
__device__ __forceinline__ void dft(C2<R>* v, const C2<R>* w);

// Composite radix RAD = A * B in registers (Cooley-Tukey): n = b + B a,
// k = kA + A kB.  A-point DFTs over a (stage twiddles fused), then B-point
// DFTs over b with the internal twiddles W_RAD^(b kA) fused.
template <int RAD> __host__ __device__ constexpr int comp_a() {
  return RAD == 6 ? 3 : RAD == 12 ? 4 : RAD == 24 ? 8 : RAD == 32 ? 8 : RAD == 48 ? 16 : 0;
}

template <typename R, bool INV, int RAD, bool TW>
__device__ __forceinline__ void dft_comp(C2<R>* v, const C2<R>* w) {
  constexpr int A = comp_a<RAD>();
  constexpr int B = RAD / A;
  static_assert(A > 0 && A * B == RAD, "unsupported composite radix");
  C2<R> y[B][A];
#pragma unroll
  for (int b = 0; b < B; ++b) {
    C2<R> t[A], tw[A];
#pragma unroll
    for (int a = 0; a < A; ++a) t[a] = v[b + B * a];
    if (TW) {
#pragma unroll
      for (int a = 1; a < A; ++a) tw[a] = w[b + B * a];
      if (b > 0) t[0] = tw_mul<R, INV>(w[b], t[0]);
    }
    dft<R, INV, A, TW>(t, tw);
#pragma unroll
    for (int k = 0; k < A; ++k) y[b][k] = t[k];
  }
  sfor<A>([&](auto kac) {
    constexpr int KA = decltype(kac)::value;
    C2<R> t[B], tw[B];
#pragma unroll
    for (int b = 0; b < B; ++b) t[b] = y[b][KA];
    if constexpr (KA == 0) {
      dft<R, INV, B, false>(t, tw);
    } else {
      sfor<B>([&](auto bc) {
        constexpr int BB = decltype(bc)::value;
        tw[BB] = cmk<R>((R)CTw<BB * KA, RAD>::c, (R)CTw<BB * KA, RAD>::s);
      });
      dft<R, INV, B, true>(t, tw);
    }
#pragma unroll
    for (int k = 0; k < B; ++k) v[KA + A * k] = t[k];
  });
}

template <typename R, bool INV, int RAD, bool TW, unsigned Z>
__device__ __forceinline__ void dft(C2<R>* v, const C2<R>* w) {
  if constexpr (comp_a<RAD>() > 0) {
    dft_comp<R, INV, RAD, TW>(v, w);
  } else if constexpr (RAD == 16) {
    rad16<R, INV, TW>(v, w);
  } else if constexpr (RAD == 8) {
    rad8<R, INV, TW, TW ? 0u : Z>(v, w);
  } else if constexpr (RAD == 4) {
    rad4<R, INV, TW, TW ? 0u : Z>(v, w);
  } else if constexpr (RAD == 3) {
    rad3<R, INV, TW>(v, w);
  } else {
    rad2<R, INV, TW>(v, w);
  }
}

// ---------------------------------------------------------------------------
// Stockham stages.  Element p of line l lives at buf[l*ld_line + p*ld_elem],
// or, for contiguous lines (ZPAD), at buf[l*ld_line + zi(p)] with one padding
// element after every 8: the first stage writes at stride RAD, which would
// otherwise put most lanes of a warp on the same shared-memory banks.
// LINE_FAST: consecutive threads take consecutive lines (use when lines are
// interleaved, ld_line == 1); otherwise consecutive butterflies of a line.
// ---------------------------------------------------------------------------
// one padding element per 128-byte row of the line: 8 complex doubles or 16
// complex floats
template <typename R> __host__ __device__ constexpr int zrow() { return 128 / (2 * (int)sizeof(R)); }
template <typename R> __host__ __device__ constexpr int zi(int p) { return p + p / zrow<R>(); }
template <typename R> __host__ __device__ constexpr int zpad_len(int L) { return L + L / zrow<R>(); }

template <typename R, int L, bool INV, int NT, int NLINES, bool LINE_FAST, int S, int NS, bool ZPAD = false>
struct StockhamStage {
  __device__ __forceinline__ static void run(C2<R>* buf, int ld_line, int ld_elem,
                                             const C2<R>* __restrict__ tw) {
    constexpr int RAD = radix_of<R>(L, S);
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
        for (int r = 0; r < RAD; ++r) v[q][r] = src[ZPAD ? zi<R>(j + r * NB) : (j + r * NB) * ld_elem];
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
        C2<R> w[RAD];
        if (S > 0) {
#pragma unroll
          for (int r = 1; r < RAD; ++r) w[r] = tw[r * k * TWS];
        }
        dft<R, INV, RAD, (S > 0)>(v[q], w);
        C2<R>* dst = buf + l * ld_line;
        const int base = (j - k) * RAD + k;
#pragma unroll
        for (int r = 0; r < RAD; ++r) dst[ZPAD ? zi<R>(base + r * NS) : (base + r * NS) * ld_elem] = v[q][r];
      }
    }
    __syncthreads();
    if constexpr (S + 1 < stages_of<R>(L)) {
      StockhamStage<R, L, INV, NT, NLINES, LINE_FAST, S + 1, NS * RAD, ZPAD>::run(buf, ld_line, ld_elem, tw);
    }
  }
};

// Transform NLINES lines held in shared memory.  Must be called by all NT
// threads of the CTA; begins and ends with the data synchronised.
template <typename R, int L, bool INV, int NT, int NLINES, bool LINE_FAST, bool ZPAD = false>
__device__ __forceinline__ void fft_smem(C2<R>* buf, int ld_line, int ld_elem,
                                         const C2<R>* __restrict__ tw) {
  static_assert(stages_of<R>(L) > 0, "unsupported FFT length");
  StockhamStage<R, L, INV, NT, NLINES, LINE_FAST, 0, 1, ZPAD>::run(buf, ld_line, ld_elem, tw);
}

// Contiguous padded lines of length L (line stride zpad_len(L)).
template <typename R, int L, bool INV, int NT, int NLINES>
__device__ __forceinline__ void fft_zlines(C2<R>* buf, const C2<R>* __restrict__ tw) {
  fft_smem<R, L, INV, NT, NLINES, false, true>(buf, zpad_len<R>(L), 1, tw);
}

}  // namespace vk
