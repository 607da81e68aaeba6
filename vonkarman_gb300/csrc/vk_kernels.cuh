// Pass kernels of the periodic pseudospectral step.
//
// Layouts (all complex arrays interleaved {re, im}, z index fastest):
//   spectral state     (N, N, H)     [ix][iy][iz]     H = N/2 + 1
//   after P1           (M, N, H) x 5 [x][iy][iz]      M = 3N/2
//   after P2           (M, M, H) x 6 [x][y][iz]
//   after P3           (M, M, H) x 3 [x][y][iz]
//   after P4           (M, N, H) x 3 [x][iy][iz]
// The spectral state keeps the reference's ndarray C order
// (vonkarman-core/src/field.rs:48-50), so host upload/download is a copy.
//
// One nonlinear evaluation N(u) = P[F(u x curl u)] with 3/2 padding
// (vonkarman-periodic/src/nonlinear.rs:15-39, vonkarman-fft/src/dealiased.rs:16-110)
// is the pass chain P1..P5:
//   P1  x-inverse of u and of i*kx*u_{y,z}, zero-pad N->M along x  (5 fields)
//   P2  y-inverse with zero-pad, forming u and omega = i k x u     (6 fields)
//   P3  z: C2R of u, omega (packed pairwise), u x omega, R2C, keep H modes
//   P4  y-forward, keep N of M modes
//   P5  x-forward, keep N of M modes, scale, Leray projection, stage epilogue
// The padded spectral arrays of the reference are never materialised.
#pragma once

#include "vk_fft.cuh"

namespace vk {

// ---------------------------------------------------------------------------
// Index helpers
// ---------------------------------------------------------------------------
// L2 prefetch hints for the inputs of a CTA that starts later (the one a
// residency wave ahead), so that its first-stage loads hit L2 instead of
// DRAM: one cache line, or a 16-byte-aligned range whose size is a multiple
// of 16 bytes (bulk form).  Hints only: nothing is returned or waited for.
__device__ __forceinline__ void prefetch_l2(const void* p) {
  asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}
__device__ __forceinline__ void prefetch_l2_bulk(const void* p, unsigned bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}


// padded position -> N-grid index, or -1 for a zero-padded slot
// (inverse of dealiased.rs:129-131)
__device__ __forceinline__ int unpad_pos(int p, int N, int M) {
  if (p < N / 2) return p;
  if (p >= M - N / 2) return p - (M - N);
  return -1;
}
// N-grid index -> padded position (dealiased.rs:129-131, :151-157)
__device__ __forceinline__ int pad_pos(int i, int N, int M) { return i < N / 2 ? i : M - (N - i); }
// rfftfreq_full index -> integer wavenumber, n/2 -> -n/2 (spectral_ops.rs:51-63)
__device__ __forceinline__ int signed_k(int i, int N) { return i < N / 2 ? i : i - N; }

__host__ __device__ constexpr int cmin(int a, int b) { return a < b ? a : b; }
__host__ __device__ constexpr int cmax(int a, int b) { return a > b ? a : b; }
__host__ __device__ constexpr int round32(int a) { return (a + 31) / 32 * 32; }

// z passes: column pairs per CTA so that CP * L == 768 (z-cross) / 512 (N grid)
template <int L, int TARGET> __host__ __device__ constexpr int zpairs() { return cmax(1, TARGET / L); }
template <typename R, int NLINES, int L>
__host__ __device__ constexpr int zthreads() { return cmax(64, cmin(1024, round32(NLINES * L / max_radix<R>(L)))); }
// Minimum resident CTAs per SM requested from the compiler: enough for 24
// warps per SM, which caps registers near 85 per thread.
template <int NT> __host__ __device__ constexpr int min_blocks() { return cmax(1, 768 / NT); }

// Grid sizes of a strided-pass op: compile-time when the op is instantiated
// for one grid (GN > 0: N = GN, padded length M = GM, H = GN/2 + 1), so that
// the zero-padding tests and index products fold per butterfly input; else
// the runtime members N, M, hz.  Offsets inside one field fit in int (at most
// (3N/2)^2 (N/2+1) < 2^31 elements for N <= 1024); the field base stays size_t.
#define VK_GRID_DIMS(GN, GM)                                                            \
  __host__ __device__ __forceinline__ int n_() const { return GN > 0 ? GN : N; }        \
  __host__ __device__ __forceinline__ int m_() const { return GN > 0 ? GM : M; }        \
  __host__ __device__ __forceinline__ int h_() const { return GN > 0 ? GN / 2 + 1 : hz; }
// Zero-padded input positions [ZERO_LO, ZERO_HI) of the inverse passes with
// the 3/2 pad (compile-time grids only).
#define VK_PAD_ZEROS(GN, GM)                                                            \
  static constexpr int ZERO_LO = GN > 0 && GN != GM ? GN / 2 : 0;                       \
  static constexpr int ZERO_HI = GN > 0 && GN != GM ? GM - GN / 2 : 0;

// P1 / N-grid X: x-inverse of the spectral state, zero-pad N -> M (M == N on
// the N grid).  Fields: 0..2 = u_c, 3 = i kx u_y, 4 = i kx u_z.  s_in folds the
// 1/M^3 of the padded c2r and the (M/N)^3 pre-scale (dealiased.rs:43,:45-62)
// into one factor 1/N^3.  Kinds: 0 = u_c, 1 = i kx u.
template <typename R, int GN = 0, int GM = 0> struct OpXInv {
  int nfields, hz;
  int N, M;
  R s_in, ks;
  const C2<R>* in; size_t cs;
  C2<R>* out; size_t fs;
  static constexpr int NKIND = 2;
  VK_GRID_DIMS(GN, GM)
  VK_PAD_ZEROS(GN, GM)
  __host__ __device__ __forceinline__ int kind(int f) const { return f < 3 ? 0 : 1; }
  __host__ __device__ __forceinline__ int src_component(int f) const { return f < 3 ? f : f - 2; }
  // L2 prefetch of row t of the input tile of field f, lines [lam0, lam0 + nl)
  // (the tile's rows are whole 128-byte lines)
  __device__ __forceinline__ void prefetch_row(int f, int lam0, int, int t) const {
    if (t < n_()) prefetch_l2(in + (size_t)src_component(f) * cs + (size_t)t * n_() * h_() + lam0);
  }
  template <int K> __device__ __forceinline__ C2<R> load(int f, int iy, int z, int p) const {
    const int ix = unpad_pos(p, n_(), m_());
    const int c = K == 0 ? f : f - 2;
    return ix < 0 ? czero<R>() : in[(size_t)c * cs + ((ix * n_() + iy) * h_() + z)];
  }
  template <int K> __device__ __forceinline__ C2<R> prep(int, int, int, int p, C2<R> v) const {
    v = cscale<R>(v, s_in);
    if constexpr (K == 1) {
      const int ix = unpad_pos(p, n_(), m_());
      const R kx = ks * (R)signed_k(ix < 0 ? 0 : ix, n_());
      v = cmk<R>(-kx * v.y, kx * v.x);
    }
    return v;
  }
  __device__ __forceinline__ int out_index(int p) const { return p; }
  __device__ __forceinline__ void store(int f, int iy, int z, int i, C2<R> v) const {
    out[(size_t)f * fs + ((i * n_() + iy) * h_() + z)] = v;
  }
};

// P2 / N-grid Y: y-inverse with zero-pad, forming u (g = 0..2) and
// omega = i k x u (g = 3..5) from the x-transformed fields
// (curl: vonkarman-core/src/spectral_ops.rs:81-108).  kx was applied in P1, ky
// and kz are applied here (both are constant along an x line).  Kind 0 = u
// (one load per position).  Omega needs two operand fields per position:
// in FP32 one kind (1) loads both raw operands (issued before any arithmetic,
// in chunks) and forms omega in prep; in FP64, whose registers the raw pairs
// would overflow, kinds 1..3 (g = 3..5) combine them at the load.
template <typename R, int GN = 0, int GM = 0> struct OpYInv {
  int nfields, hz;
  int N, M, gbase;
  R ks;
  const C2<R>* in; size_t fsin;   // (M, N, H): Ux, Uy, Uz, Vy, Vz
  C2<R>* out; size_t fsout;       // (M, M, H)
  static constexpr int MAX_L16 = 384;   // 16-line tiles up to this length (FP32; longer ones spill)
  static constexpr int NKIND = sizeof(R) == 4 ? 2 : 4;
  VK_GRID_DIMS(GN, GM)
  VK_PAD_ZEROS(GN, GM)
  __host__ __device__ __forceinline__ int kind(int f) const {
    const int g = f + gbase;
    return g < 3 ? 0 : sizeof(R) == 4 ? 1 : g - 2;
  }
  // operands of omega_g: g = 3: (Uy, Uz); g = 4: (Ux, Vz); g = 5: (Ux, Vy)
  __device__ __forceinline__ static int opa(int g) { return g == 3 ? 1 : 0; }
  __device__ __forceinline__ static int opb(int g) { return g == 3 ? 2 : g == 4 ? 4 : 3; }
  __device__ __forceinline__ C2<R> omega(int g, int z, int iy, const C2x2<R>& r) const {
    const R ky = ks * (R)signed_k(iy, n_());
    const R kz = ks * (R)z;
    if (g == 3) return cmul_i<R>(cmk<R>(ky * r.b.x - kz * r.a.x, ky * r.b.y - kz * r.a.y));  // i (ky Uz - kz Uy)
    if (g == 4) return cmk<R>(-kz * r.a.y - r.b.x, kz * r.a.x - r.b.y);                     // i kz Ux - Vz
    return cmk<R>(r.b.x + ky * r.a.y, r.b.y - ky * r.a.x);                                  // Vy - i ky Ux
  }
  template <int K> __device__ __forceinline__ auto load(int f, int x, int z, int p) const {
    const int iy = unpad_pos(p, n_(), m_());
    const C2<R>* s = in + ((x * n_() + (iy < 0 ? 0 : iy)) * h_() + z);
    if constexpr (K == 0) {
      return iy < 0 ? czero<R>() : s[(size_t)(f + gbase) * fsin];
    } else if constexpr (sizeof(R) == 8) {
      constexpr int g = K + 2;
      if (iy < 0) return czero<R>();
      C2x2<R> r;
      r.a = s[(size_t)opa(g) * fsin];
      r.b = s[(size_t)opb(g) * fsin];
      return omega(g, z, iy, r);
    } else {
      const int g = f + gbase;
      C2x2<R> r{};
      if (iy >= 0) {
        r.a = s[(size_t)opa(g) * fsin];
        r.b = s[(size_t)opb(g) * fsin];
      }
      return r;
    }
  }
  template <int K> __device__ __forceinline__ C2<R> prep(int, int, int, int, C2<R> v) const { return v; }
  template <int K> __device__ __forceinline__ C2<R> prep(int f, int, int z, int p, const C2x2<R>& r) const {
    const int iy = unpad_pos(p, n_(), m_());
    return omega(f + gbase, z, iy < 0 ? 0 : iy, r);
  }
  __device__ __forceinline__ int out_index(int p) const { return p; }
  __device__ __forceinline__ void store(int f, int x, int z, int i, C2<R> v) const {
    out[(size_t)f * fsout + ((x * m_() + i) * h_() + z)] = v;
  }
};

// P4: y-forward of the three cross-product fields, keep N of M modes
// (truncate_spectral, dealiased.rs:141-163).
template <typename R, int GN = 0, int GM = 0> struct OpYFwdTrunc {
  int nfields, hz;
  int N, M;
  const C2<R>* in; size_t fsin;   // (M, M, H)
  C2<R>* out; size_t fsout;       // (M, N, H)
  static constexpr int NKIND = 1;
  VK_GRID_DIMS(GN, GM)
  __host__ __device__ __forceinline__ int kind(int) const { return 0; }
  template <int K> __device__ __forceinline__ C2<R> load(int f, int x, int z, int p) const {
    return in[(size_t)f * fsin + ((x * m_() + p) * h_() + z)];
  }

  template <int K> __device__ __forceinline__ C2<R> prep(int, int, int, int, C2<R> v) const { return v; }
  __device__ __forceinline__ int out_index(int p) const { return unpad_pos(p, n_(), m_()); }
  __device__ __forceinline__ void store(int f, int x, int z, int i, C2<R> v) const {
    out[(size_t)f * fsout + ((x * n_() + i) * h_() + z)] = v;
  }
};

// Standalone FFT backend: C2C along x (AXIS 0) or y (AXIS 1) of an
// (nx, ny, hz) complex array, in place.
template <typename R, int AXIS> struct OpPlainC2C {
  int nfields, hz;
  int nx, ny;
  C2<R>* data;
  static constexpr int NKIND = 1;
  static constexpr int MAX_L16 = 384;   // 16-line tiles up to this length (FP32; longer ones spill)
  __host__ __device__ __forceinline__ int h_() const { return hz; }
  __host__ __device__ __forceinline__ int kind(int) const { return 0; }
  __device__ __forceinline__ size_t at(int outer, int z, int p) const {
    return AXIS == 0 ? ((size_t)p * ny + outer) * hz + z : ((size_t)outer * ny + p) * hz + z;
  }
  template <int K> __device__ __forceinline__ C2<R> load(int, int outer, int z, int p) const {
    return data[at(outer, z, p)];
  }
  template <int K> __device__ __forceinline__ C2<R> prep(int, int, int, int, C2<R> v) const { return v; }
  __device__ __forceinline__ int out_index(int p) const { return p; }
  __device__ __forceinline__ void store(int, int outer, int z, int i, C2<R> v) const { data[at(outer, z, i)] = v; }
};

// ---------------------------------------------------------------------------
// Stage epilogues (fused into P5).  Reference forms:
//   ETD-RK4 reference variant  vonkarman-periodic/src/solver.rs:221-379
//   classical RK4              vonkarman-periodic/src/rk4.rs:16-146
// ETD coefficients live in a table keyed by the integer |k|^2 index
// m = kx'^2 + ky'^2 + kz'^2 (8 doubles per entry).
// ---------------------------------------------------------------------------
template <typename R>
__device__ __forceinline__ C2<R> axpby(R a, C2<R> x, R b, C2<R> y) {
  return cmk<R>(a * x.x + b * y.x, a * x.y + b * y.y);
}

// The final stage of a step raises the context's sticky non-finite flag when
// it writes a NaN or an infinity (the NaN check of the reference's audit,
// vonkarman-diag/src/audit.rs:175-197, without a readback); the atomic runs
// only on that rare path.
template <typename R>
__device__ __forceinline__ void flag_nonfinite(const StageArgs<R>& s, C2<R> v) {
  if (!(isfinite(v.x) && isfinite(v.y)) && s.nonfinite) atomicOr(s.nonfinite, 1);
}

// Stage epilogue of NM modes at once: the inputs of all modes and all three
// components are loaded before any result is stored (a store may alias a
// later load as far as the compiler knows, so interleaving them would
// serialise the loads).  ok[q] = false skips mode q.
// KEEP: the final stages (ST_ETD_4, ST_RK4_4) also return the new state of
// each mode in un[q][c] (for diagnostics fused into the same pass).
template <typename R, int NM, bool KEEP = false>
__device__ __forceinline__ void stage_apply_n(const StageArgs<R>& s, const size_t* idx, const int* m, const R* k2,
                                              const C2<R> (*nl)[3], const bool* ok, C2<R> (*un)[3] = nullptr) {
  const size_t cs = s.cs;
  if (s.op == ST_NL_OUT) {
#pragma unroll
    for (int q = 0; q < NM; ++q) {
      if (!ok[q]) continue;
#pragma unroll
      for (int c = 0; c < 3; ++c) s.out[c * cs + idx[q]] = nl[q][c];
    }
    return;
  }
  const double dt = *s.dt;
  C2<R> u[NM][3];
#pragma unroll
  for (int q = 0; q < NM; ++q) {
#pragma unroll
    for (int c = 0; c < 3; ++c) u[q][c] = ok[q] ? s.u[c * cs + idx[q]] : czero<R>();
  }
  if (s.op >= ST_RK4_1) {
    // rhs = N + (-nu k^2) state  (rk4.rs:30-45)
    const R half = (R)(0.5 * dt);
    C2<R> st[NM][3], a[NM][3];
#pragma unroll
    for (int q = 0; q < NM; ++q) {
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const bool rd = ok[q] && s.op != ST_RK4_1;
        st[q][c] = rd ? s.temp[c * cs + idx[q]] : u[q][c];
        a[q][c] = rd ? s.acc[c * cs + idx[q]] : czero<R>();
      }
    }
#pragma unroll
    for (int q = 0; q < NM; ++q) {
      if (!ok[q]) continue;
      const R visc = (R)(-s.nu) * k2[q];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const size_t i = c * cs + idx[q];
        const C2<R> rhs = cmk<R>(nl[q][c].x + visc * st[q][c].x, nl[q][c].y + visc * st[q][c].y);
        if (s.op == ST_RK4_1) {
          s.acc[i] = rhs;
          s.temp[i] = cmk<R>(u[q][c].x + half * rhs.x, u[q][c].y + half * rhs.y);
        } else if (s.op == ST_RK4_2 || s.op == ST_RK4_3) {
          s.acc[i] = cmk<R>(a[q][c].x + R(2) * rhs.x, a[q][c].y + R(2) * rhs.y);
          const R h = s.op == ST_RK4_2 ? half : (R)dt;
          s.temp[i] = cmk<R>(u[q][c].x + h * rhs.x, u[q][c].y + h * rhs.y);
        } else {
          const R sixth = (R)(dt / 6.0);
          const C2<R> v = cmk<R>(u[q][c].x + sixth * (a[q][c].x + rhs.x), u[q][c].y + sixth * (a[q][c].y + rhs.y));
          s.u[i] = v;
          flag_nonfinite<R>(s, v);
          if constexpr (KEEP) un[q][c] = v;
        }
      }
    }
    return;
  }
  // ETD coefficients of each mode (table keyed by the |k|^2 index)
  const double* e[NM];
#pragma unroll
  for (int q = 0; q < NM; ++q) e[q] = s.etd + (size_t)(ok[q] ? m[q] : 0) * ETD_STRIDE;
  switch (s.op) {
    case ST_ETD_REF_1:    // solver.rs:264-281
    case ST_ETD_CM_1: {   // textbook: a = E2 u + (h/2) phi1(z/2) N1
      const double f = s.op == ST_ETD_REF_1 ? dt : 0.5 * dt;
      R eh[NM], qq[NM];
#pragma unroll
      for (int q = 0; q < NM; ++q) { eh[q] = (R)e[q][E_HALF]; qq[q] = (R)(f * e[q][E_A21]); }
#pragma unroll
      for (int q = 0; q < NM; ++q) {
        if (!ok[q]) continue;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          s.n1[c * cs + idx[q]] = nl[q][c];
          s.temp[c * cs + idx[q]] = axpby<R>(eh[q], u[q][c], qq[q], nl[q][c]);
        }
      }
      break;
    }
    case ST_ETD_REF_2:    // solver.rs:291-308; acc starts the final sum
    case ST_ETD_CM_2: {   // b = E2 u + (h/2) phi1(z/2) N2
      const double f = s.op == ST_ETD_REF_2 ? dt : 0.5 * dt;
      R b1[NM], b23[NM], eh[NM], qq[NM];
      C2<R> n1[NM][3];
#pragma unroll
      for (int q = 0; q < NM; ++q) {
        b1[q] = (R)e[q][E_B1]; b23[q] = (R)e[q][E_B23]; eh[q] = (R)e[q][E_HALF]; qq[q] = (R)(f * e[q][E_A21]);
#pragma unroll
        for (int c = 0; c < 3; ++c) n1[q][c] = ok[q] ? s.n1[c * cs + idx[q]] : czero<R>();
      }
#pragma unroll
      for (int q = 0; q < NM; ++q) {
        if (!ok[q]) continue;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          s.acc[c * cs + idx[q]] = axpby<R>(b1[q], n1[q][c], b23[q], nl[q][c]);
          s.temp[c * cs + idx[q]] = axpby<R>(eh[q], u[q][c], qq[q], nl[q][c]);
        }
      }
      break;
    }
    case ST_ETD_REF_3: {  // solver.rs:318-344
      R b23[NM], ef[NM], qq[NM];
      C2<R> n1[NM][3], a[NM][3];
#pragma unroll
      for (int q = 0; q < NM; ++q) {
        b23[q] = (R)e[q][E_B23]; ef[q] = (R)e[q][E_FULL]; qq[q] = (R)(dt * e[q][E_A41]);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          n1[q][c] = ok[q] ? s.n1[c * cs + idx[q]] : czero<R>();
          a[q][c] = ok[q] ? s.acc[c * cs + idx[q]] : czero<R>();
        }
      }
#pragma unroll
      for (int q = 0; q < NM; ++q) {
        if (!ok[q]) continue;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          s.acc[c * cs + idx[q]] = cmk<R>(a[q][c].x + b23[q] * nl[q][c].x, a[q][c].y + b23[q] * nl[q][c].y);
          const C2<R> dn = cmk<R>(R(2) * nl[q][c].x - n1[q][c].x, R(2) * nl[q][c].y - n1[q][c].y);
          s.temp[c * cs + idx[q]] = axpby<R>(ef[q], u[q][c], qq[q], dn);
        }
      }
      break;
    }
    case ST_ETD_4: {  // solver.rs:354-378
      R b4[NM], ef[NM];
      C2<R> a[NM][3];
#pragma unroll
      for (int q = 0; q < NM; ++q) {
        b4[q] = (R)e[q][E_B4]; ef[q] = (R)e[q][E_FULL];
#pragma unroll
        for (int c = 0; c < 3; ++c) a[q][c] = ok[q] ? s.acc[c * cs + idx[q]] : czero<R>();
      }
#pragma unroll
      for (int q = 0; q < NM; ++q) {
        if (!ok[q]) continue;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const C2<R> rhs = cmk<R>(a[q][c].x + b4[q] * nl[q][c].x, a[q][c].y + b4[q] * nl[q][c].y);
          const C2<R> v = axpby<R>(ef[q], u[q][c], (R)dt, rhs);
          s.u_out[c * cs + idx[q]] = v;
          flag_nonfinite<R>(s, v);
          if constexpr (KEEP) un[q][c] = v;
        }
      }
      break;
    }
    case ST_ETD_CM_3: {  // c = E2 a + (h/2) phi1(z/2) (2 N3 - N1), a rebuilt from u, N1
      R b23[NM], eh[NM], qq[NM];
      C2<R> n1[NM][3], ac[NM][3];
#pragma unroll
      for (int q = 0; q < NM; ++q) {
        b23[q] = (R)e[q][E_B23]; eh[q] = (R)e[q][E_HALF]; qq[q] = (R)(0.5 * dt * e[q][E_A21]);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          n1[q][c] = ok[q] ? s.n1[c * cs + idx[q]] : czero<R>();
          ac[q][c] = ok[q] ? s.acc[c * cs + idx[q]] : czero<R>();
        }
      }
#pragma unroll
      for (int q = 0; q < NM; ++q) {
        if (!ok[q]) continue;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          s.acc[c * cs + idx[q]] = cmk<R>(ac[q][c].x + b23[q] * nl[q][c].x, ac[q][c].y + b23[q] * nl[q][c].y);
          const C2<R> av = axpby<R>(eh[q], u[q][c], qq[q], n1[q][c]);
          const C2<R> dn = cmk<R>(R(2) * nl[q][c].x - n1[q][c].x, R(2) * nl[q][c].y - n1[q][c].y);
          s.temp[c * cs + idx[q]] = axpby<R>(eh[q], av, qq[q], dn);
        }
      }
      break;
    }
    default: break;
  }
}




// ---------------------------------------------------------------------------
// z-line helpers.  Two real z lines x, y of length L share one complex line
// Z = x + i y.  Packing from their half spectra X, Y (k = 0..L/2):
//   Z[k] = X[k] + i Y[k],  Z[L-k] = conj(X[k]) + i conj(Y[k]);
// the imaginary parts of X[0] and X[L/2] are dropped, which is the c2r
// convention of the reference backend (ndrustfft_backend.rs:46-57).
// Unpacking after a forward FFT:  X[k] = (Z[k] + conj Z[-k]) / 2,
//                                 Y[k] = (Z[k] - conj Z[-k]) / (2i).
// ---------------------------------------------------------------------------
// Lines are in the padded shared layout (position p at zi<R>(p)).
template <typename R>
__device__ __forceinline__ void zpack(C2<R>* line, int L, int k, C2<R> X, C2<R> Y) {
  if (k == 0 || 2 * k == L) {
    line[zi<R>(k)] = cmk<R>(X.x, Y.x);
  } else {
    line[zi<R>(k)] = cmk<R>(X.x - Y.y, X.y + Y.x);
    line[zi<R>(L - k)] = cmk<R>(X.x + Y.y, Y.x - X.y);
  }
}

template <typename R>
__device__ __forceinline__ void zunpack(const C2<R>* line, int L, int k, C2<R>& X, C2<R>& Y) {
  const C2<R> z = line[zi<R>(k)];
  const C2<R> w = line[zi<R>(k == 0 ? 0 : L - k)];
  X = cmk<R>(R(0.5) * (z.x + w.x), R(0.5) * (z.y - w.y));
  Y = cmk<R>(R(0.5) * (z.y + w.y), R(0.5) * (w.x - z.x));
}

// ---------------------------------------------------------------------------
// P3: per (x, y) column: c2r of u and omega on the padded grid, u x omega,
// r2c, keep iz < H.  Six real fields ride in three complex lines per column:
//   (u_x + i u_y), (u_z + i w_x), (w_y + i w_z).
// After the cross product the three real outputs of two columns ride in three
// lines: (c_x0 + i c_y0), (c_x1 + i c_y1), (c_z0 + i c_z1).
// ---------------------------------------------------------------------------
template <typename R> struct P3Args {
  int ncols;                        // M*M
  const C2<R>* in; size_t fsin;     // 6 fields (M, M, H)
  C2<R>* out; size_t fsout;         // 3 fields (M, M, H)
};

// ---------------------------------------------------------------------------
// N-grid z pass: c2r of u and/or omega (already x/y-inverted and scaled by
// 1/N^3) and max |u|^2, max |omega|^2 over the N^3 grid
// (solver.rs:180-218 and :537-567).  Fields in: (N, N, H) x nf, order
// u_x, u_y, u_z[, w_x, w_y, w_z].  BOTH: 6 fields -> 3 lines per column;
// otherwise 3 fields -> lines (f0_a + i f1_a), (f0_b + i f1_b), (f2_a + i f2_b)
// per column pair.
// ---------------------------------------------------------------------------
template <typename R> struct NZArgs {
  int ncols;                     // N*N
  const C2<R>* in; size_t fs;
  MaxOut* out;
  int which;                     // 1 = u only, 2 = omega only, 3 = both
};

__device__ __forceinline__ void atomic_max_pos(unsigned long long* p, double v) {
  atomicMax(p, (unsigned long long)__double_as_longlong(v));
}


// ---------------------------------------------------------------------------
// Standalone backend z passes (FftBackend::r2c_3d / c2r_3d z stage,
// ndrustfft_backend.rs:33-57).  Real lines of length L, pairs of columns per
// complex line.
// ---------------------------------------------------------------------------
template <typename R> struct FZArgs {
  int ncols;                  // nx*ny
  R* real; C2<R>* cplx;       // (ncols, L) real, (ncols, L/2+1) complex
  R scale;                    // c2r: 1/(nx ny nz)
};

template <typename R, int L, int CP, int NT>
__global__ void __launch_bounds__(NT, min_blocks<NT>()) k_fz_r2c(FZArgs<R> a, const C2<R>* __restrict__ tw) {
  constexpr int H = L / 2 + 1;
  constexpr int LP = zpad_len<R>(L);
  extern __shared__ __align__(16) unsigned char vk_smem[];
  C2<R>* lines = reinterpret_cast<C2<R>*>(vk_smem);
  const int col0 = blockIdx.x * 2 * CP;
  for (int e = threadIdx.x; e < CP * L; e += NT) {
    const int pr = e / L, p = e % L;
    const int c0 = col0 + 2 * pr;
    const R x = c0 < a.ncols ? a.real[(size_t)c0 * L + p] : R(0);
    const R y = c0 + 1 < a.ncols ? a.real[(size_t)(c0 + 1) * L + p] : R(0);
    lines[pr * LP + zi<R>(p)] = cmk<R>(x, y);
  }
  __syncthreads();
  fft_zlines<R, L, false, NT, CP>(lines, tw);
  for (int e = threadIdx.x; e < CP * H; e += NT) {
    const int pr = e / H, k = e % H;
    const int c0 = col0 + 2 * pr;
    C2<R> X, Y;
    zunpack<R>(lines + pr * LP, L, k, X, Y);
    if (c0 < a.ncols) a.cplx[(size_t)c0 * H + k] = X;
    if (c0 + 1 < a.ncols) a.cplx[(size_t)(c0 + 1) * H + k] = Y;
  }
}

template <typename R, int L, int CP, int NT>
__global__ void __launch_bounds__(NT, min_blocks<NT>()) k_fz_c2r(FZArgs<R> a, const C2<R>* __restrict__ tw) {
  constexpr int H = L / 2 + 1;
  constexpr int LP = zpad_len<R>(L);
  extern __shared__ __align__(16) unsigned char vk_smem[];
  C2<R>* lines = reinterpret_cast<C2<R>*>(vk_smem);
  const int col0 = blockIdx.x * 2 * CP;
  for (int e = threadIdx.x; e < CP * H; e += NT) {
    const int pr = e / H, k = e % H;
    const int c0 = col0 + 2 * pr;
    const C2<R> X = c0 < a.ncols ? a.cplx[(size_t)c0 * H + k] : czero<R>();
    const C2<R> Y = c0 + 1 < a.ncols ? a.cplx[(size_t)(c0 + 1) * H + k] : czero<R>();
    zpack<R>(lines + pr * LP, L, k, X, Y);
  }
  __syncthreads();
  fft_zlines<R, L, true, NT, CP>(lines, tw);
  for (int e = threadIdx.x; e < CP * L; e += NT) {
    const int pr = e / L, p = e % L;
    const int c0 = col0 + 2 * pr;
    const C2<R> z = lines[pr * LP + zi<R>(p)];
    if (c0 < a.ncols) a.real[(size_t)c0 * L + p] = z.x * a.scale;
    if (c0 + 1 < a.ncols) a.real[(size_t)(c0 + 1) * L + p] = z.y * a.scale;
  }
}

}  // namespace vk
