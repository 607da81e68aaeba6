// Discrete adjoint of the nonlinear term and of the reference-variant ETD-RK4
// stage combinations.
//
// For N(x) = P T S_out F_M cross(G_M S_in Pad x, G_M S_in Pad curl x)
// (vonkarman-periodic/src/nonlinear.rs:15-39, vonkarman-fft/src/dealiased.rs:16-110)
// the transpose in the raw Euclidean inner product of the stored R2C entries is
//   c_bar = C2R_unnorm_M( Pad(S_out P nbar) / w_M )        (F^T = C2R_unnorm o 1/w)
//   a_bar = omega x c_bar,  o_bar = c_bar x u               (cross-product transpose)
//   N'(x)^T nbar = T(w_M F_M a_bar)/N^3 + curl T(w_M F_M o_bar)/N^3   (G^T = w/M^3 F)
// with w_M the padded R2C weight (1 at kz = 0, else 2 for the kept kz) and
// curl and Leray self-adjoint per mode.  The pass chain mirrors P1..P5:
//   A1 x-inverse of x (5 fields as P1) and of the cotangent source (3 fields)
//   A2 y-inverse: u, omega (6) and c_bar (3)
//   A3 z: c2r of the 9 real fields, a_bar and o_bar, r2c of 6 fields, keep H
//   A4 y-forward with truncation (6 fields, the forward P4 kernel)
//   A5 x-forward with truncation, weights, curl of the o_bar part, stage
//      accumulation of the adjoint ETD-RK4 step
#pragma once

#include "vk_lines.cuh"

namespace vk {

// c_bar source of A1 (elementwise over the N-grid modes, before A1):
// cb = mul * S_out * P nbar / w_M with mul = fac dt etd[slot] (slot >= 0),
// P the Leray projection (spectral_ops.rs:114-151) and the padded-grid R2C
// weight 1/w_M (1 at kz = 0, 1/2 elsewhere: the N-grid Nyquist plane is
// interior on the padded grid).
template <typename R> struct CbarArgs {
  int N, H;
  R s_cbar, ks;
  const C2<R>* nb; size_t cs;
  const double* etd; int slot; double fac; const double* dt;
  C2<R>* out;
};

template <typename R>
__global__ void __launch_bounds__(256) k_adj_cbar(CbarArgs<R> a) {
  const size_t total = (size_t)a.N * a.N * a.H;
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= total) return;
  const int z = (int)(idx % a.H);
  const size_t r = idx / a.H;
  const int iy = (int)(r % a.N), ix = (int)(r / a.N);
  C2<R> b[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) b[j] = a.nb[(size_t)j * a.cs + idx];
  const int kxi = signed_k(ix, a.N), kyi = signed_k(iy, a.N);
  R mul = a.s_cbar * (z == 0 ? R(1) : R(0.5));
  if (a.slot >= 0) {
    const int m = kxi * kxi + kyi * kyi + z * z;
    mul *= (R)(a.fac * (*a.dt) * a.etd[(size_t)m * ETD_STRIDE + a.slot]);
  }
  const R kx = a.ks * (R)kxi, ky = a.ks * (R)kyi, kz = a.ks * (R)z;
  const R k2 = (kx * kx + ky * ky) + kz * kz;
  C2<R> v[3] = {b[0], b[1], b[2]};
  if (!(k2 < R(1e-30))) {
    const R inv = R(1) / k2;
    const C2<R> kd = cmk<R>((kx * b[0].x + ky * b[1].x) + kz * b[2].x, (kx * b[0].y + ky * b[1].y) + kz * b[2].y);
    v[0] = cmk<R>(b[0].x - kx * kd.x * inv, b[0].y - kx * kd.y * inv);
    v[1] = cmk<R>(b[1].x - ky * kd.x * inv, b[1].y - ky * kd.y * inv);
    v[2] = cmk<R>(b[2].x - kz * kd.x * inv, b[2].y - kz * kd.y * inv);
  }
#pragma unroll
  for (int j = 0; j < 3; ++j) a.out[(size_t)j * a.cs + idx] = cscale<R>(v[j], mul);
}

// A1: fields 0..4 as P1 on x; fields 5..7 = x-inverse of Pad(c_bar source)
// (k_adj_cbar).  Kinds: 0 = u_c, 1 = i kx u, 2 = c_bar.
template <typename R, int GN = 0, int GM = 0> struct OpAdjXInv {
  int nfields, hz;
  int N, M;
  R s_in, ks;
  const C2<R>* in; size_t cs;          // stage input x
  const C2<R>* cb;                     // c_bar source (3 components, stride cs)
  C2<R>* out; size_t fs;
  static constexpr int NKIND = 3;
  VK_GRID_DIMS(GN, GM)
  VK_PAD_ZEROS(GN, GM)
  __host__ __device__ __forceinline__ int kind(int f) const { return f < 3 ? 0 : f < 5 ? 1 : 2; }
  // L2 prefetch of row t of the input tile of field f (as OpXInv's)
  __device__ __forceinline__ void prefetch_row(int f, int lam0, int, int t) const {
    const C2<R>* src = f < 5 ? in : cb;
    const int c = f < 3 ? f : f < 5 ? f - 2 : f - 5;
    if (t < n_()) prefetch_l2(src + (size_t)c * cs + (size_t)t * n_() * h_() + lam0);
  }
  template <int K> __device__ __forceinline__ C2<R> load(int f, int iy, int z, int p) const {
    const int ix = unpad_pos(p, n_(), m_());
    const C2<R>* src = K == 2 ? cb : in;
    const int c = K == 0 ? f : K == 1 ? f - 2 : f - 5;
    return ix < 0 ? czero<R>() : src[(size_t)c * cs + ((ix * n_() + iy) * h_() + z)];
  }
  template <int K> __device__ __forceinline__ C2<R> prep(int, int, int, int p, C2<R> v) const {
    if constexpr (K == 2) {
      return v;
    } else {
      v = cscale<R>(v, s_in);
      if constexpr (K == 1) {
        const int ix = unpad_pos(p, n_(), m_());
        const R kx = ks * (R)signed_k(ix < 0 ? 0 : ix, n_());
        v = cmk<R>(-kx * v.y, kx * v.x);
      }
      return v;
    }
  }
  __device__ __forceinline__ int out_index(int p) const { return p; }
  __device__ __forceinline__ void store(int f, int iy, int z, int i, C2<R> v) const {
    out[(size_t)f * fs + ((i * n_() + iy) * h_() + z)] = v;
  }
};

// A2: fields 0..5 as P2 (u, omega), fields 6..8 = y-inverse of c_bar.
// Kinds as P2, then one more for c_bar.
template <typename R, int GN = 0, int GM = 0> struct OpAdjYInv {
  using Base = OpYInv<R, GN, GM>;
  Base base;   // reads input fields 0..4
  int nfields, hz;
  static constexpr int MAX_L16 = 0;        // 8-line tiles (16 spill)
  static constexpr int ZERO_LO = Base::ZERO_LO, ZERO_HI = Base::ZERO_HI;   // c_bar is padded too
  static constexpr int KC = Base::NKIND;   // the c_bar kind
  static constexpr int NKIND = KC + 1;
  __host__ __device__ __forceinline__ int h_() const { return base.h_(); }
  __host__ __device__ __forceinline__ int kind(int f) const { return f < 6 ? base.kind(f) : KC; }
  template <int K> __device__ __forceinline__ auto load(int f, int x, int z, int p) const {
    if constexpr (K < KC) {
      return base.template load<K>(f, x, z, p);
    } else {
      const int iy = unpad_pos(p, base.n_(), base.m_());
      return iy < 0 ? czero<R>() : base.in[(size_t)(f - 1) * base.fsin + ((x * base.n_() + iy) * base.h_() + z)];
    }
  }
  template <int K, class T> __device__ __forceinline__ C2<R> prep(int f, int x, int z, int p, const T& r) const {
    if constexpr (K < KC) {
      return base.template prep<K>(f, x, z, p, r);
    } else {
      return r;
    }
  }
  __device__ __forceinline__ int out_index(int p) const { return p; }
  __device__ __forceinline__ void store(int f, int x, int z, int i, C2<R> v) const {
    base.out[(size_t)f * base.fsout + ((x * base.m_() + i) * base.h_() + z)] = v;
  }
};

// A3: per (x, y) column: 9 real fields -> 4.5 complex lines per column
//   (u_x + i u_y), (u_z + i w_x), (w_y + i w_z), (cb_x + i cb_y), and
//   (cb_z of column 0 + i cb_z of column 1) shared by a column pair;
// after the inverse FFT: a_bar = w x cb, o_bar = cb x u; per column three
// forward lines (ab_x + i ab_y), (ab_z + i ob_x), (ob_y + i ob_z).
// Output fields: ab_x, ab_y, ab_z, ob_x, ob_y, ob_z, each (M, M, H).
template <typename R> struct A3Args {
  int ncols;
  const C2<R>* in; size_t fsin;     // 9 fields (M, M, H)
  C2<R>* out; size_t fsout;         // 6 fields (M, M, H)
};

template <typename R, int M, int CP>
__host__ __device__ constexpr int adj_z_threads() {
  return cmin(rthreads<R, M, 9 * CP, true>(), 384);
}
// Shared memory of k_adj_z: 9 CP inverse lines (exchange, then the physical
// values in place) and 6 CP forward lines.
template <typename R, int M, int CP>
__host__ __device__ constexpr int adj_z_smem_elems() {
  return 15 * CP * zpad_len<R>(M);
}

// Row unpack of A3's forward lines l = t 2CP + c: fields 2t and 2t + 1 of
// column col0 + c (the layout of the shared-memory unpack in k_adj_z).
template <typename R, int M, int CP>
struct AdjZRowUnpack {
  static constexpr bool kRowStore = true;
  C2<R>* out; size_t fsout; int ncols; int col0;
  template <int RAD, int NS>
  __device__ __forceinline__ void row(int l, int j, const C2<R>* v) const {
    constexpr int H = M / 3 + 1;
    const int t = l / (2 * CP), col = col0 + (l - t * 2 * CP);
    unpack_rows<R, RAD, NS, H>(j, v, [&](int k, const C2<R>& X, const C2<R>& Y) {
      if (col < ncols) {
        out[(size_t)(2 * t) * fsout + (size_t)col * H + k] = X;
        out[(size_t)(2 * t + 1) * fsout + (size_t)col * H + k] = Y;
      }
    });
  }
};

// On the register engine: inverse lines l < 8 CP are the packed pair
// t = l / 2CP of column c = l % 2CP; lines 8 CP + pr carry c_bar_z of the two
// columns of pair pr.  Forward lines l = t * 2CP + c: (ab_x + i ab_y),
// (ab_z + i ob_x), (ob_y + i ob_z) of column c.
template <typename R, int M, int CP, int NT>
__global__ void __launch_bounds__(NT, M >= 768 ? 1 : cmax(1, (sizeof(R) == 8 ? 768 : 512) / NT))
k_adj_z(A3Args<R> a, const C2<R>* __restrict__ tw, int pf) {
  constexpr int N = 2 * M / 3;
  constexpr int H = N / 2 + 1;
  constexpr int LP = zpad_len<R>(M);
  constexpr int NI = 9 * CP, NF = 6 * CP;
  extern __shared__ __align__(16) unsigned char vk_smem[];
  __shared__ C2<R> tw_s[twtab_elems<R, true>(M)];
  // L2 prefetch of the nine input ranges of the CTA pf blocks ahead (FP32:
  // per field 2 CP columns of H complex values, a multiple of 16 bytes at a
  // 16-byte boundary)
  if constexpr (sizeof(R) == 4) {
    const int b = (int)blockIdx.x + pf;
    if (pf > 0 && threadIdx.x < 9 && b < (int)gridDim.x && (b + 1) * 2 * CP <= a.ncols)
      prefetch_l2_bulk(a.in + (size_t)threadIdx.x * a.fsin + (size_t)b * (2 * CP * H), 2 * CP * H * sizeof(C2<R>));
  }
  load_twtab<R, M, true, NT>(tw_s, tw);
  C2<R>* A = reinterpret_cast<C2<R>*>(vk_smem);   // NI lines
  C2<R>* B = A + NI * LP;                          // NF lines
  const int col0 = blockIdx.x * 2 * CP;
  fft_lines<R, M, true, NT, NI, MapContig<R, M, NI>, true, true>(
      A, tw_s,
      [&](int l, int p) -> C2x2<R> {
        int fx, fy, cx, cy;
        if (l < 8 * CP) {
          const int t = l / (2 * CP);
          fx = 2 * t; fy = 2 * t + 1;
          cx = cy = col0 + l % (2 * CP);
        } else {
          fx = fy = 8;
          cx = col0 + 2 * (l - 8 * CP);
          cy = cx + 1;
        }
        const bool lo = p < H;
        C2x2<R> r{};
        if (lo || p > M - H) {
          const int k = lo ? p : M - p;
          if (cx < a.ncols) r.a = a.in[(size_t)fx * a.fsin + (size_t)cx * H + k];
          if (cy < a.ncols) r.b = a.in[(size_t)fy * a.fsin + (size_t)cy * H + k];
        }
        return r;
      },
      [&](int, int p, const C2x2<R>& r) -> C2<R> {   // Z = X + i Y with the Hermitian extension
        const C2<R> X = r.a, Y = r.b;
        if (p == 0) return cmk<R>(X.x, Y.x);
        return p < H ? cmk<R>(X.x - Y.y, X.y + Y.x) : cmk<R>(X.x + Y.y, Y.x - X.y);
      },
      [&](int l, int p, C2<R> v) { A[l * LP + zi<R>(p)] = v; });
  __syncthreads();
  for (int e = threadIdx.x; e < CP * M; e += NT) {
    const int pr = e / M, p = e % M;
    const int zp = zi<R>(p);
    const C2<R> Z = A[(8 * CP + pr) * LP + zp];
#pragma unroll
    for (int cc = 0; cc < 2; ++cc) {
      const int c = 2 * pr + cc;
      const C2<R> z0 = A[c * LP + zp], z1 = A[(2 * CP + c) * LP + zp], z2 = A[(4 * CP + c) * LP + zp],
                  z3 = A[(6 * CP + c) * LP + zp];
      const R ux = z0.x, uy = z0.y, uz = z1.x, wx = z1.y, wy = z2.x, wz = z2.y;
      const R cx = z3.x, cy = z3.y, cz = cc == 0 ? Z.x : Z.y;
      // a_bar = w x cb ; o_bar = cb x u
      const R abx = wy * cz - wz * cy, aby = wz * cx - wx * cz, abz = wx * cy - wy * cx;
      const R obx = cy * uz - cz * uy, oby = cz * ux - cx * uz, obz = cx * uy - cy * ux;
      B[c * LP + zp] = cmk<R>(abx, aby);
      B[(2 * CP + c) * LP + zp] = cmk<R>(abz, obx);
      B[(4 * CP + c) * LP + zp] = cmk<R>(oby, obz);
    }
  }
  __syncthreads();
  if constexpr (z_row_unpack<R, M, NF, NT>()) {
    // the kept modes unpacked from the last stage's registers
    fft_lines<R, M, false, NT, NF, MapContig<R, M, NF>, false, true>(
        A, tw_s, [&](int l, int p) { return B[l * LP + zi<R>(p)]; }, PrepNone{},
        AdjZRowUnpack<R, M, CP>{a.out, a.fsout, a.ncols, col0});
    return;
  }
  fft_lines<R, M, false, NT, NF, MapContig<R, M, NF>, false, true>(
      A, tw_s, [&](int l, int p) { return B[l * LP + zi<R>(p)]; }, PrepNone{},
      [&](int l, int p, C2<R> v) { B[l * LP + zi<R>(p)] = v; });
  __syncthreads();
  for (int e = threadIdx.x; e < 2 * CP * 3 * H; e += NT) {
    const int k = e % H;
    const int t = (e / H) % 3;
    const int c = e / (3 * H);
    const int col = col0 + c;
    if (col >= a.ncols) continue;
    C2<R> X, Y;
    zunpack<R>(B + (t * 2 * CP + c) * LP, M, k, X, Y);
    a.out[(size_t)(2 * t) * a.fsout + (size_t)col * H + k] = X;
    a.out[(size_t)(2 * t + 1) * a.fsout + (size_t)col * H + k] = Y;
  }
}

// Adjoint stage combinations of the reference ETD-RK4 step
// (vonkarman-periodic/src/solver.rs:254-378 transposed), applied per mode to
// y = N'(x)^T nbar:
//   ADJ_C  (x = c): acc = E (ub + y); nb = dt b23 ub + 2 dt a41 y; n1b = dt b1 ub - dt a41 y
//   ADJ_B  (x = b): acc += E2 y; nb = dt b23 ub + dt a21 y
//   ADJ_A  (x = a): acc += E2 y; n1b += dt a21 y
//   ADJ_U  (x = u): ub = acc + y
// (ub = cotangent of the step's output, E = exp(z), E2 = exp(z/2)).
// Inputs of all three components are loaded before any store (see
// stage_apply_n).
template <typename R>
__device__ __forceinline__ void adj_stage_apply(const AdjStageArgs<R>& s, size_t idx, int m, const C2<R>* y) {
  const size_t cs = s.cs;
  if (s.op == ADJ_NL_OUT) {
#pragma unroll
    for (int c = 0; c < 3; ++c) s.out[c * cs + idx] = y[c];
    return;
  }
  const double dt = *s.dt;
  const double* e = s.etd + (size_t)m * ETD_STRIDE;
  switch (s.op) {
    case ADJ_C: {
      const R E = (R)e[E_FULL];
      const R nb_u = (R)(dt * e[E_B23]), nb_y = (R)(2.0 * dt * e[E_A41]);
      const R n1_u = (R)(dt * e[E_B1]), n1_y = (R)(-dt * e[E_A41]);
      C2<R> ub[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) ub[c] = s.ub[c * cs + idx];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const size_t i = c * cs + idx;
        s.acc[i] = cmk<R>(E * (ub[c].x + y[c].x), E * (ub[c].y + y[c].y));
        s.nb[i] = axpby<R>(nb_u, ub[c], nb_y, y[c]);
        s.n1b[i] = axpby<R>(n1_u, ub[c], n1_y, y[c]);
      }
      break;
    }
    case ADJ_B: {
      const R E2 = (R)e[E_HALF];
      const R nb_u = (R)(dt * e[E_B23]), nb_y = (R)(dt * e[E_A21]);
      C2<R> ub[3], ac[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        ub[c] = s.ub[c * cs + idx];
        ac[c] = s.acc[c * cs + idx];
      }
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const size_t i = c * cs + idx;
        s.acc[i] = cmk<R>(ac[c].x + E2 * y[c].x, ac[c].y + E2 * y[c].y);
        s.nb[i] = axpby<R>(nb_u, ub[c], nb_y, y[c]);
      }
      break;
    }
    case ADJ_A: {
      const R E2 = (R)e[E_HALF];
      const R q = (R)(dt * e[E_A21]);
      C2<R> ac[3], n1[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        ac[c] = s.acc[c * cs + idx];
        n1[c] = s.n1b[c * cs + idx];
      }
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const size_t i = c * cs + idx;
        s.acc[i] = cmk<R>(ac[c].x + E2 * y[c].x, ac[c].y + E2 * y[c].y);
        s.n1b[i] = cmk<R>(n1[c].x + q * y[c].x, n1[c].y + q * y[c].y);
      }
      break;
    }
    case ADJ_U: {
      C2<R> ac[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) ac[c] = s.acc[c * cs + idx];
#pragma unroll
      for (int c = 0; c < 3; ++c) s.ub[c * cs + idx] = cmk<R>(ac[c].x + y[c].x, ac[c].y + y[c].y);
      break;
    }
    default: break;
  }
}

// A5: x-forward of the six fields, keep N of M, y = w_M (a_bar part + curl of
// the o_bar part) / N^3, adjoint stage epilogue.  Shared memory: FFT tile plus
// five finished fields.
template <typename R> struct A5Args {
  int N, M, H, nlines;
  R s_out, ks;
  const C2<R>* in; size_t fsin;    // 6 fields (M, N, H)
  AdjStageArgs<R> st;
};

template <typename R> struct A5Lines { static constexpr int value = sizeof(R) == 8 ? 4 : 8; };

// Transposed P5 for the six cotangent fields (a_bar, o_bar): x-forward, keep
// N of M modes, weight, and y = a_bar + i k x o_bar accumulated field by field
// in shared memory (three accumulators; the thread producing output ix of a
// field is the one that holds ix of every field, so the accumulation needs
// no barrier), then the adjoint stage epilogue over the CTA's N x NLINES
// modes.
template <typename R, int L, int NLINES, int NT>
__global__ void __launch_bounds__(NT, lines_min_blocks<R, L, NT, true>())
k_adj_p5(A5Args<R> a, const C2<R>* __restrict__ tw) {
  constexpr int N = 2 * L / 3;
  static_assert(NT % NLINES == 0, "a thread keeps one line in every stage");
  extern __shared__ __align__(16) unsigned char vk_smem[];
  __shared__ C2<R> tw_s[twtab_elems<R, false>(L)];
  load_twtab<R, L, false, NT>(tw_s, tw);
  C2<R>* xb = reinterpret_cast<C2<R>*>(vk_smem);
  C2<R>* acc = xb + rsmem_elems<R, L, NLINES>();   // 3 components x N x NLINES
  constexpr int H = N / 2 + 1;   // a.H of the launch
  {
    const int l = threadIdx.x % NLINES;
    const int lam = blockIdx.x * NLINES + l;
    const bool ok = lam < a.nlines;
    const int iy = ok ? lam / H : 0;
    const int z = ok ? lam - iy * H : 0;
    const R ky = a.ks * (R)signed_k(iy, N);
    const R kz = a.ks * (R)z;
    const R wgt = a.s_out * (z == 0 ? R(1) : R(2));
    sfor<6>([&](auto cc) {
      constexpr int C = decltype(cc)::value;
      if (C > 0) __syncthreads();   // xb is reused
      const C2<R>* src = a.in + (size_t)C * a.fsin + (iy * H + z);
      fft_lines<R, L, false, NT, NLINES, MapInterleaved<R, L, NLINES>, false, true>(
          xb, tw_s, [&](int, int p) { return src[p * (N * H)]; }, PrepNone{},
          [&](int, int p, C2<R> v) {
            const int ix = unpad_pos(p, N, L);
            if (ix < 0) return;
            v = cscale<R>(v, wgt);
            C2<R>* y0 = acc + ix * NLINES + l;
            C2<R>* y1 = y0 + N * NLINES;
            C2<R>* y2 = y1 + N * NLINES;
            const R kx = a.ks * (R)signed_k(ix, N);
            // i k x o_bar (spectral_ops.rs:92-104), one o_bar component at a time
            if constexpr (C < 3) {
              (C == 0 ? *y0 : C == 1 ? *y1 : *y2) = v;
            } else if constexpr (C == 3) {   // o_x: y_y += i kz o_x, y_z -= i ky o_x
              *y1 = cadd<R>(*y1, cmul_i<R>(cscale<R>(v, kz)));
              *y2 = csub<R>(*y2, cmul_i<R>(cscale<R>(v, ky)));
            } else if constexpr (C == 4) {   // o_y: y_x -= i kz o_y, y_z += i kx o_y
              *y0 = csub<R>(*y0, cmul_i<R>(cscale<R>(v, kz)));
              *y2 = cadd<R>(*y2, cmul_i<R>(cscale<R>(v, kx)));
            } else {                         // o_z: y_x += i ky o_z, y_y -= i kx o_z
              *y0 = cadd<R>(*y0, cmul_i<R>(cscale<R>(v, ky)));
              *y1 = csub<R>(*y1, cmul_i<R>(cscale<R>(v, kx)));
            }
          });
    });
  }
  __syncthreads();
#pragma unroll 1
  for (int e = threadIdx.x; e < N * NLINES; e += NT) {
    const int ix = e / NLINES, l = e % NLINES;
    const int lam = blockIdx.x * NLINES + l;
    if (lam >= a.nlines) continue;
    const int iy = lam / H;
    const int z = lam - iy * H;
    const int kxi = signed_k(ix, N), kyi = signed_k(iy, N);
    C2<R> y[3] = {acc[e], acc[N * NLINES + e], acc[2 * N * NLINES + e]};
    adj_stage_apply<R>(a.st, ((size_t)ix * N + iy) * H + z, kxi * kxi + kyi * kyi + z * z, y);
  }
}

// Initial cotangent of J = final enstrophy (solver.rs:436-465):
// ub = (2 / N^6) w curl curl u, and the final gradient in the weighted inner
// product: g = N^6 ub / w with zero Nyquist entries, Leray-projected (the
// Hermitian average of the kz = 0, N/2 planes is a separate kernel).
template <typename R> struct ModeArgs {
  int N, H;
  double ks;
  size_t cs;
  const C2<R>* in;
  C2<R>* out;
  int mode;   // 0 = enstrophy cotangent, 1 = to weighted + Nyquist + Leray
};

template <typename R>
__global__ void k_adj_mode(ModeArgs<R> a) {
  const size_t total = (size_t)a.N * a.N * a.H;
  const int N = a.N, H = a.H;
  const double nt = (double)N * N * N;
  for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (size_t)gridDim.x * blockDim.x) {
    const int z = (int)(idx % H);
    const int iy = (int)((idx / H) % N);
    const int ix = (int)(idx / ((size_t)H * N));
    const double kx = (double)signed_k(ix, N) * a.ks, ky = (double)signed_k(iy, N) * a.ks, kz = (double)z * a.ks;
    const double w = (z == 0 || z == N / 2) ? 1.0 : 2.0;
    double ur[3], ui[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) { const C2<R> v = a.in[c * a.cs + idx]; ur[c] = v.x; ui[c] = v.y; }
    double o_r[3], o_i[3];
    if (a.mode == 0) {
      const double w_r[3] = {-(ky * ui[2] - kz * ui[1]), -(kz * ui[0] - kx * ui[2]), -(kx * ui[1] - ky * ui[0])};
      const double w_i[3] = {ky * ur[2] - kz * ur[1], kz * ur[0] - kx * ur[2], kx * ur[1] - ky * ur[0]};
      const double f = 2.0 * w / (nt * nt);
      o_r[0] = -(ky * w_i[2] - kz * w_i[1]) * f; o_i[0] = (ky * w_r[2] - kz * w_r[1]) * f;
      o_r[1] = -(kz * w_i[0] - kx * w_i[2]) * f; o_i[1] = (kz * w_r[0] - kx * w_r[2]) * f;
      o_r[2] = -(kx * w_i[1] - ky * w_i[0]) * f; o_i[2] = (kx * w_r[1] - ky * w_r[0]) * f;
    } else {
      const bool nyq = ix == N / 2 || iy == N / 2 || z == N / 2;
      const double f = nyq ? 0.0 : nt * nt / w;
      for (int c = 0; c < 3; ++c) { o_r[c] = ur[c] * f; o_i[c] = ui[c] * f; }
      const double k2 = (kx * kx + ky * ky) + kz * kz;
      if (!(k2 < 1e-30)) {
        const double inv = 1.0 / k2;
        const double dr = (kx * o_r[0] + ky * o_r[1]) + kz * o_r[2];
        const double di = (kx * o_i[0] + ky * o_i[1]) + kz * o_i[2];
        const double kk[3] = {kx, ky, kz};
        for (int c = 0; c < 3; ++c) { o_r[c] -= kk[c] * dr * inv; o_i[c] -= kk[c] * di * inv; }
      }
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) a.out[c * a.cs + idx] = cmk<R>((R)o_r[c], (R)o_i[c]);
  }
}

// Hermitian average of the kz = 0 and kz = N/2 planes, out of place:
// out[kx, ky] = (in[kx, ky] + conj in[-kx, -ky]) / 2 there, copy elsewhere.
template <typename R>
__global__ void k_hermitian_avg(int N, int H, size_t cs, const C2<R>* __restrict__ in, C2<R>* __restrict__ out) {
  const size_t total = (size_t)N * N * H;
  for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (size_t)gridDim.x * blockDim.x) {
    const int z = (int)(idx % H);
    const int iy = (int)((idx / H) % N);
    const int ix = (int)(idx / ((size_t)H * N));
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      C2<R> v = in[c * cs + idx];
      if (z == 0 || z == N / 2) {
        const int jx = (N - ix) % N, jy = (N - iy) % N;
        const C2<R> m = in[c * cs + ((size_t)jx * N + jy) * H + z];
        v = cmk<R>(R(0.5) * (v.x + m.x), R(0.5) * (v.y - m.y));
      }
      out[c * cs + idx] = v;
    }
  }
}

}  // namespace vk
