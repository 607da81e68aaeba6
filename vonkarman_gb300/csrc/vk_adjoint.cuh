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

// A1: fields 0..4 as P1 on x; fields 5..7 = Pad(mul * S_out * P nbar / w_M).
// Kinds: 0 = u_c, 1 = i kx u, 2 = c_bar (Leray projection and ETD factor
// applied at the load, three loads per position).
template <typename R> struct OpAdjXInv {
  int nfields, hz;
  int N, M;
  R s_in, s_cbar, ks;
  const C2<R>* in; size_t cs;          // stage input x
  const C2<R>* nb;                     // cotangent source (3 components, stride cs)
  const double* etd; int slot; double fac; const double* dt;   // mul = fac dt etd[slot] if slot >= 0
  C2<R>* out; size_t fs;
  static constexpr bool STAGED_ANY = false;
  template <int K> __host__ __device__ static constexpr bool staged() { return false; }
  static constexpr int NKIND = 3;
  __host__ __device__ __forceinline__ int kind(int f) const { return f < 3 ? 0 : f < 5 ? 1 : 2; }
  template <int K> __device__ __forceinline__ C2<R> load(int f, int iy, int z, int p) const {
    const int ix = unpad_pos(p, N, M);
    if constexpr (K < 2) {
      const int c = K == 0 ? f : f - 2;
      return ix < 0 ? czero<R>() : in[(size_t)c * cs + ((size_t)ix * N + iy) * hz + z];
    } else {
      if (ix < 0) return czero<R>();
      const size_t idx = ((size_t)ix * N + iy) * hz + z;
      const int kxi = signed_k(ix, N), kyi = signed_k(iy, N);
      const int c = f - 5;
      C2<R> b[3];
#pragma unroll
      for (int j = 0; j < 3; ++j) b[j] = nb[(size_t)j * cs + idx];
      const R kx = ks * (R)kxi, ky = ks * (R)kyi, kz = ks * (R)z;
      const R k2 = (kx * kx + ky * ky) + kz * kz;
      C2<R> v = b[c];
      if (!(k2 < R(1e-30))) {
        const R inv = R(1) / k2;
        const C2<R> kd = cmk<R>((kx * b[0].x + ky * b[1].x) + kz * b[2].x, (kx * b[0].y + ky * b[1].y) + kz * b[2].y);
        const R kc = c == 0 ? kx : c == 1 ? ky : kz;
        v = cmk<R>(v.x - kc * kd.x * inv, v.y - kc * kd.y * inv);
      }
      R mul = s_cbar * (z == 0 ? R(1) : R(0.5));
      if (slot >= 0) {
        const int m = kxi * kxi + kyi * kyi + z * z;
        mul *= (R)(fac * (*dt) * etd[(size_t)m * ETD_STRIDE + slot]);
      }
      return cscale<R>(v, mul);
    }
  }
  template <int K> __device__ __forceinline__ C2<R> prep(int, int, int, int p, C2<R> v) const {
    if constexpr (K == 2) {
      return v;
    } else {
      v = cscale<R>(v, s_in);
      if constexpr (K == 1) {
        const int ix = unpad_pos(p, N, M);
        const R kx = ks * (R)signed_k(ix < 0 ? 0 : ix, N);
        v = cmk<R>(-kx * v.y, kx * v.x);
      }
      return v;
    }
  }
  __device__ __forceinline__ int out_index(int p) const { return p; }
  __device__ __forceinline__ void store(int f, int iy, int z, int i, C2<R> v) const {
    out[(size_t)f * fs + ((size_t)i * N + iy) * hz + z] = v;
  }
};

// A2: fields 0..5 as P2 (u, omega), fields 6..8 = y-inverse of c_bar.
// Kinds as P2, then one more for c_bar.
template <typename R> struct OpAdjYInv {
  OpYInv<R> base;   // reads input fields 0..4
  int nfields, hz;
  static constexpr bool STAGED_ANY = OpYInv<R>::STAGED_ANY;
  static constexpr int KC = OpYInv<R>::NKIND;   // the c_bar kind
  template <int K> __host__ __device__ static constexpr bool staged() {
    return K < KC && OpYInv<R>::template staged<K>();
  }
  static constexpr int NKIND = KC + 1;
  __host__ __device__ __forceinline__ int kind(int f) const { return f < 6 ? base.kind(f) : KC; }
  template <int K> __device__ __forceinline__ auto load(int f, int x, int z, int p) const {
    if constexpr (K < KC) {
      return base.template load<K>(f, x, z, p);
    } else {
      const int iy = unpad_pos(p, base.N, base.M);
      return iy < 0 ? czero<R>() : base.in[(size_t)(f - 1) * base.fsin + ((size_t)x * base.N + iy) * hz + z];
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
    base.out[(size_t)f * base.fsout + ((size_t)x * base.M + i) * hz + z] = v;
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

template <typename R, int M, int CP, int NT>
__global__ void __launch_bounds__(NT, min_blocks<NT>()) k_adj_z(A3Args<R> a, const C2<R>* __restrict__ tw) {
  constexpr int N = 2 * M / 3;
  constexpr int H = N / 2 + 1;
  constexpr int NL = 9 * CP;
  constexpr int LP = zpad_len<R>(M);
  extern __shared__ __align__(16) unsigned char vk_smem[];
  C2<R>* lines = reinterpret_cast<C2<R>*>(vk_smem);
  const int col0 = blockIdx.x * 2 * CP;
  constexpr int TOT = 2 * CP * 4 * H;
  constexpr int PER = (TOT + NT - 1) / NT;
  C2<R> lx[PER], ly[PER];
#pragma unroll
  for (int q = 0; q < PER; ++q) {
    const int e = threadIdx.x + q * NT;
    const int k = e % H;
    const int t = (e / H) % 4;
    const int col = col0 + e / (4 * H);
    const bool ok = e < TOT && col < a.ncols;
    lx[q] = ok ? a.in[(size_t)(2 * t) * a.fsin + (size_t)col * H + k] : czero<R>();
    ly[q] = ok ? a.in[(size_t)(2 * t + 1) * a.fsin + (size_t)col * H + k] : czero<R>();
  }
#pragma unroll
  for (int q = 0; q < PER; ++q) {
    const int e = threadIdx.x + q * NT;
    if (e < TOT) {
      const int k = e % H;
      const int t = (e / H) % 4;
      const int cr = e / (4 * H);
      zpack<R>(lines + (9 * (cr / 2) + 4 * (cr % 2) + t) * LP, M, k, lx[q], ly[q]);
    }
  }
  for (int e = threadIdx.x; e < CP * H; e += NT) {
    const int k = e % H, pr = e / H;
    const int c0 = col0 + 2 * pr;
    const C2<R> X = c0 < a.ncols ? a.in[(size_t)8 * a.fsin + (size_t)c0 * H + k] : czero<R>();
    const C2<R> Y = c0 + 1 < a.ncols ? a.in[(size_t)8 * a.fsin + (size_t)(c0 + 1) * H + k] : czero<R>();
    zpack<R>(lines + (9 * pr + 8) * LP, M, k, X, Y);
  }
  for (int e = threadIdx.x; e < NL * (N / 2 - 1); e += NT) {
    const int l = e / (N / 2 - 1), p = H + e % (N / 2 - 1);
    lines[l * LP + zi<R>(p)] = czero<R>();
  }
  __syncthreads();
  fft_zlines<R, M, true, NT, NL>(lines, tw);
  constexpr int QX = (CP * M + NT - 1) / NT;
  C2<R> res[QX][6];
#pragma unroll
  for (int q = 0; q < QX; ++q) {
    const int e = threadIdx.x + q * NT;
    if (e < CP * M) {
      const int pr = e / M, p = e % M;
      const C2<R> Z = lines[(9 * pr + 8) * LP + zi<R>(p)];
#pragma unroll
      for (int cc = 0; cc < 2; ++cc) {
        const C2<R>* L0 = lines + (9 * pr + 4 * cc) * LP;
        const C2<R> A = L0[zi<R>(p)], B = L0[LP + zi<R>(p)], C = L0[2 * LP + zi<R>(p)], D = L0[3 * LP + zi<R>(p)];
        const R ux = A.x, uy = A.y, uz = B.x, wx = B.y, wy = C.x, wz = C.y;
        const R cx = D.x, cy = D.y, cz = cc == 0 ? Z.x : Z.y;
        // a_bar = w x cb ; o_bar = cb x u
        const R abx = wy * cz - wz * cy, aby = wz * cx - wx * cz, abz = wx * cy - wy * cx;
        const R obx = cy * uz - cz * uy, oby = cz * ux - cx * uz, obz = cx * uy - cy * ux;
        res[q][3 * cc + 0] = cmk<R>(abx, aby);
        res[q][3 * cc + 1] = cmk<R>(abz, obx);
        res[q][3 * cc + 2] = cmk<R>(oby, obz);
      }
    }
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < QX; ++q) {
    const int e = threadIdx.x + q * NT;
    if (e < CP * M) {
      const int pr = e / M, p = e % M;
#pragma unroll
      for (int j = 0; j < 6; ++j) lines[(6 * pr + j) * LP + zi<R>(p)] = res[q][j];
    }
  }
  __syncthreads();
  fft_zlines<R, M, false, NT, 6 * CP>(lines, tw);
  for (int e = threadIdx.x; e < CP * 6 * H; e += NT) {
    const int k = e % H;
    const int j = (e / H) % 6;
    const int pr = e / (6 * H);
    const int cc = j / 3, t = j % 3;
    const int col = col0 + 2 * pr + cc;
    if (col >= a.ncols) continue;
    C2<R> X, Y;
    zunpack<R>(lines + (6 * pr + j) * LP, M, k, X, Y);
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
// stage_apply).
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
  C2<R>* xb = reinterpret_cast<C2<R>*>(vk_smem);
  C2<R>* acc = xb + rsmem_elems<R, L, NLINES>();   // 3 components x N x NLINES
  const int H = a.H;
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
      const C2<R>* src = a.in + (size_t)C * a.fsin + (size_t)iy * H + z;
      fft_lines<R, L, false, NT, NLINES>(
          xb, tw, [&](int, int p) { return src[(size_t)p * N * H]; }, PrepNone{},
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
