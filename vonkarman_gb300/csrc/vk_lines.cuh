// Register-resident batched line FFT and the pass kernels built on it
// (k_lines: strided x / y passes; k_p5: x-forward with the stage epilogue;
// k_p3: the z pass with the cross product; k_nz_max: the N-grid z pass).
//
// NLINES lines of length L are transformed by a Stockham auto-sort whose
// stages live in registers: the first stage reads its butterfly inputs
// straight from global memory (through the pass's load functor, which also
// applies zero-padding and derivative factors; inputs that are padding for
// every butterfly are compile-time zeros whose additions are skipped), every
// later stage reads them from a shared-memory exchange buffer written by the
// stage before, and the last stage hands its outputs straight to the pass's
// store functor (which applies truncation).  With the FP32 plans (two stages
// for every padded length up to 768) each element crosses shared memory once.
//
// Thread-to-butterfly maps: interleaved lines (x / y passes, MapInterleaved):
// thread g handles butterfly j = g / NLINES of line l = g % NLINES, so
// consecutive lanes take consecutive lines and global accesses are row
// segments of NLINES elements; contiguous lines (z passes, MapContig):
// consecutive lanes take consecutive butterflies of one line.
#pragma once

#include <type_traits>

#include "vk_kernels.cuh"
#include "vk_reduce.cuh"

// k_p3 (FP32) unpacks the forward's kept modes from the last stage's
// registers (1) or through shared memory after a barrier (0)
#ifndef VK_P3_ROW_UNPACK
#define VK_P3_ROW_UNPACK 1
#endif

namespace vk {

// FP32 plans: at most two stages up to L = 768, composite in-register radices
// 6/12/24/32; the larger radix goes first, where it carries no twiddles.  FP64 plans: radix <= 8 (register budget), as in the
// shared-memory engine.
__host__ __device__ constexpr int rplan_stages_f(int L) {
  return (L == 8 || L == 12 || L == 16 || L == 24) ? 1
       : (L == 32 || L == 48 || L == 64 || L == 96 || L == 128 || L == 192 || L == 256 || L == 384 || L == 512 || L == 768) ? 2
       : -1;
}
__host__ __device__ constexpr int rplan_radix_f(int L, int s) {
  return L <= 24 ? L
       : L == 32 ? (s == 0 ? 8 : 4)
       : L == 48 ? (s == 0 ? 16 : 3)
       : L == 64 ? (s == 0 ? 16 : 4)
       : L == 96 ? (s == 0 ? 16 : 6)
       : L == 128 ? (s == 0 ? 16 : 8)
       : L == 192 ? (s == 0 ? 16 : 12)
       : L == 256 ? 16
       : L == 384 ? (s == 0 ? 24 : 16)
       : L == 512 ? (s == 0 ? 32 : 16)
       : L == 768 ? (s == 0 ? 32 : 24)
       : 1;
}
// Contiguous lines (z passes) keep the radix-16 stage first where the
// larger radix would put the first-stage writes (stride RAD positions) on
// shared-memory banks that the one-slot-per-128-bytes padding cannot spread.
__host__ __device__ constexpr int rplan_radix_fc(int L, int s) {
  return L == 384 ? (s == 0 ? 16 : 24) : rplan_radix_f(L, s);
}
template <typename R, bool CONTIG = false> __host__ __device__ constexpr int rstages(int L) {
  return sizeof(R) == 4 ? rplan_stages_f(L) : plan_stages(L);
}
template <typename R, bool CONTIG = false> __host__ __device__ constexpr int rradix(int L, int s) {
  return sizeof(R) == 4 ? (CONTIG ? rplan_radix_fc(L, s) : rplan_radix_f(L, s)) : plan_radix(L, s);
}
// threads of a CTA: one butterfly per thread in the widest stage
template <typename R, int L, int NLINES, bool CONTIG = false, int S = 0>
__host__ __device__ constexpr int rthreads() {
  if constexpr (S >= rstages<R, CONTIG>(L)) {
    return 32;
  } else {
    return cmax(round32(L / rradix<R, CONTIG>(L, S) * NLINES), rthreads<R, L, NLINES, CONTIG, S + 1>());
  }
}
// Per-stage twiddle tables (shared memory): stage S >= 1 of a plan reads
// W_L^(r k TWS) for r = 1..RAD-1, k = 0..NS-1 at (r-1) NS + k, so that lanes
// with consecutive k read consecutive entries (no bank conflicts) and lanes
// with the same k read the same entry.
template <typename R, bool CONTIG>
__host__ __device__ constexpr int stage_ns(int L, int S) {
  int ns = 1;
  for (int s = 0; s < S; ++s) ns *= rradix<R, CONTIG>(L, s);
  return ns;
}
template <typename R, bool CONTIG>
__host__ __device__ constexpr int twtab_off(int L, int S) {
  int off = 0;
  for (int s = 1; s < S; ++s) off += (rradix<R, CONTIG>(L, s) - 1) * stage_ns<R, CONTIG>(L, s);
  return off;
}
template <typename R, bool CONTIG>
__host__ __device__ constexpr int twtab_elems(int L) {
  return cmax(1, twtab_off<R, CONTIG>(L, rstages<R, CONTIG>(L)));
}

// FP32 with 8 lines: the first stage writes at stride RAD0 positions, so a
// padding slot after every RAD0 positions spreads a warp over both halves of
// the 32 banks.  FP64 rows of 8 lines are already 128 bytes.
template <typename R, int L, int NLINES>
__host__ __device__ constexpr bool rpad() { return sizeof(R) == 4 && NLINES < 16 && rstages<R>(L) > 1; }
template <typename R, int L, int NLINES>
__host__ __device__ constexpr int rsmem_elems() {
  return rstages<R>(L) > 1 ? (L + (rpad<R, L, NLINES>() ? L / rradix<R>(L, 0) : 0)) * NLINES : 0;
}
template <typename R, int L, int NLINES, int S>
__device__ __forceinline__ int ridx(int pos, int l) {
  if constexpr (S == 0 && rpad<R, L, NLINES>()) {
    return (pos + pos / rradix<R>(L, 0)) * NLINES + l;
  } else {
    return pos * NLINES + l;
  }
}

// Minimum resident CTAs per SM requested from the compiler (caps registers):
// 24 warps per SM for the strided passes where the plan allows it; one or two
// CTAs for the long FP64 / 768-point plans and for the multi-field P5 kernels
// (EPI), whose shared memory limits residency anyway.
template <typename R, int L, int NT, bool EPI = false>
__host__ __device__ constexpr int lines_min_blocks() {
  if constexpr (sizeof(R) == 8) {
    return L >= 512 ? 1 : cmax(1, 768 / NT);
  } else {
    return L >= 768 ? (EPI ? 1 : 2) : EPI ? cmax(1, 512 / NT) : L >= 512 ? 2 : L >= 384 ? (NT >= 384 ? 2 : 3)
         : NT < 128 ? 4 : cmax(1, 768 / NT);
  }
}

// Thread-to-butterfly maps and exchange layouts.
// Interleaved lines (x / y passes, element p of line l at p * NLINES + l):
// consecutive lanes take consecutive lines, so every thread keeps one line.
template <typename R, int L, int NLINES>
struct MapInterleaved {
  static constexpr bool CONTIG = false;
  template <int NB> __device__ __forceinline__ static int line(int g) { return g % NLINES; }
  template <int NB> __device__ __forceinline__ static int bfly(int g) { return g / NLINES; }
  template <int S> __device__ __forceinline__ static int idx(int pos, int l) { return ridx<R, L, NLINES, S>(pos, l); }
  static constexpr int elems() { return rsmem_elems<R, L, NLINES>(); }
};
// Contiguous lines (z passes, element p of line l at l * LP + zi(p), one
// padding slot per 128 bytes): consecutive lanes take consecutive
// butterflies of a line, so global accesses along a line coalesce.
template <typename R, int L, int NLINES>
struct MapContig {
  static constexpr bool CONTIG = true;
  template <int NB> __device__ __forceinline__ static int line(int g) { return g / NB; }
  template <int NB> __device__ __forceinline__ static int bfly(int g) { return g % NB; }
  template <int S> __device__ __forceinline__ static int idx(int pos, int l) { return l * zpad_len<R>(L) + zi<R>(pos); }
  static constexpr int elems() { return NLINES * zpad_len<R>(L); }
};

// Inputs of the first stage at positions p in [Z0, Z1) are known to be zero
// (zero-padded modes): butterflies whose input r lies there for every j (all
// of [r NB, r NB + NB) inside the range) skip its first-layer additions.
__host__ __device__ constexpr unsigned zero_mask(int nb, int rad, int z0, int z1) {
  unsigned m = 0u;
  for (int r = 0; r < rad && r < 32; ++r)
    if (z0 < z1 && r * nb >= z0 && r * nb + nb <= z1) m |= 1u << r;
  return m;
}

// Store functors with a row<RAD, NS>(l, j, v) member take the last stage's
// whole butterfly (outputs at positions j + NS r, r < RAD) in one call, so
// that they can combine outputs across lanes (contiguous lines only).
template <class ST, class = void> struct StoreTakesRows : std::false_type {};
template <class ST> struct StoreTakesRows<ST, std::void_t<decltype(ST::kRowStore)>> : std::true_type {};

template <typename R, int L, bool INV, int NT, int NLINES, class MAP, int S, int NS, bool SL = false, bool TT = false,
          int Z0 = 0, int Z1 = 0>
struct RegStage {
  static constexpr int RAD = rradix<R, MAP::CONTIG>(L, S);
  static constexpr int NB = L / RAD;            // butterflies per line
  static constexpr int G = NB * NLINES;         // butterflies per stage
  static constexpr int Q = (G + NT - 1) / NT;
  static constexpr bool LAST = S + 1 == rstages<R, MAP::CONTIG>(L);
  static constexpr int TWS = L / (NS * RAD);    // twiddle table stride

  // ld(l, p) -> raw input of position p of line l (memory loads only),
  // pp(l, p, raw) -> the complex input (arithmetic on the loaded values),
  // st(l, p, v) takes output p.  All loads of the first stage are issued
  // before any arithmetic on them: in-order issue would otherwise wait on each
  // load before issuing the next.
  template <class LD, class PP, class ST>
  __device__ __forceinline__ static void run(C2<R>* xb, const C2<R>* __restrict__ tw, const LD& ld, const PP& pp,
                                             const ST& st) {
    const int tid = threadIdx.x;
    C2<R> v[Q][RAD];
    if constexpr (S == 0) {
      // raw inputs wider than one complex value are staged in chunks of
      // 192 (FP32) / 128 (FP64) bytes per thread (registers)
      using Raw = decltype(ld(0, 0));
      constexpr int CH = sizeof(Raw) > sizeof(C2<R>) ? cmin(RAD, (int)((sizeof(R) == 4 ? 192 : 128) / sizeof(Raw))) : RAD;
#pragma unroll
      for (int q = 0; q < Q; ++q) {
        const int g = tid + q * NT;
        if (G % NT == 0 || g < G) {
          const int l = MAP::template line<NB>(g);
          const int j = MAP::template bfly<NB>(g);
          __builtin_assume(j >= 0 && j < NB);
          __builtin_assume(l >= 0 && l < NLINES);
#pragma unroll
          for (int r0 = 0; r0 < RAD; r0 += CH) {
            Raw raw[CH];
#pragma unroll
            for (int r = 0; r < CH; ++r) {
              if (r0 + r < RAD) raw[r] = ld(l, j + (r0 + r) * NB);
            }
#pragma unroll
            for (int r = 0; r < CH; ++r) {
              if (r0 + r < RAD) v[q][r0 + r] = pp(l, j + (r0 + r) * NB, raw[r]);
            }
          }
        }
      }
    } else {
#pragma unroll
      for (int q = 0; q < Q; ++q) {
        const int g = tid + q * NT;
        if (G % NT == 0 || g < G) {
          const int l = MAP::template line<NB>(g);
          const int j = MAP::template bfly<NB>(g);
          __builtin_assume(j >= 0 && j < NB);
          __builtin_assume(l >= 0 && l < NLINES);
#pragma unroll
          for (int r = 0; r < RAD; ++r) v[q][r] = xb[MAP::template idx<S - 1>(j + r * NB, l)];
        }
      }
    }
    // a later stage writes the buffer it has just read: wait for all readers
    // (the last stage too when its outputs go back into the buffer, SL)
    if constexpr (S > 0 && (!LAST || SL)) __syncthreads();
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      const int g = tid + q * NT;
      if (G % NT == 0 || g < G) {
        const int l = MAP::template line<NB>(g);
        const int j = MAP::template bfly<NB>(g);
        __builtin_assume(j >= 0 && j < NB);
        __builtin_assume(l >= 0 && l < NLINES);
        const int k = j % NS;
        C2<R> w[RAD];
        if constexpr (S > 0) {
#pragma unroll
          for (int r = 1; r < RAD; ++r) {
            if constexpr (TT) {
              w[r] = tw[twtab_off<R, MAP::CONTIG>(L, S) + (r - 1) * NS + k];
            } else {
              w[r] = tw[r * k * TWS];
            }
          }
        }
        dft<R, INV, RAD, (S > 0), S == 0 ? zero_mask(NB, RAD, Z0, Z1) : 0u>(v[q], w);
        const int base = (j - k) * RAD + k;
        if constexpr (LAST && StoreTakesRows<ST>::value) {
          // the whole butterfly (outputs j + NS r, j = base < NS) at once
          static_assert(MAP::CONTIG && G % 32 == 0 && NT % 32 == 0 && NB == NS && (NS == 16 || NS == 32),
                        "row stores: whole warps, butterfly j on lane j of an NS-lane group");
          st.template row<RAD, NS>(l, base, v[q]);
        } else if constexpr (LAST) {
#pragma unroll
          for (int r = 0; r < RAD; ++r) st(l, base + r * NS, v[q][r]);
        } else {
#pragma unroll
          for (int r = 0; r < RAD; ++r) xb[MAP::template idx<S>(base + r * NS, l)] = v[q][r];
        }
      }
    }
    if constexpr (!LAST) {
      __syncthreads();
      RegStage<R, L, INV, NT, NLINES, MAP, S + 1, NS * RAD, SL, TT, Z0, Z1>::run(xb, tw, ld, pp, st);
    }
  }
};

// Transform NLINES lines.  All NT threads must call it; the exchange buffer
// xb (MAP::elems() elements) must not be in use by any thread.  Returns with
// no synchronisation after the last stage.
// SL: the store functor writes into xb itself (in place), so the last stage
// also waits for all readers before storing.  TT: tw is the per-stage table
// of load_twtab (shared memory), else the plain W_L^m table.
template <typename R, int L, bool INV, int NT, int NLINES, class MAP = MapInterleaved<R, L, NLINES>, bool SL = false,
          bool TT = false, int Z0 = 0, int Z1 = 0, class LD, class PP, class ST>
__device__ __forceinline__ void fft_lines(C2<R>* xb, const C2<R>* __restrict__ tw, const LD& ld, const PP& pp,
                                          const ST& st) {
  static_assert(rstages<R>(L) > 0, "unsupported FFT length");
  RegStage<R, L, INV, NT, NLINES, MAP, 0, 1, SL, TT, Z0, Z1>::run(xb, tw, ld, pp, st);
}
// pp for inputs that need no arithmetic after the load
struct PrepNone {
  template <class T> __device__ __forceinline__ T operator()(int, int, const T& v) const { return v; }
};

// Per-stage twiddle tables in shared memory: the stages read them through the
// shared-memory pipe instead of the L1/texture path, which the global loads
// and stores of the passes keep busy, and without bank conflicts.  No barrier
// is needed before the FFT: the first stage reads no twiddles and ends with
// one.
template <typename R, int L, bool CONTIG, int NT>
__device__ __forceinline__ void load_twtab(C2<R>* tab, const C2<R>* __restrict__ tw) {
  constexpr int ST = rstages<R, CONTIG>(L);
  for (int S = 1; S < ST; ++S) {
    const int rad = rradix<R, CONTIG>(L, S), ns = stage_ns<R, CONTIG>(L, S);
    const int tws = L / (ns * rad), off = twtab_off<R, CONTIG>(L, S);
    for (int i = threadIdx.x; i < (rad - 1) * ns; i += NT) {
      const int r = i / ns + 1, k = i - (r - 1) * ns;
      tab[off + i] = tw[r * k * tws];
    }
  }
}

// Positions [lo, hi) of a pass's input lines that are zero-padding for every
// line (Op::ZERO_LO / ZERO_HI; none by default).
template <class Op, class = void> struct OpZeroRange { static constexpr int lo = 0, hi = 0; };
template <class Op> struct OpZeroRange<Op, std::void_t<decltype(Op::ZERO_LO)>> {
  static constexpr int lo = Op::ZERO_LO, hi = Op::ZERO_HI;
};

// Ops that supply prefetch_row(f, lam0, nl, t) (an L2 hint for row t of a
// later CTA's input tile)
template <class Op, class = void> struct OpHasPrefetch : std::false_type {};
template <class Op>
struct OpHasPrefetch<Op, std::void_t<decltype(std::declval<const Op&>().prefetch_row(0, 0, 0, 0))>> : std::true_type {};

// Generic strided pass: NLINES consecutive lines lam = outer * hz + z of one
// field per CTA (blockIdx.x = f + nfields * tile), so no z tile is partly
// empty.  Op supplies kind(f) in [0, NKIND) (fields of one kind share their
// load/prep code, which is specialised per kind), load<K>(f, outer, z, p)
// (memory loads only, zero for padded positions), prep<K>(f, outer, z, p,
// raw), out_index(p) (-1: dropped) and store(f, outer, z, i, v).  Lines past
// the end (lam >= nlines) load line 0 and store nothing.  pf: blocks ahead
// whose input rows are prefetched into L2 (0 = none).

template <typename R, int L, bool INV, int NLINES, int NT, class Op>
__global__ void __launch_bounds__(NT, lines_min_blocks<R, L, NT>())
k_lines(Op op, const C2<R>* __restrict__ tw, int nlines, int pf) {
  static_assert(NT % NLINES == 0, "a thread keeps one line in every stage");
  extern __shared__ __align__(16) unsigned char vk_smem[];
  __shared__ C2<R> tw_s[twtab_elems<R, false>(L)];
  // the input rows of the CTA pf blocks ahead (ops with prefetch_row, whole
  // tiles whose rows are whole 128-byte lines)
  if constexpr (OpHasPrefetch<Op>::value && NLINES * sizeof(C2<R>) == 128) {
    const int b = (int)blockIdx.x + pf;
    if (pf > 0 && b < (int)gridDim.x) {
      const int lam0 = (b / op.nfields) * NLINES;
      if (lam0 + NLINES <= nlines)
        for (int t = threadIdx.x; t < L; t += NT) op.prefetch_row(b % op.nfields, lam0, NLINES, t);
    }
  }
  load_twtab<R, L, false, NT>(tw_s, tw);
  C2<R>* xb = reinterpret_cast<C2<R>*>(vk_smem);
  const int f = blockIdx.x % op.nfields;
  const int tile = blockIdx.x / op.nfields;
  const int lam = tile * NLINES + (int)(threadIdx.x % NLINES);
  const bool ok = lam < nlines;
  const int outer = ok ? lam / op.h_() : 0;
  const int z = ok ? lam - outer * op.h_() : 0;
  const int kd = op.kind(f);
  auto st = [&](int, int p, C2<R> v) {
    const int i = op.out_index(p);
    if (ok && i >= 0) op.store(f, outer, z, i, v);
  };
  sfor<Op::NKIND>([&](auto kc) {
    constexpr int K = decltype(kc)::value;
    if (kd != K) return;   // uniform over the CTA
    fft_lines<R, L, INV, NT, NLINES, MapInterleaved<R, L, NLINES>, false, true, OpZeroRange<Op>::lo,
              OpZeroRange<Op>::hi>(
        xb, tw_s, [&](int, int p) { return op.template load<K>(f, outer, z, p); },
        [&](int, int p, const auto& raw) { return op.template prep<K>(f, outer, z, p, raw); }, st);
  });
}

// ---------------------------------------------------------------------------
// P5: x-forward of the three cross-product fields, keep N of M modes, scale
// N^3/M^3 (dealiased.rs:102-109), Leray projection (spectral_ops.rs:114-151)
// and the stage epilogue.  A CTA takes NLINES consecutive (iy, z) lines; the
// fields are transformed one after another into shared memory (kept modes
// only), then the epilogue runs over the CTA's N x NLINES modes with
// consecutive lanes on consecutive z.
// ---------------------------------------------------------------------------
template <typename R> struct P5Args {
  int N, M, H, nlines;
  R s_out, ks;
  const C2<R>* in; size_t fsin;   // (M, N, H)
  StageArgs<R> st;
};

// lines per CTA of k_p5 at padded length L (the grid N = 2 L / 3), shared
// with the host's sizing of the fused-diagnostics rows
template <typename R, int L> struct P5Lines { static constexpr int value = p5_lines(2 * L / 3, sizeof(R) == 4); };
// Threads of k_p5: one butterfly per thread in the widest FFT stage; FP32 up
// to 384 points doubles them (measured 4 % faster at 384: the epilogue keeps
// the same modes in flight per CTA with one mode per thread, and twice the
// warps hide its arithmetic), two CTAs per SM.
template <typename R, int L, int NLINES>
__host__ __device__ constexpr int p5_threads() {
  return sizeof(R) == 4 && L <= 384 ? cmin(2 * rthreads<R, L, NLINES>(), 384) : cmin(rthreads<R, L, NLINES>(), 384);
}
template <typename R, int L, int NLINES, int NT>
__host__ __device__ constexpr int p5_min_blocks() {
  return NT >= 2 * rthreads<R, L, NLINES>() ? 2 : lines_min_blocks<R, L, NT, true>();
}

// DIAG: the instance for final stages whose new state also feeds the fused
// diagnostics (a.st.diag bits): per thread FP64 sums of the Tier-1 terms and a
// per-CTA FP64 shell histogram in shared memory (nsh doubles after the FFT
// buffers), written as row blockIdx.x of a.st.dpart; the rows are added by the
// Neumaier column reduction, as the separate reduction passes do.
template <typename R, int L, int NLINES, int NT, bool DIAG = false>
__global__ void __launch_bounds__(NT, p5_min_blocks<R, L, NLINES, NT>())
k_p5(P5Args<R> a, const C2<R>* __restrict__ tw) {
  constexpr int N = 2 * L / 3;
  static_assert(NT % NLINES == 0, "a thread keeps one line in every stage");
  extern __shared__ __align__(16) unsigned char vk_smem[];
  __shared__ C2<R> tw_s[twtab_elems<R, false>(L)];
  load_twtab<R, L, false, NT>(tw_s, tw);
  C2<R>* xb = reinterpret_cast<C2<R>*>(vk_smem);
  C2<R>* keep = xb + rsmem_elems<R, L, NLINES>();   // 3 fields x N x NLINES
  constexpr int H = N / 2 + 1;   // a.H of the launch
  double* hist = reinterpret_cast<double*>(keep + 3 * N * NLINES);   // DIAG: nsh shells
  const bool d_t1 = DIAG && (a.st.diag & DIAG_TIER1);
  const bool d_sp = DIAG && (a.st.diag & DIAG_SPECTRUM);
  if constexpr (DIAG) {
    if (d_sp)
      for (int i = threadIdx.x; i < a.st.nsh; i += NT) hist[i] = 0.0;   // ordered by the FFTs' barriers
  }
  double dsum[4] = {0.0, 0.0, 0.0, 0.0};
  const bool ks_one = a.st.ks == 1.0;
  {
    const int lam = blockIdx.x * NLINES + (int)(threadIdx.x % NLINES);
    const bool ok = lam < a.nlines;
    const int iy = ok ? lam / H : 0;
    const int z = ok ? lam - iy * H : 0;
    sfor<3>([&](auto cc) {
      constexpr int C = decltype(cc)::value;
      if (C > 0) __syncthreads();   // xb is reused
      const C2<R>* src = a.in + (size_t)C * a.fsin + (iy * H + z);
      fft_lines<R, L, false, NT, NLINES, MapInterleaved<R, L, NLINES>, false, true>(
          xb, tw_s, [&](int, int p) { return src[p * (N * H)]; }, PrepNone{},
          [&](int, int p, C2<R> v) {
            const int ix = unpad_pos(p, N, L);
            if (ix >= 0) keep[(C * N + ix) * NLINES + (int)(threadIdx.x % NLINES)] = v;
          });
    });
  }
  __syncthreads();
  // FP32 with the FFT's thread count: two modes per iteration, so that the
  // epilogue's loads of both are in flight together (FP64 keeps one: register
  // budget, FP64-pipe bound; doubled threads keep one)
  constexpr int EM = sizeof(R) == 4 && NT < 2 * rthreads<R, L, NLINES>() ? 2 : 1;
#pragma unroll 1
  for (int e0 = threadIdx.x; e0 < N * NLINES; e0 += EM * NT) {
    size_t idx[EM];
    int mm[EM];
    R kk[EM];
    C2<R> nl[EM][3];
    bool ok[EM];
    int kxq[EM], kyq[EM], kzq[EM];
#pragma unroll
    for (int q = 0; q < EM; ++q) {
      const int e = e0 + q * NT;
      const int ix = e / NLINES, l = e % NLINES;
      const int lam = blockIdx.x * NLINES + l;
      ok[q] = e < N * NLINES && lam < a.nlines;
      const int iy = ok[q] ? lam / H : 0;
      const int z = ok[q] ? lam - iy * H : 0;
      const int kxi = signed_k(ok[q] ? ix : 0, N), kyi = signed_k(iy, N);
      const R kx = a.ks * (R)kxi, ky = a.ks * (R)kyi, kz = a.ks * (R)z;
      const int ee = ok[q] ? e : 0;
      nl[q][0] = cscale<R>(keep[ee], a.s_out);
      nl[q][1] = cscale<R>(keep[N * NLINES + ee], a.s_out);
      nl[q][2] = cscale<R>(keep[2 * N * NLINES + ee], a.s_out);
      const R k2 = (kx * kx + ky * ky) + kz * kz;
      if (!(k2 < R(1e-30))) {
        const R inv = R(1) / k2;
        const C2<R> kd = cmk<R>((kx * nl[q][0].x + ky * nl[q][1].x) + kz * nl[q][2].x,
                                (kx * nl[q][0].y + ky * nl[q][1].y) + kz * nl[q][2].y);
        nl[q][0] = cmk<R>(nl[q][0].x - kx * kd.x * inv, nl[q][0].y - kx * kd.y * inv);
        nl[q][1] = cmk<R>(nl[q][1].x - ky * kd.x * inv, nl[q][1].y - ky * kd.y * inv);
        nl[q][2] = cmk<R>(nl[q][2].x - kz * kd.x * inv, nl[q][2].y - kz * kd.y * inv);
      }
      kk[q] = k2;
      mm[q] = kxi * kxi + kyi * kyi + z * z;
      idx[q] = ((size_t)(ok[q] ? ix : 0) * N + iy) * H + z;
      kxq[q] = kxi; kyq[q] = kyi; kzq[q] = z;
    }
    if constexpr (!DIAG) {
      stage_apply_n<R, EM>(a.st, idx, mm, kk, nl, ok);
    } else {
      C2<R> un[EM][3];
      stage_apply_n<R, EM, true>(a.st, idx, mm, kk, nl, ok, un);
#pragma unroll
      for (int q = 0; q < EM; ++q) {
        if (!ok[q]) continue;
        const R w = (kzq[q] == 0 || kzq[q] == N / 2) ? R(1) : R(2);   // R2C weight, exact in R
        if (d_t1) {
          R e, en, he, sh;
          tier1_terms<R>(a.ks * (R)kxq[q], a.ks * (R)kyq[q], a.ks * (R)kzq[q], un[q], e, en, he, sh);
          dsum[0] += (double)(w * e); dsum[1] += (double)(w * en);
          dsum[2] += (double)(w * he); dsum[3] += (double)(w * sh);
        }
        if (d_sp) {
          const int shell = shell_of(kxq[q], kyq[q], kzq[q], a.st.ks, ks_one);
          if (shell < a.st.nsh) atomicAdd(&hist[shell], (double)(w * spectrum_term<R>(un[q])));
        }
      }
    }
  }
  if constexpr (DIAG) {
    // the CTA's row: Tier-1 sums by a fixed shuffle / warp-order tree, then
    // the shell histogram
    __shared__ double wsum[4][NT / 32];
    const bool has_row = (int)blockIdx.x < a.st.dpart_rows;
    double* row = a.st.dpart + (size_t)(has_row ? blockIdx.x : 0) * (4 + a.st.nsh);
    if (d_t1) {
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        double v = dsum[j];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0) wsum[j][threadIdx.x / 32] = v;
      }
    }
    __syncthreads();
    if (d_t1 && has_row && threadIdx.x < 4) {
      double v = 0.0;
      for (int w = 0; w < NT / 32; ++w) v += wsum[threadIdx.x][w];
      row[threadIdx.x] = v;
    }
    if (d_sp && has_row)
      for (int i = threadIdx.x; i < a.st.nsh; i += NT) row[4 + i] = hist[i];
  }
}

// ---------------------------------------------------------------------------
// P3 on the register engine: per CTA CP column pairs.  Inverse lines (6 CP):
// l = t * 2CP + c, the packed pair t of column c ((u_x, u_y), (u_z, w_x),
// (w_y, w_z)); the first stage packs straight from global memory with the
// Hermitian extension (z-line helpers above), the last stage writes the
// physical values to buffer B.  The cross product then writes the forward
// lines (3 CP) to buffer A: l = t * CP + pr with (c_x^A + i c_y^A),
// (c_z^A + i c_z^B), (c_x^B + i c_y^B) for the columns A, B of pair pr.  The
// forward transform reads A, exchanges through B and writes its spectra back
// to A, from where the kept H modes are unpacked and stored.
// ---------------------------------------------------------------------------
template <typename R, int M, int CP>
__host__ __device__ constexpr int p3_threads() {
  return cmin(rthreads<R, M, 6 * CP, true>(), 384);
}
// One column pair per CTA (M >= 384): the inverse writes its physical values
// in place, the cross product overwrites three of the six lines position by
// position (each position of the pair is read and written by one thread),
// and the forward exchanges through the other three, so the CTA needs 6
// lines of shared memory instead of 12.
#ifndef VK_P3_INPLACE
#define VK_P3_INPLACE 1
#endif
template <int CP> __host__ __device__ constexpr bool p3_inplace() { return VK_P3_INPLACE && CP == 1; }
template <typename R, int M, int CP>
__host__ __device__ constexpr int p3_smem_lines() { return (p3_inplace<CP>() ? 6 : 12) * CP; }

// Hermitian unpack of a forward line from the last stage's registers:
// butterfly j (lane j of an NS-lane group) holds Z(k) at k = j + NS r, r <
// RAD; the unpack of mode k needs Z(L - k), which is output RAD - 1 - r of
// lane NS - j of the same group, or, for j = 0, output (RAD - r) mod RAD of
// this lane.  f(k, X, Y) receives the two real fields' modes k < H.  All
// lanes of the warp must call it.
template <typename R, int RAD, int NS, int H, class F>
__device__ __forceinline__ void unpack_rows(int j, const C2<R>* v, const F& f) {
  const int lane = threadIdx.x & 31;
  const int src = (lane & ~(NS - 1)) | ((NS - j) & (NS - 1));
#pragma unroll
  for (int r = 0; r * NS < H; ++r) {
    const C2<R> zs = cmk<R>(__shfl_sync(0xffffffffu, v[RAD - 1 - r].x, src),
                            __shfl_sync(0xffffffffu, v[RAD - 1 - r].y, src));
    const C2<R> z = v[r];
    const C2<R> w = j == 0 ? v[(RAD - r) % RAD] : zs;
    const int k = j + NS * r;
    if (k >= H) continue;
    f(k, cmk<R>(R(0.5) * (z.x + w.x), R(0.5) * (z.y - w.y)), cmk<R>(R(0.5) * (z.y + w.y), R(0.5) * (w.x - z.x)));
  }
}

// Row unpack of the forward z transform of k_p3 (forward line l = t CP + pr):
// the kept modes go straight to global memory, in the layout of k_p3's
// shared-memory unpack below.
template <typename R, int M, int CP>
struct P3RowUnpack {
  static constexpr bool kRowStore = true;
  C2<R>* out; size_t fsout; int ncols; int col0;
  template <int RAD, int NS>
  __device__ __forceinline__ void row(int l, int j, const C2<R>* v) const {
    constexpr int H = M / 3 + 1;
    const int t = l / CP, pr = l - t * CP;
    const int ca = col0 + 2 * pr, cb = ca + 1;
    unpack_rows<R, RAD, NS, H>(j, v, [&](int k, const C2<R>& X, const C2<R>& Y) {
      if (t == 0) {
        if (ca < ncols) {
          out[(size_t)ca * H + k] = X;
          out[fsout + (size_t)ca * H + k] = Y;
        }
      } else if (t == 1) {
        if (ca < ncols) out[2 * fsout + (size_t)ca * H + k] = X;
        if (cb < ncols) out[2 * fsout + (size_t)cb * H + k] = Y;
      } else {
        if (cb < ncols) {
          out[(size_t)cb * H + k] = X;
          out[fsout + (size_t)cb * H + k] = Y;
        }
      }
    });
  }
};
// Forward z transforms of NF lines unpack from registers where the last
// stage allows it: FP32 plans whose last stage has 16 or 32 butterflies per
// line over whole warps
template <typename R, int M, int NF, int NT>
__host__ __device__ constexpr bool z_row_unpack() {
  if (sizeof(R) != 4 || VK_P3_ROW_UNPACK == 0) return false;
  constexpr int S = rstages<R, true>(M);
  constexpr int RAD = rradix<R, true>(M, S - 1);
  constexpr int NB = M / RAD;
  return (NB == 16 || NB == 32) && (NB * NF) % 32 == 0 && NT % 32 == 0;
}

template <typename R, int M, int CP, int NT>
__global__ void __launch_bounds__(NT, M >= 768 ? (sizeof(R) == 4 && p3_inplace<CP>() ? 3 : 1)
                                              : cmax(1, (sizeof(R) == 8 ? 768 : 512) / NT))
k_p3(P3Args<R> a, const C2<R>* __restrict__ tw, int pf) {
  constexpr int N = 2 * M / 3;
  constexpr int H = N / 2 + 1;
  constexpr int LP = zpad_len<R>(M);
  constexpr int NI = 6 * CP, NF = 3 * CP;
  constexpr bool INPL = p3_inplace<CP>();
  extern __shared__ __align__(16) unsigned char vk_smem[];
  __shared__ C2<R> tw_s[twtab_elems<R, true>(M)];
  // L2 prefetch of the six input ranges of the CTA pf blocks ahead (FP32:
  // 2 CP columns of H complex values per field, a multiple of 16 bytes at a
  // 16-byte boundary)
  if constexpr (sizeof(R) == 4) {
    const int b = (int)blockIdx.x + pf;
    if (pf > 0 && threadIdx.x < 6 && b < (int)gridDim.x && (b + 1) * 2 * CP <= a.ncols)
      prefetch_l2_bulk(a.in + (size_t)threadIdx.x * a.fsin + (size_t)b * (2 * CP * H), 2 * CP * H * sizeof(C2<R>));
  }
  load_twtab<R, M, true, NT>(tw_s, tw);
  C2<R>* A = reinterpret_cast<C2<R>*>(vk_smem);
  C2<R>* B = INPL ? A : A + NI * LP;
  C2<R>* XF = INPL ? A + NF * LP : B;   // exchange of the forward transform
  const int col0 = blockIdx.x * 2 * CP;
  // positions H .. M - H of the packed lines are the z zero-padding
  fft_lines<R, M, true, NT, NI, MapContig<R, M, NI>, INPL, true, H, M - H + 1>(
      A, tw_s,
      [&](int l, int p) -> C2x2<R> {
        const int t = l / (2 * CP);
        const int col = col0 + l % (2 * CP);
        const bool lo = p < H;
        C2x2<R> r{};
        if (col < a.ncols && (lo || p > M - H)) {
          const C2<R>* src = a.in + (size_t)col * H + (lo ? p : M - p);
          r.a = src[(size_t)(2 * t) * a.fsin];
          r.b = src[(size_t)(2 * t + 1) * a.fsin];
        }
        return r;
      },
      [&](int, int p, const C2x2<R>& r) -> C2<R> {   // Z = X + i Y with the Hermitian extension
        const C2<R> X = r.a, Y = r.b;
        if (p == 0) return cmk<R>(X.x, Y.x);
        return p < H ? cmk<R>(X.x - Y.y, X.y + Y.x) : cmk<R>(X.x + Y.y, Y.x - X.y);
      },
      [&](int l, int p, C2<R> v) { B[l * LP + zi<R>(p)] = v; });
  __syncthreads();
  for (int e = threadIdx.x; e < CP * M; e += NT) {
    const int pr = e / M, p = e % M;
    const int zp = zi<R>(p);
    R c[2][3];
#pragma unroll
    for (int cc = 0; cc < 2; ++cc) {
      const int col = 2 * pr + cc;
      const C2<R> z1 = B[col * LP + zp], z2 = B[(2 * CP + col) * LP + zp], z3 = B[(4 * CP + col) * LP + zp];
      const R ux = z1.x, uy = z1.y, uz = z2.x, wx = z2.y, wy = z3.x, wz = z3.y;
      c[cc][0] = uy * wz - uz * wy;
      c[cc][1] = uz * wx - ux * wz;
      c[cc][2] = ux * wy - uy * wx;
    }
    A[pr * LP + zp] = cmk<R>(c[0][0], c[0][1]);
    A[(CP + pr) * LP + zp] = cmk<R>(c[0][2], c[1][2]);
    A[(2 * CP + pr) * LP + zp] = cmk<R>(c[1][0], c[1][1]);
  }
  __syncthreads();
  if constexpr (z_row_unpack<R, M, NF, NT>()) {
    // the kept modes unpacked from the last stage's registers
    fft_lines<R, M, false, NT, NF, MapContig<R, M, NF>, false, true>(
        XF, tw_s, [&](int l, int p) { return A[l * LP + zi<R>(p)]; }, PrepNone{},
        P3RowUnpack<R, M, CP>{a.out, a.fsout, a.ncols, col0});
    return;
  }
  fft_lines<R, M, false, NT, NF, MapContig<R, M, NF>, false, true>(
      XF, tw_s, [&](int l, int p) { return A[l * LP + zi<R>(p)]; }, PrepNone{},
      [&](int l, int p, C2<R> v) { A[l * LP + zi<R>(p)] = v; });
  __syncthreads();
  for (int e = threadIdx.x; e < CP * 3 * H; e += NT) {
    const int k = e % H;
    const int t = (e / H) % 3;
    const int pr = e / (3 * H);
    C2<R> X, Y;
    zunpack<R>(A + (t * CP + pr) * LP, M, k, X, Y);
    const int ca = col0 + 2 * pr, cb = ca + 1;
    if (t == 0) {
      if (ca < a.ncols) {
        a.out[(size_t)ca * H + k] = X;
        a.out[a.fsout + (size_t)ca * H + k] = Y;
      }
    } else if (t == 1) {
      if (ca < a.ncols) a.out[2 * a.fsout + (size_t)ca * H + k] = X;
      if (cb < a.ncols) a.out[2 * a.fsout + (size_t)cb * H + k] = Y;
    } else {
      if (cb < a.ncols) {
        a.out[(size_t)cb * H + k] = X;
        a.out[a.fsout + (size_t)cb * H + k] = Y;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// N-grid z pass on the register engine: c2r of u and/or omega (already x/y
// inverted and scaled by 1/N^3) packed in pairs, and max |u|^2, max |omega|^2
// over the N^3 grid (solver.rs:180-218 and :537-567).  Lines per column pair:
// BOTH: l = 6 pr + 3 cc + t, the pair t of column cc; otherwise l = 3 pr + cc
// (f0 + i f1 of column cc) and 3 pr + 2 (f2 of both columns).  The inverse
// writes its physical values in place; the maxima follow.
// ---------------------------------------------------------------------------
template <typename R, int N, int CP, bool BOTH>
__host__ __device__ constexpr int nz_threads() {
  return cmin(rthreads<R, N, (BOTH ? 6 : 3) * CP, true>(), 384);
}

template <typename R, int N, int CP, bool BOTH, int NT>
__global__ void __launch_bounds__(NT, N >= 512 ? 1 : cmax(1, (sizeof(R) == 8 ? 768 : 512) / NT))
k_nz_max(NZArgs<R> a, const C2<R>* __restrict__ tw, int pf) {
  constexpr int H = N / 2 + 1;
  constexpr int LPP = BOTH ? 6 : 3;   // lines per column pair
  constexpr int NL = LPP * CP;
  constexpr int LP = zpad_len<R>(N);
  extern __shared__ __align__(16) unsigned char vk_smem[];
  C2<R>* lines = reinterpret_cast<C2<R>*>(vk_smem);
  __shared__ C2<R> tw_s[twtab_elems<R, true>(N)];
  __shared__ double red[2][32];
  __shared__ int redn;
  // L2 prefetch of the input ranges of the CTA pf blocks ahead (FP32: per
  // field 2 CP columns of H complex values, a multiple of 16 bytes at a
  // 16-byte boundary)
  if constexpr (sizeof(R) == 4) {
    const int b = (int)blockIdx.x + pf;
    if (pf > 0 && threadIdx.x < (BOTH ? 6 : 3) && b < (int)gridDim.x && (b + 1) * 2 * CP <= a.ncols)
      prefetch_l2_bulk(a.in + (size_t)threadIdx.x * a.fs + (size_t)b * (2 * CP * H), 2 * CP * H * sizeof(C2<R>));
  }
  load_twtab<R, N, true, NT>(tw_s, tw);
  if (threadIdx.x == 0) redn = 0;
  const int col0 = blockIdx.x * 2 * CP;
  fft_lines<R, N, true, NT, NL, MapContig<R, N, NL>, true, true>(
      lines, tw_s,
      [&](int l, int p) -> C2x2<R> {
        const int pr = l / LPP, j = l % LPP;
        int fx, fy, cx, cy;
        if (BOTH) {
          const int cc = j / 3, t = j % 3;
          fx = 2 * t; fy = 2 * t + 1;
          cx = cy = col0 + 2 * pr + cc;
        } else if (j < 2) {
          fx = 0; fy = 1;
          cx = cy = col0 + 2 * pr + j;
        } else {
          fx = fy = 2;
          cx = col0 + 2 * pr;
          cy = cx + 1;
        }
        const int k = p < H ? p : N - p;
        C2x2<R> r{};
        if (cx < a.ncols) r.a = a.in[(size_t)fx * a.fs + (size_t)cx * H + k];
        if (cy < a.ncols) r.b = a.in[(size_t)fy * a.fs + (size_t)cy * H + k];
        return r;
      },
      [&](int, int p, const C2x2<R>& r) -> C2<R> {   // Z = X + i Y with the Hermitian extension
        const C2<R> X = r.a, Y = r.b;
        if (p == 0 || 2 * p == N) return cmk<R>(X.x, Y.x);   // c2r drops these imaginary parts
        return p < H ? cmk<R>(X.x - Y.y, X.y + Y.x) : cmk<R>(X.x + Y.y, Y.x - X.y);
      },
      [&](int l, int p, C2<R> v) { lines[l * LP + zi<R>(p)] = v; });
  __syncthreads();
  // maxima in the working precision (the FP32-bulk form keeps FP64 only for
  // the dt arithmetic that consumes them)
  R m1 = R(0), m2 = R(0);
  int bad = 0;
  for (int e = threadIdx.x; e < CP * N; e += NT) {
    const int pr = e / N, p = e % N;
#pragma unroll
    for (int cc = 0; cc < 2; ++cc) {
      if (col0 + 2 * pr + cc >= a.ncols) continue;
      if (BOTH) {
        const C2<R>* L0 = lines + (6 * pr + 3 * cc) * LP;
        const C2<R> A = L0[zi<R>(p)], B = L0[LP + zi<R>(p)], C = L0[2 * LP + zi<R>(p)];
        const R ux = A.x, uy = A.y, uz = B.x, wx = B.y, wy = C.x, wz = C.y;
        const R s1 = ux * ux + uy * uy + uz * uz;
        const R s2 = wx * wx + wy * wy + wz * wz;
        bad |= (s1 != s1) | (s2 != s2);
        m1 = fmax(m1, s1);
        m2 = fmax(m2, s2);
      } else {
        const C2<R> A = lines[(3 * pr + cc) * LP + zi<R>(p)];
        const C2<R> Z = lines[(3 * pr + 2) * LP + zi<R>(p)];
        const R fx = A.x, fy = A.y, fz = cc == 0 ? Z.x : Z.y;
        const R s = fx * fx + fy * fy + fz * fz;
        bad |= (s != s);
        m1 = fmax(m1, s);
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    m1 = fmax(m1, __shfl_xor_sync(0xffffffffu, m1, o));
    m2 = fmax(m2, __shfl_xor_sync(0xffffffffu, m2, o));
  }
  const int w = threadIdx.x / 32, ln = threadIdx.x % 32;
  if (bad) atomicOr(&redn, 1);
  if (ln == 0) { red[0][w] = (double)m1; red[1][w] = (double)m2; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double r1 = 0.0, r2 = 0.0;
    for (int i = 0; i < NT / 32; ++i) { r1 = fmax(r1, red[0][i]); r2 = fmax(r2, red[1][i]); }
    if (BOTH) {
      atomic_max_pos(&a.out->umax2, r1);
      atomic_max_pos(&a.out->wmax2, r2);
    } else if (a.which == 2) {
      atomic_max_pos(&a.out->wmax2, r1);
    } else {
      atomic_max_pos(&a.out->umax2, r1);
    }
    if (redn) atomicOr(&a.out->nan_flag, 1);
  }
}


}  // namespace vk
