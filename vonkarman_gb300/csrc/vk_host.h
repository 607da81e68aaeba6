// Declarations shared by the host API and the kernel translation units.
// Host-compilable: no device code here.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace vk {

template <typename R> struct CplxOf;
template <> struct CplxOf<double> { using T = double2; };
template <> struct CplxOf<float> { using T = float2; };
template <typename R> using C2 = typename CplxOf<R>::T;

// N-grid maxima, written with atomicMax on the bit patterns of non-negative
// doubles.
struct MaxOut {
  unsigned long long umax2;
  unsigned long long wmax2;
  int nan_flag;
  int pad;
};

// Device-resident scalars of one solver context.
struct DevScalars {
  double dt;              // current step size
  double time;            // accumulated time
  double cfl_dt;          // last CFL estimate
  int etd_recompute;      // set by the CFL update, read by the ETD table kernel
  int nonfinite;          // sticky: a NaN/Inf was seen in the state (CFL maxima or a step's output)
  int async_timeout;      // sticky: a bulk copy into shared memory did not arrive in time
  MaxOut mx;              // N-grid maxima of the current state
  double sums[4];         // Tier-1 sums (energy, enstrophy, helicity, superhelicity), raw
};

// Kassam-Trefethen contour constants (vonkarman-periodic/src/etd.rs:21-26):
// cos(theta_j), sin(theta_j), cos(sin theta_j), sin(sin theta_j) with
// theta_j = 2 pi (j + 1/2) / 32.
struct ContourConsts {
  double cth[32];
  double sth[32];
  double cos_sth[32];
  double sin_sth[32];
  double exp_cth[32];   // exp(cos theta_j)
};

// Stage epilogue selector (fused into the last pass of a nonlinear evaluation).
enum StageOp : int {
  ST_NL_OUT = 0,
  ST_ETD_REF_1 = 1, ST_ETD_REF_2 = 2, ST_ETD_REF_3 = 3, ST_ETD_4 = 4,
  ST_ETD_CM_1 = 5, ST_ETD_CM_2 = 6, ST_ETD_CM_3 = 7,
  ST_RK4_1 = 8, ST_RK4_2 = 9, ST_RK4_3 = 10, ST_RK4_4 = 11,
};
enum EtdSlot : int { E_FULL = 0, E_HALF = 1, E_A21 = 2, E_A41 = 3, E_B1 = 4, E_B23 = 5, E_B4 = 6 };
constexpr int ETD_STRIDE = 8;

template <typename R> struct StageArgs {
  int op;
  size_t cs;                       // component stride of spectral arrays
  C2<R>* u; C2<R>* temp; C2<R>* n1; C2<R>* acc; C2<R>* out;
  C2<R>* u_out;                    // where the last ETD stage writes u_{n+1} (normally u)
  const double* etd;               // table, ETD_STRIDE doubles per |k|^2 index
  const double* dt;                // device scalar
  double nu;
  int* nonfinite;                  // set when a final stage writes a non-finite value (null: no check)
  // Diagnostics fused into a final stage (ST_ETD_4 / ST_RK4_4): bit 0 = the
  // four Tier-1 sums, bit 1 = the shell spectrum of the new state, one row of
  // 4 + nsh doubles per CTA of the pass in dpart (0 / null: none).
  int diag;
  int nsh;
  double* dpart;
  int dpart_rows;                  // rows allocated in dpart (a CTA past them writes nothing)
  double ks;                       // 2 pi / L (shells of boxes other than 2 pi)
};

// Modes per CTA of the final pass (k_p5: N / 2 + 1 consecutive z per x line,
// lines tiled by this many) and its CTA count, which sizes the fused
// diagnostics' partial rows.
inline constexpr int p5_lines(int n, bool fp32) { return (void)n, fp32 ? 8 : 4; }
inline constexpr int p5_ctas(int n, bool fp32) { return (n * (n / 2 + 1) + p5_lines(n, fp32) - 1) / p5_lines(n, fp32); }
enum DiagBits : int { DIAG_TIER1 = 1, DIAG_SPECTRUM = 2 };

// Per-pass timing hook (profiling mode): brackets each kernel launch with
// CUDA events on the launching stream.  Pass ids follow enum Pass.
enum Pass : int {
  PASS_P1 = 0, PASS_P2, PASS_P3, PASS_P4, PASS_P5,
  PASS_NX, PASS_NY, PASS_NZ, PASS_ETD, PASS_SMALL, PASS_TIER1, PASS_SPECTRUM,
  PASS_FFT_Z, PASS_FFT_Y, PASS_FFT_X,
  PASS_A1, PASS_A2, PASS_A3, PASS_A4, PASS_A5,
  PASS_COUNT
};
struct KTimer {
  virtual void begin(int pass, cudaStream_t s) = 0;
  virtual void end(int pass, cudaStream_t s) = 0;
  virtual ~KTimer() {}
};
struct TimerScope {
  KTimer* t; int pass; cudaStream_t s;
  TimerScope(KTimer* t_, int pass_, cudaStream_t s_) : t(t_), pass(pass_), s(s_) { if (t) t->begin(pass, s); }
  ~TimerScope() { if (t) t->end(pass, s); }
};

template <typename R> struct NleParams {
  int N;
  double ks;                           // 2 pi / L
  const C2<R>* in;                     // spectral input (3 components)
  size_t cs;                           // component stride (N*N*H)
  C2<R>* bufA; C2<R>* bufB;            // work buffers
  const C2<R>* twM;                    // twiddles, length M = 3N/2
  StageArgs<R> st;
  KTimer* timer;                       // null unless profiling
  cudaEvent_t wait_p5;                 // if set, P5 waits for it (work P5 alone depends on)
  int* async_err;                      // set by a kernel whose bulk copy timed out
};

template <typename R> struct NgridParams {
  int N;
  double ks;
  const C2<R>* in; size_t cs;
  C2<R>* bufA; C2<R>* bufB;
  const C2<R>* twN;
  MaxOut* out;
  int which;                           // 1 = u, 2 = omega, 3 = both
  KTimer* timer;
};

template <typename R> struct FftParams {
  int nx, ny, nz;
  R* real; C2<R>* cplx;
  const C2<R>* twx; const C2<R>* twy; const C2<R>* twz;
  KTimer* timer;
};

// Adjoint stage combinations (see vk_adjoint.cuh).
enum AdjOp : int { ADJ_NL_OUT = 0, ADJ_C = 1, ADJ_B = 2, ADJ_A = 3, ADJ_U = 4 };

template <typename R> struct AdjStageArgs {
  int op;
  size_t cs;
  C2<R>* ub; C2<R>* acc; C2<R>* nb; C2<R>* n1b; C2<R>* out;
  const double* etd;
  const double* dt;
};

// One adjoint nonlinear evaluation y = N'(x)^T nbar with a stage epilogue.
template <typename R> struct NlaParams {
  int N;
  double ks;
  const C2<R>* x; size_t cs;             // stage input
  const C2<R>* nb;                       // cotangent source
  const double* etd; int slot; double fac;   // nbar = fac dt etd[slot] nb if slot >= 0
  const double* dt;
  C2<R>* bufA; C2<R>* bufB;              // >= max(8 MNH, 6 M^2H), >= max(9 M^2H, 6 MNH)
  const C2<R>* twM;
  AdjStageArgs<R> st;
  KTimer* timer;
};

template <typename R> struct Engine {
  static cudaError_t nle(const NleParams<R>& p, cudaStream_t s);
  static cudaError_t ngrid_max(const NgridParams<R>& p, cudaStream_t s);
  static cudaError_t fft_r2c(const FftParams<R>& p, cudaStream_t s);
  static cudaError_t fft_c2r(const FftParams<R>& p, cudaStream_t s);
  static cudaError_t tier1_partial(const C2<R>* u, size_t cs, int N, double ks, double* part, int nblk,
                                   cudaStream_t s);
  static cudaError_t spectrum_partial(const C2<R>* u, size_t cs, int N, double ks, int nsh, double* part,
                                      int nblk, cudaStream_t s);
  static cudaError_t nle_adjoint(const NlaParams<R>& p, cudaStream_t s);
  // mode 0: enstrophy cotangent of in; mode 1: weighted gradient (Nyquist-free, Leray)
  static cudaError_t adj_mode(int N, double ks, size_t cs, const C2<R>* in, C2<R>* out, int mode, cudaStream_t s);
  static cudaError_t hermitian_avg(int N, size_t cs, const C2<R>* in, C2<R>* out, cudaStream_t s);
};
extern template struct Engine<double>;
extern template struct Engine<float>;

constexpr int RED_THREADS = 256;

// Non-template launchers (vk_misc.cu).
cudaError_t launch_etd_table(double* tab, int nent, double nu, double ks2, const DevScalars* d, int force,
                             const ContourConsts& cc, cudaStream_t s);
cudaError_t launch_cfl_update(DevScalars* d, double dx, double nu, double safety, int mode, cudaStream_t s);
cudaError_t launch_reset_max(DevScalars* d, cudaStream_t s);
cudaError_t launch_time_advance(DevScalars* d, cudaStream_t s);
cudaError_t launch_reduce_columns(const double* part, int nblk, int width, double* out, cudaStream_t s,
                                  double scale = 1.0, int ld = 0);
// |k|^2 of every mode of an (n, n, n/2+1) grid (SpectralOps::k_mag_sq) and
// SpectralOps::apply_viscous on a device vector field (fp32: float2 data).
cudaError_t launch_k_mag_sq(double* out, int n, double ks, cudaStream_t s);
cudaError_t launch_apply_viscous(void* out, const void* in, int fp32, int n, size_t cs, double ks, double nu,
                                 cudaStream_t s);
// complex arrays: fp32 flags select float2 (1) or double2 (0)
cudaError_t launch_convert_c(void* out, int out_fp32, const void* in, int in_fp32, size_t n, cudaStream_t s);
cudaError_t launch_convert_r(void* out, int out_fp32, const void* in, int in_fp32, size_t n, cudaStream_t s);
// FP64 / FP32 FMA throughput probe (GFLOP/s, best of 5 launches).
cudaError_t probe_fma_peak(int fp64, double* gflops);

}  // namespace vk
