// C ABI of the GB300 periodic pseudospectral solver (declared in
// include/vonkarman_gpu.h).  Host orchestration only: buffers, the per-step
// launch schedule and readbacks.  All arithmetic runs in the kernels of
// vk_engine_f64.cu / vk_engine_f32.cu / vk_misc.cu.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "vk_host.h"
#include "vk_schedule.h"
#include "vonkarman_gpu.h"

using vk::C2;

namespace {

thread_local std::string g_create_error;

struct DeviceGuard {
  int prev = -1;
  bool ok = true;
  explicit DeviceGuard(int dev) {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    if (prev != dev) ok = cudaSetDevice(dev) == cudaSuccess;
  }
  ~DeviceGuard() {
    int cur = -1;
    if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
  }
};

bool is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }
bool fft_len_ok(int n) {
  if (n < 8 || n > 768) return false;
  if (is_pow2(n)) return n <= 512;
  return n % 3 == 0 && is_pow2(n / 3) && n / 3 >= 4;
}

// W_L^m = exp(-2 pi i m / L), computed in long double and rounded once.
std::vector<double> twiddle_table(int L) {
  std::vector<double> t(2 * (size_t)L);
  const long double two_pi = 6.283185307179586476925286766559005768L;
  for (int m = 0; m < L; ++m) {
    const long double a = two_pi * (long double)m / (long double)L;
    t[2 * m] = (double)cosl(a);
    t[2 * m + 1] = (double)(-sinl(a));
  }
  return t;
}

cudaError_t upload_twiddles(int L, bool fp32, void** dst) {
  std::vector<double> t = twiddle_table(L);
  size_t bytes = (size_t)L * (fp32 ? sizeof(float2) : sizeof(double2));
  cudaError_t e = cudaMalloc(dst, bytes);
  if (e != cudaSuccess) return e;
  if (fp32) {
    std::vector<float> f(t.size());
    for (size_t i = 0; i < t.size(); ++i) f[i] = (float)t[i];
    return cudaMemcpy(*dst, f.data(), bytes, cudaMemcpyHostToDevice);
  }
  return cudaMemcpy(*dst, t.data(), bytes, cudaMemcpyHostToDevice);
}

// theta_j = 2 pi (j + 1/2) / 32 evaluated as in etd.rs:22, then the constant
// parts of w = z + e^{i theta_j}.
vk::ContourConsts contour_consts() {
  vk::ContourConsts c;
  const double pi = 3.14159265358979323846;
  for (int j = 0; j < 32; ++j) {
    const double theta = 2.0 * pi * ((double)j + 0.5) / 32.0;
    c.cth[j] = 1.0 * std::cos(theta);
    c.sth[j] = 1.0 * std::sin(theta);
    c.cos_sth[j] = std::cos(c.sth[j]);
    c.sin_sth[j] = std::sin(c.sth[j]);
    c.exp_cth[j] = std::exp(c.cth[j]);
  }
  return c;
}

// Profiling mode: every pass launch is bracketed by CUDA events on the
// launching stream; durations are summed per pass after a synchronisation.
struct EventTimer : vk::KTimer {
  struct Rec { int pass; cudaEvent_t a, b; };
  std::vector<cudaEvent_t> pool;
  size_t next = 0;
  std::vector<Rec> recs;
  std::vector<std::pair<int, cudaEvent_t>> open;
  double ms[vk::PASS_COUNT] = {0};
  int64_t cnt[vk::PASS_COUNT] = {0};
  cudaEvent_t get() {
    if (next == pool.size()) {
      cudaEvent_t e = nullptr;
      cudaEventCreate(&e);
      pool.push_back(e);
    }
    return pool[next++];
  }
  void begin(int pass, cudaStream_t s) override {
    cudaEvent_t e = get();
    cudaEventRecord(e, s);
    open.push_back({pass, e});
  }
  void end(int pass, cudaStream_t s) override {
    cudaEvent_t e = get();
    cudaEventRecord(e, s);
    if (open.empty()) return;
    auto o = open.back();
    open.pop_back();
    recs.push_back({o.first, o.second, e});
  }
  // Caller has synchronised the stream.
  void collect() {
    for (const Rec& r : recs) {
      float t = 0.f;
      if (cudaEventElapsedTime(&t, r.a, r.b) == cudaSuccess) {
        ms[r.pass] += t;
        cnt[r.pass] += 1;
      }
    }
    recs.clear();
    open.clear();
    next = 0;
  }
  void reset() {
    collect();
    for (int i = 0; i < vk::PASS_COUNT; ++i) { ms[i] = 0.0; cnt[i] = 0; }
  }
  ~EventTimer() override {
    for (cudaEvent_t e : pool) cudaEventDestroy(e);
  }
};

}  // namespace

struct vk_ctx {
  vk_config cfg{};
  int N = 0, H = 0, M = 0;
  bool fp32 = false;
  size_t cs = 0;        // complex entries per spectral component
  size_t esz = 0;       // bytes per complex entry on the device
  int dev_sms = 0;
  cudaStream_t stream = nullptr;
  void* u = nullptr;
  void* temp = nullptr;
  void* n1 = nullptr;
  void* acc = nullptr;
  void* bufA = nullptr;
  void* bufB = nullptr;
  size_t bufA_bytes = 0, bufB_bytes = 0;
  void* twN = nullptr;
  void* twM = nullptr;
  double* etd = nullptr;
  int n_etd = 0;
  vk::DevScalars* dsc = nullptr;
  vk::DevScalars* records = nullptr;
  int64_t records_cap = 0;
  double* part = nullptr;
  int red_blocks = 0;
  int n_shells = 0;
  double* dspec = nullptr;
  // diagnostics fused into the final stage of a step (partial rows of k_p5)
  double* dpart = nullptr;
  int dpart_rows = 0;
  int diag_valid = 0;                 // DiagBits the rows hold for the current state
  int64_t fuse_t1_every = 0, fuse_spec_every = 0;
  // steps replayed as CUDA graphs, one per launch-sequence key (step_graph)
  struct StepGraph {
    cudaGraphExec_t exec = nullptr;
    bool eager = false;
  } graphs[8];
  // the ETD table of a new dt runs on a second stream beside the first
  // stage's P1..P4 (only its P5 reads the table): fork at ev_dt, join at ev_etd
  cudaStream_t side = nullptr;
  cudaEvent_t ev_dt = nullptr, ev_etd = nullptr;
  bool use_graphs = true;
  bool has_state = false;
  bool umax_fresh = false;   // dsc->mx.umax2 describes the current state
  uint64_t step_count = 0;
  double ks = 1.0;
  vk::ContourConsts cc{};
  EventTimer* prof = nullptr;
  // discrete adjoint (allocated on first use)
  struct Adjoint {
    int64_t nsteps = 0;
    int64_t K = 0;                  // steps per checkpoint segment
    int64_t nseg = 0;
    std::vector<void*> ckpt;        // state at the start of each segment
    std::vector<void*> seg;         // S[0..K], A[0..K-1], B[0..K-1], C[0..K-1]
    std::vector<int64_t> pos;       // binomial: step index of the state in each checkpoint slot (-1: none)
    void* ub = nullptr;
    void* acc = nullptr;
    void* nb = nullptr;
    void* n1b = nullptr;
    void* bufA = nullptr;
    void* bufB = nullptr;
    size_t bufA_bytes = 0, bufB_bytes = 0;
    bool ready = false;
    double J = 0.0;
    int schedule = VK_ADJ_TWO_LEVEL;   // for the next forward
    int used = VK_ADJ_TWO_LEVEL;       // of the last forward
  } adj;
  cudaEvent_t tev[2] = {nullptr, nullptr};
  cudaEvent_t marks[8] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  std::string err;
};

struct vk_fft {
  int nx = 0, ny = 0, nz = 0, hz = 0;
  bool fp32 = false;
  int device = 0;
  cudaStream_t stream = nullptr;
  void* real = nullptr;
  void* cplx = nullptr;
  void* stage = nullptr;   // f64 staging for the fp32 plan
  void* twx = nullptr;
  void* twy = nullptr;
  void* twz = nullptr;
  std::string err;
};

namespace {

int fail(vk_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

int cuda_fail(vk_ctx* c, cudaError_t e, const char* where) {
  std::string m = std::string(where) + ": " + cudaGetErrorString(e);
  if (c) c->err = m;
  return e == cudaErrorMemoryAllocation ? VK_ERR_OOM : VK_ERR_CUDA;
}

#define VK_CHECK(ctx, call)                                  \
  do {                                                       \
    cudaError_t _e = (call);                                 \
    if (_e != cudaSuccess) return cuda_fail((ctx), _e, #call); \
  } while (0)

template <typename R>
vk::StageArgs<R> stage_args(vk_ctx* c, int op, void* out) {
  vk::StageArgs<R> s{};
  s.op = op;
  s.cs = c->cs;
  s.u = (C2<R>*)c->u;
  s.temp = (C2<R>*)c->temp;
  s.n1 = (C2<R>*)c->n1;
  s.acc = (C2<R>*)c->acc;
  s.out = (C2<R>*)out;
  s.u_out = s.u;
  s.etd = c->etd;
  s.dt = &c->dsc->dt;
  s.nu = c->cfg.nu;
  s.nonfinite = &c->dsc->nonfinite;
  s.diag = 0;
  s.nsh = c->n_shells;
  s.dpart = c->dpart;
  s.dpart_rows = c->dpart_rows;
  s.ks = c->ks;
  return s;
}

template <typename R>
cudaError_t nle_t(vk_ctx* c, const void* in, int op, void* out, int diag, cudaEvent_t wait_p5) {
  vk::NleParams<R> p{};
  p.N = c->N;
  p.ks = c->ks;
  p.in = (const C2<R>*)in;
  p.cs = c->cs;
  p.bufA = (C2<R>*)c->bufA;
  p.bufB = (C2<R>*)c->bufB;
  p.twM = (const C2<R>*)c->twM;
  p.st = stage_args<R>(c, op, out);
  p.st.diag = diag;
  p.timer = c->prof;
  p.wait_p5 = wait_p5;
  p.async_err = &c->dsc->async_timeout;
  return vk::Engine<R>::nle(p, c->stream);
}

// diag: DiagBits to accumulate from the new state (final stages only);
// wait_p5: an event that P5 (the stage epilogue) waits for.
cudaError_t nle(vk_ctx* c, const void* in, int op, void* out = nullptr, int diag = 0,
                cudaEvent_t wait_p5 = nullptr) {
  return c->fp32 ? nle_t<float>(c, in, op, out, diag, wait_p5) : nle_t<double>(c, in, op, out, diag, wait_p5);
}

template <typename R>
cudaError_t ngrid_t(vk_ctx* c, const void* in, int which) {
  vk::NgridParams<R> p{};
  p.N = c->N;
  p.ks = c->ks;
  p.in = (const C2<R>*)in;
  p.cs = c->cs;
  p.bufA = (C2<R>*)c->bufA;
  p.bufB = (C2<R>*)c->bufB;
  p.twN = (const C2<R>*)c->twN;
  p.out = &c->dsc->mx;
  p.which = which;
  p.timer = c->prof;
  return vk::Engine<R>::ngrid_max(p, c->stream);
}

// Maxima over the N grid of the current state: which = 1 (|u|), 2 (|omega|), 3 (both).
cudaError_t ngrid(vk_ctx* c, int which) {
  cudaError_t e;
  {
    vk::TimerScope ts(c->prof, vk::PASS_SMALL, c->stream);
    e = vk::launch_reset_max(c->dsc, c->stream);
  }
  if (e != cudaSuccess) return e;
  e = c->fp32 ? ngrid_t<float>(c, c->u, which) : ngrid_t<double>(c, c->u, which);
  if (e == cudaSuccess && which != 2) c->umax_fresh = true;
  return e;
}

double dx_of(const vk_ctx* c) { return c->cfg.lx / (double)c->N; }

cudaError_t etd_table(vk_ctx* c, int force) {
  vk::TimerScope ts(c->prof, vk::PASS_ETD, c->stream);
  return vk::launch_etd_table(c->etd, c->n_etd, c->cfg.nu, c->ks * c->ks, c->dsc, force, c->cc, c->stream);
}

// The kernels of one step, enqueued on the context's stream (no host-side
// bookkeeping besides ngrid's flag, so the sequence can be captured).
cudaError_t enqueue_step(vk_ctx* c, int diag) {
  cudaError_t e;
  const bool rk4 = c->cfg.integrator == VK_INTEGRATOR_RK4;
  cudaEvent_t etd_ready = nullptr;
  if (c->cfg.dt_mode == VK_DT_CFL) {
    if (!c->umax_fresh) {
      e = ngrid(c, 1);
      if (e != cudaSuccess) return e;
    }
    {
      vk::TimerScope ts(c->prof, vk::PASS_SMALL, c->stream);
      e = vk::launch_cfl_update(c->dsc, dx_of(c), c->cfg.nu, c->cfg.cfl_safety, 0, c->stream);
    }
    if (e != cudaSuccess) return e;
    if (!rk4 && c->prof) {
      e = etd_table(c, 0);   // in order, so that the pass timers see it alone
      if (e != cudaSuccess) return e;
    } else if (!rk4) {
      // the table for the new dt beside the first stage's P1..P4
      if ((e = cudaEventRecord(c->ev_dt, c->stream)) != cudaSuccess) return e;
      if ((e = cudaStreamWaitEvent(c->side, c->ev_dt, 0)) != cudaSuccess) return e;
      e = vk::launch_etd_table(c->etd, c->n_etd, c->cfg.nu, c->ks * c->ks, c->dsc, 0, c->cc, c->side);
      if (e != cudaSuccess) return e;
      if ((e = cudaEventRecord(c->ev_etd, c->side)) != cudaSuccess) return e;
      etd_ready = c->ev_etd;
    }
  }
  int ops[4];
  if (rk4) {
    ops[0] = vk::ST_RK4_1; ops[1] = vk::ST_RK4_2; ops[2] = vk::ST_RK4_3; ops[3] = vk::ST_RK4_4;
  } else if (c->cfg.etd_variant == VK_ETD_COX_MATTHEWS) {
    ops[0] = vk::ST_ETD_CM_1; ops[1] = vk::ST_ETD_CM_2; ops[2] = vk::ST_ETD_CM_3; ops[3] = vk::ST_ETD_4;
  } else {
    ops[0] = vk::ST_ETD_REF_1; ops[1] = vk::ST_ETD_REF_2; ops[2] = vk::ST_ETD_REF_3; ops[3] = vk::ST_ETD_4;
  }
  for (int s = 0; s < 4; ++s) {
    e = nle(c, s == 0 ? c->u : c->temp, ops[s], nullptr, s == 3 ? diag : 0, s == 0 ? etd_ready : nullptr);
    if (e != cudaSuccess) return e;
  }
  vk::TimerScope ts(c->prof, vk::PASS_SMALL, c->stream);
  return vk::launch_time_advance(c->dsc, c->stream);
}

// A step as a CUDA graph: the launch sequence of a step depends only on the
// fused-diagnostics bits and on whether the N-grid maxima of the state are
// already known, so one graph per such key is captured (after the key has
// run once eagerly, which performs every kernel's one-time set-up) and then
// replayed, replacing about 30 kernel launches per step by one.
cudaError_t step_graph(vk_ctx* c, int diag) {
  const int key = diag | (c->cfg.dt_mode == VK_DT_CFL && c->umax_fresh ? 4 : 0);
  vk_ctx::StepGraph& g = c->graphs[key];
  if (g.exec) return cudaGraphLaunch(g.exec, c->stream);
  if (!g.eager) {
    g.eager = true;
    return enqueue_step(c, diag);
  }
  cudaError_t e = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return e;
  const cudaError_t e_enq = enqueue_step(c, diag);
  cudaGraph_t graph = nullptr;
  const cudaError_t e_end = cudaStreamEndCapture(c->stream, &graph);
  if (e_enq != cudaSuccess || e_end != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    return e_enq != cudaSuccess ? e_enq : e_end;
  }
  e = cudaGraphInstantiate(&g.exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) {
    g.exec = nullptr;
    return e;
  }
  return cudaGraphLaunch(g.exec, c->stream);
}

// Domain::step (solver.rs:383-400).  diag: DiagBits that the final stage
// also accumulates from the new state, besides those of the context's fused
// cadence (vk_set_fused_diagnostics).
cudaError_t step_once(vk_ctx* c, int diag = 0) {
  {
    const uint64_t next = c->step_count + 1;
    if (c->fuse_t1_every > 0 && next % (uint64_t)c->fuse_t1_every == 0) diag |= vk::DIAG_TIER1;
    if (c->fuse_spec_every > 0 && next % (uint64_t)c->fuse_spec_every == 0) diag |= vk::DIAG_SPECTRUM;
  }
  const cudaError_t e = c->use_graphs && !c->prof ? step_graph(c, diag) : enqueue_step(c, diag);
  if (e != cudaSuccess) return e;
  c->diag_valid = diag;
  c->step_count += 1;
  c->umax_fresh = false;
  return cudaSuccess;
}

// Tier-1 sums into dsc->sums and N-grid maxima (u and omega) into dsc->mx.
// When the step that produced the state already accumulated the sums
// (fused), only its partial rows are added.
cudaError_t tier1_enqueue(vk_ctx* c) {
  vk::TimerScope ts(c->prof, vk::PASS_TIER1, c->stream);
  cudaError_t e;
  if (c->diag_valid & vk::DIAG_TIER1) {
    e = vk::launch_reduce_columns(c->dpart, c->dpart_rows, 4, c->dsc->sums, c->stream, 1.0, 4 + c->n_shells);
    if (e != cudaSuccess) return e;
    return ngrid(c, 3);
  }
  e = c->fp32
      ? vk::Engine<float>::tier1_partial((const float2*)c->u, c->cs, c->N, c->ks, c->part, c->red_blocks, c->stream)
      : vk::Engine<double>::tier1_partial((const double2*)c->u, c->cs, c->N, c->ks, c->part, c->red_blocks,
                                          c->stream);
  if (e != cudaSuccess) return e;
  e = vk::launch_reduce_columns(c->part, c->red_blocks, 4, c->dsc->sums, c->stream);
  if (e != cudaSuccess) return e;
  return ngrid(c, 3);
}

void fill_tier1(const vk_ctx* c, const vk::DevScalars& d, uint64_t step, vk_tier1_out* o) {
  const double ntot = (double)c->N * (double)c->N * (double)c->N;
  const double n2 = ntot * ntot;
  const double nu = c->cfg.nu;
  o->time = d.time;
  o->step = step;
  o->dt = d.dt;
  o->energy = 0.5 * d.sums[0] / n2;
  o->enstrophy = d.sums[1] / n2;
  o->helicity = d.sums[2] / n2;
  o->superhelicity = d.sums[3] / n2;
  double w2;
  std::memcpy(&w2, &d.mx.wmax2, sizeof(double));
  o->max_vorticity = std::sqrt(w2);
  o->energy_dissipation_rate = -2.0 * nu * o->enstrophy;
  o->helicity_dissipation_rate = -2.0 * nu * o->superhelicity;
  o->cfl_number = o->max_vorticity * o->dt / dx_of(c);
}

// Device scalars of the context after a synchronisation.  A NaN or infinity
// seen in the state since it was set (by a CFL / max pass or by the final
// stage of a step) is reported here, at the first synchronising call after
// it: the checks of the reference's audit (vonkarman-diag/src/audit.rs:175-197)
// without a per-step readback.
int read_scalars(vk_ctx* c, vk::DevScalars* h) {
  VK_CHECK(c, cudaMemcpyAsync(h, c->dsc, sizeof(vk::DevScalars), cudaMemcpyDeviceToHost, c->stream));
  VK_CHECK(c, cudaStreamSynchronize(c->stream));
  if (h->async_timeout) return fail(c, VK_ERR_CUDA, "a bulk copy into shared memory did not arrive in time");
  if (h->nonfinite || h->mx.nan_flag)
    return fail(c, VK_ERR_NONFINITE, "non-finite value (NaN or Inf) in the solver state");
  return VK_OK;
}

// Upload three host f64 components into dst (device precision of the context).
int upload_state(vk_ctx* c, void* dst, const double* ux, const double* uy, const double* uz) {
  const double* src[3] = {ux, uy, uz};
  const size_t bytes64 = c->cs * sizeof(double2);
  for (int k = 0; k < 3; ++k) {
    if (!src[k]) return fail(c, VK_ERR_INVALID, "null state pointer");
    if (!c->fp32) {
      VK_CHECK(c, cudaMemcpyAsync((char*)dst + k * bytes64, src[k], bytes64, cudaMemcpyHostToDevice, c->stream));
    } else {
      VK_CHECK(c, cudaMemcpyAsync(c->bufA, src[k], bytes64, cudaMemcpyHostToDevice, c->stream));
      VK_CHECK(c, vk::launch_convert_c((char*)dst + k * c->cs * sizeof(float2), 1, c->bufA, 0, c->cs, c->stream));
    }
  }
  return VK_OK;
}

int download_state(vk_ctx* c, const void* srcdev, double* ux, double* uy, double* uz) {
  double* dst[3] = {ux, uy, uz};
  const size_t bytes64 = c->cs * sizeof(double2);
  for (int k = 0; k < 3; ++k) {
    if (!dst[k]) return fail(c, VK_ERR_INVALID, "null output pointer");
    if (!c->fp32) {
      VK_CHECK(c, cudaMemcpyAsync(dst[k], (const char*)srcdev + k * bytes64, bytes64, cudaMemcpyDeviceToHost,
                                  c->stream));
    } else {
      VK_CHECK(c, vk::launch_convert_c(c->bufA, 0, (const char*)srcdev + k * c->cs * sizeof(float2), 1, c->cs,
                                       c->stream));
      VK_CHECK(c, cudaMemcpyAsync(dst[k], c->bufA, bytes64, cudaMemcpyDeviceToHost, c->stream));
    }
  }
  VK_CHECK(c, cudaStreamSynchronize(c->stream));
  return VK_OK;
}

void free_adjoint(vk_ctx* c) {
  for (void* p : c->adj.ckpt)
    if (p) cudaFree(p);
  for (void* p : c->adj.seg)
    if (p) cudaFree(p);
  c->adj.ckpt.clear();
  c->adj.seg.clear();
  void* ptrs[] = {c->adj.ub, c->adj.acc, c->adj.nb, c->adj.n1b, c->adj.bufA, c->adj.bufB};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  c->adj = vk_ctx::Adjoint();
}

void free_graphs(vk_ctx* c) {
  for (auto& g : c->graphs) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    g = vk_ctx::StepGraph();
  }
}

void free_ctx(vk_ctx* c) {
  free_graphs(c);
  free_adjoint(c);
  delete c->prof;
  c->prof = nullptr;
  for (cudaEvent_t& e : c->tev)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t& e : c->marks)
    if (e) cudaEventDestroy(e);
  void* ptrs[] = {c->u, c->temp, c->n1, c->acc, c->bufA, c->bufB, c->twN, c->twM,
                  c->etd, c->dsc, c->records, c->part, c->dspec, c->dpart};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (c->ev_dt) cudaEventDestroy(c->ev_dt);
  if (c->ev_etd) cudaEventDestroy(c->ev_etd);
  if (c->side) cudaStreamDestroy(c->side);
  if (c->stream) cudaStreamDestroy(c->stream);
}

}  // namespace

namespace vk {
// Error message of a context-free entry point, read back by vk_last_error(NULL).
void set_global_error(const char* msg) { g_create_error = msg ? msg : ""; }
}  // namespace vk

// ============================================================================
extern "C" {

int vk_abi_version(void) { return VK_ABI_VERSION; }

const char* vk_last_error(const vk_ctx* ctx) { return ctx ? ctx->err.c_str() : g_create_error.c_str(); }

void vk_config_default(vk_config* cfg, int32_t n, double nu) {
  if (!cfg) return;
  std::memset(cfg, 0, sizeof(*cfg));
  const double two_pi = 2.0 * 3.14159265358979323846;
  cfg->nx = cfg->ny = cfg->nz = n;
  cfg->lx = cfg->ly = cfg->lz = two_pi;
  cfg->nu = nu;
  cfg->precision = VK_PRECISION_FP64;
  cfg->etd_variant = VK_ETD_REFERENCE;
  cfg->integrator = VK_INTEGRATOR_ETD_RK4;
  cfg->dt_mode = VK_DT_CFL;
  cfg->dt_fixed = 0.0;
  cfg->cfl_safety = 0.5;
  cfg->device = 0;
}

int vk_create(const vk_config* cfg, vk_ctx** out) {
  if (!cfg || !out) { g_create_error = "null argument"; return VK_ERR_INVALID; }
  *out = nullptr;
  const int n = cfg->nx;
  if (cfg->ny != n || cfg->nz != n) { g_create_error = "only cubic grids (nx == ny == nz) are supported"; return VK_ERR_UNSUPPORTED; }
  if (n < 8 || !is_pow2(n)) { g_create_error = "n must be a power of 2 and >= 8"; return VK_ERR_INVALID; }
  if (n > 512) { g_create_error = "n > 512 is not built"; return VK_ERR_UNSUPPORTED; }
  if (!(cfg->lx > 0.0) || cfg->ly != cfg->lx || cfg->lz != cfg->lx) { g_create_error = "lx == ly == lz > 0 required"; return VK_ERR_INVALID; }
  if (!(cfg->nu > 0.0)) { g_create_error = "nu must be > 0"; return VK_ERR_INVALID; }
  if (cfg->precision != VK_PRECISION_FP64 && cfg->precision != VK_PRECISION_FP32BULK) { g_create_error = "bad precision"; return VK_ERR_INVALID; }
  if (cfg->etd_variant != VK_ETD_REFERENCE && cfg->etd_variant != VK_ETD_COX_MATTHEWS) { g_create_error = "bad etd_variant"; return VK_ERR_INVALID; }
  if (cfg->integrator != VK_INTEGRATOR_ETD_RK4 && cfg->integrator != VK_INTEGRATOR_RK4) { g_create_error = "bad integrator"; return VK_ERR_INVALID; }
  if (cfg->dt_mode == VK_DT_FIXED) {
    if (!(cfg->dt_fixed > 0.0)) { g_create_error = "dt_fixed must be > 0"; return VK_ERR_INVALID; }
  } else if (cfg->dt_mode == VK_DT_CFL) {
    if (!(cfg->cfl_safety > 0.0 && cfg->cfl_safety <= 1.0)) { g_create_error = "cfl_safety must be in (0, 1]"; return VK_ERR_INVALID; }
  } else {
    g_create_error = "bad dt_mode";
    return VK_ERR_INVALID;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) { g_create_error = "no CUDA device available"; return VK_ERR_CUDA; }
  if (cfg->device < 0 || cfg->device >= ndev) { g_create_error = "device ordinal out of range"; return VK_ERR_INVALID; }
  DeviceGuard g(cfg->device);
  if (!g.ok) { g_create_error = "cudaSetDevice failed"; return VK_ERR_CUDA; }

  vk_ctx* c = new vk_ctx();
  c->cfg = *cfg;
  c->N = n;
  c->H = n / 2 + 1;
  c->M = 3 * n / 2;
  c->fp32 = cfg->precision == VK_PRECISION_FP32BULK;
  c->cs = (size_t)n * n * c->H;
  c->esz = c->fp32 ? sizeof(float2) : sizeof(double2);
  c->ks = 2.0 * 3.14159265358979323846 / cfg->lx;
  c->cc = contour_consts();
  const size_t N = n, H = c->H, M = c->M;
  auto bail = [&](cudaError_t e, const char* what) {
    g_create_error = std::string(what) + ": " + cudaGetErrorString(e);
    free_ctx(c);
    delete c;
    return e == cudaErrorMemoryAllocation ? VK_ERR_OOM : VK_ERR_CUDA;
  };
  cudaError_t e;
  cudaDeviceProp prop;
  if ((e = cudaGetDeviceProperties(&prop, cfg->device)) != cudaSuccess) return bail(e, "cudaGetDeviceProperties");
  c->dev_sms = prop.multiProcessorCount;
  if ((e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking)) != cudaSuccess) return bail(e, "cudaStreamCreate");
  if ((e = cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking)) != cudaSuccess) return bail(e, "cudaStreamCreate");
  if ((e = cudaEventCreateWithFlags(&c->ev_dt, cudaEventDisableTiming)) != cudaSuccess) return bail(e, "cudaEventCreate");
  if ((e = cudaEventCreateWithFlags(&c->ev_etd, cudaEventDisableTiming)) != cudaSuccess) return bail(e, "cudaEventCreate");
  const size_t vbytes = 3 * c->cs * c->esz;
  if ((e = cudaMalloc(&c->u, vbytes)) != cudaSuccess) return bail(e, "cudaMalloc(u)");
  if ((e = cudaMalloc(&c->temp, vbytes)) != cudaSuccess) return bail(e, "cudaMalloc(temp)");
  if ((e = cudaMalloc(&c->n1, vbytes)) != cudaSuccess) return bail(e, "cudaMalloc(n1)");
  if ((e = cudaMalloc(&c->acc, vbytes)) != cudaSuccess) return bail(e, "cudaMalloc(acc)");
  size_t a_elems = std::max(5 * M * N * H, 3 * M * M * H);
  size_t b_elems = std::max(6 * M * M * H, 3 * M * N * H);
  c->bufA_bytes = std::max(a_elems * c->esz, c->cs * sizeof(double2));  // also host-precision staging
  c->bufB_bytes = b_elems * c->esz;
  if ((e = cudaMalloc(&c->bufA, c->bufA_bytes)) != cudaSuccess) return bail(e, "cudaMalloc(bufA)");
  if ((e = cudaMalloc(&c->bufB, c->bufB_bytes)) != cudaSuccess) return bail(e, "cudaMalloc(bufB)");
  if ((e = upload_twiddles(n, c->fp32, &c->twN)) != cudaSuccess) return bail(e, "twiddles(N)");
  if ((e = upload_twiddles(c->M, c->fp32, &c->twM)) != cudaSuccess) return bail(e, "twiddles(M)");
  const int half = n / 2;
  c->n_etd = 3 * half * half + 1;
  if ((e = cudaMalloc(&c->etd, (size_t)c->n_etd * vk::ETD_STRIDE * sizeof(double))) != cudaSuccess)
    return bail(e, "cudaMalloc(etd)");
  if ((e = cudaMalloc(&c->dsc, sizeof(vk::DevScalars))) != cudaSuccess) return bail(e, "cudaMalloc(scalars)");
  if ((e = cudaMemset(c->dsc, 0, sizeof(vk::DevScalars))) != cudaSuccess) return bail(e, "cudaMemset(scalars)");
  // spectrum shells: ceil(sqrt(3 (N/2)^2)) + 1 (spectrum.rs:22-26)
  const double kmx = (double)(n / 2);
  c->n_shells = (int)std::ceil(std::sqrt(kmx * kmx + kmx * kmx + kmx * kmx)) + 1;
  c->red_blocks = 8 * c->dev_sms;   // reduction CTAs: 8 per SM keep the state read in flight
  const size_t width = std::max(4, c->n_shells);
  if ((e = cudaMalloc(&c->part, (size_t)c->red_blocks * width * sizeof(double))) != cudaSuccess)
    return bail(e, "cudaMalloc(partials)");
  if ((e = cudaMalloc(&c->dspec, width * sizeof(double))) != cudaSuccess) return bail(e, "cudaMalloc(spectrum)");
  c->dpart_rows = vk::p5_ctas(n, c->fp32);   // rows of k_p5 at this grid
  if ((e = cudaMalloc(&c->dpart, (size_t)c->dpart_rows * (4 + c->n_shells) * sizeof(double))) != cudaSuccess)
    return bail(e, "cudaMalloc(fused diagnostics)");
  *out = c;
  return VK_OK;
}

int vk_destroy(vk_ctx* ctx) {
  if (!ctx) return VK_OK;
  DeviceGuard g(ctx->cfg.device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  free_ctx(ctx);
  delete ctx;
  return VK_OK;
}

int64_t vk_spectral_len(const vk_ctx* ctx) { return ctx ? (int64_t)ctx->cs : -1; }

static int init_after_upload(vk_ctx* c, bool restore, double time, uint64_t step, double dt) {
  vk::DevScalars h;
  std::memset(&h, 0, sizeof(h));
  h.time = restore ? time : 0.0;
  h.dt = restore ? dt : (c->cfg.dt_mode == VK_DT_FIXED ? c->cfg.dt_fixed : 0.0);
  VK_CHECK(c, cudaMemcpyAsync(c->dsc, &h, sizeof(h), cudaMemcpyHostToDevice, c->stream));
  c->umax_fresh = false;
  c->diag_valid = 0;
  if (!restore && c->cfg.dt_mode == VK_DT_CFL) {
    VK_CHECK(c, ngrid(c, 1));
    VK_CHECK(c, vk::launch_cfl_update(c->dsc, dx_of(c), c->cfg.nu, c->cfg.cfl_safety, 1, c->stream));
  }
  VK_CHECK(c, etd_table(c, 1));
  VK_CHECK(c, cudaStreamSynchronize(c->stream));
  c->step_count = restore ? step : 0;
  c->has_state = true;
  return VK_OK;
}

int vk_set_state_host(vk_ctx* c, const double* ux, const double* uy, const double* uz) {
  if (!c) return VK_ERR_INVALID;
  DeviceGuard g(c->cfg.device);
  int r = upload_state(c, c->u, ux, uy, uz);
  if (r != VK_OK) return r;
  return init_after_upload(c, false, 0.0, 0, 0.0);
}

int vk_restore_host(vk_ctx* c, const double* ux, const double* uy, const double* uz, double time,
                    uint64_t step_count, double dt) {
  if (!c) return VK_ERR_INVALID;
  if (!(dt > 0.0)) return fail(c, VK_ERR_INVALID, "dt must be > 0");
  DeviceGuard g(c->cfg.device);
  int r = upload_state(c, c->u, ux, uy, uz);
  if (r != VK_OK) return r;
  return init_after_upload(c, true, time, step_count, dt);
}

int vk_get_state_host(vk_ctx* c, double* ux, double* uy, double* uz) {
  if (!c) return VK_ERR_INVALID;
  if (!c->has_state) return fail(c, VK_ERR_STATE, "no state set");
  DeviceGuard g(c->cfg.device);
  return download_state(c, c->u, ux, uy, uz);
}

int vk_step(vk_ctx* c, int64_t nsteps) {
  if (!c) return VK_ERR_INVALID;
  if (!c->has_state) return fail(c, VK_ERR_STATE, "vk_step before vk_set_state_host");
  if (nsteps < 0) return fail(c, VK_ERR_INVALID, "nsteps < 0");
  DeviceGuard g(c->cfg.device);
  for (int64_t i = 0; i < nsteps; ++i) VK_CHECK(c, step_once(c));
  return VK_OK;
}

int vk_time(vk_ctx* c, double* out) {
  if (!c || !out) return VK_ERR_INVALID;
  DeviceGuard g(c->cfg.device);
  vk::DevScalars h;
  int r = read_scalars(c, &h);
  if (r == VK_OK) *out = h.time;
  return r;
}

int vk_dt(vk_ctx* c, double* out) {
  if (!c || !out) return VK_ERR_INVALID;
  DeviceGuard g(c->cfg.device);
  vk::DevScalars h;
  int r = read_scalars(c, &h);
  if (r == VK_OK) *out = h.dt;
  return r;
}

int vk_step_count(vk_ctx* c, uint64_t* out) {
  if (!c || !out) return VK_ERR_INVALID;
  *out = c->step_count;
  return VK_OK;
}

int vk_cfl_dt(vk_ctx* c, double* out) {
  if (!c || !out) return VK_ERR_INVALID;
  if (!c->has_state) return fail(c, VK_ERR_STATE, "no state set");
  DeviceGuard g(c->cfg.device);
  if (!c->umax_fresh) VK_CHECK(c, ngrid(c, 1));
  VK_CHECK(c, vk::launch_cfl_update(c->dsc, dx_of(c), c->cfg.nu, c->cfg.cfl_safety, 2, c->stream));
  vk::DevScalars h;
  int r = read_scalars(c, &h);
  if (r == VK_OK) *out = h.cfl_dt;
  return r;
}

int vk_tier1(vk_ctx* c, vk_tier1_out* out) {
  if (!c || !out) return VK_ERR_INVALID;
  if (!c->has_state) return fail(c, VK_ERR_STATE, "no state set");
  DeviceGuard g(c->cfg.device);
  VK_CHECK(c, tier1_enqueue(c));
  vk::DevScalars h;
  int r = read_scalars(c, &h);
  if (r != VK_OK) return r;
  fill_tier1(c, h, c->step_count, out);
  return VK_OK;
}

#define VK_TIER1_FIELD(name, field)                    \
  int name(vk_ctx* c, double* out) {                   \
    if (!out) return VK_ERR_INVALID;                   \
    vk_tier1_out t;                                      \
    int r = vk_tier1(c, &t);                           \
    if (r == VK_OK) *out = t.field;                    \
    return r;                                          \
  }
VK_TIER1_FIELD(vk_energy, energy)
VK_TIER1_FIELD(vk_enstrophy, enstrophy)
VK_TIER1_FIELD(vk_helicity, helicity)
VK_TIER1_FIELD(vk_superhelicity, superhelicity)
VK_TIER1_FIELD(vk_max_vorticity, max_vorticity)
#undef VK_TIER1_FIELD

int vk_run(vk_ctx* c, int64_t nsteps, int64_t every, vk_tier1_out* out, int64_t max_records, int64_t* n_records) {
  if (!c) return VK_ERR_INVALID;
  if (!c->has_state) return fail(c, VK_ERR_STATE, "vk_run before vk_set_state_host");
  if (nsteps < 0 || every < 0 || max_records < 0) return fail(c, VK_ERR_INVALID, "negative argument");
  if (every > 0 && (!out || !n_records)) return fail(c, VK_ERR_INVALID, "null record output");
  DeviceGuard g(c->cfg.device);
  const int64_t want = every > 0 ? std::min<int64_t>(nsteps / every, max_records) : 0;
  if (want > c->records_cap) {
    if (c->records) cudaFree(c->records);
    c->records = nullptr;
    c->records_cap = 0;
    VK_CHECK(c, cudaMalloc(&c->records, (size_t)want * sizeof(vk::DevScalars)));
    c->records_cap = want;
  }
  std::vector<uint64_t> steps;
  int64_t nrec = 0;
  for (int64_t i = 1; i <= nsteps; ++i) {
    const bool record = every > 0 && i % every == 0 && nrec < want;
    VK_CHECK(c, step_once(c, record ? vk::DIAG_TIER1 : 0));   // Tier-1 sums fused into the final stage
    if (record) {
      VK_CHECK(c, tier1_enqueue(c));
      VK_CHECK(c, cudaMemcpyAsync(c->records + nrec, c->dsc, sizeof(vk::DevScalars), cudaMemcpyDeviceToDevice,
                                  c->stream));
      steps.push_back(c->step_count);
      ++nrec;
    }
  }
  std::vector<vk::DevScalars> h((size_t)nrec);
  if (nrec > 0)
    VK_CHECK(c, cudaMemcpyAsync(h.data(), c->records, (size_t)nrec * sizeof(vk::DevScalars), cudaMemcpyDeviceToHost,
                                c->stream));
  vk::DevScalars last;
  const int r = read_scalars(c, &last);   // synchronises; NaN / Inf -> VK_ERR_NONFINITE
  for (int64_t k = 0; k < nrec; ++k) fill_tier1(c, h[(size_t)k], steps[(size_t)k], out + k);
  if (n_records) *n_records = nrec;
  return r;
}

int vk_use_graphs(vk_ctx* c, int32_t enable) {
  if (!c) return VK_ERR_INVALID;
  DeviceGuard g(c->cfg.device);
  VK_CHECK(c, cudaStreamSynchronize(c->stream));
  c->use_graphs = enable != 0;
  if (!c->use_graphs) free_graphs(c);
  return VK_OK;
}

int vk_set_fused_diagnostics(vk_ctx* c, int64_t tier1_every, int64_t spectrum_every) {
  if (!c) return VK_ERR_INVALID;
  if (tier1_every < 0 || spectrum_every < 0) return fail(c, VK_ERR_INVALID, "negative cadence");
  c->fuse_t1_every = tier1_every;
  c->fuse_spec_every = spectrum_every;
  return VK_OK;
}

int vk_spectrum_len(const vk_ctx* c, int32_t* n) {
  if (!c || !n) return VK_ERR_INVALID;
  *n = c->n_shells;
  return VK_OK;
}

int vk_spectrum(vk_ctx* c, double* shells, double* spectrum, int32_t n) {
  if (!c || !spectrum) return VK_ERR_INVALID;
  if (!c->has_state) return fail(c, VK_ERR_STATE, "no state set");
  if (n < c->n_shells) return fail(c, VK_ERR_INVALID, "spectrum buffer too short");
  DeviceGuard g(c->cfg.device);
  const int nsh = c->n_shells;
  vk::TimerScope ts(c->prof, vk::PASS_SPECTRUM, c->stream);
  if (c->diag_valid & vk::DIAG_SPECTRUM) {
    // histogram rows accumulated by the final stage of the step that made the state
    VK_CHECK(c, vk::launch_reduce_columns(c->dpart + 4, c->dpart_rows, nsh, c->dspec, c->stream, 1.0, 4 + nsh));
  } else {
    cudaError_t e = c->fp32
        ? vk::Engine<float>::spectrum_partial((const float2*)c->u, c->cs, c->N, c->ks, nsh, c->part,
                                              c->red_blocks, c->stream)
        : vk::Engine<double>::spectrum_partial((const double2*)c->u, c->cs, c->N, c->ks, nsh, c->part,
                                               c->red_blocks, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "spectrum_partial");
    VK_CHECK(c, vk::launch_reduce_columns(c->part, c->red_blocks, nsh, c->dspec, c->stream));
  }
  std::vector<double> h(nsh);
  VK_CHECK(c, cudaMemcpyAsync(h.data(), c->dspec, nsh * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  VK_CHECK(c, cudaStreamSynchronize(c->stream));
  const double ntot = (double)c->N * (double)c->N * (double)c->N;
  for (int i = 0; i < nsh; ++i) {
    spectrum[i] = 0.5 * h[i] / (ntot * ntot);
    if (shells) shells[i] = (double)i;
  }
  return VK_OK;
}

int vk_nonlinear_host(vk_ctx* c, const double* ux, const double* uy, const double* uz, double* ox, double* oy,
                      double* oz) {
  if (!c) return VK_ERR_INVALID;
  DeviceGuard g(c->cfg.device);
  // temp holds the input, n1 receives the output: the solver state u is untouched.
  int r = upload_state(c, c->temp, ux, uy, uz);
  if (r != VK_OK) return r;
  VK_CHECK(c, nle(c, c->temp, vk::ST_NL_OUT, c->n1));
  return download_state(c, c->n1, ox, oy, oz);
}

int vk_apply_viscous_host(vk_ctx* c, double nu, const double* ux, const double* uy, const double* uz, double* ox,
                          double* oy, double* oz) {
  if (!c) return VK_ERR_INVALID;
  if (!std::isfinite(nu)) return fail(c, VK_ERR_INVALID, "nu must be finite");
  DeviceGuard g(c->cfg.device);
  // temp holds the input, n1 receives the output: the solver state u is untouched.
  int r = upload_state(c, c->temp, ux, uy, uz);
  if (r != VK_OK) return r;
  VK_CHECK(c, vk::launch_apply_viscous(c->n1, c->temp, c->fp32 ? 1 : 0, c->N, c->cs, c->ks, nu, c->stream));
  return download_state(c, c->n1, ox, oy, oz);
}

int vk_wavenumbers(vk_ctx* c, double* kx, double* ky, double* kz, double* k_mag_sq) {
  if (!c || !kx || !ky || !kz) return VK_ERR_INVALID;
  // rfftfreq_full / rfftfreq_half (spectral_ops.rs:51-74): index * (2 pi / L),
  // index n/2 .. n-1 of the full axes mapped to -n/2 .. -1
  const int n = c->N;
  for (int i = 0; i < n; ++i) {
    const double k = (double)(i < n / 2 ? i : i - n) * c->ks;
    kx[i] = k;
    ky[i] = k;
  }
  for (int i = 0; i < c->H; ++i) kz[i] = (double)i * c->ks;
  if (!k_mag_sq) return VK_OK;
  DeviceGuard g(c->cfg.device);
  // |k|^2 per mode on the device (bufA holds cs doubles at least), read back
  VK_CHECK(c, vk::launch_k_mag_sq((double*)c->bufA, n, c->ks, c->stream));
  VK_CHECK(c, cudaMemcpyAsync(k_mag_sq, c->bufA, c->cs * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  VK_CHECK(c, cudaStreamSynchronize(c->stream));
  return VK_OK;
}

}  // extern "C"

namespace {

size_t state_bytes(const vk_ctx* c) { return 3 * c->cs * c->esz; }

cudaError_t adj_alloc(vk_ctx* c, int64_t nseg, int64_t K) {
  auto& a = c->adj;
  const size_t sb = state_bytes(c);
  cudaError_t e;
  if ((int64_t)a.ckpt.size() != nseg || (int64_t)a.seg.size() != 4 * K + 1) {
    for (void* p : a.ckpt)
      if (p) cudaFree(p);
    for (void* p : a.seg)
      if (p) cudaFree(p);
    a.ckpt.assign((size_t)nseg, nullptr);
    a.seg.assign((size_t)(4 * K + 1), nullptr);
    for (auto& p : a.ckpt)
      if ((e = cudaMalloc(&p, sb)) != cudaSuccess) return e;
    for (auto& p : a.seg)
      if ((e = cudaMalloc(&p, sb)) != cudaSuccess) return e;
  }
  void** st[] = {&a.ub, &a.acc, &a.nb, &a.n1b};
  for (void** p : st)
    if (!*p && (e = cudaMalloc(p, sb)) != cudaSuccess) return e;
  const size_t N = c->N, H = c->H, M = c->M;
  const size_t ab = std::max(8 * M * N * H, 6 * M * M * H) * c->esz;
  const size_t bb = std::max(9 * M * M * H, 6 * M * N * H) * c->esz;
  if (!a.bufA && (e = cudaMalloc(&a.bufA, ab)) != cudaSuccess) return e;
  if (!a.bufB && (e = cudaMalloc(&a.bufB, bb)) != cudaSuccess) return e;
  a.bufA_bytes = ab;
  a.bufB_bytes = bb;
  a.K = K;
  a.nseg = nseg;
  return cudaSuccess;
}

// One forward stage NLE with explicit state pointers (recompute of a, b, c).
template <typename R>
cudaError_t nle_stage_t(vk_ctx* c, const void* in, int op, void* u, void* temp, void* u_out) {
  vk::NleParams<R> p{};
  p.N = c->N;
  p.ks = c->ks;
  p.in = (const C2<R>*)in;
  p.cs = c->cs;
  p.bufA = (C2<R>*)c->bufA;
  p.bufB = (C2<R>*)c->bufB;
  p.twM = (const C2<R>*)c->twM;
  p.st = stage_args<R>(c, op, nullptr);
  p.st.u = (C2<R>*)u;
  p.st.temp = (C2<R>*)temp;
  p.st.u_out = (C2<R>*)u_out;
  p.timer = c->prof;
  p.async_err = &c->dsc->async_timeout;
  return vk::Engine<R>::nle(p, c->stream);
}

cudaError_t nle_stage(vk_ctx* c, const void* in, int op, void* u, void* temp, void* u_out) {
  return c->fp32 ? nle_stage_t<float>(c, in, op, u, temp, u_out) : nle_stage_t<double>(c, in, op, u, temp, u_out);
}

template <typename R>
cudaError_t nla_t(vk_ctx* c, const void* x, const void* nbsrc, int slot, int op, void* out) {
  auto& a = c->adj;
  vk::NlaParams<R> p{};
  p.N = c->N;
  p.ks = c->ks;
  p.x = (const C2<R>*)x;
  p.cs = c->cs;
  p.nb = (const C2<R>*)nbsrc;
  p.etd = c->etd;
  p.slot = slot;
  p.fac = 1.0;
  p.dt = &c->dsc->dt;
  p.bufA = (C2<R>*)a.bufA;
  p.bufB = (C2<R>*)a.bufB;
  p.twM = (const C2<R>*)c->twM;
  p.st.op = op;
  p.st.cs = c->cs;
  p.st.ub = (C2<R>*)a.ub;
  p.st.acc = (C2<R>*)a.acc;
  p.st.nb = (C2<R>*)a.nb;
  p.st.n1b = (C2<R>*)a.n1b;
  p.st.out = (C2<R>*)out;
  p.st.etd = c->etd;
  p.st.dt = &c->dsc->dt;
  p.timer = c->prof;
  return vk::Engine<R>::nle_adjoint(p, c->stream);
}

cudaError_t nla(vk_ctx* c, const void* x, const void* nbsrc, int slot, int op, void* out = nullptr) {
  return c->fp32 ? nla_t<float>(c, x, nbsrc, slot, op, out) : nla_t<double>(c, x, nbsrc, slot, op, out);
}

cudaError_t adj_mode(vk_ctx* c, const void* in, void* out, int mode) {
  return c->fp32 ? vk::Engine<float>::adj_mode(c->N, c->ks, c->cs, (const float2*)in, (float2*)out, mode, c->stream)
                 : vk::Engine<double>::adj_mode(c->N, c->ks, c->cs, (const double2*)in, (double2*)out, mode,
                                                c->stream);
}

cudaError_t herm_avg(vk_ctx* c, const void* in, void* out) {
  return c->fp32 ? vk::Engine<float>::hermitian_avg(c->N, c->cs, (const float2*)in, (float2*)out, c->stream)
                 : vk::Engine<double>::hermitian_avg(c->N, c->cs, (const double2*)in, (double2*)out, c->stream);
}

// Adjoint of one reference-variant ETD-RK4 step (solver.rs:221-379 transposed)
// taken from S with stage inputs A = a, B = b, C = c; ub is updated in place.
cudaError_t adjoint_step(vk_ctx* c, void* S, void* A, void* B, void* C) {
  auto& a = c->adj;
  cudaError_t e;
  if ((e = nla(c, C, a.ub, vk::E_B4, vk::ADJ_C)) != cudaSuccess) return e;
  if ((e = nla(c, B, a.nb, -1, vk::ADJ_B)) != cudaSuccess) return e;
  if ((e = nla(c, A, a.nb, -1, vk::ADJ_A)) != cudaSuccess) return e;
  return nla(c, S, a.n1b, -1, vk::ADJ_U);
}

// Forward step from S storing the stage inputs A, B, C and the next state in Snext.
cudaError_t forward_step_store(vk_ctx* c, void* S, void* A, void* B, void* C, void* Snext) {
  cudaError_t e;
  if ((e = nle_stage(c, S, vk::ST_ETD_REF_1, S, A, S)) != cudaSuccess) return e;
  if ((e = nle_stage(c, A, vk::ST_ETD_REF_2, S, B, S)) != cudaSuccess) return e;
  if ((e = nle_stage(c, B, vk::ST_ETD_REF_3, S, C, S)) != cudaSuccess) return e;
  if (!Snext) return cudaSuccess;
  return nle_stage(c, C, vk::ST_ETD_4, S, C, Snext);
}

// Device executor of the binomial schedule (vk_schedule.h): states live in
// the checkpoint slots or the working buffer; advancing runs full steps in
// place (the last stage's epilogue reads and writes u mode by mode).
// Each slot's step index is tracked (c->adj.pos, -1 = none; the working
// buffer separately), so that a state the forward run already stored where
// the schedule wants it is not recomputed.
struct AdjBinomialEx {
  vk_ctx* c;
  void* work;
  void* A;
  void* B;
  void* C;
  size_t sb;
  int64_t work_pos = -1;
  cudaError_t err = cudaSuccess;
  void* buf(int s) const { return s < 0 ? work : c->adj.ckpt[(size_t)s]; }
  int64_t& pos(int s) { return s < 0 ? work_pos : c->adj.pos[(size_t)s]; }
  bool ok() const { return err == cudaSuccess; }
  void place(int d, int s, int64_t n) {
    const int64_t target = pos(s) + n;
    if (d == s && n == 0) return;
    if (pos(d) == target && pos(s) >= 0) return;
    if (ok() && d != s) err = cudaMemcpyAsync(buf(d), buf(s), sb, cudaMemcpyDeviceToDevice, c->stream);
    for (int64_t i = 0; i < n && ok(); ++i) err = forward_step_store(c, buf(d), A, B, C, buf(d));
    pos(d) = ok() ? target : -1;
  }
  void reverse_step(int s) {
    if (ok()) err = forward_step_store(c, buf(s), A, B, C, nullptr);
    if (ok()) err = adjoint_step(c, buf(s), A, B, C);
  }
};

int adj_supported(vk_ctx* c) {
  if (!c->has_state) return fail(c, VK_ERR_STATE, "no state set");
  if (c->cfg.dt_mode != VK_DT_FIXED)
    return fail(c, VK_ERR_UNSUPPORTED, "the adjoint needs dt_mode = fixed (the CFL dt is not differentiable)");
  if (c->cfg.integrator != VK_INTEGRATOR_ETD_RK4 || c->cfg.etd_variant != VK_ETD_REFERENCE)
    return fail(c, VK_ERR_UNSUPPORTED, "the adjoint is built for the reference ETD-RK4 variant");
  return VK_OK;
}

}  // namespace

extern "C" {

int vk_adjoint_set_schedule(vk_ctx* c, int32_t schedule) {
  if (!c) return VK_ERR_INVALID;
  if (schedule != VK_ADJ_TWO_LEVEL && schedule != VK_ADJ_BINOMIAL)
    return fail(c, VK_ERR_INVALID, "schedule must be VK_ADJ_TWO_LEVEL or VK_ADJ_BINOMIAL");
  c->adj.schedule = schedule;
  return VK_OK;
}

int vk_adjoint_forward(vk_ctx* c, int64_t nsteps, int32_t nsnap, double* J) {
  if (!c || !J) return VK_ERR_INVALID;
  int r = adj_supported(c);
  if (r != VK_OK) return r;
  if (nsteps < 1 || nsnap < 1) return fail(c, VK_ERR_INVALID, "nsteps >= 1 and nsnap >= 1 required");
  DeviceGuard g(c->cfg.device);
  const bool binomial = c->adj.schedule == VK_ADJ_BINOMIAL;
  // binomial: nsnap slots plus the working state and one step's stage inputs
  const int64_t K = binomial ? 1 : (nsteps + nsnap - 1) / nsnap;
  const int64_t nseg = binomial ? nsnap : (nsteps + K - 1) / K;
  cudaError_t e = adj_alloc(c, nseg, K);
  if (e != cudaSuccess) {
    free_adjoint(c);
    return cuda_fail(c, e, "adjoint buffers");
  }
  auto& a = c->adj;
  a.nsteps = nsteps;
  a.ready = false;
  a.used = binomial ? VK_ADJ_BINOMIAL : VK_ADJ_TWO_LEVEL;
  const size_t sb = state_bytes(c);
  if (binomial) {
    // slot 0 holds the initial state; the states of the reversal's first
    // descent are stored as the run passes them
    const auto spine = vk::treeverse_spine(nsteps, nsnap);
    a.pos.assign((size_t)nsnap, -1);
    VK_CHECK(c, cudaMemcpyAsync(a.ckpt[0], c->u, sb, cudaMemcpyDeviceToDevice, c->stream));
    a.pos[0] = 0;
    size_t next = 0;
    for (int64_t j = 0; j < nsteps; ++j) {
      if (next < spine.size() && spine[next].second == j) {
        const int slot = spine[next].first;
        VK_CHECK(c, cudaMemcpyAsync(a.ckpt[(size_t)slot], c->u, sb, cudaMemcpyDeviceToDevice, c->stream));
        a.pos[(size_t)slot] = j;
        ++next;
      }
      VK_CHECK(c, step_once(c));
    }
  } else {
    for (int64_t s = 0; s < nseg; ++s) {
      VK_CHECK(c, cudaMemcpyAsync(a.ckpt[(size_t)s], c->u, sb, cudaMemcpyDeviceToDevice, c->stream));
      const int64_t ks = std::min<int64_t>(K, nsteps - s * K);
      for (int64_t j = 0; j < ks; ++j) VK_CHECK(c, step_once(c));
    }
  }
  // J = enstrophy of the final state and its raw-Euclidean cotangent
  VK_CHECK(c, tier1_enqueue(c));
  VK_CHECK(c, adj_mode(c, c->u, a.ub, 0));
  vk::DevScalars h;
  int rr = read_scalars(c, &h);
  if (rr != VK_OK) return rr;
  const double ntot = (double)c->N * (double)c->N * (double)c->N;
  a.J = h.sums[1] / (ntot * ntot);
  a.ready = true;
  *J = a.J;
  return VK_OK;
}

int vk_adjoint_backward(vk_ctx* c, double* gx, double* gy, double* gz) {
  if (!c || !gx || !gy || !gz) return VK_ERR_INVALID;
  if (!c->adj.ready) return fail(c, VK_ERR_STATE, "vk_adjoint_backward needs a preceding vk_adjoint_forward");
  DeviceGuard g(c->cfg.device);
  auto& a = c->adj;
  const int64_t K = a.K;
  void** S = a.seg.data();
  void** A = S + (K + 1);
  void** B = A + K;
  void** C = B + K;
  const size_t sb = state_bytes(c);
  if (a.used == VK_ADJ_BINOMIAL) {
    // slots: the checkpoints (slot 0 = initial state), -1 = S[0]; one step's
    // stage inputs in A[0], B[0], C[0]
    AdjBinomialEx ex{c, S[0], A[0], B[0], C[0], sb};
    std::vector<int> free_slots;
    for (int k = (int)a.nseg - 1; k >= 1; --k) free_slots.push_back(k);
    vk::treeverse(ex, 0, a.nsteps, 0, free_slots);
    VK_CHECK(c, ex.err);
  } else {
    for (int64_t s = a.nseg - 1; s >= 0; --s) {
      const int64_t ks = std::min<int64_t>(K, a.nsteps - s * K);
      VK_CHECK(c, cudaMemcpyAsync(S[0], a.ckpt[(size_t)s], sb, cudaMemcpyDeviceToDevice, c->stream));
      for (int64_t j = 0; j < ks; ++j)
        VK_CHECK(c, forward_step_store(c, S[j], A[j], B[j], C[j], j + 1 < ks ? S[j + 1] : nullptr));
      for (int64_t j = ks - 1; j >= 0; --j) VK_CHECK(c, adjoint_step(c, S[j], A[j], B[j], C[j]));
    }
  }
  // gradient in the L2 inner product of the physical fields, projected on
  // real, divergence-free, Nyquist-free fields
  VK_CHECK(c, adj_mode(c, a.ub, a.acc, 1));
  VK_CHECK(c, herm_avg(c, a.acc, a.nb));
  a.ready = false;
  return download_state(c, a.nb, gx, gy, gz);
}

int vk_nonlinear_adjoint_host(vk_ctx* c, const double* ux, const double* uy, const double* uz, const double* bx,
                              const double* by, const double* bz, double* ox, double* oy, double* oz) {
  if (!c) return VK_ERR_INVALID;
  DeviceGuard g(c->cfg.device);
  cudaError_t e = adj_alloc(c, std::max<int64_t>(c->adj.nseg, 1), std::max<int64_t>(c->adj.K, 1));
  if (e != cudaSuccess) return cuda_fail(c, e, "adjoint buffers");
  int r = upload_state(c, c->temp, ux, uy, uz);
  if (r != VK_OK) return r;
  r = upload_state(c, c->adj.nb, bx, by, bz);
  if (r != VK_OK) return r;
  VK_CHECK(c, nla(c, c->temp, c->adj.nb, -1, vk::ADJ_NL_OUT, c->n1));
  return download_state(c, c->n1, ox, oy, oz);
}

int vk_step_timed(vk_ctx* c, int64_t nsteps, double* elapsed_ms) {
  if (!c || !elapsed_ms) return VK_ERR_INVALID;
  if (!c->has_state) return fail(c, VK_ERR_STATE, "vk_step_timed before vk_set_state_host");
  if (nsteps < 0) return fail(c, VK_ERR_INVALID, "nsteps < 0");
  DeviceGuard g(c->cfg.device);
  for (cudaEvent_t& e : c->tev)
    if (!e) VK_CHECK(c, cudaEventCreate(&e));
  VK_CHECK(c, cudaEventRecord(c->tev[0], c->stream));
  for (int64_t i = 0; i < nsteps; ++i) VK_CHECK(c, step_once(c));
  VK_CHECK(c, cudaEventRecord(c->tev[1], c->stream));
  VK_CHECK(c, cudaEventSynchronize(c->tev[1]));
  float ms = 0.f;
  VK_CHECK(c, cudaEventElapsedTime(&ms, c->tev[0], c->tev[1]));
  *elapsed_ms = ms;
  vk::DevScalars h;
  return read_scalars(c, &h);
}

int vk_profile_enable(vk_ctx* c, int32_t enable) {
  if (!c) return VK_ERR_INVALID;
  DeviceGuard g(c->cfg.device);
  VK_CHECK(c, cudaStreamSynchronize(c->stream));
  if (enable) {
    if (!c->prof) c->prof = new EventTimer();
    c->prof->reset();
  } else {
    delete c->prof;
    c->prof = nullptr;
  }
  return VK_OK;
}

int vk_profile_read(vk_ctx* c, double* ms, int64_t* launches, int32_t n) {
  if (!c || !ms || !launches) return VK_ERR_INVALID;
  if (!c->prof) return fail(c, VK_ERR_STATE, "profiling is not enabled");
  DeviceGuard g(c->cfg.device);
  VK_CHECK(c, cudaStreamSynchronize(c->stream));
  c->prof->collect();
  for (int i = 0; i < n; ++i) {
    ms[i] = i < vk::PASS_COUNT ? c->prof->ms[i] : 0.0;
    launches[i] = i < vk::PASS_COUNT ? c->prof->cnt[i] : 0;
  }
  return VK_OK;
}

const char* vk_profile_pass_name(int32_t id) {
  static const char* names[vk::PASS_COUNT] = {
      "P1_x_inverse_pad_curl", "P2_y_inverse_pad_omega", "P3_z_c2r_cross_r2c", "P4_y_forward_trunc",
      "P5_x_forward_trunc_leray_stage", "NX_ngrid_x_inverse", "NY_ngrid_y_inverse", "NZ_ngrid_z_c2r_max",
      "ETD_table", "small_scalar_kernels", "tier1_sums", "spectrum", "fft_z", "fft_y", "fft_x",
      "A1_adj_x_inverse", "A2_adj_y_inverse", "A3_adj_z_cross", "A4_adj_y_forward", "A5_adj_x_forward_stage"};
  return id >= 0 && id < vk::PASS_COUNT ? names[id] : "";
}

int vk_probe_fma_peak(int32_t device, int32_t fp64, double* gflops) {
  if (!gflops) return VK_ERR_INVALID;
  DeviceGuard g(device);
  if (!g.ok) return VK_ERR_CUDA;
  return vk::probe_fma_peak(fp64, gflops) == cudaSuccess ? VK_OK : VK_ERR_CUDA;
}

int vk_event_mark(vk_ctx* c, int32_t slot) {
  if (!c || slot < 0 || slot >= 8) return VK_ERR_INVALID;
  DeviceGuard g(c->cfg.device);
  if (!c->marks[slot]) VK_CHECK(c, cudaEventCreate(&c->marks[slot]));
  VK_CHECK(c, cudaEventRecord(c->marks[slot], c->stream));
  return VK_OK;
}

int vk_event_elapsed(vk_ctx* c, int32_t a, int32_t b, double* ms) {
  if (!c || !ms || a < 0 || a >= 8 || b < 0 || b >= 8) return VK_ERR_INVALID;
  if (!c->marks[a] || !c->marks[b]) return fail(c, VK_ERR_STATE, "event slot not recorded");
  DeviceGuard g(c->cfg.device);
  VK_CHECK(c, cudaEventSynchronize(c->marks[b]));
  float t = 0.f;
  VK_CHECK(c, cudaEventElapsedTime(&t, c->marks[a], c->marks[b]));
  *ms = t;
  return VK_OK;
}

int vk_pinned_alloc(size_t bytes, void** out) {
  if (!out) return VK_ERR_INVALID;
  *out = nullptr;
  return cudaMallocHost(out, bytes) == cudaSuccess ? VK_OK : VK_ERR_OOM;
}

int vk_pinned_free(void* p) {
  if (!p) return VK_OK;
  return cudaFreeHost(p) == cudaSuccess ? VK_OK : VK_ERR_CUDA;
}

int vk_stream(vk_ctx* c, void** stream) {
  if (!c || !stream) return VK_ERR_INVALID;
  *stream = (void*)c->stream;
  return VK_OK;
}

// ============================================================================
// FFT backend
static int fft_fail(vk_fft* p, cudaError_t e, const char* where) {
  p->err = std::string(where) + ": " + cudaGetErrorString(e);
  return e == cudaErrorMemoryAllocation ? VK_ERR_OOM : VK_ERR_CUDA;
}

int vk_fft_create(int32_t nx, int32_t ny, int32_t nz, int32_t precision, int32_t device, vk_fft** out) {
  if (!out) { g_create_error = "null argument"; return VK_ERR_INVALID; }
  *out = nullptr;
  if (!fft_len_ok(nx) || !fft_len_ok(ny) || !fft_len_ok(nz)) {
    g_create_error = "each of nx, ny, nz must be in {8..512 powers of 2} or {12..768 = 3*2^k}";
    return VK_ERR_UNSUPPORTED;
  }
  if (precision != VK_PRECISION_FP64 && precision != VK_PRECISION_FP32BULK) { g_create_error = "bad precision"; return VK_ERR_INVALID; }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) { g_create_error = "no CUDA device available"; return VK_ERR_CUDA; }
  if (device < 0 || device >= ndev) { g_create_error = "device ordinal out of range"; return VK_ERR_INVALID; }
  DeviceGuard g(device);
  vk_fft* p = new vk_fft();
  p->nx = nx; p->ny = ny; p->nz = nz; p->hz = nz / 2 + 1;
  p->fp32 = precision == VK_PRECISION_FP32BULK;
  p->device = device;
  const size_t nreal = (size_t)nx * ny * nz, ncplx = (size_t)nx * ny * p->hz;
  const size_t rs = p->fp32 ? sizeof(float) : sizeof(double);
  cudaError_t e = cudaSuccess;
  auto bail = [&](const char* what) {
    g_create_error = std::string(what) + ": " + cudaGetErrorString(e);
    void* ptrs[] = {p->real, p->cplx, p->stage, p->twx, p->twy, p->twz};
    for (void* q : ptrs) if (q) cudaFree(q);
    if (p->stream) cudaStreamDestroy(p->stream);
    delete p;
    return e == cudaErrorMemoryAllocation ? VK_ERR_OOM : VK_ERR_CUDA;
  };
  if ((e = cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking)) != cudaSuccess) return bail("cudaStreamCreate");
  if ((e = cudaMalloc(&p->real, nreal * rs)) != cudaSuccess) return bail("cudaMalloc(real)");
  if ((e = cudaMalloc(&p->cplx, ncplx * 2 * rs)) != cudaSuccess) return bail("cudaMalloc(complex)");
  if (p->fp32 && (e = cudaMalloc(&p->stage, std::max(nreal, 2 * ncplx) * sizeof(double))) != cudaSuccess)
    return bail("cudaMalloc(stage)");
  if ((e = upload_twiddles(nx, p->fp32, &p->twx)) != cudaSuccess) return bail("twiddles");
  if ((e = upload_twiddles(ny, p->fp32, &p->twy)) != cudaSuccess) return bail("twiddles");
  if ((e = upload_twiddles(nz, p->fp32, &p->twz)) != cudaSuccess) return bail("twiddles");
  *out = p;
  return VK_OK;
}

int vk_fft_destroy(vk_fft* p) {
  if (!p) return VK_OK;
  DeviceGuard g(p->device);
  if (p->stream) cudaStreamSynchronize(p->stream);
  void* ptrs[] = {p->real, p->cplx, p->stage, p->twx, p->twy, p->twz};
  for (void* q : ptrs) if (q) cudaFree(q);
  if (p->stream) cudaStreamDestroy(p->stream);
  delete p;
  return VK_OK;
}

const char* vk_fft_last_error(const vk_fft* p) { return p ? p->err.c_str() : g_create_error.c_str(); }

}  // extern "C"

template <typename R>
static cudaError_t fft_exec(vk_fft* p, bool forward, void* real, void* cplx, cudaStream_t s) {
  vk::FftParams<R> f{};
  f.nx = p->nx; f.ny = p->ny; f.nz = p->nz;
  f.real = (R*)real;
  f.cplx = (C2<R>*)cplx;
  f.twx = (const C2<R>*)p->twx;
  f.twy = (const C2<R>*)p->twy;
  f.twz = (const C2<R>*)p->twz;
  return forward ? vk::Engine<R>::fft_r2c(f, s) : vk::Engine<R>::fft_c2r(f, s);
}

static cudaError_t fft_run(vk_fft* p, bool forward, void* real, void* cplx, cudaStream_t s) {
  return p->fp32 ? fft_exec<float>(p, forward, real, cplx, s) : fft_exec<double>(p, forward, real, cplx, s);
}

extern "C" {

#define FFT_CHECK(p, call)                                   \
  do {                                                       \
    cudaError_t _e = (call);                                 \
    if (_e != cudaSuccess) return fft_fail((p), _e, #call);  \
  } while (0)

int vk_fft_r2c_host(vk_fft* p, const double* in, double* out) {
  if (!p || !in || !out) return VK_ERR_INVALID;
  DeviceGuard g(p->device);
  const size_t nreal = (size_t)p->nx * p->ny * p->nz, ncplx = (size_t)p->nx * p->ny * p->hz;
  if (!p->fp32) {
    FFT_CHECK(p, cudaMemcpyAsync(p->real, in, nreal * sizeof(double), cudaMemcpyHostToDevice, p->stream));
  } else {
    FFT_CHECK(p, cudaMemcpyAsync(p->stage, in, nreal * sizeof(double), cudaMemcpyHostToDevice, p->stream));
    FFT_CHECK(p, vk::launch_convert_r(p->real, 1, p->stage, 0, nreal, p->stream));
  }
  FFT_CHECK(p, fft_run(p, true, p->real, p->cplx, p->stream));
  if (!p->fp32) {
    FFT_CHECK(p, cudaMemcpyAsync(out, p->cplx, ncplx * sizeof(double2), cudaMemcpyDeviceToHost, p->stream));
  } else {
    FFT_CHECK(p, vk::launch_convert_c(p->stage, 0, p->cplx, 1, ncplx, p->stream));
    FFT_CHECK(p, cudaMemcpyAsync(out, p->stage, ncplx * sizeof(double2), cudaMemcpyDeviceToHost, p->stream));
  }
  FFT_CHECK(p, cudaStreamSynchronize(p->stream));
  return VK_OK;
}

int vk_fft_c2r_host(vk_fft* p, const double* in, double* out) {
  if (!p || !in || !out) return VK_ERR_INVALID;
  DeviceGuard g(p->device);
  const size_t nreal = (size_t)p->nx * p->ny * p->nz, ncplx = (size_t)p->nx * p->ny * p->hz;
  if (!p->fp32) {
    FFT_CHECK(p, cudaMemcpyAsync(p->cplx, in, ncplx * sizeof(double2), cudaMemcpyHostToDevice, p->stream));
  } else {
    FFT_CHECK(p, cudaMemcpyAsync(p->stage, in, ncplx * sizeof(double2), cudaMemcpyHostToDevice, p->stream));
    FFT_CHECK(p, vk::launch_convert_c(p->cplx, 1, p->stage, 0, ncplx, p->stream));
  }
  FFT_CHECK(p, fft_run(p, false, p->real, p->cplx, p->stream));
  if (!p->fp32) {
    FFT_CHECK(p, cudaMemcpyAsync(out, p->real, nreal * sizeof(double), cudaMemcpyDeviceToHost, p->stream));
  } else {
    FFT_CHECK(p, vk::launch_convert_r(p->stage, 0, p->real, 1, nreal, p->stream));
    FFT_CHECK(p, cudaMemcpyAsync(out, p->stage, nreal * sizeof(double), cudaMemcpyDeviceToHost, p->stream));
  }
  FFT_CHECK(p, cudaStreamSynchronize(p->stream));
  return VK_OK;
}

int vk_fft_r2c_device(vk_fft* p, const void* in, void* out, void* stream) {
  if (!p || !in || !out) return VK_ERR_INVALID;
  DeviceGuard g(p->device);
  cudaStream_t s = stream ? (cudaStream_t)stream : p->stream;
  FFT_CHECK(p, fft_run(p, true, const_cast<void*>(in), out, s));
  return VK_OK;
}

int vk_fft_c2r_device(vk_fft* p, void* in, void* out, void* stream) {
  if (!p || !in || !out) return VK_ERR_INVALID;
  DeviceGuard g(p->device);
  cudaStream_t s = stream ? (cudaStream_t)stream : p->stream;
  FFT_CHECK(p, fft_run(p, false, out, in, s));
  return VK_OK;
}

const char* vk_fft_name(const vk_fft* p) {
  if (!p) return "";
  return p->fp32 ? "vonkarman-gb300 pencil FFT (sm_103a, fp32)" : "vonkarman-gb300 pencil FFT (sm_103a, fp64)";
}

int vk_fft_precision_digits(const vk_fft* p) { return p && p->fp32 ? 6 : 15; }

}  // extern "C"
