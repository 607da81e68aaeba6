/*
 * vk_cpu.c -- C restatement of vonkarman's CPU path for the periodic step.
 *
 * TEST AND BENCHMARK INFRASTRUCTURE ONLY.  This is the reference's own CPU
 * algorithm restated in C (the Rust reference cannot be built here: no Rust
 * toolchain).  bench.py times it as the CPU baseline / reference arm; tests
 * check it against the numpy oracle.  The product never loads it.
 *
 * Fidelity to the reference's dataflow (same loops, same pass order, same
 * temporaries):
 *   FftBackend r2c_3d: z R2C -> y C2C -> x C2C, fresh temporaries per call
 *       (vonkarman-fft/src/ndrustfft_backend.rs:33-44)
 *   FftBackend c2r_3d: x iC2C (1/nx) -> y iC2C (1/ny) -> z C2R (1/nz)
 *       (ndrustfft_backend.rs:46-57); lanes are copied to contiguous scratch
 *       as ndrustfft does for every axis.
 *   dealiased_cross_product: 6 padded spectral arrays zero-filled, scaled and
 *       inverted, the M^3 cross loop, 3 padded forward transforms, truncation
 *       (vonkarman-fft/src/dealiased.rs:16-163)
 *   compute_nonlinear: curl, dealiased cross, Leray (nonlinear.rs:15-39,
 *       spectral_ops.rs:81-151)
 *   ETD-RK4 with per-mode EtdCoeffs (etd.rs:15-135, solver.rs:161-379) and the
 *       CFL / 1% re-tabulation rule of Domain::step (solver.rs:180-218, 383-400)
 * The 1-D transforms are an own mixed-radix (4/2/3) Stockham FFT with
 * precomputed twiddles; real transforms use the half-length complex trick
 * (the method of realfft, which ndrustfft calls).  OpenMP parallelises over
 * lanes and modes; with one thread it is the reference's serial schedule.
 * vkc_set_cufft(1) switches the 3-D transforms to the reference's cuFFT
 * backend pattern (per-call host <-> device copies around cuFFT, host-side
 * normalisation: vonkarman-fft/src/cufft.rs), the reference's GPU mode.
 */
#include <dlfcn.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct { double re, im; } cpx;

static inline cpx cadd(cpx a, cpx b) { cpx r = {a.re + b.re, a.im + b.im}; return r; }
static inline cpx csub(cpx a, cpx b) { cpx r = {a.re - b.re, a.im - b.im}; return r; }
static inline cpx cmul(cpx a, cpx b) { cpx r = {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; return r; }
static inline cpx cconj(cpx a) { cpx r = {a.re, -a.im}; return r; }

/* ------------------------------------------------------------------------- */
/* complex FFT, mixed radix Stockham                                          */
/* ------------------------------------------------------------------------- */
typedef struct {
  int n, nst;
  int rad[32];
  cpx* tw; /* exp(-2 pi i m / n), m < n */
} fft1d;

static void fft1d_init(fft1d* p, int n) {
  p->n = n;
  p->nst = 0;
  int m = n;
  while (m % 4 == 0) { p->rad[p->nst++] = 4; m /= 4; }
  while (m % 2 == 0) { p->rad[p->nst++] = 2; m /= 2; }
  while (m % 3 == 0) { p->rad[p->nst++] = 3; m /= 3; }
  p->tw = (cpx*)malloc(sizeof(cpx) * (size_t)n);
  const long double two_pi = 6.283185307179586476925286766559005768L;
  for (int k = 0; k < n; ++k) {
    long double a = two_pi * (long double)k / (long double)n;
    p->tw[k].re = (double)cosl(a);
    p->tw[k].im = (double)(-sinl(a));
  }
}

static void fft1d_free(fft1d* p) { free(p->tw); }

/* Unnormalised transform of x (length n) using scratch y; result in x. */
static void fft1d_exec(const fft1d* p, cpx* x, cpx* y, int inverse) {
  const int n = p->n;
  cpx* src = x;
  cpx* dst = y;
  int ns = 1;
  for (int s = 0; s < p->nst; ++s) {
    const int r = p->rad[s];
    const int nb = n / r;
    const int tws = n / (ns * r);
    for (int j = 0; j < nb; ++j) {
      const int k = j % ns;
      cpx v[4];
      for (int q = 0; q < r; ++q) {
        cpx a = src[j + q * nb];
        if (q > 0 && k > 0) {
          cpx w = p->tw[q * k * tws];
          if (inverse) w.im = -w.im;
          a = cmul(a, w);
        }
        v[q] = a;
      }
      cpx o[4];
      if (r == 2) {
        o[0] = cadd(v[0], v[1]);
        o[1] = csub(v[0], v[1]);
      } else if (r == 4) {
        cpx t0 = cadd(v[0], v[2]), t1 = csub(v[0], v[2]);
        cpx t2 = cadd(v[1], v[3]), t3 = csub(v[1], v[3]);
        cpx t3r = inverse ? (cpx){-t3.im, t3.re} : (cpx){t3.im, -t3.re};
        o[0] = cadd(t0, t2);
        o[2] = csub(t0, t2);
        o[1] = cadd(t1, t3r);
        o[3] = csub(t1, t3r);
      } else {
        const double c = 0.86602540378443864676;
        cpx t = cadd(v[1], v[2]), d = csub(v[1], v[2]);
        cpx m = {v[0].re - 0.5 * t.re, v[0].im - 0.5 * t.im};
        cpx e = inverse ? (cpx){-c * d.im, c * d.re} : (cpx){c * d.im, -c * d.re};
        o[0] = cadd(v[0], t);
        o[1] = cadd(m, e);
        o[2] = csub(m, e);
      }
      const int base = (j - k) * r + k;
      for (int q = 0; q < r; ++q) dst[base + q * ns] = o[q];
    }
    cpx* t = src; src = dst; dst = t;
    ns *= r;
  }
  if (src != x) memcpy(x, src, sizeof(cpx) * (size_t)n);
}

/* real <-> half complex of even length n via a length-n/2 complex FFT */
typedef struct {
  int n;
  fft1d half;
  cpx* w; /* exp(-2 pi i k / n), k <= n/2 */
} rfft1d;

static void rfft1d_init(rfft1d* p, int n) {
  p->n = n;
  fft1d_init(&p->half, n / 2);
  p->w = (cpx*)malloc(sizeof(cpx) * (size_t)(n / 2 + 1));
  const long double two_pi = 6.283185307179586476925286766559005768L;
  for (int k = 0; k <= n / 2; ++k) {
    long double a = two_pi * (long double)k / (long double)n;
    p->w[k].re = (double)cosl(a);
    p->w[k].im = (double)(-sinl(a));
  }
}

static void rfft1d_free(rfft1d* p) { fft1d_free(&p->half); free(p->w); }

/* scratch: >= n complex */
static void rfft_r2c(const rfft1d* p, const double* in, cpx* out, cpx* scratch) {
  const int h = p->n / 2;
  cpx* z = scratch;
  cpx* tmp = scratch + h;
  for (int m = 0; m < h; ++m) { z[m].re = in[2 * m]; z[m].im = in[2 * m + 1]; }
  fft1d_exec(&p->half, z, tmp, 0);
  for (int k = 0; k <= h; ++k) {
    cpx a = z[k % h], b = cconj(z[(h - k) % h]);
    cpx e = {0.5 * (a.re + b.re), 0.5 * (a.im + b.im)};
    cpx d = csub(a, b);
    cpx o = {0.5 * d.im, -0.5 * d.re}; /* (a - b) / (2i) */
    out[k] = cadd(e, cmul(p->w[k], o));
  }
}

/* includes 1/n; imaginary parts of in[0] and in[n/2] ignored */
static void rfft_c2r(const rfft1d* p, const cpx* in, double* out, cpx* scratch) {
  const int h = p->n / 2;
  cpx* z = scratch;
  cpx* tmp = scratch + h;
  for (int k = 0; k < h; ++k) {
    cpx xk = in[k], xm = in[h - k];
    if (k == 0) { xk.im = 0.0; xm.im = 0.0; }
    cpx a = cadd(xk, cconj(xm));
    cpx b = cmul(csub(xk, cconj(xm)), cconj(p->w[k]));
    z[k].re = a.re - b.im;
    z[k].im = a.im + b.re;
  }
  fft1d_exec(&p->half, z, tmp, 1);
  const double s = 1.0 / (double)p->n;
  for (int m = 0; m < h; ++m) { out[2 * m] = z[m].re * s; out[2 * m + 1] = z[m].im * s; }
}

/* ------------------------------------------------------------------------- */
/* 3-D backend                                                                */
/* ------------------------------------------------------------------------- */
typedef struct {
  int nx, ny, nz, hz;
  fft1d fx, fy;
  rfft1d fz;
  /* cuFFT mode (vkc_set_cufft): device buffers and D2Z / Z2D plans made once
   * per backend, as CufftBackend::new does (vonkarman-fft/src/cufft.rs:193-241) */
  int cufft;
  void* d_real;
  void* d_cplx;
  int plan_d2z, plan_z2d;
} backend;

/* ------------------------------------------------------------------------- */
/* cuFFT mode: the reference's GPU backend (vonkarman-fft/src/cufft.rs),       */
/* restated.  libcudart / libcufft are loaded at run time (cufft.rs:76-168);   */
/* every transform copies its input host -> device with a blocking cudaMemcpy, */
/* runs cufftExecD2Z / Z2D and copies the result back (cufft.rs:249-319); c2r  */
/* divides by nx ny nz on the host afterwards (cufft.rs:317-318).  Only the    */
/* timed baseline of the reference's GPU mode uses it.                         */
/* ------------------------------------------------------------------------- */
typedef struct {
  int loaded;
  void* cudart;
  void* cufft;
  int (*cuda_malloc)(void**, size_t);
  int (*cuda_free)(void*);
  int (*cuda_memcpy)(void*, const void*, size_t, int);
  int (*plan_3d)(int*, int, int, int, int);
  int (*exec_d2z)(int, double*, void*);
  int (*exec_z2d)(int, void*, double*);
  int (*destroy)(int);
} cuda_libs;

static cuda_libs g_cu;
static int g_use_cufft = 0;
static char g_cu_err[256] = "";
enum { CUFFT_D2Z_ = 0x6a, CUFFT_Z2D_ = 0x6c, MEMCPY_H2D_ = 1, MEMCPY_D2H_ = 2 };

static void* open_first(const char* const* names) {
  for (int i = 0; names[i]; ++i) {
    void* h = dlopen(names[i], RTLD_NOW | RTLD_LOCAL);
    if (h) return h;
  }
  return NULL;
}

static int cu_load(void) {
  if (g_cu.loaded) return 0;
  static const char* const rt[] = {"libcudart.so", "libcudart.so.13", "libcudart.so.12",
                                   "/usr/local/cuda/lib64/libcudart.so", NULL};
  static const char* const ff[] = {"libcufft.so", "libcufft.so.12", "libcufft.so.11",
                                   "/usr/local/cuda/lib64/libcufft.so", NULL};
  g_cu.cudart = open_first(rt);
  g_cu.cufft = open_first(ff);
  if (!g_cu.cudart || !g_cu.cufft) {
    snprintf(g_cu_err, sizeof g_cu_err, "cannot load %s", g_cu.cudart ? "libcufft.so" : "libcudart.so");
    return 1;
  }
  *(void**)&g_cu.cuda_malloc = dlsym(g_cu.cudart, "cudaMalloc");
  *(void**)&g_cu.cuda_free = dlsym(g_cu.cudart, "cudaFree");
  *(void**)&g_cu.cuda_memcpy = dlsym(g_cu.cudart, "cudaMemcpy");
  *(void**)&g_cu.plan_3d = dlsym(g_cu.cufft, "cufftPlan3d");
  *(void**)&g_cu.exec_d2z = dlsym(g_cu.cufft, "cufftExecD2Z");
  *(void**)&g_cu.exec_z2d = dlsym(g_cu.cufft, "cufftExecZ2D");
  *(void**)&g_cu.destroy = dlsym(g_cu.cufft, "cufftDestroy");
  if (!g_cu.cuda_malloc || !g_cu.cuda_free || !g_cu.cuda_memcpy || !g_cu.plan_3d || !g_cu.exec_d2z ||
      !g_cu.exec_z2d || !g_cu.destroy) {
    snprintf(g_cu_err, sizeof g_cu_err, "missing cudart / cufft symbols");
    return 1;
  }
  g_cu.loaded = 1;
  return 0;
}

static int cufft_backend_init(backend* b) {
  const size_t nreal = (size_t)b->nx * b->ny * b->nz, ncplx = (size_t)b->nx * b->ny * b->hz;
  int rc = g_cu.cuda_malloc(&b->d_real, nreal * sizeof(double));
  if (rc == 0) rc = g_cu.cuda_malloc(&b->d_cplx, ncplx * 2 * sizeof(double));
  if (rc == 0) rc = g_cu.plan_3d(&b->plan_d2z, b->nx, b->ny, b->nz, CUFFT_D2Z_);
  if (rc == 0) rc = g_cu.plan_3d(&b->plan_z2d, b->nx, b->ny, b->nz, CUFFT_Z2D_);
  if (rc != 0) snprintf(g_cu_err, sizeof g_cu_err, "cuFFT backend set-up failed (code %d)", rc);
  b->cufft = rc == 0;
  return rc;
}

static void backend_init(backend* b, int nx, int ny, int nz) {
  b->nx = nx; b->ny = ny; b->nz = nz; b->hz = nz / 2 + 1;
  fft1d_init(&b->fx, nx);
  fft1d_init(&b->fy, ny);
  rfft1d_init(&b->fz, nz);
  b->cufft = 0;
  b->d_real = b->d_cplx = NULL;
  b->plan_d2z = b->plan_z2d = 0;
  if (g_use_cufft) cufft_backend_init(b);
}

static void backend_free(backend* b) {
  fft1d_free(&b->fx); fft1d_free(&b->fy); rfft1d_free(&b->fz);
  if (b->cufft) {
    g_cu.destroy(b->plan_d2z);
    g_cu.destroy(b->plan_z2d);
  }
  if (b->d_real) g_cu.cuda_free(b->d_real);
  if (b->d_cplx) g_cu.cuda_free(b->d_cplx);
}

/* CufftBackend::r2c_3d / c2r_3d (cufft.rs:249-319).  Failures abort the
 * transform with a message (the reference panics). */
static void cufft_r2c(const backend* b, const double* in, cpx* out) {
  const size_t nreal = (size_t)b->nx * b->ny * b->nz, ncplx = (size_t)b->nx * b->ny * b->hz;
  int rc = g_cu.cuda_memcpy(b->d_real, in, nreal * sizeof(double), MEMCPY_H2D_);
  if (rc == 0) rc = g_cu.exec_d2z(b->plan_d2z, (double*)b->d_real, b->d_cplx);
  if (rc == 0) rc = g_cu.cuda_memcpy(out, b->d_cplx, ncplx * sizeof(cpx), MEMCPY_D2H_);
  if (rc != 0) { fprintf(stderr, "cuFFT r2c failed: %d\n", rc); abort(); }
}

static void cufft_c2r(const backend* b, const cpx* in, double* out) {
  const size_t nreal = (size_t)b->nx * b->ny * b->nz, ncplx = (size_t)b->nx * b->ny * b->hz;
  int rc = g_cu.cuda_memcpy(b->d_cplx, in, ncplx * sizeof(cpx), MEMCPY_H2D_);
  if (rc == 0) rc = g_cu.exec_z2d(b->plan_z2d, b->d_cplx, (double*)b->d_real);
  if (rc == 0) rc = g_cu.cuda_memcpy(out, b->d_real, nreal * sizeof(double), MEMCPY_D2H_);
  if (rc != 0) { fprintf(stderr, "cuFFT c2r failed: %d\n", rc); abort(); }
  const double n_total = (double)nreal;
#pragma omp parallel for schedule(static)
  for (long i = 0; i < (long)nreal; ++i) out[i] = out[i] / n_total;
}

static int maxi(int a, int b) { return a > b ? a : b; }

/* complex transform along axis 0 (x) or 1 (y) of (nx, ny, hz), src -> dst */
static void c2c_axis(const backend* b, int axis, const cpx* src, cpx* dst, int inverse) {
  const int nx = b->nx, ny = b->ny, hz = b->hz;
  const fft1d* f = axis == 0 ? &b->fx : &b->fy;
  const int L = f->n;
  const int nouter = axis == 0 ? ny : nx;
  const double s = inverse ? 1.0 / (double)L : 1.0;
#pragma omp parallel
  {
    cpx* lane = (cpx*)malloc(sizeof(cpx) * 2 * (size_t)L);
    cpx* tmp = lane + L;
#pragma omp for collapse(2) schedule(static)
    for (int o = 0; o < nouter; ++o)
      for (int z = 0; z < hz; ++z) {
        for (int p = 0; p < L; ++p) {
          size_t idx = axis == 0 ? ((size_t)p * ny + o) * hz + z : ((size_t)o * ny + p) * hz + z;
          lane[p] = src[idx];
        }
        fft1d_exec(f, lane, tmp, inverse);
        for (int p = 0; p < L; ++p) {
          size_t idx = axis == 0 ? ((size_t)p * ny + o) * hz + z : ((size_t)o * ny + p) * hz + z;
          cpx v = lane[p];
          if (inverse) { v.re *= s; v.im *= s; }
          dst[idx] = v;
        }
      }
    free(lane);
  }
}

static void r2c_3d(const backend* b, const double* in, cpx* out) {
  if (b->cufft) { cufft_r2c(b, in, out); return; }
  const size_t nc = (size_t)b->nx * b->ny * b->hz;
  cpx* temp_rz = (cpx*)calloc(nc, sizeof(cpx));
#pragma omp parallel
  {
    cpx* scratch = (cpx*)malloc(sizeof(cpx) * (size_t)b->nz);
#pragma omp for schedule(static)
    for (long col = 0; col < (long)b->nx * b->ny; ++col)
      rfft_r2c(&b->fz, in + (size_t)col * b->nz, temp_rz + (size_t)col * b->hz, scratch);
    free(scratch);
  }
  cpx* temp_ry = (cpx*)malloc(nc * sizeof(cpx));
  memcpy(temp_ry, temp_rz, nc * sizeof(cpx)); /* temp_rz.clone() */
  c2c_axis(b, 1, temp_rz, temp_ry, 0);
  c2c_axis(b, 0, temp_ry, out, 0);
  free(temp_rz);
  free(temp_ry);
}

static void c2r_3d(const backend* b, const cpx* in, double* out) {
  if (b->cufft) { cufft_c2r(b, in, out); return; }
  const size_t nc = (size_t)b->nx * b->ny * b->hz;
  cpx* temp_ix = (cpx*)calloc(nc, sizeof(cpx));
  c2c_axis(b, 0, in, temp_ix, 1);
  cpx* temp_iy = (cpx*)malloc(nc * sizeof(cpx));
  memcpy(temp_iy, temp_ix, nc * sizeof(cpx));
  c2c_axis(b, 1, temp_ix, temp_iy, 1);
#pragma omp parallel
  {
    cpx* scratch = (cpx*)malloc(sizeof(cpx) * (size_t)b->nz);
#pragma omp for schedule(static)
    for (long col = 0; col < (long)b->nx * b->ny; ++col)
      rfft_c2r(&b->fz, temp_iy + (size_t)col * b->hz, out + (size_t)col * b->nz, scratch);
    free(scratch);
  }
  free(temp_ix);
  free(temp_iy);
}

/* ------------------------------------------------------------------------- */
/* solver                                                                     */
/* ------------------------------------------------------------------------- */
typedef struct { double exp_full, exp_half, a21, a31, a41, b1, b23, b4; } etd_coeffs;

typedef struct {
  int n, h, m;
  double l, nu, dt, time, cfl_safety, dt_fixed;
  int dt_mode; /* 0 = cfl, 1 = fixed */
  uint64_t step_count;
  size_t ns; /* n*n*h */
  double *kx, *ky, *kz, *k2;
  cpx* u[3];
  etd_coeffs* etd;
  backend fft, fft_padded;
} solver;

static double* rfftfreq_full(int n, double l) {
  double* k = (double*)malloc(sizeof(double) * n);
  double scale = 2.0 * 3.14159265358979323846 / l;
  for (int i = 0; i < n / 2; ++i) k[i] = (double)i * scale;
  for (int i = n / 2; i < n; ++i) k[i] = ((double)i - (double)n) * scale;
  return k;
}

#define M_CONTOUR 32
static double phi_n(int which, double z) {
  if (fabs(z) < 1e-300) return which == 1 ? 1.0 : which == 2 ? 0.5 : 1.0 / 6.0;
  const double pi = 3.14159265358979323846;
  double sum = 0.0;
  for (int j = 0; j < M_CONTOUR; ++j) {
    double theta = 2.0 * pi * ((double)j + 0.5) / (double)M_CONTOUR;
    double w_re = z + 1.0 * cos(theta), w_im = 1.0 * sin(theta);
    double e = exp(w_re);
    double ew_re = e * cos(w_im), ew_im = e * sin(w_im);
    if (which == 1) {
      double num_re = ew_re - 1.0, num_im = ew_im;
      double den = w_re * w_re + w_im * w_im;
      sum += (num_re * w_re + num_im * w_im) / den;
    } else {
      double w2_re = w_re * w_re - w_im * w_im, w2_im = 2.0 * w_re * w_im;
      if (which == 2) {
        double num_re = ew_re - 1.0 - w_re, num_im = ew_im - w_im;
        double den = w2_re * w2_re + w2_im * w2_im;
        sum += (num_re * w2_re + num_im * w2_im) / den;
      } else {
        double num_re = ew_re - 1.0 - w_re - 0.5 * w2_re, num_im = ew_im - w_im - 0.5 * w2_im;
        double w3_re = w_re * w2_re - w_im * w2_im, w3_im = w_re * w2_im + w_im * w2_re;
        double den = w3_re * w3_re + w3_im * w3_im;
        sum += (num_re * w3_re + num_im * w3_im) / den;
      }
    }
  }
  return sum / (double)M_CONTOUR;
}

static void compute_etd(solver* s) {
#pragma omp parallel for schedule(static)
  for (long i = 0; i < (long)s->ns; ++i) {
    double lambda = -s->nu * s->k2[i];
    double z = lambda * s->dt, zh = z / 2.0;
    double p1h = phi_n(1, zh), p1 = phi_n(1, z), p2 = phi_n(2, z), p3 = phi_n(3, z);
    etd_coeffs c;
    c.exp_full = exp(z);
    c.exp_half = exp(zh);
    c.a21 = p1h;
    c.a31 = p1h;
    c.a41 = p1;
    c.b1 = p1 - 3.0 * p2 + 4.0 * p3;
    c.b23 = 2.0 * p2 - 4.0 * p3;
    c.b4 = -p2 + 4.0 * p3;
    s->etd[i] = c;
  }
}

static cpx* spectral_zeros(const solver* s) { return (cpx*)calloc(s->ns, sizeof(cpx)); }

static void curl(const solver* s, cpx* const u[3], cpx* o[3]) {
  const int n = s->n, h = s->h;
#pragma omp parallel for collapse(2) schedule(static)
  for (int ix = 0; ix < n; ++ix)
    for (int iy = 0; iy < n; ++iy)
      for (int iz = 0; iz < h; ++iz) {
        size_t i = ((size_t)ix * n + iy) * h + iz;
        double kx = s->kx[ix], ky = s->ky[iy], kz = s->kz[iz];
        cpx ux = u[0][i], uy = u[1][i], uz = u[2][i];
        o[0][i] = (cpx){-(ky * uz.im - kz * uy.im), ky * uz.re - kz * uy.re};
        o[1][i] = (cpx){-(kz * ux.im - kx * uz.im), kz * ux.re - kx * uz.re};
        o[2][i] = (cpx){-(kx * uy.im - ky * ux.im), kx * uy.re - ky * ux.re};
      }
}

static void leray(const solver* s, cpx* u[3]) {
  const int n = s->n, h = s->h;
#pragma omp parallel for collapse(2) schedule(static)
  for (int ix = 0; ix < n; ++ix)
    for (int iy = 0; iy < n; ++iy)
      for (int iz = 0; iz < h; ++iz) {
        size_t i = ((size_t)ix * n + iy) * h + iz;
        double k2 = s->k2[i];
        if (k2 < 1e-30) continue;
        double inv = 1.0 / k2, kx = s->kx[ix], ky = s->ky[iy], kz = s->kz[iz];
        cpx ux = u[0][i], uy = u[1][i], uz = u[2][i];
        double dr = kx * ux.re + ky * uy.re + kz * uz.re, di = kx * ux.im + ky * uy.im + kz * uz.im;
        u[0][i] = (cpx){ux.re - kx * dr * inv, ux.im - kx * di * inv};
        u[1][i] = (cpx){uy.re - ky * dr * inv, uy.im - ky * di * inv};
        u[2][i] = (cpx){uz.re - kz * dr * inv, uz.im - kz * di * inv};
      }
}

static void dealiased_cross(const solver* s, cpx* const u[3], cpx* const w[3], cpx* out[3]) {
  const int n = s->n, m = s->m, hm = m / 2 + 1, h = s->h;
  const size_t np = (size_t)m * m * m, nps = (size_t)m * m * hm;
  const double scale = (double)((size_t)m * m * m) / (double)((size_t)n * n * n);
  double* up[3];
  double* wp[3];
  for (int c = 0; c < 3; ++c) { up[c] = (double*)calloc(np, sizeof(double)); wp[c] = (double*)calloc(np, sizeof(double)); }
  for (int pass = 0; pass < 2; ++pass) {
    cpx* const* src = pass == 0 ? u : w;
    double** dst = pass == 0 ? up : wp;
    for (int c = 0; c < 3; ++c) {
      cpx* pad = (cpx*)calloc(nps, sizeof(cpx)); /* zero_pad_spectral: dst.fill(0) */
#pragma omp parallel for schedule(static)
      for (int ix = 0; ix < n; ++ix) {
        int dix = ix < n / 2 ? ix : m - (n - ix);
        for (int iy = 0; iy < n; ++iy) {
          int diy = iy < n / 2 ? iy : m - (n - iy);
          for (int iz = 0; iz < h; ++iz) pad[((size_t)dix * m + diy) * hm + iz] = src[c][((size_t)ix * n + iy) * h + iz];
        }
      }
#pragma omp parallel for schedule(static)
      for (long i = 0; i < (long)nps; ++i) { pad[i].re *= scale; pad[i].im *= scale; }
      c2r_3d(&s->fft_padded, pad, dst[c]);
      free(pad);
    }
  }
  double* cr[3];
  for (int c = 0; c < 3; ++c) cr[c] = (double*)calloc(np, sizeof(double));
#pragma omp parallel for schedule(static)
  for (long i = 0; i < (long)np; ++i) {
    double ux = up[0][i], uy = up[1][i], uz = up[2][i], ox = wp[0][i], oy = wp[1][i], oz = wp[2][i];
    cr[0][i] = uy * oz - uz * oy;
    cr[1][i] = uz * ox - ux * oz;
    cr[2][i] = ux * oy - uy * ox;
  }
  cpx* ch[3];
  for (int c = 0; c < 3; ++c) {
    ch[c] = (cpx*)calloc(nps, sizeof(cpx));
    r2c_3d(&s->fft_padded, cr[c], ch[c]);
  }
  const double inv = 1.0 / scale;
  for (int c = 0; c < 3; ++c) {
#pragma omp parallel for schedule(static)
    for (int ix = 0; ix < n; ++ix) {
      int six = ix < n / 2 ? ix : m - (n - ix);
      for (int iy = 0; iy < n; ++iy) {
        int siy = iy < n / 2 ? iy : m - (n - iy);
        for (int iz = 0; iz < h; ++iz) {
          cpx v = ch[c][((size_t)six * m + siy) * hm + iz];
          out[c][((size_t)ix * n + iy) * h + iz] = (cpx){v.re * inv, v.im * inv};
        }
      }
    }
  }
  for (int c = 0; c < 3; ++c) { free(up[c]); free(wp[c]); free(cr[c]); free(ch[c]); }
}

static void compute_nonlinear(const solver* s, cpx* const u[3], cpx* out[3]) {
  cpx* om[3];
  for (int c = 0; c < 3; ++c) om[c] = spectral_zeros(s);
  curl(s, u, om);
  dealiased_cross(s, u, om, out);
  leray(s, out);
  for (int c = 0; c < 3; ++c) free(om[c]);
}

static double cfl_dt(solver* s) {
  const size_t np = (size_t)s->n * s->n * s->n;
  double* up[3];
  for (int c = 0; c < 3; ++c) {
    up[c] = (double*)calloc(np, sizeof(double));
    c2r_3d(&s->fft, s->u[c], up[c]);
  }
  double umax = 0.0;
#pragma omp parallel for reduction(max : umax) schedule(static)
  for (long i = 0; i < (long)np; ++i) {
    double sp = sqrt(up[0][i] * up[0][i] + up[1][i] * up[1][i] + up[2][i] * up[2][i]);
    if (sp > umax) umax = sp;
  }
  for (int c = 0; c < 3; ++c) free(up[c]);
  double dx = s->l / (double)s->n;
  double adv = umax > 1e-30 ? dx / umax : 1.0;
  double visc = s->nu > 1e-30 ? dx * dx / s->nu : INFINITY;
  double a = adv < visc ? adv : visc;
  return s->cfl_safety * (a < 0.1 ? a : 0.1);
}

static void etd_rk4_step(solver* s) {
  const size_t ns = s->ns;
  const double dt = s->dt;
  cpx *n1[3], *n2[3], *n3[3], *n4[3], *temp[3];
  for (int c = 0; c < 3; ++c) {
    n1[c] = spectral_zeros(s); n2[c] = spectral_zeros(s); n3[c] = spectral_zeros(s);
    n4[c] = spectral_zeros(s); temp[c] = spectral_zeros(s);
  }
  compute_nonlinear(s, s->u, n1);
  for (int c = 0; c < 3; ++c) {
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)ns; ++i) {
      const etd_coeffs* e = &s->etd[i];
      cpx u = s->u[c][i], n = n1[c][i];
      temp[c][i] = (cpx){e->exp_half * u.re + dt * e->a21 * n.re, e->exp_half * u.im + dt * e->a21 * n.im};
    }
  }
  compute_nonlinear(s, temp, n2);
  for (int c = 0; c < 3; ++c) {
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)ns; ++i) {
      const etd_coeffs* e = &s->etd[i];
      cpx u = s->u[c][i], n = n2[c][i];
      temp[c][i] = (cpx){e->exp_half * u.re + dt * e->a31 * n.re, e->exp_half * u.im + dt * e->a31 * n.im};
    }
  }
  compute_nonlinear(s, temp, n3);
  for (int c = 0; c < 3; ++c) {
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)ns; ++i) {
      const etd_coeffs* e = &s->etd[i];
      cpx u = s->u[c][i];
      double dr = 2.0 * n3[c][i].re - n1[c][i].re, di = 2.0 * n3[c][i].im - n1[c][i].im;
      temp[c][i] = (cpx){e->exp_full * u.re + dt * e->a41 * dr, e->exp_full * u.im + dt * e->a41 * di};
    }
  }
  compute_nonlinear(s, temp, n4);
  for (int c = 0; c < 3; ++c) {
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)ns; ++i) {
      const etd_coeffs* e = &s->etd[i];
      cpx u = s->u[c][i];
      double rr = e->b1 * n1[c][i].re + e->b23 * (n2[c][i].re + n3[c][i].re) + e->b4 * n4[c][i].re;
      double ri = e->b1 * n1[c][i].im + e->b23 * (n2[c][i].im + n3[c][i].im) + e->b4 * n4[c][i].im;
      s->u[c][i] = (cpx){e->exp_full * u.re + dt * rr, e->exp_full * u.im + dt * ri};
    }
  }
  for (int c = 0; c < 3; ++c) { free(n1[c]); free(n2[c]); free(n3[c]); free(n4[c]); free(temp[c]); }
}

/* ------------------------------------------------------------------------- */
/* C API for ctypes                                                           */
/* ------------------------------------------------------------------------- */
void vkc_set_threads(int t) {
#ifdef _OPENMP
  if (t > 0) omp_set_num_threads(t);
#else
  (void)t;
#endif
}

int vkc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void* vkc_create(int n, double l, double nu, int dt_mode, double dt_fixed, double cfl_safety) {
  if (n < 8 || (n & (n - 1)) != 0) return NULL;
  solver* s = (solver*)calloc(1, sizeof(solver));
  s->n = n; s->h = n / 2 + 1; s->m = 3 * n / 2;
  s->l = l; s->nu = nu; s->dt_mode = dt_mode; s->dt_fixed = dt_fixed; s->cfl_safety = cfl_safety;
  s->ns = (size_t)n * n * s->h;
  s->kx = rfftfreq_full(n, l);
  s->ky = rfftfreq_full(n, l);
  s->kz = (double*)malloc(sizeof(double) * s->h);
  for (int i = 0; i < s->h; ++i) s->kz[i] = (double)i * (2.0 * 3.14159265358979323846 / l);
  s->k2 = (double*)malloc(sizeof(double) * s->ns);
  for (int ix = 0; ix < n; ++ix)
    for (int iy = 0; iy < n; ++iy)
      for (int iz = 0; iz < s->h; ++iz)
        s->k2[((size_t)ix * n + iy) * s->h + iz] = s->kx[ix] * s->kx[ix] + s->ky[iy] * s->ky[iy] + s->kz[iz] * s->kz[iz];
  for (int c = 0; c < 3; ++c) s->u[c] = spectral_zeros(s);
  s->etd = (etd_coeffs*)malloc(sizeof(etd_coeffs) * s->ns);
  backend_init(&s->fft, n, n, n);
  backend_init(&s->fft_padded, s->m, s->m, s->m);
  return s;
}

void vkc_destroy(void* h) {
  solver* s = (solver*)h;
  if (!s) return;
  free(s->kx); free(s->ky); free(s->kz); free(s->k2); free(s->etd);
  for (int c = 0; c < 3; ++c) free(s->u[c]);
  backend_free(&s->fft);
  backend_free(&s->fft_padded);
  free(s);
}

/* Periodic3D::new after the IC transform (solver.rs:69-108) */
int vkc_set_state(void* h, const double* ux, const double* uy, const double* uz) {
  solver* s = (solver*)h;
  const double* src[3] = {ux, uy, uz};
  for (int c = 0; c < 3; ++c) memcpy(s->u[c], src[c], sizeof(cpx) * s->ns);
  s->time = 0.0;
  s->step_count = 0;
  s->dt = s->dt_mode == 1 ? s->dt_fixed : cfl_dt(s);
  compute_etd(s);
  return 0;
}

int vkc_get_state(void* h, double* ux, double* uy, double* uz) {
  solver* s = (solver*)h;
  double* dst[3] = {ux, uy, uz};
  for (int c = 0; c < 3; ++c) memcpy(dst[c], s->u[c], sizeof(cpx) * s->ns);
  return 0;
}

/* Domain::step (solver.rs:383-400) */
int vkc_step(void* h, int nsteps) {
  solver* s = (solver*)h;
  for (int k = 0; k < nsteps; ++k) {
    if (s->dt_mode == 0) {
      double nd = cfl_dt(s);
      if (fabs(nd - s->dt) / (s->dt > 1e-30 ? s->dt : 1e-30) > 0.01) {
        s->dt = nd;
        compute_etd(s);
      }
    }
    etd_rk4_step(s);
    s->time += s->dt;
    s->step_count += 1;
  }
  return 0;
}

/* One compute_nonlinear call (nonlinear.rs:15-39) on host arrays. */
int vkc_nonlinear(void* h, const double* ux, const double* uy, const double* uz, double* ox, double* oy, double* oz) {
  solver* s = (solver*)h;
  cpx* in[3] = {(cpx*)ux, (cpx*)uy, (cpx*)uz};
  cpx* out[3] = {(cpx*)ox, (cpx*)oy, (cpx*)oz};
  compute_nonlinear(s, in, out);
  return 0;
}

/* Backend mode of the solvers created afterwards: 0 = the CPU FFT (the
 * reference's ndrustfft backend), 1 = the reference's cuFFT backend pattern.
 * Returns 0, or 1 with a message in vkc_cufft_error() when the CUDA
 * libraries cannot be loaded. */
int vkc_set_cufft(int on) {
  if (on && cu_load() != 0) return 1;
  g_use_cufft = on ? 1 : 0;
  return 0;
}

const char* vkc_cufft_error(void) { return g_cu_err; }

/* 1 if the solver's transforms run through cuFFT. */
int vkc_uses_cufft(void* h) { return ((solver*)h)->fft_padded.cufft && ((solver*)h)->fft.cufft; }

/* energy_spectrum (vonkarman-diag/src/spectrum.rs:13-60): shell round(|k|),
 * E_s += 0.5 w |u|^2 / N^6.  Per-thread histograms over x planes, added in
 * thread order. */
int vkc_spectrum(void* h, double* out, int nsh) {
  solver* s = (solver*)h;
  const int n = s->n, hz = s->h;
  const double ntot = (double)n * (double)n * (double)n;
  const double kmx = (double)(n / 2);
  const int want = (int)ceil(sqrt(kmx * kmx + kmx * kmx + kmx * kmx)) + 1;
  if (nsh < want) return 1;
  int nt = 1;
#ifdef _OPENMP
  nt = omp_get_max_threads();
#endif
  double* hist = (double*)calloc((size_t)nt * want, sizeof(double));
#pragma omp parallel
  {
    int t = 0;
#ifdef _OPENMP
    t = omp_get_thread_num();
#endif
    double* my = hist + (size_t)t * want;
#pragma omp for schedule(static)
    for (int ix = 0; ix < n; ++ix)
      for (int iy = 0; iy < n; ++iy)
        for (int iz = 0; iz < hz; ++iz) {
          const double kx = s->kx[ix], ky = s->ky[iy], kz = s->kz[iz];
          const int shell = (int)round(sqrt(kx * kx + ky * ky + kz * kz));
          if (shell >= want) continue;
          const size_t i = ((size_t)ix * n + iy) * hz + iz;
          double mag2 = 0.0;
          for (int c = 0; c < 3; ++c) mag2 += s->u[c][i].re * s->u[c][i].re + s->u[c][i].im * s->u[c][i].im;
          const double w = (iz == 0 || iz == n / 2) ? 1.0 : 2.0;
          my[shell] += 0.5 * w * mag2 / (ntot * ntot);
        }
  }
  for (int k = 0; k < want; ++k) {
    double acc = 0.0;
    for (int t = 0; t < nt; ++t) acc += hist[(size_t)t * want + k];
    out[k] = acc;
  }
  free(hist);
  return 0;
}

double vkc_time(void* h) { return ((solver*)h)->time; }
double vkc_dt(void* h) { return ((solver*)h)->dt; }

/* FftBackend on host arrays */
int vkc_r2c_3d(int nx, int ny, int nz, const double* in, double* out) {
  backend b;
  backend_init(&b, nx, ny, nz);
  r2c_3d(&b, in, (cpx*)out);
  backend_free(&b);
  return 0;
}

int vkc_c2r_3d(int nx, int ny, int nz, const double* in, double* out) {
  backend b;
  backend_init(&b, nx, ny, nz);
  c2r_3d(&b, (const cpx*)in, out);
  backend_free(&b);
  return 0;
}
