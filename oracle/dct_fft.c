/* ORACLE / TEST INFRASTRUCTURE ONLY.  See dct_fft.h for definitions and the
 * published algorithms this follows.  Only tests, the smoke check and the
 * bench's CPU-baseline leg use it. */
#include "dct_fft.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

typedef struct { double re, im; } cpx;

struct dctfft_plan {
  int n;
  int nfac;
  int fac[64];
  cpx* tw;    /* exp(-2 pi i j / n), j < n */
  cpx* half;  /* exp(-i pi k / (2n)), k < n */
};

static inline cpx cmul(cpx a, cpx b) {
  cpx r;
  r.re = a.re * b.re - a.im * b.im;
  r.im = a.re * b.im + a.im * b.re;
  return r;
}
static inline cpx cconj(cpx a) { a.im = -a.im; return a; }

dctfft_plan* dctfft_make(int n) {
  if (n < 1) return NULL;
  dctfft_plan* p = (dctfft_plan*)calloc(1, sizeof(dctfft_plan));
  p->n = n;
  int m = n;
  /* radix-4 first (fewest passes), then 2, 3, 5, then any other prime */
  while (m % 4 == 0) { p->fac[p->nfac++] = 4; m /= 4; }
  while (m % 2 == 0) { p->fac[p->nfac++] = 2; m /= 2; }
  for (int f = 3; f * f <= m; f += 2)
    while (m % f == 0) { p->fac[p->nfac++] = f; m /= f; }
  if (m > 1) p->fac[p->nfac++] = m;
  p->tw = (cpx*)malloc(sizeof(cpx) * (size_t)n);
  p->half = (cpx*)malloc(sizeof(cpx) * (size_t)n);
  for (int j = 0; j < n; ++j) {
    double a = -2.0 * M_PI * (double)j / (double)n;
    p->tw[j].re = cos(a);
    p->tw[j].im = sin(a);
    double b = -M_PI * (double)j / (2.0 * (double)n);
    p->half[j].re = cos(b);
    p->half[j].im = sin(b);
  }
  return p;
}

void dctfft_free(dctfft_plan* p) {
  if (!p) return;
  free(p->tw);
  free(p->half);
  free(p);
}

int dctfft_length(const dctfft_plan* p) { return p->n; }
int dctfft_scratch_doubles(const dctfft_plan* p) { return 8 * p->n; }

/* Decimation-in-time mixed-radix FFT.  out[0..n) receives the DFT of
 * in[0], in[istride], ...; twiddles come from the length-N table with step
 * N/n.  inv selects exp(+2 pi i ...).  tmp holds at least 2n entries. */
static void fft_rec(const dctfft_plan* P, cpx* out, const cpx* in, int n,
                    int istride, const int* fac, int inv, cpx* tmp) {
  if (n == 1) { out[0] = in[0]; return; }
  const int N = P->n;
  const int p = fac[0];
  const int m = n / p;
  for (int r = 0; r < p; ++r)
    fft_rec(P, out + r * m, in + r * istride, m, istride * p, fac + 1, inv, tmp);
  const int step = N / n;
  if (p == 2) {
    for (int k = 0; k < m; ++k) {
      cpx w = P->tw[k * step];
      if (inv) w = cconj(w);
      cpx a = out[k], b = cmul(out[m + k], w);
      out[k].re = a.re + b.re; out[k].im = a.im + b.im;
      out[m + k].re = a.re - b.re; out[m + k].im = a.im - b.im;
    }
    return;
  }
  if (p == 4) {
    for (int k = 0; k < m; ++k) {
      cpx w1 = P->tw[k * step], w2 = P->tw[2 * k * step], w3 = P->tw[3 * k * step];
      if (inv) { w1 = cconj(w1); w2 = cconj(w2); w3 = cconj(w3); }
      cpx a0 = out[k];
      cpx a1 = cmul(out[m + k], w1);
      cpx a2 = cmul(out[2 * m + k], w2);
      cpx a3 = cmul(out[3 * m + k], w3);
      cpx s02 = {a0.re + a2.re, a0.im + a2.im}, d02 = {a0.re - a2.re, a0.im - a2.im};
      cpx s13 = {a1.re + a3.re, a1.im + a3.im}, d13 = {a1.re - a3.re, a1.im - a3.im};
      /* forward: multiply d13 by -i ; inverse: by +i */
      cpx j13 = inv ? (cpx){-d13.im, d13.re} : (cpx){d13.im, -d13.re};
      out[k].re = s02.re + s13.re; out[k].im = s02.im + s13.im;
      out[m + k].re = d02.re + j13.re; out[m + k].im = d02.im + j13.im;
      out[2 * m + k].re = s02.re - s13.re; out[2 * m + k].im = s02.im - s13.im;
      out[3 * m + k].re = d02.re - j13.re; out[3 * m + k].im = d02.im - j13.im;
    }
    return;
  }
  /* generic radix p */
  const int pstep = N / p;
  for (int k = 0; k < m; ++k) {
    for (int r = 0; r < p; ++r) {
      cpx w = P->tw[((long)r * k * step) % N];
      if (inv) w = cconj(w);
      tmp[r] = cmul(out[r * m + k], w);
    }
    for (int q = 0; q < p; ++q) {
      cpx acc = tmp[0];
      for (int r = 1; r < p; ++r) {
        cpx w = P->tw[(long)((r * q) % p) * pstep];
        if (inv) w = cconj(w);
        cpx t = cmul(tmp[r], w);
        acc.re += t.re; acc.im += t.im;
      }
      tmp[p + q] = acc;
    }
    for (int q = 0; q < p; ++q) out[q * m + k] = tmp[p + q];
  }
}

void dctfft_redft10(const dctfft_plan* P, double* x, double* scratch) {
  const int n = P->n;
  cpx* v = (cpx*)scratch;
  cpx* V = v + n;
  cpx* tmp = V + n;
  for (int j = 0; 2 * j < n; ++j) { v[j].re = x[2 * j]; v[j].im = 0.0; }
  for (int j = 0; 2 * j + 1 < n; ++j) { v[n - 1 - j].re = x[2 * j + 1]; v[n - 1 - j].im = 0.0; }
  fft_rec(P, V, v, n, 1, P->fac, 0, tmp);
  for (int k = 0; k < n; ++k) {
    cpx h = P->half[k];
    x[k] = 2.0 * (h.re * V[k].re - h.im * V[k].im);
  }
}

void dctfft_redft01(const dctfft_plan* P, double* x, double* scratch) {
  const int n = P->n;
  cpx* W = (cpx*)scratch;
  cpx* w = W + n;
  cpx* tmp = w + n;
  for (int k = 0; k < n; ++k) {
    double yk = x[k];
    double ynk = (k == 0) ? 0.0 : x[n - k];
    cpx a = {yk, -ynk};               /* Y[k] - i Y[n-k] */
    W[k] = cmul(cconj(P->half[k]), a); /* times exp(+i pi k / 2n) */
  }
  fft_rec(P, w, W, n, 1, P->fac, 1, tmp);
  for (int j = 0; 2 * j < n; ++j) x[2 * j] = w[j].re;
  for (int j = 0; 2 * j + 1 < n; ++j) x[2 * j + 1] = w[n - 1 - j].re;
}

/* ---- plan cache for the 3D helpers ---- */
#define DCTFFT_CACHE 8192
static dctfft_plan* g_cache[DCTFFT_CACHE];
static pthread_mutex_t g_lock = PTHREAD_MUTEX_INITIALIZER;

static const dctfft_plan* cached_plan(int n) {
  if (n < DCTFFT_CACHE) {
    dctfft_plan* p = __atomic_load_n(&g_cache[n], __ATOMIC_ACQUIRE);
    if (p) return p;
    pthread_mutex_lock(&g_lock);
    p = g_cache[n];
    if (!p) {
      p = dctfft_make(n);
      __atomic_store_n(&g_cache[n], p, __ATOMIC_RELEASE);
    }
    pthread_mutex_unlock(&g_lock);
    return p;
  }
  return NULL;
}

static void transform_axis(double* a, int n0, int n1, int n2, int axis, int kind) {
  const int len = axis == 0 ? n0 : (axis == 1 ? n1 : n2);
  const long stride = axis == 0 ? (long)n1 * n2 : (axis == 1 ? n2 : 1);
  dctfft_plan* own = NULL;
  const dctfft_plan* P = cached_plan(len);
  if (!P) { own = dctfft_make(len); P = own; }
  double* line = (double*)malloc(sizeof(double) * (size_t)len);
  double* scratch = (double*)malloc(sizeof(double) * (size_t)dctfft_scratch_doubles(P));
  const long nlines = (long)n0 * n1 * n2 / len;
  for (long l = 0; l < nlines; ++l) {
    long base;
    if (axis == 2) base = l * n2;
    else if (axis == 1) base = (l / n2) * (long)n1 * n2 + (l % n2);
    else base = l;
    for (int i = 0; i < len; ++i) line[i] = a[base + i * stride];
    if (kind == 10) dctfft_redft10(P, line, scratch);
    else dctfft_redft01(P, line, scratch);
    for (int i = 0; i < len; ++i) a[base + i * stride] = line[i];
  }
  free(line);
  free(scratch);
  dctfft_free(own);
}

void dctfft_3d_double(int n0, int n1, int n2, int kind, const double* in, double* out) {
  const long N = (long)n0 * n1 * n2;
  if (out != in) memcpy(out, in, sizeof(double) * (size_t)N);
  transform_axis(out, n0, n1, n2, 2, kind);
  transform_axis(out, n0, n1, n2, 1, kind);
  transform_axis(out, n0, n1, n2, 0, kind);
}

void dctfft_3d_float(int n0, int n1, int n2, int kind, const float* in, float* out) {
  const long N = (long)n0 * n1 * n2;
  double* a = (double*)malloc(sizeof(double) * (size_t)N);
  for (long i = 0; i < N; ++i) a[i] = (double)in[i];
  dctfft_3d_double(n0, n1, n2, kind, a, a);
  for (long i = 0; i < N; ++i) out[i] = (float)a[i];
  free(a);
}
