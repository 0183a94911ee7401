/* ORACLE / TEST INFRASTRUCTURE ONLY -- the checker, never the product.
 *
 * Plain C restatement of one ARD time step of pjx3/ARD-simulator, run on the
 * host over a flattened scene (include/ard_gb300.h).  Only tests/, the smoke
 * check and bench.py's CPU-baseline leg load it.  It is compiled twice:
 * REAL=float (suffix _f32), which mirrors the reference's float arithmetic
 * expression by expression and, built with -ffp-contract=off, reproduces the
 * headless reference build bit for bit; and REAL=double (suffix _f64), the
 * FP64 oracle of the same algorithm with the same float-valued parameters.
 *
 * What follows which reference code (paths in ARD-simulator-190113/):
 *   step order ............ simulation.cpp:300-318  (phase A over partitions,
 *                           then phase B over boundaries in list order)
 *   source forcing ........ partition.cpp:187-197   (overwrite the force cell)
 *   modal tables .......... dct_partition.cpp:20-36 (1-based mode indices)
 *   air partition update .. dct_partition.cpp:48-73 + dct_volume.cpp:38-68
 *   PML construction ...... pml_partition.cpp:17-93 (zeta profiles, sentinel)
 *   PML update ............ pml_partition.cpp:113-200
 *   interface forcing ..... boundary.cpp:21-173
 * The DCTs are oracle/dct_fft.c (FFTW REDFT10/REDFT01 definitions).
 *
 * Parity is pinned: the _f32 instantiation is compared bit for bit with the
 * headless reference build (oracle/ref_build) on the committed fixtures in
 * tests/golden/.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "../include/ard_gb300.h"
#include "dct_fft.h"

#ifndef REAL
#define REAL float
#define SFX _f32
#endif

/* literal in the working precision: 2.0f in the float build, 2.0 in the double build */
#define L(x) ((REAL)(x))

#define CAT2(a, b) a##b
#define CAT(a, b) CAT2(a, b)
#define API(name) CAT(name, SFX)

#if defined(ORACLE_DOUBLE)
#define RPI ((REAL)M_PI)
#define DCT3D(n0, n1, n2, k, in, out) dctfft_3d_double(n0, n1, n2, k, in, out)
#define RSQRT(x) sqrt(x)
#define RCOS(x) cos(x)
#define RSIN(x) sin(x)
#define RLOG10(x) log10(x)
#define RPOW(x, y) pow(x, y)
#define REXP(x) exp(x)
#else
#define RPI ((float)M_PI)
#define DCT3D(n0, n1, n2, k, in, out) dctfft_3d_float(n0, n1, n2, k, in, out)
#define RSQRT(x) sqrtf(x)
#define RCOS(x) cosf(x)
#define RSIN(x) sinf(x)
#define RLOG10(x) log10f(x)
#define RPOW(x, y) powf(x, y)
#define REXP(x) expf(x)
#endif

typedef struct {
  int kind, pml_type;
  int xs, ys, zs, w, h, d;
  long n;
  int self_terms;
  /* air partition (DctPartition + its two DctVolumes) */
  REAL *f, *fm;        /* m_force.m_values / m_modes */
  REAL *p, *pm;        /* m_pressure.m_values / m_modes */
  REAL *prev, *next;   /* prev_modes_ / next_modes_ */
  REAL *cwt, *w2;
  /* PML partition: arrays of n+1 with a zero sentinel at [n] */
  REAL *pold, *pcur, *pnew;
  REAL *phx, *phxn, *phy, *phyn, *phz, *phzn;
  REAL *force, *zx, *zy, *zz;
  REAL thickness, zeta;
  int nsrc;
  int* src;            /* indices into the scene's source list */
} opart;

typedef struct {
  REAL dh, dt, c0, damping, R;
  int pml_layers;
  int np, nb, ns, nr;
  opart* parts;
  ard_boundary* bnd;
  ard_point* srcs;
  ard_point* recs;
  float** series;      /* per source, length series_len[i] */
  long* series_len;
  REAL scale[6];
  long t;
  REAL* hist;          /* recorder history [t][nr] */
  long hist_cap;
} osim;

static REAL* zalloc(long n) { return (REAL*)calloc((size_t)(n > 0 ? n : 1), sizeof(REAL)); }

/* PmlPartition::GetIndex (pml_partition.cpp:6-15) */
static inline long pidx(const opart* P, int x, int y, int z) {
  if (x < 0 || x >= P->w) return P->n;
  if (y < 0 || y >= P->h) return P->n;
  if (z < 0 || z >= P->d) return P->n;
  return (long)z * P->h * P->w + (long)y * P->w + x;
}

static void build_tables(osim* S, opart* P) {
  /* dct_partition.cpp:24-36 */
  REAL lx2 = P->w * P->w * S->dh * S->dh;
  REAL ly2 = P->h * P->h * S->dh * S->dh;
  REAL lz2 = P->d * P->d * S->dh * S->dh;
  for (int i = 1; i <= P->d; i++)
    for (int j = 1; j <= P->h; j++)
      for (int k = 1; k <= P->w; k++) {
        long idx = (long)(i - 1) * P->h * P->w + (long)(j - 1) * P->w + (k - 1);
        REAL w = S->c0 * RPI * RSQRT(i * i / lz2 + j * j / ly2 + k * k / lx2);
        P->w2[idx] = w * w;
        P->cwt[idx] = RCOS(w * S->dt);
      }
}

static void build_pml_profile(osim* S, opart* P) {
  /* pml_partition.cpp:26-28, 59-86; the per-face scale multiplies zeta */
  REAL pi = RPI;
  REAL z0 = P->zeta * S->scale[P->pml_type];
  REAL th = P->thickness, dh = S->dh;
  for (int k = 0; k < P->d; k++)
    for (int j = 0; j < P->h; j++)
      for (int i = 0; i < P->w; i++) {
        long I = pidx(P, i, j, k);
        switch (P->pml_type) {
          case ARD_PML_BACK:
            P->zz[I] = z0 * ((k + 1) / th * dh - RSIN(L(2.0) * pi * (k + 1) * dh / th) / L(2.0) / pi); break;
          case ARD_PML_FRONT:
            P->zz[I] = z0 * ((P->d - k) / th * dh - RSIN(L(2.0) * pi * (P->d - k) * dh / th) / L(2.0) / pi); break;
          case ARD_PML_BOTTOM:
            P->zy[I] = z0 * ((j + 1) / th * dh - RSIN(L(2.0) * pi * (j + 1) * dh / th) / L(2.0) / pi); break;
          case ARD_PML_TOP:
            P->zy[I] = z0 * ((P->h - j) / th * dh - RSIN(L(2.0) * pi * (P->h - j) * dh / th) / L(2.0) / pi); break;
          case ARD_PML_RIGHT:
            P->zx[I] = z0 * ((i + 1) / th * dh - RSIN(L(2.0) * pi * (i + 1) * dh / th) / L(2.0) / pi); break;
          case ARD_PML_LEFT:
            P->zx[I] = z0 * ((P->w - i) / th * dh - RSIN(L(2.0) * pi * (P->w - i) * dh / th) / L(2.0) / pi); break;
        }
      }
}

void* API(oracle_create)(const ard_scene* sc) {
  osim* S = (osim*)calloc(1, sizeof(osim));
  S->dh = sc->dh; S->dt = sc->dt; S->c0 = sc->c0;
  S->damping = sc->modal_damping;
  S->R = sc->pml_R;
  S->pml_layers = sc->pml_layers;
  S->np = sc->n_partitions; S->nb = sc->n_boundaries;
  S->ns = sc->n_sources; S->nr = sc->n_recorders;
  for (int f = 0; f < 6; ++f) S->scale[f] = 1;
  S->parts = (opart*)calloc((size_t)S->np, sizeof(opart));
  S->bnd = (ard_boundary*)malloc(sizeof(ard_boundary) * (size_t)(S->nb > 0 ? S->nb : 1));
  memcpy(S->bnd, sc->boundaries, sizeof(ard_boundary) * (size_t)S->nb);
  S->srcs = (ard_point*)malloc(sizeof(ard_point) * (size_t)(S->ns > 0 ? S->ns : 1));
  memcpy(S->srcs, sc->sources, sizeof(ard_point) * (size_t)S->ns);
  S->recs = (ard_point*)malloc(sizeof(ard_point) * (size_t)(S->nr > 0 ? S->nr : 1));
  memcpy(S->recs, sc->recorders, sizeof(ard_point) * (size_t)S->nr);
  S->series = (float**)calloc((size_t)(S->ns > 0 ? S->ns : 1), sizeof(float*));
  S->series_len = (long*)calloc((size_t)(S->ns > 0 ? S->ns : 1), sizeof(long));
  for (int i = 0; i < S->np; ++i) {
    const ard_partition* d = &sc->partitions[i];
    opart* P = &S->parts[i];
    P->kind = d->kind; P->pml_type = d->pml_type;
    P->xs = d->x_start; P->ys = d->y_start; P->zs = d->z_start;
    P->w = d->width; P->h = d->height; P->d = d->depth;
    P->n = (long)P->w * P->h * P->d;
    if (P->kind == ARD_PART_DCT) {
      P->self_terms = 1;
      P->f = zalloc(P->n); P->fm = zalloc(P->n);
      P->p = zalloc(P->n); P->pm = zalloc(P->n);
      P->prev = zalloc(P->n); P->next = zalloc(P->n);
      P->cwt = zalloc(P->n); P->w2 = zalloc(P->n);
      build_tables(S, P);
    } else {
      P->self_terms = 0;
      long m = P->n + 1;
      P->pold = zalloc(m); P->pcur = zalloc(m); P->pnew = zalloc(m);
      P->phx = zalloc(m); P->phxn = zalloc(m); P->phy = zalloc(m);
      P->phyn = zalloc(m); P->phz = zalloc(m); P->phzn = zalloc(m);
      P->force = zalloc(m);
      P->zx = zalloc(m); P->zy = zalloc(m); P->zz = zalloc(m);
      P->thickness = S->pml_layers * S->dh;
      P->zeta = S->c0 / P->thickness * RLOG10(L(1.0) / S->R);
      build_pml_profile(S, P);
    }
  }
  /* attach sources in list order (simulation.cpp:37-48) */
  for (int s = 0; s < S->ns; ++s) {
    int pi = S->srcs[s].partition;
    if (pi < 0) continue;
    opart* P = &S->parts[pi];
    P->src = (int*)realloc(P->src, sizeof(int) * (size_t)(P->nsrc + 1));
    P->src[P->nsrc++] = s;
  }
  return S;
}

void API(oracle_destroy)(void* h) {
  osim* S = (osim*)h;
  if (!S) return;
  for (int i = 0; i < S->np; ++i) {
    opart* P = &S->parts[i];
    REAL* arrs[] = {P->f, P->fm, P->p, P->pm, P->prev, P->next, P->cwt, P->w2,
                    P->pold, P->pcur, P->pnew, P->phx, P->phxn, P->phy, P->phyn,
                    P->phz, P->phzn, P->force, P->zx, P->zy, P->zz};
    for (size_t k = 0; k < sizeof arrs / sizeof arrs[0]; ++k) free(arrs[k]);
    free(P->src);
  }
  for (int s = 0; s < S->ns; ++s) free(S->series[s]);
  free(S->series); free(S->series_len);
  free(S->parts); free(S->bnd); free(S->srcs); free(S->recs); free(S->hist);
  free(S);
}

void API(oracle_set_source_series)(void* h, int src, const float* v, long n) {
  osim* S = (osim*)h;
  free(S->series[src]);
  S->series[src] = (float*)malloc(sizeof(float) * (size_t)(n > 0 ? n : 1));
  memcpy(S->series[src], v, sizeof(float) * (size_t)n);
  S->series_len[src] = n;
}

void API(oracle_set_pml_scale)(void* h, const double* scale6) {
  osim* S = (osim*)h;
  for (int f = 0; f < 6; ++f) S->scale[f] = (REAL)scale6[f];
  for (int i = 0; i < S->np; ++i) {
    opart* P = &S->parts[i];
    if (P->kind != ARD_PART_PML) continue;
    memset(P->zx, 0, sizeof(REAL) * (size_t)(P->n + 1));
    memset(P->zy, 0, sizeof(REAL) * (size_t)(P->n + 1));
    memset(P->zz, 0, sizeof(REAL) * (size_t)(P->n + 1));
    build_pml_profile(S, P);
  }
}

/* Extension (no reference counterpart): start an air partition at rest with
 * pressure p0, i.e. both modal levels equal DCT-II(p0) / (8N s_i), so that
 * s_i * DCT-III(modes) = p0. */
void API(oracle_set_initial_pressure)(void* h, int part, const double* p0) {
  osim* S = (osim*)h;
  opart* P = &S->parts[part];
  double* a = (double*)malloc(sizeof(double) * (size_t)P->n);
  dctfft_3d_double(P->d, P->h, P->w, 10, p0, a);
  double N = (double)P->n;
  double si = 1.0 / sqrt(2.0 * N);
  for (long i = 0; i < P->n; ++i) {
    REAL m = (REAL)(a[i] / (8.0 * N * si));
    P->pm[i] = m;
    P->prev[i] = m;
    P->p[i] = (REAL)p0[i];
  }
  free(a);
}

/* DctPartition::Update (dct_partition.cpp:48-73) with DctVolume's transforms
 * and normalisation (dct_volume.cpp:38-68). */
static void dct_update(osim* S, opart* P) {
  const long N = P->n;
  DCT3D(P->d, P->h, P->w, 10, P->f, P->fm);
  {
    REAL scale = L(1.0) / (L(2.0) * RSQRT(L(2.0) * P->d * P->w * P->h));
    for (long i = 0; i < N; i++) P->fm[i] *= scale;
  }
  for (long i = 0; i < N; i++)
    P->next[i] = S->damping * (L(2.0) * P->pm[i] * P->cwt[i] - P->prev[i] +
                               (L(2.0) * P->fm[i] / P->w2[i]) * (L(1.0) - P->cwt[i]));
  memcpy(P->prev, P->pm, sizeof(REAL) * (size_t)N);
  memcpy(P->pm, P->next, sizeof(REAL) * (size_t)N);
  DCT3D(P->d, P->h, P->w, 1, P->pm, P->p);
  {
    REAL scale = L(1.0) / RSQRT(L(2.0) * P->d * P->w * P->h);
    for (long i = 0; i < N; i++) P->p[i] *= scale;
  }
}

/* PmlPartition::Update (pml_partition.cpp:113-200) */
static void pml_update(osim* S, opart* P) {
  const REAL dh = S->dh, dt = S->dt, c0 = S->c0;
  const REAL coefs[7] = {2.0, -27.0, 270.0, -490.0, 270.0, -27.0, 2.0};
  const REAL fourth[5] = {1.0, -8.0, 0.0, 8.0, -1.0};
  REAL *p = P->pcur, *po = P->pold, *pn = P->pnew;
  for (int k = 0; k < P->d; k++)
    for (int j = 0; j < P->h; j++)
      for (int i = 0; i < P->w; i++) {
        REAL dxx = 0.0, dyy = 0.0, dzz = 0.0;
        for (int m = 0; m < 7; m++) {
          dxx += coefs[m] * p[pidx(P, i + m - 3, j, k)];
          dyy += coefs[m] * p[pidx(P, i, j + m - 3, k)];
          dzz += coefs[m] * p[pidx(P, i, j, k + m - 3)];
        }
        dxx /= (L(180.0) * dh * dh);
        dyy /= (L(180.0) * dh * dh);
        dzz /= (L(180.0) * dh * dh);
        const long I = pidx(P, i, j, k);
        const REAL zx = P->zx[I], zy = P->zy[I], zz = P->zz[I];
        REAL t1 = 2 * p[I];
        REAL t2 = -po[I];
        REAL t3 = c0 * c0 * (dxx + dyy + dzz);
        REAL t4 = -(zx + zy + zz) * (p[I] - po[I]) / dt;
        REAL t5 = -(zx * zy + zy * zz + zx * zz) * p[I];
        REAL gx = 0.0, gy = 0.0, gz = 0.0;
        for (int m = 0; m < 5; m++) {
          gx += fourth[m] * P->phx[pidx(P, i + m - 2, j, k)];
          gy += fourth[m] * P->phy[pidx(P, i, j + m - 2, k)];
          gz += fourth[m] * P->phz[pidx(P, i, j, k + m - 2)];
        }
        gx /= (L(12.0) * dh);
        gy /= (L(12.0) * dh);
        gz /= (L(12.0) * dh);
        REAL t6 = gx + gy + gz;
        pn[I] = t1 + t2 + dt * dt * (t3 + t4 + t5 + t6 + P->force[I]);
        REAL ux = L(0.0), uy = L(0.0), uz = L(0.0);
        for (int m = 0; m < 5; m++) {
          ux += fourth[m] * p[pidx(P, i + m - 2, j, k)];
          uy += fourth[m] * p[pidx(P, i, j + m - 2, k)];
          uz += fourth[m] * p[pidx(P, i, j, k + m - 2)];
        }
        ux /= (L(12.0) * dh);
        uy /= (L(12.0) * dh);
        uz /= (L(12.0) * dh);
        P->phxn[I] = P->phx[I] - dt * zx * P->phx[I] + dt * (zy + zz - zx) * ux;
        P->phyn[I] = P->phy[I] - dt * zy * P->phy[I] + dt * (zx + zz - zy) * uy;
        P->phzn[I] = P->phz[I] - dt * zz * P->phz[I] + dt * (zx + zy - zz) * uz;
      }
  REAL* t;
  t = P->phxn; P->phxn = P->phx; P->phx = t;
  t = P->phyn; P->phyn = P->phy; P->phy = t;
  t = P->phzn; P->phzn = P->phz; P->phz = t;
  t = P->pold; P->pold = P->pcur; P->pcur = P->pnew; P->pnew = t;
  memset(P->force, 0, sizeof(REAL) * (size_t)P->n);
}

static inline REAL get_p(const opart* P, int x, int y, int z) {
  if (P->kind == ARD_PART_DCT) return P->p[(long)z * P->h * P->w + (long)y * P->w + x];
  return P->pcur[pidx(P, x, y, z)];
}
static inline void set_f(opart* P, int x, int y, int z, REAL v) {
  if (P->kind == ARD_PART_DCT) P->f[(long)z * P->h * P->w + (long)y * P->w + x] = v;
  else P->force[pidx(P, x, y, z)] = v;
}

/* Boundary::ComputeForcingTerms (boundary.cpp:21-173).  The three branches
 * differ only in which axis crosses the interface, so one routine walks the
 * face with the crossing axis abstracted. */
static void boundary_forcing(osim* S, const ard_boundary* B) {
  static const REAL C[6][6] = {
      {0.0, 0.0, -2.0, 2.0, 0.0, 0.0},
      {0.0, -2.0, 27.0, -27.0, 2.0, 0.0},
      {-2.0, 27.0, -270.0, 270.0, -27.0, 2.0},
      {2.0, -27.0, 270.0, -270.0, 27.0, -2.0},
      {0.0, 2.0, -27.0, 27.0, -2.0, 0.0},
      {0.0, 0.0, 2.0, -2.0, 0.0, 0.0}};
  opart* A = &S->parts[B->a];
  opart* Bp = &S->parts[B->b];
  opart *lo, *hi;  /* left/top/front and right/bottom/back */
  int u0, u1, v0, v1;
  if (B->type == ARD_BOUNDARY_X) {
    int a_lo = (B->x_start <= A->xs + A->w && B->x_end >= A->xs + A->w);
    lo = a_lo ? A : Bp; hi = a_lo ? Bp : A;
    u0 = B->y_start; u1 = B->y_end; v0 = B->z_start; v1 = B->z_end;
  } else if (B->type == ARD_BOUNDARY_Y) {
    int a_lo = (B->y_start <= A->ys + A->h && B->y_end >= A->ys + A->h);
    lo = a_lo ? A : Bp; hi = a_lo ? Bp : A;
    u0 = B->x_start; u1 = B->x_end; v0 = B->z_start; v1 = B->z_end;
  } else {
    int a_lo = (B->z_start <= A->zs + A->d && B->z_end >= A->zs + A->d);
    lo = a_lo ? A : Bp; hi = a_lo ? Bp : A;
    u0 = B->x_start; u1 = B->x_end; v0 = B->y_start; v1 = B->y_end;
  }
  const REAL c0 = S->c0, dh = S->dh;
  for (int iu = u0; iu < u1; iu++)
    for (int iv = v0; iv < v1; iv++) {
      int lx, ly, lz, hx, hy, hz, lext;
      if (B->type == ARD_BOUNDARY_X) {
        ly = iu - lo->ys; hy = iu - hi->ys; lz = iv - lo->zs; hz = iv - hi->zs; lext = lo->w;
      } else if (B->type == ARD_BOUNDARY_Y) {
        lx = iu - lo->xs; hx = iu - hi->xs; lz = iv - lo->zs; hz = iv - hi->zs; lext = lo->h;
      } else {
        lx = iu - lo->xs; hx = iu - hi->xs; ly = iv - lo->ys; hy = iv - hi->ys; lext = lo->d;
      }
      for (int m = -3; m < 3; m++) {
        REAL sip = 0.0, sip1 = 0.0, sip2 = 0.0, fi = 0.0;
        for (int n = 0; n < 3; n++) {
          int c = lext - 3 + n;
          REAL pv = B->type == ARD_BOUNDARY_X ? get_p(lo, c, ly, lz)
                  : B->type == ARD_BOUNDARY_Y ? get_p(lo, lx, c, lz) : get_p(lo, lx, ly, c);
          sip1 += C[m + 3][n] * pv;
        }
        for (int n = 3; n < 6; n++) {
          int c = n - 3;
          REAL pv = B->type == ARD_BOUNDARY_X ? get_p(hi, c, hy, hz)
                  : B->type == ARD_BOUNDARY_Y ? get_p(hi, hx, c, hz) : get_p(hi, hx, hy, c);
          sip2 += C[m + 3][n] * pv;
        }
        if (m < 0) {
          sip = lo->self_terms ? (sip1 + sip2) : sip2;
          fi = sip * (c0 * c0) / (L(180.0) * dh * dh);
          int c = lext + m;
          if (B->type == ARD_BOUNDARY_X) set_f(lo, c, ly, lz, B->absorption * fi);
          else if (B->type == ARD_BOUNDARY_Y) set_f(lo, lx, c, lz, B->absorption * fi);
          else set_f(lo, lx, ly, c, B->absorption * fi);
        } else {
          sip = hi->self_terms ? (sip1 + sip2) : sip1;
          fi = sip * (c0 * c0) / (L(180.0) * dh * dh);
          if (B->type == ARD_BOUNDARY_X) set_f(hi, m, hy, hz, B->absorption * fi);
          else if (B->type == ARD_BOUNDARY_Y) set_f(hi, hx, m, hz, B->absorption * fi);
          else set_f(hi, hx, hy, m, B->absorption * fi);
        }
      }
    }
}

void API(oracle_step)(void* h, long nsteps) {
  osim* S = (osim*)h;
  for (long s = 0; s < nsteps; ++s) {
    const long t = S->t;
    /* phase A: independent per partition */
#pragma omp parallel for schedule(dynamic, 1)
    for (int i = 0; i < S->np; ++i) {
      opart* P = &S->parts[i];
      if (P->kind == ARD_PART_DCT) {
        for (int k = 0; k < P->nsrc; ++k) {
          const int si = P->src[k];
          const ard_point* q = &S->srcs[si];
          REAL v = (t < S->series_len[si]) ? (REAL)S->series[si][t] : (REAL)0;
          P->f[(long)(q->z - P->zs) * P->h * P->w + (long)(q->y - P->ys) * P->w + (q->x - P->xs)] = v;
        }
        dct_update(S, P);
      } else {
        pml_update(S, P);
      }
    }
    /* phase B: serial, list order => the last interface wins overlaps */
    for (int b = 0; b < S->nb; ++b) boundary_forcing(S, &S->bnd[b]);
    /* recorder samples after the step */
    if (S->nr > 0) {
      if (t >= S->hist_cap) {
        S->hist_cap = S->hist_cap ? 2 * S->hist_cap : 1024;
        S->hist = (REAL*)realloc(S->hist, sizeof(REAL) * (size_t)(S->hist_cap * S->nr));
      }
      for (int r = 0; r < S->nr; ++r) {
        const ard_point* q = &S->recs[r];
        REAL v = 0;
        if (q->partition >= 0) {
          const opart* P = &S->parts[q->partition];
          v = get_p(P, q->x - P->xs, q->y - P->ys, q->z - P->zs);
        }
        S->hist[t * S->nr + r] = v;
      }
    }
    S->t++;
  }
}

long API(oracle_time_step)(void* h) { return ((osim*)h)->t; }

/* out: [t][recorder] for t in [0, time_step) */
void API(oracle_read_recorders)(void* h, double* out) {
  osim* S = (osim*)h;
  for (long i = 0; i < S->t * S->nr; ++i) out[i] = (double)S->hist[i];
}

/* pressure (and force if non-NULL) of partition `part`, [z][y][x] */
void API(oracle_read_field)(void* h, int part, double* pressure, double* force) {
  osim* S = (osim*)h;
  const opart* P = &S->parts[part];
  for (long i = 0; i < P->n; ++i) {
    if (pressure) pressure[i] = (double)(P->kind == ARD_PART_DCT ? P->p[i] : P->pcur[i]);
    if (force) force[i] = (double)(P->kind == ARD_PART_DCT ? P->f[i] : P->force[i]);
  }
}
