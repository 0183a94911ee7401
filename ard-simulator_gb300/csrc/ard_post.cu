// Products around the time step, on the GPU, over a context's own state:
//
//  * neighbourhood recording: Recorder::RecordField's out_<id>.txt stream
//    (ARD-simulator-190113/recorder.cpp:40-57), the 10 x 10 x 10 cube of
//    pressure around every recorder after every step.  The cube is a
//    separable contraction of the partition's modes (the field is never
//    formed): rows along kx onto the cube's 10 x, then ky, then kz, each with
//    the REDFT01 basis, three small launches per air group inside the step;
//  * slice colour map: the visualization block of Simulation::Update
//    (simulation.cpp:320-420) into a caller's device buffer of RGBA8888
//    words instead of an SDL texture;
//  * impulse response and T60: matlab/auralization.m:22-36 (cross-correlation
//    of the response with the reversed source, fir1 low-pass by fftfilt,
//    normalizeIR) and matlab/t60.m (Schroeder integration and line fit), in
//    FP64 on the device over the recorded history and the injected series.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "ard_engine.h"
#include "ard_gb300.h"

namespace ard {

constexpr int kCube = 10;             // cube edge: offsets -5 .. 4 (recorder.cpp:44-52)
constexpr int kCubeCells = kCube * kCube * kCube;
constexpr int kCubeRowBlocks = 64;    // rows of stage 1 per block: 8 warps x 8

template <typename T>
struct CubeArgs {
  const T* buf;
  const DctDev* dct;
  const PointDev* recs;
  int r_lo;              // first recorder of this launch (recorders [r_lo, r_lo + nrec))
  int nrec;
  int par;               // modal level written by this step
  T* tmp;                // per recorder: T1 [d][h][10] at s1 * r, T2 [d][100] at s1 * nrec_total + s2 * r
  long long s1, s2;
  int rows_blocks;       // stage-1 blocks per recorder
  int dmax;              // stage-2 blocks per recorder
  float* hist;           // [max_steps][nrec_total][1000]
  int nrec_total;
  const long long* tcount;
  int tstep;
  long long max_steps;
};

// Stage 1: T1[kz][ky][i] = sum_kx M[kz][ky][kx] Ci(kx, x0 + i), one warp per
// (kz, ky) row of the recorder's partition (Ci^T row x0 + i is contiguous in kx).
template <typename T>
__global__ void __launch_bounds__(256) cube_rows_kernel(CubeArgs<T> a) {
  grid_dependency_wait();
  const int rl = blockIdx.x / a.rows_blocks;
  const int lane = threadIdx.x & 31;
  const PointDev q = a.recs[a.r_lo + rl];
  const DctDev& D = a.dct[q.part];
  const int rows = D.d * D.h;
  const T* ct = a.buf + D.cw + 3LL * D.w * D.w + (long long)(q.x - kCube / 2) * D.w;
  T* t1 = a.tmp + (long long)(a.r_lo + rl) * a.s1;
  const int stride = a.rows_blocks * 8;
  for (int row = (blockIdx.x % a.rows_blocks) * 8 + (threadIdx.x >> 5); row < rows; row += stride) {
    const T* m = a.buf + D.M[a.par] + (long long)row * D.wp;
    T acc[kCube];
#pragma unroll
    for (int i = 0; i < kCube; ++i) acc[i] = 0;
    for (int k = lane; k < D.w; k += 32) {
      const T v = m[k];
#pragma unroll
      for (int i = 0; i < kCube; ++i) acc[i] += v * ct[(long long)i * D.w + k];
    }
    T mine = 0;
#pragma unroll
    for (int i = 0; i < kCube; ++i) {
      const T s = warp_sum(acc[i]);
      if (lane == i) mine = s;
    }
    if (lane < kCube) t1[(long long)row * kCube + lane] = mine;
  }
}

// Stage 2: T2[kz][j][i] = sum_ky T1[kz][ky][i] Ci(ky, y0 + j); block
// (recorder, kz), thread j * 10 + i.
template <typename T>
__global__ void __launch_bounds__(128) cube_cols_kernel(CubeArgs<T> a) {
  grid_dependency_wait();
  const int rl = blockIdx.x / a.dmax, kz = blockIdx.x % a.dmax;
  const PointDev q = a.recs[a.r_lo + rl];
  const DctDev& D = a.dct[q.part];
  const int t = threadIdx.x;
  if (kz >= D.d || t >= kCube * kCube) return;
  const int j = t / kCube, i = t % kCube;
  const T* t1 = a.tmp + (long long)(a.r_lo + rl) * a.s1 + (long long)kz * D.h * kCube;
  const T* ch = a.buf + D.ch + 3LL * D.h * D.h + (long long)(q.y - kCube / 2 + j) * D.h;
  T s = 0;
  for (int ky = 0; ky < D.h; ++ky) s += t1[ky * kCube + i] * ch[ky];
  a.tmp[a.s1 * a.nrec_total + (long long)(a.r_lo + rl) * a.s2 + (long long)kz * kCube * kCube + t] = s;
}

// Stage 3: cube[k][j][i] = s_i sum_kz T2[kz][j][i] Ci(kz, z0 + k) into the
// history row of step t (one block of 1000 threads per recorder).
template <typename T>
__global__ void __launch_bounds__(1024) cube_out_kernel(CubeArgs<T> a) {
  grid_dependency_wait();
  const int rl = blockIdx.x;
  const PointDev q = a.recs[a.r_lo + rl];
  const DctDev& D = a.dct[q.part];
  const int o = threadIdx.x;
  const long long t = *a.tcount + a.tstep;
  if (o >= kCubeCells || t >= a.max_steps) return;
  const int k = o / (kCube * kCube), ji = o % (kCube * kCube);
  const T* t2 = a.tmp + a.s1 * a.nrec_total + (long long)(a.r_lo + rl) * a.s2;
  const T* cd = a.buf + D.cd + 3LL * D.d * D.d + (long long)(q.z - kCube / 2 + k) * D.d;
  T s = 0;
  for (int kz = 0; kz < D.d; ++kz) s += t2[kz * kCube * kCube + ji] * cd[kz];
  a.hist[(t * a.nrec_total + q.slot) * kCubeCells + o] = (float)(s * (T)D.si);
}

template <typename T>
int launch_cubes(Ctx* ctx, cudaStream_t s, int tstep, int par, int r_lo, int r_hi) {
  const int nrec = r_hi - r_lo;
  if (!ctx->d_cube_hist || nrec <= 0) return ARD_OK;
  CubeArgs<T> a{reinterpret_cast<const T*>(ctx->d_buf), ctx->d_dct, ctx->d_recpts, r_lo, nrec, par,
                reinterpret_cast<T*>(ctx->d_cube_tmp), ctx->cube_s1, ctx->cube_s2, ctx->cube_row_blocks,
                ctx->cube_dmax, ctx->d_cube_hist, ctx->n_rec_total, ctx->d_t, tstep, ctx->max_steps};
  ARD_CUDA(launch_dep(cube_rows_kernel<T>, (long long)nrec * a.rows_blocks, 256, 0, s, a));
  ARD_CUDA(launch_dep(cube_cols_kernel<T>, (long long)nrec * a.dmax, 128, 0, s, a));
  ARD_CUDA(launch_dep(cube_out_kernel<T>, nrec, 1024, 0, s, a));
  ARD_CUDA(cudaGetLastError());
  return ARD_OK;
}

template int launch_cubes<float>(Ctx*, cudaStream_t, int, int, int, int);
template int launch_cubes<double>(Ctx*, cudaStream_t, int, int, int, int);

void free_cubes(Ctx* ctx) {
  if (ctx->d_cube_hist) cudaFree(ctx->d_cube_hist);
  if (ctx->d_cube_tmp) cudaFree(ctx->d_cube_tmp);
  ctx->d_cube_hist = nullptr;
  ctx->d_cube_tmp = nullptr;
}

// ---------------------------------------------------------------------------
// slice colour map
// ---------------------------------------------------------------------------

// out[o * oso + c * osc] = scale * sum_{k < K} in[k * isk + c * isc] * tab[k * tk + o * to]
// for o < NO, c < NC (one thread per output, c fastest).
template <typename T>
__global__ void lin_kernel(const T* in, long long isk, long long isc, const T* tab, long long tk, long long to, int K,
                           T* out, long long oso, long long osc, int NO, int NC, T scale) {
  const long long n = (long long)NO * NC;
  for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x; g < n; g += (long long)gridDim.x * blockDim.x) {
    const int o = (int)(g / NC), c = (int)(g % NC);
    T s = 0;
    for (int k = 0; k < K; ++k) s += in[k * isk + c * isc] * tab[k * tk + o * to];
    out[o * oso + c * osc] = s * scale;
  }
}

// The colour of Simulation::Update's visualization (simulation.cpp:349-367)
// as the RGBA8888 word SDL_MapRGBA(fmt, 255, r, g, b) gives: R = 255, G = r,
// B = g, A = b (the reference passes the alpha first).  Float arithmetic in
// the reference's order, every operation rounded on its own.
__device__ __forceinline__ uint32_t slice_colour(float p, float v_coef) {
  const float pv = __fmul_rn(p, v_coef);
  const float cl = fmaxf(-1.0f, fminf(1.0f, pv));
  const float norm = __fadd_rn(__fmul_rn(0.5f, cl), 0.5f);
  int r, g, b;
  if (norm >= 0.5f) {
    const float v = __fmul_rn(510.0f, __fsub_rn(norm, 0.5f));
    r = g = static_cast<int>(255.0 - round((double)v));
    b = 255;
  } else {
    const float v = __fmul_rn(255.0f, __fsub_rn(1.0f, __fmul_rn(2.0f, norm)));
    r = 255;
    g = b = static_cast<int>(255.0 - round((double)v));
  }
  return 0xFF000000u | ((uint32_t)r << 16) | ((uint32_t)g << 8) | (uint32_t)b;
}

struct SliceArgs {
  int kind;              // ARD_PART_DCT: values from `plane` [ni][nj]; ARD_PART_PML: from the slab
  int valid;             // the slice's local coordinate lies inside the partition
  long long plane;       // DCT: pool offset of the slice plane
  long long slab;        // PML: pool offset of p (current level)
  int ptype, A, B;       // PML slab geometry (B: row pitch)
  int look_from, coord;  // view and the local coordinate passed by the reference
  int ni, nj;            // rows / columns of the partition's slice
  int off_i, off_j;      // its offset in the image
  int img_w;             // image row length
  float v_coef;
};

template <typename T>
__global__ void paint_kernel(const T* buf, SliceArgs s, uint32_t* pix, float* pres) {
  const long long n = (long long)s.ni * s.nj;
  for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x; g < n; g += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(g / s.nj), j = (int)(g % s.nj);
    T v = 0;
    if (s.valid) {
      if (s.kind == ARD_PART_DCT) {
        v = buf[s.plane + g];
      } else {
        // local (x, y, z) of the reference's get_pressure call
        const int x = s.look_from == 0 ? j : s.coord;
        const int y = s.look_from == 0 ? i : j;
        const int z = s.look_from == 0 ? s.coord : i;
        const int ax = s.ptype <= 1 ? 0 : (s.ptype <= 3 ? 1 : 2);
        long long idx;
        if (ax == 0) idx = ((long long)x * s.A + z) * s.B + y;
        else if (ax == 1) idx = ((long long)y * s.A + z) * s.B + x;
        else idx = ((long long)z * s.A + y) * s.B + x;
        v = buf[s.slab + idx];
      }
    }
    const float p = (float)v;
    const long long at = (long long)(s.off_i + i) * s.img_w + (s.off_j + j);
    pix[at] = slice_colour(p, s.v_coef);
    if (pres) pres[at] = p;
  }
}

// ---------------------------------------------------------------------------
// impulse response and T60 (FP64)
// ---------------------------------------------------------------------------

// x[i] = sum_{q <= i} rr[i - q] src[q]: the first half of xcorr(rr, reversed
// src) (auralization.m:29-30) is the causal convolution of the two.
__global__ void conv_kernel(const double* rr, const double* src, long long n, long long nsrc, double* x) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    double s = 0;
    const long long qmax = i < nsrc - 1 ? i : nsrc - 1;
    for (long long q = 0; q <= qmax; ++q) s += rr[i - q] * src[q];
    x[i] = s;
  }
}

// fir1(order, wn) (Hamming window, unit DC gain) in one block: ideal low-pass
// wn sinc(wn (k - order/2)) times 0.54 - 0.46 cos(2 pi k / order), scaled so
// that the taps sum to 1.
__global__ void fir1_kernel(int order, double wn, double* b) {
  __shared__ double part[1024];
  const double pi = 3.14159265358979323846;
  double s = 0;
  for (int k = threadIdx.x; k <= order; k += blockDim.x) {
    const double m = k - 0.5 * order;
    const double h = m == 0 ? wn : sin(pi * wn * m) / (pi * m);
    const double w = 0.54 - 0.46 * cos(2.0 * pi * k / order);
    b[k] = h * w;
    s += h * w;
  }
  part[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) part[threadIdx.x] += part[threadIdx.x + o];
    __syncthreads();
  }
  const double tot = part[0];
  for (int k = threadIdx.x; k <= order; k += blockDim.x) b[k] /= tot;
}

// fftfilt(b, x): y[i] = sum_{k <= min(i, L-1)} b[k] x[i - k], length n.
__global__ void fir_kernel(const double* b, int L, const double* x, long long n, double* y) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    double s = 0;
    const int kmax = (int)(i < L - 1 ? i : L - 1);
    for (int k = 0; k <= kmax; ++k) s += b[k] * x[i - k];
    y[i] = s;
  }
}

// Block-wide inclusive prefix sums of v[0..n) in place (one block, 1024 threads,
// contiguous chunks per thread, chunk totals scanned in shared memory).
__device__ void block_scan(double* v, long long n, double* sh) {
  const int t = threadIdx.x, nt = blockDim.x;
  const long long per = (n + nt - 1) / nt;
  const long long lo = t * per, hi = lo + per < n ? lo + per : n;
  double s = 0;
  for (long long i = lo; i < hi; ++i) s += v[i];
  sh[t] = s;
  __syncthreads();
  if (t == 0)
    for (int k = 1; k < nt; ++k) sh[k] += sh[k - 1];
  __syncthreads();
  double run = t > 0 ? sh[t - 1] : 0.0;
  for (long long i = lo; i < hi; ++i) {
    run += v[i];
    v[i] = run;
  }
  __syncthreads();
}

// normalizeIR (normalizeIR.m) then t60.m on the normalized response y[0..n):
// Schroeder's integrated decay over the first T samples, the running r^2 of
// the line fit from sample `begin`, the fit up to the last r^2 maximum.
// w: 6 scratch arrays of n doubles.  out[0] = rt (ms, rounded as t60.m),
// out[1] = the slope (dB/ms), out[2] = stop, out[3] = 1 when t60.m's window
// would have been overrun (stop clamped to T).
__global__ void __launch_bounds__(1024) t60_kernel(double* y, long long n, double sr, double* w, double* out) {
  __shared__ double sh[1024];
  __shared__ double red[1024];
  const int t = threadIdx.x, nt = blockDim.x;
  // normalizeIR: y / max |y|
  double m = 0;
  for (long long i = t; i < n; i += nt) m = fmax(m, fabs(y[i]));
  red[t] = m;
  __syncthreads();
  for (int o = nt / 2; o > 0; o >>= 1) {
    if (t < o) red[t] = fmax(red[t], red[t + o]);
    __syncthreads();
  }
  const double ymax = red[0];
  __syncthreads();
  for (long long i = t; i < n; i += nt) y[i] = ymax > 0 ? y[i] / ymax : y[i];
  __syncthreads();
  const long long begin = llround(sr * 0.05);            // t60.m:41 (1-based sample index)
  const long long T = (double)n / sr < 1.5 ? n : llround(sr * 1.5);
  // iidc: reverse cumulative sum of y^2 (w0 holds it reversed, then scanned)
  double* iidc = w;
  for (long long i = t; i < n; i += nt) iidc[i] = y[n - 1 - i] * y[n - 1 - i];
  __syncthreads();
  block_scan(iidc, n, sh);
  // Y[k] = iidc[n - 1 - k], k < T; ydb = 10 log10(Y / max |Y|)
  double mm = 0;
  for (long long k = t; k < T; k += nt) mm = fmax(mm, fabs(iidc[n - 1 - k]));
  red[t] = mm;
  __syncthreads();
  for (int o = nt / 2; o > 0; o >>= 1) {
    if (t < o) red[t] = fmax(red[t], red[t + o]);
    __syncthreads();
  }
  const double Ymax = red[0];
  __syncthreads();
  double *cx = w + n, *cy = w + 2 * n, *cxy = w + 3 * n, *cx2 = w + 4 * n, *cy2 = w + 5 * n;
  const double x1 = (double)T / (sr / 1000.0);            // linspace(1, T / (sr / 1000), T)
  for (long long k = t; k < T; k += nt) {
    const double yv = 10.0 * log10(iidc[n - 1 - k] / Ymax);
    const double xv = T > 1 ? 1.0 + (double)k * (x1 - 1.0) / (double)(T - 1) : x1;
    cx[k] = xv; cy[k] = yv; cxy[k] = xv * yv; cx2[k] = xv * xv; cy2[k] = yv * yv;
  }
  __syncthreads();
  block_scan(cx, T, sh);
  block_scan(cy, T, sh);
  block_scan(cxy, T, sh);
  block_scan(cx2, T, sh);
  block_scan(cy2, T, sh);
  // r2 over k = begin-1 .. T-1 (0-based); the last index of the maximum
  double best = -INFINITY;
  long long arg = -1;
  for (long long k = begin - 1 + t; k < T; k += nt) {
    if (k < 0) continue;
    const double s = (double)(k + 1);
    const double e = cxy[k] - cx[k] * cy[k] / s;
    const double exy2 = e * e;
    const double ex2 = cx2[k] - cx[k] * cx[k] / s;
    const double tot = cy2[k] - cy[k] * cy[k] / s;
    const double r2 = exy2 / ex2 / tot;
    if (r2 >= best) { best = r2; arg = k; }   // k increases: the last maximum of this thread
  }
  red[t] = best;
  sh[t] = (double)arg;
  __syncthreads();
  if (t == 0) {
    double b = -INFINITY;
    long long a = -1;
    for (int i = 0; i < nt; ++i)
      if (sh[i] >= 0 && (red[i] > b || (red[i] == b && (long long)sh[i] > a))) { b = red[i]; a = (long long)sh[i]; }
    // r3 (1-based position in r2) = a - (begin - 1) + 1; stop = begin + r3
    long long stop = a < 0 ? T : begin + (a - (begin - 1) + 1);
    const double overrun = stop > T ? 1.0 : 0.0;
    if (stop > T) stop = T;
    const long long e = stop - 1;
    const double S = (double)stop;
    const double mx = cx[e] / S, my = cy[e] / S, mx2 = cx2[e] / S, my2 = cy2[e] / S, mxy = cxy[e] / S;
    const double sdx = sqrt(mx2 - mx * mx), sdy = sqrt(my2 - my * my);
    const double r = (mxy - mx * my) / (sdx * sdy);
    const double slope = r * sdy / sdx;
    const double yint = -(slope * mx) + my;
    out[0] = round(fabs(60.0 / slope) - yint);
    out[1] = slope;
    out[2] = (double)stop;
    out[3] = overrun;
  }
}

}  // namespace ard

using namespace ard;

static Ctx* post_ctx(ard_ctx* c) { return reinterpret_cast<Ctx*>(c); }

extern "C" int ard_record_neighbourhoods(ard_ctx* c, int32_t enable) {
  if (!c) return ARD_ERR_INVALID;
  Ctx* ctx = post_ctx(c);
  ARD_CUDA(cudaSetDevice(ctx->device));
  ARD_CUDA(cudaStreamSynchronize(ctx->stream));
  ARD_CUDA(cudaStreamSynchronize(ctx->stream2));
  if (ctx->graph_exec) {   // the step graph is captured again with (or without) the cube launches
    cudaGraphExecDestroy(ctx->graph_exec);
    ctx->graph_exec = nullptr;
  }
  free_cubes(ctx);
  if (!enable) return ARD_OK;
  if (ctx->recpts.empty()) { ctx->err = "ard_record_neighbourhoods: the context has no recorders"; return ARD_ERR_STATE; }
  long long rows = 1, dmax = 1;
  for (const PointDev& q : ctx->recpts) {
    if (q.part < 0 || q.part >= (int)ctx->dct.size()) { ctx->err = "ard_record_neighbourhoods: a recorder has no air partition"; return ARD_ERR_INVALID; }
    const DctDev& D = ctx->dct[q.part];
    const int h = kCube / 2;
    if (q.x - h < 0 || q.x + h > D.w || q.y - h < 0 || q.y + h > D.h || q.z - h < 0 || q.z + h > D.d) {
      ctx->err = "ard_record_neighbourhoods: a recorder's 10x10x10 neighbourhood leaves its partition "
                 "(Recorder::FindPartition's margin)";
      return ARD_ERR_INVALID;
    }
    rows = std::max(rows, (long long)D.d * D.h);
    dmax = std::max(dmax, (long long)D.d);
  }
  const int nr = ctx->n_rec_total;
  ctx->cube_s1 = rows * kCube;
  ctx->cube_s2 = dmax * kCube * kCube;
  ctx->cube_row_blocks = (int)std::max(1LL, (rows + kCubeRowBlocks - 1) / kCubeRowBlocks);
  ctx->cube_dmax = (int)dmax;
  const size_t es = elem_size(ctx);
  const size_t hist_bytes = sizeof(float) * (size_t)ctx->max_steps * nr * kCubeCells;
  const size_t tmp_bytes = es * (size_t)nr * (ctx->cube_s1 + ctx->cube_s2);
  if (cudaMalloc(&ctx->d_cube_hist, hist_bytes) != cudaSuccess ||
      cudaMalloc(&ctx->d_cube_tmp, tmp_bytes) != cudaSuccess) {
    cudaGetLastError();
    free_cubes(ctx);
    ctx->err = "ard_record_neighbourhoods: out of device memory for the neighbourhood history";
    return ARD_ERR_OOM;
  }
  ARD_CUDA(cudaMemset(ctx->d_cube_hist, 0, hist_bytes));
  ctx->cube_t0 = ctx->t_host;
  return ARD_OK;
}

extern "C" int ard_read_neighbourhoods(ard_ctx* c, int32_t scene, float* out, int64_t t0, int64_t nt) {
  if (!c || (nt > 0 && !out)) return ARD_ERR_INVALID;
  Ctx* ctx = post_ctx(c);
  if (!ctx->d_cube_hist) { ctx->err = "neighbourhoods are not recorded (ard_record_neighbourhoods)"; return ARD_ERR_STATE; }
  if (scene < -1 || scene >= (int)ctx->scenes.size()) { ctx->err = "bad scene index"; return ARD_ERR_RANGE; }
  if (t0 < ctx->cube_t0 || nt < 0 || t0 + nt > ctx->t_host || t0 + nt > ctx->max_steps) {
    ctx->err = "neighbourhood time range not recorded";
    return ARD_ERR_RANGE;
  }
  const int rec0 = scene < 0 ? 0 : ctx->scenes[scene].rec0;
  const int nrec = scene < 0 ? ctx->n_rec_total : ctx->scenes[scene].nrec;
  if (nrec == 0 || nt == 0) return ARD_OK;
  ARD_CUDA(cudaSetDevice(ctx->device));
  ARD_CUDA(cudaStreamSynchronize(ctx->stream));
  const size_t row = sizeof(float) * kCubeCells;
  ARD_CUDA(cudaMemcpy2D(out, row * nrec, ctx->d_cube_hist + ((size_t)t0 * ctx->n_rec_total + rec0) * kCubeCells,
                        row * ctx->n_rec_total, row * nrec, nt, cudaMemcpyDeviceToHost));
  return ARD_OK;
}

// bounding box of a scene's partitions (Simulation::Simulation, simulation.cpp:272-288)
static void scene_box(const SceneRec& s, int lo[3], int hi[3]) {
  for (int a = 0; a < 3; ++a) { lo[a] = 2147483647; hi[a] = -2147483647 - 1; }
  for (const ard_partition& p : s.parts) {
    const int st[3] = {p.x_start, p.y_start, p.z_start}, ext[3] = {p.width, p.height, p.depth};
    for (int a = 0; a < 3; ++a) {
      lo[a] = std::min(lo[a], st[a]);
      hi[a] = std::max(hi[a], st[a] + ext[a]);
    }
  }
}

extern "C" int ard_slice_size(ard_ctx* c, int32_t scene, int32_t look_from, int32_t* width, int32_t* height) {
  if (!c || !width || !height) return ARD_ERR_INVALID;
  Ctx* ctx = post_ctx(c);
  if (scene < 0 || scene >= (int)ctx->scenes.size()) { ctx->err = "bad scene index"; return ARD_ERR_RANGE; }
  if (look_from != 0 && look_from != 1) { ctx->err = "look_from must be 0 (xy) or 1 (yz)"; return ARD_ERR_INVALID; }
  int lo[3], hi[3];
  scene_box(ctx->scenes[scene], lo, hi);
  *width = look_from == 0 ? hi[0] - lo[0] : hi[1] - lo[1];
  *height = look_from == 0 ? hi[1] - lo[1] : hi[2] - lo[2];
  return ARD_OK;
}

template <typename T>
static int render_slice(Ctx* ctx, int scene, int look_from, int coord, float v_coef, uint32_t* pix, float* pres) {
  T* buf = reinterpret_cast<T*>(ctx->d_buf);
  const SceneRec& sr = ctx->scenes[scene];
  int lo[3], hi[3];
  scene_box(sr, lo, hi);
  const int img_w = look_from == 0 ? hi[0] - lo[0] : hi[1] - lo[1];
  const int lvl = (int)((ctx->t_host - 1) & 1);   // buffer holding the latest level
  const int blocks = ctx->num_sms * 4;
  auto cos_tab = [&](int n) -> long long {
    for (auto& kv : ctx->cos_tables)
      if (kv.first == n) return kv.second;
    return -1;
  };
  for (size_t pi = 0; pi < sr.parts.size(); ++pi) {   // list order: later partitions overwrite earlier ones
    const ard_partition& p = sr.parts[pi];
    // simulation.cpp:336,382: skip partitions that do not reach the slice (end inclusive)
    if (look_from == 0 && (p.z_start > coord || p.z_start + p.depth < coord)) continue;
    if (look_from == 1 && (p.x_start > coord || p.x_start + p.width < coord)) continue;
    SliceArgs s{};
    s.kind = p.kind;
    s.look_from = look_from;
    s.coord = coord;   // passed to the partition as a local coordinate, as get_xy_plane / get_yz_plane get it
    s.ni = look_from == 0 ? p.height : p.depth;
    s.nj = look_from == 0 ? p.width : p.height;
    s.off_i = look_from == 0 ? p.y_start - lo[1] : p.z_start - lo[2];
    s.off_j = look_from == 0 ? p.x_start - lo[0] : p.y_start - lo[1];
    s.img_w = img_w;
    s.v_coef = v_coef;
    const int ext = look_from == 0 ? p.depth : p.width;
    s.valid = coord >= 0 && coord < ext;
    const int idx = sr.engine_idx[pi];
    if (p.kind == ARD_PART_DCT) {
      const DctDev& D = ctx->dct[idx];
      const long long N = (long long)D.w * D.h * D.d;
      const long long A = ctx->scratch, B = ctx->scratch + N, P = ctx->scratch + 2 * N;
      const long long cw = cos_tab(D.w) + (long long)D.w * D.w, ch = cos_tab(D.h) + (long long)D.h * D.h,
                      cd = cos_tab(D.d) + (long long)D.d * D.d;   // Ci[k][j] of each extent
      const T* M = buf + D.M[lvl];
      if (s.valid && look_from == 0) {
        // A[ky][kx] = sum_kz M[kz][ky][kx] Ci(kz, z); B[ky][x] = sum_kx A Ci(kx, x); P[y][x] = s_i sum_ky B Ci(ky, y)
        lin_kernel<T><<<blocks, 256, 0, ctx->stream>>>(M, (long long)D.h * D.wp, 1, buf + cd + coord, D.d, 0, D.d,
                                                       buf + A, 0, 1, 1, D.h * D.wp, (T)1);
        lin_kernel<T><<<blocks, 256, 0, ctx->stream>>>(buf + A, 1, D.wp, buf + cw, D.w, 1, D.w, buf + B, 1, D.w, D.w,
                                                       D.h, (T)1);
        lin_kernel<T><<<blocks, 256, 0, ctx->stream>>>(buf + B, D.w, 1, buf + ch, D.h, 1, D.h, buf + P, D.w, 1, D.h,
                                                       D.w, (T)D.si);
      } else if (s.valid) {
        // A[kz][ky] = sum_kx M[kz][ky][kx] Ci(kx, x); B[kz][y] = sum_ky A Ci(ky, y); P[z][y] = s_i sum_kz B Ci(kz, z)
        lin_kernel<T><<<blocks, 256, 0, ctx->stream>>>(M, 1, D.wp, buf + cw + coord, D.w, 0, D.w, buf + A, 0, 1, 1,
                                                       D.d * D.h, (T)1);
        lin_kernel<T><<<blocks, 256, 0, ctx->stream>>>(buf + A, 1, D.h, buf + ch, D.h, 1, D.h, buf + B, 1, D.h, D.h,
                                                       D.d, (T)1);
        lin_kernel<T><<<blocks, 256, 0, ctx->stream>>>(buf + B, D.h, 1, buf + cd, D.d, 1, D.d, buf + P, D.h, 1, D.d,
                                                       D.h, (T)D.si);
      }
      s.plane = P;
    } else {
      const PmlDev& Q = ctx->pml[idx];
      s.slab = Q.p[lvl];
      s.ptype = Q.type;
      s.A = Q.A;
      s.B = Q.Bp;   // row pitch; out of range: PmlPartition::GetIndex's zero sentinel
    }
    ARD_CUDA(cudaGetLastError());
    paint_kernel<T><<<blocks, 256, 0, ctx->stream>>>(buf, s, pix, pres);
    ARD_CUDA(cudaGetLastError());
  }
  ARD_CUDA(cudaStreamSynchronize(ctx->stream));
  return ARD_OK;
}

extern "C" int ard_render_slice(ard_ctx* c, int32_t scene, int32_t look_from, int32_t coord, float v_coef,
                                uint32_t* pixels_device, float* pressure_device) {
  if (!c || !pixels_device) return ARD_ERR_INVALID;
  Ctx* ctx = post_ctx(c);
  int w, h;
  if (int rc = ard_slice_size(c, scene, look_from, &w, &h)) return rc;
  ARD_CUDA(cudaSetDevice(ctx->device));
  ARD_CUDA(cudaStreamSynchronize(ctx->stream));
  ARD_CUDA(cudaStreamSynchronize(ctx->stream2));
  return ctx->prec == ARD_PREC_F64 ? render_slice<double>(ctx, scene, look_from, coord, v_coef, pixels_device, pressure_device)
                                   : render_slice<float>(ctx, scene, look_from, coord, v_coef, pixels_device, pressure_device);
}

extern "C" int ard_impulse_response(ard_ctx* c, int32_t scene, int32_t recorder, int32_t source, int64_t nt,
                                    int64_t truncate, double sample_rate, double fcut, int32_t fir_order,
                                    double* rir_out, double* t60_out) {
  if (!c) return ARD_ERR_INVALID;
  Ctx* ctx = post_ctx(c);
  if (scene < 0 || scene >= (int)ctx->scenes.size()) { ctx->err = "bad scene index"; return ARD_ERR_RANGE; }
  const SceneRec& sr = ctx->scenes[scene];
  if (recorder < 0 || recorder >= sr.nrec || source < 0 || source >= sr.nsrc) {
    ctx->err = "ard_impulse_response: bad recorder or source index";
    return ARD_ERR_RANGE;
  }
  if (nt < 2 || nt > ctx->t_host || nt > ctx->max_steps) { ctx->err = "ard_impulse_response: steps not recorded"; return ARD_ERR_RANGE; }
  if (fir_order < 2 || fir_order % 2 || fir_order > 8192) { ctx->err = "ard_impulse_response: fir_order must be even, 2 .. 8192"; return ARD_ERR_INVALID; }
  const double sr_hz = sample_rate > 0 ? sample_rate : 1.0 / ctx->dt;
  const double wn = fcut / (sr_hz / 2);
  if (!(wn > 0 && wn < 1)) { ctx->err = "ard_impulse_response: fcut must lie between 0 and the Nyquist rate"; return ARD_ERR_INVALID; }
  ARD_CUDA(cudaSetDevice(ctx->device));
  ARD_CUDA(cudaStreamSynchronize(ctx->stream));
  if (int rc = check_device_error(ctx)) return rc;
  const long long n = nt;
  // device work arrays: rr, src, x, b, y, 6 x n for t60, out[4]
  double* d = nullptr;
  const size_t count = (size_t)n * 10 + (size_t)fir_order + 1 + 4;
  if (cudaMalloc(&d, sizeof(double) * count) != cudaSuccess) {
    cudaGetLastError();
    ctx->err = "ard_impulse_response: out of device memory";
    return ARD_ERR_OOM;
  }
  double *rr = d, *src = d + n, *x = d + 2 * n, *y = d + 3 * n, *w = d + 4 * n, *b = d + 10 * n,
         *out = b + fir_order + 1;
  int rc = ARD_OK;
  auto chk = [&](cudaError_t e) {
    if (e != cudaSuccess && rc == ARD_OK) {
      ctx->err = std::string("ard_impulse_response: ") + cudaGetErrorString(e);
      rc = ARD_ERR_CUDA;
    }
  };
  // the recorded response (history column) and the injected series (float -> double)
  chk(cudaMemcpy2DAsync(rr, sizeof(double), ctx->d_hist + sr.rec0 + recorder, sizeof(double) * ctx->n_rec_total,
                        sizeof(double), n, cudaMemcpyDeviceToDevice, ctx->stream));
  std::vector<float> hs(n);
  chk(cudaMemcpy(hs.data(), ctx->d_series + (size_t)(sr.src0 + source) * ctx->max_steps, sizeof(float) * n,
                 cudaMemcpyDeviceToHost));
  std::vector<double> hd(hs.begin(), hs.end());
  chk(cudaMemcpy(src, hd.data(), sizeof(double) * n, cudaMemcpyHostToDevice));
  if (truncate > 0 && truncate < n) chk(cudaMemsetAsync(rr + truncate, 0, sizeof(double) * (n - truncate), ctx->stream));
  const int blocks = ctx->num_sms * 4;
  if (rc == ARD_OK) {
    conv_kernel<<<blocks, 256, 0, ctx->stream>>>(rr, src, n, n, x);
    fir1_kernel<<<1, 1024, 0, ctx->stream>>>(fir_order, wn, b);
    fir_kernel<<<blocks, 256, 0, ctx->stream>>>(b, fir_order + 1, x, n, y);
    t60_kernel<<<1, 1024, 0, ctx->stream>>>(y, n, sr_hz, w, out);
    chk(cudaGetLastError());
  }
  double res[4] = {0, 0, 0, 0};
  // the context's stream does not synchronise with the legacy default stream: copy on it, then wait
  if (rc == ARD_OK && rir_out)
    chk(cudaMemcpyAsync(rir_out, y, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
  if (rc == ARD_OK) chk(cudaMemcpyAsync(res, out, sizeof(res), cudaMemcpyDeviceToHost, ctx->stream));
  chk(cudaStreamSynchronize(ctx->stream));
  cudaFree(d);
  if (rc == ARD_OK && t60_out) {
    t60_out[0] = res[0];
    t60_out[1] = res[1];
    t60_out[2] = res[2];
    t60_out[3] = res[3];
  }
  return rc;
}
