// sm_103a kernels of the ARD time step.  Templated on the working type T
// (float: the product path; double: the FP64 GPU oracle).
//
// Per step (t, parity par = t & 1):
//   xform_rows / xform_cols   forward 2D DCT-II of the 18 force face layers
//   modal_kernel              F = expansion of the face transforms (+ point
//                             sources); M(t) = a (2 cwt M(t-1) - M(t-2) + psi F);
//                             contraction of M(t) onto the face rows and the
//                             recorder cells
//   recorder_kernel           recorder samples of step t
//   xform_cols / xform_rows   inverse 2D transforms -> pressure face layers
//   pml_kernel                Grote-Sim PML update of every slab
//   iface_kernel              6th-order interface forcing into the force
//                             face layers / PML strips (owner masks resolve
//                             overlapping strips in reference list order)
#pragma once

#include <cuda_runtime.h>

#include "ard_device.cuh"

namespace ard {

// Face layer (0..5) of coordinate c in an extent-n axis, -1 if not on the shell.
__host__ __device__ inline int face_layer(int c, int n) {
  return c < 3 ? c : (c >= n - 3 ? c - (n - 6) : -1);
}

// Offset of the force value of local cell (x, y, z) in the shell layers of D
// (X layers own x on the shell, then Y layers, then Z layers); -1 inside.
__host__ __device__ inline long long shell_index(const DctDev& D, int x, int y, int z) {
  int l = face_layer(x, D.w);
  if (l >= 0) return D.fX + ((long long)l * D.d + z) * D.h + y;
  l = face_layer(y, D.h);
  if (l >= 0) return D.fY + ((long long)l * D.d + z) * D.w + x;
  l = face_layer(z, D.d);
  if (l >= 0) return D.fZ + ((long long)l * D.h + y) * D.w + x;
  return -1;
}

__device__ __forceinline__ int find_job(const XformJob* __restrict__ jobs, int njobs, int unit) {
  int lo = 0, hi = njobs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (jobs[mid].first <= unit) lo = mid; else hi = mid - 1;
  }
  return lo;
}

template <typename T>
__device__ __forceinline__ T job_input(const T* __restrict__ buf, const XformJob& J, long long off) {
  T v = 0;
  for (int b = 0; b < J.nparts; ++b) {
    const long long o = (long long)b * J.part_stride + off;
    v += buf[J.in0 + o];
    if (J.in1 >= 0) v += (T)J.sgn * buf[J.in1 + o];
  }
  return v;
}

// Rows mode: one warp per line; the line is staged in shared memory.
// Forward jobs point ctab at C (transpose at ctab + n*n); inverse jobs point
// it at the REDFT01 matrix Ci[k][j].
template <typename T>
__global__ void __launch_bounds__(256) xform_rows_kernel(T* __restrict__ buf, const XformJob* __restrict__ jobs,
                                                          int njobs, int total, int maxn) {
  extern __shared__ unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  T* row = reinterpret_cast<T*>(smem_raw) + (long long)warp * maxn;
  for (int unit = blockIdx.x * nwarps + warp; unit < total; unit += gridDim.x * nwarps) {
    const XformJob J = jobs[find_job(jobs, njobs, unit)];
    const int line = unit - J.first;
    const int n = J.n;
    const long long lbase = (long long)line * n;
    for (int j = lane; j < n; j += 32) row[j] = job_input(buf, J, lbase + j);
    __syncwarp();
    const T scale = (T)J.scale;
    const T* C = buf + J.ctab;
    if (!J.inverse) {
      const T* Ct = C + (long long)n * n;
      for (int k = lane; k < n; k += 32) {
        T acc = 0;
        for (int j = 0; j < n; ++j) acc += Ct[(long long)j * n + k] * row[j];
        buf[J.out + lbase + k] = acc * scale;
      }
    } else {
      for (int j = lane; j < n; j += 32) {
        T acc = 0;
        for (int k = 0; k < n; ++k) acc += C[(long long)k * n + j] * row[k];
        buf[J.out + lbase + j] = acc * scale;
      }
    }
    __syncwarp();
  }
}

// Cols mode: one block per 32-column tile; the [n][32] tile is staged in
// shared memory (row pitch 33), warps split the outputs.
template <typename T>
__global__ void __launch_bounds__(256) xform_cols_kernel(T* __restrict__ buf, const XformJob* __restrict__ jobs,
                                                          int njobs, int total) {
  extern __shared__ unsigned char smem_raw[];
  T* tile = reinterpret_cast<T*>(smem_raw);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  for (int unit = blockIdx.x; unit < total; unit += gridDim.x) {
    const XformJob J = jobs[find_job(jobs, njobs, unit)];
    const int col = (unit - J.first) * 32 + lane;
    const bool act = col < J.batch;
    const int n = J.n;
    for (int j = warp; j < n; j += nwarps)
      tile[j * 33 + lane] = act ? job_input(buf, J, (long long)j * J.batch + col) : (T)0;
    __syncthreads();
    const T scale = (T)J.scale;
    const T* C = buf + J.ctab;
    for (int o = warp; o < n; o += nwarps) {
      T acc = 0;
      if (!J.inverse) {
        const T* Crow = C + (long long)o * n;
        for (int j = 0; j < n; ++j) acc += Crow[j] * tile[j * 33 + lane];
      } else {
        for (int k = 0; k < n; ++k) acc += C[(long long)k * n + o] * tile[k * 33 + lane];
      }
      if (act) buf[J.out + (long long)o * J.batch + col] = acc * scale;
    }
    __syncthreads();
  }
}

template <typename T>
struct ModalArgs {
  T* buf;
  const DctDev* dct;
  const int4* tiles;       // {air partition, kx chunk, ky block, kz block}
  int ntiles;
  const PointDev* srcs;
  const PointDev* recs;
  const float* series;     // [n_sources][max_steps]
  long long max_steps;
  const long long* tcount; // steps completed before the current graph launch
  int tstep;               // step offset inside the launch
  int par;
};

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// One warp per tile of 32 kx x kModalTY ky x TZ kz modes.  REF selects the
// reference's arithmetic (tables cos, w^2) over the accurate one (1-cos, psi).
template <typename T, bool REF>
__global__ void __launch_bounds__(128) modal_kernel(ModalArgs<T> a) {
  constexpr int TY = kModalTY;
  const int lane = threadIdx.x & 31;
  const int tile_id = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (tile_id >= a.ntiles) return;
  const int4 tl = a.tiles[tile_id];
  const DctDev& D = a.dct[tl.x];
  const int w = D.w, h = D.h, d = D.d;
  const int kx = tl.y * 32 + lane;
  const bool act = kx < w;
  const int kxc = act ? kx : w - 1;
  const int px = kx & 1;
  T* __restrict__ buf = a.buf;
  const T* Cw = buf + D.cw;
  const T* Ch = buf + D.ch;
  const T* Cd = buf + D.cd;
  // REDFT10 row kx for the expansion; REDFT01 weights (k = 0 halved) for the contraction
  T cx[3], cxi[3];
#pragma unroll
  for (int n = 0; n < 3; ++n) {
    cx[n] = Cw[(long long)kxc * w + n];
    cxi[n] = kx == 0 ? (T)0.5 * cx[n] : cx[n];
  }
  const int ky0 = tl.z * TY;
  const int nky = min(TY, h - ky0);
  const int kz0 = tl.w * D.TZ;
  const int kz1 = min(kz0 + D.TZ, d);
  const T* Mcur = buf + D.M[a.par ^ 1];   // M(t-1)
  T* Mout = buf + D.M[a.par];             // holds M(t-2); receives M(t)
  const T* tabA = buf + D.tabA;
  const T* tabB = buf + D.tabB;
  const T* PX = buf + D.PX;
  const T* PY = buf + D.PY;
  const T* PZ = buf + D.PZ;
  const long long planeZ = (long long)h * w, planeY = (long long)d * w, planeX = (long long)d * h;

  T pz[TY][2][3], rz[TY][2][3];
#pragma unroll
  for (int i = 0; i < TY; ++i)
#pragma unroll
    for (int pm = 0; pm < 2; ++pm)
#pragma unroll
      for (int n = 0; n < 3; ++n) {
        pz[i][pm][n] = (i < nky && act) ? PZ[(pm * 3 + n) * planeZ + (long long)(ky0 + i) * w + kx] : (T)0;
        rz[i][pm][n] = 0;
      }

  const long long t = *a.tcount + a.tstep;
  T sx[kMaxPointsPerPart];
  int sy[kMaxPointsPerPart], sz[kMaxPointsPerPart];
  const int nsrc = D.nsrc;
#pragma unroll
  for (int s = 0; s < kMaxPointsPerPart; ++s) {
    sx[s] = 0; sy[s] = 0; sz[s] = 0;
    if (s < nsrc) {
      const PointDev q = a.srcs[D.src0 + s];
      const float v = (t < a.max_steps) ? a.series[(long long)q.slot * a.max_steps + t] : 0.0f;
      sx[s] = (T)D.sf * (T)v * Cw[(long long)kxc * w + q.x];
      sy[s] = q.y; sz[s] = q.z;
    }
  }
  T rxc[kMaxPointsPerPart], racc[kMaxPointsPerPart];
  int ry_[kMaxPointsPerPart], rz_[kMaxPointsPerPart];
  const int nrec = D.nrec;
#pragma unroll
  for (int r = 0; r < kMaxPointsPerPart; ++r) {
    rxc[r] = 0; racc[r] = 0; ry_[r] = 0; rz_[r] = 0;
    if (r < nrec) {
      const PointDev q = a.recs[D.rec0 + r];
      rxc[r] = act ? (kx == 0 ? (T)0.5 : (T)1) * Cw[(long long)kxc * w + q.x] : (T)0;
      ry_[r] = q.y; rz_[r] = q.z;
    }
  }

  for (int kz = kz0; kz < kz1; ++kz) {
    const int pzr = kz & 1;
    T cz[3], czi[3], py[2][3], ry[2][3];
#pragma unroll
    for (int n = 0; n < 3; ++n) {
      cz[n] = Cd[(long long)kz * d + n];
      czi[n] = kz == 0 ? (T)0.5 * cz[n] : cz[n];
    }
#pragma unroll
    for (int pm = 0; pm < 2; ++pm)
#pragma unroll
      for (int n = 0; n < 3; ++n) {
        py[pm][n] = act ? PY[(pm * 3 + n) * planeY + (long long)kz * w + kx] : (T)0;
        ry[pm][n] = 0;
      }
#pragma unroll
    for (int i = 0; i < TY; ++i) {
      if (i < nky) {
        const int ky = ky0 + i;
        const int pyr = ky & 1;
        T cy[3];
#pragma unroll
        for (int n = 0; n < 3; ++n) cy[n] = Ch[(long long)ky * h + n];
        T F = 0;
#pragma unroll
        for (int n = 0; n < 3; ++n) F += cx[n] * PX[(px * 3 + n) * planeX + (long long)kz * h + ky];
#pragma unroll
        for (int n = 0; n < 3; ++n) F += cy[n] * py[pyr][n];
#pragma unroll
        for (int n = 0; n < 3; ++n) F += cz[n] * pz[i][pzr][n];
#pragma unroll
        for (int s = 0; s < kMaxPointsPerPart; ++s)
          if (s < nsrc) F += sx[s] * (Ch[(long long)ky * h + sy[s]] * Cd[(long long)kz * d + sz[s]]);
        const long long idx = ((long long)kz * h + ky) * w + kxc;
        T Mn = 0;
        if (act) {
          const T m = Mcur[idx], mp = Mout[idx], ta = tabA[idx], tb = tabB[idx];
          if (REF)  // dct_partition.cpp:68: a (2 M cwt - M_prev + (2 F / w2) (1 - cwt))
            Mn = (T)D.damping * ((T)2 * m * ta - mp + ((T)2 * F / tb) * ((T)1 - ta));
          else      // same recurrence with ta = 1 - cwt and tb = 2 (1 - cwt) / w2
            Mn = (T)D.damping * (((T)2 * m - mp) - (T)2 * ta * m + tb * F);
          Mout[idx] = Mn;
        }
        const T wy = ky == 0 ? (T)0.5 : (T)1;
#pragma unroll
        for (int n = 0; n < 3; ++n) {
          rz[i][pzr][n] += czi[n] * Mn;
          ry[pyr][n] += wy * cy[n] * Mn;
        }
        T v[6];
#pragma unroll
        for (int n = 0; n < 3; ++n) {
          const T c = cxi[n] * Mn;
          v[n] = px ? (T)0 : c;
          v[3 + n] = px ? c : (T)0;
        }
#pragma unroll
        for (int q = 0; q < 6; ++q) v[q] = warp_sum(v[q]);
        if (lane < 6) {
          T val = v[0];
#pragma unroll
          for (int q = 1; q < 6; ++q) if (lane == q) val = v[q];
          // RX[bx][pm][n][kz][ky], lane = pm*3 + n
          buf[D.RX + ((long long)tl.y * 6 + lane) * planeX + (long long)kz * h + ky] = val;
        }
#pragma unroll
        for (int r = 0; r < kMaxPointsPerPart; ++r)
          if (r < nrec)
            racc[r] += rxc[r] * (wy * Ch[(long long)ky * h + ry_[r]] * ((kz == 0 ? (T)0.5 : (T)1) * Cd[(long long)kz * d + rz_[r]])) * Mn;
      }
    }
    if (act) {
#pragma unroll
      for (int pm = 0; pm < 2; ++pm)
#pragma unroll
        for (int n = 0; n < 3; ++n)
          buf[D.RY + ((long long)tl.z * 6 + pm * 3 + n) * planeY + (long long)kz * w + kx] = ry[pm][n];
    }
  }
  if (act) {
#pragma unroll
    for (int i = 0; i < TY; ++i)
      if (i < nky)
#pragma unroll
        for (int pm = 0; pm < 2; ++pm)
#pragma unroll
          for (int n = 0; n < 3; ++n)
            buf[D.RZ + ((long long)tl.w * 6 + pm * 3 + n) * planeZ + (long long)(ky0 + i) * w + kx] = rz[i][pm][n];
  }
  if (nrec > 0) {
    const int local = (tl.y * D.nby + tl.z) * D.nbz + tl.w;
#pragma unroll
    for (int r = 0; r < kMaxPointsPerPart; ++r) {
      if (r < nrec) {
        const T s = warp_sum(racc[r]);
        if (lane == 0) buf[D.recpart + (long long)local * nrec + r] = s;
      }
    }
  }
}

// Recorder samples of the current step: sum of the modal tiles' partials.
template <typename T>
__global__ void recorder_kernel(const T* __restrict__ buf, const DctDev* __restrict__ dct, const PointDev* __restrict__ recs,
                                int nrec_total, double* __restrict__ hist, const long long* tcount, int tstep,
                                long long max_steps) {
  const int lane = threadIdx.x & 31;
  const int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (r >= nrec_total) return;
  const PointDev q = recs[r];
  const DctDev& D = dct[q.part];
  const int local_r = r - D.rec0;
  const int ntiles = D.nbx * D.nby * D.nbz;
  T s = 0;
  for (int i = lane; i < ntiles; i += 32) s += buf[D.recpart + (long long)i * D.nrec + local_r];
  s = warp_sum(s);
  const long long t = *tcount + tstep;
  if (lane == 0 && t < max_steps) hist[t * nrec_total + q.slot] = (double)(s * (T)D.si);
}

template <typename T>
struct PmlArgs {
  T* buf;
  const PmlDev* pml;
  const long long* start;  // first cell of each slab (prefix)
  int npml;
  long long total;
  int par;
  T dt, dh, c0;
};

// Grote-Sim PML (pml_partition.cpp:113-200) in slab coordinates: layer l
// along the normal, (a, b) in the plane.  Only the normal damping zeta_n is
// non-zero in a slab, so zeta_a = zeta_b = 0 in the reference's formulas.
template <typename T>
__global__ void __launch_bounds__(256) pml_kernel(PmlArgs<T> a) {
  const T c7[7] = {2, -27, 270, -490, 270, -27, 2};
  const T c5[5] = {1, -8, 0, 8, -1};
  for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x; g < a.total;
       g += (long long)gridDim.x * blockDim.x) {
    int lo = 0, hi = a.npml - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (a.start[mid] <= g) lo = mid; else hi = mid - 1;
    }
    const PmlDev& P = a.pml[lo];
    const long long cell = g - a.start[lo];
    const int AB = P.A * P.B;
    const int l = (int)(cell / AB);
    const int rem = (int)(cell - (long long)l * AB);
    const int ia = rem / P.B, ib = rem - ia * P.B;
    const T* p = a.buf + P.p[a.par ^ 1];   // p(t-1)
    T* pn = a.buf + P.p[a.par];            // p(t-2) -> p(t)
    const T* fn = a.buf + P.phn[a.par ^ 1];
    const T* fa = a.buf + P.pha[a.par ^ 1];
    const T* fb = a.buf + P.phb[a.par ^ 1];
    auto at = [&](const T* arr, int l2, int a2, int b2) -> T {
      if (l2 < 0 || l2 >= P.L || a2 < 0 || a2 >= P.A || b2 < 0 || b2 >= P.B) return (T)0;
      return arr[((long long)l2 * P.A + a2) * P.B + b2];
    };
    T ln = 0, la = 0, lb = 0;
#pragma unroll
    for (int m = 0; m < 7; ++m) {
      ln += c7[m] * at(p, l + m - 3, ia, ib);
      la += c7[m] * at(p, l, ia + m - 3, ib);
      lb += c7[m] * at(p, l, ia, ib + m - 3);
    }
    const T d180 = (T)180 * a.dh * a.dh;
    ln /= d180; la /= d180; lb /= d180;
    const T zn = a.buf[P.zeta + l];
    const long long I = cell;
    const T pc = p[I], po = pn[I];
    const T t1 = 2 * pc;
    const T t2 = -po;
    const T t3 = a.c0 * a.c0 * (ln + la + lb);
    const T t4 = -zn * (pc - po) / a.dt;
    T gn = 0, ga = 0, gb = 0, un = 0, ua = 0, ub = 0;
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      gn += c5[m] * at(fn, l + m - 2, ia, ib);
      ga += c5[m] * at(fa, l, ia + m - 2, ib);
      gb += c5[m] * at(fb, l, ia, ib + m - 2);
      un += c5[m] * at(p, l + m - 2, ia, ib);
      ua += c5[m] * at(p, l, ia + m - 2, ib);
      ub += c5[m] * at(p, l, ia, ib + m - 2);
    }
    const T d12 = (T)12 * a.dh;
    gn /= d12; ga /= d12; gb /= d12;
    un /= d12; ua /= d12; ub /= d12;
    const T t6 = gn + ga + gb;
    const int sl = l - P.strip0;
    const T f = (sl >= 0 && sl < 3) ? a.buf[P.force + ((long long)sl * P.A + ia) * P.B + ib] : (T)0;
    pn[I] = t1 + t2 + a.dt * a.dt * (t3 + t4 + t6 + f);
    const T fnc = fn[I], fac = fa[I], fbc = fb[I];
    a.buf[P.phn[a.par] + I] = fnc - a.dt * zn * fnc + a.dt * (-zn) * un;
    a.buf[P.pha[a.par] + I] = fac + a.dt * zn * ua;
    a.buf[P.phb[a.par] + I] = fbc + a.dt * zn * ub;
  }
}

template <typename T>
struct IfaceArgs {
  T* buf;
  const IfaceDev* ifs;
  int nif;
  long long total;
  const DctDev* dct;
  const PmlDev* pml;
  const unsigned char* masks;
  int par;
  T c0, dh;
};

// Pressure of one side at crossing coordinate c and face coordinates (u, v).
template <typename T>
__device__ __forceinline__ T side_pressure(const IfaceArgs<T>& a, int type, const SideDev& s, int c, int u, int v) {
  if (s.kind == 0) {
    const DctDev& D = a.dct[s.idx];
    const int layer = face_layer(c, s.ext);
    if (type == 0) return a.buf[D.pX + ((long long)layer * D.d + v) * D.h + u];
    if (type == 1) return a.buf[D.pY + ((long long)layer * D.d + v) * D.w + u];
    return a.buf[D.pZ + ((long long)layer * D.h + v) * D.w + u];
  }
  const PmlDev& P = a.pml[s.idx];
  return a.buf[P.p[a.par] + ((long long)c * P.A + v) * P.B + u];
}

template <typename T>
__device__ __forceinline__ void side_force(const IfaceArgs<T>& a, int type, const SideDev& s, int c, int u, int v, T val) {
  if (s.kind == 0) {
    const DctDev& D = a.dct[s.idx];
    const int x = type == 0 ? c : u;
    const int y = type == 0 ? u : (type == 1 ? c : v);
    const int z = type == 2 ? c : v;
    const long long o = shell_index(D, x, y, z);
    if (o >= 0) a.buf[o] = val;
    return;
  }
  const PmlDev& P = a.pml[s.idx];
  a.buf[P.force + ((long long)(c - P.strip0) * P.A + v) * P.B + u] = val;
}

// Boundary::ComputeForcingTerms (boundary.cpp:21-173) for every face cell of
// every interface; the per-cell mask keeps only the writes that survive the
// reference's list-order overwrites.
template <typename T>
__global__ void __launch_bounds__(256) iface_kernel(IfaceArgs<T> a) {
  const T C[6][6] = {{0, 0, -2, 2, 0, 0},       {0, -2, 27, -27, 2, 0},     {-2, 27, -270, 270, -27, 2},
                     {2, -27, 270, -270, 27, -2}, {0, 2, -27, 27, -2, 0},     {0, 0, 2, -2, 0, 0}};
  for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x; g < a.total;
       g += (long long)gridDim.x * blockDim.x) {
    int lo = 0, hi = a.nif - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (a.ifs[mid].cell0 <= g) lo = mid; else hi = mid - 1;
    }
    const IfaceDev& I = a.ifs[lo];
    const long long local = g - I.cell0;
    const int nu = I.u1 - I.u0;
    const int iu = I.u0 + (int)(local % nu);
    const int iv = I.v0 + (int)(local / nu);
    const unsigned mask = a.masks[I.mask + local];
    const int lu = iu - I.lo.ou, lv = iv - I.lo.ov;
    const int hu = iu - I.hi.ou, hv = iv - I.hi.ov;
    T pl[3], ph[3];
#pragma unroll
    for (int n = 0; n < 3; ++n) {
      pl[n] = side_pressure(a, I.type, I.lo, I.lo.ext - 3 + n, lu, lv);
      ph[n] = side_pressure(a, I.type, I.hi, n, hu, hv);
    }
    const T c2 = a.c0 * a.c0;
    const T d180 = (T)180 * a.dh * a.dh;
    const T absorp = (T)I.absorption;
#pragma unroll
    for (int m = -3; m < 3; ++m) {
      if (!(mask & (1u << (m + 3)))) continue;
      T sip1 = 0, sip2 = 0;
#pragma unroll
      for (int n = 0; n < 3; ++n) sip1 += C[m + 3][n] * pl[n];
#pragma unroll
      for (int n = 3; n < 6; ++n) sip2 += C[m + 3][n] * ph[n - 3];
      if (m < 0) {
        const T sip = I.lo.self ? (sip1 + sip2) : sip2;
        const T fi = sip * c2 / d180;
        side_force(a, I.type, I.lo, I.lo.ext + m, lu, lv, absorp * fi);
      } else {
        const T sip = I.hi.self ? (sip1 + sip2) : sip1;
        const T fi = sip * c2 / d180;
        side_force(a, I.type, I.hi, m, hu, hv, absorp * fi);
      }
    }
  }
}

static __global__ void advance_time_kernel(long long* tcount, int n) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *tcount += n;
}

// ---- setup kernels (FP64 arithmetic) ----

// Per extent n, three n*n tables: C[k][j] = 2 cos(pi (j + 1/2) k / n) (the
// REDFT10 matrix), its transpose, and the REDFT01 matrix Ci[k][j] = C[k][j]
// with row k = 0 halved (REDFT01 weights X_0 by 1, the others by 2).
template <typename T>
__global__ void cos_table_kernel(T* buf, long long off, int n) {
  const long long nn = (long long)n * n;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nn; i += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(i / n), j = (int)(i - (long long)k * n);
    // argument reduced exactly in integers
    const long long q = ((long long)(2 * j + 1) * k) % (4LL * n);
    const double v = 2.0 * cospi((double)q / (2.0 * n));
    buf[off + (long long)k * n + j] = (T)v;
    buf[off + nn + (long long)j * n + k] = (T)v;
    buf[off + 2 * nn + (long long)k * n + j] = (T)(k == 0 ? 0.5 * v : v);
  }
}

// Accurate-arithmetic tables: tabA = 1 - cos(w dt) = 2 sin^2(w dt / 2),
// tabB = 2 (1 - cos(w dt)) / w^2, in FP64 then rounded to T.
template <typename T>
__global__ void modal_table_kernel(T* buf, long long tabA, long long tabB, int w, int h, int d, double dh, double dt,
                                   double c0) {
  const long long N = (long long)w * h * d;
  const double lx = w * dh, ly = h * dh, lz = d * dh;
  const double pi = 3.14159265358979323846;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (long long)gridDim.x * blockDim.x) {
    const int kx = (int)(i % w);
    const int ky = (int)((i / w) % h);
    const int kz = (int)(i / ((long long)w * h));
    // 1-based mode numbers, as dct_partition.cpp:24-36
    const double ax = (kx + 1) / lx, ay = (ky + 1) / ly, az = (kz + 1) / lz;
    const double omega = c0 * pi * sqrt(az * az + ay * ay + ax * ax);
    const double th = omega * dt;
    const double s = sin(0.5 * th);
    const double vers = 2.0 * s * s;
    buf[tabA + i] = (T)vers;
    buf[tabB + i] = (T)(2.0 * vers / (omega * omega));
  }
}

}  // namespace ard
