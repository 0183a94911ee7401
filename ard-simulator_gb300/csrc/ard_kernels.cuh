// sm_103a kernels of the ARD time step.  Templated on the working type T
// (float: the product path; double: the FP64 GPU oracle).
//
// Per step (t, parity par = t & 1), in launch order:
//   pml_kernel          Grote-Sim PML update of every slab (own stream)
//   face2d_kernel       forward 2D DCT-II of the 18 force face layers of every
//                       air partition, fused per layer pair in shared memory
//                       (face_gemm_kernel: the same as two GEMM passes where
//                       a layer pair does not fit)
//   modal_kernel        F = expansion of the face transforms (+ point
//                       sources); M(t) = a (2 cos M(t-1) - M(t-2) + psi F);
//                       contraction of M(t) onto the face rows and the
//                       recorder cells
//   post_modal_kernel   recorder samples of step t + sums of the contraction
//                       partials
//   face2d_kernel       inverse 2D transforms -> pressure face layers
//                       (face_gemm_kernel: two GEMM passes)
//   iface_kernel        6th-order interface forcing into the force face
//                       layers / PML strips (owner masks resolve overlapping
//                       strips in the reference's list order)
// The air partitions' kernels (face, modal, sums) launch once per air group
// (up to two groups on two streams).  Every step kernel starts with
// grid_dependency_wait: the host launches them with programmatic stream
// serialization.  xform_gemm_kernel (register-staged GEMM) serves the dense
// whole-field transforms of the readouts and the initial pressure.
#pragma once

#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <type_traits>
#include <utility>

#include "ard_async.cuh"
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
  if (l >= 0) return D.fY + ((long long)l * D.d + z) * D.wp + x;
  l = face_layer(z, D.d);
  if (l >= 0) return D.fZ + ((long long)l * D.h + y) * D.wp + x;
  return -1;
}

// ---- 4-wide vector access (128-bit for float, 2 x 128-bit for double) ----
__device__ __forceinline__ void load4(const float* p, float (&r)[4]) {
  const float4 v = *reinterpret_cast<const float4*>(p);
  r[0] = v.x; r[1] = v.y; r[2] = v.z; r[3] = v.w;
}
__device__ __forceinline__ void load4(const double* p, double (&r)[4]) {
  const double2 a = reinterpret_cast<const double2*>(p)[0], b = reinterpret_cast<const double2*>(p)[1];
  r[0] = a.x; r[1] = a.y; r[2] = b.x; r[3] = b.y;
}
__device__ __forceinline__ void store4(float* p, const float (&r)[4]) {
  *reinterpret_cast<float4*>(p) = make_float4(r[0], r[1], r[2], r[3]);
}
__device__ __forceinline__ void store4(double* p, const double (&r)[4]) {
  reinterpret_cast<double2*>(p)[0] = make_double2(r[0], r[1]);
  reinterpret_cast<double2*>(p)[1] = make_double2(r[2], r[3]);
}

// ---- asynchronous global -> shared copies (cp.async, L2-cached) ----
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem, bool valid) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  const int n = valid ? 16 : 0;  // 0: zero-fill, nothing is read
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem), "r"(n) : "memory");
}
__device__ __forceinline__ void cp_async_scalar(float* smem, const float* gmem, bool valid) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  const int n = valid ? 4 : 0;
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(s), "l"(gmem), "r"(n) : "memory");
}
__device__ __forceinline__ void cp_async_scalar(double* smem, const double* gmem, bool valid) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  const int n = valid ? 8 : 0;
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(s), "l"(gmem), "r"(n) : "memory");
}
// 4 consecutive elements (16 B for float, 2 x 16 B for double)
__device__ __forceinline__ void cp_async4(float* smem, const float* gmem, bool valid) { cp_async16(smem, gmem, valid); }
__device__ __forceinline__ void cp_async4(double* smem, const double* gmem, bool valid) {
  cp_async16(smem, gmem, valid);
  cp_async16(smem + 2, gmem + 2, valid);
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// Programmatic dependent launch: a step kernel launched with programmatic
// stream serialization may start while its predecessor in the stream is
// finishing; griddepcontrol.wait returns once the predecessor has completed
// and its writes are visible (at once for an ordinary launch).  Every step
// kernel waits before its first global access.
__device__ __forceinline__ void grid_dependency_wait() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// ---------------------------------------------------------------------------
// Batched 1D transforms as small GEMMs (see XformJob); one 64 x 64 output
// tile per block iteration, K staged through registers and shared memory in
// chunks of 16, 4 x 4 outputs per thread.  Used for the dense whole-field
// transforms (readouts, initial pressure); the step's face passes use
// face_gemm_kernel below.
// ---------------------------------------------------------------------------

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
  const T a = buf[J.in0 + off];
  return J.in1 >= 0 ? a + (T)J.sgn * buf[J.in1 + off] : a;
}

template <typename T>
__global__ void __launch_bounds__(256) xform_gemm_kernel(T* __restrict__ buf, const XformJob* __restrict__ jobs,
                                                          int njobs, int total) {
  grid_dependency_wait();
  // two K-chunk buffers: chunk k+1 is fetched into registers while chunk k is
  // multiplied; chunks of 16 k (32 measured slower)
  constexpr int BK = 16;
  constexpr int NR = BK / 4;                     // elements of each operand a thread stages per chunk
  __shared__ __align__(16) T Ps[2][BK][64 + 4];  // P(m0 + mm, k0 + kk) at [kk][mm]
  __shared__ __align__(16) T Qs[2][BK][64 + 4];  // Q(k0 + kk, n0 + nn) at [kk][nn]
  // first unit of every job, cached in shared memory for the per-unit job search
  constexpr int kMaxCachedJobs = 1024;
  __shared__ int sfirst[kMaxCachedJobs];
  const int tid = threadIdx.x;
  const int ty = tid >> 4, tx = tid & 15;
  const bool cached = njobs <= kMaxCachedJobs;
  if (cached)
    for (int i = tid; i < njobs; i += 256) sfirst[i] = jobs[i].first;
  __syncthreads();
  for (int unit = blockIdx.x; unit < total; unit += gridDim.x) {
    int ji;
    if (cached) {
      int lo = 0, hi = njobs - 1;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (sfirst[mid] <= unit) lo = mid; else hi = mid - 1;
      }
      ji = lo;
    } else {
      ji = find_job(jobs, njobs, unit);
    }
    const XformJob J = jobs[ji];
    const int t = unit - J.first;
    const int m0 = (t / J.tn) * 64, n0 = (t % J.tn) * 64;
    const int Md = J.rows ? J.batch : J.n;
    const int Nd = J.rows ? J.n : J.batch;
    const int K = J.n;
    const T* A = buf + J.ctab;
    T pr[NR], qr[NR];
    // global -> registers for the chunk at k0
    auto fetch = [&](int k0) {
#pragma unroll
      for (int r = 0; r < NR; ++r) {
        const int e = tid + 256 * r;
        if (!J.rows) {
          // P = A (m = output o, k = j); Q = X (k = j, n = column)
          const int mm = J.inverse ? (e & 63) : (e / BK), kk = J.inverse ? (e >> 6) : (e % BK);
          const int m = m0 + mm, k = k0 + kk;
          T pv = 0;
          if (m < Md && k < K) pv = J.inverse ? A[(long long)k * K + m] : A[(long long)m * K + k];
          pr[r] = pv;
          const int nn = e & 63, kq = e >> 6;
          const int n = n0 + nn, kk2 = k0 + kq;
          qr[r] = (n < Nd && kk2 < K) ? job_input(buf, J, (long long)kk2 * J.ld + n) : (T)0;
        } else {
          // P = X (m = line, k = j); Q(k, n) = A(n, k)
          const int mm = e / BK, kk = e % BK;
          const int m = m0 + mm, k = k0 + kk;
          pr[r] = (m < Md && k < K) ? job_input(buf, J, (long long)m * J.ld + k) : (T)0;
          const int nn = J.inverse ? (e & 63) : (e / BK), kq = J.inverse ? (e >> 6) : (e % BK);
          const int n = n0 + nn, kk2 = k0 + kq;
          T qv = 0;
          if (n < Nd && kk2 < K) qv = J.inverse ? A[(long long)kk2 * K + n] : A[(long long)n * K + kk2];
          qr[r] = qv;
        }
      }
    };
    auto commit = [&](int sb) {
#pragma unroll
      for (int r = 0; r < NR; ++r) {
        const int e = tid + 256 * r;
        if (!J.rows) {
          const int mm = J.inverse ? (e & 63) : (e / BK), kk = J.inverse ? (e >> 6) : (e % BK);
          Ps[sb][kk][mm] = pr[r];
          Qs[sb][e >> 6][e & 63] = qr[r];
        } else {
          Ps[sb][e % BK][e / BK] = pr[r];
          const int nn = J.inverse ? (e & 63) : (e / BK), kq = J.inverse ? (e >> 6) : (e % BK);
          Qs[sb][kq][nn] = qr[r];
        }
      }
    };
    T acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[i][j] = 0;
    __syncthreads();  // the previous unit is done with both buffers
    fetch(0);
    commit(0);
    __syncthreads();
    int sb = 0;
    for (int k0 = 0; k0 < K; k0 += BK) {
      const bool more = k0 + BK < K;
      if (more) fetch(k0 + BK);
#pragma unroll
      for (int kk = 0; kk < BK; ++kk) {
        T pa[4], qb[4];
        load4(&Ps[sb][kk][ty * 4], pa);
        load4(&Qs[sb][kk][tx * 4], qb);
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) acc[i][j] += pa[i] * qb[j];
      }
      if (more) commit(sb ^ 1);
      __syncthreads();
      sb ^= 1;
    }
    const T scale = (T)J.scale;
    const int nb = n0 + tx * 4;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int m = m0 + ty * 4 + i;
      if (m >= Md) continue;
      const long long o = J.out + (long long)m * J.ld + nb;
      if (nb + 3 < Nd && (o & 3) == 0) {
        T v[4] = {acc[i][0] * scale, acc[i][1] * scale, acc[i][2] * scale, acc[i][3] * scale};
        store4(buf + o, v);
      } else {
#pragma unroll
        for (int j = 0; j < 4; ++j)
          if (nb + j < Nd) buf[o + j] = acc[i][j] * scale;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Face transforms of the step as GEMM passes (faces too large for the fused
// kernel): the same jobs as xform_gemm_kernel, with both operands staged by
// cp.async into a three-deep ring of 32-wide K chunks (no register staging,
// one barrier per chunk).  An operand whose source is contiguous along K
// ("k-contiguous": the X lines of a row pass, the forward tables) is kept
// [m or n][32 k] with its 16-byte chunks XOR-swizzled by (row / 4) % 8; an
// operand contiguous along m or n is kept [32 k][64 + 4].  The pass's input
// combination X = in0 + sgn in1 is formed when the X operand is read.
// Instances (one per job list, all jobs of a list alike):
//   PK, QK = 1, 1, CP: row pass, forward  (P = X lines, Q(k, n) = A[n K + k])
//   PK, QK = 1, 0:     column pass, forward (P = A[m K + k], Q = X rows) and
//                      row pass, inverse (P = X lines, Q(k, n) = A[k K + n])
//   PK, QK = 0, 0, CQ: column pass, inverse (P(m, k) = A[k K + m], Q = X rows)
// ---------------------------------------------------------------------------

constexpr int kGemmBK = 32;
constexpr int kGemmStages = 3;
constexpr int kGemmTile = kGemmBK * 68;   // elements of one staged operand tile (either layout)
__host__ __device__ constexpr int face_gemm_smem_elems(bool comb) { return kGemmStages * (comb ? 3 : 2) * kGemmTile; }

// k-contiguous tile: element (r, k) of the [64][32] tile
__device__ __forceinline__ int kc_index(int r, int k) { return r * kGemmBK + ((((k >> 2) ^ (r >> 2)) & 7) << 2) + (k & 3); }

template <typename T, bool PK, bool QK, bool CP, bool CQ>
__global__ void __launch_bounds__(256, 2) face_gemm_kernel(T* __restrict__ buf, const XformJob* __restrict__ jobs,
                                                            int njobs, int total) {
  grid_dependency_wait();
  constexpr bool COMB = CP || CQ;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* sm = reinterpret_cast<T*>(smem_raw);
  constexpr int kMaxCachedJobs = 1024;
  __shared__ int sfirst[kMaxCachedJobs];
  const int tid = threadIdx.x;
  const int ty = tid >> 4, tx = tid & 15;
  const bool cached = njobs <= kMaxCachedJobs;
  if (cached)
    for (int i = tid; i < njobs; i += 256) sfirst[i] = jobs[i].first;
  __syncthreads();
  for (int unit = blockIdx.x; unit < total; unit += gridDim.x) {
    int ji;
    if (cached) {
      int lo = 0, hi = njobs - 1;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (sfirst[mid] <= unit) lo = mid; else hi = mid - 1;
      }
      ji = lo;
    } else {
      ji = find_job(jobs, njobs, unit);
    }
    const XformJob J = jobs[ji];
    const int t = unit - J.first;
    const int m0 = (t / J.tn) * 64, n0 = (t % J.tn) * 64;
    const int Md = J.rows ? J.batch : J.n;
    const int Nd = J.rows ? J.n : J.batch;
    const int K = J.n;
    // operand sources: P (m, k) and Q (k, n); the X operand may have a second input
    long long p0, p1 = 0, q0, q1 = 0;
    int sp, sq;
    if (J.rows) { p0 = J.in0; p1 = J.in1; sp = J.ld; q0 = J.ctab; sq = K; }
    else { p0 = J.ctab; sp = K; q0 = J.in0; q1 = J.in1; sq = J.ld; }
    const T sgn = (T)J.sgn;
    // stage one operand tile: rows of the k-contiguous layout are m (or n),
    // rows of the other layout are k; lim = extent of m (or n)
    auto stage_kc = [&](T* dst, long long base, int stride, int r0, int lim, int k0) {
      const bool vec = ((stride | K) & 3) == 0 && (base & 3) == 0;
      if (vec) {
#pragma unroll
        for (int v = 0; v < 2; ++v) {
          const int e = tid + 256 * v;          // 512 vectors: row e / 8, chunk e % 8
          const int r = e >> 3, c = e & 7;
          const bool ok = r0 + r < lim && k0 + 4 * c < K;
          cp_async4(dst + kc_index(r, 4 * c), buf + (ok ? base + (long long)(r0 + r) * stride + k0 + 4 * c : 0), ok);
        }
      } else {
#pragma unroll
        for (int v = 0; v < 8; ++v) {
          const int e = tid + 256 * v;          // 2048 elements: row e / 32, k e % 32
          const int r = e >> 5, k = e & 31;
          const bool ok = r0 + r < lim && k0 + k < K;
          cp_async_scalar(dst + kc_index(r, k), buf + (ok ? base + (long long)(r0 + r) * stride + k0 + k : 0), ok);
        }
      }
    };
    auto stage_mn = [&](T* dst, long long base, int stride, int c0, int lim, int k0) {
      const bool vec = ((stride | lim) & 3) == 0 && (base & 3) == 0;
      if (vec) {
#pragma unroll
        for (int v = 0; v < 2; ++v) {
          const int e = tid + 256 * v;          // 512 vectors: k e / 16, columns 4 (e % 16)
          const int k = e >> 4, c = (e & 15) * 4;
          const bool ok = k0 + k < K && c0 + c < lim;
          cp_async4(dst + k * 68 + c, buf + (ok ? base + (long long)(k0 + k) * stride + c0 + c : 0), ok);
        }
      } else {
#pragma unroll
        for (int v = 0; v < 8; ++v) {
          const int e = tid + 256 * v;          // 2048 elements: k e / 64, column e % 64
          const int k = e >> 6, c = e & 63;
          const bool ok = k0 + k < K && c0 + c < lim;
          cp_async_scalar(dst + k * 68 + c, buf + (ok ? base + (long long)(k0 + k) * stride + c0 + c : 0), ok);
        }
      }
    };
    constexpr int NT = COMB ? 3 : 2;
    auto issue = [&](int k0, int sb) {
      T* st = sm + sb * NT * kGemmTile;
      if constexpr (PK) stage_kc(st, p0, sp, m0, Md, k0); else stage_mn(st, p0, sp, m0, Md, k0);
      if constexpr (QK) stage_kc(st + kGemmTile, q0, sq, n0, Nd, k0); else stage_mn(st + kGemmTile, q0, sq, n0, Nd, k0);
      if constexpr (CP) stage_kc(st + 2 * kGemmTile, p1, sp, m0, Md, k0);
      if constexpr (CQ) stage_mn(st + 2 * kGemmTile, q1, sq, n0, Nd, k0);
    };
    T acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[i][j] = 0;
    const int nch = (K + kGemmBK - 1) / kGemmBK;
    __syncthreads();   // the previous unit is done with the ring
#pragma unroll
    for (int p = 0; p < kGemmStages - 1; ++p) {
      if (p < nch) issue(p * kGemmBK, p);
      cp_async_commit();
    }
    for (int c = 0; c < nch; ++c) {
      cp_async_wait<kGemmStages - 2>();
      __syncthreads();   // chunk c visible; chunk c - 1's slot free
      if (c + kGemmStages - 1 < nch) issue((c + kGemmStages - 1) * kGemmBK, (c + kGemmStages - 1) % kGemmStages);
      cp_async_commit();
      const T* st = sm + (c % kGemmStages) * NT * kGemmTile;
      const T* Pt = st;
      const T* Qt = st + kGemmTile;
      const T* Xt = st + 2 * kGemmTile;
#pragma unroll 2
      for (int kq = 0; kq < kGemmBK; kq += 4) {
        T pa[4][4], qb[4][4];   // [row i or column j][k of the quad]
        if constexpr (PK) {
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            load4(Pt + kc_index(ty * 4 + i, kq), pa[i]);
            if constexpr (CP) {
              T x[4];
              load4(Xt + kc_index(ty * 4 + i, kq), x);
#pragma unroll
              for (int k = 0; k < 4; ++k) pa[i][k] += sgn * x[k];
            }
          }
        } else {
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            T v[4];
            load4(Pt + (kq + k) * 68 + ty * 4, v);
#pragma unroll
            for (int i = 0; i < 4; ++i) pa[i][k] = v[i];
          }
        }
        if constexpr (QK) {
#pragma unroll
          for (int j = 0; j < 4; ++j) load4(Qt + kc_index(tx * 4 + j, kq), qb[j]);
        } else {
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            T v[4];
            load4(Qt + (kq + k) * 68 + tx * 4, v);
            if constexpr (CQ) {
              T x[4];
              load4(Xt + (kq + k) * 68 + tx * 4, x);
#pragma unroll
              for (int j = 0; j < 4; ++j) v[j] += sgn * x[j];
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) qb[j][k] = v[j];
          }
        }
#pragma unroll
        for (int k = 0; k < 4; ++k)
#pragma unroll
          for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) acc[i][j] += pa[i][k] * qb[j][k];
      }
    }
    cp_async_wait<0>();
    const T scale = (T)J.scale;
    const int nb = n0 + tx * 4;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int m = m0 + ty * 4 + i;
      if (m >= Md) continue;
      const long long o = J.out + (long long)m * J.ld + nb;
      if (nb + 3 < Nd && (o & 3) == 0) {
        T v[4] = {acc[i][0] * scale, acc[i][1] * scale, acc[i][2] * scale, acc[i][3] * scale};
        store4(buf + o, v);
      } else {
#pragma unroll
        for (int j = 0; j < 4; ++j)
          if (nb + j < Nd) buf[o + j] = acc[i][j] * scale;
      }
    }
  }
}

// Host: a step kernel launched with programmatic stream serialization: the
// grid is scheduled while its predecessor in the stream drains and waits for
// it on the device (grid_dependency_wait), which hides the launch gap between
// the dependent kernels of a step (also inside the captured graphs).
template <typename... KArgs, typename... Args>
inline cudaError_t launch_dep(void (*kernel)(KArgs...), long long grid, int block, size_t smem, cudaStream_t s,
                              Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3((unsigned)block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

// Host: the face_gemm_kernel instance for a job list (all jobs of a list share
// rows, inverse and whether the X operand has a second input), `grid` blocks.
template <typename T>
inline cudaError_t launch_face_gemm(T* buf, const XformJob& j0, const XformJob* d_jobs, int njobs, int units, int grid,
                                    cudaStream_t s) {
  if (njobs == 0) return cudaSuccess;
  const bool comb = j0.in1 >= 0;
  const size_t s2 = (size_t)face_gemm_smem_elems(false) * sizeof(T), s3 = (size_t)face_gemm_smem_elems(true) * sizeof(T);
  if (j0.rows && !j0.inverse && comb)
    return launch_dep(face_gemm_kernel<T, true, true, true, false>, grid, 256, s3, s, buf, d_jobs, njobs, units);
  if (!comb && (j0.rows != 0) == (j0.inverse != 0))
    return launch_dep(face_gemm_kernel<T, true, false, false, false>, grid, 256, s2, s, buf, d_jobs, njobs, units);
  if (!j0.rows && j0.inverse && comb)
    return launch_dep(face_gemm_kernel<T, false, false, false, true>, grid, 256, s3, s, buf, d_jobs, njobs, units);
  return cudaErrorInvalidValue;
}

// Host: dynamic shared memory of the face_gemm_kernel instances (set in every
// translation unit that launches them).
template <typename T>
inline cudaError_t configure_face_gemm() {
  const int s2 = (int)(face_gemm_smem_elems(false) * sizeof(T)), s3 = (int)(face_gemm_smem_elems(true) * sizeof(T));
  cudaError_t e = cudaFuncSetAttribute(face_gemm_kernel<T, true, true, true, false>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, s3);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(face_gemm_kernel<T, true, false, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, s2);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(face_gemm_kernel<T, false, false, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, s3);
  return e;
}

// ---------------------------------------------------------------------------
// Fused face transform: one block per (face layer, 32-column slab); the
// layer is staged in shared memory, the U-transform of the slab goes to
// shared memory, the V-transform writes the output slab.
// ---------------------------------------------------------------------------

// In-place sum of the per-tile partial slabs of the modal contraction:
// slab 0 of each job receives the sum of its nb slabs (fixed order).  A
// job's elements occupy [first, first + count) of the launch's index space,
// first a multiple of kSumChunk.
constexpr int kSumChunk = 2048;
struct SumJob {
  long long base;     // slab 0
  long long count;    // elements per slab
  long long stride;   // slab stride
  long long first;    // first element of this job in the launch's index space
  int nb;
};

// After the modal update: the recorder samples of the step (blocks
// [0, rec_blocks): one warp per recorder, the sum of the tiles' partials
// times s_i into the double history) and the in-place partial sums (the
// other blocks: launches of at least a wave of chunks grid-stride over
// chunks of kSumChunk elements, 8 per thread; smaller ones take one element
// per thread with all its slabs in flight).  One launch for both.
template <typename T>
struct PostModalArgs {
  T* buf;
  const DctDev* dct;
  const PointDev* recs;   // all recorders; this launch takes [rec_first, rec_first + nrec)
  int rec_first, nrec;
  int nrec_total;         // row width of the history
  double* hist;
  const long long* tcount;
  int tstep;
  long long max_steps;
  int rec_blocks;
  const SumJob* jobs;     // this launch's sum jobs; their elements start at `first`
  int njobs;
  long long first;
  long long total;        // a multiple of kSumChunk
  int per;                // elements per thread: 1, 2, 4 or 8 (chunked), 0: one element per thread
};

template <typename T>
__global__ void __launch_bounds__(256) post_modal_kernel(PostModalArgs<T> a) {
  grid_dependency_wait();
  if ((int)blockIdx.x < a.rec_blocks) {
    const int lane = threadIdx.x & 31;
    const int rl = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (rl >= a.nrec) return;
    const int r = a.rec_first + rl;
    const PointDev q = a.recs[r];
    const DctDev& D = a.dct[q.part];
    const int local_r = r - D.rec0;
    const int ntiles = D.nbx * D.nby * D.nbz;
    T s = 0;
    for (int i = lane; i < ntiles; i += 32) s += a.buf[D.recpart + (long long)i * D.nrec + local_r];
    s = warp_sum(s);
    const long long t = *a.tcount + a.tstep;
    if (lane == 0 && t < a.max_steps) a.hist[t * a.nrec_total + q.slot] = (double)(s * (T)D.si);
    return;
  }
  T* __restrict__ buf = a.buf;
  // first elements of the jobs, cached for the per-chunk job search
  constexpr int kMaxCachedJobs = 1024;
  __shared__ long long sfirst[kMaxCachedJobs];
  const bool cached = a.njobs <= kMaxCachedJobs;
  if (cached)
    for (int i = threadIdx.x; i < a.njobs; i += blockDim.x) sfirst[i] = a.jobs[i].first;
  __syncthreads();
  // chunks of kSumChunk elements: a job's elements start on a chunk boundary
  // of the index space, so a chunk lies in one job; a thread sums 8 elements
  // (256 apart) over the job's slabs, slab by slab in order
  const long long nb = (long long)gridDim.x - a.rec_blocks;
  if (a.per == 0) {
    // small launches: one element per thread, all its slabs in flight at once
    for (long long g = ((long long)blockIdx.x - a.rec_blocks) * blockDim.x + threadIdx.x; g < a.total;
         g += nb * blockDim.x) {
      const long long gg = g + a.first;
      int lo = 0, hi = a.njobs - 1;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if ((cached ? sfirst[mid] : a.jobs[mid].first) <= gg) lo = mid; else hi = mid - 1;
      }
      const SumJob J = a.jobs[lo];
      const long long e = gg - J.first;
      if (e >= J.count) continue;   // the chunk padding of the index space
      const T* p = buf + J.base + e;
      T v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      int b = 0;
      for (; b + 8 <= J.nb; b += 8) {
#pragma unroll
        for (int k = 0; k < 8; ++k) v[k] += p[(long long)(b + k) * J.stride];
      }
#pragma unroll
      for (int k = 0; k < 7; ++k)
        if (b + k < J.nb) v[k] += p[(long long)(b + k) * J.stride];
      buf[J.base + e] = ((v[0] + v[1]) + (v[2] + v[3])) + ((v[4] + v[5]) + (v[6] + v[7]));
    }
    return;
  }
  // work items: a chunk in kSumChunk / (256 per) parts of 256 per elements,
  // `per` (1, 2, 4 or 8) elements per thread, 256 apart
  const int per = a.per;
  const int parts = kSumChunk / (256 * per);
  const long long nitems = a.total / kSumChunk * parts;
  for (long long item = (long long)blockIdx.x - a.rec_blocks; item < nitems; item += nb) {
    const long long ch = item / parts;
    const int part = (int)(item - ch * parts);
    const long long gg = a.first + ch * kSumChunk;   // first element of the chunk among all sum jobs
    int lo = 0, hi = a.njobs - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if ((cached ? sfirst[mid] : a.jobs[mid].first) <= gg) lo = mid; else hi = mid - 1;
    }
    const SumJob J = a.jobs[lo];
    const long long e0 = gg - J.first + (long long)part * 256 * per;
    T* p = buf + J.base + e0;
    constexpr int kPer = kSumChunk / 256;
    bool ok[kPer];
    T v[kPer];
#pragma unroll
    for (int i = 0; i < kPer; ++i) {
      const int idx = (int)threadIdx.x + 256 * i;
      ok[i] = i < per && e0 + idx < J.count;
      v[i] = ok[i] ? p[idx] : (T)0;
    }
#pragma unroll 2
    for (int b = 1; b < J.nb; ++b) {
      const T* q = p + (long long)b * J.stride;
#pragma unroll
      for (int i = 0; i < kPer; ++i)
        if (ok[i]) v[i] += q[threadIdx.x + 256 * i];
    }
#pragma unroll
    for (int i = 0; i < kPer; ++i)
      if (ok[i]) p[threadIdx.x + 256 * i] = v[i];
  }
}

constexpr int kFace2DThreads = 256;
constexpr int kFace2DWarps = kFace2DThreads / 32;

struct Face2DSmem {
  int xs;  // X0: max over the jobs of V * max(xp, ap) (the layer, then E or the A table)
  int x1;  // X1: the same (the second layer, then O or the A table)
  int bs;  // B slab, row-major [Up][32]
  int ts;  // each of T0, T1, row-major [Vp][32]
};

// Row pitch of the staged layers and of the staged A table: 4 mod 8 elements,
// so rows r .. r + 7 start in distinct 16-byte bank groups.
__host__ __device__ inline int face2d_pitch(int n) {
  const int n4 = (n + 3) & ~3;
  return n4 + ((n4 & 7) ? 8 : 4);
}

// One block per (layer pair, slab of at most 32 columns).  X0, X1 (V x U, row
// pitch ld) are staged in shared memory (cp.async) and combined into
// E = X0 + X1 and O = X0 - X1; then along U, T = E B and O B over the slab
// (B: U x U table, its slab row-major), and along V, out0 = scale A (E B),
// out1 = scale A (O B) (A: V x V table, row o contiguous).  Layer pairs are
// the two layers of the same distance from either face
// (C(k, n-1-j) = (-1)^k C(k, j)): forward (and the adjoint of the inverse)
// take the layers and give the even / odd parts, the inverse (and the
// adjoint of the forward) take the even / odd parts and give the layers.
//
// Both products are outer-product register tiles: a thread owns MR rows x 4
// columns (per output), and per step of 4 along the contraction it loads
// MR x 4 of the left operand (rows of E / O, or of A: one 16-byte load per
// row) and 4 x 4 of the right operand (rows of the B slab, or of T), then
// issues 16 MR FMAs per output.  A warp is RT x CT threads: a 32-column slab
// takes CT = 8 column quads (8 rows per warp), a 16-column one CT = 4 (16
// rows per warp), both with MR = 2.  Rows are interleaved (row = base + rt +
// RT i), so the RT rows of one left-operand load are consecutive and fall in
// distinct bank groups, and the CT column quads of a right-operand load are
// one contiguous 128 (64) byte line.
// MODE 0: acc0 = L0 R0; 1: also acc1 = L1 R0 (two left operands); 2: also
// acc1 = L0 R1 (two right operands).  A thread owns MR rows x 4 columns.  Rows < nrows; the contraction runs over
// K (a multiple of 4; the operands read as zero past their extent).  Results
// go to shared memory (W row pitch wp) or, scaled, to global memory at
// W + woff + row wp + column for columns < wcols.
template <typename T, int CT, int MR, int MODE, bool GLOBAL>
__device__ __forceinline__ void face2d_tiles(int nrows, int K, const T* L0, const T* L1, int lp, const T* R0,
                                             const T* R1, int rp, T* W0, T* W1, long long wp, long long woff,
                                             int wcols, T scale) {
  constexpr int RT = 32 / CT;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int ct = lane % CT, rt = lane / CT;
  const int c0 = 4 * ct;
  for (int rb = warp * MR * RT; rb < nrows; rb += kFace2DWarps * MR * RT) {
    int row[MR];
#pragma unroll
    for (int i = 0; i < MR; ++i) row[i] = min(rb + rt + RT * i, nrows - 1);
    T acc0[MR][4], acc1[MR][4];
#pragma unroll
    for (int i = 0; i < MR; ++i)
#pragma unroll
      for (int c = 0; c < 4; ++c) { acc0[i][c] = 0; acc1[i][c] = 0; }
#pragma unroll 2
    for (int k = 0; k < K; k += 4) {
      T r0[4][4], r1[4][4], l0[MR][4], l1[MR][4];
#pragma unroll
      for (int kk = 0; kk < 4; ++kk) {
        load4(R0 + (k + kk) * rp + c0, r0[kk]);
        if constexpr (MODE == 2) load4(R1 + (k + kk) * rp + c0, r1[kk]);
      }
#pragma unroll
      for (int i = 0; i < MR; ++i) {
        load4(L0 + row[i] * lp + k, l0[i]);
        if constexpr (MODE == 1) load4(L1 + row[i] * lp + k, l1[i]);
      }
#pragma unroll
      for (int kk = 0; kk < 4; ++kk)
#pragma unroll
        for (int i = 0; i < MR; ++i)
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            acc0[i][c] += l0[i][kk] * r0[kk][c];
            if constexpr (MODE == 1) acc1[i][c] += l1[i][kk] * r0[kk][c];
            if constexpr (MODE == 2) acc1[i][c] += l0[i][kk] * r1[kk][c];
          }
    }
#pragma unroll
    for (int i = 0; i < MR; ++i) {
      const int r = rb + rt + RT * i;
      if (r >= nrows) continue;
      if constexpr (!GLOBAL) {
        store4(W0 + r * wp + c0, acc0[i]);
        if constexpr (MODE != 0) store4(W1 + r * wp + c0, acc1[i]);
      } else {
        T* p0 = W0 + woff + r * wp + c0;
        T* p1 = (MODE != 0) ? W1 + woff + r * wp + c0 : nullptr;
#pragma unroll
        for (int c = 0; c < 4; ++c)
          if (c0 + c < wcols) {
            p0[c] = acc0[i][c] * scale;
            if constexpr (MODE != 0) p1[c] = acc1[i][c] * scale;
          }
      }
    }
  }
}

// Cluster item i is the job pair (jobs[2 i], jobs[2 i + 1]), CTA h taking
// jobs[2 i + h].  Two whole jobs: each CTA runs its own.  A row-split job
// (both entries the same): CTA h stages, combines and transforms rows
// [r0, r0 + nr) of the layers (h = 0 the first ceil(V / 2)), writes its rows
// of T, takes the other rows of T from its peer's shared memory (distributed
// shared memory, between two cluster barriers) and writes rows [r0, r0 + nr)
// of the outputs from its rows of A.  Both CTAs pass the two cluster
// barriers of every item.
//
// CLUSTER false (a launch without split jobs): one CTA per job entry,
// entries [0, 2 nitems), no cluster barriers.
template <typename T, bool CLUSTER>
__device__ __forceinline__ void face2d_body(T* __restrict__ buf, const Face2DJob* __restrict__ jobs, int nitems,
                                            const Face2DSmem& sm) {
  grid_dependency_wait();
  namespace cg = cooperative_groups;
  const int half = CLUSTER ? (int)cg::this_cluster().block_rank() : 0;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* X0 = reinterpret_cast<T*>(smem_raw);
  T* X1 = X0 + sm.xs;
  T* Bs = X1 + sm.x1;
  T* T0 = Bs + sm.bs;
  T* T1 = T0 + sm.ts;
  const T* P0 = T0;   // the peer's T (cluster launches)
  const T* P1 = T1;
  if constexpr (CLUSTER) {
    P0 = cg::this_cluster().map_shared_rank(T0, half ^ 1);
    P1 = cg::this_cluster().map_shared_rank(T1, half ^ 1);
  }
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int first = CLUSTER ? (int)(blockIdx.x >> 1) : (int)blockIdx.x;
  const int stride = CLUSTER ? (int)(gridDim.x >> 1) : (int)gridDim.x;
  const int count = CLUSTER ? nitems : 2 * nitems;
  for (int it = first; it < count; it += stride) {
    const Face2DJob J = jobs[CLUSTER ? 2 * it + half : it];
    const int V = J.V, U = J.U;
    const int Up = (U + 3) & ~3, Vp = (V + 3) & ~3;
    const int xp = face2d_pitch(U), ap = face2d_pitch(V);
    const int cq = J.narrow ? 4 : 8;    // column quads of the slab
    const int bp = 4 * cq;              // row pitch of the B slab and of T
    const int nh = (V + 1) >> 1;        // rows of the first half of a split job
    const int r0 = (J.split && half) ? nh : 0;                 // this CTA's rows
    const int nr = J.split ? (half ? V - nh : nh) : V;
    const int p0 = half ? 0 : nh;                              // the peer's rows (split jobs)
    const int pn = J.split ? (half ? nh : V - nh) : 0;
    __syncthreads();  // previous job done with shared memory
    // ---- stage rows r0 .. r0 + nr - 1 of X0, X1 (columns U .. Up-1 zero)
    // and the B slab (asynchronous) ----
    const T* g0 = buf + J.in0 + (long long)r0 * J.ld;
    const T* g1 = buf + J.in1 + (long long)r0 * J.ld;
    const int q4 = Up >> 2;
    const bool xvec = ((U | J.ld) & 3) == 0 && ((J.in0 | J.in1) & 3) == 0;
    for (int r = warp; r < nr; r += kFace2DWarps)
      for (int q = lane; q < q4; q += 32) {
        const int c = 4 * q;
        const long long off = (long long)r * J.ld + c;
        if (xvec) {
          cp_async4(X0 + r * xp + c, g0 + off, true);
          cp_async4(X1 + r * xp + c, g1 + off, true);
        } else {
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            const bool ok = c + e < U;
            cp_async_scalar(X0 + r * xp + c + e, g0 + (ok ? off + e : 0), ok);
            cp_async_scalar(X1 + r * xp + c + e, g1 + (ok ? off + e : 0), ok);
          }
        }
      }
    const T* B = buf + J.tabB;
    const bool bvec = ((U | J.u0) & 3) == 0 && (J.tabB & 3) == 0;
    for (int i = tid; i < Up * cq; i += kFace2DThreads) {
      const int j = i / cq, c = 4 * (i - j * cq);
      const long long off = (long long)j * U + J.u0 + c;
      if (bvec && j < U && c + 3 < J.ub) {
        cp_async4(Bs + j * bp + c, B + off, true);
      } else {
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const bool ok = j < U && c + e < J.ub;
          cp_async_scalar(Bs + j * bp + c + e, B + (ok ? off + e : 0), ok);
        }
      }
    }
    cp_async_commit();
    // rows V .. Vp-1 of T read as zero in the second product
    for (int i = tid; i < (Vp - V) * bp; i += kFace2DThreads) {
      T0[V * bp + i] = (T)0;
      T1[V * bp + i] = (T)0;
    }
    cp_async_wait<0>();
    __syncthreads();
    // ---- E = X0 + X1, O = X0 - X1 (a one-output job keeps its part in X0) ----
    for (int r = warp; r < nr; r += kFace2DWarps)
      for (int q = lane; q < q4; q += 32) {
        T a[4], b[4], e[4], o[4];
        load4(X0 + r * xp + 4 * q, a);
        load4(X1 + r * xp + 4 * q, b);
#pragma unroll
        for (int k = 0; k < 4; ++k) { e[k] = a[k] + b[k]; o[k] = a[k] - b[k]; }
        if (J.which == 2) {
          store4(X0 + r * xp + 4 * q, o);
        } else {
          store4(X0 + r * xp + 4 * q, e);
          if (J.which == 0) store4(X1 + r * xp + 4 * q, o);
        }
      }
    __syncthreads();
    // ---- rows r0 .. r0 + nr - 1 of A (V x V, columns V .. Vp-1 zero) into
    // X1 (one output, overlapping the first product) or into X0 after it ----
    const T* A = buf + J.tabA + (long long)r0 * V;
    const bool avec = (V & 3) == 0 && (J.tabA & 3) == 0;
    auto stage_a = [&](T* dst) {
      const int a4 = Vp >> 2;
      for (int o = warp; o < nr; o += kFace2DWarps)
        for (int q = lane; q < a4; q += 32) {
          const int r = 4 * q;
          const long long off = (long long)o * V + r;
          if (avec) {
            cp_async4(dst + o * ap + r, A + off, true);
          } else {
#pragma unroll
            for (int e = 0; e < 4; ++e) {
              const bool ok = r + e < V;
              cp_async_scalar(dst + o * ap + r + e, A + (ok ? off + e : 0), ok);
            }
          }
        }
      cp_async_commit();
    };
    const bool one = J.which != 0;
    if (one) stage_a(X1);
    // ---- along U: rows r0 .. of T0 (, T1) = E (, O) B over the slab ----
    T* W0 = T0 + r0 * bp;
    T* W1 = T1 + r0 * bp;
    if (J.narrow) {
      if (one) face2d_tiles<T, 4, 2, 0, false>(nr, Up, X0, X0, xp, Bs, Bs, bp, W0, W0, bp, 0, 0, (T)1);
      else     face2d_tiles<T, 4, 2, 1, false>(nr, Up, X0, X1, xp, Bs, Bs, bp, W0, W1, bp, 0, 0, (T)1);
    } else {
      if (one) face2d_tiles<T, 8, 2, 0, false>(nr, Up, X0, X0, xp, Bs, Bs, bp, W0, W0, bp, 0, 0, (T)1);
      else     face2d_tiles<T, 8, 2, 1, false>(nr, Up, X0, X1, xp, Bs, Bs, bp, W0, W1, bp, 0, 0, (T)1);
    }
    if constexpr (CLUSTER) cg::this_cluster().sync();   // both halves of T written; E and O consumed
    else __syncthreads();
    if (!one) stage_a(X0);
    // the peer's rows of T
    for (int i = tid; i < pn * cq; i += kFace2DThreads) {
      const int r = p0 + i / cq, c = 4 * (i % cq);
      T v[4];
      load4(P0 + r * bp + c, v);
      store4(T0 + r * bp + c, v);
      if (!one) {
        load4(P1 + r * bp + c, v);
        store4(T1 + r * bp + c, v);
      }
    }
    cp_async_wait<0>();
    if constexpr (CLUSTER) cg::this_cluster().sync();   // copies done (the peer may reuse its T); A staged
    else __syncthreads();
    // ---- along V: rows r0 .. of out = scale A T ----
    const T* As = one ? X1 : X0;
    T* o0 = (J.which == 2) ? buf + J.out1 : buf + J.out0;
    T* o1 = (J.which == 0) ? buf + J.out1 : nullptr;
    const long long w0 = J.u0 + (long long)r0 * J.ld;
    const T sc = (T)J.scale;
    if (J.narrow) {
      if (one) face2d_tiles<T, 4, 2, 0, true>(nr, Vp, As, As, ap, T0, T0, bp, o0, o0, J.ld, w0, J.ub, sc);
      else     face2d_tiles<T, 4, 2, 2, true>(nr, Vp, As, As, ap, T0, T1, bp, o0, o1, J.ld, w0, J.ub, sc);
    } else {
      if (one) face2d_tiles<T, 8, 2, 0, true>(nr, Vp, As, As, ap, T0, T0, bp, o0, o0, J.ld, w0, J.ub, sc);
      else     face2d_tiles<T, 8, 2, 2, true>(nr, Vp, As, As, ap, T0, T1, bp, o0, o1, J.ld, w0, J.ub, sc);
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(kFace2DThreads, 2) face2d_kernel(T* __restrict__ buf, const Face2DJob* __restrict__ jobs,
                                                                  int nitems, Face2DSmem sm) {
  face2d_body<T, false>(buf, jobs, nitems, sm);
}

template <typename T>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(kFace2DThreads, 2)
    face2d_cluster_kernel(T* __restrict__ buf, const Face2DJob* __restrict__ jobs, int nitems, Face2DSmem sm) {
  face2d_body<T, true>(buf, jobs, nitems, sm);
}

// Launch of the face transforms over n cluster items (2 n job entries):
// clusters of two CTAs where the list holds row-split jobs, else one CTA per
// entry; at most max_ctas CTAs.
template <typename T>
inline cudaError_t launch_face2d(bool split, long long n, int max_ctas, size_t smem, cudaStream_t s, T* buf,
                                 const Face2DJob* jobs, const Face2DSmem& sm) {
  if (n <= 0) return cudaSuccess;
  if (split) {
    const long long c = std::max(1LL, std::min(n, (long long)(max_ctas / 2)));
    return launch_dep(face2d_cluster_kernel<T>, 2 * c, kFace2DThreads, smem, s, buf, jobs, (int)n, sm);
  }
  const long long b = std::max(1LL, std::min(2 * n, (long long)max_ctas));
  return launch_dep(face2d_kernel<T>, b, kFace2DThreads, smem, s, buf, jobs, (int)n, sm);
}

// ---------------------------------------------------------------------------
// Modal update
// ---------------------------------------------------------------------------

template <typename T>
struct ModalArgs {
  T* buf;
  const DctDev* dct;
  const int4* tiles;        // {air partition, kx tile, ky tile, kz tile}
  int ntiles;
  const PointDev* srcs;
  const PointDev* recs;
  const float* series;      // [n_sources][max_steps]
  long long max_steps;
  const long long* tcount;  // steps completed before the current launch sequence
  int tstep;                // step offset inside the sequence (adjoint: counted backwards)
  int par;
  const T* resid;           // adjoint: recorder residuals [steps][n_rec_total]
  int n_rec_total;
};

// Shared memory of the modal kernel, in elements of T: the ky-contraction
// slots, point coefficients, recorder reduction, and the double-buffered
// per-plane inputs (7 four-element rows per thread + 6 PX values per ky row).
constexpr int kModalRySlot = 3 * 1024;  // [3 n][rpc * kxt = 1024]
constexpr int kModalStageCz = 7 * 4 * kModalThreads + 32 * 6;   // [8 warps][4]: Cd row kz, n = 0..2
constexpr int kModalStage = kModalStageCz + 32;
constexpr int kModalSmemElems =
    2 * kModalRySlot + 2 * kMaxPointsPerPart * 128 + 8 * kMaxPointsPerPart + 2 * kModalStage;

// One block (8 warps) per tile of kxt kx x rpc ky x TZ kz modes; a thread
// owns 4 consecutive kx of one ky row.  Per mode it reads M(t-1), M(t-2)
// and the two tables and writes M(t) (all 128-bit, row pitch wp), expands
// the face transforms into the force mode F, and contracts M(t) onto the face
// rows: along kx by a shuffle butterfly (partial per kx tile), along ky
// through shared memory (partial per ky tile), along kz in registers
// (partial per kz tile).  REF selects the reference's arithmetic.
//
// ADJ runs the transposed step of the adjoint, backwards in time, on the
// adjoint modal levels mu: mu(t) = alpha mu(t+1) - a mu(t+2) + G(t), where
// alpha and -a are the forward recurrence's coefficients of M(t-1) and M(t-2)
// and G is the expansion of the adjoint face transforms with the REDFT01
// weights plus the recorder residuals injected with the recorder basis.  The
// contraction then runs on beta mu(t) (beta: the forward coefficient of the
// force mode F) with the REDFT10 weights onto the face rows and onto the
// source cells (source-series gradient partials).
template <typename T, bool REF, bool ADJ = false>
__global__ void __launch_bounds__(kModalThreads, 2) modal_kernel(ModalArgs<T> a) {
  grid_dependency_wait();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* ry_s = reinterpret_cast<T*>(smem_raw);
  T* cws = ry_s + 2 * kModalRySlot;                  // [kMaxPointsPerPart][128]
  T* cwr = cws + kMaxPointsPerPart * 128;            // [kMaxPointsPerPart][128]
  T* red = cwr + kMaxPointsPerPart * 128;            // [8 warps][kMaxPointsPerPart]
  T* stage = red + 8 * kMaxPointsPerPart;            // [2][kModalStage]
  __shared__ int pts_y[2][kMaxPointsPerPart], pts_z[2][kMaxPointsPerPart];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  T* __restrict__ buf = a.buf;
  const long long t = ADJ ? (*a.tcount - a.tstep) : (*a.tcount + a.tstep);

  for (int tile_id = blockIdx.x; tile_id < a.ntiles; tile_id += gridDim.x) {
    const int4 tl = a.tiles[tile_id];
    const DctDev& D = a.dct[tl.x];
    const int w = D.w, h = D.h, d = D.d, wp = D.wp, G = D.G, KXT = D.kxt, RPC = D.rpc;
    const int rs = warp * (32 / G) + lane / G;   // row slot in the tile
    const int li = lane % G;
    const int kl0 = 4 * li;
    const int kx0 = tl.y * KXT + kl0;
    const int ky0 = tl.z * RPC;
    const int ky = ky0 + rs;
    const bool rowok = ky < h;
    const bool lanok = rowok && kx0 < wp;
    const int kz0 = tl.w * D.TZ, kz1 = min(kz0 + D.TZ, d);
    const int nsrc = D.nsrc, nrec = D.nrec;
    const T* Cw = buf + D.cw;
    const T* Ch = buf + D.ch;
    const T* Cd = buf + D.cd;
    const T* Cwi = Cw + (long long)w * w;
    const T* Chi = Ch + (long long)h * h;
    const T* Cdi = Cd + (long long)d * d;
    // injected points (sources; adjoint: recorders) and read-out points
    // (recorders; adjoint: sources) with their bases
    const int ninj = ADJ ? nrec : nsrc, nout = ADJ ? nsrc : nrec;
    const PointDev* injp = ADJ ? a.recs + D.rec0 : a.srcs + D.src0;
    const PointDev* outp = ADJ ? a.srcs + D.src0 : a.recs + D.rec0;
    const T* Iw = ADJ ? Cwi : Cw;
    const T* Ih = ADJ ? Chi : Ch;
    const T* Id = ADJ ? Cdi : Cd;
    const T* Ow = ADJ ? Cw : Cwi;
    const T* Oh = ADJ ? Ch : Chi;
    const T* Od = ADJ ? Cd : Cdi;

    __syncthreads();  // the previous tile is done with shared memory
    for (int i = tid; i < ninj * KXT; i += kModalThreads) {
      const int s = i / KXT, kl = i - s * KXT, kx = tl.y * KXT + kl;
      const PointDev q = injp[s];
      if constexpr (ADJ) {
        const T v = a.resid[t * a.n_rec_total + q.slot];
        cws[s * 128 + kl] = kx < w ? (T)D.si * v * Iw[(long long)kx * w + q.x] : (T)0;
      } else {
        const float v = (t < a.max_steps) ? a.series[(long long)q.slot * a.max_steps + t] : 0.0f;
        cws[s * 128 + kl] = kx < w ? (T)D.sf * (T)v * Iw[(long long)kx * w + q.x] : (T)0;
      }
      if (kl == 0) { pts_y[0][s] = q.y; pts_z[0][s] = q.z; }
    }
    for (int i = tid; i < nout * KXT; i += kModalThreads) {
      const int r = i / KXT, kl = i - r * KXT, kx = tl.y * KXT + kl;
      const PointDev q = outp[r];
      cwr[r * 128 + kl] = kx < w ? Ow[(long long)kx * w + q.x] : (T)0;
      if (kl == 0) { pts_y[1][r] = q.y; pts_z[1][r] = q.z; }
    }
    __syncthreads();

    T cx[4][3];
    bool act[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      act[e] = rowok && (kx0 + e < w);
      const int kxe = min(kx0 + e, w - 1);
#pragma unroll
      for (int n = 0; n < 3; ++n) cx[e][n] = Cw[(long long)kxe * w + n];
    }
    const T wx0 = (kx0 == 0) ? (T)0.5 : (T)1;   // REDFT01 halves the k = 0 row
    const int kyc = rowok ? ky : 0;
    T cy[3];
#pragma unroll
    for (int n = 0; n < 3; ++n) cy[n] = Ch[(long long)kyc * h + n];
    const T wy = (ky == 0) ? (T)0.5 : (T)1;
    // the REDFT01 halving of the k = 0 rows sits in the contraction (forward)
    // or in the expansion (adjoint)
    const T wxc = ADJ ? (T)1 : wx0, wyc = ADJ ? (T)1 : wy;
    const int pyr = ky & 1;
    const long long planeX = (long long)d * h, planeY = (long long)d * wp, planeZ = (long long)h * wp;
    const T* PX = buf + D.PX;
    const T* PYr = buf + D.PY + pyr * 3 * planeY;
    T pz[2][3][4], rz[2][3][4];
#pragma unroll
    for (int pm = 0; pm < 2; ++pm)
#pragma unroll
      for (int n = 0; n < 3; ++n) {
        if (lanok) {
          load4(buf + D.PZ + (pm * 3 + n) * planeZ + (long long)ky * wp + kx0, pz[pm][n]);
        } else {
#pragma unroll
          for (int e = 0; e < 4; ++e) pz[pm][n][e] = 0;
        }
#pragma unroll
        for (int e = 0; e < 4; ++e) rz[pm][n][e] = 0;
      }
    T racc[kMaxPointsPerPart];
#pragma unroll
    for (int r = 0; r < kMaxPointsPerPart; ++r) racc[r] = 0;
    const T* Mcur = buf + (ADJ ? D.AM[a.par ^ 1] : D.M[a.par ^ 1]);   // M(t-1) (adjoint: mu(t+1))
    T* Mout = buf + (ADJ ? D.AM[a.par] : D.M[a.par]);                 // M(t-2) -> M(t) (adjoint: mu(t+2) -> mu(t))
    const T* tabA = buf + D.tabA;
    const T* tabB = buf + D.tabB;
    const T damping = (T)D.damping;

    // ky contraction.  A warp holds rpw = 32 / G ky rows; with G = 8 the rows
    // r and r + 2 (same parity) are folded by one shuffle, so every warp leaves
    // rfold <= 2 partial rows in the slot, at [(warp rfold + row) 3 + n][kxt].
    // Rows past h carry zeros (their modes are masked).  The parity of a
    // partial row is (warp rpw + row) & 1 (ky0 is even).  Reducers: one
    // thread per (parity pm, n, kx quad) sums the warps' partials of parity pm
    // (start (pm 3 + n) kxt + 4 kq, stride 6 kxt: 8 terms, or 4 when a warp
    // holds a single row and only every other warp has parity pm).
    const int rpw = 32 / G;
    const int rfold = rpw < 2 ? rpw : 2;
    const int yrow = lane / G;                       // row within the warp
    const bool ywrite = yrow < rfold;
    const int yslot = (warp * rfold + (ywrite ? yrow : 0)) * 3 * KXT + kl0;
    const int nquad = KXT / 4;
    const int yterms = rfold == 2 ? 8 : 4;
    int ysrc = -1;
    T* ydst = buf;
    if (tid < 6 * nquad) {
      const int pm = tid / (3 * nquad);
      const int rem = tid - pm * 3 * nquad;
      const int n = rem / nquad, kq = rem - n * nquad;
      const int kx = tl.y * KXT + 4 * kq;
      if (kx < wp) {
        ysrc = (pm * 3 + n) * KXT + 4 * kq;
        ydst = buf + D.RY + ((long long)tl.z * 6 + pm * 3 + n) * planeY + kx;
      }
    }
    // kx contraction output of this lane (after the reduce-scatter below):
    // q = parity 3 + n for lanes whose low bits below G / 8 are zero
    const int xq = li / (G >> 3);
    const bool xwrite = rowok && (li & ((G >> 3) - 1)) == 0 && xq < 6;
    T* const xdst = buf + D.RX + ((long long)tl.y * 6 + (xwrite ? xq : 0)) * planeX + (rowok ? ky : 0);

    // per-plane inputs of plane kz into stage buffer sb (asynchronous)
    auto issue = [&](int kz, int sb) {
      T* st = stage + sb * kModalStage;
      const long long row = ((long long)kz * h + (rowok ? ky : 0)) * wp + (lanok ? kx0 : 0);
      cp_async4(st + (0 * kModalThreads + tid) * 4, Mcur + row, lanok);
      cp_async4(st + (1 * kModalThreads + tid) * 4, Mout + row, lanok);
      cp_async4(st + (2 * kModalThreads + tid) * 4, tabA + row, lanok);
      cp_async4(st + (3 * kModalThreads + tid) * 4, tabB + row, lanok);
#pragma unroll
      for (int n = 0; n < 3; ++n)
        cp_async4(st + ((4 + n) * kModalThreads + tid) * 4,
                  PYr + n * planeY + (long long)kz * wp + (lanok ? kx0 : 0), lanok);
      if (li < 6) {
        const int pm = li / 3, n = li - pm * 3;
        cp_async_scalar(st + 7 * 4 * kModalThreads + rs * 6 + li,
                        PX + (pm * 3 + n) * planeX + (long long)kz * h + (rowok ? ky : 0), rowok);
      }
      if (lane < 3) cp_async_scalar(st + kModalStageCz + warp * 4 + lane, Cd + (long long)kz * d + lane, true);
    };

    auto body = [&](auto parity, int kz, int sb) {
      constexpr int PZ = decltype(parity)::value;  // kz & 1 (kz0 is even)
      const T* st = stage + sb * kModalStage;
      T cz[3];
#pragma unroll
      for (int n = 0; n < 3; ++n) cz[n] = st[kModalStageCz + warp * 4 + n];
      const T wz = (kz == 0) ? (T)0.5 : (T)1;
      const T wzc = ADJ ? (T)1 : wz;
      T px[2][3];
#pragma unroll
      for (int pm = 0; pm < 2; ++pm)
#pragma unroll
        for (int n = 0; n < 3; ++n) px[pm][n] = st[7 * 4 * kModalThreads + rs * 6 + pm * 3 + n];
      T py[3][4];
      T m[4], mp[4], ta[4], tb[4];
      const long long row = ((long long)kz * h + ky) * wp + kx0;
      load4(st + (0 * kModalThreads + tid) * 4, m);
      load4(st + (1 * kModalThreads + tid) * 4, mp);
      load4(st + (2 * kModalThreads + tid) * 4, ta);
      load4(st + (3 * kModalThreads + tid) * 4, tb);
#pragma unroll
      for (int n = 0; n < 3; ++n) load4(st + ((4 + n) * kModalThreads + tid) * 4, py[n]);
      if (!lanok) {
#pragma unroll
        for (int e = 0; e < 4; ++e) tb[e] = 1;  // keeps the reference arithmetic finite on idle lanes
      }
      T F[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        if constexpr (ADJ) {
          T fx = 0, fy = 0, fz = 0;
#pragma unroll
          for (int n = 0; n < 3; ++n) {
            fx += cx[e][n] * px[e & 1][n];
            fy += cy[n] * py[n][e];
            fz += cz[n] * pz[PZ][n][e];
          }
          F[e] = (e == 0 ? wx0 : (T)1) * fx + wy * fy + wz * fz;
        } else {
          T f = 0;
#pragma unroll
          for (int n = 0; n < 3; ++n) f += cx[e][n] * px[e & 1][n];
#pragma unroll
          for (int n = 0; n < 3; ++n) f += cy[n] * py[n][e];
#pragma unroll
          for (int n = 0; n < 3; ++n) f += cz[n] * pz[PZ][n][e];
          F[e] = f;
        }
      }
      for (int s = 0; s < ninj; ++s) {
        const T coef = Ih[(long long)kyc * h + pts_y[0][s]] * Id[(long long)kz * d + pts_z[0][s]];
        T c[4];
        load4(cws + s * 128 + kl0, c);
#pragma unroll
        for (int e = 0; e < 4; ++e) F[e] += c[e] * coef;
      }
      T Mn[4];
      if constexpr (ADJ) {
        T beta[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          T v;
          if (REF) {
            v = damping * ((T)2 * m[e] * ta[e] - mp[e]) + F[e];
            beta[e] = damping * ((T)2 / tb[e]) * ((T)1 - ta[e]);
          } else {
            v = damping * (((T)2 * m[e] - mp[e]) - (T)2 * ta[e] * m[e]) + F[e];
            beta[e] = damping * tb[e];
          }
          Mn[e] = act[e] ? v : (T)0;
        }
        if (lanok) store4(Mout + row, Mn);
#pragma unroll
        for (int e = 0; e < 4; ++e) Mn[e] *= beta[e];   // contracted: the adjoint of the force mode
      } else {
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          T v;
          if (REF)  // dct_partition.cpp:68: a (2 M cwt - M_prev + (2 F / w2) (1 - cwt))
            v = damping * ((T)2 * m[e] * ta[e] - mp[e] + ((T)2 * F[e] / tb[e]) * ((T)1 - ta[e]));
          else      // the same recurrence with ta = 1 - cwt, tb = 2 (1 - cwt) / w2
            v = damping * (((T)2 * m[e] - mp[e]) - (T)2 * ta[e] * m[e] + tb[e] * F[e]);
          Mn[e] = act[e] ? v : (T)0;
        }
        if (lanok) store4(Mout + row, Mn);
      }
      // contraction along kz (registers) and ky (folded partial rows in the slot)
      T* slot = ry_s + PZ * kModalRySlot;
      {
        T ry[3][4];
#pragma unroll
        for (int n = 0; n < 3; ++n)
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            rz[PZ][n][e] += wzc * cz[n] * Mn[e];
            ry[n][e] = wyc * cy[n] * Mn[e];
          }
        if (rfold == 2 && rpw == 4) {
#pragma unroll
          for (int n = 0; n < 3; ++n)
#pragma unroll
            for (int e = 0; e < 4; ++e) ry[n][e] += __shfl_xor_sync(0xffffffffu, ry[n][e], 16);
        }
        if (ywrite) {
#pragma unroll
          for (int n = 0; n < 3; ++n) store4(slot + yslot + n * KXT, ry[n]);
        }
      }
      // contraction along kx: even / odd kx sums v[q], q = parity 3 + n (two
      // zero pads), then a reduce-scatter over the row's G lanes: three
      // halving exchanges leave lane li with q = li / (G / 8), completed by a
      // butterfly over the G / 8 lanes that share it
      {
        T v[8];
#pragma unroll
        for (int n = 0; n < 3; ++n) {
          v[n] = wxc * cx[0][n] * Mn[0] + cx[2][n] * Mn[2];
          v[3 + n] = cx[1][n] * Mn[1] + cx[3][n] * Mn[3];
        }
        v[6] = 0;
        v[7] = 0;
        const int o4 = G >> 1, o2 = G >> 2, o1 = G >> 3;
        const bool u4 = (li & o4) != 0, u2 = (li & o2) != 0, u1 = (li & o1) != 0;
        T h4[4], h2[2];
#pragma unroll
        for (int i = 0; i < 4; ++i)
          h4[i] = (u4 ? v[4 + i] : v[i]) + __shfl_xor_sync(0xffffffffu, u4 ? v[i] : v[4 + i], o4);
#pragma unroll
        for (int i = 0; i < 2; ++i)
          h2[i] = (u2 ? h4[2 + i] : h4[i]) + __shfl_xor_sync(0xffffffffu, u2 ? h4[i] : h4[2 + i], o2);
        T h1 = (u1 ? h2[1] : h2[0]) + __shfl_xor_sync(0xffffffffu, u1 ? h2[0] : h2[1], o1);
        for (int o = o1 >> 1; o > 0; o >>= 1) h1 += __shfl_xor_sync(0xffffffffu, h1, o);
        if (xwrite) xdst[(long long)kz * h] = h1;
      }
      for (int r = 0; r < nout; ++r) {
        const T coef = Oh[(long long)kyc * h + pts_y[1][r]] * Od[(long long)kz * d + pts_z[1][r]];
        T c[4];
        load4(cwr + r * 128 + kl0, c);
        racc[r] += coef * (c[0] * Mn[0] + c[1] * Mn[1] + c[2] * Mn[2] + c[3] * Mn[3]);
      }
      __syncthreads();
      // ky contraction of this kz: sums of the warps' partial rows of parity pm
      if (ysrc >= 0) {
        T sum[4] = {0, 0, 0, 0};
        for (int k = 0; k < yterms; ++k) {
          T p4[4];
          load4(slot + ysrc + k * 6 * KXT, p4);
#pragma unroll
          for (int e = 0; e < 4; ++e) sum[e] += p4[e];
        }
        store4(ydst + (long long)kz * wp, sum);
      }
    };

    // software pipeline: plane kz+1 loads while plane kz computes
    issue(kz0, 0);
    cp_async_commit();
    for (int kz = kz0; kz < kz1; kz += 2) {
      if (kz + 1 < kz1) issue(kz + 1, 1);
      cp_async_commit();
      cp_async_wait<1>();
      __syncwarp();
      body(std::integral_constant<int, 0>{}, kz, 0);
      if (kz + 1 < kz1) {
        if (kz + 2 < kz1) issue(kz + 2, 0);
        cp_async_commit();
        cp_async_wait<1>();
        __syncwarp();
        body(std::integral_constant<int, 1>{}, kz + 1, 1);
      }
    }
    cp_async_wait<0>();
    if (lanok) {
#pragma unroll
      for (int pm = 0; pm < 2; ++pm)
#pragma unroll
        for (int n = 0; n < 3; ++n)
          store4(buf + D.RZ + ((long long)tl.w * 6 + pm * 3 + n) * planeZ + (long long)ky * wp + kx0, rz[pm][n]);
    }
    if (nout > 0) {
#pragma unroll
      for (int r = 0; r < kMaxPointsPerPart; ++r) {
        if (r < nout) {
          const T s = warp_sum(racc[r]);
          if (lane == 0) red[warp * kMaxPointsPerPart + r] = s;
        }
      }
      __syncthreads();
      if (tid < nout) {
        T s = 0;
        for (int k = 0; k < kModalThreads / 32; ++k) s += red[k * kMaxPointsPerPart + tid];
        const int local = (tl.y * D.nby + tl.z) * D.nbz + tl.w;
        buf[(ADJ ? D.srcpart : D.recpart) + (long long)local * nout + tid] = s;
      }
    }
  }
}


// ---------------------------------------------------------------------------
// PML
// ---------------------------------------------------------------------------

// Forward PML history kept for the adjoint's damping gradient: for steps
// t0 <= t < t1 the PML kernel also writes p(t) to p[(t - t0 + 1) hlen + ...]
// and phi_n(t) to phn[(t - t0) hlen + ...] (all-slab region layout, slab at
// PmlDev::hoff).  p == null: nothing is kept.
// Strip forces: for steps ft0 <= t < ft1 the kernel also writes the strip
// force it reads (the interfaces' forcing of step t-1) to f[(t - ft0) flen +
// PmlDev::foff + ...]; with fsrc set it reads the strip force of step t from
// fsrc[(t - fs0) flen + ...] instead of the context's strips (the PML runs
// again on its own, replaying the recorded forcing).
template <typename T>
struct PmlHist {
  T* p;
  T* phn;
  long long hlen;
  long long t0, t1;
  T* f;
  long long flen;
  long long ft0, ft1;
  const T* fsrc;
  long long fs0;
};

template <typename T>
struct PmlArgs {
  T* buf;
  const PmlDev* pml;
  const int4* blocks;   // {slab, a0, b0}: 8 x 32 plane tiles
  int nblocks;
  int par;
  T dt, dh, c0;
  const PmlHist<T>* hist;   // null without the adjoint
  const long long* tcount;
  int tstep;
  const CUtensorMap* maps;  // per slab: p[0], p[1], pha[0], pha[1], phb[0], phb[1] as [L][A][B] tensors
  int* err;                 // set to 1 when a bounded wait runs out
};

// Plane tiles of the PML kernel and the boxes the TMA unit loads per layer:
// p with a halo of 3 along a and of 4 / 4 along b (x starts at b0 - 4, on a
// 16-byte boundary), phi_a with a halo of 2 along a, phi_b with a halo of 4 /
// 4 along b; each box 128-byte aligned in the stage.
constexpr int kPmlTA = 8, kPmlTB = 32;
template <typename T>
struct PmlStage {
  static constexpr int PW = kPmlTB + 8;                                  // p and phi_b box width
  static constexpr int ps = (kPmlTA + 6) * PW * (int)sizeof(T);
  static constexpr int psa = (ps + 127) & ~127;
  static constexpr int fa = (kPmlTA + 4) * kPmlTB * (int)sizeof(T);
  static constexpr int fb = kPmlTA * PW * (int)sizeof(T);
  static constexpr int fba = (fb + 127) & ~127;
  static constexpr int bytes = psa + fa + fba;
  static constexpr int tx = ps + fa + fb;                                 // bytes the three boxes deliver
};

// Grote-Sim PML (pml_partition.cpp:113-200) in slab coordinates: layer l
// along the normal, (a, b) in the plane; outside the slab every field reads
// zero (the reference's sentinel cell).  Only the normal damping zeta_n is
// non-zero in a slab (zeta_a = zeta_b = 0 in the reference's formulas).
// A block owns an 8 x 32 plane tile and walks the layers.  The in-plane
// stencils read tiles of p(t-1) (halo 3), phi_a and phi_b (halo 2 along
// their own axis) that the TMA unit brings into a two-stage ring of shared
// memory, one layer ahead, across the block's tiles; the tensor maps'
// zero fill outside the slab is the sentinel.  The normal-axis stencils run
// from register windows; p(t-2) and the strip force of the next layer are
// fetched into registers while the current one computes.  Every wait is
// bounded: one that runs out sets the kernel's error word and the block
// leaves its loops.
template <typename T>
__global__ void __launch_bounds__(256, 4) pml_kernel(PmlArgs<T> a) {
  grid_dependency_wait();
  using S = PmlStage<T>;
  constexpr int TA = kPmlTA, TB = kPmlTB, PW = S::PW;
  __shared__ __align__(128) unsigned char stage[2][S::bytes];
  __shared__ uint64_t bar[2];
  __shared__ volatile int s_abort;
  const T c7[7] = {2, -27, 270, -490, 270, -27, 2};
  const T c5[5] = {1, -8, 0, 8, -1};
  const int tb = threadIdx.x & 31, ta = threadIdx.x >> 5;
  T* hp = nullptr;
  T* hfn = nullptr;
  T* hf = nullptr;
  const T* fsrc = nullptr;
  if (a.hist) {
    const PmlHist<T> h = *a.hist;
    const long long t = *a.tcount + a.tstep;
    if (h.p && t >= h.t0 && t < h.t1) {
      hp = h.p + (t - h.t0 + 1) * h.hlen;
      hfn = h.phn + (t - h.t0) * h.hlen;
    }
    if (h.f && t >= h.ft0 && t < h.ft1) hf = h.f + (t - h.ft0) * h.flen;
    if (h.fsrc) fsrc = h.fsrc + (t - h.fs0) * h.flen;
  }
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    mbar_init_fence();
    s_abort = 0;
  }
  __syncthreads();
  // thread 0's issue cursor: the block's (tile, layer) sequence, one layer
  // ahead of the computation (two stages)
  int ibi = blockIdx.x, il = 0, iL = 0;
  uint32_t issued = 0;
  const int lev = a.par ^ 1;   // time level t-1 of p, phi_a, phi_b
  auto issue_next = [&]() {
    if (ibi >= a.nblocks) return;
    const int4 blk = a.blocks[ibi];
    if (il == 0) iL = a.pml[blk.x].L;
    const CUtensorMap* mp = a.maps + 6LL * blk.x;
    const int sg = (int)(issued & 1);
    unsigned char* sb = stage[sg];
    mbar_arrive_expect_tx(&bar[sg], (uint32_t)S::tx);
    tma_load_3d(sb, mp + lev, blk.z - 4, blk.y - 3, il, &bar[sg]);
    tma_load_3d(sb + S::psa, mp + 2 + lev, blk.z, blk.y - 2, il, &bar[sg]);
    tma_load_3d(sb + S::psa + S::fa, mp + 4 + lev, blk.z - 4, blk.y, il, &bar[sg]);
    ++issued;
    if (++il == iL) {
      il = 0;
      ibi += gridDim.x;
    }
  };
  if (threadIdx.x == 0) {
    issue_next();
    issue_next();
  }
  uint32_t used = 0;   // layers consumed by the block (uniform)
  bool stop = false;
  for (int bi = blockIdx.x; bi < a.nblocks && !stop; bi += gridDim.x) {
    const int4 blk = a.blocks[bi];
    const PmlDev& P = a.pml[blk.x];
    const int L = P.L, A = P.A, B = P.B, Bp = P.Bp;
    const int strip0 = P.strip0;       // held in registers: the layer loop stores through the pool pointer
    const long long hoff = P.hoff;
    const int a0 = blk.y, b0 = blk.z;
    const int ia = a0 + ta, ib = b0 + tb;
    const bool inside = ia < A && ib < B;
    const long long lstride = (long long)A * Bp;
    const long long col = inside ? (long long)ia * Bp + ib : 0;
    const T* p = a.buf + P.p[a.par ^ 1];   // p(t-1)
    T* pn = a.buf + P.p[a.par];            // p(t-2) -> p(t)
    const T* fn = a.buf + P.phn[a.par ^ 1];
    T* fn_o = a.buf + P.phn[a.par];
    T* fa_o = a.buf + P.pha[a.par];
    T* fb_o = a.buf + P.phb[a.par];
    const T* zeta = a.buf + P.zeta;
    const T* force = fsrc ? fsrc + P.foff : a.buf + P.force;
    T* force_rec = hf ? hf + P.foff : nullptr;
    // register windows along the normal: p(l-3 .. l+3), phi_n(l-2 .. l+2)
    T pw[7], fw[5];
#pragma unroll
    for (int m = 0; m < 7; ++m) {
      const int ll = m - 3;
      pw[m] = (inside && ll >= 0 && ll < L) ? p[ll * lstride + col] : (T)0;
    }
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      const int ll = m - 2;
      fw[m] = (inside && ll >= 0 && ll < L) ? fn[ll * lstride + col] : (T)0;
    }
    const T r180 = (T)1 / ((T)180 * a.dh * a.dh), r12 = (T)1 / ((T)12 * a.dh), rdt = (T)1 / a.dt;
    T nold = 0, nforce = 0;
    auto fetch = [&](int l) {
      const int sl = l - strip0;
      nold = inside ? pn[l * lstride + col] : (T)0;
      nforce = (inside && sl >= 0 && sl < 3) ? force[sl * lstride + col] : (T)0;
    };
    fetch(0);
    for (int l = 0; l < L; ++l) {
      const int sg = (int)(used & 1);
      mbar_wait_bounded(&bar[sg], (used >> 1) & 1, &s_abort);
      const T* Ps = reinterpret_cast<const T*>(stage[sg]);                    // [TA + 6][PW], b from b0 - 4
      const T* FA = reinterpret_cast<const T*>(stage[sg] + S::psa);           // [TA + 4][TB], b from b0
      const T* FB = reinterpret_cast<const T*>(stage[sg] + S::psa + S::fa);   // [TA][PW], b from b0 - 4
      const T pold = nold, f = nforce;
      if (l + 1 < L) fetch(l + 1);
      if (force_rec && inside) {
        const int sl = l - strip0;
        if (sl >= 0 && sl < 3) force_rec[sl * lstride + col] = f;
      }
      if (inside && !s_abort) {
        T ln = 0, la = 0, lb = 0;
#pragma unroll
        for (int m = 0; m < 7; ++m) {
          ln += c7[m] * pw[m];
          la += c7[m] * Ps[(ta + m) * PW + tb + 4];
          lb += c7[m] * Ps[(ta + 3) * PW + tb + 1 + m];
        }
        T un = 0, ua = 0, ub = 0, gn = 0, ga = 0, gb = 0;
#pragma unroll
        for (int m = 0; m < 5; ++m) {
          un += c5[m] * pw[m + 1];
          ua += c5[m] * Ps[(ta + 1 + m) * PW + tb + 4];
          ub += c5[m] * Ps[(ta + 3) * PW + tb + 2 + m];
          gn += c5[m] * fw[m];
          ga += c5[m] * FA[(ta + m) * TB + tb];
          gb += c5[m] * FB[ta * PW + tb + 2 + m];
        }
        ln *= r180; la *= r180; lb *= r180;
        un *= r12; ua *= r12; ub *= r12;
        gn *= r12; ga *= r12; gb *= r12;
        const long long I = l * lstride + col;
        const T zn = zeta[l];
        const T pcur = pw[3];
        const T t3 = a.c0 * a.c0 * (ln + la + lb);
        const T t4 = -zn * (pcur - pold) * rdt;
        const T pnew = (T)2 * pcur - pold + a.dt * a.dt * (t3 + t4 + (gn + ga + gb) + f);
        pn[I] = pnew;
        const T fnc = fw[2];
        const T fnew = fnc - a.dt * zn * fnc + a.dt * (-zn) * un;
        fn_o[I] = fnew;
        if (hp) {
          hp[hoff + I] = pnew;
          hfn[hoff + I] = fnew;
        }
        fa_o[I] = FA[(ta + 2) * TB + tb] + a.dt * zn * ua;
        fb_o[I] = FB[ta * PW + tb + 4] + a.dt * zn * ub;
      }
      // slide the windows one layer
#pragma unroll
      for (int m = 0; m < 6; ++m) pw[m] = pw[m + 1];
      pw[6] = (inside && l + 4 < L) ? p[(l + 4) * lstride + col] : (T)0;
#pragma unroll
      for (int m = 0; m < 4; ++m) fw[m] = fw[m + 1];
      fw[4] = (inside && l + 3 < L) ? fn[(l + 3) * lstride + col] : (T)0;
      __syncthreads();   // every thread is done with stage sg
      if (s_abort) {
        stop = true;
        break;
      }
      if (threadIdx.x == 0) issue_next();
      ++used;
    }
  }
  if (s_abort) {
    // a wait ran out: report it, and give loads still in flight time to land
    // (bounded) before the block's shared memory is released
    if (threadIdx.x == 0) {
      atomicExch(a.err, 1);
      const long long t0 = clock64();
      while (clock64() - t0 < 20000000LL) {
      }
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Interfaces
// ---------------------------------------------------------------------------

template <typename T>
struct IfaceArgs {
  T* buf;
  const IfaceDev* ifs;
  const int* cell_iface;   // interface of every face cell
  long long total;
  const unsigned char* masks;
  int par;
  T c0, dh;
};

// Offset of the force value of crossing coordinate c, face coordinates
// (u, v) on side S (see SideDev), -1 for an air cell off the shell.
__device__ __forceinline__ long long side_force_offset(const SideDev& S, int type, int c, int u, int v) {
  if (S.kind == 1) return S.fb + (long long)c * S.fls + (long long)v * S.fsv + u;
  const int x = type == 0 ? c : u;
  const int y = type == 0 ? u : (type == 1 ? c : v);
  const int z = type == 2 ? c : v;
  int l = face_layer(x, S.w);
  if (l >= 0) return S.fx + ((long long)l * S.d + z) * S.h + y;
  l = face_layer(y, S.h);
  if (l >= 0) return S.fy + ((long long)l * S.d + z) * S.wp + x;
  l = face_layer(z, S.d);
  if (l >= 0) return S.fz + ((long long)l * S.h + y) * S.wp + x;
  return -1;
}

// Boundary::ComputeForcingTerms (boundary.cpp:21-173) for every face cell of
// every interface; the per-cell mask keeps only the writes that survive the
// reference's list-order overwrites.
template <typename T>
__global__ void __launch_bounds__(256) iface_kernel(IfaceArgs<T> a) {
  grid_dependency_wait();
  const T C[6][6] = {{0, 0, -2, 2, 0, 0},       {0, -2, 27, -27, 2, 0},     {-2, 27, -270, 270, -27, 2},
                     {2, -27, 270, -270, 27, -2}, {0, 2, -27, 27, -2, 0},     {0, 0, 2, -2, 0, 0}};
  const T k0 = a.c0 * a.c0 / ((T)180 * a.dh * a.dh);
  for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x; g < a.total;
       g += (long long)gridDim.x * blockDim.x) {
    const IfaceDev& I = a.ifs[a.cell_iface[g]];
    const int local = (int)(g - I.cell0);   // cells of one interface: a face area, 32-bit
    const int nu = I.u1 - I.u0;
    const int iv_l = local / nu;
    const int iu = I.u0 + (local - iv_l * nu);
    const int iv = I.v0 + iv_l;
    const unsigned mask = a.masks[I.mask + local];
    const int lu = iu - I.lo.ou, lv = iv - I.lo.ov;
    const int hu = iu - I.hi.ou, hv = iv - I.hi.ov;
    T pl[3], ph[3];
#pragma unroll
    for (int n = 0; n < 3; ++n) {
      pl[n] = a.buf[I.lo.pb[n][a.par] + (long long)lv * I.lo.psv + lu];
      ph[n] = a.buf[I.hi.pb[n][a.par] + (long long)hv * I.hi.psv + hu];
    }
    const T absorp = (T)I.absorption;
    // every offset and value first, the six stores after them: a store
    // through the pool pointer may alias the descriptor table as far as the
    // compiler can tell, so descriptor fields read after a store are loaded
    // again
    long long o[6];
    T val[6];
#pragma unroll
    for (int m = -3; m < 3; ++m) {
      o[m + 3] = -1;
      val[m + 3] = 0;
      if (!(mask & (1u << (m + 3)))) continue;
      T sip1 = 0, sip2 = 0;
#pragma unroll
      for (int n = 0; n < 3; ++n) sip1 += C[m + 3][n] * pl[n];
#pragma unroll
      for (int n = 3; n < 6; ++n) sip2 += C[m + 3][n] * ph[n - 3];
      T sip;
      if (m < 0) {
        sip = I.lo.self ? (sip1 + sip2) : sip2;
        o[m + 3] = side_force_offset(I.lo, I.type, I.lo.ext + m, lu, lv);
      } else {
        sip = I.hi.self ? (sip1 + sip2) : sip1;
        o[m + 3] = side_force_offset(I.hi, I.type, m, hu, hv);
      }
      val[m + 3] = absorp * (sip * k0);
    }
#pragma unroll
    for (int m = 0; m < 6; ++m)
      if (o[m] >= 0) a.buf[o[m]] = val[m];
  }
}

static __global__ void advance_time_kernel(long long* tcount, int n) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *tcount += n;
}

// ---- setup kernels (FP64 arithmetic) ----

// Per extent n, four n*n tables: C[k][j] = 2 cos(pi (j + 1/2) k / n) (the
// REDFT10 matrix), the REDFT01 matrix Ci[k][j] = C[k][j] with row k = 0
// halved (REDFT01 weights X_0 by 1, the others by 2), and the transposes of
// both (row-contiguous access for the fused face transforms).
template <typename T>
__global__ void cos_table_kernel(T* buf, long long off, int n) {
  const long long nn = (long long)n * n;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nn; i += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(i / n), j = (int)(i - (long long)k * n);
    const long long q = ((long long)(2 * j + 1) * k) % (4LL * n);  // argument reduced exactly in integers
    const double v = 2.0 * cospi((double)q / (2.0 * n));
    const double vi = k == 0 ? 0.5 * v : v;
    const long long t = (long long)j * n + k;
    buf[off + i] = (T)v;
    buf[off + nn + i] = (T)vi;
    buf[off + 2 * nn + t] = (T)v;
    buf[off + 3 * nn + t] = (T)vi;
  }
}

// Accurate-arithmetic tables: tabA = 1 - cos(w dt) = 2 sin^2(w dt / 2),
// tabB = 2 (1 - cos(w dt)) / w^2, in FP64 then rounded to T; [d][h][wp],
// padding columns zero.
template <typename T>
__global__ void modal_table_kernel(T* buf, long long tabA, long long tabB, int w, int wp, int h, int d, double dh,
                                   double dt, double c0) {
  const long long N = (long long)wp * h * d;
  const double lx = w * dh, ly = h * dh, lz = d * dh;
  const double pi = 3.14159265358979323846;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (long long)gridDim.x * blockDim.x) {
    const int kx = (int)(i % wp);
    const int ky = (int)((i / wp) % h);
    const int kz = (int)(i / ((long long)wp * h));
    if (kx >= w) { buf[tabA + i] = 0; buf[tabB + i] = 0; continue; }
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
