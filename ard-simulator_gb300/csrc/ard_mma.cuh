// Face transforms of the step on the 5th-generation tensor cores (sm_103a):
// tcgen05.mma with TMEM accumulators, operands staged in shared memory in the
// 128-byte-swizzled K-major layout, in split TF32 precision.
//
// Every pass of the two-pass 2D face transform is one batched product
//     D[m][n] = scale * sum_k Data[m][k] * Table[n][k]
// with both operands contiguous along k:
//   Data   rows of a face layer (or of the transposed intermediate), up to six
//          layer outputs stacked along m, optionally the sum / difference of
//          two layers (the layer pairs n, 5 - n);
//   Table  the transform matrix with the output index as row: C (REDFT10)
//          for the forward passes, Ci^T (REDFT01, transposed) for the inverse.
// The result is written transposed, out[n][m] (row pitch ldo), which is what
// the next pass reads contiguously along its own k:
//   forward  X[v][u] -> T^T[ku][v] = sum_u C_U[ku][u] X[v][u]
//            T^T[ku][v] -> F[kv][ku] = sum_v C_V[kv][v] T^T[ku][v]
//   inverse  R[kv][ku] -> Y^T[u][kv] = sum_ku Ci_U[ku][u] R[kv][ku]
//            Y^T[u][kv] -> p[v][u] = sum_kv Ci_V[kv][v] Y^T[u][kv]
//
// Split precision (3xTF32): x = hi + lo with hi = tf32(x), lo = tf32(x - hi);
// the product is hi*hi + hi*lo + lo*hi accumulated in FP32 (the lo*lo term,
// ~2^-22 relative, is dropped), which keeps FP32-level accuracy.  The tables
// are split once at context creation (FP64 values), the data while staged.
//
// One CTA (8 warps) per SM, persistent over 128 x BN output tiles.  Per 32-wide
// K chunk all warps stage the data tile (128 rows, hi and lo) and the table
// tile (BN rows, hi and lo, cp.async) into one of two stages; thread 0 issues
// 4 k-steps x 3 MMAs (M = 128, N = BN, K = 8) into the TMEM accumulator and
// commits them to the stage's mbarrier, so the next chunk is staged while the
// MMAs run.  The epilogue reads the accumulator with tcgen05.ld (warp w reads
// TMEM lanes 32 (w % 4) .. +31, every other 16-column group by w / 4).
// Every mbarrier wait is bounded by a clock limit; a wait that runs out sets
// the kernel's error word, and the CTA frees its TMEM and returns.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "ard_device.cuh"
#include "ard_kernels.cuh"

namespace ard {

constexpr int kMmaThreads = 256;
constexpr int kMmaBK = 32;              // K chunk: one 128-byte swizzle row of fp32 / tf32
constexpr int kMmaBNMax = 160;          // widest N tile
constexpr int kMmaStages = 2;
constexpr int kMmaTileA = 128 * kMmaBK * 4;          // bytes of one data tile (hi or lo)
constexpr int kMmaTileB = kMmaBNMax * kMmaBK * 4;    // bytes of one table tile (hi or lo)
constexpr int kMmaStageBytes = 2 * kMmaTileA + 2 * kMmaTileB;
constexpr int kMmaSmemBytes = kMmaStages * kMmaStageBytes + 1024 /* alignment */ + 64 /* barriers */;
constexpr int kMmaTmemCols = 256;
struct MmaArgs {
  float* buf;
  const MmaJob* jobs;
  int njobs;
  int total;        // tiles of all jobs
  int* err;         // set to 1 when a bounded wait runs out
};

// ---- PTX wrappers ----
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint32_t tf32_rna(float x) {
  uint32_t u;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(u) : "f"(x));
  return u;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Waits for the phase of `parity` to complete; false after ~1 s of SM clock.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity))
    if (clock64() - t0 > 2000000000LL) return false;
  return true;
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 bytes apart (SBO), start address in 16-byte units; bits 46-47 hold
// the descriptor version (1), bits 61-63 the layout (2: 128-byte swizzle).
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

// Instruction descriptor of kind::tf32: FP32 accumulator (bits 4-5 = 1), A and
// B TF32 (bits 7-9, 10-12 = 2), both K-major (bits 15, 16 = 0), N / 8 at bit
// 17, M / 16 at bit 24.
__host__ __device__ constexpr uint32_t tf32_idesc(int M, int N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// 16 consecutive fp32 columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// byte offset of element (row r, 16-byte chunk c) in a 128-byte-swizzled K-major tile
__device__ __forceinline__ uint32_t sw128_off(int r, int c) { return (uint32_t)(r * 128 + (((c ^ r) & 7) << 4)); }

static __global__ void __launch_bounds__(kMmaThreads, 1) face_mma_kernel(MmaArgs a) {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  extern __shared__ __align__(1024) unsigned char mma_smem_raw[];
  // 1024-byte aligned stage area (the swizzle pattern is anchored at 1024-byte boundaries)
  unsigned char* sm = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(mma_smem_raw) + 1023) & ~(uintptr_t)1023);
  uint64_t* bars = reinterpret_cast<uint64_t*>(sm + kMmaStages * kMmaStageBytes);   // [kMmaStages]
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + kMmaStages);
  constexpr int kMaxCachedJobs = 512;
  __shared__ int sfirst[kMaxCachedJobs];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  float* __restrict__ buf = a.buf;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(kMmaTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    for (int s = 0; s < kMmaStages; ++s) mbar_init(&bars[s], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  const bool cached = a.njobs <= kMaxCachedJobs;
  if (cached)
    for (int i = tid; i < a.njobs; i += kMmaThreads) sfirst[i] = a.jobs[i].first;
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  uint32_t uses[kMmaStages] = {0, 0};   // completed commits per stage (uniform over the CTA)
  uint32_t it = 0;                        // chunks issued by this CTA
  bool aborted = false;                   // a bounded wait ran out (uniform: decided by __syncthreads_or)
  for (int tile = blockIdx.x; tile < a.total; tile += gridDim.x) {
    int lo = 0, hi = a.njobs - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if ((cached ? sfirst[mid] : a.jobs[mid].first) <= tile) lo = mid; else hi = mid - 1;
    }
    const MmaJob& J = a.jobs[lo];
    const int t = tile - J.first;
    const int m0 = (t / J.nt) * 128, n0 = (t % J.nt) * J.bn;
    const int Mtot = J.nout * J.R;
    const int K = J.K;
    // this thread's data rows of the tile (fixed for the tile): rows rr = (tid >> 3) + 32 i, 16-byte chunk tid & 7
    const int cq = tid & 7;
    const float* p0[4];
    const float* p1[4];
    float sg[4];
    bool rok[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int g = m0 + (tid >> 3) + 32 * i;
      rok[i] = g < Mtot;
      const int o = rok[i] ? g / J.R : 0;
      const int r = rok[i] ? g - o * J.R : 0;
      p0[i] = buf + J.in0[o] + (long long)r * J.ldb;
      p1[i] = J.in1[o] >= 0 ? buf + J.in1[o] + (long long)r * J.ldb : nullptr;
      sg[i] = (float)J.sgn[o];
    }
    const int nch = (K + kMmaBK - 1) / kMmaBK;
    const uint32_t idesc = tf32_idesc(128, J.bn);
    for (int c = 0; c < nch; ++c, ++it) {
      const int s = it & 1;
      unsigned char* st = sm + s * kMmaStageBytes;
      unsigned char* Ahi = st;
      unsigned char* Alo = st + kMmaTileA;
      unsigned char* Bhi = st + 2 * kMmaTileA;
      unsigned char* Blo = Bhi + kMmaTileB;
      const bool bad = uses[s] > 0 && !mbar_wait_bounded(&bars[s], (uses[s] - 1) & 1);   // stage free again
      const int k0 = c * kMmaBK;
      // ---- table tile: BN rows x 8 chunks, hi and lo (cp.async, zero-filled outside the table) ----
      for (int e = tid; e < J.bn * 8; e += kMmaThreads) {
        const int r = e >> 3, q = e & 7;
        const int n = n0 + r, k = k0 + 4 * q;
        const bool ok = n < J.N && k < J.tp;
        const long long off = ok ? (long long)n * J.tp + k : 0;
        cp_async16(Bhi + sw128_off(r, q), buf + J.thi + off, ok);
        cp_async16(Blo + sw128_off(r, q), buf + J.tlo + off, ok);
      }
      cp_async_commit();
      // ---- data tile: 128 rows x 8 chunks, split into hi and lo ----
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int r = (tid >> 3) + 32 * i;
        const int k = k0 + 4 * cq;
        float x[4] = {0.f, 0.f, 0.f, 0.f};
        if (rok[i] && k < K) {
          if (J.vec && k + 3 < K) {
            const float4 v = *reinterpret_cast<const float4*>(p0[i] + k);
            x[0] = v.x; x[1] = v.y; x[2] = v.z; x[3] = v.w;
            if (p1[i]) {
              const float4 w = *reinterpret_cast<const float4*>(p1[i] + k);
              x[0] += sg[i] * w.x; x[1] += sg[i] * w.y; x[2] += sg[i] * w.z; x[3] += sg[i] * w.w;
            }
          } else {
#pragma unroll
            for (int j = 0; j < 4; ++j)
              if (k + j < K) x[j] = p1[i] ? p0[i][k + j] + sg[i] * p1[i][k + j] : p0[i][k + j];
          }
        }
        uint32_t h[4], l[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          h[j] = tf32_rna(x[j]);
          l[j] = tf32_rna(x[j] - __uint_as_float(h[j]));
        }
        const uint32_t so = sw128_off(r, cq);
        *reinterpret_cast<uint4*>(Ahi + so) = make_uint4(h[0], h[1], h[2], h[3]);
        *reinterpret_cast<uint4*>(Alo + so) = make_uint4(l[0], l[1], l[2], l[3]);
      }
      cp_async_wait<0>();
      fence_async_smem();   // generic-proxy writes of this stage -> visible to the tensor cores
      if (__syncthreads_or(bad)) { aborted = true; break; }
      if (tid == 0) {
        tc_fence_after();
        const uint32_t ahi = smem_u32(Ahi), alo = smem_u32(Alo), bhi = smem_u32(Bhi), blo = smem_u32(Blo);
#pragma unroll
        for (int j = 0; j < kMmaBK / 8; ++j) {   // k-steps of 8 (32 bytes) inside the swizzled rows
          const uint32_t kb = 32u * j;
          mma_tf32(tmem, sw128_desc(ahi + kb), sw128_desc(bhi + kb), idesc, (c > 0 || j > 0) ? 1u : 0u);
          mma_tf32(tmem, sw128_desc(ahi + kb), sw128_desc(blo + kb), idesc, 1u);
          mma_tf32(tmem, sw128_desc(alo + kb), sw128_desc(bhi + kb), idesc, 1u);
        }
        mma_commit(&bars[s]);
      }
      uses[s] += 1;
    }
    if (aborted) break;
    // ---- epilogue: accumulator -> out[n][m] ----
    {
      const int sl = (it - 1) & 1;
      const bool bad = !mbar_wait_bounded(&bars[sl], (uses[sl] - 1) & 1);
      if (__syncthreads_or(bad)) { aborted = true; break; }
    }
    tc_fence_after();
    const int q = warp & 3;                 // TMEM lane quarter of this warp
    const int m = q * 32 + lane;            // accumulator row = TMEM lane
    const int g = m0 + m;
    const bool mok = g < Mtot;
    const int o = mok ? g / J.R : 0;
    const int r = mok ? g - o * J.R : 0;
    float* outp = buf + J.out[o] + r;
    const float scale = J.scale;
    for (int cg = warp >> 2; cg * 16 < J.bn; cg += 2) {
      float v[16];
      tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(cg * 16), v);
      if (mok) {
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          const int n = n0 + cg * 16 + i;
          if (n < J.N && n - n0 < J.bn) outp[(long long)n * J.ldo] = v[i] * scale;
        }
      }
    }
    tc_fence_before();
    __syncthreads();   // accumulator free for the next tile's MMAs
  }
  if (aborted && tid == 0) atomicExch(a.err, 1);
  // drain: the last commits of this CTA must land before TMEM is freed
  for (int s = 0; s < kMmaStages; ++s)
    if (uses[s] > 0) mbar_wait_bounded(&bars[s], (uses[s] - 1) & 1);
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kMmaTmemCols) : "memory");
  }
}

// FP64 -> split TF32 transform tables for the tensor-core passes, per extent
// n: forward C[k][j] = 2 cos(pi (j + 1/2) k / n) and inverse Ci^T[j][k] =
// Ci[k][j] (row k = 0 halved), each as hi / lo pairs [n][tp] (tp =
// roundup(n, 4), padding columns zero).  Layout at off: Chi, Clo, CiThi, CiTlo.
static __global__ void mma_table_kernel(float* buf, long long off, int n, int tp) {
  const long long nn = (long long)n * tp;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nn; i += (long long)gridDim.x * blockDim.x) {
    const int row = (int)(i / tp), col = (int)(i - (long long)row * tp);
    double c = 0.0, ci = 0.0;
    if (col < n) {
      // forward C[row][col]: k = row, j = col
      const long long q = ((long long)(2 * col + 1) * row) % (4LL * n);
      c = 2.0 * cospi((double)q / (2.0 * n));
      // inverse transposed Ci^T[row][col] = Ci[col][row]: k = col, j = row
      const long long q2 = ((long long)(2 * row + 1) * col) % (4LL * n);
      ci = 2.0 * cospi((double)q2 / (2.0 * n));
      if (col == 0) ci *= 0.5;
    }
    const uint32_t ch = tf32_rna((float)c);
    const uint32_t cl = tf32_rna((float)(c - (double)__uint_as_float(ch)));
    const uint32_t ih = tf32_rna((float)ci);
    const uint32_t il = tf32_rna((float)(ci - (double)__uint_as_float(ih)));
    buf[off + i] = __uint_as_float(ch);
    buf[off + nn + i] = __uint_as_float(cl);
    buf[off + 2 * nn + i] = __uint_as_float(ih);
    buf[off + 3 * nn + i] = __uint_as_float(il);
  }
}

}  // namespace ard
