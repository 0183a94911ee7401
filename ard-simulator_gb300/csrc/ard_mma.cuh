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
// are split once at context creation (from FP64 values) and stored pre-tiled
// in the swizzled shared-memory image, so a K chunk of a table tile is one
// contiguous TMA bulk copy; the data are split while staged.
//
// One CTA per SM, persistent over 128 x BN output tiles, warp-specialized,
// with a ring of kMmaStages shared-memory stages (data hi / lo, table hi / lo):
//   warps 0-7   producers: the raw data of the next kMmaDepth K chunks (128
//               rows x 32 k, across tile boundaries) are in flight in their
//               registers; per chunk they wait for a free stage (empty
//               barrier), split the chunk into hi / lo, store the swizzled
//               images and arrive on the stage's full barrier, then issue
//               the loads of the chunk kMmaDepth ahead; thread 0 brings the
//               chunk's table blocks in by two bulk copies whose bytes the
//               full barrier counts;
//   warp 12     the MMA issuer (one thread): per chunk wait for the full
//               barrier, issue 4 k-steps x 3 MMAs (M = 128, N = BN, K = 8)
//               into one of two TMEM accumulators, commit them to the
//               stage's empty barrier; per tile commit to the accumulator's
//               full barrier;
//   warps 8-11  the epilogue: wait for a full accumulator, read it with
//               tcgen05.ld (warp 8 + q reads TMEM lanes 32 q .. 32 q + 31),
//               scale and store it transposed, release the accumulator.
// The stages only have to cover the MMAs' latency (the loads' latency is
// covered by the register prefetch), and the two accumulators let the
// epilogue of one tile overlap the MMAs of the next.  Every wait is bounded
// by a clock limit; one that runs out raises the CTA's abort flag and the
// kernel's error word, every role leaves its loop, and the CTA frees its
// TMEM and returns.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "ard_device.cuh"
#include "ard_kernels.cuh"

namespace ard {

constexpr int kMmaStages = 3;
constexpr int kMmaProducers = 256;                   // warps 0-7
constexpr int kMmaEpilogueWarp0 = 8;                 // warps 8-11
constexpr int kMmaIssuerWarp = 12;
constexpr int kMmaThreads = 416;
constexpr int kMmaDepth = 2;                         // K chunks whose data loads are in flight per producer thread
constexpr int kMmaTileA = 128 * kMmaBK * 4;          // bytes of one data tile (hi or lo)
constexpr int kMmaTileB = kMmaBNMax * kMmaBK * 4;    // bytes of one table tile (hi or lo)
constexpr int kMmaStageBytes = 2 * kMmaTileA + 2 * kMmaTileB;
constexpr int kMmaBarBytes = 128;
constexpr int kMmaSmemBytes = kMmaStages * kMmaStageBytes + 1024 /* alignment */ + kMmaBarBytes;
constexpr int kMmaAccCols = 256;                     // columns of one accumulator
constexpr int kMmaTmemCols = 2 * kMmaAccCols;

struct MmaArgs {
  float* buf;
  const MmaJob* jobs;
  int njobs;
  int total;        // tiles of all jobs
  int* err;         // set to 1 when a bounded wait runs out
};

// ---- PTX wrappers (the mbarrier and bulk-copy ones are in ard_async.cuh) ----
__device__ __forceinline__ uint32_t tf32_rna(float x) {
  uint32_t u;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(u) : "f"(x));
  return u;
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

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

// byte offset of 16-byte chunk c of row r in a 128-byte-swizzled K-major tile
__device__ __forceinline__ uint32_t sw128_off(int r, int c) { return (uint32_t)(r * 128 + (((c ^ r) & 7) << 4)); }

// The tile's job: binary search of the first tile of every job (cached in
// shared memory when the list is short).
__device__ __forceinline__ int mma_find_job(const MmaArgs& a, const int* sfirst, bool cached, int tile) {
  int lo = 0, hi = a.njobs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if ((cached ? sfirst[mid] : a.jobs[mid].first) <= tile) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// 32 consecutive fp32 columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// A producer thread's view of the tile it is loading: the sources of its four
// data rows and the table blocks of the tile's N tile.
struct MmaRows {
  const float* p0[4];  // row i of the first input
  int d1[4];           // second input - first input (elements)
  const float* thi;    // table hi block of K chunk 0; the lo block is dlo elements further
  int dlo;
  int K;
  uint32_t okm;        // bit i: row i lies inside the job (rows past it read as zeros)
  uint32_t sgm;        // bit i: row i subtracts its second input
  int tile, c, nch;
  uint32_t tbytes;     // bytes of one table block (bn x 32 fp32)
  bool comb, vec;
};

// One prefetched K chunk of a producer thread: its raw data (in0 and in1
// values of its four rows) in registers, and what its conversion needs.
struct MmaSlot {
  float4 x0[4], x1[4];
  const float* thi;
  int dlo;
  uint32_t tbytes;
  uint32_t sgm;
  bool comb, valid;
};

static __global__ void __launch_bounds__(kMmaThreads, 1) face_mma_kernel(MmaArgs a) {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  extern __shared__ __align__(1024) unsigned char mma_smem_raw[];
  // 1024-byte aligned stage area (the swizzle pattern is anchored at 1024-byte boundaries)
  unsigned char* sm = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(mma_smem_raw) + 1023) & ~(uintptr_t)1023);
  uint64_t* full = reinterpret_cast<uint64_t*>(sm + kMmaStages * kMmaStageBytes);   // [kMmaStages]
  uint64_t* empty = full + kMmaStages;                                                // [kMmaStages]
  uint64_t* accfull = empty + kMmaStages;                                             // [2]
  uint64_t* accempty = accfull + 2;                                                   // [2]
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(accempty + 2);
  __shared__ volatile int s_abort;
  constexpr int kMaxCachedJobs = 512;
  __shared__ int sfirst[kMaxCachedJobs];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  float* __restrict__ buf = a.buf;

  if (warp == kMmaIssuerWarp) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(kMmaTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    for (int s = 0; s < kMmaStages; ++s) {
      mbar_init(&full[s], kMmaProducers + 1);   // every producer, plus the arrival that sets the table bytes
      mbar_init(&empty[s], 1);
    }
    for (int q = 0; q < 2; ++q) {
      mbar_init(&accfull[q], 1);
      mbar_init(&accempty[q], 128);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    s_abort = 0;
  }
  const bool cached = a.njobs <= kMaxCachedJobs;
  if (cached)
    for (int i = tid; i < a.njobs; i += kMmaThreads) sfirst[i] = a.jobs[i].first;
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp < kMmaProducers / 32) {
    // ---------------- producers ----------------
    // Thread tid owns 16-byte chunk tid % 8 of rows tid / 8 + 32 i (i < 4) of
    // every data tile.  The raw data of the next kMmaDepth chunks (across tile
    // boundaries) are in flight in registers; per chunk the thread waits for a
    // free stage, forms x = in0 + sgn in1, splits it into hi / lo and stores
    // both at their swizzled places, then issues the loads of the chunk
    // kMmaDepth ahead into the registers it just used.  Thread 0 also brings
    // the chunk's table blocks in by two bulk copies counted by the stage's
    // full barrier.
    const int cq = tid & 7, rbase = tid >> 3;
    MmaRows R;
    auto setup = [&](int tile) {
      const MmaJob& J = a.jobs[mma_find_job(a, sfirst, cached, tile)];
      const int t = tile - J.first;
      const int mi = t / J.nt, ni = t - mi * J.nt;
      const int m0 = mi * 128;
      const int Mtot = J.nout * J.R;
      R.tile = tile;
      R.c = 0;
      R.nch = J.nch;
      R.K = J.K;
      R.comb = J.in1[0] >= 0;   // every output of a job has a second input, or none has
      R.vec = J.vec != 0;
      R.tbytes = (uint32_t)J.bn * kMmaBK * 4;
      R.thi = buf + J.thi + (long long)ni * J.nch * J.bn * kMmaBK;
      R.dlo = (int)(J.tlo - J.thi);
      R.okm = 0;
      R.sgm = 0;
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int g = m0 + rbase + 32 * i;
        const bool ok = g < Mtot;
        const int o = ok ? g / J.R : 0;
        const int r = ok ? g - o * J.R : 0;
        R.p0[i] = buf + J.in0[o] + (long long)r * J.ldb;
        R.d1[i] = R.comb ? (int)(J.in1[o] - J.in0[o]) : 0;
        R.okm |= ok ? 1u << i : 0u;
        R.sgm |= J.sgn[o] < 0 ? 1u << i : 0u;
      }
    };
    // issue the loads of the next chunk of the sequence into S
    auto fetch = [&](MmaSlot& S) {
      if (R.c == R.nch) {
        R.tile += gridDim.x;
        if (R.tile >= a.total) { S.valid = false; return; }
        setup(R.tile);
      }
      S.valid = true;
      S.comb = R.comb;
      S.sgm = R.sgm;
      S.tbytes = R.tbytes;
      S.thi = R.thi + (long long)R.c * (R.tbytes >> 2);
      S.dlo = R.dlo;
      const int k = R.c * kMmaBK + 4 * cq;
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int kv = (R.okm >> i) & 1 ? R.K : 0;
        const float* q0 = R.p0[i] + k;
        const float* q1 = q0 + R.d1[i];
        if (R.vec && k + 3 < kv) {
          S.x0[i] = *reinterpret_cast<const float4*>(q0);
          if (R.comb) S.x1[i] = *reinterpret_cast<const float4*>(q1);
        } else {   // K tail, rows past the job, or rows not on 16-byte boundaries: element loads, zero-filled
          S.x0[i] = make_float4(k < kv ? q0[0] : 0.f, k + 1 < kv ? q0[1] : 0.f, k + 2 < kv ? q0[2] : 0.f,
                                k + 3 < kv ? q0[3] : 0.f);
          if (R.comb)
            S.x1[i] = make_float4(k < kv ? q1[0] : 0.f, k + 1 < kv ? q1[1] : 0.f, k + 2 < kv ? q1[2] : 0.f,
                                  k + 3 < kv ? q1[3] : 0.f);
        }
      }
      ++R.c;
    };
    // x = in0 + sgn in1 -> hi / lo images of stage st
    auto convert = [&](const MmaSlot& S, unsigned char* st) {
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        float x[4] = {S.x0[i].x, S.x0[i].y, S.x0[i].z, S.x0[i].w};
        if (S.comb) {
          const float sg = (S.sgm >> i) & 1 ? -1.f : 1.f;
          x[0] += sg * S.x1[i].x; x[1] += sg * S.x1[i].y;
          x[2] += sg * S.x1[i].z; x[3] += sg * S.x1[i].w;
        }
        uint32_t h[4], l[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          h[j] = tf32_rna(x[j]);
          l[j] = tf32_rna(x[j] - __uint_as_float(h[j]));
        }
        const uint32_t so = sw128_off(rbase + 32 * i, cq);
        *reinterpret_cast<uint4*>(st + so) = make_uint4(h[0], h[1], h[2], h[3]);
        *reinterpret_cast<uint4*>(st + kMmaTileA + so) = make_uint4(l[0], l[1], l[2], l[3]);
      }
    };
    if (blockIdx.x < a.total) {
      setup(blockIdx.x);
    } else {
      R.tile = blockIdx.x;
      R.c = R.nch = 0;
    }
    MmaSlot S[kMmaDepth];
#pragma unroll
    for (int d = 0; d < kMmaDepth; ++d) fetch(S[d]);
    uint32_t seq = 0;   // chunks handed to the MMA issuer
    bool done = false;
    while (!done) {
#pragma unroll
      for (int d = 0; d < kMmaDepth; ++d) {
        if (done) continue;
        if (!S[d].valid) { done = true; continue; }
        const int s = (int)(seq % kMmaStages);
        if (!mbar_wait_bounded(&empty[s], ((seq / kMmaStages) & 1) ^ 1, &s_abort)) { done = true; continue; }
        unsigned char* st = sm + s * kMmaStageBytes;
        if (tid == 0) {   // the table chunk: two bulk copies counted by the stage's full barrier
          mbar_arrive_expect_tx(&full[s], 2 * S[d].tbytes);
          bulk_g2s(st + 2 * kMmaTileA, S[d].thi, S[d].tbytes, &full[s]);
          bulk_g2s(st + 2 * kMmaTileA + kMmaTileB, S[d].thi + S[d].dlo, S[d].tbytes, &full[s]);
        }
        convert(S[d], st);
        fence_async_smem();   // these generic-proxy writes -> visible to the tensor cores
        mbar_arrive(&full[s]);
        ++seq;
        fetch(S[d]);
      }
    }
    // the MMAs' commits to the last stages must land before the CTA can exit
    for (uint32_t u = seq > kMmaStages ? seq - kMmaStages : 0; u < seq && !s_abort; ++u)
      mbar_wait_bounded(&empty[u % kMmaStages], (u / kMmaStages) & 1, &s_abort);
  } else if (warp == kMmaIssuerWarp) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      uint32_t it = 0, tc = 0;
      for (int tile = blockIdx.x; tile < a.total && !s_abort; tile += gridDim.x, ++tc) {
        const MmaJob& J = a.jobs[mma_find_job(a, sfirst, cached, tile)];
        const uint32_t acc = tc & 1;
        const uint32_t d_tmem = tmem + acc * kMmaAccCols;
        const uint32_t idesc = tf32_idesc(128, J.bn);
        if (!mbar_wait_bounded(&accempty[acc], ((tc >> 1) & 1) ^ 1, &s_abort)) break;
        tc_fence_after();
        const int nch = J.nch;
        for (int c = 0; c < nch; ++c, ++it) {
          const int s = it % kMmaStages;
          if (!mbar_wait_bounded(&full[s], (it / kMmaStages) & 1, &s_abort)) break;
          tc_fence_after();
          unsigned char* st = sm + s * kMmaStageBytes;
          const uint32_t ahi = smem_u32(st), alo = ahi + kMmaTileA;
          const uint32_t bhi = ahi + 2 * kMmaTileA, blo = bhi + kMmaTileB;
#pragma unroll
          for (int j = 0; j < kMmaBK / 8; ++j) {   // k-steps of 8 (32 bytes) inside the swizzled rows
            const uint32_t kb = 32u * j;
            mma_tf32(d_tmem, sw128_desc(ahi + kb), sw128_desc(bhi + kb), idesc, (c > 0 || j > 0) ? 1u : 0u);
            mma_tf32(d_tmem, sw128_desc(ahi + kb), sw128_desc(blo + kb), idesc, 1u);
            mma_tf32(d_tmem, sw128_desc(alo + kb), sw128_desc(bhi + kb), idesc, 1u);
          }
          mma_commit(&empty[s]);   // the stage is free once these MMAs have read it
        }
        mma_commit(&accfull[acc]);
      }
    }
    __syncwarp();
  } else {
    // ---------------- epilogue ----------------
    const int q = warp - kMmaEpilogueWarp0;   // TMEM lane quarter (warp % 4)
    const int m = q * 32 + lane;             // accumulator row = TMEM lane
    uint32_t tc = 0;
    for (int tile = blockIdx.x; tile < a.total && !s_abort; tile += gridDim.x, ++tc) {
      // the job's fields in registers: the stores below go through a float
      // pointer into the pool, which the compiler cannot prove leaves the job
      // table alone, so fields read through J inside the loop would be loaded
      // again after every store
      const MmaJob& J = a.jobs[mma_find_job(a, sfirst, cached, tile)];
      const int t = tile - J.first;
      const int nt = J.nt, bn = J.bn, R = J.R;
      const int mi = t / nt, ni = t - mi * nt;
      const int n0 = ni * bn;
      const int ncols = min(bn, J.N - n0);          // columns of this tile inside the transform
      const long long ldo = J.ldo;
      const float scale = J.scale;
      const int g = mi * 128 + m;
      const bool mok = g < J.nout * R;
      const int o = mok ? g / R : 0;
      const int r = mok ? g - o * R : 0;
      float* outp = buf + J.out[o] + r + (long long)n0 * ldo;
      const uint32_t acc = tc & 1;
      if (!mbar_wait_bounded(&accfull[acc], (tc >> 1) & 1, &s_abort)) break;
      tc_fence_after();
      for (int cg = 0; cg * 32 < bn; ++cg) {
        float v[32];
        tmem_ld32(tmem + acc * kMmaAccCols + ((uint32_t)(q * 32) << 16) + (uint32_t)(cg * 32), v);
        if (mok) {
          float* op = outp + (long long)(cg * 32) * ldo;
          const int lim = ncols - cg * 32;
#pragma unroll
          for (int i = 0; i < 32; ++i)
            if (i < lim) op[(long long)i * ldo] = v[i] * scale;
        }
      }
      tc_fence_before();
      mbar_arrive(&accempty[acc]);
    }
  }
  // teardown: every MMA of this CTA has completed once the epilogue has read
  // the last accumulator; after an abort, give commits still in flight time
  // to land (bounded) before the TMEM is freed
  if (s_abort) {
    if (tid == 0) atomicExch(a.err, 1);
    if (tid == kMmaIssuerWarp * 32) {
      const long long t0 = clock64();
      while (clock64() - t0 < 20000000LL) {
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == kMmaIssuerWarp) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kMmaTmemCols) : "memory");
  }
}

// FP64 -> split TF32 transform tables of the tensor-core passes for extent n,
// pre-tiled (mma_ntile), each as hi / lo, with the output index as row:
//   C    [k][j] = 2 cos(pi (j + 1/2) k / n)           forward (REDFT10)
//   Ci^T [j][k] = Ci[k][j], Ci = C with row k = 0 halved  inverse (REDFT01)
//   C^T  [j][k] = C[k][j]                             adjoint of the forward
//   Ci   [k][j]                                       adjoint of the inverse
// Layout at off: Chi, Clo, CiThi, CiTlo, CThi, CTlo, Cihi, Cilo,
// mma_table_elems(n) each.
static __global__ void mma_table_kernel(float* buf, long long off, int n) {
  int nt, bn;
  mma_ntile(n, &nt, &bn);
  const int nch = (n + kMmaBK - 1) / kMmaBK;
  const long long S = (long long)nt * nch * bn * kMmaBK;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < S; i += (long long)gridDim.x * blockDim.x) {
    // logical (N tile, K chunk, row, k) of element i; its position in the swizzled image
    const int k = (int)(i % kMmaBK);
    const long long rest = i / kMmaBK;
    const int r = (int)(rest % bn);
    const long long blk = rest / bn;
    const int ic = (int)(blk % nch), it = (int)(blk / nch);
    const int row = it * bn + r, col = ic * kMmaBK + k;
    const long long dst = (blk * bn + r) * kMmaBK + ((((k >> 2) ^ r) & 7) << 2) + (k & 3);
    double v[4] = {0.0, 0.0, 0.0, 0.0};   // C, Ci^T, C^T, Ci at (row, col)
    if (row < n && col < n) {
      const long long q = ((long long)(2 * col + 1) * row) % (4LL * n);    // C[row][col]: k = row, j = col
      const double c = 2.0 * cospi((double)q / (2.0 * n));
      const long long q2 = ((long long)(2 * row + 1) * col) % (4LL * n);   // C[col][row]: k = col, j = row
      const double ct = 2.0 * cospi((double)q2 / (2.0 * n));
      v[0] = c;
      v[1] = col == 0 ? 0.5 * ct : ct;
      v[2] = ct;
      v[3] = row == 0 ? 0.5 * c : c;
    }
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const uint32_t h = tf32_rna((float)v[t]);
      const uint32_t l = tf32_rna((float)(v[t] - (double)__uint_as_float(h)));
      buf[off + (2 * t) * S + dst] = __uint_as_float(h);
      buf[off + (2 * t + 1) * S + dst] = __uint_as_float(l);
    }
  }
}

}  // namespace ard
