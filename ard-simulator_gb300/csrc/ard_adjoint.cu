// Adjoint of the ARD time step: gradients of the recorder misfit
//   J = 0.5 sum_{t < T} sum_r (rec[t][r] - target[t][r])^2
// with respect to the source series, the initial pressure of the air
// partitions and the per-face PML damping scales.
//
// The step is linear in its state (modal levels, shell forces, PML fields),
// so the adjoint recursion needs no forward state except for the damping
// gradient, whose terms multiply forward PML values (p(t), p(t-1), phi_n(t)).
// Without that gradient the call is one forward run (recorder residuals)
// and one backward run.  With it the forward PML values come back in
// reverse order by one of:
//   - the whole PML history, kept in the forward run when it fits;
//   - segments of K steps swept backwards from the last.  A segment's PML
//     history is made again before its backward sweep, either by PML replay
//     (the forward run recorded the interfaces' forcing of the PML strips
//     for its steps and kept its PML state at its start: the PML runs again
//     on its own) or by recompute (the forward run kept the whole state at
//     its start: the whole segment runs again).  The trailing segments are
//     replayed, as many as the forcing record allows in the free memory, and
//     the ones before them recomputed.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <string>
#include <vector>

#include "ard_adjoint_kernels.cuh"
#include "ard_engine.h"
#include "ard_gb300.h"
#include "ard_kernels.cuh"

using namespace ard;

namespace {

int grid_for(long long work, int per_block, int max_blocks) {
  long long b = (work + per_block - 1) / per_block;
  if (b < 1) b = 1;
  if (b > max_blocks) b = max_blocks;
  return (int)b;
}

// Device buffers of one ard_adjoint call.
struct AdjBuffers {
  void* resid = nullptr;      // [T][n_rec_total] residuals (context precision)
  double* gsrc = nullptr;     // [T][n_src_total]
  double* gz = nullptr;       // [pml blocks][kMaxPmlLayers]
  void* ckpt = nullptr;       // segment checkpoints and the state after step T (adjoint_impl)
  void* hist_p = nullptr;     // [K + 1][region]
  void* hist_phn = nullptr;   // [K][region]
  void* fhist = nullptr;      // [T][strip region] (PML replay)
  CUtensorMap* hmaps = nullptr;   // tensor maps of hist_p per slab (the adjoint PML kernel's p(t) tiles)
  ~AdjBuffers() {
    void* ptrs[] = {resid, gsrc, gz, ckpt, hist_p, hist_phn, fhist, hmaps};
    for (void* p : ptrs)
      if (p) cudaFree(p);
  }
};

// Launch attributes of the kernels launched from this file.
template <typename T>
int configure_adjoint(Ctx* ctx) {
  const int msmem = (int)(kModalSmemElems * sizeof(T));
  ARD_CUDA(cudaFuncSetAttribute(modal_kernel<T, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, msmem));
  ARD_CUDA(cudaFuncSetAttribute(modal_kernel<T, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, msmem));
  if (ctx->fused_faces) {
    const int f2d = std::max(ctx->smem_optin, (int)ctx->f2d_bytes);
    ARD_CUDA(cudaFuncSetAttribute(face2d_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, f2d));
    ARD_CUDA(cudaFuncSetAttribute(face2d_cluster_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, f2d));
  }
  ARD_CUDA(configure_face_gemm<T>());
  return ARD_OK;
}

struct HistView {
  const void* p = nullptr;
  const void* phn = nullptr;
  long long hlen = 0;
  double* gz = nullptr;
  const CUtensorMap* hmaps = nullptr;
};

// One adjoint step t (tstep: position inside the launch sequence, counted
// backwards from the counter d_tb[0]).
template <typename T>
int launch_adjoint_step(Ctx* ctx, int t, int tstep, cudaStream_t s, cudaStream_t s2, const AdjBuffers& ab,
                        const HistView& hv) {
  T* buf = reinterpret_cast<T*>(ctx->d_buf);
  const int lout = t % 3, lin = (t + 1) % 3, ly = (t + 2) % 3;
  const int par = t & 1;
  if (ctx->q_end > ctx->q_begin)
    ARD_CUDA(cudaMemsetAsync(buf + ctx->q_begin, 0, sizeof(T) * (size_t)(ctx->q_end - ctx->q_begin), s));
  if (ctx->n_face_cells > 0) {
    IfaceAdjArgs<T> ia{buf, ctx->d_ifs, (int)ctx->ifs.size(), ctx->n_face_cells, ctx->d_dct, ctx->d_pml,
                       ctx->d_mask, lin, lout, (T)ctx->c0, (T)ctx->dh, (T)ctx->dt, ctx->d_cell_iface};
    ARD_CUDA(launch_dep(iface_adjoint_kernel<T>, grid_for(ctx->n_face_cells, 256, ctx->num_sms * 16), 256, 0, s, ia));
    ARD_CUDA(cudaGetLastError());
  }
  const bool fork = !ctx->pml_blocks.empty() && !ctx->dct.empty();
  if (fork) {
    ARD_CUDA(cudaEventRecord(ctx->ev_fork, s));
    ARD_CUDA(cudaStreamWaitEvent(s2, ctx->ev_fork, 0));
  }
  if (!ctx->pml_blocks.empty()) {
    PmlAdjArgs<T> pa{buf, ctx->d_pml, ctx->d_pml_blocks, (int)ctx->pml_blocks.size(), lin, ly, lout, (t + 1) & 1,
                     (T)ctx->dt, (T)ctx->dh, (T)ctx->c0, (const T*)hv.p, (const T*)hv.phn, hv.hlen, ctx->d_tb,
                     tstep, hv.gz, ctx->d_pml_amaps, hv.hmaps, ctx->d_err};
    ARD_CUDA(launch_dep(pml_adjoint_kernel<T>, grid_for((long long)ctx->pml_blocks.size(), 1, ctx->num_sms * 8), 256,
                        0, fork ? s2 : s, pa));
    ARD_CUDA(cudaGetLastError());
  }
  if (!ctx->dct.empty()) {
    const int gx = ctx->num_sms * 4;
    if (ctx->fused_faces) {
      ARD_CUDA(launch_face2d<T>(ctx->adj1_split, (long long)ctx->adj1_2d.size() / 2, gx, ctx->f2d_bytes, s, buf,
                                ctx->d_adj1_2d, ctx->f2d_smem));
    } else if (ctx->mma_faces) {
      ARD_CUDA(launch_mma(ctx, 4, s));
      ARD_CUDA(launch_mma(ctx, 5, s));
    } else {
      for (int k = 0; k < 2; ++k)
        ARD_CUDA(launch_face_gemm<T>(buf, ctx->adjg[k].jobs[0], ctx->d_adjg[k], (int)ctx->adjg[k].jobs.size(),
                                     ctx->adjg[k].units, grid_for(ctx->adjg[k].units, 1, ctx->num_sms * 2), s));
    }
    ARD_CUDA(cudaGetLastError());
    ModalArgs<T> ma{buf, ctx->d_dct, ctx->d_tiles, (int)ctx->tiles.size(), ctx->d_srcpts, ctx->d_recpts,
                    ctx->d_series, ctx->max_steps, ctx->d_tb, tstep, par, (const T*)ab.resid, ctx->n_rec_total};
    const size_t msmem = kModalSmemElems * sizeof(T);
    const int mgrid = grid_for((long long)ctx->tiles.size(), 1, ctx->num_sms * 2);
    if (ctx->arith == ARD_ARITH_REFERENCE)
      ARD_CUDA(launch_dep(modal_kernel<T, true, true>, mgrid, kModalThreads, msmem, s, ma));
    else
      ARD_CUDA(launch_dep(modal_kernel<T, false, true>, mgrid, kModalThreads, msmem, s, ma));
    ARD_CUDA(cudaGetLastError());
    if (!ctx->srcpts.empty()) {
      ARD_CUDA(launch_dep(srcgrad_kernel<T>, grid_for((long long)ctx->srcpts.size() * 32, 128, 1 << 30), 128, 0, s,
                          (const T*)buf, ctx->d_dct, ctx->d_srcpts, (int)ctx->srcpts.size(), ctx->n_src_total,
                          ab.gsrc, ctx->d_tb, tstep));
      ARD_CUDA(cudaGetLastError());
    }
    if (int rc2 = launch_post_modal<T>(ctx, s, 0, false)) return rc2;
    if (ctx->fused_faces) {
      ARD_CUDA(launch_face2d<T>(ctx->adj2_split, (long long)ctx->adj2_2d.size() / 2, gx, ctx->f2d_bytes, s, buf,
                                ctx->d_adj2_2d, ctx->f2d_smem));
    } else if (ctx->mma_faces) {
      ARD_CUDA(launch_mma(ctx, 6, s));
      ARD_CUDA(launch_mma(ctx, 7, s));
    } else {
      for (int k = 2; k < 4; ++k)
        ARD_CUDA(launch_face_gemm<T>(buf, ctx->adjg[k].jobs[0], ctx->d_adjg[k], (int)ctx->adjg[k].jobs.size(),
                                     ctx->adjg[k].units, grid_for(ctx->adjg[k].units, 1, ctx->num_sms * 2), s));
    }
    ARD_CUDA(cudaGetLastError());
  }
  if (fork) {
    ARD_CUDA(cudaEventRecord(ctx->ev_join, s2));
    ARD_CUDA(cudaStreamWaitEvent(s, ctx->ev_join, 0));
  }
  if (ctx->debug_sync) {
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
      ctx->err = std::string("adjoint step ") + std::to_string(t) + ": " + cudaGetErrorString(e);
      return ARD_ERR_CUDA;
    }
  }
  return ARD_OK;
}

static __global__ void retreat_counter_kernel(long long* tc, int n) {
  if (threadIdx.x == 0 && blockIdx.x == 0) tc[0] -= n;
}

// Adjoint steps captured as one CUDA graph: kAdjGraphSteps steps starting at
// a step t = 5 (mod 6) (the level choices t % 3 and t & 1 repeat every 6
// steps), the step counter lowered by kAdjGraphSteps at the end.
constexpr int kAdjGraphSteps = 48;

struct AdjGraph {
  cudaGraphExec_t exec = nullptr;
  ~AdjGraph() {
    if (exec) cudaGraphExecDestroy(exec);
  }
};

template <typename T>
int capture_adjoint_graph(Ctx* ctx, const AdjBuffers& ab, const HistView& hv, AdjGraph* g) {
  if (g->exec) return ARD_OK;
  cudaGraph_t graph = nullptr;
  ARD_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  const int t_pattern = 6 * 1000 + 5;
  int rc = ARD_OK;
  for (int i = 0; i < kAdjGraphSteps && rc == ARD_OK; ++i)
    rc = launch_adjoint_step<T>(ctx, t_pattern - i, i, ctx->stream, ctx->stream2, ab, hv);
  if (rc == ARD_OK) retreat_counter_kernel<<<1, 32, 0, ctx->stream>>>(ctx->d_tb, kAdjGraphSteps);
  cudaError_t e = cudaStreamEndCapture(ctx->stream, &graph);
  if (rc) { if (graph) cudaGraphDestroy(graph); return rc; }
  if (e != cudaSuccess) { ctx->err = std::string("adjoint graph capture: ") + cudaGetErrorString(e); return ARD_ERR_CUDA; }
  e = cudaGraphInstantiate(&g->exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) { ctx->err = std::string("adjoint graph instantiate: ") + cudaGetErrorString(e); return ARD_ERR_CUDA; }
  return ARD_OK;
}

// Adjoint steps t_hi - 1 down to t_lo: direct launches up to a step t = 5
// (mod 6), then 48-step graphs, then direct launches for the rest.  Every
// launch finds its step as counter - tstep.
template <typename T>
int run_backward(Ctx* ctx, long long t_hi, long long t_lo, long long hist_t0, const AdjBuffers& ab,
                 const HistView& hv, AdjGraph* graph) {
  cudaStream_t s = ctx->stream;
  long long t = t_hi - 1;
  long long base = t;
  set_counters_kernel<<<1, 32, 0, s>>>(ctx->d_tb, base, hist_t0);
  ARD_CUDA(cudaGetLastError());
  const bool graphs = ctx->use_graphs && !ctx->debug_sync;
  while (t >= t_lo) {
    if (graphs && t % 6 == 5 && t - t_lo + 1 >= kAdjGraphSteps) break;
    int rc = launch_adjoint_step<T>(ctx, (int)t, (int)(base - t), s, ctx->stream2, ab, hv);
    if (rc) return rc;
    --t;
  }
  if (graphs && t >= t_lo && t - t_lo + 1 >= kAdjGraphSteps) {
    int rc = capture_adjoint_graph<T>(ctx, ab, hv, graph);
    if (rc) return rc;
    set_counters_kernel<<<1, 32, 0, s>>>(ctx->d_tb, t, hist_t0);
    ARD_CUDA(cudaGetLastError());
    while (t - t_lo + 1 >= kAdjGraphSteps) {
      ARD_CUDA(cudaGraphLaunch(graph->exec, s));
      t -= kAdjGraphSteps;
    }
    base = t;   // the counter now holds t
  }
  for (; t >= t_lo; --t) {
    int rc = launch_adjoint_step<T>(ctx, (int)t, (int)(base - t), s, ctx->stream2, ab, hv);
    if (rc) return rc;
  }
  return ARD_OK;
}

static __global__ void set_step_counter_kernel(long long* tcount, long long v) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *tcount = v;
}

template <typename T>
int adjoint_impl(Ctx* ctx, long long T_steps, const float* target, int checkpoint_every, float* grad_source,
                 float* grad_scale, float* loss) {
  const size_t es = sizeof(T);
  cudaStream_t s = ctx->stream;
  int rc = configure_adjoint<T>(ctx);
  if (rc) return rc;
  const bool need_hist = grad_scale != nullptr && !ctx->pml.empty();
  const long long state_len = ctx->state_end - ctx->state_begin;
  const long long hlen = ctx->pml_region[0][1] - ctx->pml_region[0][0];
  // How the forward PML values reach the backward sweep (damping gradient only):
  //   kFull     the whole history p(t), phi_n(t) kept in one forward run
  //   kSegments the run in segments of K steps, the backward sweep segment by
  //             segment from the last; a segment's history comes back either
  //             by replay (its strip forcing recorded in the forward run and
  //             the PML state kept at its start: the PML runs again on its
  //             own) or by recompute (the whole state kept at its start: the
  //             whole segment runs again).  The first n_rc segments are
  //             recomputed and the rest replayed, n_rc as small as the memory
  //             allows: 0 (all replayed) where the forcing record fits.
  enum { kNone, kFull, kSegments } mode = kNone;
  long long K = T_steps, n_seg = 1, n_rc = 0;
  const long long pml_begin = ctx->pml_region[0][0];
  const long long pml_len = ctx->state_end - pml_begin;       // PML fields + strip forces
  const long long flen = ctx->state_end - ctx->force_begin;    // strip forces
  AdjBuffers ab;
  // memory of a segmented run (elements): history of one segment, PML
  // checkpoints of the replayed segments, whole-state checkpoints of the
  // recomputed ones, the state after T (whole, or its PML part where nothing
  // is recomputed), the forcing record of the replayed steps
  auto seg_need = [&](long long k, long long nrc) {
    const long long ns = (T_steps + k - 1) / k;
    const long long t_rep = std::max(0LL, T_steps - nrc * k);
    return (2 * k + 1) * hlen + (ns - nrc) * pml_len + (nrc > 0 ? (nrc + 1) * state_len : pml_len) + t_rep * flen;
  };
  if (need_hist) {
    size_t free_b = 0, total_b = 0;
    ARD_CUDA(cudaMemGetInfo(&free_b, &total_b));
    const long long budget = (long long)(free_b / 10 * 9 / es);
    const long long full = (2 * T_steps + 1) * hlen;
    auto segment_k = [&](long long ckpt_len) {
      // balance checkpoint memory (one copy per segment) against history memory (2 K PML regions)
      const double k = std::sqrt((double)T_steps * (double)ckpt_len / (2.0 * (double)std::max(1LL, hlen)));
      return std::max(1LL, std::min(T_steps, (long long)std::ceil(k)));
    };
    // ARD_ADJOINT_RECOMPUTE=1 (tests): every segment recomputed; =n (n > 1): the first n - 1
    const char* force_rc = std::getenv("ARD_ADJOINT_RECOMPUTE");
    const long long forced = force_rc ? std::atoll(force_rc) : 0;
    if (checkpoint_every <= 0 && (size_t)full * es <= free_b / 2 && forced <= 0) {
      mode = kFull;
    } else {
      mode = kSegments;
      K = checkpoint_every > 0 ? std::min<long long>(checkpoint_every, T_steps) : segment_k(pml_len);
      n_seg = (T_steps + K - 1) / K;
      if (forced > 0 || seg_need(K, 0) > budget) {
        if (checkpoint_every <= 0) K = segment_k(state_len);
        n_seg = (T_steps + K - 1) / K;
        if (forced == 1) {
          n_rc = n_seg;
        } else if (forced > 1) {
          n_rc = std::min(n_seg, forced - 1);
        } else {
          n_rc = 1;
          while (n_rc < n_seg && seg_need(K, n_rc) > budget) ++n_rc;
        }
      }
      if (seg_need(K, n_rc) > budget) {
        ctx->err = "ard_adjoint: checkpoints and PML history need " + std::to_string((seg_need(K, n_rc) * es) >> 20) +
                   " MiB (segments of " + std::to_string(K) + " steps, " + std::to_string(n_rc) +
                   " recomputed); " + std::to_string(free_b >> 20) + " MiB free";
        return ARD_ERR_OOM;
      }
      const long long n_rep = n_seg - n_rc;
      ARD_CUDA(cudaMalloc(&ab.ckpt, std::max<size_t>(1, (size_t)(n_rep * pml_len + (n_rc > 0 ? (n_rc + 1) * state_len : pml_len)) * es)));
      if (n_rep > 0) ARD_CUDA(cudaMalloc(&ab.fhist, std::max<size_t>(1, (size_t)(T_steps - n_rc * K) * flen * es)));
    }
    const long long hk = mode == kFull ? T_steps : K;
    ARD_CUDA(cudaMalloc(&ab.hist_p, (size_t)(hk + 1) * hlen * es));
    ARD_CUDA(cudaMalloc(&ab.hist_phn, (size_t)hk * hlen * es));
    if ((rc = build_pml_hist_maps(ctx, ab.hist_p, hlen, hk + 1, &ab.hmaps))) return rc;
  }
  ctx->adj_mode = mode == kFull ? "whole PML history"
                 : mode == kNone ? "no forward values"
                 : n_rc == 0     ? "PML replay"
                 : n_rc == n_seg ? "segment recompute"
                                 : "hybrid: segment recompute for the first " + std::to_string(n_rc) + " of " +
                                       std::to_string(n_seg) + " segments, PML replay after them";
  ctx->adj_k = mode == kSegments ? K : 0;
  const int nrec = ctx->n_rec_total, nsrc = ctx->n_src_total;
  ARD_CUDA(cudaMalloc(&ab.resid, std::max<size_t>(1, (size_t)T_steps * nrec * es)));
  ARD_CUDA(cudaMalloc(&ab.gsrc, std::max<size_t>(1, (size_t)T_steps * nsrc * sizeof(double))));
  ARD_CUDA(cudaMalloc(&ab.gz, std::max<size_t>(1, ctx->pml_blocks.size() * kMaxPmlLayers * sizeof(double))));
  ARD_CUDA(cudaMemsetAsync(ab.gsrc, 0, (size_t)T_steps * nsrc * sizeof(double), s));
  ARD_CUDA(cudaMemsetAsync(ab.gz, 0, ctx->pml_blocks.size() * kMaxPmlLayers * sizeof(double), s));

  T* buf = reinterpret_cast<T*>(ctx->d_buf);
  T* state = buf + ctx->state_begin;
  T* pml_state = buf + pml_begin;
  const long long t_rc = n_rc * K;   // steps [0, t_rc) recomputed, [t_rc, T) replayed
  // checkpoint storage: whole states of the recomputed segments' starts, then
  // the state after T (whole where anything is recomputed, else its PML
  // part), then the PML states of the replayed segments' starts
  T* ckbase = reinterpret_cast<T*>(ab.ckpt);
  auto full_ckpt = [&](long long i) { return ckbase + i * state_len; };
  T* final_ckpt = ckbase + n_rc * state_len;
  const long long final_len = n_rc > 0 ? state_len : pml_len;
  T* final_src = n_rc > 0 ? state : pml_state;
  auto pml_ckpt = [&](long long i) { return final_ckpt + final_len + (i - n_rc) * pml_len; };

  // What the PML kernel records or replays (PmlHist): p(t), phi_n(t) of
  // steps t0 <= t < t1 (the slot of p(t0 - 1) filled here from the state
  // before step t0), the strip forcing of the replayed steps [t_rc, T), and
  // the forcing it replays.
  T* hp = reinterpret_cast<T*>(ab.hist_p);
  T* hphn = reinterpret_cast<T*>(ab.hist_phn);
  T* fh = reinterpret_cast<T*>(ab.fhist);
  auto set_hist = [&](bool keep, long long t0, long long t1, bool rec_force, bool replay) -> int {
    PmlHist<T> h{};
    if (keep) {
      h.p = hp; h.phn = hphn; h.hlen = hlen; h.t0 = t0; h.t1 = t1;
      const int q_prev = (int)((t0 + 1) & 1);   // level of p(t0 - 1)
      ARD_CUDA(cudaMemcpyAsync(hp, buf + ctx->pml_region[q_prev][0], hlen * es, cudaMemcpyDeviceToDevice, s));
    }
    h.flen = flen;
    if (rec_force) { h.f = fh; h.ft0 = t_rc; h.ft1 = T_steps; }
    if (replay) { h.fsrc = fh; h.fs0 = t_rc; }
    ARD_CUDA(cudaMemcpyAsync(ctx->d_phist, &h, sizeof(h), cudaMemcpyHostToDevice, s));
    return ARD_OK;
  };

  // ---- forward run ----
  ard_ctx* handle = reinterpret_cast<ard_ctx*>(ctx);
  if (mode == kSegments) {
    if (n_seg > n_rc && (rc = set_hist(false, 0, 0, true, false))) return rc;   // record the replayed steps' forcing
    for (long long i = 0; i < n_seg; ++i) {
      if (i < n_rc)
        ARD_CUDA(cudaMemcpyAsync(full_ckpt(i), state, state_len * es, cudaMemcpyDeviceToDevice, s));
      else
        ARD_CUDA(cudaMemcpyAsync(pml_ckpt(i), pml_state, pml_len * es, cudaMemcpyDeviceToDevice, s));
      rc = ard_step(handle, std::min(K, T_steps - i * K), nullptr);
      if (rc) return rc;
    }
    ARD_CUDA(cudaMemcpyAsync(final_ckpt, final_src, final_len * es, cudaMemcpyDeviceToDevice, s));
    if ((rc = set_hist(false, 0, 0, false, false))) return rc;
  } else {
    if (mode == kFull && (rc = set_hist(true, 0, T_steps, false, false))) return rc;
    rc = ard_step(handle, T_steps, nullptr);
    if (rc) return rc;
    if (mode == kFull && (rc = set_hist(false, 0, 0, false, false))) return rc;
  }

  // ---- residuals and misfit ----
  ARD_CUDA(cudaStreamSynchronize(s));
  std::vector<double> rec((size_t)T_steps * nrec);
  if (nrec > 0)
    ARD_CUDA(cudaMemcpy(rec.data(), ctx->d_hist, rec.size() * sizeof(double), cudaMemcpyDeviceToHost));
  std::vector<T> res(rec.size());
  std::vector<double> scene_loss(ctx->scenes.size(), 0.0);
  for (size_t si = 0; si < ctx->scenes.size(); ++si) {
    const SceneRec& sr = ctx->scenes[si];
    for (long long t = 0; t < T_steps; ++t)
      for (int r = 0; r < sr.nrec; ++r) {
        const int g = sr.rec0 + r;
        // target rows are concatenated over scenes: scene si's block is T x nrec(si)
        const double tg = target[(size_t)sr.rec0 * T_steps + (size_t)t * sr.nrec + r];
        const double e = rec[(size_t)t * nrec + g] - tg;
        res[(size_t)t * nrec + g] = (T)e;
        scene_loss[si] += 0.5 * e * e;
      }
  }
  if (nrec > 0)
    ARD_CUDA(cudaMemcpy(ab.resid, res.data(), res.size() * es, cudaMemcpyHostToDevice));

  // ---- backward run ----
  const long long adj_len = ctx->adj_end - ctx->adj_begin;
  ARD_CUDA(cudaMemsetAsync(buf + ctx->adj_begin, 0, adj_len * es, s));
  const HistView hv = need_hist ? HistView{ab.hist_p, ab.hist_phn, hlen, ab.gz, ab.hmaps} : HistView{};
  AdjGraph graph;   // captured on first use, for this call's buffers
  if (mode == kSegments) {
    for (long long i = n_seg - 1; i >= 0; --i) {
      const long long t0 = i * K, t1 = std::min(T_steps, t0 + K);
      const bool replay = i >= n_rc;
      // the segment again from its checkpoint, keeping its PML history
      if (replay)
        ARD_CUDA(cudaMemcpyAsync(pml_state, pml_ckpt(i), pml_len * es, cudaMemcpyDeviceToDevice, s));
      else
        ARD_CUDA(cudaMemcpyAsync(state, full_ckpt(i), state_len * es, cudaMemcpyDeviceToDevice, s));
      set_step_counter_kernel<<<1, 32, 0, s>>>(ctx->d_t, t0);
      ARD_CUDA(cudaGetLastError());
      if ((rc = set_hist(true, t0, t1, false, replay))) return rc;
      if (replay) {
        // the PML on its own, driven by the recorded strip forcing
        for (long long t = t0; t < t1; ++t)
          if ((rc = launch_pml<T>(ctx, (int)(t & 1), (int)(t - t0), s))) return rc;
      } else {
        ctx->t_host = t0;
        rc = ard_step(handle, t1 - t0, nullptr);
        if (rc) return rc;
      }
      if ((rc = set_hist(false, 0, 0, false, false))) return rc;
      rc = run_backward<T>(ctx, t1, t0, t0, ab, hv, &graph);
      if (rc) return rc;
    }
    // leave the forward state as after step T
    ARD_CUDA(cudaMemcpyAsync(final_src, final_ckpt, final_len * es, cudaMemcpyDeviceToDevice, s));
    set_step_counter_kernel<<<1, 32, 0, s>>>(ctx->d_t, T_steps);
    ARD_CUDA(cudaGetLastError());
    ctx->t_host = T_steps;
  } else {
    rc = run_backward<T>(ctx, T_steps, 0, 0, ab, hv, &graph);
    if (rc) return rc;
  }
  ARD_CUDA(cudaStreamSynchronize(s));
  ARD_CUDA(cudaStreamSynchronize(ctx->stream2));

  // ---- outputs ----
  if (grad_source && nsrc > 0) {
    std::vector<double> g((size_t)T_steps * nsrc);
    ARD_CUDA(cudaMemcpy(g.data(), ab.gsrc, g.size() * sizeof(double), cudaMemcpyDeviceToHost));
    // [source][t], sources numbered scene by scene (the layout of the source series)
    for (int q = 0; q < nsrc; ++q)
      for (long long t = 0; t < T_steps; ++t) grad_source[(size_t)q * T_steps + t] = (float)g[(size_t)t * nsrc + q];
  }
  if (grad_scale) {
    for (size_t si = 0; si < ctx->scenes.size(); ++si)
      for (int f = 0; f < 6; ++f) grad_scale[si * 6 + f] = 0.f;
    if (need_hist) {
      std::vector<double> gz(ctx->pml_blocks.size() * kMaxPmlLayers);
      ARD_CUDA(cudaMemcpy(gz.data(), ab.gz, gz.size() * sizeof(double), cudaMemcpyDeviceToHost));
      std::vector<std::vector<double>> per_slab(ctx->pml.size());
      for (size_t k = 0; k < ctx->pml.size(); ++k) per_slab[k].assign(ctx->pml[k].L, 0.0);
      for (size_t b = 0; b < ctx->pml_blocks.size(); ++b) {
        const int slab = ctx->pml_blocks[b].x;
        for (int l = 0; l < ctx->pml[slab].L; ++l) per_slab[slab][l] += gz[b * kMaxPmlLayers + l];
      }
      std::vector<double> acc(ctx->scenes.size() * 6, 0.0);
      for (size_t k = 0; k < ctx->pml.size(); ++k) {
        const PmlDev& P = ctx->pml[k];
        std::vector<double> z0;
        pml_profile_unit(ctx, P.type, P.L, &z0);
        for (int l = 0; l < P.L; ++l) acc[(size_t)P.scene * 6 + P.type] += per_slab[k][l] * z0[l];
      }
      for (size_t i = 0; i < acc.size(); ++i) grad_scale[i] = (float)acc[i];
    }
  }
  if (loss)
    for (size_t si = 0; si < ctx->scenes.size(); ++si) loss[si] = (float)scene_loss[si];
  ctx->adj_valid = true;
  return ARD_OK;
}

}  // namespace

extern "C" int ard_adjoint(ard_ctx* c, int64_t T, const float* target, int32_t checkpoint_every, float* grad_source,
                           float* grad_scale, float* loss) {
  if (!c) return ARD_ERR_INVALID;
  Ctx* ctx = reinterpret_cast<Ctx*>(c);
  if (!ctx->adjoint) { ctx->err = "ard_adjoint: context created without options.adjoint"; return ARD_ERR_STATE; }
  if (T < 1 || T > ctx->max_steps) { ctx->err = "ard_adjoint: T must be in [1, max_steps]"; return ARD_ERR_RANGE; }
  if (ctx->n_rec_total > 0 && !target) { ctx->err = "ard_adjoint: target is NULL"; return ARD_ERR_INVALID; }
  if (ctx->t_host != 0) {
    ctx->err = "ard_adjoint: runs the forward from step 0 (call ard_reset, then set the initial pressure)";
    return ARD_ERR_STATE;
  }
  ARD_CUDA(cudaSetDevice(ctx->device));
  ctx->adj_valid = false;
  return ctx->prec == ARD_PREC_F64
             ? adjoint_impl<double>(ctx, T, target, checkpoint_every, grad_source, grad_scale, loss)
             : adjoint_impl<float>(ctx, T, target, checkpoint_every, grad_source, grad_scale, loss);
}

extern "C" int ard_read_initial_pressure_grad(ard_ctx* c, int32_t scene, int32_t partition, float* out) {
  if (!c || !out) return ARD_ERR_INVALID;
  Ctx* ctx = reinterpret_cast<Ctx*>(c);
  if (!ctx->adj_valid) { ctx->err = "ard_read_initial_pressure_grad: no adjoint run since the last reset"; return ARD_ERR_STATE; }
  if (scene < 0 || scene >= (int)ctx->scenes.size()) { ctx->err = "bad scene index"; return ARD_ERR_RANGE; }
  const SceneRec& sr = ctx->scenes[scene];
  if (partition < 0 || partition >= (int)sr.parts.size()) { ctx->err = "bad partition index"; return ARD_ERR_RANGE; }
  if (sr.parts[partition].kind != ARD_PART_DCT) {
    ctx->err = "initial pressure applies to air partitions";
    return ARD_ERR_INVALID;
  }
  ARD_CUDA(cudaSetDevice(ctx->device));
  ARD_CUDA(cudaStreamSynchronize(ctx->stream));
  const DctDev& D = ctx->dct[sr.engine_idx[partition]];
  const long long N = (long long)D.w * D.h * D.d;
  const long long s0 = ctx->scratch;
  const int blocks = (int)std::min<long long>((N + 255) / 256, 8192);
  // the modes are m0 = kappa C^3 p0 with kappa = 1 / (8 N s_i); dJ/dp0 = kappa (C^T)^3 dJ/dm0
  const double kappa = 1.0 / (8.0 * (double)N / std::sqrt(2.0 * (double)N));
  int rc;
  if (ctx->prec == ARD_PREC_F64) {
    if (ctx->arith == ARD_ARITH_REFERENCE) init_grad_kernel<double, true><<<blocks, 256, 0, ctx->stream>>>((double*)ctx->d_buf, D, s0 + N);
    else init_grad_kernel<double, false><<<blocks, 256, 0, ctx->stream>>>((double*)ctx->d_buf, D, s0 + N);
    ARD_CUDA(cudaGetLastError());
    rc = dense_transform_ex<double>(ctx, D, s0 + N, s0 + N, s0, 0, true, kappa);
    if (rc) return rc;
    std::vector<double> h((size_t)N);
    ARD_CUDA(cudaMemcpy(h.data(), (double*)ctx->d_buf + s0 + N, N * sizeof(double), cudaMemcpyDeviceToHost));
    for (long long i = 0; i < N; ++i) out[i] = (float)h[i];
  } else {
    if (ctx->arith == ARD_ARITH_REFERENCE) init_grad_kernel<float, true><<<blocks, 256, 0, ctx->stream>>>((float*)ctx->d_buf, D, s0 + N);
    else init_grad_kernel<float, false><<<blocks, 256, 0, ctx->stream>>>((float*)ctx->d_buf, D, s0 + N);
    ARD_CUDA(cudaGetLastError());
    rc = dense_transform_ex<float>(ctx, D, s0 + N, s0 + N, s0, 0, true, kappa);
    if (rc) return rc;
    ARD_CUDA(cudaMemcpy(out, (float*)ctx->d_buf + s0 + N, N * sizeof(float), cudaMemcpyDeviceToHost));
  }
  return ARD_OK;
}
