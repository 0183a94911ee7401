// GB300 ARD engine: context creation (work tables, HBM layout), the per-step
// launch sequence and its CUDA-graph capture, and the C ABI of
// include/ard_gb300.h for stepping, readout and setup.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <utility>
#include <vector>

#include "ard_device.cuh"
#include "ard_engine.h"
#include "ard_gb300.h"
#include "ard_kernels.cuh"
#include "ard_mma.cuh"

using namespace ard;

namespace {

thread_local std::string g_create_error;

int grid_for(long long work, int per_block, int max_blocks) {
  long long b = (work + per_block - 1) / per_block;
  if (b < 1) b = 1;
  if (b > max_blocks) b = max_blocks;
  return (int)b;
}

}  // namespace

namespace ard {
// One tensor-core face pass (job list k) on stream s: one CTA per SM at most.
// (The adjoint's passes launch through here too, so that one instance of the
// kernel, configured in ard_create, serves both.)
cudaError_t launch_mma(Ctx* ctx, int k, cudaStream_t s) {
  if (ctx->mtiles[k] == 0) return cudaSuccess;
  MmaArgs a{reinterpret_cast<float*>(ctx->d_buf), ctx->d_mjobs[k], (int)ctx->mjobs[k].size(), ctx->mtiles[k], ctx->d_err};
  return launch_dep(face_mma_kernel, grid_for(ctx->mtiles[k], 1, ctx->num_sms), kMmaThreads, kMmaSmemBytes, s, a);
}
}  // namespace ard

// ---------------------------------------------------------------------------
// context construction
// ---------------------------------------------------------------------------

namespace ard {

int build_layout(Ctx* ctx, const ard_scene* scenes, int n_scenes);

}  // namespace ard

static int validate_scene(const ard_scene& s, std::string* err) {
  if (!(s.dh > 0) || !(s.dt > 0) || !(s.c0 > 0)) { *err = "scene: dh, dt, c0 must be positive"; return ARD_ERR_INVALID; }
  if (s.n_partitions < 1 || !s.partitions) { *err = "scene: no partitions"; return ARD_ERR_INVALID; }
  if (s.pml_layers < 4) { *err = "scene: pml_layers must be >= 4"; return ARD_ERR_INVALID; }
  // The modal update is exact in time; the PML leapfrog is not.  The bare
  // 6th-order Laplacian allows c dt / h <= sqrt(4 * 180 / (3 * 1088)) = 0.470;
  // with the PML damping terms the step is stable at 0.43 (the reference's
  // own dh = 0.1 m, dt = 1/8000 s) and diverges at 0.45, so refuse above 0.44.
  const double cfl = (double)s.c0 * s.dt / s.dh;
  if (cfl > 0.44) {
    *err = "scene: c0*dt/dh = " + std::to_string(cfl) + " exceeds the PML leapfrog stability limit (0.44)";
    return ARD_ERR_UNSTABLE;
  }
  for (int i = 0; i < s.n_partitions; ++i) {
    const ard_partition& p = s.partitions[i];
    if (p.width < 1 || p.height < 1 || p.depth < 1) { *err = "scene: empty partition " + std::to_string(i); return ARD_ERR_INVALID; }
    if (p.kind == ARD_PART_DCT) {
      if (p.width < 6 || p.height < 6 || p.depth < 6) {
        *err = "scene: air partition " + std::to_string(i) + " has an extent below 6 cells";
        return ARD_ERR_INVALID;
      }
    } else if (p.kind == ARD_PART_PML) {
      if (p.pml_type < 0 || p.pml_type > 5) { *err = "scene: bad pml_type"; return ARD_ERR_INVALID; }
      const int L = (p.pml_type <= 1) ? p.width : (p.pml_type <= 3 ? p.height : p.depth);
      if (L < 3) { *err = "scene: PML thinner than 3 cells"; return ARD_ERR_INVALID; }
    } else {
      *err = "scene: bad partition kind"; return ARD_ERR_INVALID;
    }
  }
  return ARD_OK;
}

// Kernel attributes must be set on the instances this file launches (each
// translation unit holds its own instances of the kernel templates): the FP64
// modal kernel needs more than 48 KB of dynamic shared memory.
static int configure_kernels(Ctx* ctx) {
  const int modal_smem = (int)(kModalSmemElems * elem_size(ctx));
  // The attribute belongs to the kernel, process-wide, not to the context:
  // set the device's opt-in maximum so that contexts with different layer
  // sizes can be interleaved in one process.
  const int f2d = std::max(ctx->smem_optin, (int)ctx->f2d_bytes);
  if (ctx->prec == ARD_PREC_F64) {
    ARD_CUDA(cudaFuncSetAttribute(modal_kernel<double, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, modal_smem));
    ARD_CUDA(cudaFuncSetAttribute(modal_kernel<double, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, modal_smem));
    if (ctx->fused_faces) {
      ARD_CUDA(cudaFuncSetAttribute(face2d_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, f2d));
      ARD_CUDA(cudaFuncSetAttribute(face2d_cluster_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, f2d));
    }
  } else {
    ARD_CUDA(cudaFuncSetAttribute(modal_kernel<float, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, modal_smem));
    ARD_CUDA(cudaFuncSetAttribute(modal_kernel<float, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, modal_smem));
    if (ctx->fused_faces) {
      ARD_CUDA(cudaFuncSetAttribute(face2d_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, f2d));
      ARD_CUDA(cudaFuncSetAttribute(face2d_cluster_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, f2d));
    }
  }
  ARD_CUDA(ctx->prec == ARD_PREC_F64 ? configure_face_gemm<double>() : configure_face_gemm<float>());
  if (ctx->mma_faces)
    ARD_CUDA(cudaFuncSetAttribute(face_mma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kMmaSmemBytes));
  return ARD_OK;
}

extern "C" int ard_abi_version(void) { return ARD_ABI_VERSION; }

extern "C" int ard_create(const ard_scene* scenes, int32_t n_scenes, const ard_options* opt, ard_ctx** out) {
  g_create_error.clear();
  if (!scenes || n_scenes < 1 || !out) { g_create_error = "ard_create: need >= 1 scene and an output pointer"; return ARD_ERR_INVALID; }
  for (int s = 0; s < n_scenes; ++s) {
    std::string err;
    int rc = validate_scene(scenes[s], &err);
    if (rc) { g_create_error = "scene " + std::to_string(s) + ": " + err; return rc; }
  }
  auto ctx = std::make_unique<Ctx>();
  ctx->prec = opt ? opt->precision : ARD_PREC_F32;
  ctx->max_steps = (opt && opt->max_steps > 0) ? opt->max_steps : 4096;
  ctx->use_graphs = opt ? (opt->use_graphs != 0) : true;
  ctx->device = opt ? opt->device : 0;
  ctx->arith = opt ? opt->arithmetic : ARD_ARITH_ACCURATE;
  ctx->adjoint = opt ? (opt->adjoint != 0) : false;
  {
    const char* dbg = std::getenv("ARD_DEBUG_SYNC");
    ctx->debug_sync = dbg && dbg[0] == '1';
    if (ctx->debug_sync) ctx->use_graphs = false;
    // ARD_FACE_TWO_PASS=1: the two-pass face transforms (tensor-core passes in
    // FP32) even where the fused face kernel fits
    const char* tp = std::getenv("ARD_FACE_TWO_PASS");
    if (tp && tp[0] == '1') ctx->tune_gemm = 1;
  }
  if (ctx->arith != ARD_ARITH_ACCURATE && ctx->arith != ARD_ARITH_REFERENCE) {
    g_create_error = "ard_create: bad arithmetic mode";
    return ARD_ERR_INVALID;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    g_create_error = "ard_create: no CUDA device";
    return ARD_ERR_NOGPU;
  }
  if (ctx->device < 0 || ctx->device >= ndev) { g_create_error = "ard_create: bad device ordinal"; return ARD_ERR_INVALID; }
  if (cudaSetDevice(ctx->device) != cudaSuccess) { g_create_error = "ard_create: cudaSetDevice failed"; return ARD_ERR_CUDA; }
  cudaDeviceProp prop;
  cudaGetDeviceProperties(&prop, ctx->device);
  if (prop.major * 10 + prop.minor != 103) {
    g_create_error = "ard_create: kernels are built for sm_103a; device is sm_" + std::to_string(prop.major) + std::to_string(prop.minor);
    return ARD_ERR_NOGPU;
  }
  ctx->num_sms = prop.multiProcessorCount;
  ctx->smem_optin = (int)prop.sharedMemPerBlockOptin;
  ctx->smem_per_sm = prop.sharedMemPerMultiprocessor;
  const bool autotune = opt && opt->autotune != 0;
  auto describe = [](const Ctx* c) {
    return std::string("tiles x") + std::to_string(c->tune_tiles) + ", lanes/row " +
           (c->tune_g_shift == 0 ? "fit" : (c->tune_g_shift == 1 ? "narrow" : "narrower")) + ", faces " + (c->fused_faces ? "fused" : (c->mma_faces ? "tensor-core" : "gemm")) + ", " +
           std::to_string(c->tiles.size()) + " modal tiles, " + std::to_string(c->ngroups) + " air stream(s)";
  };
  if (!autotune) {
    int rc = build_layout(ctx.get(), scenes, n_scenes);
    if (rc == ARD_OK) rc = configure_kernels(ctx.get());
    if (rc) {
      g_create_error = ctx->err;
      free_ctx_device(ctx.get());
      return rc;
    }
    ctx->tuning = describe(ctx.get());
    *out = reinterpret_cast<ard_ctx*>(ctx.release());
    return ARD_OK;
  }
  // Autotuner: build the context for each candidate layout, time real steps
  // (CUDA graphs, the production path), keep the fastest.
  struct Cand { int tiles, gshift, gemm; };
  const Cand cands[] = {{1, 2, 0}, {2, 2, 0}, {4, 2, 0}, {1, 1, 0}, {2, 1, 0}, {1, 0, 0}, {2, 0, 0}, {1, 2, 1}};
  std::unique_ptr<Ctx> best;
  float best_ms = 0.f;
  std::string report;
  const int warm = 64, timed = 64;
  for (const Cand& cd : cands) {
    auto c = std::make_unique<Ctx>();
    c->prec = ctx->prec; c->max_steps = std::max<long long>(ctx->max_steps, warm + timed);
    c->use_graphs = ctx->use_graphs; c->device = ctx->device; c->arith = ctx->arith; c->adjoint = ctx->adjoint;
    c->debug_sync = ctx->debug_sync; c->num_sms = ctx->num_sms; c->smem_optin = ctx->smem_optin;
    c->smem_per_sm = ctx->smem_per_sm;
    c->tune_tiles = cd.tiles; c->tune_g_shift = cd.gshift; c->tune_gemm = cd.gemm;
    int rc = build_layout(c.get(), scenes, n_scenes);
    if (rc == ARD_OK) rc = configure_kernels(c.get());
    // the GEMM candidate is a distinct layout only where the fused transforms fit
    if (rc == ARD_OK && cd.gemm &&
        (c->dct.empty() || c->f2d_bytes > (size_t)std::min(c->smem_optin, 200 * 1024)))
      rc = ARD_ERR_INVALID;
    float ms = 0.f;
    if (rc == ARD_OK) {
      ard_ctx* h = reinterpret_cast<ard_ctx*>(c.get());
      cudaEvent_t e0 = nullptr, e1 = nullptr;
      rc = ard_step(h, warm, nullptr);
      if (rc == ARD_OK && cudaEventCreate(&e0) == cudaSuccess && cudaEventCreate(&e1) == cudaSuccess) {
        cudaEventRecord(e0, c->stream);
        rc = ard_step(h, timed, nullptr);
        cudaEventRecord(e1, c->stream);
        if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) rc = ARD_ERR_CUDA;
      }
      if (e0) cudaEventDestroy(e0);
      if (e1) cudaEventDestroy(e1);
    }
    if (rc != ARD_OK) {
      free_ctx_device(c.get());
      continue;
    }
    report += "[" + describe(c.get()) + ": " + std::to_string(ms / timed * 1000.f) + " us/step] ";
    if (!best || ms < best_ms) {
      if (best) free_ctx_device(best.get());
      best = std::move(c);
      best_ms = ms;
    } else {
      free_ctx_device(c.get());
    }
  }
  if (!best) {
    g_create_error = "ard_create: no autotuner candidate could be built";
    return ARD_ERR_INVALID;
  }
  best->max_steps = ctx->max_steps < best->max_steps ? best->max_steps : ctx->max_steps;
  int rc = ard_reset(reinterpret_cast<ard_ctx*>(best.get()));
  if (rc == ARD_OK) rc = configure_kernels(best.get());   // attributes of the kept layout last
  if (rc) {
    g_create_error = best->err;
    free_ctx_device(best.get());
    return rc;
  }
  best->tuning = "autotuned: " + describe(best.get()) + "; candidates " + report;
  *out = reinterpret_cast<ard_ctx*>(best.release());
  return ARD_OK;
}

extern "C" int ard_describe(const ard_ctx* c, char* buf, int64_t n) {
  if (!c || !buf || n < 1) return ARD_ERR_INVALID;
  const Ctx* ctx = reinterpret_cast<const Ctx*>(c);
  std::string e = ctx->tuning;
  if (!ctx->adj_mode.empty())
    e += "; last adjoint: " + ctx->adj_mode + (ctx->adj_k ? ", segments of " + std::to_string(ctx->adj_k) + " steps" : "");
  const size_t k = std::min<size_t>((size_t)(n - 1), e.size());
  std::memcpy(buf, e.data(), k);
  buf[k] = 0;
  return ARD_OK;
}

extern "C" int ard_destroy(ard_ctx* c) {
  if (!c) return ARD_OK;
  Ctx* ctx = reinterpret_cast<Ctx*>(c);
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  free_ctx_device(ctx);
  delete ctx;
  return ARD_OK;
}

extern "C" int ard_last_error(const ard_ctx* c, char* buf, int64_t n) {
  const std::string& e = c ? reinterpret_cast<const Ctx*>(c)->err : g_create_error;
  if (buf && n > 0) {
    const size_t k = std::min<size_t>((size_t)(n - 1), e.size());
    std::memcpy(buf, e.data(), k);
    buf[k] = 0;
  }
  return ARD_OK;
}

extern "C" int ard_kernels_per_step(const ard_ctx* c, int32_t* out) {
  if (!c || !out) return ARD_ERR_INVALID;
  const Ctx* ctx = reinterpret_cast<const Ctx*>(c);
  int n = ctx->pml_blocks.empty() ? 0 : 1;
  for (int g = 0; g < (ctx->dct.empty() ? 0 : ctx->ngroups); ++g) {
    const Ctx::AirGroup& G = ctx->groups[g];
    if (ctx->fused_faces) n += (G.f_hi > G.f_lo ? 1 : 0) + (G.i_hi > G.i_lo ? 1 : 0);   // face transforms
    else n += 4;
    n += G.t_hi > G.t_lo ? 1 : 0;                                                       // modal update
    n += (G.r_hi > G.r_lo || G.s_total > 0) ? 1 : 0;                                    // recorder + partial sums
    n += (ctx->d_cube_hist && G.r_hi > G.r_lo) ? 3 : 0;                                  // recorder neighbourhoods
  }
  n += ctx->n_face_cells > 0 ? 1 : 0;        // interfaces
  *out = n;
  return ARD_OK;
}

extern "C" int ard_time_step(const ard_ctx* c, int64_t* out) {
  if (!c || !out) return ARD_ERR_INVALID;
  *out = reinterpret_cast<const Ctx*>(c)->t_host;
  return ARD_OK;
}

extern "C" int ard_synchronize(ard_ctx* c) {
  if (!c) return ARD_ERR_INVALID;
  Ctx* ctx = reinterpret_cast<Ctx*>(c);
  ARD_CUDA(cudaSetDevice(ctx->device));
  ARD_CUDA(cudaStreamSynchronize(ctx->stream));
  ARD_CUDA(cudaStreamSynchronize(ctx->stream2));
  return check_device_error(ctx);
}

// ---------------------------------------------------------------------------
// step launches
// ---------------------------------------------------------------------------

namespace ard {

// Stage order of one step; with `ev` (kNumStages + 1 events, direct launches
// on one stream) event k is recorded before stage k and event kNumStages
// after the last stage.
template <typename T>
int launch_step(Ctx* ctx, int par, int tstep, cudaStream_t s, cudaStream_t s2, bool fork, cudaEvent_t* ev) {
  T* buf = reinterpret_cast<T*>(ctx->d_buf);
  // checked mode (ARD_DEBUG_SYNC=1): every stage is synchronised and its error
  // reported with the stage name, so a failing kernel is identified
  const char* stage_names[] = {"pml", "fwd", "fwd2", "modal", "recorder", "inv", "inv2", "iface", "end"};
  auto mark = [&](int k) -> cudaError_t {
    if (ctx->debug_sync && k > 0) {
      cudaError_t e = cudaStreamSynchronize(s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s2);
      if (e != cudaSuccess) {
        std::fprintf(stderr, "ard: stage before '%s' failed: %s\n", stage_names[k], cudaGetErrorString(e));
        return e;
      }
    }
    return ev ? cudaEventRecord(ev[k], s) : cudaSuccess;
  };
  // PML branch depends only on the previous step's interface forcing
  if (fork) {
    ARD_CUDA(cudaEventRecord(ctx->ev_fork, s));
    ARD_CUDA(cudaStreamWaitEvent(s2, ctx->ev_fork, 0));
  }
  cudaStream_t sp = fork ? s2 : s;
  ARD_CUDA(mark(kStagePml));
  if (int rc = launch_pml<T>(ctx, par, tstep, sp)) return rc;
  if (!ctx->dct.empty()) {
    const int gx = ctx->num_sms * 4;
    const size_t msmem = kModalSmemElems * sizeof(T);
    // one stage of one group's air branch on stream `st`
    auto stage = [&](int k, const Ctx::AirGroup& G, cudaStream_t st) -> int {
      if (k == kStageFwdRows) {
        if (ctx->fused_faces) {
          const int n = G.f_hi - G.f_lo;
          ARD_CUDA(launch_face2d<T>(G.f_split, n, gx, ctx->f2d_bytes, st, buf, ctx->d_fwd2d + 2 * G.f_lo,
                                    ctx->f2d_smem));
        } else if (ctx->mma_faces) {
          ARD_CUDA(launch_mma(ctx, 0, st));
        } else {
          ARD_CUDA(launch_face_gemm<T>(buf, ctx->fwd1.jobs[0], ctx->d_fwd1, (int)ctx->fwd1.jobs.size(), ctx->fwd1.units,
                                        grid_for(ctx->fwd1.units, 1, ctx->num_sms * 2), st));
        }
      } else if (k == kStageFwdCols) {
        if (ctx->mma_faces)
          ARD_CUDA(launch_mma(ctx, 1, st));
        else if (!ctx->fused_faces)
          ARD_CUDA(launch_face_gemm<T>(buf, ctx->fwd2.jobs[0], ctx->d_fwd2, (int)ctx->fwd2.jobs.size(), ctx->fwd2.units,
                                        grid_for(ctx->fwd2.units, 1, ctx->num_sms * 2), st));
      } else if (k == kStageModal) {
        const int n = G.t_hi - G.t_lo;
        if (n > 0) {
          ModalArgs<T> ma{buf, ctx->d_dct, ctx->d_tiles + G.t_lo, n, ctx->d_srcpts, ctx->d_recpts,
                          ctx->d_series, ctx->max_steps, ctx->d_t, tstep, par, nullptr, 0};
          const int mgrid = grid_for(n, 1, ctx->num_sms * 2);
          if (ctx->arith == ARD_ARITH_REFERENCE)
            ARD_CUDA(launch_dep(modal_kernel<T, true, false>, mgrid, kModalThreads, msmem, st, ma));
          else
            ARD_CUDA(launch_dep(modal_kernel<T, false, false>, mgrid, kModalThreads, msmem, st, ma));
        }
      } else if (k == kStageRecorder) {
        if (int rc = launch_post_modal_range<T>(ctx, st, tstep, G.r_lo, G.r_hi, G.s_lo, G.s_hi, G.s_first, G.s_total))
          return rc;
        return launch_cubes<T>(ctx, st, tstep, par, G.r_lo, G.r_hi);
      } else if (k == kStageInvCols) {
        if (ctx->fused_faces) {
          const int n = G.i_hi - G.i_lo;
          ARD_CUDA(launch_face2d<T>(G.i_split, n, gx, ctx->f2d_bytes, st, buf, ctx->d_inv2d + 2 * G.i_lo,
                                    ctx->f2d_smem));
        } else if (ctx->mma_faces) {
          ARD_CUDA(launch_mma(ctx, 2, st));
        } else {
          ARD_CUDA(launch_face_gemm<T>(buf, ctx->inv1.jobs[0], ctx->d_inv1, (int)ctx->inv1.jobs.size(), ctx->inv1.units,
                                        grid_for(ctx->inv1.units, 1, ctx->num_sms * 2), st));
        }
      } else if (k == kStageInvRows) {
        if (ctx->mma_faces)
          ARD_CUDA(launch_mma(ctx, 3, st));
        else if (!ctx->fused_faces)
          ARD_CUDA(launch_face_gemm<T>(buf, ctx->inv2.jobs[0], ctx->d_inv2, (int)ctx->inv2.jobs.size(), ctx->inv2.units,
                                        grid_for(ctx->inv2.units, 1, ctx->num_sms * 2), st));
      }
      ARD_CUDA(cudaGetLastError());
      return ARD_OK;
    };
    const int stages[] = {kStageFwdRows, kStageFwdCols, kStageModal, kStageRecorder, kStageInvCols, kStageInvRows};
    if (fork && ctx->ngroups == 2) {
      // the second group's air branch on its own stream (independent until the interfaces)
      ARD_CUDA(cudaStreamWaitEvent(ctx->stream3, ctx->ev_fork, 0));
      for (int k : stages) {
        if (int rc = stage(k, ctx->groups[0], s)) return rc;
        if (int rc = stage(k, ctx->groups[1], ctx->stream3)) return rc;
      }
      ARD_CUDA(cudaEventRecord(ctx->ev_join3, ctx->stream3));
      ARD_CUDA(cudaStreamWaitEvent(s, ctx->ev_join3, 0));
    } else {
      for (int k : stages) {
        ARD_CUDA(mark(k));
        for (int g = 0; g < ctx->ngroups; ++g)
          if (int rc = stage(k, ctx->groups[g], s)) return rc;
      }
    }
  }
  if (fork) {
    ARD_CUDA(cudaEventRecord(ctx->ev_join, s2));
    ARD_CUDA(cudaStreamWaitEvent(s, ctx->ev_join, 0));
  }
  ARD_CUDA(mark(kStageIface));
  if (ctx->n_face_cells > 0) {
    IfaceArgs<T> ia{buf, ctx->d_ifs, ctx->d_cell_iface, ctx->n_face_cells, ctx->d_mask, par, (T)ctx->c0,
                    (T)ctx->dh};
    ARD_CUDA(launch_dep(iface_kernel<T>, grid_for(ctx->n_face_cells, 256, ctx->num_sms * 16), 256, 0, s, ia));
    ARD_CUDA(cudaGetLastError());
  }
  ARD_CUDA(mark(kNumStages));
  return ARD_OK;
}

// The PML update of every slab for step (*d_t + tstep).
template <typename T>
int launch_pml(Ctx* ctx, int par, int tstep, cudaStream_t s) {
  if (ctx->pml_blocks.empty()) return ARD_OK;
  PmlArgs<T> pa{reinterpret_cast<T*>(ctx->d_buf), ctx->d_pml, ctx->d_pml_blocks, (int)ctx->pml_blocks.size(), par,
                (T)ctx->dt, (T)ctx->dh, (T)ctx->c0, (const PmlHist<T>*)ctx->d_phist, ctx->d_t, tstep,
                ctx->d_pml_maps, ctx->d_err};
  ARD_CUDA(launch_dep(pml_kernel<T>, grid_for((long long)ctx->pml_blocks.size(), 1, ctx->num_sms * 8), 256, 0, s, pa));
  ARD_CUDA(cudaGetLastError());
  return ARD_OK;
}

template int launch_pml<float>(Ctx*, int, int, cudaStream_t);
template int launch_pml<double>(Ctx*, int, int, cudaStream_t);

// Recorder sums of recorders [r_lo, r_hi) and partial sums of jobs
// [s_lo, s_hi) (their elements start at s_first, s_total of them) in one launch.
template <typename T>
int launch_post_modal_range(Ctx* ctx, cudaStream_t s, int tstep, int r_lo, int r_hi, int s_lo, int s_hi,
                            long long s_first, long long s_total) {
  const int nrec = r_hi - r_lo;
  const int rec_blocks = (nrec * 32 + 255) / 256;
  // chunks of 8 elements per thread where the chunks fill a wave of blocks;
  // one element per thread for smaller launches
  const int wave = ctx->num_sms * 8;
  const long long nchunks = s_total / kSumChunk;
  const int per = nchunks >= wave ? 8 : 0;
  const int sum_blocks = s_total <= 0 ? 0 : (per ? grid_for(nchunks, 1, wave) : grid_for(s_total, 256, wave));
  if (rec_blocks + sum_blocks == 0) return ARD_OK;
  PostModalArgs<T> a{reinterpret_cast<T*>(ctx->d_buf), ctx->d_dct, ctx->d_recpts, r_lo, nrec, ctx->n_rec_total,
                     ctx->d_hist, ctx->d_t, tstep, ctx->max_steps, rec_blocks, ctx->d_psum + s_lo, s_hi - s_lo,
                     s_first, s_total, per};
  ARD_CUDA(launch_dep(post_modal_kernel<T>, rec_blocks + sum_blocks, 256, 0, s, a));
  ARD_CUDA(cudaGetLastError());
  return ARD_OK;
}

template int launch_post_modal_range<float>(Ctx*, cudaStream_t, int, int, int, int, int, long long, long long);
template int launch_post_modal_range<double>(Ctx*, cudaStream_t, int, int, int, int, int, long long, long long);

// Recorder sums (with_recorders) and partial sums of all air partitions in one launch.
template <typename T>
int launch_post_modal(Ctx* ctx, cudaStream_t s, int tstep, bool with_recorders) {
  return launch_post_modal_range<T>(ctx, s, tstep, 0, with_recorders ? (int)ctx->recpts.size() : 0, 0,
                                    (int)ctx->psum.size(), 0, ctx->psum_total);
}

template int launch_post_modal<float>(Ctx*, cudaStream_t, int, bool);
template int launch_post_modal<double>(Ctx*, cudaStream_t, int, bool);
template int launch_step<float>(Ctx*, int, int, cudaStream_t, cudaStream_t, bool, cudaEvent_t*);
template int launch_step<double>(Ctx*, int, int, cudaStream_t, cudaStream_t, bool, cudaEvent_t*);

int launch_steps_direct(Ctx* ctx, int n, cudaStream_t s) {
  for (int i = 0; i < n; ++i) {
    const int par = (int)((ctx->t_host + i) & 1);
    int rc = ctx->prec == ARD_PREC_F64 ? launch_step<double>(ctx, par, i, s, s, false, nullptr)
                                       : launch_step<float>(ctx, par, i, s, s, false, nullptr);
    if (rc) return rc;
  }
  advance_time_kernel<<<1, 32, 0, s>>>(ctx->d_t, n);
  ARD_CUDA(cudaGetLastError());
  ctx->t_host += n;
  return ARD_OK;
}

int ensure_graph(Ctx* ctx) {
  if (ctx->graph_exec) return ARD_OK;
  cudaGraph_t g = nullptr;
  ARD_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  int rc = ARD_OK;
  for (int i = 0; i < ctx->graph_steps && rc == ARD_OK; ++i) {
    rc = ctx->prec == ARD_PREC_F64 ? launch_step<double>(ctx, i & 1, i, ctx->stream, ctx->stream2, true, nullptr)
                                   : launch_step<float>(ctx, i & 1, i, ctx->stream, ctx->stream2, true, nullptr);
  }
  if (rc == ARD_OK) advance_time_kernel<<<1, 32, 0, ctx->stream>>>(ctx->d_t, ctx->graph_steps);
  cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
  if (rc) { if (g) cudaGraphDestroy(g); return rc; }
  if (e != cudaSuccess) { ctx->err = std::string("graph capture: ") + cudaGetErrorString(e); return ARD_ERR_CUDA; }
  e = cudaGraphInstantiate(&ctx->graph_exec, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) { ctx->err = std::string("graph instantiate: ") + cudaGetErrorString(e); return ARD_ERR_CUDA; }
  return ARD_OK;
}

}  // namespace ard

extern "C" int ard_step(ard_ctx* c, int64_t nsteps, void* stream) {
  if (!c || nsteps < 0) return ARD_ERR_INVALID;
  Ctx* ctx = reinterpret_cast<Ctx*>(c);
  ARD_CUDA(cudaSetDevice(ctx->device));
  cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
  if (s != ctx->stream) {
    // order the caller's stream after everything queued on ours and vice versa
    ARD_CUDA(cudaEventRecord(ctx->ev_fork, ctx->stream));
    ARD_CUDA(cudaStreamWaitEvent(s, ctx->ev_fork, 0));
  }
  int64_t left = nsteps;
  if (ctx->use_graphs && ctx->graph_steps > 0 && left >= ctx->graph_steps) {
    if (ctx->t_host & 1) {
      int rc = launch_steps_direct(ctx, 1, s);
      if (rc) return rc;
      --left;
    }
    int rc = ensure_graph(ctx);
    if (rc) return rc;
    while (left >= ctx->graph_steps) {
      ARD_CUDA(cudaGraphLaunch(ctx->graph_exec, s));
      ctx->t_host += ctx->graph_steps;
      left -= ctx->graph_steps;
    }
  }
  if (left > 0) {
    int rc = launch_steps_direct(ctx, (int)left, s);
    if (rc) return rc;
  }
  if (s != ctx->stream) {
    ARD_CUDA(cudaEventRecord(ctx->ev_join, s));
    ARD_CUDA(cudaStreamWaitEvent(ctx->stream, ctx->ev_join, 0));
  }
  if (ctx->debug_sync) {
    ARD_CUDA(cudaStreamSynchronize(s));
    return check_guards(ctx);
  }
  return ARD_OK;
}

extern "C" int ard_profile_steps(ard_ctx* c, int64_t nsteps, void* stream, float* stage_ms, int32_t nstages) {
  if (!c || nsteps < 1 || !stage_ms || nstages < kNumStages) return ARD_ERR_INVALID;
  Ctx* ctx = reinterpret_cast<Ctx*>(c);
  ARD_CUDA(cudaSetDevice(ctx->device));
  cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
  if (s != ctx->stream) {
    ARD_CUDA(cudaEventRecord(ctx->ev_fork, ctx->stream));
    ARD_CUDA(cudaStreamWaitEvent(s, ctx->ev_fork, 0));
  }
  std::vector<cudaEvent_t> ev((size_t)nsteps * (kNumStages + 1));
  for (auto& e : ev) ARD_CUDA(cudaEventCreate(&e));
  int rc = ARD_OK;
  for (int64_t i = 0; i < nsteps && rc == ARD_OK; ++i) {
    const int par = (int)((ctx->t_host + i) & 1);
    cudaEvent_t* e = ev.data() + i * (kNumStages + 1);
    rc = ctx->prec == ARD_PREC_F64 ? launch_step<double>(ctx, par, (int)i, s, s, false, e)
                                   : launch_step<float>(ctx, par, (int)i, s, s, false, e);
  }
  if (rc == ARD_OK) {
    advance_time_kernel<<<1, 32, 0, s>>>(ctx->d_t, (int)nsteps);
    ctx->t_host += nsteps;
    cudaError_t err = cudaEventSynchronize(ev.back());
    for (int k = 0; k < nstages; ++k) stage_ms[k] = 0.f;
    for (int64_t i = 0; i < nsteps && err == cudaSuccess; ++i)
      for (int k = 0; k < kNumStages; ++k) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ev[i * (kNumStages + 1) + k], ev[i * (kNumStages + 1) + k + 1]);
        stage_ms[k] += ms / (float)nsteps;
      }
    if (err != cudaSuccess) { ctx->err = cudaGetErrorString(err); rc = ARD_ERR_CUDA; }
  }
  for (auto& e : ev) cudaEventDestroy(e);
  if (s != ctx->stream && rc == ARD_OK) {
    ARD_CUDA(cudaEventRecord(ctx->ev_join, s));
    ARD_CUDA(cudaStreamWaitEvent(ctx->stream, ctx->ev_join, 0));
  }
  return rc;
}
