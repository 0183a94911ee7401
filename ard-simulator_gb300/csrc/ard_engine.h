// Host-side context of the GB300 ARD engine (internal; the public ABI is
// include/ard_gb300.h).
#pragma once

#include <cuda_runtime.h>

#include <array>
#include <string>
#include <vector>

#include "ard_device.cuh"
#include "ard_gb300.h"
#include "ard_kernels.cuh"

// Host: a CUDA runtime call inside an entry point with a Ctx* named ctx;
// a failure records the call and the CUDA error on the context and returns
// ARD_ERR_OOM (allocation) or ARD_ERR_CUDA.
#define ARD_CUDA(call)                                                                                   \
  do {                                                                                                   \
    cudaError_t e_ = (call);                                                                             \
    if (e_ != cudaSuccess) {                                                                             \
      ctx->err = std::string(#call) + ": " + cudaGetErrorName(e_) + " (" + cudaGetErrorString(e_) + ")"; \
      return e_ == cudaErrorMemoryAllocation ? ARD_ERR_OOM : ARD_ERR_CUDA;                               \
    }                                                                                                    \
  } while (0)

namespace ard {

struct JobList {
  std::vector<XformJob> jobs;
  int units = 0;
  void add(XformJob j, int units_of_job) {
    j.first = units;
    jobs.push_back(j);
    units += units_of_job;
  }
};

struct SceneRec {
  std::vector<ard_partition> parts;
  std::vector<int> engine_idx;   // per scene partition: DctDev or PmlDev index
  int src0 = 0, nsrc = 0;        // global source slots
  int rec0 = 0, nrec = 0;        // global recorder slots
  std::array<double, 6> scale{{1, 1, 1, 1, 1, 1}};
};

struct Ctx {
  // configuration
  int prec = ARD_PREC_F32;
  int arith = ARD_ARITH_ACCURATE;
  int device = 0;
  int num_sms = 1;
  int smem_optin = 48 * 1024;
  size_t smem_per_sm = 228 * 1024;
  long long max_steps = 4096;
  bool use_graphs = true;
  bool debug_sync = false;          // ARD_DEBUG_SYNC=1: synchronise and check after every stage
  int graph_steps = 32;
  double dh = 0, dt = 0, c0 = 0, pml_R = 1e-5, damping = 0.999;
  int pml_layers = 0;
  std::string err;

  // work tables (host copies)
  std::vector<SceneRec> scenes;
  std::vector<DctDev> dct;
  std::vector<PmlDev> pml;
  std::vector<int4> pml_blocks;
  std::vector<IfaceDev> ifs;
  std::vector<unsigned char> masks;
  std::vector<int> cell_iface;              // interface of every face cell
  std::vector<PointDev> srcpts, recpts;
  std::vector<int4> tiles;
  JobList fwd1, fwd2, inv1, inv2;           // two-pass GEMM face transforms
  std::vector<Face2DJob> fwd2d, inv2d;      // fused face transforms
  std::vector<SumJob> psum;                 // partial sums before the inverse transforms
  long long psum_total = 0;
  std::vector<int> psum_lo;                 // first partial-sum job of every air partition
  // Air partitions in up to two groups whose air branches (face transforms,
  // modal update, sums) run on two streams inside the step graph; ranges
  // into the forward job lists, the tiles, the recorders and the sums.
  struct AirGroup {
    int part_lo = 0, part_hi = 0;
    int f_lo = 0, f_hi = 0, i_lo = 0, i_hi = 0;
    bool f_split = false, i_split = false;   // the range holds row-split face jobs (cluster launch)
    int t_lo = 0, t_hi = 0, r_lo = 0, r_hi = 0, s_lo = 0, s_hi = 0;
    long long s_first = 0, s_total = 0;
  };
  int ngroups = 1;
  AirGroup groups[2];
  bool fused_faces = false;
  // Tensor-core face transforms (FP32 contexts whose faces take the two-pass
  // form): the four passes as batched split-TF32 products (ard_mma.cuh), with
  // the split transform tables of every extent in the pool.
  bool mma_faces = false;
  std::vector<MmaJob> mjobs[8];            // forward pass 1, 2; inverse pass 1, 2; adjoint passes 1 .. 4
  int mtiles[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  std::vector<std::pair<int, long long>> mma_tables;   // extent -> offset of Chi, Clo, CiThi, CiTlo
  Face2DSmem f2d_smem{0, 0, 0, 0};
  size_t f2d_bytes = 0;
  std::vector<std::pair<int, long long>> cos_tables;  // extent -> offset
  long long n_pml_cells = 0, n_face_cells = 0;
  long long n_air_cells = 0;
  int n_src_total = 0, n_rec_total = 0;
  int maxn = 0;
  long long pool_elems = 0;
  long long scratch = 0;          // dense-transform scratch (3 x largest air partition)
  long long state_begin = 0, state_end = 0;  // checkpointed state block
  long long adj_begin = 0, adj_end = 0;      // adjoint state block
  long long pml_region[8][2] = {};           // all slabs' p0, p1, phn0, phn1, pha0, pha1, phb0, phb1
  long long force_begin = 0;                 // all slabs' strip forces: [force_begin, state_end)
  bool adjoint = false;
  // layout choices (the autotuner varies them; defaults are the heuristics)
  int tune_tiles = 1;      // modal tiles per wave slot (x 2 per SM): kz split finer when > 1
  int tune_g_shift = 2;    // k > 0: ky rows k lane-sizes narrower (more kx tiles, more ky rows per tile)
  int tune_gemm = 0;       // 1: two-pass GEMM face transforms even when the fused ones fit
  std::string tuning;      // description of the chosen layout
  // adjoint face transforms (options.adjoint): fused 2D jobs and the two-pass
  // GEMM form (q rows, q columns, R columns, R rows)
  std::vector<Face2DJob> adj1_2d, adj2_2d;
  bool adj1_split = false, adj2_split = false;
  JobList adjg[4];
  long long q_begin = 0, q_end = 0;          // adjoint face pressure (zeroed every adjoint step)
  bool adj_valid = false;                    // adjoint levels hold mu(0), mu(1) of the last ard_adjoint
  std::string adj_mode;                      // how the last ard_adjoint obtained forward PML values
  long long adj_k = 0;                       // its segment length

  // device memory
  void* d_buf = nullptr;          // element pool (float or double)
  void* d_buf_base = nullptr;     // allocation holding the pool (and guards in checked mode)
  size_t guard_bytes = 0;
  unsigned char* d_mask = nullptr;
  DctDev* d_dct = nullptr;
  PmlDev* d_pml = nullptr;
  int4* d_pml_blocks = nullptr;
  IfaceDev* d_ifs = nullptr;
  int* d_cell_iface = nullptr;
  PointDev* d_srcpts = nullptr;
  PointDev* d_recpts = nullptr;
  int4* d_tiles = nullptr;
  XformJob *d_fwd1 = nullptr, *d_fwd2 = nullptr, *d_inv1 = nullptr, *d_inv2 = nullptr;
  Face2DJob *d_fwd2d = nullptr, *d_inv2d = nullptr;
  SumJob* d_psum = nullptr;
  float* d_series = nullptr;
  double* d_hist = nullptr;
  long long* d_t = nullptr;
  Face2DJob *d_adj1_2d = nullptr, *d_adj2_2d = nullptr;
  XformJob* d_adjg[4] = {nullptr, nullptr, nullptr, nullptr};
  long long* d_tb = nullptr;      // adjoint counters {current step, first step of the PML history}
  void* d_phist = nullptr;        // PmlHist<T> read by the PML kernel (adjoint contexts only)
  MmaJob* d_mjobs[8] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  int* d_err = nullptr;           // set by a kernel whose bounded wait ran out (checked on synchronize)
  CUtensorMap* d_pml_maps = nullptr;   // tensor maps of the PML tile loads (build_pml_maps)
  CUtensorMap* d_pml_amaps = nullptr;  // the adjoint PML kernel's (options.adjoint)

  // neighbourhood recording (ard_record_neighbourhoods): the 10 x 10 x 10
  // pressure cube around every recorder after every step, [max_steps][n_rec_total][1000]
  float* d_cube_hist = nullptr;
  void* d_cube_tmp = nullptr;     // contraction scratch (T): per recorder T1 [d][h][10], T2 [d][100]
  long long cube_s1 = 0, cube_s2 = 0;
  int cube_row_blocks = 0, cube_dmax = 0;
  long long cube_t0 = 0;          // first step whose cube is recorded

  cudaStream_t stream = nullptr, stream2 = nullptr, stream3 = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_join3 = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  long long t_host = 0;
};

// stages of one step, in launch order (per-stage timing)
enum { kStagePml = 0, kStageFwdRows, kStageFwdCols, kStageModal, kStageRecorder, kStageInvCols, kStageInvRows,
       kStageIface, kNumStages };

int build_layout(Ctx* ctx, const ard_scene* scenes, int n_scenes);
int build_pml_maps(Ctx* ctx);
int build_pml_hist_maps(Ctx* ctx, const void* hist, long long hlen, long long slots, CUtensorMap** out);
cudaError_t launch_mma(Ctx* ctx, int k, cudaStream_t s);
void free_ctx_device(Ctx* ctx);
template <typename T>
int launch_step(Ctx* ctx, int par, int tstep, cudaStream_t s, cudaStream_t s2, bool fork, cudaEvent_t* ev);
int launch_steps_direct(Ctx* ctx, int n, cudaStream_t s);
template <typename T>
int launch_pml(Ctx* ctx, int par, int tstep, cudaStream_t s);
int ensure_graph(Ctx* ctx);
int check_guards(Ctx* ctx);
int check_device_error(Ctx* ctx);
template <typename T>
int launch_post_modal(Ctx* ctx, cudaStream_t s, int tstep, bool with_recorders);
template <typename T>
int launch_post_modal_range(Ctx* ctx, cudaStream_t s, int tstep, int r_lo, int r_hi, int s_lo, int s_hi,
                            long long s_first, long long s_total);
void build_adjoint_jobs(Ctx* ctx);
void pml_profile_unit(const Ctx* ctx, int type, int L, std::vector<double>* out);
template <typename T>
int dense_transform_ex(Ctx* ctx, const DctDev& D, long long in, long long out, long long scratch, int which,
                       bool transpose, double scale);
size_t elem_size(const Ctx* ctx);
template <typename T>
int launch_cubes(Ctx* ctx, cudaStream_t s, int tstep, int par, int r_lo, int r_hi);
void free_cubes(Ctx* ctx);

}  // namespace ard
