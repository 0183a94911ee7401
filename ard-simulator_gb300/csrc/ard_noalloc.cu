// ard_read_field_noalloc: the air-partition field readout without any
// allocation, for callers that cannot allocate device memory themselves --
// code running inside another framework's memory pool or arena, or in a
// process whose allocator is owned by someone else -- and so cannot let a
// library call cudaMalloc behind their back.
//
// The readout is the inverse 3D transform of the partition's current modes
// (REDFT01 on each axis, scaled by 1/sqrt(2N)), computed by the same GEMM
// kernel as ard_read_field.  ard_read_field works through the context's own
// scratch area; this variant works entirely inside the file-scope array
// g_field_scratch below (the unpadded modes, the three inverse tables and
// both intermediates of the three passes), writes the caller's device buffer
// only with the final copy, and returns without synchronising.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <string>

#include "ard_engine.h"
#include "ard_gb300.h"
#include "ard_kernels.cuh"

using namespace ard;

namespace {

// Largest air partition the variant accepts: 4,194,304 cells, every extent
// at most 1024.  The array holds two such fields and one 1024 x 1024 table
// per axis: 44 MiB of device memory on every GPU that loads the library,
// kept until the process exits.
constexpr long long kNoAllocMaxCells = 1LL << 22;
constexpr int kNoAllocMaxExtent = 1024;
constexpr long long kNoAllocTable = (long long)kNoAllocMaxExtent * kNoAllocMaxExtent;
constexpr int kNoAllocMaxJobs = 1 + kNoAllocMaxExtent + 1;  // x pass, one y job per z-slice, z pass

// element offsets inside the scratch array
constexpr long long kFieldA = 0;
constexpr long long kFieldB = kNoAllocMaxCells;
constexpr long long kTabX = 2 * kNoAllocMaxCells;
constexpr long long kTabY = kTabX + kNoAllocTable;
constexpr long long kTabZ = kTabY + kNoAllocTable;
constexpr long long kScratchElems = kTabZ + kNoAllocTable;

static __device__ __align__(256) float g_field_scratch[kScratchElems];
static __device__ __align__(256) XformJob g_field_jobs[kNoAllocMaxJobs];

// Device addresses of the two arrays, looked up once per device with that
// device current (host code must not use the array names as addresses:
// they are host-side stand-ins).  A cudaDeviceReset ends every context of
// this library on that device and with them the addresses kept here; the
// library is not used across a device reset.
struct DeviceSetup {
  bool done = false;
  float* scratch = nullptr;
  XformJob* jobs = nullptr;
};
constexpr int kMaxDevices = 64;
DeviceSetup g_setup[kMaxDevices];
std::mutex g_setup_lock;

int setup_device(Ctx* ctx) {
  if (ctx->device < 0 || ctx->device >= kMaxDevices) { ctx->err = "device ordinal out of range"; return ARD_ERR_INVALID; }
  std::lock_guard<std::mutex> lock(g_setup_lock);
  DeviceSetup& s = g_setup[ctx->device];
  if (s.done) return ARD_OK;
  cudaError_t e = cudaGetSymbolAddress((void**)&s.scratch, g_field_scratch);
  if (e == cudaSuccess) e = cudaGetSymbolAddress((void**)&s.jobs, g_field_jobs);
  if (e != cudaSuccess) {
    ctx->err = std::string("ard_read_field_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e);
    return ARD_ERR_CUDA;
  }
  s.done = true;
  return ARD_OK;
}

// Fills the job table on the device: the three passes of the inverse
// transform, element offsets relative to the scratch array:
// x pass A -> B, y pass (per z-slice) B -> A, z pass A -> B.
__global__ void build_jobs_kernel(XformJob* jobs, int w, int h, int d, double scale) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const long long plane = (long long)h * w;
  auto make = [&](long long in0, long long out, long long tab, int n, int batch, int ld, int rows, double sc) {
    XformJob j{};
    j.in0 = in0; j.in1 = -1; j.sgn = 1;
    j.out = out; j.ctab = tab; j.n = n; j.batch = batch; j.ld = ld;
    j.inverse = 1; j.rows = rows; j.scale = sc;
    const int Md = rows ? batch : n, Nd = rows ? n : batch;
    j.tn = (Nd + 63) / 64;
    j.ntiles = ((Md + 63) / 64) * j.tn;
    j.first = 0;
    return j;
  };
  if (i == 0) jobs[0] = make(kFieldA, kFieldB, kTabX, w, d * h, w, 1, 1.0);                 // along x
  if (i < d) {                                                                             // along y, per z-slice
    XformJob j = make(kFieldB + i * plane, kFieldA + i * plane, kTabY, h, w, w, 0, 1.0);
    j.first = i * j.ntiles;
    jobs[1 + i] = j;
  }
  if (i == 0) jobs[1 + d] = make(kFieldA, kFieldB, kTabZ, d, (int)plane, (int)plane, 0, scale);  // along z
}

}  // namespace

extern "C" int ard_read_field_noalloc(ard_ctx* c, int32_t scene, int32_t partition, float* out_device, void* stream) {
  if (!c || !out_device) return ARD_ERR_INVALID;
  Ctx* ctx = reinterpret_cast<Ctx*>(c);
  // every argument check before any work is queued
  if (ctx->prec != ARD_PREC_F32) { ctx->err = "ard_read_field_noalloc: FP32 contexts only"; return ARD_ERR_INVALID; }
  if (scene < 0 || scene >= (int)ctx->scenes.size()) { ctx->err = "bad scene index"; return ARD_ERR_RANGE; }
  const SceneRec& sr = ctx->scenes[scene];
  if (partition < 0 || partition >= (int)sr.parts.size()) { ctx->err = "bad partition index"; return ARD_ERR_RANGE; }
  if (sr.parts[partition].kind != ARD_PART_DCT) {
    ctx->err = "ard_read_field_noalloc: air partitions only";
    return ARD_ERR_INVALID;
  }
  if ((uintptr_t)out_device % sizeof(float)) { ctx->err = "ard_read_field_noalloc: output not float-aligned"; return ARD_ERR_INVALID; }
  const DctDev& D = ctx->dct[sr.engine_idx[partition]];
  const long long N = (long long)D.w * D.h * D.d;
  if (N > kNoAllocMaxCells || D.w > kNoAllocMaxExtent || D.h > kNoAllocMaxExtent || D.d > kNoAllocMaxExtent) {
    ctx->err = "ard_read_field_noalloc: partition " + std::to_string(D.w) + " x " + std::to_string(D.h) + " x " +
               std::to_string(D.d) + " exceeds the limit of " + std::to_string(kNoAllocMaxCells) +
               " cells with every extent <= " + std::to_string(kNoAllocMaxExtent);
    return ARD_ERR_RANGE;
  }
  if (cudaSetDevice(ctx->device) != cudaSuccess) { ctx->err = "cudaSetDevice failed"; return ARD_ERR_CUDA; }
  int rc = setup_device(ctx);
  if (rc) return rc;
  const DeviceSetup& S = g_setup[ctx->device];
  cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
  cudaError_t e = cudaSuccess;
  if (s != ctx->stream) {  // after everything already queued on the context
    e = cudaEventRecord(ctx->ev_fork, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, ctx->ev_fork, 0);
  }
  const float* pool = (const float*)ctx->d_buf;
  const int lvl = (int)((ctx->t_host - 1) & 1);
  // the modes without the row padding -> field A; the inverse (REDFT01) tables of the three extents
  if (e == cudaSuccess)
    e = cudaMemcpy2DAsync(S.scratch + kFieldA, D.w * sizeof(float), pool + D.M[lvl], D.wp * sizeof(float),
                          D.w * sizeof(float), (size_t)D.h * D.d, cudaMemcpyDeviceToDevice, s);
  const long long tab_src[3] = {D.cw + (long long)D.w * D.w, D.ch + (long long)D.h * D.h, D.cd + (long long)D.d * D.d};
  const long long tab_dst[3] = {kTabX, kTabY, kTabZ};
  const long long tab_n[3] = {D.w, D.h, D.d};
  for (int k = 0; k < 3 && e == cudaSuccess; ++k)
    e = cudaMemcpyAsync(S.scratch + tab_dst[k], pool + tab_src[k], sizeof(float) * tab_n[k] * tab_n[k],
                        cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess) {
    build_jobs_kernel<<<(D.d + 127) / 128, 128, 0, s>>>(S.jobs, D.w, D.h, D.d, D.si);
    e = cudaGetLastError();
  }
  const int gb = ctx->num_sms * 4;
  auto tiles = [](int n, int batch, int rows) {
    const int Md = rows ? batch : n, Nd = rows ? n : batch;
    return ((Md + 63) / 64) * ((Nd + 63) / 64);
  };
  const int tx = tiles(D.w, D.d * D.h, 1), ty = tiles(D.h, D.w, 0) * D.d, tz = tiles(D.d, D.h * D.w, 0);
  if (e == cudaSuccess) {
    xform_gemm_kernel<float><<<std::min(gb, tx), 256, 0, s>>>(S.scratch, S.jobs, 1, tx);
    xform_gemm_kernel<float><<<std::min(gb, ty), 256, 0, s>>>(S.scratch, S.jobs + 1, D.d, ty);
    xform_gemm_kernel<float><<<std::min(gb, tz), 256, 0, s>>>(S.scratch, S.jobs + 1 + D.d, 1, tz);
    e = cudaGetLastError();
  }
  // the z pass wrote the field into field B
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(out_device, S.scratch + kFieldB, N * sizeof(float), cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess && s != ctx->stream) {
    e = cudaEventRecord(ctx->ev_join, s);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(ctx->stream, ctx->ev_join, 0);
  }
  if (e != cudaSuccess) {
    ctx->err = std::string("ard_read_field_noalloc: ") + cudaGetErrorString(e);
    return ARD_ERR_CUDA;
  }
  return ARD_OK;
}
