// Text output in the reference's formats (ARD-simulator-190113/output/README.md):
// response_<i>.txt (Recorder::RecordField's response stream, recorder.cpp:
// 15-16,55) and source_<i>.txt (SoundSource::RecordSource, sound_source.cpp:
// 14-15,50-56): one value per line; out_<i>.txt (Recorder::RecordField's
// output stream, recorder.cpp:13-14,44-53): one line of the 10x10x10
// neighbourhood per step.  Values are written as an ostream writes a float
// (6 significant digits).  Host code over the context's recorded history and
// source series; nothing here runs on the GPU besides the copies.
#include <cuda_runtime.h>

#include <cstdio>
#include <fstream>
#include <string>
#include <vector>

#include "ard_engine.h"
#include "ard_gb300.h"

using namespace ard;

extern "C" int ard_write_outputs(ard_ctx* c, int32_t scene, const char* dir, int64_t nt) {
  if (!c || !dir) return ARD_ERR_INVALID;
  Ctx* ctx = reinterpret_cast<Ctx*>(c);
  if (scene < 0 || scene >= (int)ctx->scenes.size()) { ctx->err = "bad scene index"; return ARD_ERR_RANGE; }
  if (nt < 0 || nt > ctx->t_host || nt > ctx->max_steps) { ctx->err = "ard_write_outputs: steps not recorded"; return ARD_ERR_RANGE; }
  const SceneRec& sr = ctx->scenes[scene];
  if (cudaSetDevice(ctx->device) != cudaSuccess || cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
    ctx->err = "ard_write_outputs: device synchronisation failed";
    return ARD_ERR_CUDA;
  }
  auto write = [&](const std::string& name, const std::vector<float>& v) -> bool {
    std::ofstream f(std::string(dir) + "/" + name, std::ios::out);
    if (!f) return false;
    for (float x : v) f << x << '\n';
    return (bool)f;
  };
  // recorders: history rows are n_rec_total wide (double)
  if (sr.nrec > 0 && nt > 0) {
    std::vector<double> h((size_t)nt * ctx->n_rec_total);
    if (cudaMemcpy(h.data(), ctx->d_hist, h.size() * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess) {
      ctx->err = "ard_write_outputs: history copy failed";
      return ARD_ERR_CUDA;
    }
    for (int r = 0; r < sr.nrec; ++r) {
      std::vector<float> v((size_t)nt);
      for (int64_t t = 0; t < nt; ++t) v[t] = (float)h[(size_t)t * ctx->n_rec_total + sr.rec0 + r];
      if (!write("response_" + std::to_string(r) + ".txt", v)) { ctx->err = "ard_write_outputs: cannot write in " + std::string(dir); return ARD_ERR_INVALID; }
    }
  }
  // neighbourhoods (recorded from step 0): one line of 1000 values per step,
  // each followed by a space (recorder.cpp:44-53)
  if (ctx->d_cube_hist && ctx->cube_t0 == 0 && sr.nrec > 0 && nt > 0) {
    const size_t cells = 1000;
    std::vector<float> cube((size_t)nt * cells);
    for (int r = 0; r < sr.nrec; ++r) {
      if (cudaMemcpy2D(cube.data(), sizeof(float) * cells, ctx->d_cube_hist + (size_t)(sr.rec0 + r) * cells,
                       sizeof(float) * cells * ctx->n_rec_total, sizeof(float) * cells, nt,
                       cudaMemcpyDeviceToHost) != cudaSuccess) {
        ctx->err = "ard_write_outputs: neighbourhood copy failed";
        return ARD_ERR_CUDA;
      }
      std::ofstream f(std::string(dir) + "/out_" + std::to_string(r) + ".txt", std::ios::out);
      if (!f) { ctx->err = "ard_write_outputs: cannot write in " + std::string(dir); return ARD_ERR_INVALID; }
      for (int64_t t = 0; t < nt; ++t) {
        const float* row = cube.data() + (size_t)t * cells;
        for (size_t k = 0; k < cells; ++k) f << row[k] << ' ';
        f << '\n';
      }
      if (!f) { ctx->err = "ard_write_outputs: cannot write in " + std::string(dir); return ARD_ERR_INVALID; }
    }
  }
  // sources: the series as injected, [source][max_steps] (float)
  if (sr.nsrc > 0 && nt > 0) {
    std::vector<float> s((size_t)sr.nsrc * ctx->max_steps);
    if (cudaMemcpy(s.data(), ctx->d_series + (size_t)sr.src0 * ctx->max_steps, s.size() * sizeof(float),
                   cudaMemcpyDeviceToHost) != cudaSuccess) {
      ctx->err = "ard_write_outputs: series copy failed";
      return ARD_ERR_CUDA;
    }
    for (int q = 0; q < sr.nsrc; ++q) {
      std::vector<float> v(s.begin() + (size_t)q * ctx->max_steps, s.begin() + (size_t)q * ctx->max_steps + nt);
      if (!write("source_" + std::to_string(q) + ".txt", v)) { ctx->err = "ard_write_outputs: cannot write in " + std::string(dir); return ARD_ERR_INVALID; }
    }
  }
  return ARD_OK;
}
