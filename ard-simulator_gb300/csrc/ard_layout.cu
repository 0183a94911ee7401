// Context layout: turns flattened scenes (the reference's partitions,
// boundaries, sources and recorders) into device work tables and an HBM
// element pool; plus the setup and readout entry points of the C ABI.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "ard_device.cuh"
#include "ard_engine.h"
#include "ard_gb300.h"
#include "ard_kernels.cuh"
#include "ard_mma.cuh"

using namespace ard;

namespace ard {

size_t elem_size(const Ctx* ctx) { return ctx->prec == ARD_PREC_F64 ? sizeof(double) : sizeof(float); }

namespace {

struct Pool {
  long long off = 0;
  long long take(long long n) {
    const long long o = off;
    off += (n + 31) / 32 * 32;  // 128-byte (fp32) alignment of every array
    return o;
  }
};

// Face-coordinate view of a partition for an interface of a given type:
// u fast, v slow, c the crossing axis.
struct FaceView {
  int ou, ov, nu, nv, oc, ext;
};

FaceView face_view(const ard_partition& p, int type) {
  FaceView f{};
  if (type == ARD_BOUNDARY_X) { f.ou = p.y_start; f.ov = p.z_start; f.nu = p.height; f.nv = p.depth; f.oc = p.x_start; f.ext = p.width; }
  else if (type == ARD_BOUNDARY_Y) { f.ou = p.x_start; f.ov = p.z_start; f.nu = p.width; f.nv = p.depth; f.oc = p.y_start; f.ext = p.height; }
  else { f.ou = p.x_start; f.ov = p.y_start; f.nu = p.width; f.nv = p.height; f.oc = p.z_start; f.ext = p.depth; }
  return f;
}

int pml_axis(int pml_type) { return pml_type <= 1 ? ARD_BOUNDARY_X : (pml_type <= 3 ? ARD_BOUNDARY_Y : ARD_BOUNDARY_Z); }

// Reference damping profile of one PML slab (pml_partition.cpp:26-28,59-86)
// in the context's precision, multiplied by `scale`.
template <typename R>
void pml_profile(const Ctx* ctx, int type, int L, double scale, std::vector<double>* out) {
  const R dh = (R)(float)ctx->dh;
  const R c0 = (R)(float)ctx->c0;
  const R Rr = (R)(float)ctx->pml_R;
  const R thickness = ctx->pml_layers * dh;
  const R zeta = c0 / thickness * (R)std::log10((R)1 / Rr);
  const R pi = (R)M_PI;
  out->assign(L, 0.0);
  for (int l = 0; l < L; ++l) {
    // distance index counted from the air side: LEFT/TOP/FRONT use (L - l), others (l + 1)
    const int s = (type == ARD_PML_LEFT || type == ARD_PML_TOP || type == ARD_PML_FRONT) ? (L - l) : (l + 1);
    const R z = zeta * (R)scale * (s / thickness * dh - (R)std::sin((R)2 * pi * s * dh / thickness) / (R)2 / pi);
    (*out)[l] = (double)z;
  }
}

}  // namespace

// Damping profile of a slab for face scale 1 (zeta is linear in the scale).
void pml_profile_unit(const Ctx* ctx, int type, int L, std::vector<double>* out) {
  if (ctx->prec == ARD_PREC_F64) pml_profile<double>(ctx, type, L, 1.0, out);
  else pml_profile<float>(ctx, type, L, 1.0, out);
}

// Reference-arithmetic modal tables, computed on the host exactly as
// DctPartition's constructor does (dct_partition.cpp:24-36): 1-based mode
// numbers, w and cos(w dt) in the working precision with the C library's
// sqrt / cos; tabA = cos(w dt), tabB = w^2.
template <typename R>
int upload_reference_tables(Ctx* ctx, const DctDev& D) {
  const long long N = (long long)D.wp * D.h * D.d;
  std::vector<R> a((size_t)N, (R)0), b((size_t)N, (R)0);
  const R dh = (R)(float)ctx->dh, dt = (R)(float)ctx->dt, c0 = (R)(float)ctx->c0;
  const R lx2 = D.w * D.w * dh * dh, ly2 = D.h * D.h * dh * dh, lz2 = D.d * D.d * dh * dh;
  const R pi = (R)M_PI;
  for (int i = 1; i <= D.d; ++i)
    for (int j = 1; j <= D.h; ++j)
      for (int k = 1; k <= D.w; ++k) {
        const long long idx = ((long long)(i - 1) * D.h + (j - 1)) * D.wp + (k - 1);
        const R w = c0 * pi * std::sqrt(i * i / lz2 + j * j / ly2 + k * k / lx2);
        b[idx] = w * w;
        a[idx] = std::cos(w * dt);
      }
  const size_t es = sizeof(R);
  ARD_CUDA(cudaMemcpy((char*)ctx->d_buf + D.tabA * es, a.data(), N * es, cudaMemcpyHostToDevice));
  ARD_CUDA(cudaMemcpy((char*)ctx->d_buf + D.tabB * es, b.data(), N * es, cudaMemcpyHostToDevice));
  return ARD_OK;
}

int upload_pml_zeta(Ctx* ctx) {
  // zeta tables live in the pool; rebuilt whenever a scale changes
  const size_t es = elem_size(ctx);
  for (size_t i = 0; i < ctx->pml.size(); ++i) {
    const PmlDev& P = ctx->pml[i];
    const double scale = ctx->scenes[P.scene].scale[P.type];
    std::vector<double> z;
    if (ctx->prec == ARD_PREC_F64) pml_profile<double>(ctx, P.type, P.L, scale, &z);
    else pml_profile<float>(ctx, P.type, P.L, scale, &z);
    if (ctx->prec == ARD_PREC_F64) {
      ARD_CUDA(cudaMemcpy((char*)ctx->d_buf + P.zeta * es, z.data(), P.L * sizeof(double), cudaMemcpyHostToDevice));
    } else {
      std::vector<float> zf(z.begin(), z.end());
      ARD_CUDA(cudaMemcpy((char*)ctx->d_buf + P.zeta * es, zf.data(), P.L * sizeof(float), cudaMemcpyHostToDevice));
    }
  }
  return ARD_OK;
}

int zero_state(Ctx* ctx) {
  const size_t es = elem_size(ctx);
  char* base = (char*)ctx->d_buf;
  ARD_CUDA(cudaMemsetAsync(base + ctx->state_begin * es, 0, (ctx->state_end - ctx->state_begin) * es, ctx->stream));
  if (ctx->adjoint)
    ARD_CUDA(cudaMemsetAsync(base + ctx->adj_begin * es, 0, (ctx->adj_end - ctx->adj_begin) * es, ctx->stream));
  ARD_CUDA(cudaMemsetAsync(ctx->d_t, 0, sizeof(long long), ctx->stream));
  if (ctx->n_rec_total > 0)
    ARD_CUDA(cudaMemsetAsync(ctx->d_hist, 0, sizeof(double) * ctx->max_steps * ctx->n_rec_total, ctx->stream));
  ctx->t_host = 0;
  return ARD_OK;
}

// Balances the face jobs of one launch and pairs them for the two CTAs of a
// cluster.  While the launch still fits in one wave of `slots` CTAs (it then
// lasts as long as its largest job), the largest job is split: a two-output
// job into one job per output (the same staging, half the arithmetic), then
// a one-output job's rows between the two CTAs of its cluster (half the
// staging and arithmetic each, the halves of T exchanged through distributed
// shared memory).  A launch of many waves keeps whole jobs, two to a cluster,
// one per CTA.  A 16-column job costs its warps as much as a 32-column one
// (16 rows per warp instead of 8), so column splits would not shorten the
// launch and are not made.  Output: pairs (jobs[2 i], jobs[2 i + 1]) for the
// cluster of item i, largest first: a split job twice, or two whole jobs (the
// last one padded by an empty job).  Returns whether any job's rows are split
// (the launch then runs in clusters; without, one CTA per entry).
bool balance_face_jobs(std::vector<Face2DJob>* jobs, int slots) {
  // the arithmetic of one warp of a CTA of the job: rows of the warp's row
  // blocks x the slab's columns x both contractions, for one or two outputs
  auto work = [](const Face2DJob& j) {
    const int rows = j.narrow ? 16 : 8, per_block = rows * kFace2DWarps;
    const int nr = j.split ? (j.V + 1) / 2 : j.V;
    return (long long)((nr + per_block - 1) / per_block) * rows * (j.narrow ? 16 : 32) * (j.U + j.V) *
           (j.which == 0 ? 2 : 1);
  };
  for (Face2DJob& j : *jobs) {
    j.narrow = j.ub <= 16 ? 1 : 0;
    j.split = 0;
  }
  long long ctas = (long long)jobs->size();
  while (ctas < slots && !jobs->empty()) {
    size_t k = 0;
    for (size_t i = 1; i < jobs->size(); ++i)
      if (work((*jobs)[i]) > work((*jobs)[k])) k = i;
    Face2DJob& J = (*jobs)[k];
    if (J.which == 0) {            // one job per output
      Face2DJob b = J;
      J.which = 1;
      b.which = 2;
      jobs->push_back(b);
      ctas += 1;
    } else if (!J.split && J.V > 1) {   // rows split over the cluster
      J.split = 1;
      ctas += 1;
    } else {
      break;                       // the largest job cannot be split further
    }
  }
  std::stable_sort(jobs->begin(), jobs->end(),
                   [&](const Face2DJob& a, const Face2DJob& b) { return work(a) > work(b); });
  bool split = false;
  for (const Face2DJob& J : *jobs) split = split || J.split;
  std::vector<Face2DJob> out;
  out.reserve(2 * jobs->size() + 2);
  bool pending = false;
  Face2DJob wait{};
  for (const Face2DJob& J : *jobs) {
    if (J.split) {
      out.push_back(J);
      out.push_back(J);
    } else if (pending) {
      out.push_back(wait);
      out.push_back(J);
      pending = false;
    } else {
      wait = J;
      pending = true;
    }
  }
  if (pending) {
    Face2DJob idle{};              // V = 0: no rows, no stores
    idle.which = 1;
    out.push_back(wait);
    out.push_back(idle);
  }
  *jobs = std::move(out);
  return split;
}

// Face transforms of the adjoint step, the transposes of the forward ones:
//   adjoint of the inverse transform: Q[pm][n] = s_i Ci_V (q_n +/- q_{5-n}) Ci_U^T
//     (the adjoint face pressure q -> the P arrays read by the adjoint modal step)
//   adjoint of the forward transform: a_L = s_f C_V^T (sum of R partials, combined
//     as for the inverse) C_U (-> the adjoint shell force)
// as fused 2D jobs and as two-pass GEMM jobs.
void build_adjoint_jobs(Ctx* ctx) {
  auto add_job = [](JobList& list, XformJob j) {
    const int Md = j.rows ? j.batch : j.n, Nd = j.rows ? j.n : j.batch;
    j.tn = (Nd + 63) / 64;
    j.ntiles = ((Md + 63) / 64) * j.tn;
    list.add(j, j.ntiles);
  };
  for (const DctDev& D : ctx->dct) {
    struct Ax { long long q, a, P, R, tmp; int U, V, ld; long long cU, cV; int nb; };
    const Ax axes[3] = {{D.qX, D.aX, D.PX, D.RX, D.tmpX, D.h, D.d, D.h, D.ch, D.cd, D.nbx},
                        {D.qY, D.aY, D.PY, D.RY, D.tmpY, D.w, D.d, D.wp, D.cw, D.cd, D.nby},
                        {D.qZ, D.aZ, D.PZ, D.RZ, D.tmpZ, D.w, D.h, D.wp, D.cw, D.ch, D.nbz}};
    for (const Ax& a : axes) {
      const long long LS = (long long)a.V * a.ld;
      const long long UU = (long long)a.U * a.U, VV = (long long)a.V * a.V;
      for (int u0 = 0; u0 < a.U; u0 += 32) {
        const int ub = std::min(32, a.U - u0);
        for (int n = 0; n < 3; ++n) {
          Face2DJob j{};   // q layers n, 5-n -> P[0][n], P[1][n]
          j.in0 = a.q + n * LS; j.in1 = a.q + (5 - n) * LS;
          j.out0 = a.P + n * LS; j.out1 = a.P + (3 + n) * LS;
          j.tabA = a.cV + VV; j.tabB = a.cU + 3 * UU;   // Ci_V, Ci_U^T
          j.V = a.V; j.U = a.U; j.ld = a.ld; j.u0 = u0; j.ub = ub; j.scale = D.si;
          ctx->adj1_2d.push_back(j);
          Face2DJob k{};   // summed partials R[n], R[3+n] -> adjoint force layers n, 5-n
          k.in0 = a.R + n * LS; k.in1 = a.R + (3 + n) * LS;
          k.out0 = a.a + n * LS; k.out1 = a.a + (5 - n) * LS;
          k.tabA = a.cV + 2 * VV; k.tabB = a.cU;          // C_V^T, C_U
          k.V = a.V; k.U = a.U; k.ld = a.ld; k.u0 = u0; k.ub = ub; k.scale = D.sf;
          ctx->adj2_2d.push_back(k);
        }
      }
      // two-pass GEMM form (partitions whose layers do not fit in shared memory)
      for (int pm = 0; pm < 2; ++pm)
        for (int n = 0; n < 3; ++n) {
          XformJob j{};   // rows along U with Ci_U: A(o, j) = Ci_U[o][j]
          j.in0 = a.q + n * LS; j.in1 = a.q + (5 - n) * LS; j.sgn = pm ? -1 : 1;
          j.out = a.tmp + (pm * 3 + n) * LS; j.ctab = a.cU + UU; j.n = a.U; j.batch = a.V; j.ld = a.ld;
          j.inverse = 0; j.rows = 1; j.scale = 1.0;
          add_job(ctx->adjg[0], j);
          XformJob k{};   // columns along V with Ci_V
          k.in0 = a.tmp + (pm * 3 + n) * LS; k.in1 = -1; k.sgn = 1;
          k.out = a.P + (pm * 3 + n) * LS; k.ctab = a.cV + VV; k.n = a.V; k.batch = a.U; k.ld = a.ld;
          k.inverse = 0; k.rows = 0; k.scale = D.si;
          add_job(ctx->adjg[1], k);
        }
      for (int L = 0; L < 6; ++L) {
        const int n = L < 3 ? L : 5 - L;
        XformJob j{};     // columns along V with C_V^T: A(o, r) = C_V[r][o]
        j.in0 = a.R + (0 * 3 + n) * LS; j.in1 = a.R + (1 * 3 + n) * LS; j.sgn = L < 3 ? 1 : -1;
       
        j.out = a.tmp + L * LS; j.ctab = a.cV; j.n = a.V; j.batch = a.U; j.ld = a.ld;
        j.inverse = 1; j.rows = 0; j.scale = 1.0;
        add_job(ctx->adjg[2], j);
        XformJob k{};     // rows along U with C_U: A(o, j) = C_U[j][o]
        k.in0 = a.tmp + L * LS; k.in1 = -1; k.sgn = 1;
        k.out = a.a + L * LS; k.ctab = a.cU; k.n = a.U; k.batch = a.V; k.ld = a.ld;
        k.inverse = 1; k.rows = 1; k.scale = D.sf;
        add_job(ctx->adjg[3], k);
      }
    }
  }
}

// Job lists of the tensor-core face transforms (ard_mma.cuh) and the pool
// space of their split, pre-tiled tables.  Per air partition and axis (layer [V][ld],
// transforms along U then V), with the transposed intermediate [6][U][Vp]
// in the axis's tmp area (Vp = roundup(V, 4)):
//   forward 1  X = f_n +/- f_{5-n}  [V][ld]   -> T^T [ku][v]   table C_U
//   forward 2  T^T [ku][v]                    -> P  [kv][ku]   table C_V, scale s_f
//   inverse 1  R = R_n +/- R_{3+n}  [kv][ld]  -> Y^T [u][kv]   table Ci_U^T
//   inverse 2  Y^T [u][kv]                    -> p  [v][u]     table Ci_V^T, scale s_i
// Outputs are stacked along the product's rows: forward o = pm 3 + n (the
// even / odd parts of layer pair n), inverse o = layer L.
template <typename Take>
void build_mma_jobs(Ctx* ctx, Take take) {
  std::map<int, long long> tab;
  auto table = [&](int n) {
    auto it = tab.find(n);
    if (it != tab.end()) return it->second;
    const long long o = take(8LL * mma_table_elems(n));
    tab[n] = o;
    return o;
  };
  for (int k = 0; k < 8; ++k) { ctx->mjobs[k].clear(); ctx->mtiles[k] = 0; }
  auto add = [&](int list, MmaJob j) {
    mma_ntile(j.N, &j.nt, &j.bn);
    j.nch = (j.K + kMmaBK - 1) / kMmaBK;
    j.mt = (j.nout * j.R + 127) / 128;
    j.first = ctx->mtiles[list];
    bool vec = j.ldb % 4 == 0;
    for (int o = 0; o < j.nout; ++o) vec = vec && j.in0[o] % 4 == 0 && (j.in1[o] < 0 || j.in1[o] % 4 == 0);
    j.vec = vec ? 1 : 0;
    ctx->mtiles[list] += j.mt * j.nt;
    ctx->mjobs[list].push_back(j);
  };
  for (const DctDev& D : ctx->dct) {
    struct Axis { long long f, p, P, R, tmp, q, adj; int nU, nV, ld; };
    const Axis axes[3] = {{D.fX, D.pX, D.PX, D.RX, D.tmpX, D.qX, D.aX, D.h, D.d, D.h},
                          {D.fY, D.pY, D.PY, D.RY, D.tmpY, D.qY, D.aY, D.w, D.d, D.wp},
                          {D.fZ, D.pZ, D.PZ, D.RZ, D.tmpZ, D.qZ, D.aZ, D.w, D.h, D.wp}};
    for (const Axis& a : axes) {
      const long long LS = (long long)a.nV * a.ld;
      const int Vp = (a.nV + 3) & ~3;
      const long long TS = (long long)a.nU * Vp;   // one transposed intermediate
      const long long tU = table(a.nU), tV = table(a.nV);
      // Chi, Clo, CiThi, CiTlo, CThi, CTlo, Cihi, Cilo: mma_table_elems each
      const long long SU = mma_table_elems(a.nU), SV = mma_table_elems(a.nV);
      MmaJob f1{}, f2{}, i1{}, i2{};
      f1.nout = f2.nout = i1.nout = i2.nout = 6;
      for (int o = 0; o < 6; ++o) {
        const int pm = o / 3, n = o % 3;
        f1.in0[o] = a.f + n * LS; f1.in1[o] = a.f + (5 - n) * LS; f1.sgn[o] = pm ? -1 : 1;
        f1.out[o] = a.tmp + o * TS;
        f2.in0[o] = a.tmp + o * TS; f2.in1[o] = -1; f2.sgn[o] = 1;
        f2.out[o] = a.P + o * LS;
        const int L = o, nl = L < 3 ? L : 5 - L;
        i1.in0[o] = a.R + nl * LS; i1.in1[o] = a.R + (3 + nl) * LS; i1.sgn[o] = L < 3 ? 1 : -1;
        i1.out[o] = a.tmp + L * TS;
        i2.in0[o] = a.tmp + L * TS; i2.in1[o] = -1; i2.sgn[o] = 1;
        i2.out[o] = a.p + L * LS;
      }
      f1.R = a.nV; f1.ldb = a.ld; f1.K = f1.N = a.nU; f1.thi = tU; f1.tlo = tU + SU;
      f1.ldo = Vp; f1.scale = 1.f;
      f2.R = a.nU; f2.ldb = Vp; f2.K = f2.N = a.nV; f2.thi = tV; f2.tlo = tV + SV;
      f2.ldo = a.ld; f2.scale = (float)D.sf;
      i1.R = a.nV; i1.ldb = a.ld; i1.K = i1.N = a.nU; i1.thi = tU + 2 * SU; i1.tlo = tU + 3 * SU;
      i1.ldo = Vp; i1.scale = 1.f;
      i2.R = a.nU; i2.ldb = Vp; i2.K = i2.N = a.nV; i2.thi = tV + 2 * SV; i2.tlo = tV + 3 * SV;
      i2.ldo = a.ld; i2.scale = (float)D.si;
      add(0, f1); add(1, f2); add(2, i1); add(3, i2);
      if (ctx->adjoint) {
        // the adjoint step's transposes: the adjoint face pressure q through
        // the transposed inverse (passes 1, 2: the forward passes' form with
        // Ci in place of C, scale s_i), the summed contraction partials R
        // through the transposed forward (passes 3, 4: the inverse passes'
        // form with C^T in place of Ci^T, scale s_f) into the adjoint force
        MmaJob a1 = f1, a2 = f2, a3 = i1, a4 = i2;
        for (int o = 0; o < 6; ++o) {
          const int n = o % 3;
          a1.in0[o] = a.q + n * LS; a1.in1[o] = a.q + (5 - n) * LS;
          a4.out[o] = a.adj + o * LS;
        }
        a1.thi = tU + 6 * SU; a1.tlo = tU + 7 * SU;
        a2.thi = tV + 6 * SV; a2.tlo = tV + 7 * SV; a2.scale = (float)D.si;
        a3.thi = tU + 4 * SU; a3.tlo = tU + 5 * SU;
        a4.thi = tV + 4 * SV; a4.tlo = tV + 5 * SV; a4.scale = (float)D.sf;
        add(4, a1); add(5, a2); add(6, a3); add(7, a4);
      }
    }
  }
  ctx->mma_tables.assign(tab.begin(), tab.end());
}

int build_layout(Ctx* ctx, const ard_scene* scenes, int n_scenes) {
  const ard_scene& s0 = scenes[0];
  ctx->dh = s0.dh; ctx->dt = s0.dt; ctx->c0 = s0.c0;
  ctx->pml_layers = s0.pml_layers; ctx->pml_R = s0.pml_R; ctx->damping = s0.modal_damping;
  for (int s = 1; s < n_scenes; ++s) {
    const ard_scene& q = scenes[s];
    if (q.dh != s0.dh || q.dt != s0.dt || q.c0 != s0.c0 || q.pml_layers != s0.pml_layers || q.pml_R != s0.pml_R ||
        q.modal_damping != s0.modal_damping) {
      ctx->err = "batched scenes must share dh, dt, c0, pml_layers, pml_R and modal_damping";
      return ARD_ERR_INVALID;
    }
  }
  Pool pool;
  std::map<int, long long> cos_off;
  auto cos_table = [&](int n) {
    auto it = cos_off.find(n);
    if (it != cos_off.end()) return it->second;
    const long long o = pool.take(4LL * n * n);
    cos_off[n] = o;
    ctx->maxn = std::max(ctx->maxn, n);
    return o;
  };

  // ---- partitions ----
  std::vector<std::vector<std::vector<int>>> src_by_part;  // [scene][part] -> source indices
  for (int s = 0; s < n_scenes; ++s) {
    const ard_scene& sc = scenes[s];
    SceneRec rec;
    rec.parts.assign(sc.partitions, sc.partitions + sc.n_partitions);
    rec.engine_idx.assign(sc.n_partitions, -1);
    rec.src0 = ctx->n_src_total; rec.nsrc = sc.n_sources;
    rec.rec0 = ctx->n_rec_total; rec.nrec = sc.n_recorders;
    ctx->n_src_total += sc.n_sources;
    ctx->n_rec_total += sc.n_recorders;
    for (int i = 0; i < sc.n_partitions; ++i) {
      const ard_partition& p = sc.partitions[i];
      if (p.kind == ARD_PART_DCT) {
        DctDev D{};
        D.w = p.width; D.h = p.height; D.d = p.depth;
        D.wp = (D.w + 3) / 4 * 4;
        const long long N = (long long)D.w * D.h * D.d;
        const long long Np = (long long)D.wp * D.h * D.d;
        ctx->n_air_cells += N;
        (void)Np;
        D.damping = sc.modal_damping;
        D.sf = 1.0 / (2.0 * std::sqrt(2.0 * (double)N));
        D.si = 1.0 / std::sqrt(2.0 * (double)N);
        rec.engine_idx[i] = (int)ctx->dct.size();
        ctx->dct.push_back(D);
      } else {
        PmlDev P{};
        P.type = p.pml_type;
        P.scene = s;
        const int ax = pml_axis(p.pml_type);
        if (ax == ARD_BOUNDARY_X) { P.L = p.width; P.A = p.depth; P.B = p.height; }
        else if (ax == ARD_BOUNDARY_Y) { P.L = p.height; P.A = p.depth; P.B = p.width; }
        else { P.L = p.depth; P.A = p.height; P.B = p.width; }
        P.Bp = (P.B + 3) & ~3;
        P.n = (long long)P.L * P.A * P.Bp;
        P.strip0 = -1;
        rec.engine_idx[i] = (int)ctx->pml.size();
        ctx->pml.push_back(P);
      }
    }
    ctx->scenes.push_back(rec);
  }

  // ---- sources / recorders attached to air partitions ----
  std::vector<std::vector<PointDev>> srcs_of(ctx->dct.size()), recs_of(ctx->dct.size());
  for (int s = 0; s < n_scenes; ++s) {
    const ard_scene& sc = scenes[s];
    const SceneRec& rec = ctx->scenes[s];
    for (int i = 0; i < sc.n_sources; ++i) {
      const ard_point& q = sc.sources[i];
      if (q.partition < 0) continue;  // not inside any air partition: never injected
      if (q.partition >= sc.n_partitions || sc.partitions[q.partition].kind != ARD_PART_DCT) {
        ctx->err = "source " + std::to_string(i) + " refers to a partition that is not an air partition";
        return ARD_ERR_INVALID;
      }
      const ard_partition& p = sc.partitions[q.partition];
      PointDev d{rec.engine_idx[q.partition], q.x - p.x_start, q.y - p.y_start, q.z - p.z_start, rec.src0 + i};
      if (d.x < 0 || d.y < 0 || d.z < 0 || d.x >= p.width || d.y >= p.height || d.z >= p.depth) {
        ctx->err = "source " + std::to_string(i) + " lies outside its partition";
        return ARD_ERR_INVALID;
      }
      auto& list = srcs_of[d.part];
      // two sources on one cell: the later overwrites (partition.cpp:187-197)
      list.erase(std::remove_if(list.begin(), list.end(),
                                [&](const PointDev& o) { return o.x == d.x && o.y == d.y && o.z == d.z; }),
                 list.end());
      list.push_back(d);
    }
    for (int i = 0; i < sc.n_recorders; ++i) {
      const ard_point& q = sc.recorders[i];
      if (q.partition < 0 || q.partition >= sc.n_partitions || sc.partitions[q.partition].kind != ARD_PART_DCT) {
        ctx->err = "recorder " + std::to_string(i) + " is not attached to an air partition";
        return ARD_ERR_INVALID;
      }
      const ard_partition& p = sc.partitions[q.partition];
      PointDev d{rec.engine_idx[q.partition], q.x - p.x_start, q.y - p.y_start, q.z - p.z_start, rec.rec0 + i};
      if (d.x < 0 || d.y < 0 || d.z < 0 || d.x >= p.width || d.y >= p.height || d.z >= p.depth) {
        ctx->err = "recorder " + std::to_string(i) + " lies outside its partition";
        return ARD_ERR_INVALID;
      }
      recs_of[d.part].push_back(d);
    }
  }
  for (size_t k = 0; k < ctx->dct.size(); ++k) {
    if (srcs_of[k].size() > (size_t)kMaxPointsPerPart || recs_of[k].size() > (size_t)kMaxPointsPerPart) {
      ctx->err = "more than " + std::to_string(kMaxPointsPerPart) + " sources or recorders in one air partition";
      return ARD_ERR_INVALID;
    }
    DctDev& D = ctx->dct[k];
    D.src0 = (int)ctx->srcpts.size(); D.nsrc = (int)srcs_of[k].size();
    ctx->srcpts.insert(ctx->srcpts.end(), srcs_of[k].begin(), srcs_of[k].end());
    D.rec0 = (int)ctx->recpts.size(); D.nrec = (int)recs_of[k].size();
    ctx->recpts.insert(ctx->recpts.end(), recs_of[k].begin(), recs_of[k].end());
  }

  // ---- modal tiling ----
  // A tile is 8 warps; a thread owns 4 consecutive kx.  G lanes cover one ky
  // row (G = 8, 16 or 32, the smallest with 4 G >= min(wp, 128)), so a tile
  // spans kxt = 4 G kx and rpc = 256 / G ky rows.  The kz extent TZ (even, or
  // the whole depth) is chosen so that the tiles fill the GPU at least twice.
  long long col_tiles = 0;
  for (DctDev& D : ctx->dct) {
    const int need = std::min(D.wp, 128) / 4;
    D.G = need <= 8 ? 8 : (need <= 16 ? 16 : 32);
    for (int k = 0; k < ctx->tune_g_shift && D.G > 8; ++k) D.G /= 2;
    D.kxt = 4 * D.G;
    D.rpc = kModalThreads / D.G;
    D.nbx = (D.wp + D.kxt - 1) / D.kxt;
    D.nby = (D.h + D.rpc - 1) / D.rpc;
    col_tiles += (long long)D.nbx * D.nby;
  }
  // resident slots: 2 tiles per SM.  kz splits: as many as still fit one
  // wave, then more while that evens out the last wave (the blocks take the
  // tiles round-robin, so a last wave that is half full costs a whole tile
  // time: c4's 749 full-depth columns are 2.46 waves of 304 slots, split in
  // two they are 4.93)
  const long long slots = (long long)ctx->num_sms * 2 * std::max(1, ctx->tune_tiles);
  long long nbz_all = col_tiles > 0 ? std::max(1LL, slots / col_tiles) : 1;
  if (col_tiles > 0) {
    auto wave_eff = [&](long long nb) {
      const long long T = col_tiles * nb, waves = (T + slots - 1) / slots;
      return (double)T / (double)(waves * slots);
    };
    const long long base = nbz_all;
    double best = wave_eff(base);
    for (long long nb = base + 1; nb <= 4 * base + 4; ++nb)
      if (wave_eff(nb) > best + 0.03) { best = wave_eff(nb); nbz_all = nb; }
  }
  for (size_t k = 0; k < ctx->dct.size(); ++k) {
    DctDev& D = ctx->dct[k];
    long long nbz = std::max(1LL, std::min<long long>(nbz_all, D.d / 2));
    int TZ = (int)((D.d + nbz - 1) / nbz);
    if (TZ < D.d) TZ += TZ & 1;  // even, so every kz tile starts on an even plane
    D.TZ = TZ;
    D.nbz = (D.d + D.TZ - 1) / D.TZ;
    D.tile0 = (int)ctx->tiles.size();
    for (int bx = 0; bx < D.nbx; ++bx)
      for (int by = 0; by < D.nby; ++by)
        for (int bz = 0; bz < D.nbz; ++bz) ctx->tiles.push_back(make_int4((int)k, bx, by, bz));
  }

  // ---- state block: everything a checkpoint holds, contiguous ----
  // (modal levels, shell forces, PML fields and strips; the adjoint's carried
  // state follows in a block of its own)
  auto faces = [](const DctDev& D) { return 6LL * D.d * D.h + 6LL * D.d * D.wp + 6LL * D.h * D.wp; };
  auto set_faces = [](DctDev& D, long long base, long long* fx, long long* fy, long long* fz) {
    *fx = base; *fy = base + 6LL * D.d * D.h; *fz = *fy + 6LL * D.d * D.wp;
  };
  ctx->state_begin = pool.off;
  for (DctDev& D : ctx->dct) D.M[0] = pool.take((long long)D.wp * D.h * D.d);
  for (DctDev& D : ctx->dct) D.M[1] = pool.take((long long)D.wp * D.h * D.d);
  for (DctDev& D : ctx->dct) set_faces(D, pool.take(faces(D)), &D.fX, &D.fY, &D.fZ);
  for (int q = 0; q < 8; ++q) {
    ctx->pml_region[q][0] = pool.off;
    for (PmlDev& P : ctx->pml) {
      long long* slot[8] = {&P.p[0], &P.p[1], &P.phn[0], &P.phn[1], &P.pha[0], &P.pha[1], &P.phb[0], &P.phb[1]};
      *slot[q] = pool.take(P.n);
    }
    ctx->pml_region[q][1] = pool.off;
  }
  ctx->force_begin = pool.off;
  for (PmlDev& P : ctx->pml) {
    P.force = pool.take(3LL * P.A * P.Bp);
    P.foff = P.force - ctx->force_begin;
  }
  ctx->state_end = pool.off;
  // a slab sits at the same offset inside each of the eight regions
  for (PmlDev& P : ctx->pml) {
    P.hoff = P.p[0] - ctx->pml_region[0][0];
    const long long* slot[8] = {&P.p[0], &P.p[1], &P.phn[0], &P.phn[1], &P.pha[0], &P.pha[1], &P.phb[0], &P.phb[1]};
    for (int q = 0; q < 8; ++q)
      if (*slot[q] - ctx->pml_region[q][0] != P.hoff) { ctx->err = "internal: PML regions out of step"; return ARD_ERR_STATE; }
  }
  if (ctx->adjoint) {
    ctx->adj_begin = pool.off;
    for (DctDev& D : ctx->dct) D.AM[0] = pool.take((long long)D.wp * D.h * D.d);
    for (DctDev& D : ctx->dct) D.AM[1] = pool.take((long long)D.wp * D.h * D.d);
    for (DctDev& D : ctx->dct) set_faces(D, pool.take(faces(D)), &D.aX, &D.aY, &D.aZ);   // adjoint of the shell force
    ctx->q_begin = pool.off;
    for (DctDev& D : ctx->dct) set_faces(D, pool.take(faces(D)), &D.qX, &D.qY, &D.qZ);   // adjoint of the face pressure
    ctx->q_end = pool.off;
    for (PmlDev& P : ctx->pml) {
      for (int k = 0; k < 3; ++k) P.ap[k] = pool.take(P.n);
      for (int k = 0; k < 2; ++k) { P.aphn[k] = pool.take(P.n); P.apha[k] = pool.take(P.n); P.aphb[k] = pool.take(P.n); }
      P.aforce = pool.take(3LL * P.A * P.Bp);
    }
    ctx->adj_end = pool.off;
  }

  // ---- constants and per-step scratch ----
  for (DctDev& D : ctx->dct) {
    const long long Np = (long long)D.wp * D.h * D.d;
    D.tabA = pool.take(Np); D.tabB = pool.take(Np);
    D.cw = cos_table(D.w); D.ch = cos_table(D.h); D.cd = cos_table(D.d);
    const long long FX = 6LL * D.d * D.h, FY = 6LL * D.d * D.wp, FZ = 6LL * D.h * D.wp;
    set_faces(D, pool.take(faces(D)), &D.pX, &D.pY, &D.pZ);
    D.PX = pool.take(FX); D.PY = pool.take(FY); D.PZ = pool.take(FZ);
    D.RX = pool.take(FX * D.nbx); D.RY = pool.take(FY * D.nby); D.RZ = pool.take(FZ * D.nbz);
    // transform scratch: room for the [6][V][ld] GEMM intermediate and for the
    // transposed [6][U][roundup(V, 4)] intermediate of the tensor-core passes
    const int dp = (D.d + 3) & ~3, hp = (D.h + 3) & ~3;
    D.tmpX = pool.take(std::max(FX, 6LL * D.h * dp));
    D.tmpY = pool.take(std::max(FY, 6LL * D.w * dp));
    D.tmpZ = pool.take(std::max(FZ, 6LL * D.w * hp));
    D.recpart = pool.take(std::max(1, D.nrec) * (long long)D.nbx * D.nby * D.nbz);
    D.srcpart = pool.take(std::max(1, D.nsrc) * (long long)D.nbx * D.nby * D.nbz);
  }

  // ---- dense-transform scratch (initial pressure, field readout): 3 x the largest air partition ----
  {
    long long maxN = 0;
    for (const DctDev& D : ctx->dct) maxN = std::max(maxN, (long long)D.w * D.h * D.d);
    ctx->scratch = pool.take(3 * maxN);
  }

  // ---- PML arrays and 8 x 32 plane tiles ----
  for (size_t k = 0; k < ctx->pml.size(); ++k) {
    PmlDev& P = ctx->pml[k];
    if (P.L > kMaxPmlLayers) {
      ctx->err = "PML thicker than " + std::to_string(kMaxPmlLayers) + " layers";
      return ARD_ERR_INVALID;
    }
    P.zeta = pool.take(P.L);
    ctx->n_pml_cells += (long long)P.L * P.A * P.B;
    for (int a0 = 0; a0 < P.A; a0 += 8)
      for (int b0 = 0; b0 < P.B; b0 += 32) ctx->pml_blocks.push_back(make_int4((int)k, a0, b0, 0));
  }

  // ---- interfaces + owner masks ----
  std::vector<std::vector<int>> owner(ctx->dct.size());
  auto shell_local = [&](int k, int x, int y, int z) {
    DctDev D = ctx->dct[k];
    D.fX = 0; D.fY = 6LL * D.d * D.h; D.fZ = D.fY + 6LL * D.d * D.wp;
    return shell_index(D, x, y, z);
  };
  for (size_t k = 0; k < ctx->dct.size(); ++k) {
    const DctDev& D = ctx->dct[k];
    owner[k].assign(6LL * ((long long)D.d * D.h + (long long)D.d * D.wp + (long long)D.h * D.wp), -1);
  }
  struct PendingIface { IfaceDev dev; int scene; };
  std::vector<PendingIface> pend;
  std::vector<int> pml_iface_count(ctx->pml.size(), 0);
  for (int s = 0; s < n_scenes; ++s) {
    const ard_scene& sc = scenes[s];
    const SceneRec& rec = ctx->scenes[s];
    for (int bi = 0; bi < sc.n_boundaries; ++bi) {
      const ard_boundary& b = sc.boundaries[bi];
      if (b.a < 0 || b.b < 0 || b.a >= sc.n_partitions || b.b >= sc.n_partitions || b.type < 0 || b.type > 2) {
        ctx->err = "boundary " + std::to_string(bi) + ": bad partition index or type";
        return ARD_ERR_INVALID;
      }
      const ard_partition& A = sc.partitions[b.a];
      bool a_lo;
      int u0, u1, v0, v1;
      if (b.type == ARD_BOUNDARY_X) {
        const int ae = A.x_start + A.width;
        a_lo = (b.x_start <= ae && b.x_end >= ae);
        u0 = b.y_start; u1 = b.y_end; v0 = b.z_start; v1 = b.z_end;
      } else if (b.type == ARD_BOUNDARY_Y) {
        const int ae = A.y_start + A.height;
        a_lo = (b.y_start <= ae && b.y_end >= ae);
        u0 = b.x_start; u1 = b.x_end; v0 = b.z_start; v1 = b.z_end;
      } else {
        const int ae = A.z_start + A.depth;
        a_lo = (b.z_start <= ae && b.z_end >= ae);
        u0 = b.x_start; u1 = b.x_end; v0 = b.y_start; v1 = b.y_end;
      }
      if (u1 <= u0 || v1 <= v0) continue;  // empty face: writes nothing
      const int ilo = a_lo ? b.a : b.b, ihi = a_lo ? b.b : b.a;
      IfaceDev I{};
      I.type = b.type; I.u0 = u0; I.u1 = u1; I.v0 = v0; I.v1 = v1;
      I.absorption = b.absorption;
      const int sides[2] = {ilo, ihi};
      for (int side = 0; side < 2; ++side) {
        const ard_partition& p = sc.partitions[sides[side]];
        const FaceView f = face_view(p, b.type);
        SideDev& S = side ? I.hi : I.lo;
        S.kind = p.kind == ARD_PART_DCT ? 0 : 1;
        S.idx = rec.engine_idx[sides[side]];
        S.ou = f.ou; S.ov = f.ov; S.ext = f.ext;
        S.self = p.kind == ARD_PART_DCT ? 1 : 0;
        if (u0 < f.ou || u1 > f.ou + f.nu || v0 < f.ov || v1 > f.ov + f.nv || f.ext < 3) {
          ctx->err = "boundary " + std::to_string(bi) + " reaches outside partition " + std::to_string(sides[side]) +
                     " (only 2.5D scenes with equal z ranges are supported, as in the reference)";
          return ARD_ERR_INVALID;
        }
        if (S.kind == 1) {
          PmlDev& P = ctx->pml[S.idx];
          if (pml_axis(P.type) != b.type) {
            ctx->err = "boundary " + std::to_string(bi) + " crosses a PML along its plane";
            return ARD_ERR_INVALID;
          }
          const int strip0 = side == 0 ? f.ext - 3 : 0;
          if (P.strip0 >= 0 && P.strip0 != strip0) {
            ctx->err = "PML partition forced from both sides";
            return ARD_ERR_INVALID;
          }
          P.strip0 = strip0;
          pml_iface_count[S.idx]++;
        }
      }
      pend.push_back({I, s});
    }
  }
  // owners in list order: the last interface that writes a shell cell keeps it
  for (size_t i = 0; i < pend.size(); ++i) {
    const IfaceDev& I = pend[i].dev;
    for (int side = 0; side < 2; ++side) {
      const SideDev& S = side ? I.hi : I.lo;
      if (S.kind != 0) continue;
      for (int v = I.v0; v < I.v1; ++v)
        for (int u = I.u0; u < I.u1; ++u)
          for (int m = -3; m < 3; ++m) {
            if ((m < 0) != (side == 0)) continue;
            const int c = side == 0 ? S.ext + m : m;
            const int lu = u - S.ou, lv = v - S.ov;
            const int x = I.type == 0 ? c : lu;
            const int y = I.type == 0 ? lu : (I.type == 1 ? c : lv);
            const int z = I.type == 2 ? c : lv;
            const long long o = shell_local(S.idx, x, y, z);
            if (o >= 0) owner[S.idx][o] = (int)i;
          }
    }
  }
  // sources overwrite their cell after every interface (next step's phase A)
  for (const PointDev& q : ctx->srcpts) {
    const long long o = shell_local(q.part, q.x, q.y, q.z);
    if (o >= 0) owner[q.part][o] = -2;
  }
  for (size_t i = 0; i < pend.size(); ++i) {
    IfaceDev I = pend[i].dev;
    if ((long long)(I.u1 - I.u0) * (I.v1 - I.v0) >= (1LL << 31)) {   // the interface kernel indexes cells in 32 bits
      ctx->err = "interface with 2^31 or more face cells";
      return ARD_ERR_RANGE;
    }
    I.mask = (long long)ctx->masks.size();
    I.cell0 = ctx->n_face_cells;
    for (int v = I.v0; v < I.v1; ++v)
      for (int u = I.u0; u < I.u1; ++u) {
        unsigned char bits = 0;
        for (int m = -3; m < 3; ++m) {
          const SideDev& S = m < 0 ? I.lo : I.hi;
          const int c = m < 0 ? S.ext + m : m;
          bool on = true;
          if (S.kind == 0) {
            const int lu = u - S.ou, lv = v - S.ov;
            const int x = I.type == 0 ? c : lu;
            const int y = I.type == 0 ? lu : (I.type == 1 ? c : lv);
            const int z = I.type == 2 ? c : lv;
            const long long o = shell_local(S.idx, x, y, z);
            on = o >= 0 && owner[S.idx][o] == (int)i;
          }
          if (on) bits |= (unsigned char)(1u << (m + 3));
        }
        ctx->masks.push_back(bits);
      }
    ctx->n_face_cells += (long long)(I.u1 - I.u0) * (I.v1 - I.v0);
    for (int side = 0; side < 2; ++side) {
      SideDev& S = side ? I.hi : I.lo;
      for (int n = 0; n < 3; ++n) {
        const int c = side == 0 ? S.ext - 3 + n : n;
        if (S.kind == 0) {
          const DctDev& D = ctx->dct[S.idx];
          const int L = face_layer(c, S.ext);
          long long b;
          if (I.type == 0) { b = D.pX + (long long)L * D.d * D.h; S.psv = D.h; }
          else if (I.type == 1) { b = D.pY + (long long)L * D.d * D.wp; S.psv = D.wp; }
          else { b = D.pZ + (long long)L * D.h * D.wp; S.psv = D.wp; }
          S.pb[n][0] = S.pb[n][1] = b;
        } else {
          const PmlDev& P = ctx->pml[S.idx];
          S.pb[n][0] = P.p[0] + (long long)c * P.A * P.Bp;
          S.pb[n][1] = P.p[1] + (long long)c * P.A * P.Bp;
          S.psv = P.Bp;
        }
      }
      if (S.kind == 0) {
        const DctDev& D = ctx->dct[S.idx];
        S.fx = D.fX; S.fy = D.fY; S.fz = D.fZ;
        S.w = D.w; S.h = D.h; S.d = D.d; S.wp = D.wp;
      } else {
        const PmlDev& P = ctx->pml[S.idx];
        S.fls = (long long)P.A * P.Bp;
        S.fb = P.force - (long long)P.strip0 * S.fls;
        S.fsv = P.Bp;
      }
    }
    for (long long k = 0; k < (long long)(I.u1 - I.u0) * (I.v1 - I.v0); ++k) ctx->cell_iface.push_back((int)ctx->ifs.size());
    ctx->ifs.push_back(I);
  }
  for (size_t k = 0; k < ctx->pml.size(); ++k) {
    if (pml_iface_count[k] != 1) {
      ctx->err = "every PML partition needs exactly one interface (found " + std::to_string(pml_iface_count[k]) + ")";
      return ARD_ERR_INVALID;
    }
  }

  // ---- sums of the modal tiles' contraction partials (slab 0 receives the sum) ----
  for (const DctDev& D : ctx->dct) {
    ctx->psum_lo.push_back((int)ctx->psum.size());
    const long long LX = 6LL * D.d * D.h, LY = 6LL * D.d * D.wp, LZ = 6LL * D.h * D.wp;
    const long long base[3] = {D.RX, D.RY, D.RZ}, cnt[3] = {LX, LY, LZ};
    const int nb[3] = {D.nbx, D.nby, D.nbz};
    for (int k = 0; k < 3; ++k) {
      if (nb[k] < 2) continue;
      SumJob j{base[k], cnt[k], cnt[k], ctx->psum_total, nb[k]};
      ctx->psum.push_back(j);
      ctx->psum_total += (cnt[k] + kSumChunk - 1) / kSumChunk * kSumChunk;   // chunk-aligned index space
    }
  }

  // ---- transform jobs (GEMMs over the face layers) ----
  auto add_job = [](JobList& list, XformJob j) {
    const int Md = j.rows ? j.batch : j.n, Nd = j.rows ? j.n : j.batch;
    j.tn = (Nd + 63) / 64;
    j.ntiles = ((Md + 63) / 64) * j.tn;
    list.add(j, j.ntiles);
  };
  for (const DctDev& D : ctx->dct) {
    // layer [V][ld], transforms along U (fast) and V (slow)
    struct Axis { long long f, p, P, R, tmp; int nU, nV, ld; long long cU, cV; int nb; };
    const Axis axes[3] = {
        {D.fX, D.pX, D.PX, D.RX, D.tmpX, D.h, D.d, D.h, D.ch, D.cd, D.nbx},
        {D.fY, D.pY, D.PY, D.RY, D.tmpY, D.w, D.d, D.wp, D.cw, D.cd, D.nby},
        {D.fZ, D.pZ, D.PZ, D.RZ, D.tmpZ, D.w, D.h, D.wp, D.cw, D.ch, D.nbz},
    };
    for (const Axis& a : axes) {
      const long long LS = (long long)a.nV * a.ld;  // layer stride
      for (int pm = 0; pm < 2; ++pm)
        for (int n = 0; n < 3; ++n) {
          XformJob j{};
          j.in0 = a.f + n * LS; j.in1 = a.f + (5 - n) * LS; j.sgn = pm ? -1 : 1;
          j.out = a.tmp + (pm * 3 + n) * LS; j.ctab = a.cU; j.n = a.nU; j.batch = a.nV; j.ld = a.ld;
          j.inverse = 0; j.rows = 1; j.scale = 1.0;
          add_job(ctx->fwd1, j);
          XformJob k{};
          k.in0 = a.tmp + (pm * 3 + n) * LS; k.in1 = -1; k.sgn = 1;
          k.out = a.P + (pm * 3 + n) * LS; k.ctab = a.cV; k.n = a.nV; k.batch = a.nU; k.ld = a.ld;
          k.inverse = 0; k.rows = 0; k.scale = D.sf;
          add_job(ctx->fwd2, k);
        }
      for (int L = 0; L < 6; ++L) {
        const int n = L < 3 ? L : 5 - L;
        XformJob j{};
        j.in0 = a.R + (0 * 3 + n) * LS; j.in1 = a.R + (1 * 3 + n) * LS; j.sgn = L < 3 ? 1 : -1;
       
        j.out = a.tmp + L * LS; j.ctab = a.cV + (long long)a.nV * a.nV; j.n = a.nV; j.batch = a.nU; j.ld = a.ld;
        j.inverse = 1; j.rows = 0; j.scale = 1.0;
        add_job(ctx->inv1, j);
        XformJob k{};
        k.in0 = a.tmp + L * LS; k.in1 = -1; k.sgn = 1;
        k.out = a.p + L * LS; k.ctab = a.cU + (long long)a.nU * a.nU; k.n = a.nU; k.batch = a.nV; k.ld = a.ld;
        k.inverse = 1; k.rows = 1; k.scale = D.si;
        add_job(ctx->inv2, k);
      }
    }
  }

  // ---- fused face transforms (one kernel per direction) when a layer fits in shared memory ----
  {
    const size_t es0 = elem_size(ctx);
    long long xs = 0, x1 = 0, bs = 0, ts = 0;
    for (size_t pi = 0; pi < ctx->dct.size(); ++pi) {
      const DctDev& D = ctx->dct[pi];
      struct Ax { long long f, p, P, R; int U, V, ld; long long cU, cV; };
      const Ax axes[3] = {{D.fX, D.pX, D.PX, D.RX, D.h, D.d, D.h, D.ch, D.cd},
                          {D.fY, D.pY, D.PY, D.RY, D.w, D.d, D.wp, D.cw, D.cd},
                          {D.fZ, D.pZ, D.PZ, D.RZ, D.w, D.h, D.wp, D.cw, D.ch}};
      for (const Ax& a : axes) {
        const long long LS = (long long)a.V * a.ld;
        const long long UU = (long long)a.U * a.U, VV = (long long)a.V * a.V;
        const long long xp = face2d_pitch(a.U), ap = face2d_pitch(a.V);
        xs = std::max(xs, (long long)a.V * std::max(xp, ap));   // whole jobs (the eligibility of the fused form)
        x1 = xs;
        bs = std::max(bs, 32LL * ((a.U + 3) & ~3));
        ts = std::max(ts, 32LL * ((a.V + 3) & ~3));
        for (int u0 = 0; u0 < a.U; u0 += 32) {
          const int ub = std::min(32, a.U - u0);
          for (int n = 0; n < 3; ++n) {
            // forward: layers n, 5-n -> even / odd parts P[0][n], P[1][n]
            Face2DJob j{};
            j.in0 = a.f + n * LS; j.in1 = a.f + (5 - n) * LS;
            j.out0 = a.P + n * LS; j.out1 = a.P + (3 + n) * LS;
            j.tabA = a.cV; j.tabB = a.cU + 2 * UU;
            j.V = a.V; j.U = a.U; j.ld = a.ld; j.u0 = u0; j.ub = ub; j.scale = D.sf; j.part = (int)pi;
            ctx->fwd2d.push_back(j);
            // inverse: even / odd parts (partials summed beforehand) -> layers n, 5-n
            Face2DJob k{};
            k.in0 = a.R + n * LS; k.in1 = a.R + (3 + n) * LS;
            k.out0 = a.p + n * LS; k.out1 = a.p + (5 - n) * LS;
            k.tabA = a.cV + 3 * VV; k.tabB = a.cU + UU;
            k.V = a.V; k.U = a.U; k.ld = a.ld; k.u0 = u0; k.ub = ub; k.scale = D.si; k.part = (int)pi;
            ctx->inv2d.push_back(k);
          }
        }
      }
    }
    ctx->f2d_smem = Face2DSmem{(int)xs, (int)x1, (int)bs, (int)ts};
    ctx->f2d_bytes = (size_t)(xs + x1 + bs + 2 * ts) * es0;
    ctx->fused_faces = !ctx->dct.empty() && !ctx->tune_gemm &&
                       ctx->f2d_bytes <= (size_t)std::min(ctx->smem_optin, 200 * 1024);
  }
  if (ctx->adjoint) build_adjoint_jobs(ctx);
  // every GEMM job list runs as one face_gemm_kernel instance: its jobs must
  // agree on the pass direction, the table orientation and the input pair
  {
    const JobList* lists[] = {&ctx->fwd1, &ctx->fwd2, &ctx->inv1, &ctx->inv2,
                              &ctx->adjg[0], &ctx->adjg[1], &ctx->adjg[2], &ctx->adjg[3]};
    for (const JobList* L : lists)
      for (const XformJob& j : L->jobs)
        if (j.rows != L->jobs[0].rows || j.inverse != L->jobs[0].inverse ||
            (j.in1 >= 0) != (L->jobs[0].in1 >= 0)) {
          ctx->err = "internal: mixed GEMM job list";
          return ARD_ERR_STATE;
        }
  }
  // ---- tensor-core face transforms (FP32, two-pass form; ARD_FACE_MMA=0 keeps the CUDA-core passes) ----
  {
    const char* env = std::getenv("ARD_FACE_MMA");
    ctx->mma_faces = ctx->prec == ARD_PREC_F32 && !ctx->fused_faces && !ctx->dct.empty() && !(env && env[0] == '0');
    if (ctx->mma_faces) build_mma_jobs(ctx, [&](long long n) { return pool.take(n); });
  }
  // ---- air partition groups: two streams in the step graph when the fused
  // face transforms are used and a split leaves each side >= 20 % of the cells ----
  ctx->ngroups = 1;
  {
    const int np = (int)ctx->dct.size();
    std::vector<long long> cells(np + 1, 0);
    for (int i = 0; i < np; ++i) cells[i + 1] = cells[i] + (long long)ctx->dct[i].w * ctx->dct[i].h * ctx->dct[i].d;
    int best = -1;
    long long best_gap = cells[np];
    for (int k = 1; k < np; ++k) {
      const long long gap = std::llabs(cells[np] - 2 * cells[k]);
      if (gap < best_gap) { best_gap = gap; best = k; }
    }
    if (ctx->fused_faces && best > 0 && std::min(cells[best], cells[np] - cells[best]) * 5 >= cells[np]) {
      ctx->ngroups = 2;
      ctx->groups[0].part_lo = 0; ctx->groups[0].part_hi = best;
      ctx->groups[1].part_lo = best; ctx->groups[1].part_hi = np;
    } else {
      ctx->groups[0].part_lo = 0; ctx->groups[0].part_hi = np;
    }
    for (int g = 0; g < ctx->ngroups; ++g) {
      Ctx::AirGroup& G = ctx->groups[g];
      const int lo = G.part_lo, hi = G.part_hi;
      G.t_lo = np ? ctx->dct[lo].tile0 : 0;
      G.t_hi = hi < np ? ctx->dct[hi].tile0 : (int)ctx->tiles.size();
      G.r_lo = np ? ctx->dct[lo].rec0 : 0;
      G.r_hi = hi < np ? ctx->dct[hi].rec0 : (int)ctx->recpts.size();
      G.s_lo = np ? ctx->psum_lo[lo] : 0;
      G.s_hi = hi < np ? ctx->psum_lo[hi] : (int)ctx->psum.size();
      G.s_first = G.s_lo < (int)ctx->psum.size() ? ctx->psum[G.s_lo].first : ctx->psum_total;
      G.s_total = (G.s_hi < (int)ctx->psum.size() ? ctx->psum[G.s_hi].first : ctx->psum_total) - G.s_first;
    }
  }
  if (ctx->fused_faces) {
    // CTAs of one wave: two per SM (the kernel's bound; the shared memory of
    // row-split jobs, sized below, is about half that of whole ones)
    const int slots = ctx->num_sms * 2;
    // each group gets a share of one wave in proportion to its arithmetic
    auto grouped = [&](std::vector<Face2DJob>* list, auto set_range) {
      if (ctx->ngroups == 1) {
        const bool sp = balance_face_jobs(list, slots);
        set_range(0, 0, (int)list->size() / 2, sp);
        return;
      }
      std::vector<Face2DJob> parts[2];
      double w[2] = {0, 0};
      for (const Face2DJob& j : *list) {
        const int g = j.part >= ctx->groups[1].part_lo ? 1 : 0;
        parts[g].push_back(j);
        w[g] += (double)j.V * (j.U + j.V) * j.ub;
      }
      list->clear();
      for (int g = 0; g < 2; ++g) {
        const int sg = std::max(1, (int)std::lround(slots * w[g] / std::max(1.0, w[0] + w[1])));
        const bool sp = balance_face_jobs(&parts[g], sg);
        const int lo = (int)list->size() / 2;
        list->insert(list->end(), parts[g].begin(), parts[g].end());
        set_range(g, lo, (int)list->size() / 2, sp);
      }
    };
    grouped(&ctx->fwd2d, [&](int g, int lo, int hi, bool sp) {
      ctx->groups[g].f_lo = lo; ctx->groups[g].f_hi = hi; ctx->groups[g].f_split = sp;
    });
    grouped(&ctx->inv2d, [&](int g, int lo, int hi, bool sp) {
      ctx->groups[g].i_lo = lo; ctx->groups[g].i_hi = hi; ctx->groups[g].i_split = sp;
    });
    ctx->adj1_split = balance_face_jobs(&ctx->adj1_2d, slots);
    ctx->adj2_split = balance_face_jobs(&ctx->adj2_2d, slots);
    // shared memory of the balanced jobs: a CTA stages its rows of the layers
    // (all V, or half of a split job) and all of T
    const size_t es0 = elem_size(ctx);
    long long xs = 0, bs = 0, ts = 0;
    for (const std::vector<Face2DJob>* L : {&ctx->fwd2d, &ctx->inv2d, &ctx->adj1_2d, &ctx->adj2_2d})
      for (const Face2DJob& j : *L) {
        if (j.V == 0) continue;
        const long long rows = j.split ? (j.V + 1) / 2 : j.V;
        xs = std::max(xs, rows * std::max(face2d_pitch(j.U), face2d_pitch(j.V)));
        bs = std::max(bs, 32LL * ((j.U + 3) & ~3));
        ts = std::max(ts, 32LL * ((j.V + 3) & ~3));
      }
    ctx->f2d_smem = Face2DSmem{(int)xs, (int)xs, (int)bs, (int)ts};
    ctx->f2d_bytes = (size_t)(2 * xs + bs + 2 * ts) * es0;
  }

  // ---- device allocation ----
  const size_t es = elem_size(ctx);
  ctx->pool_elems = pool.off;
  ARD_CUDA(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
  ARD_CUDA(cudaStreamCreateWithFlags(&ctx->stream2, cudaStreamNonBlocking));
  ARD_CUDA(cudaStreamCreateWithFlags(&ctx->stream3, cudaStreamNonBlocking));
  ARD_CUDA(cudaEventCreateWithFlags(&ctx->ev_join3, cudaEventDisableTiming));
  ARD_CUDA(cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming));
  ARD_CUDA(cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming));
  // checked mode: 16 MiB sentinel guards on both sides of the pool catch stray writes
  ctx->guard_bytes = ctx->debug_sync ? ((size_t)16 << 20) : 0;
  ARD_CUDA(cudaMalloc(&ctx->d_buf_base, std::max<size_t>(1, pool.off * es) + 2 * ctx->guard_bytes));
  ctx->d_buf = (char*)ctx->d_buf_base + ctx->guard_bytes;
  if (ctx->guard_bytes) {
    ARD_CUDA(cudaMemset(ctx->d_buf_base, 0xA5, ctx->guard_bytes));
    ARD_CUDA(cudaMemset((char*)ctx->d_buf + pool.off * es, 0xA5, ctx->guard_bytes));
  }
  ARD_CUDA(cudaMemset(ctx->d_buf, 0, pool.off * es));
  ARD_CUDA(cudaDeviceSynchronize());
  auto up = [&](auto** dptr, const auto& vec) -> int {
    using E = typename std::decay<decltype(vec)>::type::value_type;
    const size_t bytes = std::max<size_t>(1, vec.size() * sizeof(E));
    ARD_CUDA(cudaMalloc((void**)dptr, bytes));
    if (!vec.empty()) ARD_CUDA(cudaMemcpy((void*)*dptr, vec.data(), vec.size() * sizeof(E), cudaMemcpyHostToDevice));
    return ARD_OK;
  };
  int rc;
  if ((rc = up(&ctx->d_mask, ctx->masks))) return rc;
  if ((rc = up(&ctx->d_dct, ctx->dct))) return rc;
  if ((rc = up(&ctx->d_pml, ctx->pml))) return rc;
  if ((rc = up(&ctx->d_pml_blocks, ctx->pml_blocks))) return rc;
  if ((rc = up(&ctx->d_ifs, ctx->ifs))) return rc;
  if ((rc = up(&ctx->d_cell_iface, ctx->cell_iface))) return rc;
  if ((rc = up(&ctx->d_srcpts, ctx->srcpts))) return rc;
  if ((rc = up(&ctx->d_recpts, ctx->recpts))) return rc;
  if ((rc = up(&ctx->d_tiles, ctx->tiles))) return rc;
  if ((rc = up(&ctx->d_fwd1, ctx->fwd1.jobs))) return rc;
  if ((rc = up(&ctx->d_fwd2, ctx->fwd2.jobs))) return rc;
  if ((rc = up(&ctx->d_inv1, ctx->inv1.jobs))) return rc;
  if ((rc = up(&ctx->d_inv2, ctx->inv2.jobs))) return rc;
  if ((rc = up(&ctx->d_fwd2d, ctx->fwd2d))) return rc;
  if ((rc = up(&ctx->d_inv2d, ctx->inv2d))) return rc;
  if ((rc = up(&ctx->d_psum, ctx->psum))) return rc;
  for (int k = 0; k < 8; ++k)
    if (ctx->mma_faces && !ctx->mjobs[k].empty() && (rc = up(&ctx->d_mjobs[k], ctx->mjobs[k]))) return rc;
  ARD_CUDA(cudaMalloc(&ctx->d_err, sizeof(int)));
  ARD_CUDA(cudaMemset(ctx->d_err, 0, sizeof(int)));
  if (int rc = build_pml_maps(ctx)) return rc;
  if (ctx->adjoint) {
    if ((rc = up(&ctx->d_adj1_2d, ctx->adj1_2d))) return rc;
    if ((rc = up(&ctx->d_adj2_2d, ctx->adj2_2d))) return rc;
    for (int k = 0; k < 4; ++k)
      if ((rc = up(&ctx->d_adjg[k], ctx->adjg[k].jobs))) return rc;
    ARD_CUDA(cudaMalloc(&ctx->d_tb, 2 * sizeof(long long)));
    ARD_CUDA(cudaMemset(ctx->d_tb, 0, 2 * sizeof(long long)));
    ARD_CUDA(cudaMalloc(&ctx->d_phist, sizeof(PmlHist<double>)));
    ARD_CUDA(cudaMemset(ctx->d_phist, 0, sizeof(PmlHist<double>)));
  }
  ARD_CUDA(cudaMalloc(&ctx->d_series, sizeof(float) * std::max(1LL, (long long)ctx->n_src_total * ctx->max_steps)));
  ARD_CUDA(cudaMemset(ctx->d_series, 0, sizeof(float) * (long long)ctx->n_src_total * ctx->max_steps));
  ARD_CUDA(cudaMalloc(&ctx->d_hist, sizeof(double) * std::max(1LL, (long long)ctx->n_rec_total * ctx->max_steps)));
  ARD_CUDA(cudaMalloc(&ctx->d_t, sizeof(long long)));

  // ---- tables (FP64 arithmetic on the device) ----
  for (auto& kv : cos_off) {
    ctx->cos_tables.push_back(kv);
    const long long nn = (long long)kv.first * kv.first;
    const int blocks = (int)std::min<long long>((nn + 255) / 256, 4096);
    if (ctx->prec == ARD_PREC_F64) cos_table_kernel<double><<<blocks, 256, 0, ctx->stream>>>((double*)ctx->d_buf, kv.second, kv.first);
    else cos_table_kernel<float><<<blocks, 256, 0, ctx->stream>>>((float*)ctx->d_buf, kv.second, kv.first);
    ARD_CUDA(cudaGetLastError());
  }
  for (auto& kv : ctx->mma_tables) {   // split TF32 tables of the tensor-core face passes (FP32 contexts)
    const int n = kv.first;
    const int blocks = (int)std::min<long long>((mma_table_elems(n) + 255) / 256, 4096);
    mma_table_kernel<<<blocks, 256, 0, ctx->stream>>>((float*)ctx->d_buf, kv.second, n);
    ARD_CUDA(cudaGetLastError());
  }
  for (const DctDev& D : ctx->dct) {
    const long long N = (long long)D.wp * D.h * D.d;
    if (ctx->arith == ARD_ARITH_REFERENCE) {
      ARD_CUDA(cudaStreamSynchronize(ctx->stream));
      int rc2 = ctx->prec == ARD_PREC_F64 ? upload_reference_tables<double>(ctx, D) : upload_reference_tables<float>(ctx, D);
      if (rc2) return rc2;
      continue;
    }
    const int blocks = (int)std::min<long long>((N + 255) / 256, 8192);
    if (ctx->prec == ARD_PREC_F64)
      modal_table_kernel<double><<<blocks, 256, 0, ctx->stream>>>((double*)ctx->d_buf, D.tabA, D.tabB, D.w, D.wp, D.h, D.d,
                                                                   (double)(float)ctx->dh, (double)(float)ctx->dt,
                                                                   (double)(float)ctx->c0);
    else
      modal_table_kernel<float><<<blocks, 256, 0, ctx->stream>>>((float*)ctx->d_buf, D.tabA, D.tabB, D.w, D.wp, D.h, D.d,
                                                                  (double)(float)ctx->dh, (double)(float)ctx->dt,
                                                                  (double)(float)ctx->c0);
    ARD_CUDA(cudaGetLastError());
  }
  // the synchronous uploads below run on the legacy stream: finish the table kernels first
  ARD_CUDA(cudaStreamSynchronize(ctx->stream));
  if ((rc = upload_pml_zeta(ctx))) return rc;
  if ((rc = zero_state(ctx))) return rc;
  ARD_CUDA(cudaStreamSynchronize(ctx->stream));
  return ARD_OK;
}

void free_ctx_device(Ctx* ctx) {
  if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
  free_cubes(ctx);
  void* ptrs[] = {ctx->d_buf_base, ctx->d_mask, ctx->d_dct, ctx->d_pml, ctx->d_pml_blocks, ctx->d_ifs, ctx->d_srcpts,
                  ctx->d_recpts, ctx->d_tiles, ctx->d_fwd1, ctx->d_fwd2, ctx->d_inv1, ctx->d_inv2, ctx->d_fwd2d,
                  ctx->d_inv2d, ctx->d_series,
                  ctx->d_hist, ctx->d_t, ctx->d_adj1_2d, ctx->d_adj2_2d, ctx->d_adjg[0], ctx->d_adjg[1],
                  ctx->d_adjg[2], ctx->d_adjg[3], ctx->d_tb, ctx->d_phist, ctx->d_psum,
                  ctx->d_cell_iface, ctx->d_mjobs[0], ctx->d_mjobs[1], ctx->d_mjobs[2], ctx->d_mjobs[3],
                  ctx->d_mjobs[4], ctx->d_mjobs[5], ctx->d_mjobs[6], ctx->d_mjobs[7],
                  ctx->d_err, ctx->d_pml_maps, ctx->d_pml_amaps};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
  if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
  if (ctx->ev_join3) cudaEventDestroy(ctx->ev_join3);
  if (ctx->stream3) cudaStreamDestroy(ctx->stream3);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  if (ctx->stream2) cudaStreamDestroy(ctx->stream2);
  ctx->graph_exec = nullptr;
  ctx->d_buf = nullptr;
  ctx->d_buf_base = nullptr;
}

// cuTensorMapEncodeTiled, reached through the runtime's driver entry point
// (the library links only the CUDA runtime).
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

// One PML slab field as a [L][A][B] tensor (row pitch Bp) at `base`, or with
// `slots` > 0 as [slots][L][A][B] with `slot_stride` elements between slots,
// read in boxes of box_b x box_a (x 1 x 1).  Elements outside the tensor read
// as zero, the reference's sentinel.
static int encode_slab_map(Ctx* ctx, CUtensorMap* map, const PmlDev& P, const void* base, cuuint32_t box_b,
                           cuuint32_t box_a, long long slots = 0, long long slot_stride = 0) {
  PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
  if (!enc) { ctx->err = "cuTensorMapEncodeTiled is not available from the driver"; return ARD_ERR_CUDA; }
  const size_t es = elem_size(ctx);
  const CUtensorMapDataType type =
      ctx->prec == ARD_PREC_F64 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
  const cuuint32_t rank = slots > 0 ? 4 : 3;
  const cuuint64_t dims[4] = {(cuuint64_t)P.B, (cuuint64_t)P.A, (cuuint64_t)P.L, (cuuint64_t)std::max(1LL, slots)};
  const cuuint64_t strides[3] = {(cuuint64_t)P.Bp * es, (cuuint64_t)P.A * P.Bp * es, (cuuint64_t)slot_stride * es};
  const cuuint32_t box[4] = {box_b, box_a, 1, 1};
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  const CUresult r = enc(map, type, rank, const_cast<void*>(base), dims, strides, box, estr,
                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    ctx->err = "cuTensorMapEncodeTiled failed for a PML slab (error " + std::to_string((int)r) + ")";
    return ARD_ERR_CUDA;
  }
  return ARD_OK;
}

// The tensor maps of the PML kernels' tile loads, with the box of the tile
// each one feeds (PmlStage, PmlAdjStage): per slab p (halo 3, x from b0 - 4),
// phi_a (halo 2 along a) and phi_b (halo 2 along b, x from b0 - 4) of both
// time levels; with the adjoint also its three levels of p and two of each
// phi.
int build_pml_maps(Ctx* ctx) {
  if (ctx->pml.empty()) return ARD_OK;
  const size_t es = elem_size(ctx);
  const cuuint32_t PW = kPmlTB + 8;
  char* base = (char*)ctx->d_buf;
  std::vector<CUtensorMap> maps(6 * ctx->pml.size()), amaps(ctx->adjoint ? 7 * ctx->pml.size() : 0);
  for (size_t k = 0; k < ctx->pml.size(); ++k) {
    const PmlDev& P = ctx->pml[k];
    const long long offs[6] = {P.p[0], P.p[1], P.pha[0], P.pha[1], P.phb[0], P.phb[1]};
    const cuuint32_t bb[3] = {PW, (cuuint32_t)kPmlTB, PW}, ba[3] = {kPmlTA + 6, kPmlTA + 4, kPmlTA};
    for (int q = 0; q < 6; ++q)
      if (int rc = encode_slab_map(ctx, &maps[6 * k + q], P, base + offs[q] * es, bb[q / 2], ba[q / 2])) return rc;
    if (ctx->adjoint) {
      const long long aoffs[7] = {P.ap[0], P.ap[1], P.ap[2], P.apha[0], P.apha[1], P.aphb[0], P.aphb[1]};
      const int kind[7] = {0, 0, 0, 1, 1, 2, 2};
      for (int q = 0; q < 7; ++q)
        if (int rc = encode_slab_map(ctx, &amaps[7 * k + q], P, base + aoffs[q] * es, bb[kind[q]], ba[kind[q]]))
          return rc;
    }
  }
  ARD_CUDA(cudaMalloc(&ctx->d_pml_maps, sizeof(CUtensorMap) * maps.size()));
  ARD_CUDA(cudaMemcpy(ctx->d_pml_maps, maps.data(), sizeof(CUtensorMap) * maps.size(), cudaMemcpyHostToDevice));
  if (ctx->adjoint) {
    ARD_CUDA(cudaMalloc(&ctx->d_pml_amaps, sizeof(CUtensorMap) * amaps.size()));
    ARD_CUDA(cudaMemcpy(ctx->d_pml_amaps, amaps.data(), sizeof(CUtensorMap) * amaps.size(), cudaMemcpyHostToDevice));
  }
  return ARD_OK;
}

// Tensor maps of a PML history buffer (`slots` copies of the all-slab p
// region, `hlen` elements apart) for the adjoint PML kernel's p(t) tiles:
// per slab a [slots][L][A][B] tensor read in boxes of the p(t) tile.
int build_pml_hist_maps(Ctx* ctx, const void* hist, long long hlen, long long slots, CUtensorMap** out) {
  *out = nullptr;
  if (ctx->pml.empty()) return ARD_OK;
  const size_t es = elem_size(ctx);
  std::vector<CUtensorMap> maps(ctx->pml.size());
  for (size_t k = 0; k < ctx->pml.size(); ++k) {
    const PmlDev& P = ctx->pml[k];
    if (int rc = encode_slab_map(ctx, &maps[k], P, (const char*)hist + P.hoff * es, kPmlTB + 8, kPmlTA + 4, slots, hlen))
      return rc;
  }
  ARD_CUDA(cudaMalloc(out, sizeof(CUtensorMap) * maps.size()));
  ARD_CUDA(cudaMemcpy(*out, maps.data(), sizeof(CUtensorMap) * maps.size(), cudaMemcpyHostToDevice));
  return ARD_OK;
}

// Dense 3D transform of one air partition, unpadded [d][h][w], from pool
// offset `in` to `out` through `scratch` (in == out allowed), with the GEMM
// kernel: forward applies REDFT10 (matrix C) on each axis, inverse REDFT01
// (matrix Ci^T); `scale` multiplies the result.
template <typename T>
int dense_transform(Ctx* ctx, const DctDev& D, long long in, long long out, long long scratch, bool inverse,
                    double scale) {
  return dense_transform_ex<T>(ctx, D, in, out, scratch, inverse ? 1 : 0, inverse, scale);
}

// General form: `table` 0 applies C, 1 applies Ci, each transposed when
// `transpose` (C^T on every axis is the transpose of the forward transform).
template <typename T>
int dense_transform_ex(Ctx* ctx, const DctDev& D, long long in, long long out, long long scratch, int which,
                       bool transpose, double scale) {
  T* buf = reinterpret_cast<T*>(ctx->d_buf);
  const long long plane = (long long)D.h * D.w;
  const bool inverse = transpose;
  auto table = [&](int n) {
    for (auto& kv : ctx->cos_tables)
      if (kv.first == n) return kv.second + (which ? (long long)n * n : 0);
    return -1LL;
  };
  auto make = [&](long long i0, long long o0, int n, int batch, int ld, int rows, double sc) {
    XformJob j{};
    j.in0 = i0; j.in1 = -1; j.sgn = 1;
    j.out = o0; j.ctab = table(n); j.n = n; j.batch = batch; j.ld = ld;
    j.inverse = inverse ? 1 : 0; j.rows = rows; j.scale = sc;
    const int Md = rows ? batch : n, Nd = rows ? n : batch;
    j.tn = (Nd + 63) / 64;
    j.ntiles = ((Md + 63) / 64) * j.tn;
    return j;
  };
  JobList px, py, pz;
  const long long b = scratch;
  {
    XformJob j = make(in, b, D.w, D.d * D.h, D.w, 1, 1.0);
    px.add(j, j.ntiles);
  }
  for (int z = 0; z < D.d; ++z) {
    XformJob j = make(b + z * plane, out + z * plane, D.h, D.w, D.w, 0, 1.0);
    py.add(j, j.ntiles);
  }
  {
    XformJob j = make(out, b, D.d, (int)plane, (int)plane, 0, scale);
    pz.add(j, j.ntiles);
  }
  XformJob *dx = nullptr, *dy = nullptr, *dz = nullptr;
  ARD_CUDA(cudaMalloc(&dx, sizeof(XformJob)));
  ARD_CUDA(cudaMalloc(&dy, sizeof(XformJob) * py.jobs.size()));
  ARD_CUDA(cudaMalloc(&dz, sizeof(XformJob)));
  ARD_CUDA(cudaMemcpy(dx, px.jobs.data(), sizeof(XformJob), cudaMemcpyHostToDevice));
  ARD_CUDA(cudaMemcpy(dy, py.jobs.data(), sizeof(XformJob) * py.jobs.size(), cudaMemcpyHostToDevice));
  ARD_CUDA(cudaMemcpy(dz, pz.jobs.data(), sizeof(XformJob), cudaMemcpyHostToDevice));
  const int gb = ctx->num_sms * 4;
  xform_gemm_kernel<T><<<std::min(gb, px.units), 256, 0, ctx->stream>>>(buf, dx, 1, px.units);
  xform_gemm_kernel<T><<<std::min(gb, py.units), 256, 0, ctx->stream>>>(buf, dy, (int)py.jobs.size(), py.units);
  xform_gemm_kernel<T><<<std::min(gb, pz.units), 256, 0, ctx->stream>>>(buf, dz, 1, pz.units);
  ARD_CUDA(cudaGetLastError());
  ARD_CUDA(cudaMemcpyAsync(buf + out, buf + b, sizeof(T) * (size_t)D.w * D.h * D.d, cudaMemcpyDeviceToDevice, ctx->stream));
  ARD_CUDA(cudaStreamSynchronize(ctx->stream));
  cudaFree(dx); cudaFree(dy); cudaFree(dz);
  return ARD_OK;
}

template int dense_transform<float>(Ctx*, const DctDev&, long long, long long, long long, bool, double);
template int dense_transform<double>(Ctx*, const DctDev&, long long, long long, long long, bool, double);
template int dense_transform_ex<float>(Ctx*, const DctDev&, long long, long long, long long, int, bool, double);
template int dense_transform_ex<double>(Ctx*, const DctDev&, long long, long long, long long, int, bool, double);

}  // namespace ard

// ---------------------------------------------------------------------------
// setup / readout entry points
// ---------------------------------------------------------------------------

static Ctx* as_ctx(ard_ctx* c) { return reinterpret_cast<Ctx*>(c); }

extern "C" int ard_set_source_series(ard_ctx* c, int32_t scene, int32_t source, const float* series, int64_t n) {
  if (!c) return ARD_ERR_INVALID;
  Ctx* ctx = as_ctx(c);
  if (n < 0 || n > ctx->max_steps || (n > 0 && !series)) { ctx->err = "series longer than max_steps"; return ARD_ERR_RANGE; }
  ARD_CUDA(cudaSetDevice(ctx->device));
  ARD_CUDA(cudaStreamSynchronize(ctx->stream));
  if (scene == -1 && source == -1) {
    // every source of every scene: series is [n_sources_total][n]
    if (ctx->n_src_total == 0) return ARD_OK;
    ARD_CUDA(cudaMemset(ctx->d_series, 0, sizeof(float) * ctx->max_steps * ctx->n_src_total));
    if (n > 0)
      ARD_CUDA(cudaMemcpy2D(ctx->d_series, sizeof(float) * ctx->max_steps, series, sizeof(float) * n,
                            sizeof(float) * n, ctx->n_src_total, cudaMemcpyHostToDevice));
    return ARD_OK;
  }
  if (scene < 0 || scene >= (int)ctx->scenes.size()) { ctx->err = "bad scene index"; return ARD_ERR_RANGE; }
  const SceneRec& s = ctx->scenes[scene];
  if (source < 0 || source >= s.nsrc) { ctx->err = "bad source index"; return ARD_ERR_RANGE; }
  float* dst = ctx->d_series + (long long)(s.src0 + source) * ctx->max_steps;
  ARD_CUDA(cudaMemset(dst, 0, sizeof(float) * ctx->max_steps));
  if (n > 0) ARD_CUDA(cudaMemcpy(dst, series, sizeof(float) * n, cudaMemcpyHostToDevice));
  return ARD_OK;
}

extern "C" int ard_set_source_samples(ard_ctx* c, int32_t scene, int32_t source, int64_t t0, int64_t n,
                                      const float* samples) {
  if (!c) return ARD_ERR_INVALID;
  Ctx* ctx = as_ctx(c);
  if (t0 < 0 || n < 0 || t0 + n > ctx->max_steps || (n > 0 && !samples)) {
    ctx->err = "source samples outside [0, max_steps)";
    return ARD_ERR_RANGE;
  }
  long long first = 0, count = 0;
  if (scene == -1 && source == -1) {
    count = ctx->n_src_total;   // samples is [n_sources_total][n]
  } else {
    if (scene < 0 || scene >= (int)ctx->scenes.size()) { ctx->err = "bad scene index"; return ARD_ERR_RANGE; }
    const SceneRec& s = ctx->scenes[scene];
    if (source < 0 || source >= s.nsrc) { ctx->err = "bad source index"; return ARD_ERR_RANGE; }
    first = s.src0 + source;
    count = 1;
  }
  if (n == 0 || count == 0) return ARD_OK;
  ARD_CUDA(cudaSetDevice(ctx->device));
  ARD_CUDA(cudaStreamSynchronize(ctx->stream));
  ARD_CUDA(cudaMemcpy2D(ctx->d_series + first * ctx->max_steps + t0, sizeof(float) * ctx->max_steps, samples,
                        sizeof(float) * n, sizeof(float) * n, (size_t)count, cudaMemcpyHostToDevice));
  return ARD_OK;
}

extern "C" int ard_set_pml_scale(ard_ctx* c, int32_t scene, const float scale[6]) {
  if (!c || !scale) return ARD_ERR_INVALID;
  Ctx* ctx = as_ctx(c);
  if (scene < 0 || scene >= (int)ctx->scenes.size()) { ctx->err = "bad scene index"; return ARD_ERR_RANGE; }
  for (int f = 0; f < 6; ++f) ctx->scenes[scene].scale[f] = scale[f];
  ARD_CUDA(cudaSetDevice(ctx->device));
  ARD_CUDA(cudaStreamSynchronize(ctx->stream));
  return ard::upload_pml_zeta(ctx);
}

extern "C" int ard_reset(ard_ctx* c) {
  if (!c) return ARD_ERR_INVALID;
  Ctx* ctx = as_ctx(c);
  ARD_CUDA(cudaSetDevice(ctx->device));
  int rc = ard::zero_state(ctx);
  if (rc) return rc;
  ctx->cube_t0 = 0;   // neighbourhood rows are recorded again from step 0
  ARD_CUDA(cudaStreamSynchronize(ctx->stream));
  return ARD_OK;
}

static int part_lookup(Ctx* ctx, int scene, int part, int* kind, int* idx) {
  if (scene < 0 || scene >= (int)ctx->scenes.size()) { ctx->err = "bad scene index"; return ARD_ERR_RANGE; }
  const SceneRec& s = ctx->scenes[scene];
  if (part < 0 || part >= (int)s.parts.size()) { ctx->err = "bad partition index"; return ARD_ERR_RANGE; }
  *kind = s.parts[part].kind;
  *idx = s.engine_idx[part];
  return ARD_OK;
}

extern "C" int ard_set_initial_pressure(ard_ctx* c, int32_t scene, int32_t partition, const float* pressure) {
  if (!c || !pressure) return ARD_ERR_INVALID;
  Ctx* ctx = as_ctx(c);
  int kind, idx;
  int rc = part_lookup(ctx, scene, partition, &kind, &idx);
  if (rc) return rc;
  if (kind != ARD_PART_DCT) { ctx->err = "initial pressure applies to air partitions"; return ARD_ERR_INVALID; }
  if (ctx->t_host != 0) { ctx->err = "initial pressure only before the first step (call ard_reset)"; return ARD_ERR_STATE; }
  ARD_CUDA(cudaSetDevice(ctx->device));
  ARD_CUDA(cudaStreamSynchronize(ctx->stream));
  const DctDev& D = ctx->dct[idx];
  const long long N = (long long)D.w * D.h * D.d;
  const size_t es = elem_size(ctx);
  // p0 -> scratch (unpadded), transform there, then copy into both padded levels
  const long long s0 = ctx->scratch;
  char* base = (char*)ctx->d_buf;
  if (ctx->prec == ARD_PREC_F64) {
    std::vector<double> h(pressure, pressure + N);
    ARD_CUDA(cudaMemcpy(base + (s0 + N) * es, h.data(), N * es, cudaMemcpyHostToDevice));
  } else {
    ARD_CUDA(cudaMemcpy(base + (s0 + N) * es, pressure, N * es, cudaMemcpyHostToDevice));
  }
  // modes = DCT-II(p0) / (8 N s_i) with s_i = 1 / sqrt(2N)
  const double scale = 1.0 / (8.0 * (double)N / std::sqrt(2.0 * (double)N));
  rc = ctx->prec == ARD_PREC_F64 ? ard::dense_transform<double>(ctx, D, s0 + N, s0 + N, s0, false, scale)
                                 : ard::dense_transform<float>(ctx, D, s0 + N, s0 + N, s0, false, scale);
  if (rc) return rc;
  for (int lvl = 0; lvl < 2; ++lvl)
    ARD_CUDA(cudaMemcpy2D(base + D.M[lvl] * es, D.wp * es, base + (s0 + N) * es, D.w * es, D.w * es,
                          (size_t)D.h * D.d, cudaMemcpyDeviceToDevice));
  return ARD_OK;
}

extern "C" int ard_read_recorders_f64(ard_ctx* c, int32_t scene, double* out, int64_t t0, int64_t nt) {
  if (!c || (nt > 0 && !out)) return ARD_ERR_INVALID;
  Ctx* ctx = as_ctx(c);
  if (scene < -1 || scene >= (int)ctx->scenes.size()) { ctx->err = "bad scene index"; return ARD_ERR_RANGE; }
  if (t0 < 0 || nt < 0 || t0 + nt > ctx->t_host || t0 + nt > ctx->max_steps) { ctx->err = "recorder time range not recorded"; return ARD_ERR_RANGE; }
  const int rec0 = scene < 0 ? 0 : ctx->scenes[scene].rec0;
  const int nrec = scene < 0 ? ctx->n_rec_total : ctx->scenes[scene].nrec;
  if (nrec == 0 || nt == 0) return ARD_OK;
  ARD_CUDA(cudaSetDevice(ctx->device));
  ARD_CUDA(cudaStreamSynchronize(ctx->stream));
  if (int rc = ard::check_device_error(ctx)) return rc;
  // rows of the history are n_rec_total wide; copy only this scene's columns
  ARD_CUDA(cudaMemcpy2D(out, sizeof(double) * nrec, ctx->d_hist + t0 * ctx->n_rec_total + rec0,
                        sizeof(double) * ctx->n_rec_total, sizeof(double) * nrec, nt, cudaMemcpyDeviceToHost));
  for (int64_t i = 0; i < nt * nrec; ++i)
    if (!std::isfinite(out[i])) { ctx->err = "non-finite recorder sample (unstable scene?)"; return ARD_ERR_UNSTABLE; }
  return ARD_OK;
}

extern "C" int ard_read_recorders(ard_ctx* c, int32_t scene, float* out, int64_t t0, int64_t nt) {
  if (!c || (nt > 0 && !out)) return ARD_ERR_INVALID;
  Ctx* ctx = as_ctx(c);
  if (scene < -1 || scene >= (int)ctx->scenes.size()) { ctx->err = "bad scene index"; return ARD_ERR_RANGE; }
  const int nrec = scene < 0 ? ctx->n_rec_total : ctx->scenes[scene].nrec;
  std::vector<double> tmp((size_t)std::max<int64_t>(0, nt) * nrec);
  int rc = ard_read_recorders_f64(c, scene, tmp.data(), t0, nt);
  for (size_t i = 0; i < tmp.size(); ++i) out[i] = (float)tmp[i];
  return rc;
}

extern "C" int ard_read_field(ard_ctx* c, int32_t scene, int32_t partition, float* out) {
  if (!c || !out) return ARD_ERR_INVALID;
  Ctx* ctx = as_ctx(c);
  int kind, idx;
  int rc = part_lookup(ctx, scene, partition, &kind, &idx);
  if (rc) return rc;
  ARD_CUDA(cudaSetDevice(ctx->device));
  ARD_CUDA(cudaStreamSynchronize(ctx->stream));
  const size_t es = elem_size(ctx);
  const int lvl = (int)((ctx->t_host - 1) & 1);  // buffer holding the latest level
  if (kind == ARD_PART_DCT) {
    const DctDev& D = ctx->dct[idx];
    const long long N = (long long)D.w * D.h * D.d;
    const long long s0 = ctx->scratch;
    char* base = (char*)ctx->d_buf;
    // unpad the modes into the scratch, transform there: p = s_i * Ci^T Ci^T Ci^T M
    ARD_CUDA(cudaMemcpy2D(base + (s0 + 2 * N) * es, D.w * es, base + D.M[lvl] * es, D.wp * es, D.w * es,
                          (size_t)D.h * D.d, cudaMemcpyDeviceToDevice));
    rc = ctx->prec == ARD_PREC_F64 ? ard::dense_transform<double>(ctx, D, s0 + 2 * N, s0 + 2 * N, s0, true, D.si)
                                   : ard::dense_transform<float>(ctx, D, s0 + 2 * N, s0 + 2 * N, s0, true, D.si);
    if (rc == ARD_OK) {
      if (ctx->prec == ARD_PREC_F64) {
        std::vector<double> h(N);
        ARD_CUDA(cudaMemcpy(h.data(), base + (s0 + 2 * N) * es, N * es, cudaMemcpyDeviceToHost));
        for (long long i = 0; i < N; ++i) out[i] = (float)h[i];
      } else {
        ARD_CUDA(cudaMemcpy(out, base + (s0 + 2 * N) * es, N * es, cudaMemcpyDeviceToHost));
      }
    }
    return rc;
  }
  const PmlDev& P = ctx->pml[idx];
  const ard_partition& p = ctx->scenes[scene].parts[partition];
  std::vector<double> h(P.n);
  if (ctx->prec == ARD_PREC_F64) {
    ARD_CUDA(cudaMemcpy(h.data(), (char*)ctx->d_buf + P.p[lvl] * es, P.n * es, cudaMemcpyDeviceToHost));
  } else {
    std::vector<float> f(P.n);
    ARD_CUDA(cudaMemcpy(f.data(), (char*)ctx->d_buf + P.p[lvl] * es, P.n * es, cudaMemcpyDeviceToHost));
    h.assign(f.begin(), f.end());
  }
  // slab [l][a][b] -> [z][y][x]
  const int ax = P.type <= 1 ? 0 : (P.type <= 3 ? 1 : 2);
  for (int z = 0; z < p.depth; ++z)
    for (int y = 0; y < p.height; ++y)
      for (int x = 0; x < p.width; ++x) {
        long long s;
        if (ax == 0) s = ((long long)x * P.A + z) * P.Bp + y;
        else if (ax == 1) s = ((long long)y * P.A + z) * P.Bp + x;
        else s = ((long long)z * P.A + y) * P.Bp + x;
        out[((long long)z * p.height + y) * p.width + x] = (float)h[s];
      }
  return ARD_OK;
}

namespace ard {
// The error word of the kernels with bounded waits (tensor-core face passes):
// nonzero when one of them gave up.  Synchronous.
int check_device_error(Ctx* ctx) {
  if (!ctx->d_err) return ARD_OK;
  int v = 0;
  ARD_CUDA(cudaMemcpy(&v, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (v) {
    ctx->err = "a kernel gave up waiting at one of its barriers (device error word set)";
    return ARD_ERR_CUDA;
  }
  return ARD_OK;
}

// Checked mode: the guards around the pool must still hold their sentinel.
int check_guards(Ctx* ctx) {
  if (!ctx->guard_bytes) return ARD_OK;
  std::vector<unsigned char> h(ctx->guard_bytes);
  const size_t es = elem_size(ctx);
  const char* sides[2] = {"before", "after"};
  const char* addr[2] = {(const char*)ctx->d_buf_base, (const char*)ctx->d_buf + ctx->pool_elems * es};
  for (int k = 0; k < 2; ++k) {
    ARD_CUDA(cudaMemcpy(h.data(), addr[k], ctx->guard_bytes, cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < h.size(); ++i)
      if (h[i] != 0xA5) {
        const long long off = k == 0 ? -(long long)(ctx->guard_bytes - i) : (long long)i;
        ctx->err = std::string("stray write ") + sides[k] + " the element pool at byte offset " + std::to_string(off);
        std::fprintf(stderr, "ard: %s\n", ctx->err.c_str());
        return ARD_ERR_CUDA;
      }
  }
  return ARD_OK;
}
}  // namespace ard
