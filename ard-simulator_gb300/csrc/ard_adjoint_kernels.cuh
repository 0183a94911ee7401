// sm_103a kernels of the adjoint ARD step (gradients of a recorder misfit).
//
// The forward step is linear in its state, so the adjoint runs the
// transposed step backwards in time.  Per adjoint step t (after the forward
// step t's adjoint variables of step t + 1 are known):
//   iface_adjoint_kernel   transposed interface forcing: the adjoint shell
//                          force and PML strip force -> adjoint face pressure
//                          and adjoint PML pressure (atomic accumulation)
//   pml_adjoint_kernel     transposed Grote-Sim update; accumulates the
//                          gradient of every damping layer zeta(l) from the
//                          forward PML history
//   face2d / GEMM jobs     adjoint of the inverse face transform
//   modal_kernel<ADJ>      transposed modal recurrence, recorder residual
//                          injection, source-series gradient partials
//   srcgrad_kernel         source-series gradient of step t
//   face2d / GEMM jobs     adjoint of the forward face transform -> adjoint
//                          shell force of step t - 1
#pragma once

#include <cuda_runtime.h>

#include "ard_device.cuh"
#include "ard_kernels.cuh"

namespace ard {

// ---------------------------------------------------------------------------
// Interface forcing, transposed
// ---------------------------------------------------------------------------

template <typename T>
struct IfaceAdjArgs {
  T* buf;
  const IfaceDev* ifs;
  int nif;
  long long total;
  const DctDev* dct;
  const PmlDev* pml;
  const unsigned char* masks;
  int lin;    // level of the adjoint PML pressure of step t + 1 (the strip force enters p(t + 1) times dt^2)
  int lout;   // level of the adjoint PML pressure of step t (accumulated)
  T c0, dh, dt;
  const int* cell_iface;   // interface of every face cell
};

// Adjoint of the force value that the forward step writes at crossing
// coordinate c, face coordinates (u, v) of side s.
template <typename T>
__device__ __forceinline__ T adj_force(const IfaceAdjArgs<T>& a, int type, const SideDev& s, int c, int u, int v) {
  if (s.kind == 0) {
    const DctDev& D = a.dct[s.idx];
    const int x = type == 0 ? c : u;
    const int y = type == 0 ? u : (type == 1 ? c : v);
    const int z = type == 2 ? c : v;
    const long long o = shell_index(D, x, y, z);
    return o >= 0 ? a.buf[o - D.fX + D.aX] : (T)0;
  }
  const PmlDev& P = a.pml[s.idx];
  return a.dt * a.dt * a.buf[P.ap[a.lin] + ((long long)c * P.A + v) * P.Bp + u];
}

// Offset of the adjoint pressure value of crossing coordinate c, face
// coordinates (u, v) of side s (the cell the forward step read the pressure
// of).
template <typename T>
__device__ __forceinline__ long long adj_pressure_offset(const IfaceAdjArgs<T>& a, int type, const SideDev& s, int c,
                                                         int u, int v) {
  if (s.kind == 0) {
    const DctDev& D = a.dct[s.idx];
    const int layer = face_layer(c, s.ext);
    if (type == 0) return D.qX + ((long long)layer * D.d + v) * D.h + u;
    if (type == 1) return D.qY + ((long long)layer * D.d + v) * D.wp + u;
    return D.qZ + ((long long)layer * D.h + v) * D.wp + u;
  }
  const PmlDev& P = a.pml[s.idx];
  return P.ap[a.lout] + ((long long)c * P.A + v) * P.Bp + u;
}

// Transpose of iface_kernel: every force value the forward step writes
// (mask bit set) sends its adjoint back through the same 6-point stencil to
// the three pressure layers on each side that it was computed from.
template <typename T>
__global__ void __launch_bounds__(256) iface_adjoint_kernel(IfaceAdjArgs<T> a) {
  grid_dependency_wait();
  const T C[6][6] = {{0, 0, -2, 2, 0, 0},       {0, -2, 27, -27, 2, 0},     {-2, 27, -270, 270, -27, 2},
                     {2, -27, 270, -270, 27, -2}, {0, 2, -27, 27, -2, 0},     {0, 0, 2, -2, 0, 0}};
  for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x; g < a.total;
       g += (long long)gridDim.x * blockDim.x) {
    const IfaceDev& I = a.ifs[a.cell_iface[g]];
    const long long local = g - I.cell0;
    const int nu = I.u1 - I.u0;
    const int iu = I.u0 + (int)(local % nu);
    const int iv = I.v0 + (int)(local / nu);
    const unsigned mask = a.masks[I.mask + local];
    const int lu = iu - I.lo.ou, lv = iv - I.lo.ov;
    const int hu = iu - I.hi.ou, hv = iv - I.hi.ov;
    const T k = (T)I.absorption * (a.c0 * a.c0) / ((T)180 * a.dh * a.dh);
    T gl[3] = {0, 0, 0}, gh[3] = {0, 0, 0};
#pragma unroll
    for (int m = -3; m < 3; ++m) {
      if (!(mask & (1u << (m + 3)))) continue;
      const T fb = m < 0 ? adj_force(a, I.type, I.lo, I.lo.ext + m, lu, lv) : adj_force(a, I.type, I.hi, m, hu, hv);
      const T g = k * fb;
      const bool use_lo = m < 0 ? I.lo.self != 0 : true;
      const bool use_hi = m < 0 ? true : I.hi.self != 0;
#pragma unroll
      for (int n = 0; n < 3; ++n) {
        if (use_lo) gl[n] += g * C[m + 3][n];
        if (use_hi) gh[n] += g * C[m + 3][3 + n];
      }
    }
    // every target offset first, the atomics after them: descriptor fields
    // read after an atomic through the pool pointer would be loaded again
    long long ol[3], oh[3];
#pragma unroll
    for (int n = 0; n < 3; ++n) {
      ol[n] = adj_pressure_offset(a, I.type, I.lo, I.lo.ext - 3 + n, lu, lv);
      oh[n] = adj_pressure_offset(a, I.type, I.hi, n, hu, hv);
    }
#pragma unroll
    for (int n = 0; n < 3; ++n) {
      if (gl[n] != (T)0) atomicAdd(a.buf + ol[n], gl[n]);
      if (gh[n] != (T)0) atomicAdd(a.buf + oh[n], gh[n]);
    }
  }
}

// ---------------------------------------------------------------------------
// PML, transposed
// ---------------------------------------------------------------------------

template <typename T>
struct PmlAdjArgs {
  T* buf;
  const PmlDev* pml;
  const int4* blocks;   // {slab, a0, b0}: the forward kernel's 8 x 32 plane tiles
  int nblocks;
  int lx, ly, lo;       // adjoint pressure levels of steps t + 1, t + 2 (read, then cleared) and t (accumulated)
  int fin;              // level of the adjoint phi of step t + 1; step t's goes to fin ^ 1
  T dt, dh, c0;
  // forward PML history for the damping gradient (null: no gradient):
  // hist_p[j] = p(t0 - 1 + j), hist_phn[j] = phi_n(t0 + j), each `hlen`
  // elements in the all-slab region layout (slab at PmlDev::hoff)
  const T* hist_p;
  const T* hist_phn;
  long long hlen;
  const long long* tc;  // {t of the first step of the launch sequence, t0}
  int tstep;
  double* gz;           // [nblocks][kMaxPmlLayers] damping-gradient sums (accumulated)
  const CUtensorMap* amaps;   // per slab: ap[0..2], apha[0..1], aphb[0..1] as [L][A][B] tensors
  const CUtensorMap* hmaps;   // per slab: the history of p as a [K+1][L][A][B] tensor (null: no gradient)
  int* err;                   // set to 1 when a bounded wait runs out
};

// The adjoint PML kernel's tile boxes per layer (each 128-byte aligned in the
// stage): X = adjoint p(t+1) with a halo of 3 (x from b0 - 4), Phi_a with a
// halo of 2 along a, Phi_b with a halo of 2 along b (x from b0 - 4), and for
// the damping gradient the forward p(t) with a halo of 2 along both (x from
// b0 - 4).
template <typename T>
struct PmlAdjStage {
  static constexpr int PW = kPmlTB + 8;
  static constexpr int xs = (kPmlTA + 6) * PW * (int)sizeof(T);
  static constexpr int xsa = (xs + 127) & ~127;
  static constexpr int fa = (kPmlTA + 4) * kPmlTB * (int)sizeof(T);
  static constexpr int fb = kPmlTA * PW * (int)sizeof(T);
  static constexpr int fba = (fb + 127) & ~127;
  static constexpr int qs = (kPmlTA + 4) * PW * (int)sizeof(T);
  static constexpr int qsa = (qs + 127) & ~127;
  static constexpr int bytes = xsa + fa + fba + qsa;
};

// With X = adjoint p(t+1), Y = adjoint p(t+2), Phi = adjoint phi(t+1) and
// the forward operators of pml_kernel (L: 7-point Laplacian, D: 5-point
// derivative; L^T = L and D^T = -D under the zero-outside-the-slab rule):
//   p~(t)    += 2 X + dt^2 c^2 L X - dt z X + (-1 + dt z) Y
//               + dt Dn(z Phi_n) - dt z (Da Phi_a + Db Phi_b)
//   phi~n(t)  = (1 - dt z) Phi_n - dt^2 Dn X
//   phi~a(t)  = Phi_a - dt^2 Da X,   phi~b(t) = Phi_b - dt^2 Db X
// and, from the forward p(t), p(t-1), phi_n(t), the derivative of the
// forward step t + 1 with respect to z(l):
//   dJ/dz(l) += sum over layer l of  -dt X (p(t) - p(t-1))
//               - dt Phi_n (phi_n(t) + Dn p(t)) + dt Phi_a Da p(t) + dt Phi_b Db p(t)
template <typename T>
__global__ void __launch_bounds__(256, 4) pml_adjoint_kernel(PmlAdjArgs<T> a) {
  grid_dependency_wait();
  using S = PmlAdjStage<T>;
  constexpr int TA = kPmlTA, TB = kPmlTB, PW = S::PW;
  __shared__ __align__(128) unsigned char stage[2][S::bytes];
  __shared__ uint64_t bar[2];
  __shared__ volatile int s_abort;
  __shared__ double red[8][kMaxPmlLayers];
  const T c7[7] = {2, -27, 270, -490, 270, -27, 2};
  const T c5[5] = {1, -8, 0, 8, -1};
  const int tb = threadIdx.x & 31, ta = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const bool zgrad = a.hist_p != nullptr;
  long long hofs = 0;
  if (zgrad) {
    const long long t = a.tc[0] - a.tstep;
    hofs = t - a.tc[1];   // hist_p[hofs + 1] = p(t), hist_p[hofs] = p(t-1), hist_phn[hofs] = phi_n(t)
  }
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    mbar_init_fence();
    s_abort = 0;
  }
  __syncthreads();
  // thread 0's issue cursor over the block's (tile, layer) sequence, one layer
  // ahead of the computation: X, Phi_a, Phi_b (and p(t)) boxes of the layer
  int ibi = blockIdx.x, il = 0, iL = 0;
  uint32_t issued = 0;
  const uint32_t tx = (uint32_t)(S::xs + S::fa + S::fb + (zgrad ? S::qs : 0));
  auto issue_next = [&]() {
    if (ibi >= a.nblocks) return;
    const int4 blk = a.blocks[ibi];
    if (il == 0) iL = a.pml[blk.x].L;
    const CUtensorMap* mp = a.amaps + 7LL * blk.x;
    const int sg = (int)(issued & 1);
    unsigned char* sb = stage[sg];
    mbar_arrive_expect_tx(&bar[sg], tx);
    tma_load_3d(sb, mp + a.lx, blk.z - 4, blk.y - 3, il, &bar[sg]);
    tma_load_3d(sb + S::xsa, mp + 3 + a.fin, blk.z, blk.y - 2, il, &bar[sg]);
    tma_load_3d(sb + S::xsa + S::fa, mp + 5 + a.fin, blk.z - 4, blk.y, il, &bar[sg]);
    if (zgrad) tma_load_4d(sb + S::xsa + S::fa + S::fba, a.hmaps + blk.x, blk.z - 4, blk.y - 2, il, (int)(hofs + 1), &bar[sg]);
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
  uint32_t used = 0;
  bool stop = false;
  const T dt = a.dt, dt2 = a.dt * a.dt;
  const T r180 = (T)1 / ((T)180 * a.dh * a.dh), r12 = (T)1 / ((T)12 * a.dh);
  for (int bi = blockIdx.x; bi < a.nblocks && !stop; bi += gridDim.x) {
    const int4 blk = a.blocks[bi];
    const PmlDev& P = a.pml[blk.x];
    const int L = P.L, A = P.A, B = P.B, Bp = P.Bp;
    const long long hoff = P.hoff;   // in registers: the layer loop stores through the pool pointer
    const int a0 = blk.y, b0 = blk.z;
    const int ia = a0 + ta, ib = b0 + tb;
    const bool inside = ia < A && ib < B;
    const long long lstride = (long long)A * Bp;
    const long long col = inside ? (long long)ia * Bp + ib : 0;
    const T* X = a.buf + P.ap[a.lx];
    T* Y = a.buf + P.ap[a.ly];
    T* O = a.buf + P.ap[a.lo];
    const T* Fn = a.buf + P.aphn[a.fin];
    T* Fn_o = a.buf + P.aphn[a.fin ^ 1];
    T* Fa_o = a.buf + P.apha[a.fin ^ 1];
    T* Fb_o = a.buf + P.aphb[a.fin ^ 1];
    const T* zeta = a.buf + P.zeta;
    const T* hp = zgrad ? a.hist_p + (hofs + 1) * a.hlen + hoff : nullptr;    // p(t)
    const T* hpp = zgrad ? a.hist_p + hofs * a.hlen + hoff : nullptr;         // p(t-1)
    const T* hfn = zgrad ? a.hist_phn + hofs * a.hlen + hoff : nullptr;       // phi_n(t)
    // register windows along the normal: X(l-3 .. l+3), z Phi_n(l-2 .. l+2), p(t)(l-2 .. l+2)
    T xw[7], zw[5], qw[5];
#pragma unroll
    for (int m = 0; m < 7; ++m) {
      const int ll = m - 3;
      xw[m] = (inside && ll >= 0 && ll < L) ? X[ll * lstride + col] : (T)0;
    }
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      const int ll = m - 2;
      const bool ok = inside && ll >= 0 && ll < L;
      zw[m] = ok ? zeta[ll] * Fn[ll * lstride + col] : (T)0;
      qw[m] = (ok && zgrad) ? hp[ll * lstride + col] : (T)0;
    }
    if (zgrad) {
      if (threadIdx.x < 8 * kMaxPmlLayers) red[threadIdx.x / kMaxPmlLayers][threadIdx.x % kMaxPmlLayers] = 0;
      __syncthreads();   // cleared before any warp adds its first layer sum
    }
    // the next layer's point values, fetched while the current layer computes
    T ny = 0, no = 0, nfn = 0, npp = 0, nhf = 0;
    auto fetch = [&](int l) {
      const long long I = l * lstride + col;
      ny = inside ? Y[I] : (T)0;
      no = inside ? O[I] : (T)0;
      nfn = inside ? Fn[I] : (T)0;
      if (zgrad) {
        npp = inside ? hpp[I] : (T)0;
        nhf = inside ? hfn[I] : (T)0;
      }
    };
    fetch(0);
    for (int l = 0; l < L; ++l) {
      const int sg = (int)(used & 1);
      mbar_wait_bounded(&bar[sg], (used >> 1) & 1, &s_abort);
      const T* Xs = reinterpret_cast<const T*>(stage[sg]);                                  // [TA + 6][PW]
      const T* FA = reinterpret_cast<const T*>(stage[sg] + S::xsa);                         // [TA + 4][TB]
      const T* FB = reinterpret_cast<const T*>(stage[sg] + S::xsa + S::fa);                 // [TA][PW]
      const T* Qs = reinterpret_cast<const T*>(stage[sg] + S::xsa + S::fa + S::fba);        // [TA + 4][PW]
      const T y0 = ny, o0 = no, fn0 = nfn, pp0 = npp, hf0 = nhf;
      if (l + 1 < L) fetch(l + 1);
      T g = 0;
      if (inside && !s_abort) {
        T lx = 0;
#pragma unroll
        for (int m = 0; m < 7; ++m) lx += c7[m] * (xw[m] + Xs[(ta + m) * PW + tb + 4] + Xs[(ta + 3) * PW + tb + 1 + m]);
        T dnx = 0, dax = 0, dbx = 0, dnz = 0, daf = 0, dbf = 0;
#pragma unroll
        for (int m = 0; m < 5; ++m) {
          dnx += c5[m] * xw[m + 1];
          dax += c5[m] * Xs[(ta + 1 + m) * PW + tb + 4];
          dbx += c5[m] * Xs[(ta + 3) * PW + tb + 2 + m];
          dnz += c5[m] * zw[m];
          daf += c5[m] * FA[(ta + m) * TB + tb];
          dbf += c5[m] * FB[ta * PW + tb + 2 + m];
        }
        lx *= r180;
        dnx *= r12; dax *= r12; dbx *= r12;
        dnz *= r12; daf *= r12; dbf *= r12;
        const long long I = l * lstride + col;
        const T zn = zeta[l];
        const T x0 = xw[3];
        const T fa0 = FA[(ta + 2) * TB + tb], fb0 = FB[ta * PW + tb + 4];
        O[I] = o0 + (T)2 * x0 + dt2 * a.c0 * a.c0 * lx - dt * zn * x0 + (dt * zn - (T)1) * y0 + dt * dnz -
               dt * zn * (daf + dbf);
        Y[I] = 0;
        Fn_o[I] = ((T)1 - dt * zn) * fn0 - dt2 * dnx;
        Fa_o[I] = fa0 - dt2 * dax;
        Fb_o[I] = fb0 - dt2 * dbx;
        if (zgrad) {
          T dnp = 0, dap = 0, dbp = 0;
#pragma unroll
          for (int m = 0; m < 5; ++m) {
            dnp += c5[m] * qw[m];
            dap += c5[m] * Qs[(ta + m) * PW + tb + 4];
            dbp += c5[m] * Qs[(ta + 2) * PW + tb + 2 + m];
          }
          dnp *= r12; dap *= r12; dbp *= r12;
          g = -dt * x0 * (qw[2] - pp0) - dt * fn0 * (hf0 + dnp) + dt * (fa0 * dap + fb0 * dbp);
        }
      }
      if (zgrad) {
        // the warp's sum in the working type (FP64 arithmetic is scarce on
        // this GPU), the block's sums over warps and tiles in double
        const T sw = warp_sum(g);
        if (lane == 0) red[warp][l] += (double)sw;
      }
      // slide the windows one layer
#pragma unroll
      for (int m = 0; m < 6; ++m) xw[m] = xw[m + 1];
      xw[6] = (inside && l + 4 < L) ? X[(l + 4) * lstride + col] : (T)0;
#pragma unroll
      for (int m = 0; m < 4; ++m) { zw[m] = zw[m + 1]; qw[m] = qw[m + 1]; }
      const bool ok3 = inside && l + 3 < L;
      zw[4] = ok3 ? zeta[l + 3] * Fn[(l + 3) * lstride + col] : (T)0;
      qw[4] = (ok3 && zgrad) ? hp[(l + 3) * lstride + col] : (T)0;
      __syncthreads();   // every thread is done with stage sg
      if (s_abort) {
        stop = true;
        break;
      }
      if (threadIdx.x == 0) issue_next();
      ++used;
    }
    if (stop) break;
    if (zgrad) {
      if (threadIdx.x < L) {
        double sum = 0;
        for (int w8 = 0; w8 < 8; ++w8) sum += red[w8][threadIdx.x];
        a.gz[(long long)bi * kMaxPmlLayers + threadIdx.x] += sum;
      }
      __syncthreads();   // the layer sums are read before the next tile clears them
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
// Source-series gradient, initial-pressure gradient, counters
// ---------------------------------------------------------------------------

// dJ/d series[slot][t] = s_f * (sum of the modal tiles' partials); one warp per source.
// g is [steps][ld], columns = global source slots.
template <typename T>
__global__ void srcgrad_kernel(const T* __restrict__ buf, const DctDev* __restrict__ dct,
                               const PointDev* __restrict__ srcs, int npts, int ld, double* __restrict__ g,
                               const long long* tc, int tstep) {
  grid_dependency_wait();
  const int lane = threadIdx.x & 31;
  const int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (r >= npts) return;
  const PointDev q = srcs[r];
  const DctDev& D = dct[q.part];
  const int local = r - D.src0;
  const int ntiles = D.nbx * D.nby * D.nbz;
  T s = 0;
  for (int i = lane; i < ntiles; i += 32) s += buf[D.srcpart + (long long)i * D.nsrc + local];
  s = warp_sum(s);
  const long long t = tc[0] - tstep;
  if (lane == 0) g[t * ld + q.slot] = (double)s * D.sf;
}

// dJ/dm0 for modes that start at rest (M(-1) = M(-2) = m0):
// (alpha - a) mu(0) - a mu(1), written unpadded [kz][ky][kx] at `out`.
template <typename T, bool REF>
__global__ void init_grad_kernel(T* buf, DctDev D, long long out) {
  const long long N = (long long)D.w * D.h * D.d;
  const T a = (T)D.damping;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(i % D.w);
    const long long yz = i / D.w;
    const long long pi = yz * D.wp + x;
    const T ta = buf[D.tabA + pi];
    const T c1 = REF ? a * ((T)2 * ta - (T)1) : a * ((T)1 - (T)2 * ta);
    buf[out + i] = c1 * buf[D.AM[0] + pi] - a * buf[D.AM[1] + pi];
  }
}

static __global__ void set_counters_kernel(long long* tc, long long t, long long t0) {
  if (threadIdx.x == 0 && blockIdx.x == 0) { tc[0] = t; tc[1] = t0; }
}

}  // namespace ard
