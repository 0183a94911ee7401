// Device-side work tables of the GB300 ARD engine.
//
// Memory layout in HBM (one allocation per element type; table entries hold
// element offsets into it).  kx-indexed arrays use the row pitch
// wp = roundup(w, 4) so that four consecutive modes are one 128-bit access;
// the padding columns stay zero.
//
//   air partition (w x h x d cells)
//     M[2]           modal amplitudes, two time levels, [kz][ky][wp]
//     tabA, tabB     modal tables [kz][ky][wp]: accurate arithmetic
//                    1-cos(w dt) and 2(1-cos(w dt))/w^2 built in FP64;
//                    reference arithmetic cos(w dt) and w^2 as the
//                    reference computes them
//     fX, fY, fZ     force on the 3-cell shell: X layers [6][d][h] own the
//                    cells with x in {0,1,2,w-3,w-2,w-1}; Y layers [6][d][wp]
//                    own y in {0,1,2,h-3,h-2,h-1} with x inside; Z layers
//                    [6][h][wp] own z in {0,1,2,d-3,d-2,d-1} with x, y inside
//     pX, pY, pZ     pressure on the same face layers, each layer complete
//     PX, PY, PZ     2D DCT-II of the force layers, combined as
//                    layer(n) +/- layer(5-n): [2][3][..]
//     RX, RY, RZ     contractions of the new modes onto the face rows, one
//                    slab per modal tile along the contracted axis
//     tmpX..tmpZ     transform scratch [6][..]
//   PML slab (L layers along its normal, plane A x B, B fastest)
//     p[2], phi_n[2], phi_a[2], phi_b[2]   [L][A][B]
//     force strip    [3][A][B] (the 3 layers next to the air partition)
//
// The modal update of an air partition needs the force only on the shell and
// yields pressure only where the interfaces (shell) and recorders read it, so
// the dense 3D DCT pair of the reference (dct_partition.cpp:48-73) becomes
// 2D transforms of 18 face layers, one fused pass over the modes (expansion
// of the face transforms along the third axis + modal update + contraction
// onto the face rows) and 2D inverse transforms of the face layers.
// Forward basis (REDFT10) C_n(k, j) = 2 cos(pi (j + 1/2) k / n); inverse
// basis (REDFT01) Ci_n(k, j) = C_n(k, j) with k = 0 halved;
// C_n(k, n-1-j) = (-1)^k C_n(k, j) pairs layer j with layer 5-j.
#pragma once

#include <cstdint>

namespace ard {

constexpr int kMaxPointsPerPart = 8;  // sources or recorders per air partition
constexpr int kModalThreads = 256;    // 8 warps per modal tile
constexpr int kMaxPmlLayers = 12;

struct DctDev {
  int w, h, d, wp;
  int G, rpc, kxt;         // lanes per ky row, ky rows per tile, kx per tile (4 G)
  int nbx, nby, nbz, TZ;   // tiles along kx, ky, kz
  int tile0;
  int src0, nsrc;          // attached sources (PointDev table)
  int rec0, nrec;          // attached recorders
  long long M[2];
  long long tabA, tabB;
  long long fX, fY, fZ;
  long long pX, pY, pZ;
  long long PX, PY, PZ;
  long long RX, RY, RZ;
  long long tmpX, tmpY, tmpZ;
  long long cw, ch, cd;    // cosine tables of extents w, h, d: C, Ci, C^T, Ci^T (n*n each)
  long long recpart;       // [ntiles][nrec]
  long long srcpart;       // [ntiles][nsrc] (adjoint: source-gradient partials)
  long long AM[2];         // adjoint of the modal levels
  long long aX, aY, aZ;    // adjoint of the shell force
  long long qX, qY, qZ;    // adjoint of the face pressure
  double sf;               // forward scale 1 / (2 sqrt(2N))
  double si;               // inverse scale 1 / sqrt(2N)
  double damping;
};

struct PointDev {
  int part;     // air partition (engine index)
  int x, y, z;  // local cell
  int slot;     // global source / recorder index
};

struct PmlDev {
  int type;               // ARD_PML_*
  int L, A, B;            // layers along the normal; plane A x B (B fastest)
  int Bp;                 // row pitch of the plane: B rounded up to 4 (rows start on 16-byte
                          // boundaries, as the tensor-map tile loads of the PML kernel need)
  int strip0;             // first layer of the forced strip (L-3 or 0)
  int scene;
  long long p[2];
  long long phn[2], pha[2], phb[2];
  long long force;        // [3][A][Bp]
  long long ap[3];         // adjoint of p (three rotating levels)
  long long aphn[2], apha[2], aphb[2];
  long long aforce;        // adjoint of the strip force [3][A][Bp]
  long long zeta;         // [L] damping profile (scaled)
  long long n;            // L*A*Bp elements (padding columns stay zero)
  long long hoff;         // offset of the slab inside each all-slab region (p, phi: same for all eight)
  long long foff;         // offset of the slab's strip force inside the all-slab strip region
};

// Side of an interface: an air partition's face layers or a PML slab, both
// seen as [layer][v][u] arrays in the face's (u fast, v slow) coordinates.
struct SideDev {
  int kind;     // 0 air, 1 PML
  int idx;      // engine index (DctDev or PmlDev)
  int ou, ov;   // global (u, v) of the side's origin
  int ext;      // extent along the crossing axis
  int self;     // include_self_terms_
  // Direct addressing (filled at layout time, so the interface kernel reads
  // no partition tables): pressure of the n-th stencil layer (crossing
  // coordinate ext-3+n on the lo side, n on the hi side) at (u, v) is
  // pb[n][parity] + v * psv + u; the force of crossing coordinate c is, for
  // a PML side, fb + c * fls + v * fsv + u, for an air side the shell cell
  // of the layers fx / fy / fz of an extent-(w, h, d) partition (pitch wp).
  long long pb[3][2];
  int psv;
  int fsv;
  long long fb, fls;
  long long fx, fy, fz;
  int w, h, d, wp;
};

struct IfaceDev {
  int type;               // ARD_BOUNDARY_X/Y/Z: crossing axis
  int u0, u1, v0, v1;     // global face range
  SideDev lo, hi;         // left/top/front and right/bottom/back
  double absorption;
  long long mask;         // [cells] 6-bit write masks (bit m+3)
  long long cell0;        // first global face-cell index of this interface
};

// One batched 1D transform as a small GEMM, Out[m][nn] (row pitch ld):
//   cols (rows == 0): lines are columns of [n][ld];  Out = A X,   M = n, N = batch
//   rows (rows == 1): lines are rows of [batch][ld]; Out = X A^T, M = batch, N = n
// A(o, j) = C[o][j] (forward, REDFT10) or Ci[j][o] (inverse, REDFT01); ctab
// points at the matrix used.  X = in0 + sgn * in1 (in1 < 0: absent).
struct XformJob {
  long long in0, in1;
  long long out;
  long long ctab;
  int sgn;
  int n;
  int batch;
  int ld;
  int inverse;
  int rows;
  int first;    // first 64 x 64 output tile of this job
  int tn;       // tiles along N
  int ntiles;
  double scale;
};

// One fused 2D transform of a pair of face layers, for output columns
// [u0, u0 + ub):
//   out0 = scale A (X0 + X1) B,   out1 = scale A (X0 - X1) B
// X0, X1: V x U, row pitch ld; A: V x V, B: U x U (row-contiguous copies
// of the transform matrices, restricted to the slab's columns for B).
// Forward: A = C_V, B(j, u) = C_U[u][j]; inverse: A(o, r) = Ci_V[r][o],
// B(j, u) = Ci_U[j][u].
struct Face2DJob {
  long long in0, in1;
  long long out0, out1;
  long long tabA, tabB;
  int V, U, ld;
  int u0, ub;
  int which;     // 0: both outputs; 1: out0 only; 2: out1 only (a pair split over two blocks)
  int narrow;    // 1: at most 16 columns (16 rows per warp)
  int split;     // 1: the rows are split between the two CTAs of the cluster
  int part;      // air partition (engine index)
  double scale;
};

// One batched product of the tensor-core face transforms (ard_mma.cuh): one
// pass over the stacked layer outputs of one axis of one air partition,
//   out[o][n][r] = scale * sum_k Data(o, r)[k] * Table[n][k],
// data row m = o * R + r (output o, row r of it).
constexpr int kMmaMaxOut = 6;
constexpr int kMmaBK = 32;       // K chunk: one 128-byte swizzle row of fp32 / tf32
constexpr int kMmaBNMax = 160;   // widest N tile

// N tiling of a transform of length n: nt tiles of bn rows (bn a multiple of
// 16, at most kMmaBNMax).  The split tables are stored pre-tiled as
// [nt][nch][bn][32] with nch = ceil(n / 32): each (N tile, K chunk) block is
// the 128-byte-swizzled K-major image the tensor cores read, zero-padded.
__host__ __device__ inline void mma_ntile(int n, int* nt, int* bn) {
  const int t = (n + kMmaBNMax - 1) / kMmaBNMax;
  const int b = ((n + t - 1) / t + 15) & ~15;
  *bn = b;
  *nt = (n + b - 1) / b;
}
__host__ __device__ inline long long mma_table_elems(int n) {
  int nt, bn;
  mma_ntile(n, &nt, &bn);
  return (long long)nt * ((n + kMmaBK - 1) / kMmaBK) * bn * kMmaBK;
}

struct MmaJob {
  long long in0[kMmaMaxOut];   // data row r of output o: in0[o] + r * ldb  (+ sgn[o] * (in1[o] + r * ldb))
  long long in1[kMmaMaxOut];   // -1: no second input
  long long out[kMmaMaxOut];   // out[o] + n * ldo + r
  long long thi, tlo;          // split table, pre-tiled [nt][nch][bn][32] (mma_ntile)
  int sgn[kMmaMaxOut];
  int nout, R;                 // outputs, data rows per output
  int K, N, nch;               // contraction length, output columns, K chunks
  int ldb, ldo;
  int bn;                      // N tile width (multiple of 16, <= kMmaBNMax)
  int mt, nt;                  // tiles along M (128 rows) and N
  int first;                   // first tile of the job in its list
  int vec;                     // data rows start on 16-byte boundaries (ldb and inputs multiples of 4)
  float scale;
};

}  // namespace ard
