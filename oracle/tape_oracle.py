"""ORACLE / TEST INFRASTRUCTURE ONLY -- the checker, never the product.

FP64 autograd tape of the ARD time step: the algorithm of oracle/ard_oracle.c
(itself a restatement of the reference CPU solver) written with torch tensor
operations on the CPU, so that torch's reverse mode gives the gradients of a
recorder misfit with respect to the source series, the initial pressure of
the air partitions and the six PML face scales.  It checks the hand-written
adjoint of the GPU library.  Dense and slow: for scenes of a few thousand
cells and a few tens of steps.

What follows which reference code (paths in ARD-simulator-190113/):
  step order ............ simulation.cpp:300-318 (phase A per partition, then
                          phase B per boundary in list order, last write wins)
  source forcing ........ partition.cpp:187-197 (overwrite the force cell)
  modal tables .......... dct_partition.cpp:20-36 (1-based mode numbers)
  air partition update .. dct_partition.cpp:48-73, dct_volume.cpp:38-68
  PML profile ........... pml_partition.cpp:26-28,59-86 (times the face scale)
  PML update ............ pml_partition.cpp:113-200 (force cleared after use)
  interface forcing ..... boundary.cpp:21-173
Scenes are the flat scenes of oracle/oracle.py.
"""
from __future__ import annotations

import math

import numpy as np
import torch

DCT, PML = 0, 1
P_LEFT, P_RIGHT, P_TOP, P_BOTTOM, P_FRONT, P_BACK = range(6)
BX, BY, BZ = 0, 1, 2
_C6 = [[0, 0, -2, 2, 0, 0], [0, -2, 27, -27, 2, 0], [-2, 27, -270, 270, -27, 2],
       [2, -27, 270, -270, 27, -2], [0, 2, -27, 27, -2, 0], [0, 0, 2, -2, 0, 0]]
_L7 = [2.0, -27.0, 270.0, -490.0, 270.0, -27.0, 2.0]
_D5 = [1.0, -8.0, 0.0, 8.0, -1.0]


def _redft10(n):
    """Y = C X along an axis: Y_k = 2 sum_j X_j cos(pi (j + 1/2) k / n)."""
    k = torch.arange(n, dtype=torch.float64)[:, None]
    j = torch.arange(n, dtype=torch.float64)[None, :]
    return 2.0 * torch.cos(math.pi * (j + 0.5) * k / n)


def _redft01(n):
    """Y = D X along an axis: Y_j = X_0 + 2 sum_{k>=1} X_k cos(pi k (j + 1/2) / n)."""
    j = torch.arange(n, dtype=torch.float64)[:, None]
    k = torch.arange(n, dtype=torch.float64)[None, :]
    D = 2.0 * torch.cos(math.pi * k * (j + 0.5) / n)
    D[:, 0] = 1.0
    return D


def _apply3(Mz, My, Mx, a):
    """The separable 3D transform of a [z][y][x] array."""
    return torch.einsum("zc,yb,xa,cba->zyx", Mz, My, Mx, a)


def _shift(a, axis, s):
    """a shifted by s along axis with zeros entering: out[i] = a[i + s] (0 outside)."""
    n = a.shape[axis]
    out = torch.zeros_like(a)
    if abs(s) >= n:
        return out
    src = [slice(None)] * 3
    dst = [slice(None)] * 3
    if s >= 0:
        src[axis] = slice(s, n)
        dst[axis] = slice(0, n - s)
    else:
        src[axis] = slice(0, n + s)
        dst[axis] = slice(-s, n)
    out[tuple(dst)] = a[tuple(src)]
    return out


def _stencil(a, axis, coefs, half):
    return sum(c * _shift(a, axis, m - half) for m, c in enumerate(coefs) if c != 0.0)


class TapeOracle:
    def __init__(self, flat):
        p = flat["params"]
        # the scene carries float parameters (include/ard_gb300.h): their float values, in double
        f32 = lambda v: float(np.float32(v))
        self.dh, self.dt, self.c0 = f32(p["dh"]), f32(p["dt"]), f32(p["c0"])
        self.R = f32(p.get("pml_R", 1e-5) or 1e-5)
        self.damping = f32(p.get("modal_damping", 0.999) or 0.999)
        self.layers = int(p["pml_layers"])
        self.parts = [tuple(q) for q in flat["partitions"]]
        self.bnds = [tuple(b) for b in flat["boundaries"]]
        self.srcs = [tuple(s) for s in flat["sources"]]
        self.recs = [tuple(r) for r in flat["recorders"]]
        self.tables = {}
        for i, (kind, _, _, _, _, w, h, d) in enumerate(self.parts):
            if kind != DCT:
                continue
            lx2, ly2, lz2 = (w * self.dh) ** 2, (h * self.dh) ** 2, (d * self.dh) ** 2
            kz = torch.arange(1, d + 1, dtype=torch.float64)[:, None, None]
            ky = torch.arange(1, h + 1, dtype=torch.float64)[None, :, None]
            kx = torch.arange(1, w + 1, dtype=torch.float64)[None, None, :]
            om = self.c0 * math.pi * torch.sqrt(kz ** 2 / lz2 + ky ** 2 / ly2 + kx ** 2 / lx2)
            self.tables[i] = dict(cwt=torch.cos(om * self.dt), w2=om ** 2,
                                  Cz=_redft10(d), Cy=_redft10(h), Cx=_redft10(w),
                                  Dz=_redft01(d), Dy=_redft01(h), Dx=_redft01(w),
                                  N=w * h * d)

    def _profile(self, i, scale6):
        """zx, zy, zz of PML partition i (pml_partition.cpp:59-86) times its face scale."""
        kind, ptype, _, _, _, w, h, d = self.parts[i]
        th = self.layers * self.dh
        zeta = self.c0 / th * math.log10(1.0 / self.R)
        z0 = zeta * scale6[ptype]

        def prof(n, rev):
            s = torch.arange(n, dtype=torch.float64)
            s = (n - s) if rev else (s + 1)
            return z0 * (s / th * self.dh - torch.sin(2.0 * math.pi * s * self.dh / th) / 2.0 / math.pi)

        zero = torch.zeros((d, h, w), dtype=torch.float64)
        zx, zy, zz = zero, zero, zero
        if ptype in (P_LEFT, P_RIGHT):
            zx = prof(w, ptype == P_LEFT)[None, None, :].expand(d, h, w)
        elif ptype in (P_TOP, P_BOTTOM):
            zy = prof(h, ptype == P_TOP)[None, :, None].expand(d, h, w)
        else:
            zz = prof(d, ptype == P_FRONT)[:, None, None].expand(d, h, w)
        return zx, zy, zz

    def run(self, series, T, p0=None, scale6=None):
        """Recorder samples [T][n_recorders] (float64 tensor, differentiable in
        series [n_sources][>= T], p0 {partition: [d][h][w]} and scale6 [6])."""
        dt, dh, c0 = self.dt, self.dh, self.c0
        if scale6 is None:
            scale6 = torch.ones(6, dtype=torch.float64)
        st = {}
        for i, (kind, _, _, _, _, w, h, d) in enumerate(self.parts):
            z = torch.zeros((d, h, w), dtype=torch.float64)
            if kind == DCT:
                tb = self.tables[i]
                pm, prev, pres = z, z, z
                if p0 is not None and i in p0:
                    si = 1.0 / math.sqrt(2.0 * tb["N"])
                    pm = _apply3(tb["Cz"], tb["Cy"], tb["Cx"], p0[i]) / (8.0 * tb["N"] * si)
                    prev, pres = pm, p0[i]
                st[i] = dict(f=z, pm=pm, prev=prev, p=pres)
            else:
                zx, zy, zz = self._profile(i, scale6)
                st[i] = dict(pold=z, p=z, phx=z, phy=z, phz=z, force=z, zx=zx, zy=zy, zz=zz)
        out = []
        for t in range(T):
            # ---- phase A ----
            for i, (kind, _, xs, ys, zs, w, h, d) in enumerate(self.parts):
                S = st[i]
                if kind == DCT:
                    tb = self.tables[i]
                    f = S["f"]
                    for sidx, (x, y, zc, part) in enumerate(self.srcs):
                        if part == i:
                            f = f.clone()
                            f[zc - zs, y - ys, x - xs] = series[sidx][t]
                    N = tb["N"]
                    fm = _apply3(tb["Cz"], tb["Cy"], tb["Cx"], f) / (2.0 * math.sqrt(2.0 * N))
                    nxt = self.damping * (2.0 * S["pm"] * tb["cwt"] - S["prev"] +
                                          (2.0 * fm / tb["w2"]) * (1.0 - tb["cwt"]))
                    p = _apply3(tb["Dz"], tb["Dy"], tb["Dx"], nxt) / math.sqrt(2.0 * N)
                    st[i] = dict(f=f, pm=nxt, prev=S["pm"], p=p)
                else:
                    p, po = S["p"], S["pold"]
                    zx, zy, zz = S["zx"], S["zy"], S["zz"]
                    lap = sum(_stencil(p, ax, _L7, 3) for ax in (2, 1, 0)) / (180.0 * dh * dh)
                    div = (_stencil(S["phx"], 2, _D5, 2) + _stencil(S["phy"], 1, _D5, 2) +
                           _stencil(S["phz"], 0, _D5, 2)) / (12.0 * dh)
                    pn = (2 * p - po + dt * dt * (c0 * c0 * lap - (zx + zy + zz) * (p - po) / dt -
                                                  (zx * zy + zy * zz + zx * zz) * p + div + S["force"]))
                    ux = _stencil(p, 2, _D5, 2) / (12.0 * dh)
                    uy = _stencil(p, 1, _D5, 2) / (12.0 * dh)
                    uz = _stencil(p, 0, _D5, 2) / (12.0 * dh)
                    st[i] = dict(pold=p, p=pn,
                                 phx=S["phx"] - dt * zx * S["phx"] + dt * (zy + zz - zx) * ux,
                                 phy=S["phy"] - dt * zy * S["phy"] + dt * (zx + zz - zy) * uy,
                                 phz=S["phz"] - dt * zz * S["phz"] + dt * (zx + zy - zz) * uz,
                                 force=torch.zeros_like(p), zx=zx, zy=zy, zz=zz)
            # ---- phase B: interfaces in list order ----
            for (btype, ia, ib, bxs, bxe, bys, bye, bzs, bze, absorp) in self.bnds:
                self._forcing(st, btype, ia, ib, (bxs, bxe, bys, bye, bzs, bze), float(absorp))
            # ---- recorders ----
            row = []
            for (x, y, zc, part) in self.recs:
                kind, _, xs, ys, zs, _, _, _ = self.parts[part]
                row.append(st[part]["p"][zc - zs, y - ys, x - xs])
            out.append(torch.stack(row) if row else torch.zeros(0, dtype=torch.float64))
        return torch.stack(out)

    def _forcing(self, st, btype, ia, ib, box, absorp):
        bxs, bxe, bys, bye, bzs, bze = box
        A, B = self.parts[ia], self.parts[ib]
        # crossing axis in [z][y][x] arrays: X -> 2, Y -> 1, Z -> 0
        ax = {BX: 2, BY: 1, BZ: 0}[btype]
        start = {2: 2, 1: 3, 0: 4}[ax]          # x_start / y_start / z_start in the partition tuple
        ext_i = {2: 5, 1: 6, 0: 7}[ax]          # width / height / depth
        a_end = A[start] + A[ext_i]
        lo_is_a = {BX: bxs <= a_end and bxe >= a_end, BY: bys <= a_end and bye >= a_end,
                   BZ: bzs <= a_end and bze >= a_end}[btype]
        lo, hi = (ia, ib) if lo_is_a else (ib, ia)
        # face range in global coordinates of the two other axes, as slices per side
        rng = {2: (bxs, bxe), 1: (bys, bye), 0: (bzs, bze)}

        def face(part):
            P = self.parts[part]
            org = {2: P[2], 1: P[3], 0: P[4]}
            sl = [None, None, None]
            for a in (0, 1, 2):
                if a != ax:
                    sl[a] = slice(rng[a][0] - org[a], rng[a][1] - org[a])
            return sl

        def read(part, c):
            sl = face(part)
            sl[ax] = c
            return st[part]["p"][tuple(sl)]

        def write(part, c, val):
            key = "f" if self.parts[part][0] == DCT else "force"
            arr = st[part][key].clone()
            sl = face(part)
            sl[ax] = c
            arr[tuple(sl)] = val
            st[part][key] = arr

        lext = self.parts[lo][ext_i]
        pl = [read(lo, lext - 3 + n) for n in range(3)]
        ph = [read(hi, n) for n in range(3)]
        lself = self.parts[lo][0] == DCT
        hself = self.parts[hi][0] == DCT
        k = self.c0 * self.c0 / (180.0 * self.dh * self.dh)
        for m in range(-3, 3):
            sip1 = sum(_C6[m + 3][n] * pl[n] for n in range(3))
            sip2 = sum(_C6[m + 3][n + 3] * ph[n] for n in range(3))
            if m < 0:
                sip = sip1 + sip2 if lself else sip2
                write(lo, lext + m, absorp * (sip * k))
            else:
                sip = sip1 + sip2 if hself else sip1
                write(hi, m, absorp * (sip * k))
