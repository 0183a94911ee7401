"""Index arithmetic of face2d_kernel (ard_kernels.cuh), mirrored on the CPU.

Both 256-thread CTAs of a job's cluster run through the job here as they do
on the device: the staging loops (cp.async, zero fill), the combine, the two
register-tiled products, the exchange of the halves of T and the global
stores, against shared-memory regions sized as build_layout sizes them
(ard_layout.cu) and poisoned with NaN.  The test asserts that every access
stays inside its region, that no poisoned (never written) element reaches a
product, that every output element of the slab is written exactly once,
that the rows of one left-operand load fall in distinct 16-byte bank
groups, and that the result is scale A (X0 +/- X1) B over the slab.
"""
import numpy as np
import pytest

THREADS, WARPS = 256, 8


def pitch(n):
    n4 = (n + 3) & ~3
    return n4 + (8 if n4 & 7 else 4)


def up4(n):
    return (n + 3) & ~3


class Region:
    def __init__(self, n, name):
        self.a = np.full(n, np.nan)
        self.name = name

    def read(self, i, n=1):
        assert 0 <= i and i + n <= len(self.a), (self.name, i, n, len(self.a))
        v = self.a[i:i + n].copy()
        assert not np.isnan(v).any(), (self.name, "poisoned read", i)
        return v

    def write(self, i, v):
        v = np.atleast_1d(v)
        assert 0 <= i and i + len(v) <= len(self.a), (self.name, i, len(v), len(self.a))
        self.a[i:i + len(v)] = v


def tiles(CT, MR, MODE, nrows, K, L0, L1, lp, R0, R1, rp, store):
    """face2d_tiles: thread (warp, lane) rows rb + rt + RT i, columns 4 ct .. +3."""
    RT = 32 // CT
    for warp in range(WARPS):
        for lane in range(32):
            ct, rt = lane % CT, lane // CT
            c0 = 4 * ct
            rb = warp * MR * RT
            while rb < nrows:
                rows = [min(rb + rt + RT * i, nrows - 1) for i in range(MR)]
                acc0 = np.zeros((MR, 4))
                acc1 = np.zeros((MR, 4))
                for k in range(0, K, 4):
                    r0 = np.array([R0.read((k + kk) * rp + c0, 4) for kk in range(4)])
                    r1 = np.array([R1.read((k + kk) * rp + c0, 4) for kk in range(4)]) if MODE == 2 else None
                    l0 = np.array([L0.read(r * lp + k, 4) for r in rows])
                    acc0 += l0 @ r0
                    if MODE == 1:
                        acc1 += np.array([L1.read(r * lp + k, 4) for r in rows]) @ r0
                    if MODE == 2:
                        acc1 += l0 @ r1
                for i in range(MR):
                    r = rb + rt + RT * i
                    if r < nrows:
                        store(r, c0, acc0[i], acc1[i] if MODE else None)
                rb += WARPS * MR * RT


def bank_groups_distinct(CT, MR, lp):
    """The RT lanes-groups of one left-operand load read RT consecutive rows."""
    RT = 32 // CT
    for i in range(MR):
        rows = [0 + rt + RT * i for rt in range(RT)]
        groups = [((r * lp * 4) // 16) % 8 for r in rows]
        for q in range(0, RT, 8):
            assert len(set(groups[q:q + 8])) == len(groups[q:q + 8])


def run_job(V, U, ld, u0, ub, which, rng, split=True):
    """The two CTAs of the job's cluster, h = 0, 1, with their own shared
    memory: a row-split job, or (split False) a whole job on CTA 0 while CTA 1
    runs an empty one (no rows, no stores) of the same pair."""
    narrow = 1 if ub <= 16 else 0
    xp, ap = pitch(U), pitch(V)
    Up, Vp = up4(U), up4(V)
    nh = (V + 1) // 2
    xs = (nh if split else V) * max(xp, ap)
    sm = dict(xs=xs, x1=xs, bs=32 * Up, ts=32 * Vp)
    x0 = rng.standard_normal((V, ld))
    x1 = rng.standard_normal((V, ld))
    Bt = rng.standard_normal((U, U))
    At = rng.standard_normal((V, V))
    scale = 0.37
    out = {0: np.full((V, ld), np.nan), 1: np.full((V, ld), np.nan)}
    written = {0: np.zeros((V, ld), int), 1: np.zeros((V, ld), int)}
    cq = 4 if narrow else 8
    bp = 4 * cq
    q4 = Up >> 2
    one = which != 0
    CT, MR = (4, 2) if narrow else (8, 2)
    bank_groups_distinct(CT, MR, xp)
    bank_groups_distinct(CT, MR, ap)
    cta = []
    for h in (0, 1):
        if split:
            r0, nr = (nh, V - nh) if h else (0, nh)
        else:
            r0, nr = 0, (0 if h else V)
        X0, X1 = Region(sm["xs"], f"X0[{h}]"), Region(sm["x1"], f"X1[{h}]")
        Bs, T0, T1 = Region(sm["bs"], "Bs"), Region(sm["ts"], f"T0[{h}]"), Region(sm["ts"], f"T1[{h}]")
        cta.append(dict(r0=r0, nr=nr, X0=X0, X1=X1, Bs=Bs, T0=T0, T1=T1))
        for tid in range(THREADS):
            warp, lane = tid >> 5, tid & 31
            for r in range(warp, nr, WARPS):
                for q in range(lane, q4, 32):
                    c = 4 * q
                    for e in range(4):
                        ok = c + e < U
                        X0.write(r * xp + c + e, x0[r0 + r, c + e] if ok else 0.0)
                        X1.write(r * xp + c + e, x1[r0 + r, c + e] if ok else 0.0)
            for i in range(tid, Up * cq, THREADS):
                j, c = i // cq, 4 * (i - (i // cq) * cq)
                for e in range(4):
                    ok = j < U and c + e < ub
                    Bs.write(j * bp + c + e, Bt[j, u0 + c + e] if ok else 0.0)
            for i in range(tid, (Vp - V) * bp, THREADS):
                T0.write(V * bp + i, 0.0)
                T1.write(V * bp + i, 0.0)
        for r in range(nr):
            for q in range(q4):
                a, b = X0.read(r * xp + 4 * q, 4), X1.read(r * xp + 4 * q, 4)
                if which == 2:
                    X0.write(r * xp + 4 * q, a - b)
                else:
                    X0.write(r * xp + 4 * q, a + b)
                    if which == 0:
                        X1.write(r * xp + 4 * q, a - b)

    def stage_a(c, dst):
        for o in range(c["nr"]):
            for q in range(Vp >> 2):
                r = 4 * q
                for e in range(4):
                    dst.write(o * ap + r + e, At[c["r0"] + o, r + e] if r + e < V else 0.0)

    for c in cta:                      # first product: own rows of T
        if one:
            stage_a(c, c["X1"])
        T0, T1, r0 = c["T0"], c["T1"], c["r0"]

        def to_t(r, c0, a0, a1, T0=T0, T1=T1, r0=r0):
            T0.write((r0 + r) * bp + c0, a0)
            if a1 is not None:
                T1.write((r0 + r) * bp + c0, a1)

        tiles(CT, MR, 0 if one else 1, c["nr"], Up, c["X0"], c["X1"], xp, c["Bs"], c["Bs"], bp, to_t)
    # cluster barrier; each CTA copies its peer's rows of T
    copies = []
    for h, c in enumerate(cta):
        if not one:
            stage_a(c, c["X0"])
        p = cta[h ^ 1]
        if not split:
            continue
        for tid in range(THREADS):
            for i in range(tid, p["nr"] * cq, THREADS):
                r, cc = p["r0"] + i // cq, 4 * (i % cq)
                copies.append((c["T0"], r * bp + cc, p["T0"].read(r * bp + cc, 4)))
                if not one:
                    copies.append((c["T1"], r * bp + cc, p["T1"].read(r * bp + cc, 4)))
    for dst, i, v in copies:
        dst.write(i, v)
    # cluster barrier; second product: own rows of the outputs
    o0 = 1 if which == 2 else 0
    for c in cta:
        As = c["X1"] if one else c["X0"]

        def to_out(r, c0, a0, a1, r0=c["r0"]):
            for k in range(4):
                if c0 + k < ub:
                    out[o0][r0 + r, u0 + c0 + k] = a0[k] * scale
                    written[o0][r0 + r, u0 + c0 + k] += 1
                    if a1 is not None:
                        out[1][r0 + r, u0 + c0 + k] = a1[k] * scale
                        written[1][r0 + r, u0 + c0 + k] += 1

        tiles(CT, MR, 0 if one else 2, c["nr"], Vp, As, As, ap, c["T0"], c["T1"], bp, to_out)
    E, O = x0[:, :U] + x1[:, :U], x0[:, :U] - x1[:, :U]
    want = {0: scale * At @ E @ Bt[:, u0:u0 + ub], 1: scale * At @ O @ Bt[:, u0:u0 + ub]}
    outs = [0, 1] if which == 0 else [which - 1]
    for k in outs:
        assert np.all(written[k][:, u0:u0 + ub] == 1)
        assert written[k].sum() == V * ub
        np.testing.assert_allclose(out[k][:, u0:u0 + ub], want[k], rtol=1e-10, atol=1e-10)
    for k in {0, 1} - set(outs):
        assert written[k].sum() == 0


@pytest.mark.parametrize("V,U,ld,u0,ub,which", [
    (12, 8, 8, 0, 8, 0),        # one narrow slab, both outputs
    (1, 4, 4, 0, 4, 1),         # one row: the second CTA has none
    (10, 7, 9, 0, 7, 1),        # ragged extents, row pitch != U (scalar staging)
    (9, 13, 13, 0, 13, 2),      # odd V (A columns and T rows padded), O only
    (20, 40, 40, 32, 8, 0),     # the tail slab of a 40-wide face
    (37, 36, 40, 0, 32, 0),     # a wide slab, odd V: halves of 19 and 18 rows
    (40, 64, 64, 32, 32, 1),    # wide, one output (A staged during the first product)
    (17, 20, 24, 16, 4, 2),     # a 4-column tail
])
def test_face2d_job_indexing(V, U, ld, u0, ub, which):
    run_job(V, U, ld, u0, ub, which, np.random.default_rng(V * 1000 + U))
    run_job(V, U, ld, u0, ub, which, np.random.default_rng(V * 1000 + U), split=False)


def test_face2d_rows_beyond_one_block_iteration():
    """Half of V larger than 8 warps x 8 rows: the warps loop over row blocks."""
    run_job(136, 8, 8, 0, 8, 0, np.random.default_rng(7))
