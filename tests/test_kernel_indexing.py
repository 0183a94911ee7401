"""Index algebra of the step kernels, checked on the CPU: the formulas below
restate the kernels' own (ard_kernels.cuh) and test the properties the
kernels rely on, so a change that breaks one fails here without a GPU.

- face_gemm_kernel: the XOR swizzle of k-contiguous operand tiles is a
  bijection inside each row and spreads the 16-byte chunks that one warp
  reads over distinct bank groups.
- modal_kernel: the ky fold (per-warp partial rows in the slot) and the quad
  reducers read every partial of a parity exactly once; the reduce-scatter of
  the kx contraction leaves each writing lane with the full sum of its value.
"""
import itertools

import numpy as np
import pytest


def kc_index(r, k):
    return r * 32 + ((((k >> 2) ^ (r >> 2)) & 7) << 2) + (k & 3)


@pytest.mark.parametrize("rows", [64, 128])
def test_gemm_swizzle_is_a_row_bijection(rows):
    for r in range(rows):
        idx = sorted(kc_index(r, k) for k in range(32))
        assert idx == list(range(r * 32, r * 32 + 32))


def test_gemm_swizzle_reads_hit_distinct_bank_groups():
    # P reads: rows ty*4 + i of the two ty values of a warp, one 16-byte chunk each
    for w in range(8):
        for i in range(4):
            for kq in range(0, 32, 4):
                groups = {(kc_index((2 * w + t) * 4 + i, kq) // 4) % 8 for t in (0, 1)}
                assert len(groups) == 2
    # Q reads: rows tx*4 + j of the 16 tx values; 16 distinct 16-byte chunks need
    # two wavefronts at best: each of the 8 bank groups is hit exactly twice
    for j in range(4):
        for kq in range(0, 32, 4):
            groups = [(kc_index(tx * 4 + j, kq) // 4) % 8 for tx in range(16)]
            assert sorted(np.bincount(groups, minlength=8)) == [2] * 8


@pytest.mark.parametrize("G", [8, 16, 32])
def test_modal_ky_fold_and_quad_reducers(G):
    KXT, threads = 4 * G, 256
    rpw = 32 // G
    rfold = min(rpw, 2)
    writes = {}   # slot index -> parity of the partial row written there
    for warp in range(threads // 32):
        for lane in range(32):
            yrow = lane // G
            if yrow >= rfold:
                continue
            li = lane % G
            for n in range(3):
                base = (warp * rfold + yrow) * 3 * KXT + 4 * li + n * KXT
                parity = (warp * rpw + yrow) & 1
                for e in range(4):
                    assert base + e not in writes
                    writes[base + e] = (parity, n, 4 * li + e)
    assert max(writes) < 3 * 1024          # fits one ry slot
    nquad = KXT // 4
    yterms = 8 if rfold == 2 else 4
    read = {}
    for tid in range(6 * nquad):
        pm = tid // (3 * nquad)
        rem = tid - pm * 3 * nquad
        n, kq = rem // nquad, rem % nquad
        ysrc = (pm * 3 + n) * KXT + 4 * kq
        for k in range(yterms):
            for e in range(4):
                i = ysrc + k * 6 * KXT + e
                assert writes[i] == (pm, n, 4 * kq + e)
                read[i] = read.get(i, 0) + 1
    assert set(read) == set(writes) and set(read.values()) == {1}
    # with G = 8 a warp's rows r and r + 2 share a parity: the xor-16 fold pairs them
    if rpw == 4:
        for lane in range(16):
            assert ((lane ^ 16) // G) & 1 == (lane // G) & 1


@pytest.mark.parametrize("G", [8, 16, 32])
def test_modal_kx_reduce_scatter(G):
    rng = np.random.default_rng(G)
    v = rng.integers(-1000, 1000, size=(G, 8)).astype(np.int64)
    v[:, 6:] = 0
    o4, o2, o1 = G >> 1, G >> 2, G >> 3
    h4 = np.zeros((G, 4), np.int64)
    for li in range(G):
        u4 = (li & o4) != 0
        p = li ^ o4
        for i in range(4):
            send_p = v[p, i] if (p & o4) else v[p, 4 + i]
            h4[li, i] = (v[li, 4 + i] if u4 else v[li, i]) + send_p
    h2 = np.zeros((G, 2), np.int64)
    for li in range(G):
        u2 = (li & o2) != 0
        p = li ^ o2
        for i in range(2):
            send_p = h4[p, i] if (p & o2) else h4[p, 2 + i]
            h2[li, i] = (h4[li, 2 + i] if u2 else h4[li, i]) + send_p
    h1 = np.zeros(G, np.int64)
    for li in range(G):
        u1 = (li & o1) != 0
        p = li ^ o1
        send_p = h2[p, 0] if (p & o1) else h2[p, 1]
        h1[li] = (h2[li, 1] if u1 else h2[li, 0]) + send_p
    o = o1 >> 1
    while o > 0:
        h1 = h1 + h1[np.arange(G) ^ o]
        o >>= 1
    total = v.sum(axis=0)
    for li in range(G):
        if li & (o1 - 1) == 0:
            q = li // o1
            assert q == 4 * bool(li & o4) + 2 * bool(li & o2) + bool(li & o1)
            assert h1[li] == total[q]


@pytest.mark.parametrize("per", [1, 2, 4, 8])
def test_partial_sum_items_cover_every_element_once(per):
    """post_modal_kernel's partial sums (ard_kernels.cuh): jobs start on
    kSumChunk boundaries of the index space; work item -> (chunk, part),
    thread tid takes elements e0 + tid + 256 i for i < per.  Every element of
    every job is summed exactly once, for each elements-per-thread choice."""
    chunk = 2048
    counts = [6, 2047, 2048, 2049, 9600, 5000, 1, 4096]
    first, t = [], 0
    for c in counts:
        first.append(t)
        t += (c + chunk - 1) // chunk * chunk
    parts = chunk // (256 * per)
    seen = [np.zeros(c, int) for c in counts]
    for item in range(t // chunk * parts):
        ch, part = divmod(item, parts)
        gg = ch * chunk
        lo = max(i for i in range(len(first)) if first[i] <= gg)
        e0 = gg - first[lo] + part * 256 * per
        idx = np.arange(256)[:, None] + 256 * np.arange(per)[None, :]
        e = (e0 + idx).ravel()
        e = e[e < counts[lo]]
        np.add.at(seen[lo], e, 1)
    assert all((s == 1).all() for s in seen)
