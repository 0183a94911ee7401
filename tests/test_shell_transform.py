"""The air-partition update on the 3-cell shell equals the dense 3D DCT pair.

The GPU modal kernel never forms dense force or pressure fields: the force
lives on 18 face layers, each 2D-transformed and expanded along its third
axis (layers j and 5-j combined by the parity of the mode index), and the
pressure is contracted back onto the same layers.  This checks that algebra
in numpy against scipy's REDFT10 / REDFT01 (scipy.fft.dctn type 2 / 3, the
definitions FFTW uses, as the reference's DctVolume does in
dct_volume.cpp:38-68).
"""
import numpy as np
import pytest
import scipy.fft as sf


def C(n):
    k = np.arange(n)[:, None]
    j = np.arange(n)[None, :]
    return 2.0 * np.cos(np.pi * (j + 0.5) * k / n)


def Ci(n):
    m = C(n).copy()
    m[0] *= 0.5
    return m


def layers(n):
    return [0, 1, 2, n - 3, n - 2, n - 1]


def shell_mask(w, h, d):
    m = np.zeros((d, h, w), bool)
    m[:, :, layers(w)] = True
    m[:, layers(h), :] = True
    m[layers(d), :, :] = True
    return m


@pytest.mark.parametrize("w,h,d", [(7, 11, 13), (10, 10, 40), (6, 9, 8), (16, 12, 6)])
def test_forward_expansion_matches_dense(w, h, d):
    rng = np.random.default_rng(w * 100 + h * 10 + d)
    f = rng.standard_normal((d, h, w)) * shell_mask(w, h, d)
    dense = sf.dctn(f, type=2)                       # [kz][ky][kx]
    Cw, Ch, Cd = C(w), C(h), C(d)
    X, Y, Z = layers(w), layers(h), layers(d)
    # owner decomposition: X layers own x on the shell, Y own y (x inside), Z the rest
    fX = np.stack([f[:, :, x] for x in X])            # [6][d][h]
    fY = np.stack([np.where(np.isin(np.arange(w), X), 0, f[:, y, :]) for y in Y])      # [6][d][w]
    inside_xy = ~np.isin(np.arange(w), X)[None, :] & ~np.isin(np.arange(h), Y)[:, None]
    fZ = np.stack([np.where(inside_xy, f[z], 0) for z in Z])                           # [6][h][w]
    F = np.zeros((d, h, w))
    for n in range(3):
        for pm, sg in ((0, 1), (1, -1)):
            PX = Cd @ (fX[n] + sg * fX[5 - n]) @ Ch.T    # [kz][ky]
            PY = Cd @ (fY[n] + sg * fY[5 - n]) @ Cw.T    # [kz][kx]
            PZ = Ch @ (fZ[n] + sg * fZ[5 - n]) @ Cw.T    # [ky][kx]
            par = lambda k: (np.arange(k) % 2) == pm
            F += (Cw[:, n] * par(w))[None, None, :] * PX[:, :, None]
            F += (Ch[:, n] * par(h))[None, :, None] * PY[:, None, :]
            F += (Cd[:, n] * par(d))[:, None, None] * PZ[None, :, :]
    np.testing.assert_allclose(F, dense, rtol=1e-10, atol=1e-10 * np.abs(dense).max())


@pytest.mark.parametrize("w,h,d", [(7, 11, 13), (10, 10, 40), (6, 9, 8)])
def test_inverse_contraction_matches_dense(w, h, d):
    rng = np.random.default_rng(7 + w)
    M = rng.standard_normal((d, h, w))
    dense = sf.dctn(M, type=3)                        # [z][y][x]
    Cwi, Chi, Cdi = Ci(w), Ci(h), Ci(d)
    X, Y, Z = layers(w), layers(h), layers(d)
    ev = lambda k: (np.arange(k) % 2) == 0
    for n in range(3):
        # contraction onto face row n, split by the parity of the contracted index
        for axis, Cc, Lst in ((2, Cwi, X), (1, Chi, Y), (0, Cdi, Z)):
            k = M.shape[axis]
            wgt_e = Cc[:, n] * ev(k)
            wgt_o = Cc[:, n] * ~ev(k)
            Re = np.tensordot(M, wgt_e, axes=([axis], [0]))
            Ro = np.tensordot(M, wgt_o, axes=([axis], [0]))
            for layer, R in ((n, Re + Ro), (5 - n, Re - Ro)):
                if axis == 2:   # R [kz][ky] -> p(x, y, z) on layer
                    p = Cdi.T @ R @ Chi
                    got, want = p, dense[:, :, Lst[layer]]
                elif axis == 1:  # R [kz][kx]
                    p = Cdi.T @ R @ Cwi
                    got, want = p, dense[:, Lst[layer], :]
                else:            # R [ky][kx]
                    p = Chi.T @ R @ Cwi
                    got, want = p, dense[Lst[layer], :, :]
                np.testing.assert_allclose(got, want, rtol=1e-10, atol=1e-10 * np.abs(dense).max())


def test_round_trip_gain_is_two():
    """REDFT01(REDFT10(x)) = 8N x, and the reference's scales give gain 2."""
    rng = np.random.default_rng(3)
    x = rng.standard_normal((5, 6, 7))
    N = x.size
    sf_ = 1.0 / (2.0 * np.sqrt(2.0 * N))
    si = 1.0 / np.sqrt(2.0 * N)
    y = si * sf.dctn(sf_ * sf.dctn(x, type=2), type=3)
    np.testing.assert_allclose(y, 2.0 * x, rtol=1e-12)
