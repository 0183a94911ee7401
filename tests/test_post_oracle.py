"""CPU checks of the oracle's restatements of the reference's post-step
products (oracle/post_oracle.py): MATLAB's fir1 / xcorr / fftfilt against
scipy's and numpy's implementations of the same published definitions,
t60.m on decays of known reverberation time, the colour map on the values
whose colours the reference's formula fixes, and the out_ cube order."""
import numpy as np
import pytest

from oracle import post_oracle as P


def test_fir1_matches_scipy_firwin():
    sig = pytest.importorskip("scipy.signal")
    for order, wn in ((1024, 3000 / 8000), (1024, 1500 / 4000), (64, 0.3), (10, 0.9)):
        b = P.fir1(order, wn)
        ref = sig.firwin(order + 1, wn, window="hamming", scale=True)
        assert np.abs(b - ref).max() < 1e-13
        assert abs(b.sum() - 1) < 1e-12


def test_xcorr_half_is_causal_convolution():
    rng = np.random.default_rng(3)
    rr, src = rng.standard_normal(300), rng.standard_normal(300)
    x = P.xcorr_first_half(rr, src[::-1])
    assert np.allclose(x, np.convolve(rr, src)[:300], rtol=0, atol=1e-12)
    # the definition: c[m] = sum_n x[n + m] y[n] over lags -(n-1) .. 0
    y = src[::-1]
    for lag in (-299, -150, -1, 0):
        want = sum(rr[n + lag] * y[n] for n in range(300) if 0 <= n + lag < 300)
        assert abs(x[lag + 299] - want) < 1e-10


def test_fftfilt_is_fir_filter():
    sig = pytest.importorskip("scipy.signal")
    rng = np.random.default_rng(4)
    x = rng.standard_normal(2000)
    b = P.fir1(64, 0.25)
    assert np.allclose(P.fftfilt(b, x), sig.lfilter(b, [1.0], x), rtol=0, atol=1e-12)


@pytest.mark.parametrize("t60_true_ms", [300.0, 700.0, 1200.0])
def test_t60_on_exponential_decay(t60_true_ms):
    """Noise with an exponential envelope of known T60 (60 dB of energy decay):
    the Schroeder fit of t60.m recovers it within a few percent."""
    sr = 16000.0
    n = int(2.0 * sr)
    rng = np.random.default_rng(5)
    t = np.arange(n) / sr
    env = 10 ** (-3 * t / (t60_true_ms / 1000.0))     # amplitude: -60 dB of energy at T60
    imp = env * rng.standard_normal(n)
    rt, slope, stop, overrun = P.t60(imp, sr)
    assert abs(rt - t60_true_ms) < 0.05 * t60_true_ms, (rt, t60_true_ms)
    assert slope < 0 and 0 < stop <= int(1.5 * sr)


def test_colour_map_fixed_points():
    w = P.slice_colour(np.array([0.0, 0.1, -0.1, 1.0, -1.0, np.nan], np.float32))
    assert w[0] == 0xFFFFFFFF          # norm 0.5: r = g = 255, b = 255
    assert w[1] == 0xFF0000FF          # norm 1: r = g = 0, b = 255
    assert w[2] == 0xFFFF0000          # norm 0: r = 255, g = b = 0
    assert w[3] == 0xFF0000FF and w[4] == 0xFFFF0000
    assert w[5] == 0xFF0000FF          # std::min(1.0f, NaN) is 1.0f


def test_colour_map_against_formula():
    """Per value, the reference's expressions evaluated one by one in float32."""
    rng = np.random.default_rng(6)
    p = (rng.standard_normal(2000) * 0.05).astype(np.float32)
    got = P.slice_colour(p)
    f = np.float32
    for v, word in zip(p, got):
        norm = f(f(0.5) * max(f(-1.0), min(f(1.0), f(v * f(10.0))))) + f(0.5)
        norm = f(norm)
        rnd = lambda x: int(np.floor(abs(float(x)) + 0.5) * np.sign(float(x)))
        if norm >= f(0.5):
            r = g = 255 - rnd(f(f(255.0) * f(2.0) * f(norm - f(0.5))))
            b = 255
        else:
            r = 255
            g = b = 255 - rnd(f(f(255.0) * f(f(1.0) - f(f(2.0) * norm))))
        assert word == (0xFF000000 | (r << 16) | (g << 8) | b)


def test_neighbourhood_order():
    field = np.arange(20 * 21 * 22, dtype=np.float64).reshape(20, 21, 22)   # [z][y][x]
    cube = P.neighbourhood(field, 10, 9, 8)
    assert cube.shape == (1000,)
    assert cube[0] == field[3, 4, 5] and cube[1] == field[3, 4, 6]        # x fastest
    assert cube[10] == field[3, 5, 5] and cube[100] == field[4, 4, 5]     # then y, then z
    assert cube[999] == field[12, 13, 14]
    assert np.array_equal(cube.reshape(10, 10, 10), field[3:13, 4:14, 5:15])


def test_render_slice_overwrite_order_and_local_coordinate():
    """Later partitions overwrite earlier ones; the slice coordinate is used
    as each partition's local coordinate, and reads outside it give 0."""
    parts = [(0, -1, 0, 0, 0, 4, 3, 5), (1, 0, 2, 0, 0, 3, 3, 2)]
    f0 = np.full((5, 3, 4), 0.05, np.float32)
    f1 = np.full((2, 3, 3), -0.05, np.float32)
    pix, pres = P.render_slice(parts, [f0, f1], 0, 1)
    assert pix.shape == (3, 5)
    assert np.all(pres[:, :2] == np.float32(0.05)) and np.all(pres[:, 2:] == np.float32(-0.05))
    pix, pres = P.render_slice(parts, [f0, f1], 0, 2)       # local z 2 lies outside the second partition
    assert np.all(pres[:, 2:] == 0) and np.all(pres[:, :2] == np.float32(0.05))
