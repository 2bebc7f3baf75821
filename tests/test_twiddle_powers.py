"""CPU: the twiddle-power scheme of the FFT stages (fft.cuh ``twiddle_powers``),
restated in float32 with numpy.  A radix-R stage reads w, w^2, w^4 and w^8 of
its butterfly from the exp(-2 pi i m / 8192) table (each rounded once from
double) and forms w^3, w^5, w^6, w^7 and w^(8+r) as complex products of those,
rounding every real operation to float32 as the device does (with or without
a fused multiply-add the error is of the same order).  The error of every
power, for every table index a stage uses, stays below 4e-7 -- small against
the 1e-5 relative-L2 parity gate of the propagation paths."""
import numpy as np

FFT_MAX = 8192


def table():
    m = np.arange(FFT_MAX)
    a = -2.0 * np.pi * m / FFT_MAX
    return np.cos(a).astype(np.float32), np.sin(a).astype(np.float32)


def cmul(a, b):
    (ar, ai), (br, bi) = a, b
    f = np.float32
    return (f(ar * br) - f(ai * bi)).astype(np.float32), (f(ar * bi) + f(ai * br)).astype(np.float32)


def powers(c, s, m):
    """w^r, r = 1..15, as the device forms them from four table reads."""
    w = {k: (c[k * m], s[k * m]) for k in (1, 2, 4, 8)}
    w[3] = cmul(w[2], w[1])
    w[5], w[6], w[7] = cmul(w[4], w[1]), cmul(w[4], w[2]), cmul(w[4], w[3])
    out = {r: w[r] for r in range(1, 9)}
    return w, out


def test_powers_error_bound_all_indices():
    c, s = table()
    worst = 0.0
    for R, N in ((16, 8192), (16, 4096), (8, 2048), (16, 256)):
        # last-stage indices m = j * STEP (j < N / 16) and middle-stage k * STEP
        step = FFT_MAX // N
        m = np.arange(N // 16) * step
        m = m[(R - 1) * m < FFT_MAX]
        w, out = powers(c, s, m)
        for r in range(1, R):
            if r <= 8:
                got = out[r]
            else:  # v * w^8 * w^(r-8): the product the stage applies, taken on v = 1
                got = cmul(w[8], w[r - 8])
            exact = np.exp(-2j * np.pi * (r * m) / FFT_MAX)
            err = np.abs((got[0].astype(np.float64) + 1j * got[1].astype(np.float64)) - exact).max()
            worst = max(worst, err)
    assert worst < 4e-7, worst


def test_direct_table_is_the_reference_point():
    # the direct lookups the scheme replaces are within one float32 rounding
    c, s = table()
    m = np.arange(FFT_MAX)
    exact = np.exp(-2j * np.pi * m / FFT_MAX)
    err = np.abs(c.astype(np.float64) + 1j * s.astype(np.float64) - exact).max()
    assert err < 1e-7
