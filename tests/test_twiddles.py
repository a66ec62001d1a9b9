"""Twiddle factors of the large shared-memory transforms, restated in
numpy float32: a radix-4 stage with Ns previous points reads w^k from the
quarter-wave table (exact to float32 rounding) and forms w^2k and w^3k as
complex products.  The products stay within a few float32 roundings of the
exact values for every stage of transforms up to 2^14 points.  CPU only."""
import numpy as np


def _cmul32(a, b):
    ar, ai = np.float32(a.real), np.float32(a.imag)
    br, bi = np.float32(b.real), np.float32(b.imag)
    return np.complex64(complex(ar * br - ai * bi, ar * bi + ai * br))


def test_product_twiddles_stay_within_float32_rounding():
    eps = float(np.finfo(np.float32).eps)
    for logN in (11, 12, 14):
        N = 1 << logN
        m = np.arange(N // 2)
        tab = np.exp(-2j * np.pi * m / (2 * N)).astype(np.complex64)   # quarter-wave table
        worst = 0.0
        lgNs = 2
        while lgNs + 2 <= logN:
            Ns = 1 << lgNs
            lg = lgNs + 2
            for k in range(0, Ns, max(1, Ns // 256)):
                w1 = tab[k << (logN + 1 - lg)]
                exact1 = np.exp(-2j * np.pi * k / (1 << lg))
                assert abs(complex(w1) - exact1) <= eps   # a table entry: one rounding
                w2 = _cmul32(w1, w1)
                w3 = _cmul32(w2, w1)
                for w, e in ((w2, np.exp(-2j * np.pi * 2 * k / (1 << lg))),
                             (w3, np.exp(-2j * np.pi * 3 * k / (1 << lg)))):
                    worst = max(worst, abs(complex(w) - e))
            lgNs += 2
        assert worst <= 4 * eps, (logN, worst / eps)
