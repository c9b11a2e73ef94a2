"""CPU restatement (numpy) of Prealign's vertical profile alignment: the
correlation loops of TubeAlign::profile_gc_img and ::profile_cc_img
(Prealign/Prealign/TubeAlign.cpp:128-223) with ccorr1d and findMaxCC_fit
(TubeAlign_utils.cpp:220-253, 465-479).

Test infrastructure only (the oracle): imported by tests/ and never by the
product package.
"""
import numpy as np


def ccorr1d(x, y):
    """IDFT(conj(DFT x) DFT y), unnormalised; double FFT rounded to float."""
    x = np.asarray(x, np.float64)
    y = np.asarray(y, np.float64)
    n = len(x)
    return (np.fft.irfft(np.conj(np.fft.rfft(x)) * np.fft.rfft(y), n) * n).astype(np.float32)


def _prb1d7(B):
    b1, b2, b3, b4, b5, b6, b7 = (float(v) for v in B)
    c2 = 49. * b1 + 6. * b2 - 21. * b3 - 32. * b4 - 27. * b5 - 6. * b6 + 31. * b7
    c3 = 5. * b1 - 3. * b3 - 4. * b4 - 3. * b5 + 5. * b7
    return c2 / (2. * c3) - 4 if c3 != 0.0 else 0.0


def find_max_cc_fit(c):
    """findMaxCC_fit (TubeAlign_utils.cpp:465-479): first arg max, 7-point fit,
    wrapped: > length / 2 (integer division) moves down by the length."""
    n = len(c)
    m = int(np.argmax(c))
    r = 1.0 * (m + _prb1d7([c[(m + k + n) % n] for k in range(-3, 4)]))
    if r > n // 2:
        r -= n
    return r


def _fit_pair(x, y):
    return find_max_cc_fit(ccorr1d(x, y))


def profile_shifts(profiles, pad, successive=False, fit_pair=_fit_pair):
    """(shifts after mean removal, spread) as the two TubeAlign loops compute
    them; the caller applies sY -= shifts.  fit_pair(x, y) is
    findMaxCC_fit(ccorr1d(x, y)) (replaceable by the reference's own)."""
    p = np.asarray(profiles, np.float32)
    prof_y, prof_x = p.shape
    L = prof_x - 2 * pad
    s = np.zeros(prof_y)
    if not successive:
        mean = np.zeros(prof_x, np.float32)
        for j in range(prof_y):
            mean = mean + p[j] / np.float32(prof_y)
        for j in range(prof_y):
            s[j] = fit_pair(p[j, pad:pad + L], mean[pad:pad + L])
            shift = abs(s[j])
            if shift > 10.0:
                s[j] *= pad
                s[j] /= shift * shift
    else:
        for j in range(1, prof_y):
            s[j] = fit_pair(p[j, pad:pad + L], p[j - 1, pad:pad + L])
        for j in range(1, prof_y):
            s[j] += s[j - 1]
    spread = abs(s.max() - s.min())
    m = 0.0
    for v in s:
        m += v
    m /= prof_y
    return s - m, spread
