"""CPU restatement (numpy) of the reference's preprocessing of the image stack:
arecImageTakeLog and periodicDecomposition.

Test infrastructure only (the oracle): imported by tests/ and never by the
product package.  The FFTs run in double (numpy) and are rounded to float
where the reference's single-precision FFTW returns float.
"""
import math

import numpy as np

PI = math.atan(1.0) * 4  # piFunc(), AREC3D/AREC3D/arecConstants.h:7


_logf = None


def take_log(data):
    """arecImageTakeLog (AREC3D/AREC3D/arecImage.cpp:358-381): -log(v) of the
    float overload (the C library's logf, called here) for v > 0, else 0."""
    global _logf
    if _logf is None:
        import ctypes

        _logf = ctypes.CDLL("libm.so.6").logf
        _logf.argtypes = [ctypes.c_float]
        _logf.restype = ctypes.c_float
    d = np.asarray(data, np.float32)
    out = np.zeros_like(d)
    flat, o = d.ravel(), out.ravel()
    for k in np.flatnonzero(flat > 0):
        o[k] = -np.float32(_logf(float(flat[k])))
    return o.reshape(d.shape)


def make_periodic_slice(img):
    """makePeriodicSlice (AREC3D/AREC3D/imagetools.cpp:17-75): the smooth part S
    of Moisan's periodic-plus-smooth decomposition."""
    d = np.asarray(img, np.float32)
    ny, nx = d.shape
    v = np.zeros_like(d)
    v[0, :] = d[ny - 1, :] - d[0, :]
    v[ny - 1, :] = d[0, :] - d[ny - 1, :]
    v[:, 0] += d[:, nx - 1] - d[:, 0]
    v[:, nx - 1] += d[:, 0] - d[:, nx - 1]
    ff = np.fft.fft2(v.astype(np.float64))
    ff = (ff.real.astype(np.float32) + 1j * ff.imag.astype(np.float32))  # float spectrum
    i = np.arange(nx)[None, :]
    j = np.arange(ny)[:, None]
    D = 2 * np.cos(2.0 * PI * i / nx) + 2 * np.cos(2.0 * PI * j / ny) - 4
    with np.errstate(divide="ignore", invalid="ignore"):
        re = (ff.real.astype(np.float64) / D).astype(np.float32)
        im = (ff.imag.astype(np.float64) / D).astype(np.float32)
    re[0, 0] = 0.0
    im[0, 0] = 0.0
    s = np.fft.ifft2(re.astype(np.float64) + 1j * im.astype(np.float64)) * (nx * ny)
    return (s.real.astype(np.float32) / np.float32(nx * ny)).astype(np.float32)


def periodic_decomposition(stack):
    """periodicDecomposition (AREC3D/AREC3D/imagetools.cpp:77-114):
    d -= exp(-dist^2 / (2 * 5^2)) * S per image, dist = distance to the
    nearest border."""
    out = np.array(stack, np.float32, copy=True)
    nz, ny, nx = out.shape
    ix = np.arange(nx)[None, :]
    iy = np.arange(ny)[:, None]
    dist = 1.0 * np.minimum(np.minimum(ix, np.abs(nx - 1 - ix)),
                            np.minimum(iy, np.abs(ny - 1 - iy)))
    W = np.exp(-1.0 * dist * dist / (2 * 5.0 * 5.0))
    for z in range(nz):
        S = make_periodic_slice(out[z])
        out[z] = (out[z].astype(np.float64) - W * S.astype(np.float64)).astype(np.float32)
    return out
