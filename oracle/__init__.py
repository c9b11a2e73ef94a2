"""ctypes bindings to the ORACLE (oracle/liboracle.so, a CPU restatement of the
AREC3D path) and, where it was built, to the reference itself
(oracle/_ref/libarec_ref.so, compiled from its own sources by
oracle/build_ref.sh).

Test infrastructure only: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, never by the product package.

Array conventions are the reference's: cylindrical volumes are [nrays][ny]
(slice fastest), projection stacks are [nangles][ny][nx] (detector fastest),
alignment images are [nz][ny][nx].
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libarec_ref.so")

LIN, KB, SQ = 1, 2, 3
MAX_TRACE = 4096

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")


class Trace(C.Structure):
    _fields_ = [("iterations", C.c_int), ("restarts", C.c_int), ("iterbest", C.c_int),
                ("status", C.c_int), ("lam_final", C.c_float), ("rnorm0", C.c_double),
                ("rel", C.c_double * MAX_TRACE), ("rnorm", C.c_double * MAX_TRACE)]

    def rel_history(self):
        return np.array(self.rel[:min(self.iterations, MAX_TRACE)])

    def rnorm_history(self):
        return np.array(self.rnorm[:min(self.iterations, MAX_TRACE)])


def build():
    """Compile liboracle.so (gcc, seconds)."""
    subprocess.check_call(["make", "-s", "-C", HERE], stdout=subprocess.DEVNULL)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        L.oc_cyl_count.argtypes = [C.c_double, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.oc_cyl_cord.argtypes = [C.c_double, _i32p]
        L.oc_project.argtypes = [C.c_int, C.c_double, C.c_int, _f32p, _f32p, C.c_int, _f32p]
        L.oc_backproject.argtypes = [C.c_int, C.c_double, C.c_int, _f32p, _f32p, C.c_int, _f32p]
        L.oc_sirt.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _f32p, _f32p, C.c_float, C.c_int,
                              C.c_float, _f32p, C.c_int, C.c_int, C.POINTER(Trace)]
        L.oc_cgls.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _f32p, _f32p, C.c_int, C.c_float,
                              _f32p, C.c_int, C.c_double, C.c_int, C.c_int, C.POINTER(Trace)]
        L.oc_cgls_stat.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _f32p, _f32p, C.c_int,
                                   C.c_float, _f32p, C.c_int, C.c_int, C.c_int, C.POINTER(Trace)]
        L.oc_cgls_stat64.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _f64p, _f32p, C.c_int,
                                     C.c_float, _f64p, C.c_int, C.c_int, C.c_int,
                                     C.POINTER(Trace)]
        L.oc_project64.argtypes = [C.c_int, C.c_double, C.c_int, _f64p, _f32p, C.c_int, _f64p]
        L.oc_backproject64.argtypes = [C.c_int, C.c_double, C.c_int, _f64p, _f32p, C.c_int, _f64p]
        L.oc_sirt64.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _f64p, _f32p, C.c_float,
                                C.c_int, C.c_float, _f64p, C.c_int, C.c_int, C.POINTER(Trace)]
        L.oc_cgls64.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _f64p, _f32p, C.c_int,
                                C.c_float, _f64p, C.c_int, C.c_double, C.c_int, C.c_int,
                                C.POINTER(Trace)]
        L.oc_ccorr2d.argtypes = [C.c_int, C.c_int, _f32p, _f32p, _f32p]
        L.oc_quad2dfit.argtypes = [_f32p, C.POINTER(C.c_float), C.POINTER(C.c_float),
                                   C.POINTER(C.c_float)]
        L.oc_speak.argtypes = [C.c_int, C.c_int, _f32p, C.POINTER(C.c_float), C.POINTER(C.c_float),
                               C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.oc_cc_images.argtypes = [C.c_int, C.c_int, C.c_int, _f32p, _f32p, _f32p, _f32p, C.c_int]
        L.oc_set_op_threads.argtypes = [C.c_int]
        L.oc_set_op_threads.restype = None
        _lib = L
    return _lib


def f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def host_threads():
    """Host cores this process may use (the CPU affinity mask, else cpu_count)."""
    try:
        return len(os.sched_getaffinity(0))
    except (AttributeError, OSError):
        return os.cpu_count() or 1


class op_threads:
    """Context manager: threads inside every projector call of the oracle
    (angles split in the forward projector, rays in the back projector; results
    are bit-identical to one thread).  `with op_threads(): ...` uses all host
    cores."""

    def __init__(self, n=None):
        self.n = n or host_threads()

    def __enter__(self):
        lib().oc_set_op_threads(self.n)
        return self

    def __exit__(self, *exc):
        lib().oc_set_op_threads(1)
        return False


# --- geometry ------------------------------------------------------------------------------
def cyl(radius):
    """(nx, nrays, cord[nrays, 2] as (ix, iz)) of arecAllocateCylImage."""
    nx, nr = C.c_int(), C.c_int()
    lib().oc_cyl_count(radius, C.byref(nx), C.byref(nr))
    cord = np.zeros(2 * nr.value, np.int32)
    lib().oc_cyl_cord(radius, cord)
    return nx.value, nr.value, cord.reshape(-1, 2)


# --- projectors -----------------------------------------------------------------------------
def project(weighting, radius, x, angles):
    x = f32(x)
    nx, nr, _ = cyl(radius)
    assert x.shape[0] == nr
    ny = x.shape[1]
    angles = f32(angles)
    q = np.zeros((len(angles), ny, nx), np.float32)
    lib().oc_project(weighting, radius, ny, x, angles, len(angles), q)
    return q


def backproject(weighting, radius, q, angles):
    q = f32(q)
    nx, nr, _ = cyl(radius)
    na, ny, nxq = q.shape
    assert nxq == nx and na == len(angles)
    angles = f32(angles)
    g = np.zeros((nr, ny), np.float32)
    lib().oc_backproject(weighting, radius, ny, q, angles, na, g)
    return g


# --- solvers --------------------------------------------------------------------------------
def sirt(weighting, b, angles, lam=5e-6, maxit=10, tol=1e-3, nthreads=1, verbose=False):
    b = f32(b)
    na, ny, nx = b.shape
    _, nr, _ = cyl(0.5 * (nx - 1))
    x = np.zeros((nr, ny), np.float32)
    tr = Trace()
    lib().oc_sirt(weighting, nx, ny, na, b, f32(angles), lam, maxit, tol, x, nthreads,
                  int(verbose), C.byref(tr))
    return x, tr


def cgls(weighting, b, angles, maxit=10, tol=1e-3, x0=None, rnorm_ref=0.0, nthreads=1,
         verbose=False):
    b = f32(b)
    na, ny, nx = b.shape
    _, nr, _ = cyl(0.5 * (nx - 1))
    x = np.zeros((nr, ny), np.float32) if x0 is None else f32(x0).copy()
    tr = Trace()
    lib().oc_cgls(weighting, nx, ny, na, b, f32(angles), maxit, tol, x, int(x0 is not None),
                  float(rnorm_ref), nthreads, int(verbose), C.byref(tr))
    return x, tr


def cgls_stat(weighting, b, angles, maxit=10, tol=1e-3, x0=None, nthreads=1, verbose=False):
    """cyl_cgls[_KB|_SQ]_stat (statistical weights exp(-b), Tukey taper); odd nx."""
    b = f32(b)
    na, ny, nx = b.shape
    _, nr, _ = cyl(0.5 * (nx - 1))
    x = np.zeros((nr, ny), np.float32) if x0 is None else f32(x0).copy()
    tr = Trace()
    lib().oc_cgls_stat(weighting, nx, ny, na, b, f32(angles), maxit, tol, x, int(x0 is not None),
                       nthreads, int(verbose), C.byref(tr))
    return x, tr


def cgls_stat64(weighting, b, angles, maxit=10, tol=1e-3, x0=None, nthreads=1):
    b = f64(b)
    na, ny, nx = b.shape
    _, nr, _ = cyl(0.5 * (nx - 1))
    x = np.zeros((nr, ny), np.float64) if x0 is None else f64(x0).copy()
    tr = Trace()
    lib().oc_cgls_stat64(weighting, nx, ny, na, b, f32(angles), maxit, tol, x, int(x0 is not None),
                         nthreads, 0, C.byref(tr))
    return x, tr


# --- FP64 oracle: the reference's weights, every sum and update in double ---------------------
def f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def project64(weighting, radius, x, angles):
    x = f64(x)
    nx, nr, _ = cyl(radius)
    angles = f32(angles)
    q = np.zeros((len(angles), x.shape[1], nx), np.float64)
    lib().oc_project64(weighting, radius, x.shape[1], x, angles, len(angles), q)
    return q


def backproject64(weighting, radius, q, angles):
    q = f64(q)
    nx, nr, _ = cyl(radius)
    angles = f32(angles)
    g = np.zeros((nr, q.shape[1]), np.float64)
    lib().oc_backproject64(weighting, radius, q.shape[1], q, angles, len(angles), g)
    return g


def sirt64(weighting, b, angles, lam=5e-6, maxit=10, tol=1e-3, nthreads=1):
    b = f64(b)
    na, ny, nx = b.shape
    _, nr, _ = cyl(0.5 * (nx - 1))
    x = np.zeros((nr, ny), np.float64)
    tr = Trace()
    lib().oc_sirt64(weighting, nx, ny, na, b, f32(angles), lam, maxit, tol, x, nthreads, 0,
                    C.byref(tr))
    return x, tr


def cgls64(weighting, b, angles, maxit=10, tol=1e-3, x0=None, rnorm_ref=0.0, nthreads=1):
    b = f64(b)
    na, ny, nx = b.shape
    _, nr, _ = cyl(0.5 * (nx - 1))
    x = np.zeros((nr, ny), np.float64) if x0 is None else f64(x0).copy()
    tr = Trace()
    lib().oc_cgls64(weighting, nx, ny, na, b, f32(angles), maxit, tol, x, int(x0 is not None),
                    float(rnorm_ref), nthreads, 0, C.byref(tr))
    return x, tr


# --- Fourier shift --------------------------------------------------------------------------
def fshift2d(image, sx, sy):
    """fshift2d (AREC3D/AREC3D/align2dstack.cpp:566-630): the frequencies and
    sx*kx + sy*ky in float, the phase rounded to float, float cosine and sine;
    the transforms in double (the reference uses FFTW in float)."""
    img = np.asarray(image, np.float64)
    ny, nx = img.shape

    def freqs(n):
        h = -(-n // 2)
        return np.array([np.float32(i) / np.float32(n) if i < h else np.float32(i - n) / np.float32(n)
                         for i in range(n)], np.float32)

    kx, ky = freqs(nx), freqs(ny)
    t = (np.float32(sx) * kx[None, :] + np.float32(sy) * ky[:, None]).astype(np.float32)
    phase = (-2.0 * np.pi * t.astype(np.float64)).astype(np.float32)
    cs, sn = np.cos(phase).astype(np.float64), np.sin(phase).astype(np.float64)
    F = np.fft.fft2(img)
    G = (F.real * cs - F.imag * sn) + 1j * (F.real * sn + F.imag * cs)
    return np.fft.ifft2(G).real.astype(np.float32)


# --- cross-correlation ----------------------------------------------------------------------
def ccorr2d(x, y):
    x, y = f32(x), f32(y)
    ny, nx = x.shape
    c = np.zeros_like(x)
    lib().oc_ccorr2d(nx, ny, x, y, c)
    return c


def quad2dfit(z):
    xs, ys, pv = C.c_float(), C.c_float(), C.c_float()
    lib().oc_quad2dfit(f32(z).ravel(), C.byref(xs), C.byref(ys), C.byref(pv))
    return xs.value, ys.value, pv.value


def speak(c):
    c = f32(c)
    ny, nx = c.shape
    xt, yt, ix, iy = C.c_float(), C.c_float(), C.c_int(), C.c_int()
    lib().oc_speak(nx, ny, c, C.byref(xt), C.byref(yt), C.byref(ix), C.byref(iy))
    return xt.value, yt.value, ix.value, iy.value


def cc_images(d1, d2, nthreads=1):
    d1, d2 = f32(d1), f32(d2)
    nz, ny, nx = d1.shape
    sx = np.zeros(nz, np.float32)
    sy = np.zeros(nz, np.float32)
    lib().oc_cc_images(nx, ny, nz, d1, d2, sx, sy, nthreads)
    return sx, sy


# --- the reference itself (only where oracle/build_ref.sh has run) --------------------------
class ArecImage(C.Structure):
    """`arecImage` (AREC3D/AREC3D/arecImage.h:5-18)."""
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("radius", C.c_double),
                ("height", C.c_int), ("nnz", C.c_int), ("nrays", C.c_int),
                ("cord", C.POINTER(C.c_int)), ("is_cyl", C.c_int),
                ("data", C.POINTER(C.c_float))]


def reference_available():
    return os.path.exists(REF_PATH)


class Reference:
    """The reference's own functions, called through its arecImage interface."""

    def __init__(self):
        L = C.CDLL(REF_PATH)
        img = ArecImage
        L._Z20arecAllocateCylImageP5Imagedi.argtypes = [C.POINTER(img), C.c_double, C.c_int]
        self.L = L
        self._sym = {}
        # C++ mangled names of the entry points (g++ Itanium ABI).
        names = {
            "arecProject2D": "_Z13arecProject2D5ImagePfiPS_",
            "arecProject2D_KB": "_Z16arecProject2D_KB5ImagePfiPS_",
            "arecProject2D_SQ": "_Z16arecProject2D_SQ5ImagePfiPS_",
            "arecBackProject2D": "_Z17arecBackProject2D5ImagePfiPS_",
            "arecBackProject2D_KB": "_Z20arecBackProject2D_KB5ImagePfiPS_",
            "arecBackProject2D_SQ": "_Z20arecBackProject2D_SQ5ImagePfiPS_",
            "cyl_sirt": "_Z8cyl_sirti5ImagePfPS_fif",
            "cyl_sirt_KB": "_Z11cyl_sirt_KBi5ImagePfPS_fif",
            "cyl_sirt_SQ": "_Z11cyl_sirt_SQi5ImagePfPS_fif",
            "cyl_cgls": "_Z8cyl_cglsi5ImagePfPS_fif",
            "cyl_cgls_KB": "_Z11cyl_cgls_KBi5ImagePfPS_fif",
            "cyl_cgls_SQ": "_Z11cyl_cgls_SQi5ImagePfPS_fif",
            "cyl_cgls_stat": "_Z13cyl_cgls_stati5ImagePfPS_fif",
            "cyl_cgls_KB_stat": "_Z16cyl_cgls_KB_stati5ImagePfPS_fif",
            "cyl_cgls_SQ_stat": "_Z16cyl_cgls_SQ_stati5ImagePfPS_fif",
            "ccorr2d": "_Z7ccorr2diiPfS_S_",
            "speak": "_Z5speakiiPfS_S_",
            "fshift2d": "_Z8fshift2diiPfS_ff",
            "arecCCImages": "_Z12arecCCImagesi5ImageS_PfS0_",
            "arecRotCCImages": "_Z15arecRotCCImagesi5ImageS_iPf",
            "arecRotateImages": "_Z16arecRotateImagesP5ImagePf",
            "arecRotateImages_skew": "_Z21arecRotateImages_skewP5ImagePf",
            "arecRotateImages_skew_safe": "_Z26arecRotateImages_skew_safeP5ImageS0_Pf",
            "getRadialProfile": "_Z16getRadialProfile5ImageiPfii",
            "findPeak1d": "_Z10findPeak1diPf",
            "shearX_circ": "_Z11shearX_circPffii",
            "shearY_circ": "_Z11shearY_circPffii",
            "rotate2d": "_Z8rotate2diiPfS_f",
            "ncc_filtered": "_Z39getNormalizedCrossCorrelationWithFilterPfS_ii",
        }
        for k, v in names.items():
            self._sym[k] = getattr(L, v)
        for k in ("arecProject2D", "arecProject2D_KB", "arecProject2D_SQ", "arecBackProject2D",
                  "arecBackProject2D_KB", "arecBackProject2D_SQ"):
            self._sym[k].argtypes = [img, C.POINTER(C.c_float), C.c_int, C.POINTER(img)]
            self._sym[k].restype = C.c_int
        for k in ("cyl_sirt", "cyl_sirt_KB", "cyl_sirt_SQ", "cyl_cgls", "cyl_cgls_KB",
                  "cyl_cgls_SQ", "cyl_cgls_stat", "cyl_cgls_KB_stat", "cyl_cgls_SQ_stat"):
            self._sym[k].argtypes = [C.c_int, img, C.POINTER(C.c_float), C.POINTER(img), C.c_float,
                                     C.c_int, C.c_float]
            self._sym[k].restype = C.c_int
        self._sym["ccorr2d"].argtypes = [C.c_int, C.c_int, _f32p, _f32p, _f32p]
        self._sym["speak"].argtypes = [C.c_int, C.c_int, _f32p, C.POINTER(C.c_float),
                                       C.POINTER(C.c_float)]
        self._sym["fshift2d"].argtypes = [C.c_int, C.c_int, _f32p, _f32p, C.c_float, C.c_float]
        self._sym["fshift2d"].restype = None
        self._sym["arecCCImages"].argtypes = [C.c_int, img, img, _f32p, _f32p]
        self._sym["arecCCImages"].restype = C.c_int
        self._sym["arecRotCCImages"].argtypes = [C.c_int, img, img, C.c_int, _f32p]
        self._sym["arecRotCCImages"].restype = C.c_int
        for k in ("arecRotateImages", "arecRotateImages_skew"):
            self._sym[k].argtypes = [C.POINTER(img), _f32p]
            self._sym[k].restype = None
        self._sym["arecRotateImages_skew_safe"].argtypes = [C.POINTER(img), C.POINTER(img), _f32p]
        self._sym["arecRotateImages_skew_safe"].restype = None
        self._sym["getRadialProfile"].argtypes = [img, C.c_int, _f32p, C.c_int, C.c_int]
        self._sym["getRadialProfile"].restype = None
        self._sym["findPeak1d"].argtypes = [C.c_int, _f32p]
        self._sym["findPeak1d"].restype = C.c_float
        for k in ("shearX_circ", "shearY_circ"):
            self._sym[k].argtypes = [_f32p, C.c_float, C.c_int, C.c_int]
            self._sym[k].restype = None
        self._sym["rotate2d"].argtypes = [C.c_int, C.c_int, _f32p, _f32p, C.c_float]
        self._sym["rotate2d"].restype = None
        self._sym["ncc_filtered"].argtypes = [_f32p, _f32p, C.c_int, C.c_int]
        self._sym["ncc_filtered"].restype = C.c_double
        self._keep = []

    # helpers building arecImage views over numpy buffers
    def _cyl(self, radius, ny, data=None):
        """A cylindrical arecImage whose cord table and data are numpy buffers.

        The geometry comes from the reference's own arecAllocateCylImage; the
        table is then copied into a buffer with three zero entries appended,
        because the reference's linear weighting reads two entries past its end
        (arecproject.cpp:75-77): with this buffer those reads return zero
        instead of whatever follows the allocation."""
        tmp = ArecImage()
        self.L._Z20arecAllocateCylImageP5Imagedi(C.byref(tmp), radius, ny)
        nr = tmp.nrays
        cord = np.zeros(2 * nr + 3, np.int32)
        cord[:2 * nr] = np.ctypeslib.as_array(tmp.cord, shape=(2 * nr,))
        buf = np.zeros(max(nr * ny, 1), np.float32)
        if data is not None:
            buf[:nr * ny] = f32(data).ravel()
        self._keep += [cord, buf]
        im = ArecImage()
        im.nx, im.ny, im.nz = tmp.nx, tmp.ny, tmp.nz
        im.radius, im.height, im.nnz, im.nrays, im.is_cyl = radius, ny, nr * ny, nr, 1
        im.cord = cord.ctypes.data_as(C.POINTER(C.c_int))
        im.data = buf.ctypes.data_as(C.POINTER(C.c_float))
        return im

    def _cb(self, arr):
        arr = f32(arr)
        self._keep.append(arr)
        im = ArecImage()
        im.nz, im.ny, im.nx = arr.shape
        im.is_cyl = 0
        im.data = arr.ctypes.data_as(C.POINTER(C.c_float))
        return im

    def project(self, name, radius, x, angles):
        x = f32(x)
        im = self._cyl(radius, x.shape[1], x)
        angles = f32(angles)
        q = np.zeros((len(angles), x.shape[1], im.nx), np.float32)
        out = self._cb(q)
        st = self._sym[name](im, angles.ctypes.data_as(C.POINTER(C.c_float)), len(angles),
                             C.byref(out))
        return q, st

    def backproject(self, name, radius, q, angles):
        q = f32(q)
        im = self._cb(q)
        vol = self._cyl(radius, q.shape[1])
        angles = f32(angles)
        st = self._sym[name](im, angles.ctypes.data_as(C.POINTER(C.c_float)), len(angles),
                             C.byref(vol))
        g = np.ctypeslib.as_array(vol.data, shape=(vol.nrays, q.shape[1])).copy()
        return g, st

    def solve(self, name, b, angles, lam, maxit, tol, x0=None):
        b = f32(b)
        im = self._cb(b)
        angles = f32(angles)
        if x0 is None:
            vol = ArecImage()
            vol.data = C.POINTER(C.c_float)()
        else:
            vol = self._cyl(0.5 * (b.shape[2] - 1), b.shape[1], x0)
        st = self._sym[name](0, im, angles.ctypes.data_as(C.POINTER(C.c_float)), C.byref(vol),
                             lam, maxit, tol)
        x = np.ctypeslib.as_array(vol.data, shape=(vol.nrays, b.shape[1])).copy()
        return x, st

    def fshift2d(self, image, sx, sy):
        a = f32(image).copy()
        out = np.zeros_like(a)
        self._sym["fshift2d"](a.shape[1], a.shape[0], a, out, float(sx), float(sy))
        return out

    # rotational alignment (AREC3D/AREC3D/arecImage.cpp:534-790, imagetools.cpp)
    def rot_cc_images(self, stack1, stack2, r2):
        a, b = self._cb(f32(stack1).copy()), self._cb(f32(stack2).copy())
        ang = np.zeros(len(stack1), np.float32)
        st = self._sym["arecRotCCImages"](0, a, b, r2, ang)
        return ang, st

    def rotate_images(self, stack, angles, kind=""):
        """kind "", "_skew": the stack rotated in place (a copy) and the angles."""
        arr = f32(stack).copy()
        ang = f32(angles).copy()
        im = self._cb(arr)
        self._sym["arecRotateImages" + kind](C.byref(im), ang)
        return arr, ang

    def rotate_images_skew_safe(self, stack, ref, angles):
        arr = f32(stack).copy()
        ang = f32(angles).copy()
        im, rf = self._cb(arr), self._cb(f32(ref).copy())
        self._sym["arecRotateImages_skew_safe"](C.byref(im), C.byref(rf), ang)
        return arr, ang

    def radial_profile(self, img, n, R):
        arr = f32(img)[None].copy()
        out = np.zeros(n, np.float32)
        self._sym["getRadialProfile"](self._cb(arr), 0, out, n, R)
        return out

    def find_peak_1d(self, c):
        c = f32(c).copy()
        return self._sym["findPeak1d"](len(c), c)

    def shear(self, img, shear, axis):
        a = f32(img).copy()
        ny, nx = a.shape
        self._sym["shearX_circ" if axis == "x" else "shearY_circ"](a, float(shear), nx, ny)
        return a

    def rotate2d(self, img, theta):
        a = f32(img).copy()
        ny, nx = a.shape
        out = np.zeros_like(a)
        self._sym["rotate2d"](nx, ny, a, out, float(theta))
        return out

    def ncc_filtered(self, a, b):
        a, b = f32(a).copy(), f32(b).copy()
        ny, nx = a.shape
        return self._sym["ncc_filtered"](a, b, nx, ny)

    # MRC files (AREC3D/AREC3D/arecImageIO.cpp, arecImageIO_mpi.cpp; one rank)
    def write_image(self, fname, stack, merge=""):
        a = f32(stack).copy()
        im = self._cb(a)
        if merge:
            f = getattr(self.L, "_Z20arecWriteImageMerge%siPKc5Image" % merge)
            f.argtypes = [C.c_int, C.c_char_p, ArecImage]
            f.restype = None
            f(0, os.fsencode(fname), im)
            return 0
        f = self.L._Z14arecWriteImagePc5Image
        f.argtypes = [C.c_char_p, ArecImage]
        f.restype = C.c_int
        return f(os.fsencode(fname), im)

    def read_image(self, fname, dist=""):
        im = ArecImage()
        if dist:
            f = getattr(self.L, "_Z20arecReadImageDistby%siPKcP5Image" % dist)
            f.argtypes = [C.c_int, C.c_char_p, C.POINTER(ArecImage)]
            f.restype = None
            f(0, os.fsencode(fname), C.byref(im))
            st = 0
        else:
            f = self.L._Z13arecReadImagePcP5Image
            f.argtypes = [C.c_char_p, C.POINTER(ArecImage)]
            f.restype = C.c_int
            st = f(os.fsencode(fname), C.byref(im))
        a = np.ctypeslib.as_array(im.data, shape=(im.nz, im.ny, im.nx)).copy()
        C.CDLL("libc.so.6").free(C.cast(im.data, C.c_void_p))
        return a, st

    def ccorr2d(self, x, y):
        x, y = f32(x).copy(), f32(y).copy()
        ny, nx = x.shape
        c = np.zeros_like(x)
        self._sym["ccorr2d"](nx, ny, x, y, c)
        return c

    def speak(self, c):
        c = f32(c).copy()
        ny, nx = c.shape
        xt, yt = C.c_float(), C.c_float()
        self._sym["speak"](nx, ny, c, C.byref(xt), C.byref(yt))
        return xt.value, yt.value

    def cc_images(self, d1, d2):
        i1, i2 = self._cb(f32(d1).copy()), self._cb(f32(d2).copy())
        nz = d1.shape[0]
        sx = np.zeros(nz, np.float32)
        sy = np.zeros(nz, np.float32)
        st = self._sym["arecCCImages"](0, i1, i2, sx, sy)
        return sx, sy, st
