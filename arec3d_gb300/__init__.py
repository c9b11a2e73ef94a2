"""arec3d_gb300 — GB300 (sm_103a) implementation of the AREC3D reconstruction
path, behind a C ABI (include/arec_gb300.h, include/arec_compat.h).

This module is the Python host-side mirror of that ABI (ctypes):

* ``Plan``: a geometry plan with device-resident projectors and solvers that
  take raw CUDA device pointers (for example ``torch.Tensor.data_ptr()``) in
  the device layouts (volume ``[nrays][ys]``, sinogram ``[nangles][nx][ys]``).
* The reference's own entry points with the reference's argument meaning over
  host numpy arrays: ``arecProject2D[_KB|_SQ]``, ``arecBackProject2D[_KB|_SQ]``,
  ``cyl_sirt[_KB|_SQ]``, ``cyl_cgls[_KB|_SQ]``, ``arecCCImages``, ``ccorr2d``,
  ``speak``, and the data model (``arecAllocateCylImage`` ...).

There is no CPU fallback: importing works anywhere, but every call goes to the
CUDA library and raises ``RuntimeError`` when it is missing.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libarec_gb300.so")

LIN, KB, SQ = 1, 2, 3
ERR_ARG, ERR_NOMEM, ERR_CUDA_BASE = -90, -91, -100


class Problem(C.Structure):
    """`arecgb_problem`: one cylinder of an uneven batch (device buffers)."""
    _fields_ = [("weighting", C.c_int), ("radius", C.c_double), ("ny", C.c_int),
                ("nangles", C.c_int), ("angles", C.POINTER(C.c_float)), ("d_b", C.c_void_p),
                ("d_x", C.c_void_p)]


class SolveInfo(C.Structure):
    _fields_ = [("iterations", C.c_int), ("iterbest", C.c_int), ("restarts", C.c_int),
                ("status", C.c_int), ("lam_final", C.c_float), ("rnorm0", C.c_double),
                ("rel_final", C.c_double)]


class ArecImage(C.Structure):
    """The reference's ``arecImage`` (AREC3D/AREC3D/arecImage.h:5-18)."""
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("radius", C.c_double),
                ("height", C.c_int), ("nnz", C.c_int), ("nrays", C.c_int),
                ("cord", C.POINTER(C.c_int)), ("is_cyl", C.c_int),
                ("data", C.POINTER(C.c_float))]


_lib = None


def build(force=False):
    """Compile libarec_gb300.so (nvcc, sm_103a)."""
    from . import builder

    return builder.build(force=force)


def lib():
    """The loaded CUDA library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libarec_gb300.so is not built (run arec3d_gb300.build()); "
                               "there is no CPU fallback")
        L = C.CDLL(LIB_PATH)
        vp, ip, dp, fp = C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double), C.POINTER(C.c_float)
        L.arecgb_last_error.restype = C.c_char_p
        L.arecgb_plan_create.argtypes = [C.POINTER(vp), C.c_int, C.c_double, C.c_int, C.c_int, fp]
        L.arecgb_plan_destroy.argtypes = [vp]
        L.arecgb_plan_info.argtypes = [vp, ip, ip, ip]
        L.arecgb_plan_check.argtypes = [vp]
        L.arecgb_project.argtypes = [vp, vp, vp, vp, vp]
        L.arecgb_backproject.argtypes = [vp, vp, vp, vp, vp]
        L.arecgb_fbp.argtypes = [vp, vp, vp, vp, vp, vp]
        L.arecgb_ramp_filter.argtypes = [vp, vp, vp, vp]
        L.arecgb_cgls.argtypes = [vp, vp, vp, C.c_int, C.c_int, C.c_float, C.c_double, dp,
                                  C.POINTER(SolveInfo), vp]
        L.arecgb_sirt.argtypes = [vp, vp, vp, C.c_float, C.c_int, C.c_float, dp,
                                  C.POINTER(SolveInfo), vp]
        for n in ("arecgb_sino_from_reference", "arecgb_sino_to_reference"):
            getattr(L, n).argtypes = [vp, vp, C.c_int, C.c_int, C.c_int, C.c_int, vp]
        L.arecgb_cc_shifts.argtypes = [vp, vp, C.c_int, C.c_int, C.c_int, vp, vp, vp, vp, vp]
        L.arecgb_ccorr2d_device.argtypes = [vp, vp, vp, C.c_int, C.c_int, vp]
        L.arecgb_fshift2d_device.argtypes = [vp, vp, C.c_int, C.c_int, C.c_int, vp, vp, vp]
        L.arecgb_fshift2d.argtypes = [C.c_int, C.c_int, fp, fp, C.c_float, C.c_float]
        L.arecgb_fshift2d.restype = None
        L.arecgb_rot_cc_images.argtypes = [vp, vp, C.c_int, C.c_int, C.c_int, C.c_int, vp, vp]
        L.arecgb_rotate_images.argtypes = [vp, C.c_int, C.c_int, C.c_int, vp, vp]
        L.arecgb_rotate_images_skew.argtypes = [vp, C.c_int, C.c_int, C.c_int, vp, vp]
        L.arecgb_rotate_images_skew_safe.argtypes = [vp, vp, C.c_int, C.c_int, C.c_int, vp,
                                                     C.POINTER(C.c_int), C.POINTER(C.c_double), vp]
        L.arecgb_ncc_filtered.argtypes = [vp, vp, C.c_int, C.c_int, C.c_int, vp, vp]
        L.arecgb_take_log.argtypes = [vp, C.c_size_t, vp]
        L.arecgb_plan_shapes.argtypes = [vp, ip, ip, ip, ip]
        L.arecgb_plan_set_shapes.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_int]
        L.arecgb_plan_table_bytes.argtypes = [vp]
        L.arecgb_plan_table_bytes.restype = C.c_longlong
        L.arecgb_profile_shifts.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_int, dp, dp, vp]
        L.arecgb_periodic_decomposition.argtypes = [vp, C.c_int, C.c_int, C.c_int, vp, vp]
        ip_ = C.POINTER(C.c_int)
        L.arecgb_mrc_read_header.argtypes = [C.c_char_p, ip_, ip_, ip_, ip_]
        L.arecgb_mrc_read_device.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int, vp,
                                             C.c_size_t, ip_, ip_, ip_, vp]
        L.arecgb_mrc_write_device.argtypes = [C.c_char_p, vp, C.c_int, C.c_int, C.c_int, vp]
        L.arecgb_cc_shifts_static.argtypes = [vp, vp, C.c_int, C.c_int, C.c_int, vp, vp, vp, vp,
                                              vp]
        img, pimg = ArecImage, C.POINTER(ArecImage)
        for n in ("arecProject2D", "arecProject2D_KB", "arecProject2D_SQ", "arecBackProject2D",
                  "arecBackProject2D_KB", "arecBackProject2D_SQ"):
            f = getattr(L, "arecgb_" + n)
            f.argtypes = [img, fp, C.c_int, pimg]
            f.restype = C.c_int
        for n in ("cyl_sirt", "cyl_sirt_KB", "cyl_sirt_SQ", "cyl_cgls", "cyl_cgls_KB",
                  "cyl_cgls_SQ", "cyl_cgls_stat", "cyl_cgls_KB_stat", "cyl_cgls_SQ_stat"):
            f = getattr(L, "arecgb_" + n)
            f.argtypes = [C.c_int, img, fp, pimg, C.c_float, C.c_int, C.c_float]
            f.restype = C.c_int
        L.arecgb_arecCCImages.argtypes = [C.c_int, img, img, fp, fp]
        L.arecgb_arecRotCCImages.argtypes = [C.c_int, img, img, C.c_int, fp]
        for n in ("arecgb_arecImageTakeLog", "arecgb_periodicDecomposition"):
            getattr(L, n).argtypes = [img]
            getattr(L, n).restype = None
        L.arecgb_makePeriodicSlice.argtypes = [C.c_int, C.c_int, fp, fp]
        L.arecgb_makePeriodicSlice.restype = None
        L.arecgb_arecReadImageHeader.argtypes = [C.c_char_p, ip, ip, ip]
        L.arecgb_arecReadImage.argtypes = [C.c_char_p, pimg]
        L.arecgb_arecWriteImage.argtypes = [C.c_char_p, img]
        for n in ("arecgb_arecReadImageDistbyZ", "arecgb_arecReadImageDistbyY"):
            getattr(L, n).argtypes = [C.c_int, C.c_char_p, pimg]
            getattr(L, n).restype = None
        for n in ("arecgb_arecWriteImageMergeY", "arecgb_arecWriteImageMergeZ"):
            getattr(L, n).argtypes = [C.c_int, C.c_char_p, img]
            getattr(L, n).restype = None
        for n in ("arecgb_arecRotateImages", "arecgb_arecRotateImages_skew"):
            getattr(L, n).argtypes = [pimg, fp]
            getattr(L, n).restype = None
        L.arecgb_arecRotateImages_skew_safe.argtypes = [pimg, pimg, fp]
        L.arecgb_arecRotateImages_skew_safe.restype = None
        L.arecgb_ccorr2d.argtypes = [C.c_int, C.c_int, fp, fp, fp]
        L.arecgb_ccorr2d.restype = None
        L.arecgb_speak.argtypes = [C.c_int, C.c_int, fp, fp, fp]
        L.arecgb_speak.restype = None
        L.arecgb_arecAllocateCylImage.argtypes = [pimg, C.c_double, C.c_int]
        L.arecgb_arecAllocateCBImage.argtypes = [pimg, C.c_int, C.c_int, C.c_int]
        L.arecgb_arecImageFree.argtypes = [pimg]
        L.arecgb_arecImageFree.restype = None
        L.arecgb_ImageCyl2CB.argtypes = [img, img, C.c_int, C.c_int, C.c_int]
        L.arecgb_ImageCB2Cyl.argtypes = [img, img, C.c_int, C.c_int, C.c_double, C.c_int]
        L.arecgb_reset.argtypes = [pimg]
        L.arecgb_reset.restype = None
        L.arecgb_soft_noneg.argtypes = [pimg]
        L.arecgb_soft_noneg.restype = None
        L.arecgb_last_trace.argtypes = [dp, C.c_int, C.POINTER(SolveInfo)]
        L.arecgb_conv3x3_bf16.argtypes = [vp] * 4 + [C.c_int] * 7 + [vp, vp]
        L.arecgb_unet_create.argtypes = [C.POINTER(vp), C.c_int, C.c_int, C.c_int, C.c_int,
                                         C.c_ulonglong]
        L.arecgb_unet_destroy.argtypes = [vp]
        L.arecgb_unet_num_params.argtypes = [vp]
        L.arecgb_unet_num_params.restype = C.c_longlong
        lp = C.POINTER(C.c_longlong)
        L.arecgb_unet_layer_offsets.argtypes = [vp, lp, lp, ip, ip]
        L.arecgb_unet_get_params.argtypes = [vp, vp, vp]
        L.arecgb_unet_set_params.argtypes = [vp, vp, vp]
        L.arecgb_unet_forward.argtypes = [vp, vp, vp, C.c_int, vp]
        L.arecgb_unet_backward.argtypes = [vp, vp, vp, vp]
        L.arecgb_unet_train_step.argtypes = [vp, vp, vp, C.c_int, C.c_float, C.c_float, dp, vp]
        for n in ("arecgb_unet_images_from_volume", "arecgb_unet_images_to_volume"):
            getattr(L, n).argtypes = [vp, vp, vp, C.c_int, C.c_int, C.c_int, C.c_float, vp]
        L.arecgb_warm_start.argtypes = [vp, vp, vp, vp, vp, vp, vp]
        L.arecgb_unet_shape.argtypes = [vp, ip, ip, ip]
        L.arecgb_unet_set_loss.argtypes = [vp, C.c_int, C.c_float]
        L.arecgb_cylinder_info.argtypes = [C.c_double, C.c_int, ip, ip, ip]
        L.arecgb_solve_uneven.argtypes = [C.POINTER(Problem), C.c_int, C.c_size_t,
                                          C.POINTER(vp), C.c_int, C.c_int, C.c_double, C.c_int,
                                          C.c_float, C.POINTER(SolveInfo), ip, vp]
        L.arecgb_reconstruct_host.argtypes = [vp, vp, vp, vp, C.c_int, C.c_float, C.c_int,
                                              C.c_float, C.POINTER(SolveInfo), vp]
        L.arecgb_plan_timing.argtypes = [vp, C.c_int, dp, C.POINTER(C.c_longlong), dp,
                                         C.POINTER(C.c_longlong)]
        L.arecgb_launch_count.restype = C.c_longlong
        L.arecgb_plan_autotune.argtypes = [vp, vp, vp, ip, ip, vp]
        L.arecgb_cgls_stat.argtypes = [vp, vp, vp, C.c_int, C.c_int, C.c_float, dp,
                                       C.POINTER(SolveInfo), vp]
        L.arecgb_cgls_batch.argtypes = [C.POINTER(vp), C.POINTER(vp), C.POINTER(vp),
                                        C.POINTER(C.c_int), C.c_int, C.c_int, C.c_float, dp,
                                        C.POINTER(SolveInfo), vp]
        _lib = L
    return _lib


def last_error():
    return lib().arecgb_last_error().decode()


def _check(rc, what):
    if rc != 0:
        raise RuntimeError("%s failed (status %d): %s" % (what, rc, last_error()))


def _ptr(t):
    """Device pointer of a torch tensor, or an int pointer as given."""
    if t is None:
        return None
    if isinstance(t, int):
        return t
    return t.data_ptr()


def _stream(s):
    if s is None:
        return None
    if isinstance(s, int):
        return s
    return s.cuda_stream


# ---------------------------------------------------------------------------------------------
class Plan:
    """Geometry plan of one cylinder (radius, ny slices, float radian angles)."""

    def __init__(self, weighting, radius, ny, angles):
        self.weighting = int(weighting)
        self.radius = float(radius)
        self.ny = int(ny)
        self.angles = np.ascontiguousarray(angles, dtype=np.float32)
        h = C.c_void_p()
        rc = lib().arecgb_plan_create(C.byref(h), self.weighting, self.radius, self.ny,
                                      len(self.angles),
                                      self.angles.ctypes.data_as(C.POINTER(C.c_float)))
        _check(rc, "arecgb_plan_create")
        self._h = h
        nx, nr, ys = C.c_int(), C.c_int(), C.c_int()
        lib().arecgb_plan_info(h, C.byref(nx), C.byref(nr), C.byref(ys))
        self.nx, self.nrays, self.ys = nx.value, nr.value, ys.value
        self.nangles = len(self.angles)

    def close(self):
        if getattr(self, "_h", None):
            lib().arecgb_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self):
        """Device-side consistency flag since the last check (0 = fine); clears it."""
        return lib().arecgb_plan_check(self._h)

    @property
    def vol_shape(self):
        return (self.nrays, self.ys)

    @property
    def sino_shape(self):
        return (self.nangles, self.nx, self.ys)

    def project(self, x, q, norm2=None, stream=None):
        _check(lib().arecgb_project(self._h, _ptr(x), _ptr(q), _ptr(norm2), _stream(stream)),
               "arecgb_project")

    def backproject(self, s, g, norm2=None, stream=None):
        _check(lib().arecgb_backproject(self._h, _ptr(s), _ptr(g), _ptr(norm2), _stream(stream)),
               "arecgb_backproject")

    def fbp(self, b, x, work, atb_norm2=None, stream=None):
        """x = (pi / nangles) A^T (ramp * b); work receives the filtered
        sinogram; atb_norm2 (device double), if given, ||A^T b||^2."""
        _check(lib().arecgb_fbp(self._h, _ptr(b), _ptr(x), _ptr(work), _ptr(atb_norm2),
                                _stream(stream)), "arecgb_fbp")

    def ramp_filter(self, s, f, stream=None):
        _check(lib().arecgb_ramp_filter(self._h, _ptr(s), _ptr(f), _stream(stream)),
               "arecgb_ramp_filter")

    def cgls(self, b, x, maxit, tol, warm=False, rnorm_ref=0.0, stream=None):
        hist = np.zeros(max(maxit, 1), np.float64)
        info = SolveInfo()
        rc = lib().arecgb_cgls(self._h, _ptr(b), _ptr(x), int(bool(warm)), int(maxit), float(tol),
                               float(rnorm_ref), hist.ctypes.data_as(C.POINTER(C.c_double)),
                               C.byref(info), _stream(stream))
        _check(rc, "arecgb_cgls")
        return hist[:info.iterations].copy(), info

    def cgls_stat(self, b, x, maxit, tol, warm=False, stream=None):
        """Statistically weighted CGLS (weights from b)."""
        hist = np.zeros(max(maxit, 1), np.float64)
        info = SolveInfo()
        rc = lib().arecgb_cgls_stat(self._h, _ptr(b), _ptr(x), int(bool(warm)), int(maxit),
                                    float(tol), hist.ctypes.data_as(C.POINTER(C.c_double)),
                                    C.byref(info), _stream(stream))
        _check(rc, "arecgb_cgls_stat")
        return hist[:info.iterations].copy(), info

    def sirt(self, b, x, lam, maxit, tol, stream=None):
        hist = np.zeros(max(maxit, 1), np.float64)
        info = SolveInfo()
        rc = lib().arecgb_sirt(self._h, _ptr(b), _ptr(x), float(lam), int(maxit), float(tol),
                               hist.ctypes.data_as(C.POINTER(C.c_double)), C.byref(info),
                               _stream(stream))
        _check(rc, "arecgb_sirt")
        return hist[:min(info.iterations, maxit)].copy(), info

    def autotune(self, x, q, stream=None):
        """Choose launch shapes by timing (overwrites x and q); returns
        (forward band height, back-projection slice chunks per block)."""
        band, nsc = C.c_int(), C.c_int()
        _check(lib().arecgb_plan_autotune(self._h, _ptr(x), _ptr(q), C.byref(band), C.byref(nsc),
                                          _stream(stream)), "arecgb_plan_autotune")
        return band.value, nsc.value

    def set_shapes(self, fp_band, fp_vec, bp_vec, bp_nsc):
        """Launch shapes as (forward band, forward VEC, back VEC, chunks)."""
        _check(lib().arecgb_plan_set_shapes(self._h, fp_band, fp_vec, bp_vec, bp_nsc),
               "arecgb_plan_set_shapes")

    def table_bytes(self):
        """Device bytes of the plan's projector tables (0: none)."""
        return lib().arecgb_plan_table_bytes(self._h)

    def shapes(self):
        """(forward band height, forward VEC, back-projection VEC, slice chunks
        per block)."""
        band, fvec, vec, nsc = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        _check(lib().arecgb_plan_shapes(self._h, C.byref(band), C.byref(fvec), C.byref(vec),
                                        C.byref(nsc)), "arecgb_plan_shapes")
        return band.value, fvec.value, vec.value, nsc.value

    def timing(self, mode):
        """Projector timing (mode 1 start, 2 report, 0 report and stop):
        (fp_ms, fp_calls, bp_ms, bp_calls)."""
        fm, bm = C.c_double(), C.c_double()
        fc, bc = C.c_longlong(), C.c_longlong()
        _check(lib().arecgb_plan_timing(self._h, mode, C.byref(fm), C.byref(fc), C.byref(bm),
                                        C.byref(bc)), "arecgb_plan_timing")
        return fm.value, fc.value, bm.value, bc.value

    def sino_from_reference(self, ref, dev, stream=None):
        _check(lib().arecgb_sino_from_reference(_ptr(ref), _ptr(dev), self.nangles, self.ny,
                                                self.nx, self.ys, _stream(stream)),
               "arecgb_sino_from_reference")

    def sino_to_reference(self, dev, ref, stream=None):
        _check(lib().arecgb_sino_to_reference(_ptr(dev), _ptr(ref), self.nangles, self.ny,
                                              self.nx, self.ys, _stream(stream)),
               "arecgb_sino_to_reference")

    def reconstruct_host(self, b_host, x_host, net=None, sirt_iters=0, sirt_lam=0.0,
                         maxit=200, tol=1e-3, stream=None):
        """One reconstruction over host buffers in the reference's layouts
        (arecgb_reconstruct_host): b_host [nangles][ny][nx] and x_host
        [nrays][ny] float32, as pointers or CPU tensors / arrays (page-locked
        memory copies at full speed).  With `net`: the network's input (SIRT
        of sirt_iters iterations, or the filtered back projection when
        sirt_iters is 0) -> warm start -> CGLS; without: CGLS from zero.
        Returns the CGLS SolveInfo."""
        def hp(a):
            if isinstance(a, int):
                return a
            if hasattr(a, "data_ptr"):
                return a.data_ptr()
            return a.ctypes.data
        info = SolveInfo()
        _check(lib().arecgb_reconstruct_host(self._h, hp(b_host), hp(x_host),
                                             net._h if net is not None else None,
                                             int(sirt_iters), float(sirt_lam), int(maxit),
                                             float(tol), C.byref(info), _stream(stream)),
               "arecgb_reconstruct_host")
        return info


class UNet:
    """Learned warm start network (BF16 4-level U-Net, 32 base channels) on
    square images [n][size][size] (size a multiple of 8)."""

    LAYERS = ("c1a", "c1b", "c2a", "c2b", "c3a", "c3b", "c4a", "c4b", "u3", "d3a", "d3b",
              "u2", "d2a", "d2b", "u1", "d1a", "d1b", "out")

    def __init__(self, size, max_batch, train=False, seed=0):
        h = C.c_void_p()
        _check(lib().arecgb_unet_create(C.byref(h), size, size, max_batch, int(train), seed),
               "arecgb_unet_create")
        self._h, self.size, self.max_batch, self.train = h, size, max_batch, train
        self.nparams = int(lib().arecgb_unet_num_params(h))
        n = len(self.LAYERS)
        wo, bo = (C.c_longlong * n)(), (C.c_longlong * n)()
        ci, co = (C.c_int * n)(), (C.c_int * n)()
        lib().arecgb_unet_layer_offsets(h, wo, bo, ci, co)
        self.layers = [dict(name=self.LAYERS[i], w_off=wo[i], b_off=bo[i], cin=ci[i],
                            cout=co[i]) for i in range(n)]

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().arecgb_unet_destroy(h)
            self._h = None

    def get_params(self, out, stream=None):
        _check(lib().arecgb_unet_get_params(self._h, _ptr(out), _stream(stream)),
               "arecgb_unet_get_params")

    def set_params(self, params, stream=None):
        _check(lib().arecgb_unet_set_params(self._h, _ptr(params), _stream(stream)),
               "arecgb_unet_set_params")

    def forward(self, x, y, stream=None):
        _check(lib().arecgb_unet_forward(self._h, _ptr(x), _ptr(y), x.shape[0], _stream(stream)),
               "arecgb_unet_forward")

    def backward(self, dout, grads=None, stream=None):
        _check(lib().arecgb_unet_backward(self._h, _ptr(dout), _ptr(grads), _stream(stream)),
               "arecgb_unet_backward")

    def set_loss(self, levels=0, ratio=1.0):
        """Training loss: MSE (levels 0), or MSE plus ratio^s-weighted mean
        squares of the error pooled over 2^s blocks, s = 1..levels."""
        _check(lib().arecgb_unet_set_loss(self._h, int(levels), float(ratio)),
               "arecgb_unet_set_loss")

    def train_step(self, x, target, lr, weight_decay=0.0, stream=None):
        loss = C.c_double()
        _check(lib().arecgb_unet_train_step(self._h, _ptr(x), _ptr(target), x.shape[0], lr,
                                            weight_decay, C.byref(loss), _stream(stream)),
               "arecgb_unet_train_step")
        return loss.value

    def warm_start(self, plan, x_early, x0, img_in, img_out, stream=None):
        _check(lib().arecgb_warm_start(plan._h, self._h, _ptr(x_early), _ptr(x0), _ptr(img_in),
                                       _ptr(img_out), _stream(stream)), "arecgb_warm_start")


def images_from_volume(plan, vol, img, npad, y0, count, scale=1.0, stream=None):
    _check(lib().arecgb_unet_images_from_volume(plan._h, _ptr(vol), _ptr(img), npad, y0, count,
                                                scale, _stream(stream)),
           "arecgb_unet_images_from_volume")


def images_to_volume(plan, img, vol, npad, y0, count, scale=1.0, stream=None):
    _check(lib().arecgb_unet_images_to_volume(plan._h, _ptr(img), _ptr(vol), npad, y0, count,
                                              scale, _stream(stream)),
           "arecgb_unet_images_to_volume")


def cgls_batch(plans, bs, xs, maxit, tol, warm=None, rnorm_ref=None, stream=None):
    """CGLS over several problems at once (one plan each): lists of plans,
    device sinograms and volumes.  Returns the list of SolveInfo."""
    n = len(plans)
    hp = (C.c_void_p * n)(*[p._h.value for p in plans])
    hb = (C.c_void_p * n)(*[b.data_ptr() for b in bs])
    hx = (C.c_void_p * n)(*[x.data_ptr() for x in xs])
    w = (C.c_int * n)(*([int(bool(v)) for v in warm] if warm else [0] * n))
    rr = (C.c_double * n)(*(rnorm_ref if rnorm_ref else [0.0] * n))
    info = (SolveInfo * n)()
    _check(lib().arecgb_cgls_batch(hp, hb, hx, w, n, maxit, tol, rr, info, _stream(stream)),
           "arecgb_cgls_batch")
    return list(info)


def cylinder_info(radius, ny):
    """(nx, nrays, ys) of the reference's cylinder of this radius with ny slices."""
    nx, nr, ys = C.c_int(), C.c_int(), C.c_int()
    _check(lib().arecgb_cylinder_info(float(radius), int(ny), C.byref(nx), C.byref(nr),
                                      C.byref(ys)), "arecgb_cylinder_info")
    return nx.value, nr.value, ys.value


def solve_uneven(problems, budget_bytes, maxit=200, tol=1e-3, nets=None, stream=None):
    """Uneven batch (arecgb_solve_uneven).  problems: list of dicts with
    weighting, radius, ny, angles (float32 array), b and x (device tensors in
    the device layouts); nets: warm-start networks (the same parameters at
    several image sizes) or None.  Returns (list of SolveInfo, list of wave
    indices)."""
    nets = list(nets or [])
    n = len(problems)
    arr = (Problem * n)()
    keep = []
    for i, p in enumerate(problems):
        ang = np.ascontiguousarray(p["angles"], dtype=np.float32)
        keep.append(ang)
        arr[i] = Problem(int(p.get("weighting", SQ)), float(p["radius"]), int(p["ny"]), len(ang),
                         ang.ctypes.data_as(C.POINTER(C.c_float)), _ptr(p["b"]), _ptr(p["x"]))
    info = (SolveInfo * n)()
    waves = (C.c_int * n)()
    hn = (C.c_void_p * max(1, len(nets)))(*[nt._h.value for nt in nets])
    sirt_iters = getattr(nets[0], "sirt_iters", 0) if nets else 0
    lam_scale = getattr(nets[0], "sirt_lam_scale", 1.0) if nets else 1.0
    _check(lib().arecgb_solve_uneven(arr, n, int(budget_bytes), hn, len(nets), int(sirt_iters),
                                     float(lam_scale), int(maxit), float(tol), info, waves,
                                     _stream(stream)), "arecgb_solve_uneven")
    return list(info), list(waves)


def launch_count():
    """Kernel launches issued by the library so far."""
    return int(lib().arecgb_launch_count())


def cc_shifts(img1, img2, sx, sy, ix=None, iy=None, stream=None):
    """Shift search over device image stacks [nz][ny][nx] (torch tensors)."""
    nz, ny, nx = img1.shape
    _check(lib().arecgb_cc_shifts(_ptr(img1), _ptr(img2), nz, ny, nx, _ptr(sx), _ptr(sy),
                                  _ptr(ix), _ptr(iy), _stream(stream)), "arecgb_cc_shifts")


def cc_shifts_static(img1, img2, sx, sy, ix=None, iy=None, stream=None):
    """Shift search that allocates nothing (static 3.5 MiB scratch per device;
    nx, ny powers of two in [16, 512], nz*ny*nx <= 262144).  The scratch is
    shared: do not let two calls overlap."""
    nz, ny, nx = img1.shape
    _check(lib().arecgb_cc_shifts_static(_ptr(img1), _ptr(img2), nz, ny, nx, _ptr(sx),
                                         _ptr(sy), _ptr(ix), _ptr(iy), _stream(stream)),
           "arecgb_cc_shifts_static")


def fshift2d_device(images, out, sx, sy, stream=None):
    """Fourier shift of device image stacks [nz][ny][nx] by per-image (sx, sy)."""
    nz, ny, nx = images.shape
    _check(lib().arecgb_fshift2d_device(_ptr(images), _ptr(out), nz, ny, nx, _ptr(sx), _ptr(sy),
                                        _stream(stream)), "arecgb_fshift2d_device")


def fshift2d(image, sx, sy):
    """The reference's fshift2d on one host image [ny][nx]."""
    a = np.ascontiguousarray(image, dtype=np.float32)
    out = np.zeros_like(a)
    lib().arecgb_fshift2d(a.shape[1], a.shape[0], _f32p(a), _f32p(out), float(sx), float(sy))
    return out


def rot_cc_images(images1, images2, r2, angles, stream=None):
    """Rotation (degrees) of each device image of images2 against images1
    (arecRotCCImages) into the device vector angles."""
    nz, ny, nx = images1.shape
    _check(lib().arecgb_rot_cc_images(_ptr(images1), _ptr(images2), nz, ny, nx, int(r2),
                                      _ptr(angles), _stream(stream)), "arecgb_rot_cc_images")


def rotate_images(images, angles, stream=None):
    """Bilinear rotation of a device stack in place (arecRotateImages)."""
    nz, ny, nx = images.shape
    _check(lib().arecgb_rotate_images(_ptr(images), nz, ny, nx, _ptr(angles), _stream(stream)),
           "arecgb_rotate_images")


def rotate_images_skew(images, angles, stream=None):
    """Shear rotation of a device stack in place; angles updated
    (arecRotateImages_skew)."""
    nz, ny, nx = images.shape
    _check(lib().arecgb_rotate_images_skew(_ptr(images), nz, ny, nx, _ptr(angles),
                                           _stream(stream)), "arecgb_rotate_images_skew")


def rotate_images_skew_safe(images, ref, angles, stream=None):
    """Guarded shear rotation of a device stack against ref, in place; returns
    (slices rotated, mean kept correlation) (arecRotateImages_skew_safe)."""
    nz, ny, nx = images.shape
    n_rot, mean_cc = C.c_int(), C.c_double()
    _check(lib().arecgb_rotate_images_skew_safe(_ptr(images), _ptr(ref), nz, ny, nx, _ptr(angles),
                                                C.byref(n_rot), C.byref(mean_cc),
                                                _stream(stream)), "arecgb_rotate_images_skew_safe")
    return n_rot.value, mean_cc.value


def ncc_filtered(a, b, cc, stream=None):
    """Tukey-filtered normalised cross-correlation per device image pair into
    the float64 device vector cc."""
    nz, ny, nx = a.shape
    _check(lib().arecgb_ncc_filtered(_ptr(a), _ptr(b), nz, ny, nx, _ptr(cc), _stream(stream)),
           "arecgb_ncc_filtered")


def profile_shifts(profiles, pad, successive=False, stream=None):
    """(shifts, spread) of Prealign's profile alignment over a CUDA tensor of
    profiles [prof_y][prof_x]; the caller applies sY -= shifts."""
    prof_y, prof_x = profiles.shape
    out = np.zeros(prof_y, np.float64)
    spread = C.c_double()
    _check(lib().arecgb_profile_shifts(_ptr(profiles), prof_y, prof_x, int(pad), int(successive),
                                       out.ctypes.data_as(C.POINTER(C.c_double)),
                                       C.byref(spread), _stream(stream)), "arecgb_profile_shifts")
    return out, spread.value


def take_log(data, stream=None):
    """-log(v) for v > 0, else 0, in place on a float32 CUDA tensor."""
    _check(lib().arecgb_take_log(_ptr(data), data.numel(), _stream(stream)), "arecgb_take_log")


def periodic_decomposition(images, smooth=None, stream=None):
    """Periodic-plus-smooth decomposition of a CUDA stack [nz][ny][nx] in place
    (or, with `smooth`, its smooth parts written there and the images left)."""
    nz, ny, nx = images.shape
    _check(lib().arecgb_periodic_decomposition(_ptr(images), nz, ny, nx,
                                               _ptr(smooth) if smooth is not None else None,
                                               _stream(stream)), "arecgb_periodic_decomposition")


def mrc_read_header(fname):
    """(nx, ny, nz, mode) of an MRC file."""
    v = [C.c_int() for _ in range(4)]
    _check(lib().arecgb_mrc_read_header(os.fsencode(fname), *[C.byref(x) for x in v]),
           "arecgb_mrc_read_header")
    return tuple(x.value for x in v)


def mrc_read_device(fname, rank=0, nranks=1, by_y=False, stream=None):
    """This rank's part of an MRC stack as a float32 CUDA tensor [nz][ny][nx]
    (by_y: the reference's distribution by rows, else by images)."""
    import torch

    nx, nyl, nzl = C.c_int(), C.c_int(), C.c_int()
    L = lib()
    _check(L.arecgb_mrc_read_device(os.fsencode(fname), rank, nranks, int(by_y), None, 0,
                                    C.byref(nx), C.byref(nyl), C.byref(nzl), None),
           "arecgb_mrc_read_device")
    out = torch.empty(nzl.value, nyl.value, nx.value, dtype=torch.float32, device="cuda")
    _check(L.arecgb_mrc_read_device(os.fsencode(fname), rank, nranks, int(by_y), _ptr(out),
                                    out.numel(), C.byref(nx), C.byref(nyl), C.byref(nzl),
                                    _stream(stream)), "arecgb_mrc_read_device")
    return out


def mrc_write_device(fname, images, stream=None):
    """Write a float32 CUDA tensor [nz][ny][nx] as a mode-2 MRC file."""
    nz, ny, nx = images.shape
    _check(lib().arecgb_mrc_write_device(os.fsencode(fname), _ptr(images), nz, ny, nx,
                                         _stream(stream)), "arecgb_mrc_write_device")


def ccorr2d_device(x, y, c, stream=None):
    ny, nx = x.shape
    _check(lib().arecgb_ccorr2d_device(_ptr(x), _ptr(y), _ptr(c), ny, nx, _stream(stream)),
           "arecgb_ccorr2d_device")


# ---------------------------------------------------------------------------------------------
# The reference's entry points over host arrays (reference layouts).
def _f32p(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _cb_image(arr):
    """arecImage view of a C-contiguous float32 [nz][ny][nx] array (caller keeps it alive)."""
    im = ArecImage()
    im.nz, im.ny, im.nx = arr.shape
    im.is_cyl = 0
    im.data = _f32p(arr)
    return im


def arecAllocateCylImage(radius, height):
    """arecImage allocated by the library (free with arecImageFree)."""
    im = ArecImage()
    _check(lib().arecgb_arecAllocateCylImage(C.byref(im), float(radius), int(height)),
           "arecAllocateCylImage")
    return im


def arecImageFree(im):
    lib().arecgb_arecImageFree(C.byref(im))


def cyl_data(im):
    """numpy view [nrays][ny] of a cylindrical arecImage's data."""
    return np.ctypeslib.as_array(im.data, shape=(im.nrays, im.ny))


def cyl_cord(im):
    return np.ctypeslib.as_array(im.cord, shape=(im.nrays, 2))


def _project(name, radius, x, angles):
    x = np.ascontiguousarray(x, dtype=np.float32)
    angles = np.ascontiguousarray(angles, dtype=np.float32)
    cyl = arecAllocateCylImage(radius, x.shape[1])
    try:
        if cyl.nrays != x.shape[0]:
            raise ValueError("x has %d rays, the cylinder %d" % (x.shape[0], cyl.nrays))
        cyl_data(cyl)[:] = x
        q = np.zeros((len(angles), x.shape[1], cyl.nx), np.float32)
        out = _cb_image(q)
        st = getattr(lib(), "arecgb_" + name)(cyl, _f32p(angles), len(angles), C.byref(out))
    finally:
        arecImageFree(cyl)
    return q, st


def _backproject(name, radius, q, angles):
    q = np.ascontiguousarray(q, dtype=np.float32)
    angles = np.ascontiguousarray(angles, dtype=np.float32)
    img = _cb_image(q)
    vol = arecAllocateCylImage(radius, q.shape[1])
    try:
        st = getattr(lib(), "arecgb_" + name)(img, _f32p(angles), len(angles), C.byref(vol))
        g = cyl_data(vol).copy()
    finally:
        arecImageFree(vol)
    return g, st


def arecProject2D(radius, x, angles):
    """(q[nangles][ny][nx], status) for volume x[nrays][ny] (pmethod=1)."""
    return _project("arecProject2D", radius, x, angles)


def arecProject2D_KB(radius, x, angles):
    return _project("arecProject2D_KB", radius, x, angles)


def arecProject2D_SQ(radius, x, angles):
    return _project("arecProject2D_SQ", radius, x, angles)


def arecBackProject2D(radius, q, angles):
    return _backproject("arecBackProject2D", radius, q, angles)


def arecBackProject2D_KB(radius, q, angles):
    return _backproject("arecBackProject2D_KB", radius, q, angles)


def arecBackProject2D_SQ(radius, q, angles):
    return _backproject("arecBackProject2D_SQ", radius, q, angles)


def _solve(name, b, angles, lam, maxit, tol, x0=None):
    b = np.ascontiguousarray(b, dtype=np.float32)
    angles = np.ascontiguousarray(angles, dtype=np.float32)
    img = _cb_image(b)
    if x0 is None:
        vol = ArecImage()
        vol.data = C.POINTER(C.c_float)()
    else:
        nx = b.shape[2]
        radius = (nx // 2) if name == "cyl_cgls_KB" or name.endswith("_stat") else 0.5 * (nx - 1)
        vol = arecAllocateCylImage(radius, b.shape[1])
        cyl_data(vol)[:] = np.asarray(x0, np.float32)
    st = getattr(lib(), "arecgb_" + name)(0, img, _f32p(angles), C.byref(vol), float(lam),
                                          int(maxit), float(tol))
    x = cyl_data(vol).copy() if vol.data else None
    if vol.data:
        arecImageFree(vol)
    return x, st


def last_trace(cap=4096):
    """(relative residuals, SolveInfo) of the last solver call on this thread."""
    rel = np.zeros(cap, np.float64)
    info = SolveInfo()
    n = lib().arecgb_last_trace(rel.ctypes.data_as(C.POINTER(C.c_double)), cap, C.byref(info))
    return rel[:n].copy(), info


def cyl_sirt(b, angles, lam=5e-6, maxit=10, tol=1e-3):
    """(x[nrays][ny], status) — reference cyl_sirt over b[nangles][ny][nx]."""
    return _solve("cyl_sirt", b, angles, lam, maxit, tol)


def cyl_sirt_KB(b, angles, lam=5e-6, maxit=10, tol=1e-3):
    return _solve("cyl_sirt_KB", b, angles, lam, maxit, tol)


def cyl_sirt_SQ(b, angles, lam=5e-6, maxit=10, tol=1e-3):
    return _solve("cyl_sirt_SQ", b, angles, lam, maxit, tol)


def cyl_cgls(b, angles, maxit=10, tol=1e-3, x0=None):
    return _solve("cyl_cgls", b, angles, 0.0, maxit, tol, x0)


def cyl_cgls_KB(b, angles, maxit=10, tol=1e-3, x0=None):
    return _solve("cyl_cgls_KB", b, angles, 0.0, maxit, tol, x0)


def cyl_cgls_SQ(b, angles, maxit=10, tol=1e-3, x0=None):
    return _solve("cyl_cgls_SQ", b, angles, 0.0, maxit, tol, x0)


def cyl_cgls_SQ_stat(b, angles, maxit=10, tol=1e-3, x0=None):
    """Statistically weighted CGLS (the reference's integer radius nx/2: odd nx)."""
    return _solve("cyl_cgls_SQ_stat", b, angles, 0.0, maxit, tol, x0)


def cyl_cgls_KB_stat(b, angles, maxit=10, tol=1e-3, x0=None):
    return _solve("cyl_cgls_KB_stat", b, angles, 0.0, maxit, tol, x0)


def cyl_cgls_stat(b, angles, maxit=10, tol=1e-3, x0=None):
    return _solve("cyl_cgls_stat", b, angles, 0.0, maxit, tol, x0)


def arecCCImages(images1, images2):
    """(sx, sy, status): shift of each images2[i] against images1[i] ([nz][ny][nx])."""
    a = np.ascontiguousarray(images1, dtype=np.float32)
    b = np.ascontiguousarray(images2, dtype=np.float32)
    sx = np.zeros(a.shape[0], np.float32)
    sy = np.zeros(a.shape[0], np.float32)
    st = lib().arecgb_arecCCImages(0, _cb_image(a), _cb_image(b), _f32p(sx), _f32p(sy))
    return sx, sy, st


def arecRotCCImages(images1, images2, r2):
    """(angles, status): rotation of each images2[i] against images1[i] (degrees)."""
    a = np.ascontiguousarray(images1, dtype=np.float32)
    b = np.ascontiguousarray(images2, dtype=np.float32)
    ang = np.zeros(a.shape[0], np.float32)
    st = lib().arecgb_arecRotCCImages(0, _cb_image(a), _cb_image(b), int(r2), _f32p(ang))
    return ang, st


def arecRotateImages(images, angles, kind=""):
    """(rotated copy, angles) of a host stack; kind "" (bilinear) or "_skew"."""
    a = np.ascontiguousarray(images, dtype=np.float32).copy()
    ang = np.ascontiguousarray(angles, dtype=np.float32).copy()
    im = _cb_image(a)
    getattr(lib(), "arecgb_arecRotateImages" + kind)(C.byref(im), _f32p(ang))
    return a, ang


def arecRotateImages_skew_safe(images, ref, angles):
    """(rotated copy, angles) of a host stack against ref."""
    a = np.ascontiguousarray(images, dtype=np.float32).copy()
    r = np.ascontiguousarray(ref, dtype=np.float32)
    ang = np.ascontiguousarray(angles, dtype=np.float32).copy()
    im, rf = _cb_image(a), _cb_image(r)
    lib().arecgb_arecRotateImages_skew_safe(C.byref(im), C.byref(rf), _f32p(ang))
    return a, ang


def _take_image(im):
    """Copy an arecImage the library allocated into numpy and free it."""
    if not im.data:
        return None
    a = np.ctypeslib.as_array(im.data, shape=(im.nz, im.ny, im.nx)).copy()
    arecImageFree(im)
    return a


def arecReadImage(fname, dist=""):
    """(stack [nz][ny][nx], status) through arecReadImage, or through
    arecReadImageDistbyZ / DistbyY with dist "Z" / "Y"."""
    im = ArecImage()
    if dist:
        getattr(lib(), "arecgb_arecReadImageDistby" + dist)(0, os.fsencode(fname), C.byref(im))
        st = 0 if im.data else -1
    else:
        st = lib().arecgb_arecReadImage(os.fsencode(fname), C.byref(im))
    return _take_image(im), st


def arecImageTakeLog(stack):
    """arecImageTakeLog on a copy of a host stack [nz][ny][nx]."""
    a = np.ascontiguousarray(stack, dtype=np.float32).copy()
    lib().arecgb_arecImageTakeLog(_cb_image(a))
    return a


def periodicDecomposition(stack):
    """periodicDecomposition on a copy of a host stack [nz][ny][nx]."""
    a = np.ascontiguousarray(stack, dtype=np.float32).copy()
    lib().arecgb_periodicDecomposition(_cb_image(a))
    return a


def makePeriodicSlice(image):
    """The smooth part S of one host image [ny][nx]."""
    a = np.ascontiguousarray(image, dtype=np.float32).copy()
    out = np.zeros_like(a)
    lib().arecgb_makePeriodicSlice(a.shape[1], a.shape[0], _f32p(a), _f32p(out))
    return out


def arecReadImageHeader(fname):
    nx, ny, nz = C.c_int(), C.c_int(), C.c_int()
    st = lib().arecgb_arecReadImageHeader(os.fsencode(fname), C.byref(nx), C.byref(ny),
                                          C.byref(nz))
    return (nx.value, ny.value, nz.value), st


def arecWriteImage(fname, stack, merge=""):
    """arecWriteImage, or arecWriteImageMergeY / MergeZ with merge "Y" / "Z"."""
    a = np.ascontiguousarray(stack, dtype=np.float32)
    if merge:
        getattr(lib(), "arecgb_arecWriteImageMerge" + merge)(0, os.fsencode(fname), _cb_image(a))
        return 0
    return lib().arecgb_arecWriteImage(os.fsencode(fname), _cb_image(a))


def ccorr2d(x, y):
    x = np.ascontiguousarray(x, dtype=np.float32).copy()
    y = np.ascontiguousarray(y, dtype=np.float32).copy()
    ny, nx = x.shape
    c = np.zeros_like(x)
    lib().arecgb_ccorr2d(nx, ny, _f32p(x), _f32p(y), _f32p(c))
    return c


def speak(c):
    c = np.ascontiguousarray(c, dtype=np.float32).copy()
    ny, nx = c.shape
    xt, yt = C.c_float(), C.c_float()
    lib().arecgb_speak(nx, ny, _f32p(c), C.byref(xt), C.byref(yt))
    return xt.value, yt.value
