"""CPU restatement (numpy) of the reference's rotational alignment: the rotation
search arecRotCCImages and the rotations arecRotateImages, _skew, _skew_safe.

Test infrastructure only (the oracle): imported by tests/ and never by the
product package.  Each function follows the reference expression for
expression; float32 steps are numpy float32 operations (no contraction) and
double steps Python / float64 operations.  Where the reference calls the float
overloads of sin / cos (std::sin(float) through <math.h>), this file rounds the
double-precision value to float.

Images are [ny][nx] float32 (a stack [nz][ny][nx]); angles are degrees.
"""
import math

import numpy as np

PI = math.atan(1.0) * 4  # piFunc(), AREC3D/AREC3D/arecConstants.h:7
F32 = np.float32


def _f(x):
    return F32(x)


def radial_profile(img, n, R):
    """getRadialProfile (AREC3D/AREC3D/arecImage.cpp:534-553) with
    getCoord_blerp_raw (:515-532): out[i] = sum_{ri<R} blerp(xc + cos(a_i) ri,
    yc + sin(a_i) ri) * ri, a_i = 2 pi i / n, accumulated in float."""
    img = np.asarray(img, np.float32)
    ny, nx = img.shape
    xc, yc = 0.5 * (nx - 1), 0.5 * (ny - 1)
    alpha = np.array([2 * PI * i / n for i in range(n)])
    c, s = np.cos(alpha), np.sin(alpha)
    acc = np.zeros(n, np.float32)
    for ri in range(R):
        x = (xc + c * ri).astype(np.float32)
        y = (yc + s * ri).astype(np.float32)
        xb, yb = x.astype(np.int32), y.astype(np.int32)
        xf = (x - xb.astype(np.float32)).astype(np.float64)
        yf = (y - yb.astype(np.float32)).astype(np.float64)
        xf[xf < 0] = 0.0
        yf[yf < 0] = 0.0
        ll = img[yb, xb].astype(np.float64)
        lr = img[yb, xb + 1].astype(np.float64)
        ur = img[yb + 1, xb + 1].astype(np.float64)
        ul = img[yb + 1, xb].astype(np.float64)
        up = ul + xf * (ur - ul)
        lo = ll + xf * (lr - ll)
        v = (lo + yf * (up - lo)).astype(np.float32)
        acc = acc + v * np.float32(ri)
    return acc


def ccorr1d(x, y):
    """ccorr1d (AREC3D/AREC3D/align2dstack.cpp:437-476): IDFT(conj(DFT x) DFT y),
    unnormalised (n * sum_i x[i] y[i+k]); computed in double, stored float."""
    x = np.asarray(x, np.float64)
    y = np.asarray(y, np.float64)
    n = len(x)
    c = np.fft.irfft(np.conj(np.fft.rfft(x)) * np.fft.rfft(y), n) * n
    return c.astype(np.float32)


def prb1d7(B):
    """PRB1D with NPOINT = 7 (AREC3D/AREC3D/align2dstack.cpp:1028-1056): vertex
    of the least-squares parabola through 7 points, relative to the centre."""
    b1, b2, b3, b4, b5, b6, b7 = (float(v) for v in B)
    c2 = 49. * b1 + 6. * b2 - 21. * b3 - 32. * b4 - 27. * b5 - 6. * b6 + 31. * b7
    c3 = 5. * b1 - 3. * b3 - 4. * b4 - 3. * b5 + 5. * b7
    return c2 / (2. * c3) - 4 if c3 != 0.0 else 0.0


def find_peak_1d(c):
    """findPeak1d (AREC3D/AREC3D/arecImage.cpp:502-513): first arg max, 7-point
    fit with wrap-around, returned as float."""
    n = len(c)
    m = int(np.argmax(c))
    B = [c[(m + k + n) % n] for k in range(-3, 4)]
    return _f(prb1d7(B) + m)


def rot_cc_angle(img1, img2, r2):
    """arecRotCCImages for one pair (AREC3D/AREC3D/arecImage.cpp:555-598)."""
    n = int(r2 * 2 * PI)
    p1 = radial_profile(img1, n, r2)
    p2 = radial_profile(img2, n, r2)
    a = find_peak_1d(ccorr1d(p1, p2))
    a = _f(float(a) * (2 * PI / n))
    if float(a) > PI:
        a = _f(float(a) - 2.0 * PI)
    a = _f(float(a) * (180.0 / PI))
    if abs(float(a)) > 45:
        a = F32(0.0)
    return a


def rot_cc_angles(stack1, stack2, r2):
    return np.array([rot_cc_angle(a, b, r2) for a, b in zip(stack1, stack2)], np.float32)


def _shear_rows(img, shear, centre_len):
    """Rows of img sheared: row j circularly shifted by floor(skew_j), then the
    linear tap (p - p f) + p_prev f (shearX_circ, AREC3D/AREC3D/imagetools.cpp:244-266)."""
    img = np.asarray(img, np.float32)
    out = np.empty_like(img)
    centre = 0.5 * (centre_len - 1)
    for j in range(img.shape[0]):
        skew = _f(float(shear) * (j - centre))
        si = int(math.floor(float(skew)))
        f = _f(float(skew) - 1.0 * si)
        p = np.roll(img[j], si)
        q = np.roll(p, 1)
        out[j] = (p - p * f) + q * f
    return out


def shear_x(img, shear):
    """shearX_circ (AREC3D/AREC3D/imagetools.cpp:244-266)."""
    img = np.asarray(img, np.float32)
    return _shear_rows(img, shear, img.shape[0])


def shear_y(img, shear):
    """shearY_circ (AREC3D/AREC3D/imagetools.cpp:268-291): the same on columns,
    skew from the column index about 0.5 (nx - 1)."""
    img = np.asarray(img, np.float32)
    return np.ascontiguousarray(_shear_rows(img.T, shear, img.shape[1]).T)


def _rad(a):
    return _f(float(a) * PI / 180.0)


def rotate_shears(img, angle):
    """The three-shear rotation of arecRotateImages_skew / _skew_safe
    (AREC3D/AREC3D/arecImage.cpp:733-736, 767-770)."""
    r = _rad(angle)
    shx = _f(-math.tan(-0.5 * float(r)))
    shy = _f(math.sin(float(-r)))
    return shear_x(shear_y(shear_x(img, shx), shy), shx)


def rotate2d(img, theta):
    """rotate2d (AREC3D/AREC3D/align2dstack.cpp:774-816): bilinear, zero where
    the source cell leaves the image, centre (nx/2 + 1, ny/2 + 1) 1-based."""
    img = np.asarray(img, np.float32)
    ny, nx = img.shape
    th = _rad(theta)
    if float(th) > PI:
        th = _f(-2.0 * PI + float(th))
    if float(th) < -PI:
        th = _f(2. * PI + float(th))
    cod = float(_f(math.cos(float(th))))
    sid = float(_f(math.sin(float(th))))
    kcent, icent = nx // 2 + 1, ny // 2 + 1
    I = np.arange(1, ny + 1, dtype=np.float64)[:, None]
    K = np.arange(1, nx + 1, dtype=np.float64)[None, :]
    Y = I - icent
    ycod = Y * cod + icent
    ysid = -Y * sid + kcent
    X = K - kcent
    xold = X * cod + ysid
    yold = X * sid + ycod
    iy = np.trunc(yold).astype(np.int64)
    ix = np.trunc(xold).astype(np.int64)
    ok = (iy >= 1) & (iy <= ny - 1) & (ix >= 1) & (ix <= nx - 1)
    ydif = yold - iy
    yrem = 1.0 - ydif
    xdif = xold - ix
    xrem = 1.0 - xdif
    f = img.astype(np.float64).ravel()
    a = np.where(ok, (iy - 1) * nx + ix - 1, 0)  # 0-based index of imagein(NADDR)
    v = ydif * (f[a + np.where(ok, nx, 0)] * xrem + f[a + np.where(ok, nx + 1, 0)] * xdif) + \
        yrem * (f[a] * xrem + f[a + np.where(ok, 1, 0)] * xdif)
    return np.where(ok, v, 0.0).astype(np.float32)


def tukey_axis(n, alpha=0.3):
    """tukey_filter along one axis (AREC3D/AREC3D/imagetools.cpp:331-366)."""
    a, b = 0.5 * alpha * (n - 1), (1.0 - 0.5 * alpha) * (n - 1)
    A = 2.0 * PI / alpha
    h = np.empty(n)
    for i in range(n):
        va = 0.5 * (1.0 + math.cos(A * (1.0 * i / (n - 1) - alpha / 2)))
        vb = 0.5 * (1.0 + math.cos(A * (1.0 * i / (n - 1) - 1.0 + alpha / 2)))
        h[i] = va if i < a else (vb if i > b else 1.0)
    return h


def ncc_filtered(im1, im2):
    """getNormalizedCrossCorrelationWithFilter (AREC3D/AREC3D/imagetools.cpp:415-446)."""
    im1 = np.asarray(im1, np.float32)
    im2 = np.asarray(im2, np.float32)
    ny, nx = im1.shape
    filt = (tukey_axis(ny)[:, None] * tukey_axis(nx)[None, :]).astype(np.float32)
    a = (im1 * filt).astype(np.float64)
    b = (im2 * filt).astype(np.float64)
    m1 = a.sum() / (1.0 * nx * ny)
    m2 = b.sum() / (1.0 * nx * ny)
    d1, d2 = a - m1, b - m2
    return float((d1 * d2).sum() / math.sqrt((d1 * d1).sum() * (d2 * d2).sum()))


def rotate_images(stack, angles):
    """arecRotateImages (AREC3D/AREC3D/arecImage.cpp:674-690)."""
    return np.stack([rotate2d(im, a) for im, a in zip(stack, angles)])


def rotate_images_skew(stack, angles):
    """arecRotateImages_skew (AREC3D/AREC3D/arecImage.cpp:692-738); returns the
    rotated stack and the updated angles."""
    out = np.array(stack, np.float32, copy=True)
    ang = np.array(angles, np.float32, copy=True)
    for j in range(len(out)):
        if ang[j] < -180:
            ang[j] = _f(float(ang[j]) + 360)
        if ang[j] > 180:
            ang[j] = _f(float(ang[j]) - 360)
        if abs(float(ang[j])) > 45:
            ang[j] = 0.0
        elif abs(float(ang[j])) > 10:
            out[j] = rotate2d(out[j], ang[j])
        else:
            out[j] = rotate_shears(out[j], ang[j])
    return out, ang


def rotate_images_skew_safe(stack, ref, angles):
    """arecRotateImages_skew_safe (AREC3D/AREC3D/arecImage.cpp:740-790); returns
    the stack, the updated angles, the number of slices rotated and the mean
    kept correlation."""
    out = np.array(stack, np.float32, copy=True)
    ang = np.array(angles, np.float32, copy=True)
    cc_sum, n_rot = 0.0, 0
    for j in range(len(out)):
        rot = rotate_shears(out[j], ang[j])
        cc1 = ncc_filtered(rot, ref[j])
        cc2 = ncc_filtered(out[j], ref[j])
        if cc2 + 0.00001 < cc1:
            out[j] = rot
            cc_sum += cc1
            n_rot += 1
            ang[j] = _f(float(ang[j]) * 0.5)
        else:
            ang[j] = 0.0
            cc_sum += cc2
    return out, ang, n_rot, cc_sum / len(out)
