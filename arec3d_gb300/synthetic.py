"""Seeded synthetic phantoms and sinograms with the shapes of the reference's
benchmark configurations (there is no public dataset for this path).

Line integrals are analytic (exact chord lengths through ellipses / spheres at
the detector-bin centres), noise is Poisson at a given incident photon count,
and the measured data are b = -ln(max(counts, 1) / I0).  Geometry follows the
projector's convention: detector bin u sees the line X*cos(a) + Z*sin(a) = u - r
with X = ix - r, Z = iz - r and r = (nx - 1) / 2.

Generated on the GPU with torch (plumbing only; the product path never imports
this module).  Outputs are returned in the device sinogram layout
[nangles][nx][ys] unless stated otherwise.
"""
import math

import numpy as np


def _torch():
    import torch

    return torch


def uniform_angles(na, span=math.pi):
    return (np.arange(na) * (span / na)).astype(np.float32)


def sphere_cylinder_phantom(seed, nx, ny, n_spheres=200, cyl_radius=None, r_min=3.0,
                            r_max=80.0, mu_max=0.02, mu_cyl=0.001):
    """Random-sphere cylinder (config: 'random cylinder of radius 500 px holding
    200 random spheres (radius 3-80 px, attenuation 0-0.02/px)').  Returns a
    dict of sphere parameters in pixel units, centres relative to the axis."""
    rng = np.random.default_rng(seed)
    R = cyl_radius if cyl_radius is not None else min(500.0, 0.5 * (nx - 1) - 4)
    rad = rng.uniform(r_min, r_max, n_spheres)
    # centres uniform inside the cylinder, spheres kept inside its radius
    rr = (R - rad) * np.sqrt(rng.uniform(0, 1, n_spheres))
    th = rng.uniform(0, 2 * math.pi, n_spheres)
    return {
        "cx": rr * np.cos(th), "cz": rr * np.sin(th), "cy": rng.uniform(0, ny, n_spheres),
        "r": rad, "mu": rng.uniform(0, mu_max, n_spheres), "R": R, "mu_cyl": mu_cyl,
    }


def ellipse_phantom(seed, nx, ny, n_ellipses=10, centre_radius=120.0, a_min=5.0, a_max=60.0,
                    mu_max=0.02):
    """Per-slice random ellipses (config: 10 ellipses per slice, centres uniform
    in a disk of radius 120, semi-axes 5-60 px, attenuation 0-0.02/px)."""
    rng = np.random.default_rng(seed)
    n = ny * n_ellipses
    rr = centre_radius * np.sqrt(rng.uniform(0, 1, n))
    th = rng.uniform(0, 2 * math.pi, n)
    return {
        "cx": rr * np.cos(th), "cz": rr * np.sin(th), "slice": np.repeat(np.arange(ny), n_ellipses),
        "a": rng.uniform(a_min, a_max, n), "b": rng.uniform(a_min, a_max, n),
        "phi": rng.uniform(0, math.pi, n), "mu": rng.uniform(0, mu_max, n),
    }


def sphere_sinogram(ph, nx, ny, angles, ys=None, device="cuda", chunk=64):
    """Analytic line integrals of a sphere phantom, [na][nx][ys] float32 (torch)."""
    torch = _torch()
    ys = ys or ((ny + 7) // 8) * 8
    na = len(angles)
    r = 0.5 * (nx - 1)
    out = torch.zeros(na, nx, ys, dtype=torch.float32, device=device)
    ang = torch.tensor(np.asarray(angles, np.float64), device=device)
    t = torch.arange(nx, device=device, dtype=torch.float64) - r
    # cylinder body: same chord in every slice
    R = ph["R"]
    chord = 2 * torch.sqrt(torch.clamp(R * R - t * t, min=0))
    out[:, :, :ny] += (ph["mu_cyl"] * chord).float()[None, :, None]
    c, s = torch.cos(ang), torch.sin(ang)
    for i in range(len(ph["r"])):
        rad, mu = float(ph["r"][i]), float(ph["mu"][i])
        cy = float(ph["cy"][i])
        y0, y1 = max(0, int(math.floor(cy - rad))), min(ny, int(math.ceil(cy + rad)) + 1)
        if y1 <= y0:
            continue
        yy = torch.arange(y0, y1, device=device, dtype=torch.float64)
        rho2 = torch.clamp(rad * rad - (yy - cy) ** 2, min=0)          # [Y]
        pc = float(ph["cx"][i]) * c + float(ph["cz"][i]) * s            # [na]
        w = int(2 * rad) + 4
        u0 = torch.floor(pc + r - rad - 1).long()                       # [na]
        uu = u0[:, None] + torch.arange(w, device=device)[None, :]      # [na, W]
        d = (uu.double() - r) - pc[:, None]                             # [na, W]
        val = 2 * torch.sqrt(torch.clamp(rho2[None, None, :] - (d * d)[:, :, None], min=0))
        val = (mu * val).float()                                        # [na, W, Y]
        ok = (uu >= 0) & (uu < nx)
        ai = torch.arange(na, device=device)[:, None].expand(na, w)
        for a0 in range(0, na, chunk * 16):
            sl = slice(a0, a0 + chunk * 16)
            m = ok[sl]
            out[ai[sl][m], uu[sl][m], y0:y1] += val[sl][m]
    return out


def ellipse_sinogram(ph, nx, ny, angles, ys=None, device="cuda"):
    """Analytic line integrals of per-slice ellipses, [na][nx][ys] (torch)."""
    torch = _torch()
    ys = ys or ((ny + 7) // 8) * 8
    na = len(angles)
    r = 0.5 * (nx - 1)
    out = torch.zeros(na, nx, ys, dtype=torch.float32, device=device)
    ang = torch.tensor(np.asarray(angles, np.float64), device=device)
    t = torch.arange(nx, device=device, dtype=torch.float64) - r
    c, s = torch.cos(ang), torch.sin(ang)
    for i in range(len(ph["a"])):
        a, b, phi, mu = float(ph["a"][i]), float(ph["b"][i]), float(ph["phi"][i]), float(ph["mu"][i])
        pc = float(ph["cx"][i]) * c + float(ph["cz"][i]) * s
        # support half-width of the ellipse along the detector at angle theta
        ct = torch.cos(ang - phi)
        st_ = torch.sin(ang - phi)
        h2 = (a * ct) ** 2 + (b * st_) ** 2
        d = t[None, :] - pc[:, None]
        val = 2 * a * b * torch.sqrt(torch.clamp(h2[:, None] - d * d, min=0)) / h2[:, None]
        out[:, :, int(ph["slice"][i])] += (mu * val).float()
    return out


def poisson_log(p, photons, seed, ny, device="cuda", chunk=64):
    """b = -ln(max(Poisson(I0 exp(-p)), 1) / I0) for a [na][nx][ys] torch
    tensor of line integrals, computed in place in angle chunks; padding
    slices (index >= ny) stay zero."""
    torch = _torch()
    g = torch.Generator(device=device)
    g.manual_seed(int(seed))
    for a0 in range(0, p.shape[0], chunk):
        blk = p[a0:a0 + chunk, :, :ny]
        counts = torch.poisson(photons * torch.exp(-blk), generator=g)
        blk.copy_(-torch.log(torch.clamp(counts, min=1.0) / photons))
    return p


def cylinder_coords(radius):
    """Pixel-centre coordinates (x, z) relative to the axis of the rays of the
    reference's cylinder of this radius, in its ray order (iz-major; a pixel is
    a ray when (int)(ix - r)^2 + (int)(iz - r)^2 <= (int)(r r), truncation
    toward zero: arecAllocateCylImage, AREC3D/AREC3D/arecImage.cpp:29-86)."""
    n = int(round(2 * radius + 1))
    ix, iz = np.meshgrid(np.arange(n), np.arange(n))
    xs = np.trunc(ix - radius).astype(np.int64)
    zs = np.trunc(iz - radius).astype(np.int64)
    m = xs * xs + zs * zs <= int(radius * radius)
    return (ix[m] - radius).astype(np.float64), (iz[m] - radius).astype(np.float64)


def sphere_volume(ph, radius, ny, ys=None, device="cuda"):
    """The sphere phantom's attenuation at the pixel centres of the cylinder,
    [nrays][ys] float32 (torch; padding slices zero): the ground truth a
    reconstruction is compared with."""
    torch = _torch()
    ys = ys or ((ny + 7) // 8) * 8
    cx, cz = cylinder_coords(radius)
    px = torch.tensor(cx, device=device)
    pz = torch.tensor(cz, device=device)
    out = torch.zeros(px.numel(), ys, dtype=torch.float64, device=device)
    out[:, :ny] += ph["mu_cyl"] * ((px * px + pz * pz) <= ph["R"] ** 2).double()[:, None]
    for i in range(len(ph["r"])):
        rad, mu, cy = float(ph["r"][i]), float(ph["mu"][i]), float(ph["cy"][i])
        y0, y1 = max(0, int(math.floor(cy - rad))), min(ny, int(math.ceil(cy + rad)) + 1)
        if y1 <= y0:
            continue
        d2 = (px - float(ph["cx"][i])) ** 2 + (pz - float(ph["cz"][i])) ** 2
        idx = torch.nonzero(d2 <= rad * rad).squeeze(1)
        if idx.numel() == 0:
            continue
        yy = torch.arange(y0, y1, device=device, dtype=torch.float64)
        inside = (d2[idx][:, None] + (yy[None, :] - cy) ** 2) <= rad * rad
        out[idx, y0:y1] += mu * inside.double()
    return out.float()
