"""Initial states for the 2D and 3D steps (inputs, not part of the hot path).

* ``orszag_tang``: the Orszag-Tang vortex of the reference's sample script
  (InitializationFiles/SampleSimulations/2D_MHD/OrszagTang_InitializationFile.py:117-194),
  optionally with face B taken from the corner vector potential (the form the
  4096^2 / batched workloads use) instead of the cell-averaged faces the
  reference's ``SimulationGrid`` builds when no faces are passed
  (Source/SimulationGrid.py:147-156).
* ``turbulence``: the seeded driven-free turbulence state (Gaussian random
  density, velocity and vector-potential fields with power-law spectra).
* ``turbulence_hydro_3d``: seeded 3D hydro turbulence for the 3D step, generated
  with torch (on the GPU for the large boxes).
* ``prim_to_cons_mhd`` / ``prim_to_cons_hydro``: the conserved variables the
  reference's grid derives at construction
  (Source/PrimCons_HelperModule.py:23-35 and :314-340).

Spectral convention (frozen): a field with "power ~ k^-a for k1 <= |k| <= k2"
is ``irfft2`` of complex coefficients c(kx, ky) = (N(0,1) + i N(0,1)) * |k|^(-a/2)
on the integer wavevectors of the periodic box with k1 <= |k| <= k2, zero
elsewhere (per-mode power, not shell power), drawn from
``numpy.random.default_rng(seed)`` in the order g, vx, vy, Az, then shifted to
zero mean and scaled as each field requires.
"""
from __future__ import annotations

import math

import numpy as np

OUTFLOW = 0
PERIODIC = 1


def cell_centres(n, lo, hi):
    d = (hi - lo) / n
    return lo + (np.arange(n) + 0.5) * d, d


def prim_to_cons_mhd(prim, gamma):
    """Conserved 8-vector from the primitive 8-vector (same arithmetic order as the reference)."""
    p = np.asarray(prim, dtype=np.float64)
    c = np.empty_like(p)
    c[0] = p[0]
    c[1] = p[0] * p[1]
    c[2] = p[0] * p[2]
    c[3] = p[0] * p[3]
    c[4] = p[4]
    c[5] = p[5]
    c[6] = p[6]
    c[7] = p[7] / (gamma - 1.0) + 0.5 * p[0] * (p[1] * p[1] + p[2] * p[2] + p[3] * p[3])
    c[7] += 0.5 * (p[4] * p[4] + p[5] * p[5] + p[6] * p[6])
    return c


def prim_to_cons_hydro(prim, gamma):
    p = np.asarray(prim, dtype=np.float64)
    c = np.empty_like(p)
    c[0] = p[0]
    c[1] = p[0] * p[1]
    c[2] = p[0] * p[2]
    c[3] = p[0] * p[3]
    c[4] = (p[4] / (gamma - 1.0)) + 0.5 * p[0] * (np.square(p[1]) + np.square(p[2]) + np.square(p[3]))
    return c


def faces_from_cells(bx, by, bcx, bcy):
    """Face B as the mean of the two neighbouring cell values (Source/CT_HelperModule.py:29-70)."""
    if bcx == OUTFLOW:
        lx = np.concatenate([bx[:, :1], bx], axis=1)
        rx = np.concatenate([bx, bx[:, -1:]], axis=1)
    else:
        lx = np.concatenate([bx[:, -1:], bx], axis=1)
        rx = np.concatenate([bx, bx[:, :1]], axis=1)
    if bcy == OUTFLOW:
        ty = np.concatenate([by[:1], by], axis=0)
        by_ = np.concatenate([by, by[-1:]], axis=0)
    else:
        ty = np.concatenate([by[-1:], by], axis=0)
        by_ = np.concatenate([by, by[:1]], axis=0)
    return (lx + rx) / 2.0, (ty + by_) / 2.0


def faces_from_potential(az):
    """Periodic face B from a corner vector potential az[j, i] at (x_i - dx/2, y_j - dy/2).

    Returns (faceBx (Ny, Nx+1), faceBy (Ny+1, Nx)) with dx = dy = 1 (callers scale),
    the duplicate periodic faces equal bit for bit.
    """
    bxf = np.roll(az, -1, axis=0) - az            # Bx = dAz/dy at x-face i of row j
    byf = -(np.roll(az, -1, axis=1) - az)          # By = -dAz/dx at y-face j of column i
    fbx = np.concatenate([bxf, bxf[:, :1]], axis=1)
    fby = np.concatenate([byf, byf[:1, :]], axis=0)
    return fbx, fby


def orszag_tang(nx, ny, gamma=5.0 / 3.0, b0_scale=1.0, faces="potential",
                rho_perturb=0.0, seed=None):
    """Orszag-Tang vortex on the periodic unit square.

    Returns (prim (8,Ny,Nx), cons (8,Ny,Nx), faceBx (Ny,Nx+1), faceBy (Ny+1,Nx), dx, dy).
    ``faces="potential"`` takes the faces from A_z (divergence-free to roundoff);
    ``faces="cells"`` re-averages them from the cell values as the reference grid does.
    ``rho_perturb`` multiplies the density by (1 + rho_perturb * N(0,1)) (seeded).
    """
    pi = math.pi
    x, dx = cell_centres(nx, 0.0, 1.0)
    y, dy = cell_centres(ny, 0.0, 1.0)
    X, Y = np.meshgrid(x, y)
    b0 = b0_scale / np.sqrt(4.0 * pi)
    az = (b0 / (4.0 * pi)) * np.cos(4.0 * pi * (X - dx / 2.0)) \
        + (b0 / (2.0 * pi)) * np.cos(2.0 * pi * (Y - dy / 2.0))
    fbx_u, fby_u = faces_from_potential(az)
    left_bx = fbx_u[:, :-1] / dy
    top_by = fby_u[:-1, :] / dx
    cbx = (left_bx + np.roll(left_bx, -1, axis=1)) / 2.0
    cby = (top_by + np.roll(top_by, -1, axis=0)) / 2.0
    prim = np.zeros((8, ny, nx))
    prim[0] = 25.0 / (36.0 * pi)
    if rho_perturb:
        rng = np.random.default_rng(seed)
        prim[0] *= 1.0 + rho_perturb * rng.standard_normal((ny, nx))
    prim[1] = -np.sin(2.0 * pi * Y)
    prim[2] = np.sin(2.0 * pi * X)
    prim[4] = cbx
    prim[5] = cby
    prim[7] = 5.0 / (12.0 * pi)
    if faces == "potential":
        fbx = fbx_u / dy
        fby = fby_u / dx
    else:
        fbx, fby = faces_from_cells(cbx, cby, PERIODIC, PERIODIC)
    return prim, prim_to_cons_mhd(prim, gamma), fbx, fby, dx, dy


def _gaussian_field(rng, n, slope, kmin, kmax):
    kx = np.fft.rfftfreq(n, d=1.0 / n)
    ky = np.fft.fftfreq(n, d=1.0 / n)
    KX, KY = np.meshgrid(kx, ky)
    k = np.sqrt(KX * KX + KY * KY)
    mask = (k >= kmin) & (k <= kmax)
    amp = np.zeros_like(k)
    amp[mask] = k[mask] ** (-slope / 2.0)
    c = (rng.standard_normal(k.shape) + 1j * rng.standard_normal(k.shape)) * amp
    f = np.fft.irfft2(c, s=(n, n))
    return f - f.mean()


def turbulence(n, seed=1, gamma=5.0 / 3.0, kmax_v=32, kmax_a=16, mach=1.0, beta=1.0):
    """Driven-free turbulence initial state on the periodic unit square, n x n cells.

    rho = exp(0.1 g) with g a unit-variance field, power ~ k^-2 (1 <= k <= kmax_v);
    vx, vy independent fields of the same spectrum scaled to rms Mach ``mach``
    (sqrt(<(vx^2+vy^2)/c_s^2>) = mach, c_s^2 = gamma p / rho); p = 1/gamma;
    A_z with power ~ k^-3 (1 <= k <= kmax_a) scaled so 2p/<B^2> = ``beta``.
    Returns (prim, cons, faceBx, faceBy, dx, dy).
    """
    rng = np.random.default_rng(seed)
    g = _gaussian_field(rng, n, 2.0, 1.0, kmax_v)
    g /= g.std()
    vx = _gaussian_field(rng, n, 2.0, 1.0, kmax_v)
    vy = _gaussian_field(rng, n, 2.0, 1.0, kmax_v)
    az = _gaussian_field(rng, n, 3.0, 1.0, kmax_a)
    dx = dy = 1.0 / n
    rho = np.exp(0.1 * g)
    p = np.full((n, n), 1.0 / gamma)
    cs2 = gamma * p / rho
    vscale = mach / np.sqrt(np.mean((vx * vx + vy * vy) / cs2))
    vx *= vscale
    vy *= vscale
    fbx_u, fby_u = faces_from_potential(az)
    fbx = fbx_u / dy
    fby = fby_u / dx
    cbx = (fbx[:, :-1] + fbx[:, 1:]) / 2.0
    cby = (fby[:-1, :] + fby[1:, :]) / 2.0
    bscale = np.sqrt(2.0 * (1.0 / gamma) / beta / np.mean(cbx * cbx + cby * cby))
    fbx *= bscale
    fby *= bscale
    cbx = (fbx[:, :-1] + fbx[:, 1:]) / 2.0
    cby = (fby[:-1, :] + fby[1:, :]) / 2.0
    prim = np.zeros((8, n, n))
    prim[0] = rho
    prim[1] = vx
    prim[2] = vy
    prim[4] = cbx
    prim[5] = cby
    prim[7] = p
    return prim, prim_to_cons_mhd(prim, gamma), fbx, fby, dx, dy


def orszag_tang_batch(count=256, seed=0, sizes=tuple(range(64, 513, 32)), gamma_range=(1.4, 5.0 / 3.0),
                      b0_range=(0.5, 2.0), rho_perturb=0.01):
    """The uneven batch of Orszag-Tang instances (the batched workload).

    Each instance draws Nx and Ny independently and uniformly from ``sizes``,
    gamma uniformly from ``gamma_range``, a B0 scale uniformly from ``b0_range``,
    and gets a seeded ``rho_perturb`` Gaussian density perturbation (its own seed
    ``seed * 100003 + k``).  Returns a list of dicts with the state arrays and
    grid parameters.
    """
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        nx = int(rng.choice(sizes))
        ny = int(rng.choice(sizes))
        gamma = float(rng.uniform(*gamma_range))
        b0 = float(rng.uniform(*b0_range))
        prim, cons, fbx, fby, dx, dy = orszag_tang(nx, ny, gamma=gamma, b0_scale=b0, faces="potential",
                                                   rho_perturb=rho_perturb, seed=seed * 100003 + k)
        out.append(dict(prim=prim, cons=cons, fbx=fbx, fby=fby, dx=dx, dy=dy, nx=nx, ny=ny, gamma=gamma,
                        bcx=PERIODIC, bcy=PERIODIC))
    return out


# ---------------------------------------------------------------------------
# the same generator with the transforms and field algebra on the GPU
# ---------------------------------------------------------------------------
def _band(rng, n, slope, kmin, kmax):
    """The in-band coefficients of ``_gaussian_field``'s spectrum: flat indices into the
    (n, n//2 + 1) half-spectrum and the real and imaginary parts, drawn from the same
    NumPy stream in the same order (whole arrays of normals, then the band's share)."""
    kx = np.fft.rfftfreq(n, d=1.0 / n)
    ky = np.fft.fftfreq(n, d=1.0 / n)
    KX, KY = np.meshgrid(kx, ky)
    k = np.sqrt(KX * KX + KY * KY)
    mask = (k >= kmin) & (k <= kmax)
    amp = k[mask] ** (-slope / 2.0)
    re = rng.standard_normal(k.shape)
    im = rng.standard_normal(k.shape)
    return np.flatnonzero(mask).astype(np.int32), re[mask] * amp, im[mask] * amp


def _gaussian_field_device(lib, rng, n, slope, kmin, kmax, device, stream):
    """``_gaussian_field`` before its zero-mean shift, on the device: the band's
    coefficients (a few thousand) are uploaded and scattered into the half-spectrum
    by the project's kernel (``mhd_ic_scatter_spectrum``), and cuFFT inverts it."""
    import ctypes

    import torch
    idx, re, im = _band(rng, n, slope, kmin, kmax)
    spec = torch.zeros((n, n // 2 + 1), dtype=torch.complex128, device=device)
    t_idx = torch.from_numpy(idx).to(device)
    t_re = torch.from_numpy(np.ascontiguousarray(re)).to(device)
    t_im = torch.from_numpy(np.ascontiguousarray(im)).to(device)
    rc = lib.mhd_ic_scatter_spectrum(len(idx), ctypes.c_void_p(t_idx.data_ptr()), ctypes.c_void_p(t_re.data_ptr()),
                                     ctypes.c_void_p(t_im.data_ptr()), ctypes.c_void_p(spec.data_ptr()), stream)
    from . import _lib
    _lib.check(rc, "mhd_ic_scatter_spectrum")
    return torch.fft.irfft2(spec, s=(n, n)).contiguous()


def turbulence_device(n, seed=1, gamma=5.0 / 3.0, kmax_v=32, kmax_a=16, mach=1.0, beta=1.0, device="cuda"):
    """``turbulence`` generated on the GPU: returns (prim, cons, faceBx, faceBy) as
    float64 torch tensors on ``device`` plus dx, dy, ready for
    ``mhd2d_upload_device`` -- no n^2 field on the host.  The random coefficients
    come from the same seeded NumPy stream; the inverse transforms run in cuFFT and
    the field algebra in the project's kernels (``mhd_ic_turbulence_2d``), so the
    state equals ``turbulence``'s to rounding."""
    import ctypes

    import torch

    from . import _lib
    lib = _lib.load()
    device = torch.device(device)
    stream = ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)
    rng = np.random.default_rng(seed)
    fields = [_gaussian_field_device(lib, rng, n, sl, 1.0, km, device, stream)
              for sl, km in ((2.0, kmax_v), (2.0, kmax_v), (2.0, kmax_v), (3.0, kmax_a))]
    prim = torch.empty((8, n, n), dtype=torch.float64, device=device)
    cons = torch.empty_like(prim)
    fbx = torch.empty((n, n + 1), dtype=torch.float64, device=device)
    fby = torch.empty((n + 1, n), dtype=torch.float64, device=device)
    words = int(lib.mhd_ic_work_words())
    work = torch.empty(words, dtype=torch.float64, device=device)
    ptr = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    _lib.check(lib.mhd_ic_turbulence_2d(n, float(gamma), float(mach), float(beta), *[ptr(f) for f in fields],
                                        ptr(prim), ptr(cons), ptr(fbx), ptr(fby), ptr(work), words, stream),
               "mhd_ic_turbulence_2d")
    torch.cuda.current_stream(device).synchronize()
    return prim, cons, fbx, fby, 1.0 / n, 1.0 / n


def orszag_tang_batch_device(count=256, seed=0, sizes=tuple(range(64, 513, 32)), gamma_range=(1.4, 5.0 / 3.0),
                             b0_range=(0.5, 2.0), rho_perturb=0.01, device="cuda"):
    """``orszag_tang_batch`` with the states built on the GPU (``mhd_ic_orszag_tang``):
    the same draws from the same seeded streams (sizes, gamma, B0 scale, and each
    instance's density noise, uploaded), the vortex evaluated on the device.  The
    instances' prim, cons, fbx, fby are float64 torch tensors on ``device``; they
    equal the host generator's to rounding (device sin/cos)."""
    import ctypes

    import torch

    from . import _lib
    lib = _lib.load()
    device = torch.device(device)
    stream = ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        nx = int(rng.choice(sizes))
        ny = int(rng.choice(sizes))
        gamma = float(rng.uniform(*gamma_range))
        b0 = float(rng.uniform(*b0_range))
        noise = None
        if rho_perturb:
            noise = torch.from_numpy(np.random.default_rng(seed * 100003 + k).standard_normal((ny, nx))).to(device)
        prim = torch.empty((8, ny, nx), dtype=torch.float64, device=device)
        cons = torch.empty_like(prim)
        fbx = torch.empty((ny, nx + 1), dtype=torch.float64, device=device)
        fby = torch.empty((ny + 1, nx), dtype=torch.float64, device=device)
        ptr = lambda t: ctypes.c_void_p(t.data_ptr()) if t is not None else None  # noqa: E731
        _lib.check(lib.mhd_ic_orszag_tang(nx, ny, gamma, b0, float(rho_perturb), ptr(noise), ptr(prim), ptr(cons),
                                          ptr(fbx), ptr(fby), stream), "mhd_ic_orszag_tang")
        out.append(dict(prim=prim, cons=cons, fbx=fbx, fby=fby, dx=1.0 / nx, dy=1.0 / ny, nx=nx, ny=ny, gamma=gamma,
                        bcx=PERIODIC, bcy=PERIODIC))
    torch.cuda.current_stream(device).synchronize()
    return out


# ---------------------------------------------------------------------------
# 3D hydro turbulence (inputs of the 3D step; arrays (5, ny, nx, nz), z fastest)
# ---------------------------------------------------------------------------
def _gaussian_field_3d(rng, n, slope, kmin, kmax, device):
    """A 3D Gaussian random field on an n^3 periodic box with the 2D generator's
    convention: ``irfftn`` of (N(0,1) + i N(0,1)) |k|^(-slope/2) on the integer
    wavevectors with kmin <= |k| <= kmax (axes y, x, z; z is the half axis), zero
    mean.  The transform runs in torch on ``device``."""
    import torch
    k1 = np.fft.fftfreq(n, d=1.0 / n)
    kz = np.fft.rfftfreq(n, d=1.0 / n)
    KY, KX, KZ = np.meshgrid(k1, k1, kz, indexing="ij")
    k = np.sqrt(KX * KX + KY * KY + KZ * KZ)
    mask = (k >= kmin) & (k <= kmax)
    amp = np.zeros_like(k)
    amp[mask] = k[mask] ** (-slope / 2.0)
    re = rng.standard_normal(k.shape)
    im = rng.standard_normal(k.shape)
    c = torch.complex(torch.from_numpy(re * amp), torch.from_numpy(im * amp)).to(device)
    f = torch.fft.irfftn(c, s=(n, n, n))
    return f - f.mean()


def turbulence_hydro_3d(n, seed=1, gamma=1.4, kmax=16, mach=1.0, device="cuda"):
    """Seeded 3D hydro turbulence on the unit n^3 periodic box: density exp(0.1 g),
    velocities with power ~ k^-2 up to ``kmax`` scaled to rms Mach ``mach``, uniform
    pressure 1/gamma.  Returns (prim, cons) float64 torch tensors of shape
    (5, n, n, n) on ``device`` and the cell size."""
    import torch
    rng = np.random.default_rng(seed)
    g = _gaussian_field_3d(rng, n, 2.0, 1.0, kmax, device)
    g = g / g.std(unbiased=False)
    v = [_gaussian_field_3d(rng, n, 2.0, 1.0, kmax, device) for _ in range(3)]
    rho = torch.exp(0.1 * g)
    p = torch.full_like(rho, 1.0 / gamma)
    vsq = v[0] * v[0] + v[1] * v[1] + v[2] * v[2]
    scale = mach / torch.sqrt(torch.mean(vsq / (gamma * p / rho)))
    v = [c * scale for c in v]
    prim = torch.stack([rho, v[0], v[1], v[2], p])
    e = p / (gamma - 1.0) + 0.5 * rho * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2])
    cons = torch.stack([rho, rho * v[0], rho * v[1], rho * v[2], e])
    return prim.contiguous(), cons.contiguous(), 1.0 / n


def turbulence_mhd_3d(n, seed=1, gamma=5.0 / 3.0, kmax=16, mach=1.0, beta=1.0, device="cuda"):
    """Seeded 3D MHD turbulence on the unit n^3 periodic box: density exp(0.1 g),
    velocities with power ~ k^-2 up to ``kmax`` scaled to rms Mach ``mach``, uniform
    pressure 1/gamma, and face B from the edge-centred vector potential of three
    fields with power ~ k^-3 (div B = 0 to round-off), scaled to plasma beta ``beta``.
    Returns (prim, cons, faceBx, faceBy, faceBz) float64 torch tensors on ``device``
    in the reference's 3D layout, and the cell size."""
    import torch
    rng = np.random.default_rng(seed)
    g = _gaussian_field_3d(rng, n, 2.0, 1.0, kmax, device)
    g = g / g.std(unbiased=False)
    v = [_gaussian_field_3d(rng, n, 2.0, 1.0, kmax, device) for _ in range(3)]
    a = [_gaussian_field_3d(rng, n, 3.0, 1.0, kmax, device) for _ in range(3)]   # A_x, A_y, A_z on edges
    d = 1.0 / n
    rho = torch.exp(0.1 * g)
    p = torch.full_like(rho, 1.0 / gamma)
    vsq = v[0] * v[0] + v[1] * v[1] + v[2] * v[2]
    scale = mach / torch.sqrt(torch.mean(vsq / (gamma * p / rho)))
    v = [c * scale for c in v]

    def up(t, dim):   # t[i+1] - t[i] along dim, periodic
        return torch.roll(t, -1, dims=dim) - t

    # arrays are (y, x, z): dims 0 y, 1 x, 2 z
    bx = up(a[2], 0) / d - up(a[1], 2) / d
    by = up(a[0], 2) / d - up(a[2], 1) / d
    bz = up(a[1], 1) / d - up(a[0], 0) / d
    cbx = 0.5 * (bx + torch.roll(bx, -1, dims=1))
    cby = 0.5 * (by + torch.roll(by, -1, dims=0))
    cbz = 0.5 * (bz + torch.roll(bz, -1, dims=2))
    bscale = torch.sqrt(2.0 * (1.0 / gamma) / beta / torch.mean(cbx * cbx + cby * cby + cbz * cbz))
    bx, by, bz = bx * bscale, by * bscale, bz * bscale
    fbx = torch.cat([bx, bx[:, :1, :]], dim=1)
    fby = torch.cat([by, by[:1, :, :]], dim=0)
    fbz = torch.cat([bz, bz[:, :, :1]], dim=2)
    cbx = 0.5 * (fbx[:, :-1, :] + fbx[:, 1:, :])
    cby = 0.5 * (fby[:-1, :, :] + fby[1:, :, :])
    cbz = 0.5 * (fbz[:, :, :-1] + fbz[:, :, 1:])
    prim = torch.stack([rho, v[0], v[1], v[2], cbx, cby, cbz, p])
    e = p / (gamma - 1.0) + 0.5 * rho * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2])
    e = e + 0.5 * (cbx * cbx + cby * cby + cbz * cbz)
    cons = torch.stack([rho, rho * v[0], rho * v[1], rho * v[2], cbx, cby, cbz, e])
    return (prim.contiguous(), cons.contiguous(), fbx.contiguous(), fby.contiguous(), fbz.contiguous(), d)
