"""Differentiable map from initial fields (rho, vx, vy, p, A_z) to the packed MHD state.

The gradient problem on the step is posed on the fields a user sets up a run
from -- density, in-plane velocity, pressure and the corner vector potential --
rather than on the redundant (prim, cons, face B) triple the step consumes.  The
map is the one the turbulence generator uses (periodic box):

    faceBx = (A_z[j+1, i] - A_z[j, i]) / dy,   faceBy = -(A_z[j, i+1] - A_z[j, i]) / dx
    Bx, By = face averages,  v_z = B_z = 0,  cons from prim

written in torch so that autograd carries the gradient from the packed state
back to the fields (a few elementwise ops; the step's own reverse sweep is the
hand-written one).
"""
from __future__ import annotations

import numpy as np
import torch

from .. import initial_conditions as ic


def _gaussian_field(rng, ny, nx, slope, kmin, kmax):
    """The generator's Gaussian random field on an ny x nx periodic grid (integer
    wavevectors of the box; per-mode power |k|^-slope for kmin <= |k| <= kmax)."""
    if ny == nx:
        return ic._gaussian_field(rng, nx, slope, kmin, kmax)
    kx = np.fft.rfftfreq(nx, d=1.0 / nx)
    ky = np.fft.fftfreq(ny, d=1.0 / ny)
    KX, KY = np.meshgrid(kx, ky)
    k = np.sqrt(KX * KX + KY * KY)
    mask = (k >= kmin) & (k <= kmax)
    amp = np.zeros_like(k)
    amp[mask] = k[mask] ** (-slope / 2.0)
    c = (rng.standard_normal(k.shape) + 1j * rng.standard_normal(k.shape)) * amp
    f = np.fft.irfft2(c, s=(ny, nx))
    return f - f.mean()


def turbulence_fields(n, seed=1, gamma=5.0 / 3.0, kmax_v=16, kmax_a=16, mach=1.0, beta=1.0, ny=None):
    """Seeded turbulence fields on an ny x n periodic unit box (ny defaults to n;
    the turbulence generator's spectra and normalisation), with A_z scaled to
    plasma beta ``beta``.

    Returns dict(rho, vx, vy, p, az, dx, dy, gamma, kmax_v, kmax_a) of NumPy arrays.
    """
    nx = n
    ny = n if ny is None else ny
    rng = np.random.default_rng(seed)
    g = _gaussian_field(rng, ny, nx, 2.0, 1.0, kmax_v)
    g /= g.std()
    vx = _gaussian_field(rng, ny, nx, 2.0, 1.0, kmax_v)
    vy = _gaussian_field(rng, ny, nx, 2.0, 1.0, kmax_v)
    az = _gaussian_field(rng, ny, nx, 3.0, 1.0, kmax_a)
    dx, dy = 1.0 / nx, 1.0 / ny
    rho = np.exp(0.1 * g)
    p = np.full((ny, nx), 1.0 / gamma)
    vscale = mach / np.sqrt(np.mean((vx * vx + vy * vy) / (gamma * p / rho)))
    vx *= vscale
    vy *= vscale
    fbx_u, fby_u = ic.faces_from_potential(az)
    cbx = (fbx_u[:, :-1] + fbx_u[:, 1:]) / (2.0 * dy)
    cby = (fby_u[:-1, :] + fby_u[1:, :]) / (2.0 * dx)
    az = az * np.sqrt(2.0 * (1.0 / gamma) / beta / np.mean(cbx * cbx + cby * cby))
    return dict(rho=rho, vx=vx, vy=vy, p=p, az=az, dx=dx, dy=dy, gamma=gamma, kmax_v=kmax_v, kmax_a=kmax_a)


def turbulence_batch(count=64, seed=0, sizes=tuple(range(128, 1025, 64)), gamma_range=(1.4, 5.0 / 3.0),
                     kmax=16, mach=1.0, cells_per_wave=None, kmax_v=None, kmax_a=None):
    """Uneven batch of turbulence fields: Nx and Ny drawn independently and uniformly
    from ``sizes``, gamma uniformly from ``gamma_range``, rms Mach ``mach``, instance k
    generated with seed ``seed * 100003 + k``.  The density and velocity spectra end at
    ``kmax_v`` and the vector potential's at ``kmax_a`` (both default to ``kmax``).
    With ``cells_per_wave`` each cutoff is further limited to min(Nx, Ny) //
    cells_per_wave, so the shortest wave spans at least that many cells.  Returns a
    list of field dicts with nx, ny added."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        nx = int(rng.choice(sizes))
        ny = int(rng.choice(sizes))
        gamma = float(rng.uniform(*gamma_range))
        kv = kmax if kmax_v is None else kmax_v
        ka = kmax if kmax_a is None else kmax_a
        if cells_per_wave is not None:
            kv = max(1, min(kv, min(nx, ny) // cells_per_wave))
            ka = max(1, min(ka, min(nx, ny) // cells_per_wave))
        f = turbulence_fields(nx, seed=seed * 100003 + k, gamma=gamma, kmax_v=kv, kmax_a=ka, ny=ny, mach=mach)
        f.update(nx=nx, ny=ny)
        out.append(f)
    return out


def perturbed(fields, frac, seed):
    """The fields with rho, vx, vy, p and A_z each multiplied by (1 + frac g), g a
    seeded unit-variance Gaussian random field with the generator's spectrum
    (k^-2 up to kmax_v; k^-3 up to kmax_a for A_z): a smooth perturbation."""
    rng = np.random.default_rng(seed)
    ny, nx = fields["rho"].shape
    out = dict(fields)
    for k in ("rho", "vx", "vy", "p", "az"):
        slope, kmax = (3.0, fields["kmax_a"]) if k == "az" else (2.0, fields["kmax_v"])
        g = _gaussian_field(rng, ny, nx, slope, 1.0, kmax)
        out[k] = fields[k] * (1.0 + frac * (g / g.std()))
    return out


def state_from_fields(rho, vx, vy, p, az, gamma, dx, dy):
    """Packed state ``prim (8) | cons (8) | faceBx | faceBy`` (flattened) from torch fields."""
    fbx_c = (torch.roll(az, -1, dims=0) - az) / dy           # (ny, nx): face i of row j
    fby_c = -(torch.roll(az, -1, dims=1) - az) / dx          # (ny, nx): face j of column i
    fbx = torch.cat([fbx_c, fbx_c[:, :1]], dim=1)
    fby = torch.cat([fby_c, fby_c[:1, :]], dim=0)
    bx = (fbx[:, :-1] + fbx[:, 1:]) / 2.0
    by = (fby[:-1, :] + fby[1:, :]) / 2.0
    zero = torch.zeros_like(rho)
    prim = torch.stack([rho, vx, vy, zero, bx, by, zero, p])
    ke = 0.5 * rho * (vx * vx + vy * vy + zero * zero)
    etot = p / (gamma - 1.0) + ke + 0.5 * (bx * bx + by * by + zero * zero)
    cons = torch.stack([rho, rho * vx, rho * vy, rho * zero, bx, by, zero, etot])
    return torch.cat([prim.reshape(-1), cons.reshape(-1), fbx.reshape(-1), fby.reshape(-1)])


def fields_to_torch(fields, device, requires_grad=False):
    return [torch.tensor(fields[k], dtype=torch.float64, device=device, requires_grad=requires_grad)
            for k in ("rho", "vx", "vy", "p", "az")]
