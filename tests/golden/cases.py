"""Seeded input states shared by the golden-fixture generator and the parity tests.

Each case is (name, physics, builder); ``builder()`` returns a dict with the
state arrays and the evolve parameters. The cases are chosen to drive every
branch of the step: PPM and first-order reconstruction, both boundary
conditions on each axis, the entropy fix, zero normal/transverse B, exactly
zero mass flux at the corners, supersonic upwinding, the density/pressure
floors, and the tEnd clip of dt.
"""
from __future__ import annotations

import math

import numpy as np

from pythonmhd_gb300 import initial_conditions as ic

G53 = 5.0 / 3.0


def _params(**kw):
    p = dict(t_start=0.0, t_end=10.0, start_cycle=0, max_cycles=2, gamma=G53, cfl=0.4,
             min_d=1e-12, min_p=1e-12, min_e=1e-12, order=2, efix=False, eps=0.5,
             bcx=ic.PERIODIC, bcy=ic.PERIODIC)
    p.update(kw)
    return p


def _smooth_random(rng, ny, nx, kmax=3):
    """A smooth random field on the grid (sum of a few Fourier modes)."""
    x = (np.arange(nx) + 0.5) / nx
    y = (np.arange(ny) + 0.5) / ny
    X, Y = np.meshgrid(x, y)
    f = np.zeros((ny, nx))
    for _ in range(4):
        kx, ky = rng.integers(1, kmax + 1, size=2)
        ph = rng.uniform(0, 2 * math.pi, size=2)
        f += rng.standard_normal() * np.sin(2 * math.pi * kx * X + ph[0]) * np.cos(2 * math.pi * ky * Y + ph[1])
    return f / 4.0


def _mhd_state(prim, gamma, bcx, bcy):
    fbx, fby = ic.faces_from_cells(prim[4], prim[5], bcx, bcy)
    return prim, ic.prim_to_cons_mhd(prim, gamma), fbx, fby


def mhd_cases():
    out = []

    def ot(nx, ny, faces, **kw):
        prim, cons, fbx, fby, dx, dy = ic.orszag_tang(nx, ny, gamma=G53, faces=faces)
        return dict(prim=prim, cons=cons, fbx=fbx, fby=fby, dx=dx, dy=dy, **_params(**kw))

    out.append(("ot_ppm", lambda: ot(24, 16, "potential", max_cycles=3)))
    out.append(("ot_order0", lambda: ot(24, 16, "potential", order=0, max_cycles=3)))
    out.append(("ot_cellfaces_efix", lambda: ot(20, 20, "cells", efix=True, eps=0.5)))
    out.append(("ot_tend_clip", lambda: ot(16, 16, "potential", t_end=0.012, max_cycles=50)))
    out.append(("ot_no_cycle", lambda: ot(8, 8, "potential", start_cycle=5, max_cycles=5)))

    def turb():
        prim, cons, fbx, fby, dx, dy = ic.turbulence(32, seed=3, gamma=G53, kmax_v=8, kmax_a=4)
        return dict(prim=prim, cons=cons, fbx=fbx, fby=fby, dx=dx, dy=dy, **_params())
    out.append(("turb_ppm", turb))

    def rand(seed, ny, nx, bcx, bcy, b_on=(1, 1, 1), v_scale=0.5, rho_lo=0.5, **kw):
        rng = np.random.default_rng(seed)
        prim = np.zeros((8, ny, nx))
        prim[0] = rho_lo + np.abs(1.0 + _smooth_random(rng, ny, nx))
        for k in (1, 2, 3):
            prim[k] = v_scale * _smooth_random(rng, ny, nx)
        for k, on in zip((4, 5, 6), b_on):
            prim[k] = on * (0.7 * _smooth_random(rng, ny, nx) + 0.3 * rng.standard_normal())
        prim[7] = 0.4 + np.abs(0.5 + _smooth_random(rng, ny, nx))
        prim, cons, fbx, fby = _mhd_state(prim, G53, bcx, bcy)
        return dict(prim=prim, cons=cons, fbx=fbx, fby=fby, dx=1.0 / nx, dy=1.0 / ny,
                    **_params(bcx=bcx, bcy=bcy, **kw))

    out.append(("rand_outflow_ppm", lambda: rand(11, 18, 22, 0, 0)))
    out.append(("rand_px_oy_ppm", lambda: rand(12, 20, 14, 1, 0)))
    out.append(("rand_ox_py_order0", lambda: rand(13, 14, 20, 0, 1, order=0)))
    out.append(("rand_efix_small_eps", lambda: rand(14, 16, 16, 1, 1, efix=True, eps=0.05)))
    out.append(("zero_b", lambda: rand(15, 16, 18, 0, 0, b_on=(0, 0, 0))))
    out.append(("zero_bx", lambda: _zero_bx(16)))
    out.append(("zero_btran", lambda: _zero_btran(17)))
    out.append(("uniform_static", lambda: _uniform(static=True)))
    out.append(("supersonic", lambda: _supersonic(18)))
    out.append(("floors", lambda: rand(19, 16, 16, 0, 1, v_scale=2.0, rho_lo=0.01,
                                      min_d=0.8, min_p=0.6, min_e=1.5)))
    out.append(("tiny_outflow", lambda: rand(20, 3, 5, 0, 0)))
    out.append(("tiny_periodic", lambda: rand(21, 2, 4, 1, 1)))
    return out


def _zero_bx(seed):
    rng = np.random.default_rng(seed)
    ny, nx = 16, 16
    prim = np.zeros((8, ny, nx))
    prim[0] = 1.0 + 0.2 * _smooth_random(rng, ny, nx)
    prim[1] = 0.3 * _smooth_random(rng, ny, nx)
    prim[2] = 0.3 * _smooth_random(rng, ny, nx)
    prim[5] = 0.5 + 0.2 * _smooth_random(rng, ny, nx)
    prim[6] = 0.2 * _smooth_random(rng, ny, nx)
    prim[7] = 1.0 + 0.2 * _smooth_random(rng, ny, nx)
    prim, cons, fbx, fby = _mhd_state(prim, G53, 1, 1)
    return dict(prim=prim, cons=cons, fbx=fbx, fby=fby, dx=1 / nx, dy=1 / ny, **_params())


def _zero_btran(seed):
    """A 1D-invariant Brio-Wu-like state: only Bx (normal in x) is nonzero."""
    rng = np.random.default_rng(seed)
    ny, nx = 6, 24
    prim = np.zeros((8, ny, nx))
    left = np.arange(nx) < nx // 2
    prim[0] = np.where(left, 1.0, 0.125)[None, :].repeat(ny, 0)
    prim[7] = np.where(left, 1.0, 0.1)[None, :].repeat(ny, 0)
    prim[4] = 0.75
    prim[1] = 0.01 * rng.standard_normal((ny, nx))
    prim, cons, fbx, fby = _mhd_state(prim, 2.0, 0, 1)
    return dict(prim=prim, cons=cons, fbx=fbx, fby=fby, dx=1 / nx, dy=1 / nx,
                **_params(gamma=2.0, bcx=0, bcy=1))


def _uniform(static):
    ny, nx = 8, 10
    prim = np.zeros((8, ny, nx))
    prim[0] = 1.0
    prim[4] = 0.3
    prim[5] = -0.2
    prim[6] = 0.1
    prim[7] = 0.6
    if not static:
        prim[1] = 0.2
    prim, cons, fbx, fby = _mhd_state(prim, G53, 1, 0)
    return dict(prim=prim, cons=cons, fbx=fbx, fby=fby, dx=0.1, dy=0.125, **_params(bcy=0))


def _supersonic(seed):
    rng = np.random.default_rng(seed)
    ny, nx = 12, 12
    prim = np.zeros((8, ny, nx))
    prim[0] = 1.0 + 0.1 * _smooth_random(rng, ny, nx)
    prim[1] = 6.0 + 0.2 * _smooth_random(rng, ny, nx)
    prim[2] = -6.0 + 0.2 * _smooth_random(rng, ny, nx)
    prim[4] = 0.2
    prim[5] = 0.1 * _smooth_random(rng, ny, nx)
    prim[7] = 0.5 + 0.05 * _smooth_random(rng, ny, nx)
    prim, cons, fbx, fby = _mhd_state(prim, G53, 1, 1)
    return dict(prim=prim, cons=cons, fbx=fbx, fby=fby, dx=1 / nx, dy=1 / ny, **_params())


def hydro_cases():
    out = []

    def rand(seed, ny, nx, bcx, bcy, v_scale=0.5, rho_lo=0.5, **kw):
        rng = np.random.default_rng(seed)
        prim = np.zeros((5, ny, nx))
        prim[0] = rho_lo + np.abs(1.0 + _smooth_random(rng, ny, nx))
        for k in (1, 2, 3):
            prim[k] = v_scale * _smooth_random(rng, ny, nx)
        prim[4] = 0.4 + np.abs(0.5 + _smooth_random(rng, ny, nx))
        return dict(prim=prim, cons=ic.prim_to_cons_hydro(prim, G53), dx=1.0 / nx, dy=1.0 / ny,
                    **_params(bcx=bcx, bcy=bcy, **kw))

    def blast():
        ny, nx = 20, 24
        x = (np.arange(nx) + 0.5) / nx - 0.5
        y = (np.arange(ny) + 0.5) / ny - 0.5
        X, Y = np.meshgrid(x, y)
        prim = np.zeros((5, ny, nx))
        prim[0] = 1.0
        prim[4] = np.where(X * X + Y * Y < 0.04, 10.0, 0.1)
        return dict(prim=prim, cons=ic.prim_to_cons_hydro(prim, 1.4), dx=1 / nx, dy=1 / ny,
                    **_params(gamma=1.4, bcx=0, bcy=0, max_cycles=3))

    out.append(("blast_ppm", blast))
    out.append(("rand_periodic_ppm_efix", lambda: rand(31, 16, 20, 1, 1, efix=True, eps=0.3)))
    out.append(("rand_order0", lambda: rand(32, 14, 18, 1, 0, order=0)))
    out.append(("rand_outflow_ppm", lambda: rand(33, 18, 14, 0, 0)))
    out.append(("supersonic", lambda: rand(34, 12, 12, 1, 1, v_scale=0.2) | {}))
    out.append(("floors", lambda: rand(35, 16, 16, 0, 1, v_scale=2.0, rho_lo=0.01,
                                       min_d=0.8, min_p=0.6)))
    out.append(("tiny", lambda: rand(36, 3, 4, 1, 0)))
    out.append(("tend_clip", lambda: rand(37, 10, 10, 1, 1, t_end=0.03, max_cycles=40)))
    return out


def supersonic_hydro_fix(case):
    """Shift the hydro 'supersonic' case to |v| > c in both directions."""
    prim = case["prim"].copy()
    prim[1] += 4.0
    prim[2] -= 4.0
    case["prim"] = prim
    case["cons"] = ic.prim_to_cons_hydro(prim, case["gamma"])
    return case


def build(physics, name):
    table = dict(mhd_cases() if physics == "mhd" else hydro_cases())
    case = table[name]()
    if physics == "hydro" and name == "supersonic":
        case = supersonic_hydro_fix(case)
    return case


def names(physics):
    return [n for n, _ in (mhd_cases() if physics == "mhd" else hydro_cases())]


# ---------------------------------------------------------------------------
# 1D cases (evolve_1D_mhd / evolve_1D_hydro): state arrays (nvars, N)
# ---------------------------------------------------------------------------
def _p1(**kw):
    p = dict(t_start=0.0, t_end=10.0, start_cycle=0, max_cycles=6, gamma=G53, cfl=0.4,
             min_d=1e-12, min_p=1e-12, min_e=1e-12, order=2, efix=False, eps=0.5, bcx=ic.OUTFLOW)
    p.update(kw)
    return p


def _brio_wu(n, gamma=2.0):
    prim = np.zeros((8, n))
    left = np.arange(n) < n // 2
    prim[0] = np.where(left, 1.0, 0.125)
    prim[4] = 0.75
    prim[5] = np.where(left, 1.0, -1.0)
    prim[7] = np.where(left, 1.0, 0.1)
    return prim, ic.prim_to_cons_mhd(prim, gamma)


def _random_mhd_1d(n, seed, gamma=G53):
    rng = np.random.default_rng(seed)
    x = (np.arange(n) + 0.5) / n
    prim = np.zeros((8, n))
    prim[0] = 1.0 + 0.3 * np.sin(2 * math.pi * x) + 0.05 * rng.standard_normal(n)
    prim[1] = 0.4 * np.cos(2 * math.pi * x) + 0.05 * rng.standard_normal(n)
    prim[2] = 0.2 * np.sin(4 * math.pi * x)
    prim[3] = 0.1 * np.cos(6 * math.pi * x)
    prim[4] = 0.6
    prim[5] = 0.5 * np.sin(2 * math.pi * x + 0.3)
    prim[6] = 0.3 * np.cos(2 * math.pi * x + 0.1)
    prim[7] = 0.8 + 0.2 * np.cos(2 * math.pi * x) + 0.02 * rng.standard_normal(n)
    return prim, ic.prim_to_cons_mhd(prim, gamma)


def mhd1d_cases():
    def brio_wu(order, **kw):
        def f():
            prim, cons = _brio_wu(64)
            return dict(prim=prim, cons=cons, dx=1.0 / 64, **_p1(gamma=2.0, order=order, max_cycles=12, **kw))
        return f

    def random(order, bc, **kw):
        def f():
            prim, cons = _random_mhd_1d(48, 3)
            return dict(prim=prim, cons=cons, dx=1.0 / 48, **_p1(order=order, bcx=bc, **kw))
        return f

    def tend_clip():
        prim, cons = _brio_wu(40)
        return dict(prim=prim, cons=cons, dx=1.0 / 40, **_p1(gamma=2.0, t_end=0.011, max_cycles=50))

    def floors():
        prim, cons = _random_mhd_1d(32, 5)
        return dict(prim=prim, cons=cons, dx=1.0 / 32, **_p1(min_d=0.9, min_p=0.75, bcx=ic.PERIODIC))

    return [("brio_wu_ppm", brio_wu(2)), ("brio_wu_order0", brio_wu(0)),
            ("brio_wu_efix", brio_wu(2, efix=True, eps=0.3)),
            ("random_periodic_ppm", random(2, ic.PERIODIC)), ("random_outflow_ppm", random(2, ic.OUTFLOW)),
            ("random_periodic_order0", random(0, ic.PERIODIC)), ("tend_clip", tend_clip), ("floors", floors)]


def _sod(n, gamma=1.4):
    prim = np.zeros((5, n))
    left = np.arange(n) < n // 2
    prim[0] = np.where(left, 1.0, 0.125)
    prim[4] = np.where(left, 1.0, 0.1)
    return prim, ic.prim_to_cons_hydro(prim, gamma)


def hydro1d_cases():
    def sod(order, **kw):
        def f():
            prim, cons = _sod(64)
            p = dict(gamma=1.4, order=order, max_cycles=12)
            p.update(kw)
            return dict(prim=prim, cons=cons, dx=1.0 / 64, **_p1(**p))
        return f

    def random(order, bc, **kw):
        def f():
            rng = np.random.default_rng(7)
            n = 40
            x = (np.arange(n) + 0.5) / n
            prim = np.zeros((5, n))
            prim[0] = 1.0 + 0.3 * np.sin(2 * math.pi * x) + 0.05 * rng.standard_normal(n)
            prim[1] = 0.5 * np.cos(2 * math.pi * x)
            prim[2] = 0.2 * np.sin(2 * math.pi * x)
            prim[3] = 0.1 * np.cos(4 * math.pi * x)
            prim[4] = 0.7 + 0.1 * np.cos(2 * math.pi * x)
            return dict(prim=prim, cons=ic.prim_to_cons_hydro(prim, 1.4), dx=1.0 / n,
                        **_p1(gamma=1.4, order=order, bcx=bc, **kw))
        return f

    # (the reference's 1D hydro PPM with periodic boundaries raises in np.append,
    # Source/Reconstruction_PPM_Hydro_HelperModule.py:355, so no periodic PPM case)
    return [("sod_ppm", sod(2)), ("sod_order0", sod(0)), ("sod_efix", sod(2, efix=True, eps=0.4)),
            ("random_outflow_ppm", random(2, ic.OUTFLOW)), ("random_periodic_order0", random(0, ic.PERIODIC)),
            ("random_outflow_order0", random(0, ic.OUTFLOW)), ("tend_clip", sod(2, t_end=0.013, max_cycles=50))]


def build1d(physics, name):
    table = dict(mhd1d_cases() if physics == "mhd" else hydro1d_cases())
    return table[name]()


def names1d(physics):
    return [n for n, _ in (mhd1d_cases() if physics == "mhd" else hydro1d_cases())]


# ----------------------------------------------------------------------------
# 3D hydro (evolve_3D_hydro): arrays (nvars, ny, nx, nz).  The reference's 3D
# step raises with an outflow x boundary (Source/EvolveFunctions_Hydro.py:700-703
# reshape a z-flux slab to a y-flux shape), so every 3D case has a periodic x.
# ----------------------------------------------------------------------------
def _p3(**kw):
    p = dict(t_start=0.0, t_end=10.0, start_cycle=0, max_cycles=3, gamma=1.4, cfl=0.4, min_d=1e-12,
             min_p=1e-12, min_e=1e-12, order=2, efix=False, eps=0.5, bcx=ic.PERIODIC, bcy=ic.PERIODIC,
             bcz=ic.PERIODIC)
    p.update(kw)
    return p


def _random_hydro_3d(ny, nx, nz, seed, gamma=1.4, mach=0.5):
    """Smooth random fields (a few 3D Fourier modes) plus a little cell noise."""
    rng = np.random.default_rng(seed)
    y, x, z = np.meshgrid((np.arange(ny) + 0.5) / ny, (np.arange(nx) + 0.5) / nx, (np.arange(nz) + 0.5) / nz,
                          indexing="ij")

    def field():
        f = np.zeros((ny, nx, nz))
        for _ in range(3):
            k = rng.integers(1, 3, size=3)
            ph = rng.uniform(0, 2 * math.pi, size=3)
            f += (rng.standard_normal() * np.sin(2 * math.pi * k[0] * x + ph[0]) * np.cos(2 * math.pi * k[1] * y + ph[1])
                  * np.cos(2 * math.pi * k[2] * z + ph[2]))
        return f / 3.0 + 0.02 * rng.standard_normal((ny, nx, nz))

    prim = np.zeros((5, ny, nx, nz))
    prim[0] = 1.0 + 0.3 * field()
    prim[0] = np.maximum(prim[0], 0.3)
    prim[1] = mach * field()
    prim[2] = mach * field()
    prim[3] = mach * field()
    prim[4] = 1.0 / gamma + 0.2 * field()
    prim[4] = np.maximum(prim[4], 0.1)
    return prim, ic.prim_to_cons_hydro(prim, gamma)


def _blast_3d(ny, nx, nz, gamma=1.4):
    prim = np.zeros((5, ny, nx, nz))
    prim[0] = 1.0
    prim[4] = 0.1
    prim[4, ny // 2 - 1:ny // 2 + 1, nx // 2 - 1:nx // 2 + 1, nz // 2 - 1:nz // 2 + 1] = 10.0
    return prim, ic.prim_to_cons_hydro(prim, gamma)


def hydro3d_cases():
    def rnd(shape=(6, 8, 5), seed=11, mach=0.5, **kw):
        def f():
            ny, nx, nz = shape
            prim, cons = _random_hydro_3d(ny, nx, nz, seed, mach=mach)
            return dict(prim=prim, cons=cons, dx=1.0 / nx, dy=1.0 / ny, dz=1.0 / nz, **_p3(**kw))
        return f

    def blast(**kw):
        def f():
            prim, cons = _blast_3d(8, 8, 8)
            return dict(prim=prim, cons=cons, dx=1.0 / 8, dy=1.0 / 8, dz=1.0 / 8, **_p3(**kw))
        return f

    def floors(order):
        # one interior cell below both floors: the reference's 3D floor routine raises
        # while it formats its message once three or more values of one array are
        # floored (Source/PrimCons_HelperModule.py:537-548 index with the message
        # loop's counter), so only that cell's own face states are floored
        def f():
            prim, _ = _random_hydro_3d(6, 8, 5, 15, mach=0.3)
            prim[0, 3, 4, 2] = 0.2
            prim[4, 3, 4, 2] = 0.05
            return dict(prim=prim, cons=ic.prim_to_cons_hydro(prim, 1.4), dx=1.0 / 8, dy=1.0 / 6, dz=1.0 / 5,
                        **_p3(min_d=0.25, min_p=0.06, order=order, max_cycles=1))
        return f

    def uniform():
        prim = np.zeros((5, 4, 5, 6))
        prim[0] = 1.0
        prim[4] = 0.6
        return dict(prim=prim, cons=ic.prim_to_cons_hydro(prim, 1.4), dx=0.2, dy=0.25, dz=1.0 / 6, **_p3())

    O, P = ic.OUTFLOW, ic.PERIODIC
    return [("random_ppm", rnd()), ("random_ppm_ybc_outflow", rnd(bcy=O)),
            ("random_ppm_zbc_outflow", rnd(bcz=O)), ("random_ppm_yzbc_outflow", rnd(bcy=O, bcz=O, seed=12)),
            ("random_order0", rnd(order=0)), ("random_order0_yzbc_outflow", rnd(order=0, bcy=O, bcz=O)),
            ("random_efix", rnd(efix=True, eps=0.4)), ("supersonic", rnd(mach=2.5, seed=13)),
            ("supersonic_order0_efix", rnd(mach=2.5, seed=14, order=0, efix=True, eps=0.3)),
            ("floors_ppm", floors(2)), ("floors_order0", floors(0)), ("blast_ppm", blast(max_cycles=4)),
            ("blast_tend_clip", blast(t_end=0.011, max_cycles=50)), ("uniform_static", uniform),
            ("no_cycle", rnd(start_cycle=4, max_cycles=4)), ("cube_4", rnd(shape=(4, 4, 4), seed=16))]


def build3d(physics, name):
    return dict(hydro3d_cases() if physics == "hydro" else mhd3d_cases())[name]()


def names3d(physics):
    return [n for n, _ in (hydro3d_cases() if physics == "hydro" else mhd3d_cases())]


# ----------------------------------------------------------------------------
# 3D MHD (evolve_3D_mhd): prim/cons (8, ny, nx, nz), faceBx (ny, nx+1, nz),
# faceBy (ny+1, nx, nz), faceBz (ny, nx, nz+1).  The reference runs PPM on cubes
# for every boundary combination and on other boxes when y and z are periodic;
# its first-order path needs a periodic y (Source/EvolveFunctions_MHD.py:857-866
# reshape an outflow y slab to 3 dimensions).
# ----------------------------------------------------------------------------
def _random_mhd_3d(ny, nx, nz, seed, gamma=G53, mach=0.6, b0=0.5):
    """Smooth random fields; face B from a smooth random edge vector potential, so the
    discrete divergence of B is zero."""
    rng = np.random.default_rng(seed)

    def smooth(y, x, z):
        f = np.zeros(np.broadcast(y, x, z).shape)
        for _ in range(3):
            k = rng.integers(1, 3, size=3)
            ph = rng.uniform(0, 2 * math.pi, size=3)
            f = f + rng.standard_normal() * (np.sin(2 * math.pi * k[0] * x + ph[0]) * np.cos(2 * math.pi * k[1] * y + ph[1])
                                             * np.cos(2 * math.pi * k[2] * z + ph[2]))
        return f / 3.0

    dx, dy, dz = 1.0 / nx, 1.0 / ny, 1.0 / nz
    yc, xc, zc = (np.arange(ny) + 0.5) * dy, (np.arange(nx) + 0.5) * dx, (np.arange(nz) + 0.5) * dz
    yf, xf, zf = np.arange(ny + 1) * dy, np.arange(nx + 1) * dx, np.arange(nz + 1) * dz
    Y, X, Z = np.meshgrid(yc, xc, zc, indexing="ij")
    ax = b0 * smooth(*np.meshgrid(yf, xc, zf, indexing="ij")) * dy
    ay = b0 * smooth(*np.meshgrid(yc, xf, zf, indexing="ij")) * dx
    az = b0 * smooth(*np.meshgrid(yf, xf, zc, indexing="ij")) * dx
    fbx = (az[1:, :, :] - az[:-1, :, :]) / dy - (ay[:, :, 1:] - ay[:, :, :-1]) / dz
    fby = (ax[:, :, 1:] - ax[:, :, :-1]) / dz - (az[:, 1:, :] - az[:, :-1, :]) / dx
    fbz = (ay[:, 1:, :] - ay[:, :-1, :]) / dx - (ax[1:, :, :] - ax[:-1, :, :]) / dy
    prim = np.zeros((8, ny, nx, nz))
    prim[0] = 1.0 + 0.25 * smooth(Y, X, Z) + 0.01 * rng.standard_normal((ny, nx, nz))
    prim[1] = mach * smooth(Y, X, Z)
    prim[2] = mach * smooth(Y, X, Z)
    prim[3] = mach * smooth(Y, X, Z)
    prim[4] = 0.5 * (fbx[:, :-1] + fbx[:, 1:])
    prim[5] = 0.5 * (fby[:-1] + fby[1:])
    prim[6] = 0.5 * (fbz[:, :, :-1] + fbz[:, :, 1:])
    prim[7] = 0.6 + 0.1 * smooth(Y, X, Z)
    return prim, ic.prim_to_cons_mhd(prim, gamma), fbx, fby, fbz, dx, dy, dz


def mhd3d_cases():
    def rnd(shape=(6, 6, 6), seed=31, **kw):
        def f():
            prim, cons, fbx, fby, fbz, dx, dy, dz = _random_mhd_3d(*shape, seed)
            p = dict(_p3(gamma=G53, efix=True, max_cycles=2), **kw)
            return dict(prim=prim, cons=cons, fbx=fbx, fby=fby, fbz=fbz, dx=dx, dy=dy, dz=dz, **p)
        return f

    O, P = ic.OUTFLOW, ic.PERIODIC

    def floors():
        prim, cons, fbx, fby, fbz, dx, dy, dz = _random_mhd_3d(6, 6, 6, 37)
        prim[0, 3, 2, 3] = 0.3
        prim[7, 3, 2, 3] = 0.05
        cons = ic.prim_to_cons_mhd(prim, G53)
        return dict(prim=prim, cons=cons, fbx=fbx, fby=fby, fbz=fbz, dx=dx, dy=dy, dz=dz,
                    **_p3(gamma=G53, efix=True, max_cycles=1, min_d=0.35, min_p=0.06))

    return [("ppm_periodic", rnd()), ("ppm_periodic_noncubic", rnd(shape=(4, 5, 6), seed=32)),
            ("ppm_outflow", rnd(bcx=O, bcy=O, bcz=O)), ("ppm_x_outflow", rnd(bcx=O, seed=33)),
            ("ppm_y_outflow", rnd(bcy=O, seed=34)), ("ppm_z_outflow", rnd(bcz=O, seed=35)),
            ("ppm_xz_outflow_no_efix", rnd(bcx=O, bcz=O, efix=False)), ("ppm_xy_outflow", rnd(bcx=O, bcy=O, seed=36)),
            ("order0_periodic", rnd(order=0)), ("order0_xz_outflow", rnd(order=0, bcx=O, bcz=O, seed=38)),
            ("order0_noncubic_periodic", rnd(shape=(4, 5, 6), order=0, seed=39)),
            ("ppm_8cube_4cycles", rnd(shape=(8, 8, 8), seed=40, max_cycles=4)),
            ("tend_clip", rnd(t_end=0.011, max_cycles=50)), ("no_cycle", rnd(start_cycle=3, max_cycles=3)),
            ("floors", floors)]


