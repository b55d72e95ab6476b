"""CPU checks of the adjoint's building blocks.

* The NumPy assembly of the SSA stage functions (pythonmhd_gb300.adjoint.assembly_np)
  reproduces the oracle's cycle bit for bit (first order, PLM and PPM, periodic
  and outflow, with and without the entropy fix).
* Its reverse sweep matches central finite differences of the oracle's cycle
  along random directions, on generic states (perturbed away from the exact
  ties -- uniform p, v_z = B_z = 0 -- where the limiters and clamps have kinks).
* The CUDA stage functions can be generated from the same definitions.
"""
import numpy as np
import pytest

from oracle import mhd2d
from pythonmhd_gb300 import initial_conditions as ic
from pythonmhd_gb300.adjoint import assembly_np, codegen
from tests.golden import cases

GAMMA = 5.0 / 3.0


@pytest.mark.parametrize("name", ["ot_ppm", "rand_outflow_ppm", "rand_px_oy_ppm", "rand_efix_small_eps",
                                  "zero_bx", "floors", "supersonic", "tiny_periodic"])
@pytest.mark.parametrize("order", [0, 1, 2])
def test_numpy_assembly_forward_is_bitwise(name, order):
    c = cases.build("mhd", name)
    dt = mhd2d.calc_dt(c["cons"], c["fbx"], c["fby"], c["gamma"], c["cfl"], c["dx"], c["dy"])
    args = (dt, c["dx"], c["dy"], c["bcx"], c["bcy"], c["gamma"], c["min_d"], c["min_p"], c["min_e"], order,
            c["efix"], c["eps"])
    got = assembly_np.Cycle(c["prim"], c["cons"], c["fbx"], c["fby"], *args).outputs()
    want = mhd2d.cycle(c["prim"], c["cons"], c["fbx"], c["fby"], *args)
    for a, b in zip(got, want):
        np.testing.assert_array_equal(a, b)


def generic_state(kind, bc, seed):
    rng = np.random.default_rng(seed)
    if kind == "turb":
        p, _, bx, by, dx, dy = ic.turbulence(24, seed=3, kmax_v=6, kmax_a=4)
        p = p[:, :, :20].copy()
        bx = bx[:, :21].copy()
        by = by[:, :20].copy()
    else:
        p, _, bx, by, dx, dy = ic.orszag_tang(20, 24)
    p = p * (1 + 0.01 * rng.standard_normal(p.shape))
    p[3] += 0.01 * rng.standard_normal(p[3].shape)
    p[6] += 0.01 * rng.standard_normal(p[6].shape)
    c = ic.prim_to_cons_mhd(p, GAMMA)
    return p, c, bx, by, dx, dy


@pytest.mark.parametrize("kind,bc,order,efix", [("turb", 1, 1, False), ("ot", 1, 0, False),
                                                ("ot", 0, 1, True), ("turb", 0, 0, True),
                                                ("turb", 1, 2, False), ("ot", 0, 2, True)])
def test_numpy_reverse_matches_finite_differences(kind, bc, order, efix):
    p, c, bx, by, dx, dy = generic_state(kind, bc, seed=7)
    dt = mhd2d.calc_dt(c, bx, by, GAMMA, 0.4, dx, dy)
    args = (dt, dx, dy, bc, bc, GAMMA, 1e-12, 1e-12, 1e-12, order, efix, 0.3)
    x0 = [p, c, bx, by]
    rng = np.random.default_rng(11)
    wts = [rng.standard_normal(a.shape) for a in x0]

    def loss(x):
        out = mhd2d.cycle(*x, *args)
        return sum(float(np.sum(w * o)) for w, o in zip(wts, out))

    g = assembly_np.Cycle(*x0, *args).reverse(*wts)
    for _ in range(2):
        d = [rng.standard_normal(a.shape) * np.maximum(np.abs(a), 1e-3) for a in x0]
        ad = sum(float(np.sum(gg * dd)) for gg, dd in zip(g, d))
        # the step is piecewise smooth (limiters, clamps, upwind switches): a
        # central difference whose stencil straddles a kink is off by O(eps), so
        # the best of three step sizes must agree
        errs = []
        for eps in (1e-6, 1e-7, 1e-8):
            fd = (loss([a + eps * b for a, b in zip(x0, d)]) - loss([a - eps * b for a, b in zip(x0, d)])) / (2 * eps)
            errs.append(abs(ad - fd) / abs(fd))
        assert min(errs) <= 1e-6, (ad, errs)


def test_codegen_emits_every_stage():
    src = codegen.generate()
    for name, *_ in codegen.STAGES:
        assert f"void g_{name}_fwd(" in src
        assert f"void g_{name}_rev(" in src
        assert f"g_{name}_NI" in src


@pytest.mark.parametrize("name,order", [("ot_ppm", 1), ("rand_outflow_ppm", 1), ("rand_efix_small_eps", 1),
                                        ("zero_b", 1), ("zero_btran", 1), ("zero_bx", 0),
                                        ("ot_ppm", 2), ("rand_outflow_ppm", 2),
                                        ("rand_px_oy_ppm", 0), ("floors", 1)])
def test_torch_transcription_forward_is_bitwise(name, order):
    torch = pytest.importorskip("torch")
    c = cases.build("mhd", name)
    dt = mhd2d.calc_dt(c["cons"], c["fbx"], c["fby"], c["gamma"], c["cfl"], c["dx"], c["dy"])
    args = (dt, c["dx"], c["dy"], c["bcx"], c["bcy"], c["gamma"], c["min_d"], c["min_p"], c["min_e"], order,
            c["efix"], c["eps"])
    xs = [torch.tensor(c[k]) for k in ("prim", "cons", "fbx", "fby")]
    got = assembly_np.Cycle(*xs, *args, backend="torch").outputs()
    want = mhd2d.cycle(c["prim"], c["cons"], c["fbx"], c["fby"], *args)
    for a, b in zip(got, want):
        np.testing.assert_array_equal(a.numpy(), b)


@pytest.mark.parametrize("kind,bc,order,efix", [("turb", 1, 1, False), ("ot", 0, 1, True), ("ot", 1, 0, False),
                                                ("turb", 1, 2, False)])
def test_torch_autograd_matches_numpy_reverse(kind, bc, order, efix):
    """torch's reverse mode and forward mode through the torch transcription agree
    with the hand-written reverse sweep."""
    torch = pytest.importorskip("torch")
    import torch.autograd.forward_ad as fwAD
    p, c, bx, by, dx, dy = generic_state(kind, bc, seed=7)
    dt = mhd2d.calc_dt(c, bx, by, GAMMA, 0.4, dx, dy)
    args = (dt, dx, dy, bc, bc, GAMMA, 1e-12, 1e-12, 1e-12, order, efix, 0.3)
    rng = np.random.default_rng(11)
    wts = [rng.standard_normal(a.shape) for a in (p, c, bx, by)]
    want = assembly_np.Cycle(p, c, bx, by, *args).reverse(*wts)
    xs = [torch.tensor(a, requires_grad=True) for a in (p, c, bx, by)]
    outs = assembly_np.Cycle(*xs, *args, backend="torch").outputs()
    sum(torch.sum(torch.tensor(w) * o) for w, o in zip(wts, outs)).backward()
    for x, w in zip(xs, want):
        scale = np.max(np.abs(w))
        assert np.max(np.abs(x.grad.numpy() - w)) <= 1e-12 * scale
    d = [rng.standard_normal(a.shape) for a in (p, c, bx, by)]
    with fwAD.dual_level():
        duals = [fwAD.make_dual(torch.tensor(a), torch.tensor(dd)) for a, dd in zip((p, c, bx, by), d)]
        outs = assembly_np.Cycle(*duals, *args, backend="torch").outputs()
        jvp = sum(float(torch.sum(torch.tensor(w) * fwAD.unpack_dual(o).tangent)) for w, o in zip(wts, outs))
    vjp = sum(float(np.sum(g * dd)) for g, dd in zip(want, d))
    assert abs(jvp - vjp) <= 1e-12 * abs(vjp)
