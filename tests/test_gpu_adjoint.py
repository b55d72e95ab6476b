"""GPU adjoint of the MHD step (mhd2d_adj_* through pythonmhd_gb300.adjoint.device).

* Its forward cycle equals the oracle's cycle bit for bit (first order, PLM and PPM).
* Its vector-Jacobian product of one cycle equals the NumPy assembly's reverse
  sweep (itself checked against finite differences on the CPU) to round-off:
  the GPU scatters input adjoints with atomic adds, so the summation order of
  the few terms landing on one value differs.
* A checkpointed multi-cycle backward equals the chain of one-cycle products,
  for any checkpoint interval, and its forward equals the exact-arithmetic step.
* The gradient of a density-matching loss with respect to the initial fields
  (rho, vx, vy, p, A_z) agrees with central finite differences (dt frozen).
"""
import numpy as np
import pytest
import torch

from oracle import mhd2d
from pythonmhd_gb300 import initial_conditions as ic
from pythonmhd_gb300.adjoint import assembly_np, fields
from pythonmhd_gb300.adjoint.device import Adjoint2D, evolve
from pythonmhd_gb300.solver import Grid2D
from tests.golden import cases
from tests.gpu_util import field_rel_err
from tests.test_adjoint_cpu import generic_state

pytestmark = pytest.mark.gpu
GAMMA = 5.0 / 3.0
CASES = ["ot_ppm", "rand_outflow_ppm", "rand_px_oy_ppm", "rand_efix_small_eps", "zero_bx", "floors",
         "supersonic", "tiny_periodic"]


def _adj(c, order):
    ny, nx = c["prim"].shape[1:]
    return Adjoint2D(ny, nx, c["dx"], c["dy"], c["bcx"], c["bcy"], c["gamma"], recon=order,
                     entropy_fix=c["efix"], eps=c["eps"], min_d=c["min_d"], min_p=c["min_p"], min_e=c["min_e"])


def _np(parts):
    return [t.cpu().numpy() for t in parts]


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("order", [0, 1, 2])
def test_cycle_bitwise_vs_oracle(name, order):
    c = cases.build("mhd", name)
    dt = mhd2d.calc_dt(c["cons"], c["fbx"], c["fby"], c["gamma"], c["cfl"], c["dx"], c["dy"])
    a = _adj(c, order)
    out = a.cycle(a.pack(c["prim"], c["cons"], c["fbx"], c["fby"]), dt)
    want = mhd2d.cycle(c["prim"], c["cons"], c["fbx"], c["fby"], dt, c["dx"], c["dy"], c["bcx"], c["bcy"],
                       c["gamma"], c["min_d"], c["min_p"], c["min_e"], order, c["efix"], c["eps"])
    for g, w in zip(_np(a.unpack(out)), want):
        np.testing.assert_array_equal(g, w)


@pytest.mark.parametrize("kind,bc,order,efix", [("turb", 1, 1, False), ("ot", 1, 0, False),
                                                ("ot", 0, 1, True), ("turb", 0, 0, True),
                                                ("turb", 1, 2, False), ("ot", 0, 2, True)])
def test_cycle_vjp_matches_numpy_reverse(kind, bc, order, efix):
    p, c, bx, by, dx, dy = generic_state(kind, bc, seed=7)
    dt = mhd2d.calc_dt(c, bx, by, GAMMA, 0.4, dx, dy)
    args = (dt, dx, dy, bc, bc, GAMMA, 1e-12, 1e-12, 1e-12, order, efix, 0.3)
    rng = np.random.default_rng(11)
    wts = [rng.standard_normal(x.shape) for x in (p, c, bx, by)]
    want = assembly_np.Cycle(p, c, bx, by, *args).reverse(*wts)
    ny, nx = p.shape[1:]
    a = Adjoint2D(ny, nx, dx, dy, bc, bc, GAMMA, recon=order, entropy_fix=efix, eps=0.3)
    got = _np(a.unpack(a.cycle_vjp(a.pack(p, c, bx, by), dt, a.pack(*wts))))
    for g, w in zip(got, want):
        assert field_rel_err(g, w) <= 1e-12


def _turb_state(n, seed):
    p, c, bx, by, dx, dy = ic.turbulence(n, seed=seed, kmax_v=n // 8, kmax_a=n // 16)
    rng = np.random.default_rng(seed + 1)
    p = p * (1.0 + 0.01 * rng.standard_normal(p.shape))
    p[3] += 0.01 * rng.standard_normal(p[3].shape)
    c = ic.prim_to_cons_mhd(p, GAMMA)
    return p, c, bx, by, dx, dy


@pytest.mark.parametrize("recon", [1, 2])
def test_forward_equals_step_and_backward_equals_chained_vjps(recon):
    n, steps = 64, 7
    p, c, bx, by, dx, dy = _turb_state(n, 5)
    a = Adjoint2D(n, n, dx, dy, 1, 1, GAMMA, recon=recon)
    s0 = a.pack(p, c, bx, by)
    out = a.forward(s0, steps, cfl=0.4, every=3)
    dts = a.dts.copy()
    g = Grid2D(n, n, dx, dy, 1, 1, GAMMA, mhd=True, recon=recon, arith="exact")
    g.upload(p, c, bx, by)
    g.advance(0.0, 1e30, 0, steps, 0.4)
    assert g.last_cycles == steps
    for got, want in zip(_np(a.unpack(out)), g.download()):
        np.testing.assert_array_equal(got, want)
    # the stage kernels (the fixed-dt forward, and the backward's recomputation)
    # give the same states
    for got, want in zip(_np(a.unpack(a.forward(s0, steps, dts=dts))), g.download()):
        np.testing.assert_array_equal(got, want)
    rng = np.random.default_rng(3)
    bar = torch.tensor(rng.standard_normal(a.state_words), device=s0.device)
    grads = {}
    # stored mode (a segment's cycles stay resident) and recompute mode (a budget
    # too small to hold them) for several checkpoint intervals, without a tail; then
    # with the forward pass's resident tail (the whole run, or the last 4 cycles after
    # segments of 2), whose dts come from the stage kernels' CFL reduction and must
    # equal the production step's bit for bit
    for every, budget, sets, tail, want_tail in ((3, 0, 3, 0, 0), (3, 1, 1, 0, 0), (1, 0, 1, 0, 0),
                                                 (0, 0, 3, 0, 0), (7, 0, 7, 0, 0), (3, 0, 3, -1, 7),
                                                 (2, 0, 2, 4, 4), (3, 1, 1, -1, 0)):
        a.configure(budget, tail=tail)
        out_t = a.forward(s0, steps, cfl=0.4, every=every)
        assert a.info()["segment_sets"] == sets
        assert a.record() == dict(steps=steps, every=every or 3, tail=want_tail)
        np.testing.assert_array_equal(a.dts, dts)
        assert torch.equal(out_t, out)
        grads[(every, budget, tail)] = a.backward(bar).cpu().numpy()
        if want_tail:
            # a second backward pass recomputes the tail from its checkpoint
            again = a.backward(bar).cpu().numpy()
            assert np.max(np.abs(again - grads[(every, budget, tail)])) <= 1e-12 * np.max(np.abs(again))
        # the fixed-dt forward (stage kernels, tail included) gives the same state
        assert torch.equal(a.forward(s0, steps, dts=dts, every=every), out)
    a.configure(0, tail=-1)
    states = [s0]
    for k in range(steps - 1):
        states.append(a.cycle(states[-1], dts[k]))
    b = bar
    for k in reversed(range(steps)):
        b = a.cycle_vjp(states[k], dts[k], b)
    chained = b.cpu().numpy()
    scale = np.max(np.abs(chained))
    for every, gr in grads.items():
        assert np.max(np.abs(gr - chained)) <= 1e-12 * scale, every


def _loss_and_grad(a, fl, target, steps, dev):
    xs = fields.fields_to_torch(fl, dev, requires_grad=True)
    state = fields.state_from_fields(*xs, fl["gamma"], fl["dx"], fl["dy"])
    out = evolve(state, a, steps, cfl=0.4)
    rho = a.unpack(out)[0][0]
    loss = torch.mean((rho - target) ** 2)
    loss.backward()
    return float(loss.detach()), [x.grad.cpu().numpy() for x in xs]


def _loss_fixed_dt(a, fl, target, steps, dts, dev):
    xs = fields.fields_to_torch(fl, dev)
    state = fields.state_from_fields(*xs, fl["gamma"], fl["dx"], fl["dy"]).contiguous()
    out = a.forward(state, steps, dts=dts)
    return float(torch.mean((a.unpack(out)[0][0] - target) ** 2))


# At the turbulence generator's state p is uniform, so the PLM step that keeps
# each edge value between the cell and its neighbour (a min/max against equal
# bounds) sits at a tie in every cell: the loss has a kink there and only
# one-sided derivatives with respect to p.  The check therefore perturbs
# (rho, vx, vy, A_z) at that state, and all five fields at a state whose p
# carries a 5% seeded perturbation (generic, differentiable).  The step itself
# is only piecewise smooth (limiter and clamp kinks, upwind switches of the Roe
# flux and of the corner EMF, which jump): a central difference whose stencil
# crosses one of them is off, so the best of three step sizes must agree.
@pytest.mark.parametrize("n,steps,ndir,p_jitter", [(64, 10, 4, 0.0), (64, 10, 4, 0.05)])
def test_gradient_matches_finite_differences(n, steps, ndir, p_jitter):
    dev = torch.device("cuda", 0)
    fl = fields.turbulence_fields(n, seed=2)
    if p_jitter:
        fl["p"] = fl["p"] * (1.0 + p_jitter * np.random.default_rng(4).standard_normal(fl["p"].shape))
    keys = ("rho", "vx", "vy", "p", "az") if p_jitter else ("rho", "vx", "vy", "az")
    tgt_fl = fields.perturbed(fl, 0.02, seed=9)
    a = Adjoint2D(n, n, fl["dx"], fl["dy"], 1, 1, fl["gamma"], recon=1)
    xs = fields.fields_to_torch(tgt_fl, dev)
    target = a.unpack(a.forward(fields.state_from_fields(*xs, GAMMA, fl["dx"], fl["dy"]).contiguous(),
                                steps, cfl=0.4))[0][0].clone()
    loss0, grad = _loss_and_grad(a, fl, target, steps, dev)
    grad = dict(zip(("rho", "vx", "vy", "p", "az"), grad))
    dts = a.dts.copy()
    assert loss0 > 0.0
    rng = np.random.default_rng(17)
    worst = 0.0
    for _ in range(ndir):
        d = {k: rng.standard_normal(fl[k].shape) * (np.mean(fl[k]) if k == "p" else np.std(fl[k])) for k in keys}
        ad = sum(float(np.sum(grad[k] * d[k])) for k in keys)
        errs = []
        for eps in (1e-6, 1e-7, 1e-8):
            fp = dict(fl, **{k: fl[k] + eps * d[k] for k in keys})
            fm = dict(fl, **{k: fl[k] - eps * d[k] for k in keys})
            fd = (_loss_fixed_dt(a, fp, target, steps, dts, dev) - _loss_fixed_dt(a, fm, target, steps, dts, dev)) \
                / (2 * eps)
            errs.append(abs(fd - ad) / abs(fd))
        worst = max(worst, min(errs))
    assert worst <= 1e-5, worst


@pytest.mark.parametrize("recon", [1, 2])
def test_backward_matches_torch_autograd_of_transcription(recon):
    """Several cycles: the GPU backward equals torch's reverse mode through the
    plain torch transcription of the step (run on the GPU, frozen dts), whose
    forward equals the GPU forward bit for bit."""
    n, steps = 48, 6
    dev = torch.device("cuda", 0)
    p, c, bx, by, dx, dy = _turb_state(n, 8)
    a = Adjoint2D(n, n, dx, dy, 1, 1, GAMMA, recon=recon)
    s0 = a.pack(p, c, bx, by)
    out = a.forward(s0, steps, cfl=0.4, every=2)
    dts = a.dts.copy()
    rng = np.random.default_rng(5)
    bar = torch.tensor(rng.standard_normal(a.state_words), device=dev)
    got = a.backward(bar)
    parts = [t.clone().requires_grad_(True) for t in a.unpack(s0)]
    cur = list(parts)
    for k in range(steps):
        cur = list(assembly_np.Cycle(*cur, float(dts[k]), dx, dy, 1, 1, GAMMA, 1e-12, 1e-12, 1e-12, recon, False,
                                     0.5, backend="torch").outputs())
    for t_out, g_out in zip(cur, a.unpack(out)):
        assert torch.equal(t_out.detach(), g_out)
    loss = sum(torch.sum(b * o) for b, o in zip(a.unpack(bar), cur))
    loss.backward()
    for t_in, g_in in zip(parts, a.unpack(got)):
        scale = float(t_in.grad.abs().max())
        assert float((t_in.grad - g_in).abs().max()) <= 1e-11 * scale


def _frozen_loss(a, fl, target, dts, dev):
    xs = fields.fields_to_torch(fl, dev)
    state = fields.state_from_fields(*xs, fl["gamma"], fl["dx"], fl["dy"]).contiguous()
    out = a.branches("replay", state, dts)
    return float(torch.mean((a.unpack(out)[0][0] - target) ** 2))


@pytest.mark.parametrize("recon,efix", [(0, False), (1, False), (2, False), (1, True), (2, True)])
def test_branch_record_and_replay_reproduce_the_forward(recon, efix):
    """Recording the branch decisions and replaying them from the same state both give
    the forward pass's final state bit for bit (first order, PLM, PPM, entropy fix)."""
    n, steps = 40, 6
    dev = torch.device("cuda", 0)
    fl = fields.turbulence_fields(n, seed=3)
    fl["p"] = fl["p"] * (1.0 + 0.05 * np.random.default_rng(5).standard_normal(fl["p"].shape))
    a = Adjoint2D(n, n, fl["dx"], fl["dy"], 1, 1, fl["gamma"], recon=recon, entropy_fix=efix, eps=0.3)
    s0 = fields.state_from_fields(*fields.fields_to_torch(fl, dev), fl["gamma"], fl["dx"], fl["dy"]).contiguous()
    want = a.forward(s0, steps, cfl=0.4)
    dts = a.dts.copy()
    rec = a.branches("record", s0, dts)
    rep = a.branches("replay", s0, dts)
    assert torch.equal(rec, want) and torch.equal(rep, want)
    with pytest.raises(Exception):
        a.branches("replay", s0, np.concatenate([dts, dts[:1]]))   # longer than the record
    a.close()


@pytest.mark.parametrize("recon,efix", [(1, False), (2, False), (2, True)])
def test_gradient_matches_branch_frozen_differences(recon, efix):
    """Central differences of the branch-frozen forward pass (every limiter, clamp,
    upwind and |x| decision replayed from the unperturbed run, dts frozen) measure
    the derivative of the same piece the adjoint differentiates: along every
    direction in all five fields, p included at the generator's uniform-p state, the
    difference at its best step of 1e-6, 1e-7 and 1e-8 agrees to 1e-6."""
    n, steps, ndir = 64, 10, 6
    dev = torch.device("cuda", 0)
    fl = fields.turbulence_fields(n, seed=2, kmax_v=8, kmax_a=8)
    keys = ("rho", "vx", "vy", "p", "az")
    tgt_fl = fields.perturbed(fl, 0.02, seed=9)
    a = Adjoint2D(n, n, fl["dx"], fl["dy"], 1, 1, fl["gamma"], recon=recon, entropy_fix=efix, eps=0.3)
    xs = fields.fields_to_torch(tgt_fl, dev)
    target = a.unpack(a.forward(fields.state_from_fields(*xs, GAMMA, fl["dx"], fl["dy"]).contiguous(),
                                steps, cfl=0.4))[0][0].clone()
    loss0, grad = _loss_and_grad(a, fl, target, steps, dev)
    grad = dict(zip(keys, grad))
    dts = a.dts.copy()
    s0 = fields.state_from_fields(*fields.fields_to_torch(fl, dev), fl["gamma"], fl["dx"], fl["dy"]).contiguous()
    a.branches("record", s0, dts)
    assert _frozen_loss(a, fl, target, dts, dev) == loss0
    rng = np.random.default_rng(23)
    worst = 0.0
    for _ in range(ndir):
        d = {k: rng.standard_normal(fl[k].shape) * (np.mean(fl[k]) if k == "p" else np.std(fl[k])) for k in keys}
        ad = sum(float(np.sum(grad[k] * d[k])) for k in keys)
        errs = []
        for eps in (1e-6, 1e-7, 1e-8):
            fp = dict(fl, **{k: fl[k] + eps * d[k] for k in keys})
            fm = dict(fl, **{k: fl[k] - eps * d[k] for k in keys})
            fd = (_frozen_loss(a, fp, target, dts, dev) - _frozen_loss(a, fm, target, dts, dev)) / (2 * eps)
            e = abs(fd - ad) / abs(ad)
            if e == e:
                errs.append(e)
        worst = max(worst, min(errs))
    a.close()
    assert worst <= 1e-6, worst


def test_reverse_quotient_within_two_ulps_of_the_division():
    """The reverse statements divide by a refined reciprocal (``dsl_div``).  For divisors
    of magnitude 2^-1000 .. 2^1000 its quotient lies within two ulps of the correctly
    rounded division (NumPy's); other divisors (zeros, subnormals, huge, inf, NaN) take
    the IEEE division itself, so the result is the same bits."""
    from pythonmhd_gb300 import _lib
    lib = _lib.load()
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(5)
    n = 1 << 20
    # quotients stay in the normal range: |b| in [1e-20, 2e20], |v| in [2^-950, 2^951)
    b = np.sign(rng.standard_normal(n)) * rng.uniform(1, 2, n) * 10.0 ** rng.uniform(-20, 20, n)
    v = np.sign(rng.standard_normal(n)) * rng.uniform(1, 2, n) * 2.0 ** rng.integers(-950, 951, n)
    edge = np.array([2.0 ** -1000, -(2.0 ** -1000), 2.0 ** 1000 * 1.9999, 2.0 ** -1001, 2.0 ** 1001, 0.0, -0.0,
                     5e-324, -2.2e-308, 1e308, np.inf, -np.inf, np.nan, 1.0, -3.0, 0.1])
    v = np.concatenate([v, edge, edge])
    b = np.concatenate([b, np.ones(edge.size), np.full(edge.size, -7.5)])
    bd, vd = torch.from_numpy(b).to(dev), torch.from_numpy(v).to(dev)
    qd = torch.empty_like(bd)
    _lib.check(lib.mhd2d_adj_quotient(bd.data_ptr(), vd.data_ptr(), qd.data_ptr(), b.size), "mhd2d_adj_quotient")
    with np.errstate(all="ignore"):
        q, ref = qd.cpu().numpy(), b / v
    ex = (v.view(np.int64) >> 52) & 0x7ff
    fast = (ex >= 23) & (ex <= 2023)
    assert fast.sum() >= n
    qi, ri = q[fast].view(np.int64), ref[fast].view(np.int64)
    assert np.all(np.isfinite(ref[fast])) and np.all(np.sign(q[fast]) == np.sign(ref[fast]))
    assert int(np.max(np.abs(qi - ri))) <= 2
    qs, rs = q[~fast], ref[~fast]
    assert np.array_equal(np.isnan(qs), np.isnan(rs))
    np.testing.assert_array_equal(qs[~np.isnan(rs)].view(np.int64), rs[~np.isnan(rs)].view(np.int64))
