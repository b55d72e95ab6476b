"""The batched adjoint (pythonmhd_gb300.adjoint.batch.BatchAdjoint).

Uneven instances (non-square grids, per-instance gamma, turbulence fields at
per-instance seeds), PPM:
* the batched forward pass equals each instance's single-grid exact run bit
  for bit, and so do its recorded dts;
* the batched backward pass equals each instance's single-grid forward +
  backward pass to round-off (atomic adds reorder a few sums), with the
  segments resident and with a budget that forces recomputation;
* the gradient of the summed density-matching loss with respect to every
  instance's fields agrees with torch autograd through the torch
  transcription of the step.
"""
import numpy as np
import pytest
import torch

from pythonmhd_gb300.adjoint import assembly_np, fields
from pythonmhd_gb300.adjoint.batch import BatchAdjoint
from pythonmhd_gb300.adjoint.device import Adjoint2D

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda", 0)


def _batch(count, sizes, seed=3):
    fl = fields.turbulence_batch(count=count, seed=seed, sizes=sizes, kmax=8)
    grids = [dict(nx=f["nx"], ny=f["ny"], dx=f["dx"], dy=f["dy"], gamma=f["gamma"]) for f in fl]
    return fl, grids


def _state(f):
    return fields.state_from_fields(*fields.fields_to_torch(f, DEV), f["gamma"], f["dx"], f["dy"]).contiguous()


@pytest.mark.parametrize("budget", [0, 1])
def test_batched_passes_equal_single_grid_passes(budget):
    steps, every = 9, 4
    fl, grids = _batch(4, (32, 40, 48, 64))
    states = [_state(f) for f in fl]
    ba = BatchAdjoint(grids, recon=2, budget=budget)
    outs = ba.forward(states, steps, cfl=0.4, every=every)
    rng = np.random.default_rng(1)
    bars = [torch.tensor(rng.standard_normal(o.numel()), device=DEV) for o in outs]
    got = ba.backward(bars)
    for k, f in enumerate(fl):
        a = Adjoint2D(f["ny"], f["nx"], f["dx"], f["dy"], 1, 1, f["gamma"], recon=2)
        out = a.forward(states[k], steps, cfl=0.4, every=every)
        assert torch.equal(out, outs[k])
        np.testing.assert_array_equal(a.dts, ba.dts[k])
        want = a.backward(bars[k])
        scale = float(want.abs().max())
        assert float((got[k] - want).abs().max()) <= 1e-12 * scale
        a.close()


def test_batched_gradient_matches_torch_autograd():
    steps = 6
    fl, grids = _batch(3, (32, 48))
    targets = []
    ba = BatchAdjoint(grids, recon=2)
    tgt_states = [_state(fields.perturbed(f, 0.02, seed=11 + k)) for k, f in enumerate(fl)]
    for k, o in enumerate(ba.forward(tgt_states, steps)):
        targets.append(ba.unpack(k, o)[0][0].clone())
    xs = [fields.fields_to_torch(f, DEV, requires_grad=True) for f in fl]
    states = [fields.state_from_fields(*x, f["gamma"], f["dx"], f["dy"]) for x, f in zip(xs, fl)]
    outs = ba.forward([s.detach().contiguous() for s in states], steps)
    # loss = sum over instances of mean((rho - rho_target)^2); its gradient w.r.t. the final states
    bars = []
    loss = 0.0
    for k, o in enumerate(outs):
        o = o.clone().requires_grad_(True)
        lk = torch.mean((ba.unpack(k, o)[0][0] - targets[k]) ** 2)
        lk.backward()
        loss += float(lk.detach())
        bars.append(o.grad)
    bar0 = ba.backward(bars)
    torch.autograd.backward(states, bar0)
    for k, f in enumerate(fl):
        xt = fields.fields_to_torch(f, DEV, requires_grad=True)
        parts = list(ba.unpack(k, fields.state_from_fields(*xt, f["gamma"], f["dx"], f["dy"])))
        for c in range(steps):
            parts = list(assembly_np.Cycle(*parts, float(ba.dts[k][c]), f["dx"], f["dy"], 1, 1, f["gamma"], 1e-12,
                                           1e-12, 1e-12, 2, False, 0.5, backend="torch").outputs())
        assert torch.equal(parts[0].detach(), ba.unpack(k, outs[k])[0])
        torch.mean((parts[0][0] - targets[k]) ** 2).backward()
        for x_ours, x_torch in zip(xs[k], xt):
            scale = float(x_torch.grad.abs().max())
            assert float((x_ours.grad - x_torch.grad).abs().max()) <= 1e-11 * scale


def _screen(grids, states, steps):
    """Instances whose run of `steps` cycles turns non-finite (time, dt or state), by
    one batched run of all of them: the reference algorithm has no positivity fix, and
    on under-resolved turbulence it can drive the pressure negative."""
    from pythonmhd_gb300 import _lib
    from pythonmhd_gb300.solver import Batch2D
    b = Batch2D(grids, mhd=True, recon=2, arith="exact")
    try:
        for k, st in enumerate(states):
            p, c, bx, by = st
            b.upload_device(k, p.contiguous(), c.contiguous(), bx.contiguous(), by.contiguous())
        try:
            b.advance(0.0, 1e300, 0, steps, 0.4)
        except _lib.MhdError:
            pass
        _, nan = b.stats()
        status = b.instance_status()
        bad = {k for k in range(len(grids)) if nan[k] or status[k] != 0}
        for k in range(len(grids)):
            if k not in bad and not all(np.isfinite(a).all() for a in b.download(k)):
                bad.add(k)
        return sorted(bad)
    finally:
        b.close()


@pytest.mark.skipif("PYTHONMHD_GB300_ADJ_BATCH_FULL" not in __import__("os").environ,
                    reason="full batched-adjoint workload: set PYTHONMHD_GB300_ADJ_BATCH_FULL=<report.json>")
def test_batched_adjoint_full_workload():
    """The batched-adjoint workload as stated: 64 instances, Nx and Ny uniform in
    {128, 192, ..., 1024}, gamma in [1.4, 5/3], the 4096^2 workload's turbulence
    generator at per-instance seeds (density and velocity spectra to k = 32, vector
    potential to k = 16, rms Mach 1, beta 1), PPM, 200 cycles: forward pass on the
    batched step, backward pass instance by instance; timed against the batched
    forward step alone.  The step, like the reference, has no positivity fix: the
    instances whose run (or whose target's run) turns non-finite within the 200
    cycles are listed in the report with their seeds and sizes, and the gradient runs
    over the others.  Writes the numbers to the JSON path in the variable."""
    import json
    import os
    import time
    steps = int(os.environ.get("PYTHONMHD_GB300_ADJ_BATCH_STEPS", "200"))
    every = int(os.environ.get("PYTHONMHD_GB300_ADJ_BATCH_EVERY", "0"))
    seed = 4
    fl_all = fields.turbulence_batch(count=64, seed=seed, sizes=tuple(range(128, 1025, 64)), kmax_v=32, kmax_a=16,
                                     mach=1.0)
    grids_all = [dict(nx=f["nx"], ny=f["ny"], dx=f["dx"], dy=f["dy"], gamma=f["gamma"]) for f in fl_all]
    tg_fl = [fields.perturbed(f, 0.02, seed=100 + k) for k, f in enumerate(fl_all)]

    def unpacked(f, k):
        st = _state(f)
        g = grids_all[k]
        ny, nx = g["ny"], g["nx"]
        a, b = 8 * ny * nx, ny * (nx + 1)
        return (st[:a].view(8, ny, nx), st[a:2 * a].view(8, ny, nx), st[2 * a:2 * a + b].view(ny, nx + 1),
                st[2 * a + b:].view(ny + 1, nx))

    bad_run = _screen(grids_all, [unpacked(f, k) for k, f in enumerate(fl_all)], steps)
    bad_tgt = _screen(grids_all, [unpacked(f, k) for k, f in enumerate(tg_fl)], steps)
    keep = [k for k in range(64) if k not in set(bad_run) | set(bad_tgt)]
    excluded = [{"instance": k, "seed": seed * 100003 + k, "nx": grids_all[k]["nx"], "ny": grids_all[k]["ny"],
                 "gamma": grids_all[k]["gamma"], "run_nonfinite": k in bad_run, "target_nonfinite": k in bad_tgt}
                for k in sorted(set(bad_run) | set(bad_tgt))]
    fl = [fl_all[k] for k in keep]
    grids = [grids_all[k] for k in keep]
    zones = sum(g["nx"] * g["ny"] for g in grids)
    ba = BatchAdjoint(grids, recon=2)
    targets = [ba.unpack(i, o)[0][0].clone() for i, o in
               enumerate(ba.forward([_state(tg_fl[k]) for k in keep], steps))]
    states = [_state(f) for f in fl]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    outs = ba.forward(states, steps, every=every)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    bars = []
    for k, o in enumerate(outs):
        o = o.clone().requires_grad_(True)
        torch.mean((ba.unpack(k, o)[0][0] - targets[k]) ** 2).backward()
        bars.append(o.grad)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    bar0 = ba.backward(bars)
    torch.cuda.synchronize()
    t3 = time.perf_counter()
    assert all(bool(torch.isfinite(b).all()) for b in bar0)
    # the batched step alone, all cycles in one call (no dt record, no checkpoints)
    from pythonmhd_gb300.solver import Batch2D
    b = Batch2D(grids, mhd=True, recon=2, arith="exact")
    for k in range(len(grids)):
        p, c, bx, by = ba.unpack(k, states[k])
        b.upload_device(k, p.contiguous(), c.contiguous(), bx.contiguous(), by.contiguous())
    torch.cuda.synchronize()
    t4 = time.perf_counter()
    b.advance(0.0, 1e300, 0, steps, 0.4)
    torch.cuda.synchronize()
    t_plain = time.perf_counter() - t4
    b.close()
    per = sorted(zip(ba.backward_seconds, [g["nx"] * g["ny"] for g in grids]), key=lambda x: -x[1])
    report = {"instances_stated": 64, "instances_run": len(grids), "excluded_nonfinite": excluded,
              "zones_per_step": zones, "steps": steps,
              "batched_step_alone_s": t_plain, "backward_over_batched_step": (t3 - t2) / t_plain,
              "gradient_over_batched_step": (t3 - t2 + t1 - t0) / t_plain,
              "checkpoint_intervals": sorted(set(ba.every)),
              "backward_s_by_instance_largest_first": [[round(t, 3), z] for t, z in per],
              "forward_s": t1 - t0, "backward_s": t3 - t2, "checkpoint_arena_bytes": ba.arena.numel() * 8,
              "backward_over_forward": (t3 - t2) / (t1 - t0),
              "gradient_over_forward": (t3 - t2 + t1 - t0) / (t1 - t0),
              "forward_zone_updates_per_s": zones * steps / (t1 - t0)}
    print(report)
    with open(os.environ["PYTHONMHD_GB300_ADJ_BATCH_FULL"], "w") as f:
        json.dump(report, f, indent=1)


def test_reshaped_handle_equals_fresh_handle():
    """A handle re-targeted to a smaller grid gives the fresh handle's results."""
    fl, grids = _batch(2, (48, 64), seed=5)
    big, small = sorted(fl, key=lambda f: -f["nx"] * f["ny"])
    a = Adjoint2D(big["ny"], big["nx"], big["dx"], big["dy"], 1, 1, big["gamma"], recon=2)
    s_big = _state(big)
    a.forward(s_big, 5, every=2)
    a.backward(torch.ones(a.state_words, dtype=torch.float64, device=DEV))
    a.reshape(small["ny"], small["nx"], small["dx"], small["dy"], 1, 1, small["gamma"])
    s_small = _state(small)
    out = a.forward(s_small, 5, every=3)
    bar = torch.linspace(-1.0, 1.0, a.state_words, dtype=torch.float64, device=DEV)
    got = a.backward(bar)
    b = Adjoint2D(small["ny"], small["nx"], small["dx"], small["dy"], 1, 1, small["gamma"], recon=2)
    assert torch.equal(b.forward(s_small, 5, every=3), out)
    want = b.backward(bar)
    assert float((got - want).abs().max()) <= 1e-12 * float(want.abs().max())
