"""Benchmark of the 2D MHD CTU+CT step on GB300.

Workload (default): 2D ideal-MHD driven-free turbulence, 4096 x 4096 periodic,
gamma = 5/3, FP64, PPM + Roe + CTU+CT, CFL 0.4 (seeded synthetic state from
``pythonmhd_gb300.initial_conditions.turbulence_device``, the turbulence
generator with its transforms on the GPU).  One step = one cycle over
the whole grid.  Metric: zone-updates/s (cells x cycles / s), whole job.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--arith exact|fast] [--n 4096]

Our arm prints one JSON line with the device-resident throughput (``value``),
the end-to-end throughput through the C ABI with host buffers (``e2e``), the
roofline of the step, the CPU-oracle baseline and the clocks seen during the
timed region.  ``--impl reference`` times the CPU restatement of the reference
algorithm (``oracle/``) on the host cores instead.  Under torchrun each rank
runs its own replica (the 2D step is advanced as independent replicas; no
collective is involved), and rank 0 prints the line.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "zone-updates/s @4096^2 FP64 MHD (PPM+Roe+CTU+CT)"
UNIT = "zone-updates/s"
ALG_BYTES_PER_ZONE = 128          # 8 state words read + 8 written per zone-update (MHD)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--arith", choices=["exact", "fast"], default="exact")
    ap.add_argument("--other-arith-steps", type=int, default=10,
                    help="cycles timed in the other arithmetic mode beside the headline (0 = skip)")
    ap.add_argument("--n", type=int, default=4096)
    ap.add_argument("--recon", type=int, choices=[0, 1, 2], default=2,
                    help="reconstruction of the single-grid workload (2 = PPM, the headline; 1 = PLM and "
                         "0 = first order serve instruction-mix captures)")
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--cpu-sample", type=int, default=512, help="grid size of the CPU baseline sample")
    ap.add_argument("--cpu-steps", type=int, default=2)
    ap.add_argument("--e2e-steps", type=int, default=0, help="0 = same as --steps")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--batch-steps", type=int, default=200,
                    help="cycles of the 256-instance batched workload (0 = skip it)")
    ap.add_argument("--batch-step-major-steps", type=int, default=20,
                    help="cycles of the step-major per-instance loop (one advance call per instance and cycle)")
    ap.add_argument("--batch-count", type=int, default=256)
    ap.add_argument("--adjoint-steps", type=int, default=400,
                    help="cycles of the 512^2 PLM adjoint workload (0 = skip it)")
    ap.add_argument("--adjoint-n", type=int, default=512)
    ap.add_argument("--adjoint-recon", type=int, choices=[0, 1, 2], default=1,
                    help="reconstruction of the adjoint workload (1 = PLM, as stated; 2 = PPM)")
    ap.add_argument("--adjoint-tail", type=int, default=-1,
                    help="cycles the adjoint's forward pass leaves resident (-1 as many as fit, 0 none)")
    ap.add_argument("--hydro3d-steps", type=int, default=10,
                    help="cycles of the 3D hydro turbulence workload (0 = skip it)")
    ap.add_argument("--hydro3d-n", type=int, default=256)
    ap.add_argument("--mhd3d-steps", type=int, default=5,
                    help="cycles of the 3D MHD turbulence workload (0 = skip it)")
    ap.add_argument("--mhd3d-n", type=int, default=192)
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def max_over_ranks(values, device):
    """Each of ``values`` maxed over the ranks of the default process group (the
    values themselves when no group is up or it has one rank)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return [float(v) for v in values]
    tt = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return tt.tolist()


def replica_throughput(world, units_per_rank, ms_per_step):
    """Whole-job units/s of ``world`` replicas that each process ``units_per_rank``
    units per step, timed by the slowest rank's ``ms_per_step``."""
    return world * units_per_rank / (ms_per_step * 1e-3)


# ----------------------------------------------------------------------------
# CPU legs (oracle = CPU restatement of the reference algorithm)
# ----------------------------------------------------------------------------
def _cpu_cycles(n, steps, warmup, seed):
    """Time ``steps`` oracle cycles on an n x n turbulence state; returns seconds per cycle."""
    from oracle import mhd2d
    from pythonmhd_gb300 import initial_conditions as ic
    prim, cons, fbx, fby, dx, dy = ic.turbulence(n, seed=seed, gamma=5.0 / 3.0)
    g = 5.0 / 3.0
    times = []
    for k in range(warmup + steps):
        dt = mhd2d.calc_dt(cons, fbx, fby, g, 0.4, dx, dy)
        t0 = time.perf_counter()
        prim, cons, fbx, fby = mhd2d.cycle(prim, cons, fbx, fby, dt, dx, dy, 1, 1, g, 1e-12, 1e-12, 1e-12,
                                           2, False, 0.5)
        if k >= warmup:
            times.append(time.perf_counter() - t0)
    return float(np.mean(times))


def _cpu_worker(args):
    n, steps, warmup, seed = args
    os.environ.setdefault("OMP_NUM_THREADS", "1")
    return _cpu_cycles(n, steps, warmup, seed)


def _batch_cpu_instance(args):
    """The oracle's PLM cycle on one batched instance (its own CFL dt): seconds for
    ``steps`` cycles and the zone-updates done."""
    inst, steps = args
    os.environ.setdefault("OMP_NUM_THREADS", "1")
    from oracle import mhd2d
    prim, cons, fbx, fby = (inst[k].copy() for k in ("prim", "cons", "fbx", "fby"))
    g, dx, dy = inst["gamma"], inst["dx"], inst["dy"]
    t0 = time.perf_counter()
    for _ in range(steps):
        dt = mhd2d.calc_dt(cons, fbx, fby, g, 0.4, dx, dy)
        prim, cons, fbx, fby = mhd2d.cycle(prim, cons, fbx, fby, dt, dx, dy, 1, 1, g, 1e-12, 1e-12, 1e-12,
                                           1, False, 0.5)
    return time.perf_counter() - t0, inst["nx"] * inst["ny"] * steps


def batch_cpu_baseline(insts, count, steps):
    """The oracle on a seeded subset of the batched workload's instances: one host core,
    and one process per host core (the instances are independent); zone-updates/s."""
    import multiprocessing as mp
    sample = [dict((k, i[k]) for k in ("prim", "cons", "fbx", "fby", "gamma", "dx", "dy", "nx", "ny"))
              for i in insts[:count]]
    one = [_batch_cpu_instance((i, steps)) for i in sample]
    t1, z1 = sum(t for t, _ in one), sum(z for _, z in one)
    cores = os.cpu_count() or 1
    work = [(sample[k % len(sample)], steps) for k in range(cores)]
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(cores) as pool:
        res = pool.map(_batch_cpu_instance, work)
    wall = time.perf_counter() - t0
    zp = sum(z for _, z in res)
    return {"value": z1 / t1, "unit": UNIT, "cores": 1, "kind": "port",
            "processes_value": zp / wall, "processes": cores,
            "sample": f"oracle (NumPy restatement of the reference step, PLM), the first {len(sample)} instances of "
                      f"the batch x {steps} cycles each: {t1:.2f} s on 1 host core; {cores} processes over the same "
                      f"instances in turn, {wall:.2f} s wall (pool start included); a sample, not the 256 x 200 run"}


def cpu_baseline(n, steps):
    t = _cpu_cycles(n, steps, 1, 7)
    return {"value": n * n / t, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"oracle (NumPy restatement of the reference step), {n}x{n} turbulence, PPM MHD, "
                      f"1 untimed + {steps} timed cycles, {t:.3f} s/cycle on 1 host core"}


def run_reference(a):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import multiprocessing as mp
    cores = os.cpu_count() or 1
    n = min(a.cpu_sample, 256)
    steps = max(1, a.steps)
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(cores) as pool:
        per = pool.map(_cpu_worker, [(n, steps, a.warmup, 100 + i) for i in range(cores)])
    wall = time.perf_counter() - t0
    sec_per_cycle = float(np.mean(per))
    value = cores * n * n / sec_per_cycle
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": a.gpus, "steps": steps,
            "warmup": a.warmup, "ms_per_step": sec_per_cycle * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": f"2D MHD turbulence {n}x{n} per host process (bounded sample of the "
                                   f"4096x4096 workload), PPM+Roe+CTU+CT, CFL 0.4, FP64",
                       "processes": cores},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{cores} independent processes x {steps} timed cycles of a {n}x{n} "
                                       f"turbulence state (oracle restatement of the reference NumPy step); "
                                       f"wall {wall:.1f} s"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------
# clocks sampled during the timed region
# ----------------------------------------------------------------------------
class ClockSampler:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.dev = device_index
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        out, _ = self.proc.communicate(timeout=10)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except Exception:
        return {}


RECON_NAME = {0: "first", 1: "plm", 2: "ppm"}


def profile_summary(arith, recon=2):
    """Per-cycle DRAM traffic / FP64 instruction counts from the committed ncu summary."""
    try:
        with open(os.path.join(ROOT, "profiles", f"mhd_{RECON_NAME[recon]}_cycle_ncu_{arith}.json")) as f:
            return json.load(f)
    except Exception:
        return None


PROBE_SRC = os.path.join(ROOT, "fp64_probe.cu")
PROBE_EXE = os.path.join(ROOT, "_build", "fp64_probe")


def build_probe() -> str:
    """Build the FP64 pipe throughput probe (fp64_probe.cu beside this file) for sm_103a."""
    from pythonmhd_gb300 import build as _build
    if os.path.exists(PROBE_EXE) and os.path.getmtime(PROBE_EXE) > os.path.getmtime(PROBE_SRC):
        return PROBE_EXE
    os.makedirs(os.path.dirname(PROBE_EXE), exist_ok=True)
    r = subprocess.run([_build.nvcc_path(), _build.ARCH, "-O3", "-o", PROBE_EXE, PROBE_SRC],
                       stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError("probe build failed:\n" + r.stdout.decode(errors="replace"))
    return PROBE_EXE


_PROBE = {}


def fp64_peak():
    """DFMA / DADD / DMUL lane-ops/s of this GPU from the FP64 probe (fp64_probe.cu),
    measured once per run."""
    if "rates" not in _PROBE:
        try:
            exe = build_probe()
            out = subprocess.run([exe, "--json"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True,
                                 timeout=120).stdout
            _PROBE["rates"] = json.loads(out.strip().splitlines()[-1])
        except Exception:
            _PROBE["rates"] = None
    return _PROBE["rates"]


def fp64_roof_3d(kind, arith, zones, ms_per):
    """The FP64-issue roof of a 3D cycle from its committed instruction mix
    (profiles/<kind>_cycle_ncu_<arith>.json), flattened for the bench line."""
    try:
        with open(os.path.join(ROOT, "profiles", f"{kind}_cycle_ncu_{arith}.json")) as f:
            prof = json.load(f)
    except Exception:
        return {}
    r = fp64_roof(prof, fp64_peak(), zones, ms_per)
    if not r:
        return {}
    return {"fp64_frac_of_floor": r["frac"], "fp64_floor_ms": r["floor_ms_per_step"],
            "fp64_achieved_ginstr_s": r["achieved"], "fp64_peak_ginstr_s": r["peak"],
            "fp64_ops_source": r["ops_source"]}


def fp64_roof(prof, probe, zones, ms_per):
    """FP64-issue roof of one step: each instruction class at its own measured rate.

    The floor is dfma/r_fma + (dadd + dmul)/r_add lane-instructions' worth of time per
    step; ``frac`` = floor / measured step time.  ``peak`` is the mix-weighted rate
    (total instructions / floor), so achieved / peak = frac as well."""
    dfma, dadd, dmul = (prof.get(k) for k in ("dfma_per_zone", "dadd_per_zone", "dmul_per_zone"))
    if None in (dfma, dadd, dmul) or not probe:
        return None
    r_fma, r_add, r_mul = probe["dfma_gops"], probe["dadd_gops"], probe["dmul_gops"]
    floor_s = zones * (dfma / r_fma + dadd / r_add + dmul / r_mul) / 1e9
    ops = (dfma + dadd + dmul) * zones
    ach = ops / (ms_per * 1e-3) / 1e9
    peak = ops / floor_s / 1e9
    return {"achieved": ach, "peak": peak, "unit": "G FP64 lane-instr/s", "frac": ach / peak,
            "floor_ms_per_step": floor_s * 1e3,
            "ops_per_zone": {"dfma": dfma, "dadd": dadd, "dmul": dmul},
            "rates_gops": {"dfma": r_fma, "dadd": r_add, "dmul": r_mul},
            "peak_source": "mix-weighted measured DFMA/DADD/DMUL rates (fp64_probe.cu, same box)",
            "ops_source": prof.get("source")}


# ----------------------------------------------------------------------------
# batched form vs a per-instance loop of the single-grid path
# ----------------------------------------------------------------------------
def run_batch(a, torch):
    """256 uneven Orszag-Tang instances (Nx, Ny in {64..512}, PLM): one batched
    handle vs a loop of single-grid handles advancing each instance in turn."""
    from pythonmhd_gb300 import initial_conditions as ic
    from pythonmhd_gb300.solver import Batch2D, Grid2D
    # the instances are built on the GPU (the project's generator kernels); the host
    # copies serve the autotuner and the per-instance loop's uploads
    dev_insts = ic.orszag_tang_batch_device(count=a.batch_count, seed=0)
    insts = [dict(d, prim=d["prim"].cpu().numpy(), cons=d["cons"].cpu().numpy(), fbx=d["fbx"].cpu().numpy(),
                  fby=d["fby"].cpu().numpy()) for d in dev_insts]
    zones = sum(i["nx"] * i["ny"] for i in insts)
    k, w = a.batch_steps, 1
    from pythonmhd_gb300 import autotune
    b = Batch2D(insts, mhd=True, recon=1, arith=a.arith)
    tuned = autotune.tune_batch(b, insts, recon=1, cycles=1)
    for j, d in enumerate(dev_insts):
        b.upload_device(j, d["prim"], d["cons"], d["fbx"], d["fby"])
    del dev_insts
    b.advance(0.0, 1e30, 0, w, 0.4)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    b.advance(0.0, 1e30, w, w + k, 0.4)
    torch.cuda.synchronize()
    tb = time.perf_counter() - t0
    launches = b.info()["last_launches"]
    b.close()
    singles = []
    for i in insts:
        g = Grid2D(i["ny"], i["nx"], i["dx"], i["dy"], 1, 1, i["gamma"], mhd=True, recon=1, arith=a.arith)
        g.upload(i["prim"], i["cons"], i["fbx"], i["fby"])
        g.advance(0.0, 1e30, 0, w, 0.4)
        singles.append(g)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for g in singles:
        g.advance(0.0, 1e30, w, w + k, 0.4)
    torch.cuda.synchronize()
    tl = time.perf_counter() - t0
    # step-major loop: every instance advanced one cycle per call, instance after instance
    ks = max(1, min(k, a.batch_step_major_steps))
    t0 = time.perf_counter()
    for s in range(ks):
        for g in singles:
            g.advance(0.0, 1e30, w + k + s, w + k + s + 1, 0.4)
    torch.cuda.synchronize()
    ts = time.perf_counter() - t0
    for g in singles:
        g.close()
    # the FP64-issue roof from the single-grid PLM cycle's instruction mix: the batched
    # kernels run the same per-zone bodies (tile edges add a little on top)
    cpu = batch_cpu_baseline(insts, 8, 2) if not a.no_cpu else None
    roof = {}
    plm = profile_summary(a.arith, 1)
    r = fp64_roof(plm, fp64_peak(), zones * k, tb * 1e3) if plm else None
    if r:
        roof = {"fp64_frac_of_floor": r["frac"], "fp64_floor_s": r["floor_ms_per_step"] * 1e-3,
                "looped_fp64_frac_of_floor": r["frac"] * tb / tl, "fp64_ops_source": r["ops_source"]}
    return {"workload": f"{len(insts)} Orszag-Tang instances, Nx,Ny uniform in 64..512 step 32, gamma in "
                        f"[1.4,5/3], B0 x U[0.5,2], 1% density perturbation, PLM+Roe+CTU+CT, per-instance dt",
            "zones_per_step": zones, "steps": k,
            "batched_zone_updates_per_s": zones * k / tb, "looped_zone_updates_per_s": zones * k / tl,
            "speedup_vs_loop": tl / tb, "batched_launches": launches,
            "launch_shape": {"tile_width": tuned["tile_width"], "fuse": tuned["fuse"], "blocks": tuned["blocks"],
                             "autotuned": True, "from_cache": tuned["cached"]},
            "loop": "one single-grid handle per instance, each advanced k cycles in turn (CUDA graphs)",
            "step_major_loop_zone_updates_per_s": zones * ks / ts, "step_major_steps": ks,
            "speedup_vs_step_major_loop": (ts / ks) / (tb / k), **roof, "cpu_baseline": cpu,
            "timing": "host wall clock around device-synchronised calls"}


# ----------------------------------------------------------------------------
# 3D hydro step
# ----------------------------------------------------------------------------
def run_hydro3d(a, torch):
    """3D hydro turbulence, n^3 periodic, PPM + Roe + CTU, FP64: device-resident
    zone-updates/s of the 3D step, timed with CUDA events on the handle's stream;
    the oracle's 3D restatement on one host core on a 48^3 sample."""
    from oracle import hydro3d
    from pythonmhd_gb300 import initial_conditions as ic
    from pythonmhd_gb300.solver import Grid3D
    n = a.hydro3d_n
    dev = torch.device("cuda", torch.cuda.current_device())
    prim, cons, d = ic.turbulence_hydro_3d(n, seed=a.seed, gamma=1.4, kmax=16, mach=1.0, device=dev)
    g = Grid3D(n, n, n, d, d, d, 1, 1, 1, 1.4, recon=2, arith=a.arith)
    g.upload_device(prim, cons)
    del prim, cons
    torch.cuda.empty_cache()
    stream = torch.cuda.ExternalStream(g.stream(), device=dev)
    t, cyc, _ = g.advance(0.0, 1e30, 0, 2, 0.4)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    t, cyc, _ = g.advance(t, 1e30, cyc, cyc + a.hydro3d_steps, 0.4)
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / a.hydro3d_steps
    launches = g.last_launches()
    dev_bytes = g.device_bytes()
    w, _ = g.download(0)
    g.close()
    if not np.isfinite(w).all():
        raise RuntimeError("non-finite 3D state after the timed cycles")
    zones = n ** 3
    peaks = measured_peaks()
    hbm = peaks.get("hbm_gbs") or 6800.0
    achieved = 80.0 * zones / (ms * 1e-3) / 1e9
    m = 48
    pc, cc, dc = ic.turbulence_hydro_3d(m, seed=a.seed, gamma=1.4, kmax=8, mach=1.0, device="cpu")
    pc, cc = pc.numpy(), cc.numpy()
    t0 = time.perf_counter()
    hydro3d.evolve(pc, cc, dc, dc, dc, 1, 1, 1, 0.0, 1e30, 0, 2, 1.4, 0.4, 1e-12, 1e-12, 1e-12, 2, False, 0.5)
    cpu_s = time.perf_counter() - t0
    return {"workload": f"3D hydro turbulence {n}^3 periodic, gamma=1.4, rms Mach 1, k<=16, PPM+Roe+CTU, "
                        f"CFL 0.4, FP64, seeded (seed {a.seed})",
            "zone_updates_per_s": zones / (ms * 1e-3), "ms_per_cycle": ms, "steps": a.hydro3d_steps,
            "gpu_launches": launches, "device_bytes": dev_bytes,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                         "kernel": "one full 3D cycle (19 kernels per cycle, CUDA graphs), 80 algorithmic B/zone",
                         "compute_bound": "fp64", **fp64_roof_3d("hydro3d", a.arith, zones, ms)},
            "cpu_baseline": {"value": m ** 3 * 2 / cpu_s, "unit": "zone-updates/s", "cores": 1, "kind": "port",
                             "sample": f"oracle/hydro3d.py, {m}^3 periodic turbulence, 2 PPM cycles"},
            "timing": "CUDA events on the handle's stream; state 0.67 GB per buffer >> 129 MB L2"}


def run_mhd3d(a, torch):
    """3D MHD turbulence, n^3 periodic, PPM + Roe + CTU+CT with three EMF components,
    FP64: device-resident zone-updates/s of the 3D MHD step (CUDA events on the
    handle's stream); the oracle's 3D restatement on one host core on a 24^3 sample."""
    from oracle import mhd3d
    from pythonmhd_gb300 import initial_conditions as ic
    from pythonmhd_gb300.solver import Grid3D
    n = a.mhd3d_n
    dev = torch.device("cuda", torch.cuda.current_device())
    st = ic.turbulence_mhd_3d(n, seed=a.seed, gamma=5.0 / 3.0, kmax=16, mach=1.0, device=dev)
    d = st[5]
    g = Grid3D(n, n, n, d, d, d, 1, 1, 1, 5.0 / 3.0, recon=2, entropy_fix=True, arith=a.arith, mhd=True)
    g.upload_device(*st[:5])
    del st
    torch.cuda.empty_cache()
    stream = torch.cuda.ExternalStream(g.stream(), device=dev)
    t, cyc, _ = g.advance(0.0, 1e30, 0, 2, 0.4)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    t, cyc, _ = g.advance(t, 1e30, cyc, cyc + a.mhd3d_steps, 0.4)
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / a.mhd3d_steps
    launches = g.last_launches()
    dev_bytes = g.device_bytes()
    out = g.download(0)
    g.close()
    if not np.isfinite(out[1]).all():
        raise RuntimeError("non-finite 3D MHD state after the timed cycles")
    zones = n ** 3
    peaks = measured_peaks()
    hbm = peaks.get("hbm_gbs") or 6800.0
    achieved = 176.0 * zones / (ms * 1e-3) / 1e9
    m = 24
    sc = ic.turbulence_mhd_3d(m, seed=a.seed, gamma=5.0 / 3.0, kmax=4, mach=1.0, device="cpu")
    arrs = [x.numpy() for x in sc[:5]]
    t0 = time.perf_counter()
    mhd3d.evolve(*arrs, sc[5], sc[5], sc[5], 1, 1, 1, 0.0, 1e30, 0, 2, 5.0 / 3.0, 0.4, 1e-12, 1e-12, 1e-12, 2, True,
                 0.5)
    cpu_s = time.perf_counter() - t0
    return {"workload": f"3D ideal-MHD turbulence {n}^3 periodic, gamma=5/3, rms Mach 1, beta 1, k<=16, "
                        f"PPM+Roe+CTU+CT (three edge EMFs), entropy fix, CFL 0.4, FP64, seeded (seed {a.seed})",
            "zone_updates_per_s": zones / (ms * 1e-3), "ms_per_cycle": ms, "steps": a.mhd3d_steps,
            "gpu_launches": launches, "device_bytes": dev_bytes,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                         "kernel": "one full 3D MHD cycle (29 kernels, CUDA graphs), 176 algorithmic B/zone "
                                   "(8 conserved and 3 face-B words in and out)", "compute_bound": "fp64",
                         **fp64_roof_3d("mhd3d", a.arith, zones, ms)},
            "cpu_baseline": {"value": m ** 3 * 2 / cpu_s, "unit": "zone-updates/s", "cores": 1, "kind": "port",
                             "sample": f"oracle/mhd3d.py, {m}^3 periodic turbulence, 2 PPM cycles"},
            "timing": "CUDA events on the handle's stream; state 1.3 GB per buffer >> 129 MB L2"}


# ----------------------------------------------------------------------------
# adjoint: gradient of a density-matching loss through many cycles
# ----------------------------------------------------------------------------
def run_adjoint(a, torch):
    """512^2 periodic MHD turbulence (seeded, k <= 16), PLM + Roe + CTU+CT (PPM with
    --adjoint-recon 2), 400 cycles at CFL 0.4; loss = mean squared difference between the final density and the
    final density of a run from a smoothly 2%-perturbed initial state; gradient
    with respect to the initial rho, vx, vy, p, A_z by the hand-written backward
    pass with sqrt(N) checkpoints (the last cycles run with tapes in the forward pass
    and stay resident).  Timed against the production forward step on the same
    state (exact arithmetic)."""
    from pythonmhd_gb300.adjoint import fields
    from pythonmhd_gb300.adjoint.device import Adjoint2D, evolve
    from pythonmhd_gb300.solver import Grid2D
    n, steps = a.adjoint_n, a.adjoint_steps
    dev = torch.device("cuda", torch.cuda.current_device())
    fl = fields.turbulence_fields(n, seed=1, kmax_v=16, kmax_a=16)
    tgt = fields.perturbed(fl, 0.02, seed=2)
    g0 = fl["gamma"]
    recon = a.adjoint_recon
    adj = Adjoint2D(n, n, fl["dx"], fl["dy"], 1, 1, g0, recon=recon)
    adj.configure(0, tail=a.adjoint_tail)
    st_t = fields.state_from_fields(*fields.fields_to_torch(tgt, dev), g0, fl["dx"], fl["dy"]).contiguous()
    target = adj.unpack(adj.forward(st_t, steps, cfl=0.4))[0][0].clone()
    # production forward on the same initial state (the denominator)
    xs = fields.fields_to_torch(fl, dev)
    s0 = fields.state_from_fields(*xs, g0, fl["dx"], fl["dy"]).contiguous()
    prim, cons, fbx, fby = [t.cpu().numpy() for t in adj.unpack(s0)]
    grid = Grid2D(n, n, fl["dx"], fl["dy"], 1, 1, g0, mhd=True, recon=recon, arith="exact")
    grid.upload(prim, cons, fbx, fby)
    grid.advance(0.0, 1e30, 0, 3, 0.4)
    grid.upload(prim, cons, fbx, fby)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    grid.advance(0.0, 1e30, 0, steps, 0.4)
    torch.cuda.synchronize()
    t_fwd = time.perf_counter() - t0
    grid.close()
    # warm-up (untimed): one short gradient through the same handle (first launches of
    # the reverse kernels, the autograd path)
    xw = fields.fields_to_torch(fl, dev, requires_grad=True)
    ow = evolve(fields.state_from_fields(*xw, g0, fl["dx"], fl["dy"]), adj, min(8, steps), cfl=0.4)
    torch.mean((adj.unpack(ow)[0][0] - target) ** 2).backward()
    torch.cuda.synchronize()
    # gradient: forward pass (records dt, keeps checkpoints) + backward pass
    xs = fields.fields_to_torch(fl, dev, requires_grad=True)
    state = fields.state_from_fields(*xs, g0, fl["dx"], fl["dy"])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out = evolve(state, adj, steps, cfl=0.4)
    loss = torch.mean((adj.unpack(out)[0][0] - target) ** 2)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    loss.backward()
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    info = adj.info()
    rec = adj.record()
    gnorm = float(sum(float(torch.sum(x.grad * x.grad)) for x in xs)) ** 0.5
    adj.close()
    label = {0: "first-order", 1: "PLM", 2: "PPM"}[recon]
    return {"workload": f"{n}x{n} periodic MHD turbulence (seeded, k<=16), {label}+Roe+CTU+CT, {steps} cycles, CFL 0.4; "
                        "loss = mean((rho_final - rho_target)^2), target from a smoothly 2%-perturbed state; "
                        "gradient w.r.t. initial rho, vx, vy, p, A_z; dt frozen",
            "steps": steps, "loss": float(loss.detach()), "grad_norm": gnorm,
            "forward_ms_per_cycle": 1e3 * t_fwd / steps,
            "gradient_forward_pass_ms_per_cycle": 1e3 * (t1 - t0) / steps,
            "backward_ms_per_cycle": 1e3 * (t2 - t1) / steps,
            "gradient_over_forward": (t2 - t0) / t_fwd, "backward_over_forward": (t2 - t1) / t_fwd,
            "checkpoint_every": rec["every"], "segment_cycles_resident": info["segment_sets"],
            "tail_cycles_resident_from_forward": rec["tail"],
            "device_bytes": info["device_bytes"],
            "timing": "host wall clock around device-synchronised calls, after an untimed gradient of min(8, steps) cycles; "
                      "forward = production exact step"}


# ----------------------------------------------------------------------------
# our arm
# ----------------------------------------------------------------------------
def run_ours(a):
    rank, world, local = dist_env()
    import torch
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    from pythonmhd_gb300 import build as _build
    if rank == 0:
        _build.build()
    if world > 1:
        torch.distributed.barrier()
    from pythonmhd_gb300 import initial_conditions as ic
    from pythonmhd_gb300.solver import Grid2D

    n = a.n
    gamma = 5.0 / 3.0
    # the seeded state, generated on the device (same generator as the host one, to rounding)
    prim, cons, fbx, fby, dx, dy = ic.turbulence_device(n, seed=a.seed + rank, gamma=gamma, device=dev)
    g = Grid2D(n, n, dx, dy, 1, 1, gamma, mhd=True, recon=a.recon, arith=a.arith)
    g.upload_device(prim, cons, fbx, fby)
    shapes = (tuple(prim.shape), tuple(cons.shape), tuple(fbx.shape), tuple(fby.shape))
    del prim, cons, fbx, fby
    torch.cuda.empty_cache()
    stream = torch.cuda.ExternalStream(g.stream(), device=dev)

    t, cyc = 0.0, 0
    big = 1e30
    # warm-up (untimed)
    t, cyc, _ = g.advance(t, big, cyc, cyc + a.warmup, 0.4)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()

    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    time.sleep(0.4)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    t, cyc, _ = g.advance(t, big, cyc, cyc + a.steps, 0.4)
    e1.record(stream)
    e1.synchronize()
    launches = g.last_launches()
    ms_total = e0.elapsed_time(e1)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()

    # e2e: host buffers through the C ABI, copies inside the timed region
    e2e_steps = a.e2e_steps or a.steps
    pin = lambda shape: torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()
    hp, hc, hbx, hby = (pin(sh) for sh in shapes)
    g.download(0, hp, hc, hbx, hby)
    h2d = (hp.nbytes + hc.nbytes + hbx.nbytes + hby.nbytes)
    d2h = h2d
    torch.cuda.synchronize()
    e2 = torch.cuda.Event(enable_timing=True)
    e3 = torch.cuda.Event(enable_timing=True)
    # per step: upload | cycle | download, each ended by the call's own stream sync
    ph = [[torch.cuda.Event(enable_timing=True) for _ in range(4)] for _ in range(e2e_steps)]
    e2.record(stream)
    for k in range(e2e_steps):
        ph[k][0].record(stream)
        g.upload(hp, hc, hbx, hby)
        ph[k][1].record(stream)
        t, cyc, _ = g.advance(t, big, cyc, cyc + 1, 0.4)
        ph[k][2].record(stream)
        g.download(0, hp, hc, hbx, hby)
        ph[k][3].record(stream)
    e3.record(stream)
    e3.synchronize()
    ms_e2e = e2.elapsed_time(e3)
    phase_ms = {name: sum(ph[k][i].elapsed_time(ph[k][i + 1]) for k in range(e2e_steps)) / e2e_steps
                for i, name in enumerate(("upload", "cycle", "download"))}
    # the copies alone, after the e2e loop: the link rate that e2e pays on this host
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    ev[0].record(stream)
    g.upload(hp, hc, hbx, hby)
    ev[1].record(stream)
    g.download(0, hp, hc, hbx, hby)
    ev[2].record(stream)
    ev[2].synchronize()
    copy_gbs = {"h2d": h2d / (ev[0].elapsed_time(ev[1]) * 1e-3) / 1e9,
                "d2h": d2h / (ev[1].elapsed_time(ev[2]) * 1e-3) / 1e9}
    clk = clocks.stop()
    dev_bytes = g.device_bytes()
    if not np.isfinite(hp).all():
        raise RuntimeError("non-finite state after the timed cycles")

    # max over ranks
    ms_per = ms_total / a.steps
    ms_e2e_per = ms_e2e / e2e_steps
    ms_per, ms_e2e_per = max_over_ranks([ms_per, ms_e2e_per], dev)
    zones = n * n
    value = replica_throughput(world, zones, ms_per)
    e2e_value = replica_throughput(world, zones, ms_e2e_per)

    peaks = measured_peaks()
    hbm_peak = peaks.get("hbm_gbs")
    peak_src = "measured" if hbm_peak else "fallback"
    hbm_peak = hbm_peak or 6800.0
    achieved = ALG_BYTES_PER_ZONE * zones / (ms_per * 1e-3) / 1e9
    prof = profile_summary(a.arith, a.recon)
    probe = fp64_peak() if rank == 0 else None
    traffic = None
    fp64 = None
    if prof:
        scale = zones / prof.get("zones", zones)
        if prof.get("dram_bytes_per_cycle"):
            traffic = prof["dram_bytes_per_cycle"] * scale
        fp64 = fp64_roof(prof, probe, zones, ms_per)
    roof = {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
            "frac": achieved / hbm_peak, "traffic": traffic,
            "kernel": f"one full cycle (CUDA graph of {launches // max(a.steps, 1)} kernels), 128 algorithmic B/zone",
            "peak_source": peak_src, "compute_bound": "fp64", "fp64": fp64}
    if fp64:
        # the binding roof, flat: fraction of the FP64-issue floor (each instruction class
        # at its own measured rate) and the floor itself
        roof.update({"fp64_frac_of_floor": fp64["frac"], "fp64_floor_ms": fp64["floor_ms_per_step"],
                     "fp64_achieved_ginstr_s": fp64["achieved"], "fp64_peak_ginstr_s": fp64["peak"]})

    # the other arithmetic mode on the same state (a fresh handle, the same warm-up)
    other = None
    if a.other_arith_steps > 0:
        other_mode = "fast" if a.arith == "exact" else "exact"
        torch.cuda.synchronize()
        prim0, cons0, fbx0, fby0, _, _ = ic.turbulence_device(n, seed=a.seed + rank, gamma=gamma, device=dev)
        g2 = Grid2D(n, n, dx, dy, 1, 1, gamma, mhd=True, recon=a.recon, arith=other_mode)
        g2.upload_device(prim0, cons0, fbx0, fby0)
        del prim0, cons0, fbx0, fby0
        torch.cuda.empty_cache()
        s2 = torch.cuda.ExternalStream(g2.stream(), device=dev)
        t2, c2, _ = g2.advance(0.0, big, 0, a.warmup, 0.4)
        torch.cuda.synchronize()
        f0 = torch.cuda.Event(enable_timing=True)
        f1 = torch.cuda.Event(enable_timing=True)
        f0.record(s2)
        g2.advance(t2, big, c2, c2 + a.other_arith_steps, 0.4)
        f1.record(s2)
        f1.synchronize()
        ms2 = f0.elapsed_time(f1) / a.other_arith_steps
        g2.close()
        torch.cuda.empty_cache()
        r2 = fp64_roof(profile_summary(other_mode, a.recon) or {}, probe, zones, ms2) if probe else None
        other = {"arith": other_mode, "value": zones / (ms2 * 1e-3), "ms_per_step": ms2,
                 "steps": a.other_arith_steps, "speed_vs_headline": ms_per / ms2,
                 "fp64_frac_of_floor": r2["frac"] if r2 else None,
                 "fp64_floor_ms": r2["floor_ms_per_step"] if r2 else None,
                 "parity": "per cycle within 1e-12 of the reference on every well-conditioned golden state and "
                           "along the full Orszag-Tang run (exact: bit for bit)"}

    cpu = None
    if rank == 0 and not a.no_cpu:
        cpu = cpu_baseline(a.cpu_sample, a.cpu_steps)
    batched = None
    if a.batch_steps > 0:
        g.close()
        batched = run_batch(a, torch)
    adjoint = None
    if a.adjoint_steps > 0:
        g.close()
        adjoint = run_adjoint(a, torch)
    hydro_3d = None
    if a.hydro3d_steps > 0:
        g.close()
        hydro_3d = run_hydro3d(a, torch)
    mhd_3d = None
    if a.mhd3d_steps > 0:
        g.close()
        mhd_3d = run_mhd3d(a, torch)

    recon_label = {0: "first-order", 1: "PLM", 2: "PPM"}[a.recon]
    metric = METRIC if a.recon == 2 else METRIC.replace("PPM", recon_label)
    line = {"metric": metric, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": ms_per, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"2D ideal-MHD driven-free turbulence {n}x{n} periodic, gamma=5/3, "
                                   f"{recon_label}+Roe+CTU+CT, CFL 0.4, FP64, seeded (seed {a.seed})",
                       "arith": a.arith, "cells": zones, "l2": "state 2.4 GB >> 129 MB L2 (no flush needed)",
                       "parallelism": f"replicas x{world}"},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "steps": e2e_steps, "ms_per_step": ms_e2e_per,
                    # flat numbers (nested objects do not survive every reader of this line)
                    "upload_ms": phase_ms["upload"], "cycle_ms": phase_ms["cycle"],
                    "download_ms": phase_ms["download"],
                    "other_ms": ms_e2e_per - sum(phase_ms.values()),
                    "h2d_gbs_alone": copy_gbs["h2d"], "d2h_gbs_alone": copy_gbs["d2h"]},
            "gpu_launches": launches, "roofline": roof, "cpu_baseline": cpu, "clocks": clk,
            "other_arith": other,
            "device_bytes": dev_bytes, "final_cycle": cyc, "final_time": t, "batched": batched,
            "adjoint": adjoint, "hydro3d": hydro_3d, "mhd3d": mhd_3d}
    if rank == 0:
        print(json.dumps(line), flush=True)
    g.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    else:
        run_ours(a)


if __name__ == "__main__":
    main()
