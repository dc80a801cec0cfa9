"""Throughput benchmark: particle-steps/s of the delta-SPH time step on one GB300.

Default workload: the dam break with mDBC walls at dx = 1/1024 (2,097,152 fluid particles,
tank 4x2, 3 wall layers), one step = integrate (symplectic Euler, two right-hand sides) +
delta+ shifting, as the reference runner does it. Synthetic inputs (the scene generator),
device-resident state larger than L2 (so no L2 flush between steps).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload NAME]

Prints one JSON line. ``--impl reference`` times the CPU restatement of the reference's
step (the oracle) on the host cores on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import copy
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s (plain delta-SPH step)"
WORKLOADS = {
    "dambreak_dx1024": dict(scene="dam_break", dx=1.0 / 1024),
    "dambreak_dx512": dict(scene="dam_break", dx=1.0 / 512),
    "dambreak_dx256": dict(scene="dam_break", dx=1.0 / 256),
    "tgv_64": dict(scene="taylor_green", nx=64),
}


def make_scene(name):
    from diffsph_gb300 import scenes
    w = WORKLOADS[name]
    if w["scene"] == "dam_break":
        return scenes.dam_break(dx=w["dx"])
    return scenes.taylor_green(w["nx"])


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) == 6:
                self.samples.append(parts)

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4) if s[2 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def algorithmic_bytes(nbar):
    """Per fluid particle (fixed, implementation-independent definition): pass B of one
    right-hand side reads the neighbor list (4 nbar + 4) and x, u, rho, gradRho (28) and
    writes the two rates (12); the whole plain step moves 24 nbar + 352."""
    return {"pass_b": 4 * nbar + 44, "step": 24 * nbar + 352}


def cpu_baseline(workload, budget_s=20.0):
    """The oracle (numpy restatement of the reference step) on a bounded sample."""
    from oracle import sph_oracle as O
    from diffsph_gb300 import scenes
    w = WORKLOADS[workload]
    if w["scene"] == "dam_break":
        cfg, st = scenes.dam_break(dx=1.0 / 64)
        sample = "dam break dx=1/64 (same scene and parameters, coarser lattice)"
    else:
        cfg, st = make_scene(workload)
        sample = workload
    n = st["fluid"]["positions"].shape[0]
    steps = 0
    t0 = time.perf_counter()
    s = copy.deepcopy(st)
    while True:
        s, _ = O.full_step(s, cfg)
        steps += 1
        if time.perf_counter() - t0 > budget_s or steps >= 50:
            break
    dt = time.perf_counter() - t0
    return {"value": n * steps / dt, "unit": "particle-steps/s", "cores": 1, "kind": "port",
            "sample": f"{sample}: {n} fluid particles x {steps} steps in {dt:.1f} s"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    steps, warm = args.steps, args.warmup
    from oracle import sph_oracle as O
    from diffsph_gb300 import scenes
    cfg, st = scenes.dam_break(dx=1.0 / 64) if WORKLOADS[args.workload]["scene"] == "dam_break" else make_scene(args.workload)
    n = st["fluid"]["positions"].shape[0]
    s = copy.deepcopy(st)
    for _ in range(warm):
        s, _ = O.full_step(s, cfg)
    t0 = time.perf_counter()
    for _ in range(steps):
        s, _ = O.full_step(s, cfg)
    dt = time.perf_counter() - t0
    v = n * steps / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "particle-steps/s", "n_gpus": args.gpus,
        "steps": steps, "warmup": warm, "ms_per_step": 1e3 * dt / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": args.workload, "sample": f"dam break dx=1/64, {n} fluid particles"},
        "cpu_baseline": {"value": v, "unit": "particle-steps/s", "cores": 1, "kind": "port",
                         "sample": f"{n} fluid particles x {steps} steps"},
        "e2e": {"value": v, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def run_ours(args):
    import torch
    import __graft_entry__ as ge
    from diffsph_gb300.neighborhood import exact_pairs
    from diffsph_gb300.solver import Solver

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        torch.distributed.init_process_group("nccl")
    torch.cuda.set_device(local)
    ge.build()
    cfg, st = make_scene(args.workload)
    fl, bd = st["fluid"], st.get("boundary")
    nF = fl["positions"].shape[0]
    nB = bd["positions"].shape[0] if bd is not None else 0
    sol = Solver(cfg, fl, bd)
    # mean exact neighbors per fluid particle (fluid + boundary neighbors, incl. self)
    allx = fl["positions"] if bd is None else __import__("numpy").concatenate([fl["positions"], bd["positions"]])
    allh = fl["supports"] if bd is None else __import__("numpy").concatenate([fl["supports"], bd["supports"]])
    _, offsets = exact_pairs(fl["positions"], allx, allh, cfg, count_only=True)
    nbar = int(offsets[-1].item()) / nF
    del offsets
    stream = torch.cuda.current_stream()
    shape, shape_ms = sol.autotune()
    for _ in range(args.warmup):
        sol.step(1)
    sol.check()
    torch.cuda.synchronize()
    # timed region: device-resident state, CUDA events on the launching stream
    sol.set_timing(["pass_b_rates", "pass_a_gradient", "shift", "cell_sort", "gather", "mdbc_ghosts"])
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            sol.step(1)
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    ktimes = sol.kernel_times()
    sol.set_timing([])
    sol.check()
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
        torch.distributed.barrier()
    value = world * nF * args.steps / (ms / 1e3)

    # end to end through the public API with host buffers: every step uploads the state
    # from pinned host memory, advances one step, and reads the state back
    hx = torch.from_numpy(fl["positions"]).pin_memory()
    hu = torch.from_numpy(fl["velocities"]).pin_memory()
    hr = torch.from_numpy(fl["densities"]).pin_memory()
    bx = torch.from_numpy(bd["positions"]).pin_memory() if nB else None
    bn = torch.from_numpy(bd["normals"]).pin_memory() if nB else None
    bdd = torch.from_numpy(bd["distances"]).pin_memory() if nB else None
    br = torch.from_numpy(bd["densities"]).pin_memory() if nB else None
    ox, ou, orr = torch.empty_like(hx).pin_memory(), torch.empty_like(hu).pin_memory(), torch.empty_like(hr).pin_memory()
    obr = torch.empty_like(br).pin_memory() if nB else None
    dev = {k: torch.empty(v.shape, device="cuda") for k, v in
           {"x": hx, "u": hu, "r": hr, **({"bx": bx, "bn": bn, "bd": bdd, "br": br} if nB else {})}.items()}
    e_steps = max(1, min(args.steps, 10))

    def e2e_step():
        dev["x"].copy_(hx, non_blocking=True)
        dev["u"].copy_(hu, non_blocking=True)
        dev["r"].copy_(hr, non_blocking=True)
        fluid = {"positions": dev["x"], "velocities": dev["u"], "densities": dev["r"]}
        bnd = None
        if nB:
            for k, h in (("bx", bx), ("bn", bn), ("bd", bdd), ("br", br)):
                dev[k].copy_(h, non_blocking=True)
            bnd = {"positions": dev["bx"], "normals": dev["bn"], "distances": dev["bd"], "densities": dev["br"]}
        sol.upload(fluid, bnd)
        sol.step(1)
        got = sol.download()
        ox.copy_(got["positions"], non_blocking=True)
        ou.copy_(got["velocities"], non_blocking=True)
        orr.copy_(got["densities"], non_blocking=True)
        if nB:
            obr.copy_(got["boundary_densities"], non_blocking=True)

    for _ in range(2):
        e2e_step()
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(e_steps):
        e2e_step()
    e1.record(stream)
    torch.cuda.synchronize()
    ms_e2e = e0.elapsed_time(e1)
    h2d = (hx.numel() + hu.numel() + hr.numel()) * 4 + ((bx.numel() + bn.numel() + bdd.numel() + br.numel()) * 4 if nB else 0)
    d2h = (ox.numel() + ou.numel() + orr.numel()) * 4 + (obr.numel() * 4 if nB else 0)
    e2e = {"value": world * nF * e_steps / (ms_e2e / 1e3), "unit": "particle-steps/s",
           "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "steps": e_steps}

    pk, pk_kind = peaks()
    ab = algorithmic_bytes(nbar)
    pb_ms, pb_n = ktimes.get("pass_b_rates", (0.0, 0))
    pb_avg = pb_ms / max(pb_n, 1)
    achieved = ab["pass_b"] * nF / (pb_avg / 1e3) / 1e9 if pb_avg > 0 else None
    step_achieved = ab["step"] * nF * args.steps / (ms / 1e3) / 1e9
    launches = sol.launches_per_step() * args.steps
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": args.workload, "fluid_particles": nF, "boundary_particles": nB,
                   "mean_neighbors": round(nbar, 3), "l2": "state and lists (> 1 GB) exceed L2; no flush",
                   "parallelism": "replicas" if world > 1 else "single",
                   "launch_shape": shape, "shape_ms": [round(v, 4) for v in shape_ms]},
        "e2e": e2e,
        "roofline": {"bound": "hbm", "kernel": "pass_b_rates", "achieved": achieved, "peak": pk,
                     "peak_kind": pk_kind, "unit": "GB/s",
                     "frac": (achieved / pk) if achieved else None, "traffic": None,
                     "alg_bytes_per_particle": ab["pass_b"], "avg_launch_ms": pb_avg,
                     "step_alg_bytes_per_particle": ab["step"], "step_achieved_gbs": step_achieved,
                     "step_frac": step_achieved / pk},
        "kernel_ms": {k: {"total_ms": v[0], "launches": v[1]} for k, v in ktimes.items() if v[1]},
        "gpu_launches": launches,
        "clocks": clk.summary(),
    }
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args.workload, budget_s=args.cpu_budget)
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="dambreak_dx1024", choices=list(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
