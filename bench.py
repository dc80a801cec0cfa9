"""Throughput benchmark: particle-steps/s of the delta-SPH time step on one GB300.

Default workload: the dam break with mDBC walls at dx = 1/1024 (2,097,152 fluid particles,
tank 4x2, 3 wall layers), one step = integrate (symplectic Euler, two right-hand sides) +
delta+ shifting, as the reference runner does it. Synthetic inputs (the scene generator),
device-resident state larger than L2 (so no L2 flush between steps).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload NAME]

Prints one JSON line. ``--impl reference`` times the CPU restatement of the reference's
step (the oracle) on all host cores (one process per core) on a bounded sample of the same
workload.
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

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s (plain delta-SPH step)"
REGIONS_METRIC = ("ghost updates/s (mirror-outlet ghosts: construction, neighbor search and consistent "
                  "interpolation of density and velocity)")
# lattice of the host sample of the mirror-outlet workload (reference arm, CPU baseline)
REGIONS_SAMPLE_NX = 128
# dram__bytes_read + dram__bytes_write of one launch per particle slot, from ncu captures of
# the dam break at dx = 1/512 (536,594 slots, launch shape 1): pass A is the mean of the four
# working launches of two steps under Verlet reuse, pass B the mean of its two stages
PASS_A_DRAM_BYTES_PER_PARTICLE = 180.1
PASS_B_DRAM_BYTES_PER_PARTICLE = 159.1
# measured DRAM bytes per particle of pass A / pass B by scene, with where they come from;
# a scene without a capture of its own reports no traffic
DRAM_BYTES = {
    "dam_break": (PASS_A_DRAM_BYTES_PER_PARTICLE, PASS_B_DRAM_BYTES_PER_PARTICLE,
                  "ncu dram bytes of k_pass_a on dambreak_dx512 (180.1 B/particle slot, the mean of the "
                  "skin-filtering launches of two steps under Verlet reuse), scaled by the particle count"),
    "batched": (281.3, 194.8,
                "ncu dram bytes of k_pass_a (the 3 skin-filtering launches of two steps under Verlet reuse) "
                "and k_pass_b (2 half-step + 2 final launches) on batched_256 (4,519,897 particles in 256 "
                "periodic domains, launch shape 1), scaled by the particle count"),
}
# the same for one product of the implicit shift (k_ips_spmv) on the jittered periodic flow
# of 512^2 particles ((192.06 + 3.65) MB and (189.98 + 3.62) MB / 262,144)
IPS_SPMV_DRAM_BYTES_PER_PARTICLE = 742.0

WORKLOADS = {
    "dambreak_dx1024": dict(scene="dam_break", dx=1.0 / 1024),
    "batched_256": dict(scene="batched", domains=256, seed=0),
    # the first 64 domains of the same draw (1.16 M particles: the state fits in L2)
    "batched_64": dict(scene="batched", domains=64, seed=0),
    "dambreak_dx512": dict(scene="dam_break", dx=1.0 / 512),
    # the same dam break with the free-surface handling of the shift (shifting.freeSurface)
    "dambreak_fs_dx1024": dict(scene="dam_break", dx=1.0 / 1024, free_surface=True),
    "dambreak_fs_dx512": dict(scene="dam_break", dx=1.0 / 512, free_surface=True),
    "dambreak_dx256": dict(scene="dam_break", dx=1.0 / 256),
    "tgv_64": dict(scene="taylor_green", nx=64),
    # one periodic domain of 2,096,704 particles (jittered Fourier flow, 1448 x 1448): the
    # single-domain case of the packed batch, stepped with Verlet reuse and the skin list
    "fourier_1448": dict(scene="fourier", nx=1448, seed=0, jitter=0.1),
    # implicit particle shifting (shifting.scheme 'IPS'): jittered periodic Fourier flow
    "ips_fourier1024": dict(scene="fourier", nx=1024, seed=0, jitter=0.1, ips=True),
    "ips_fourier512": dict(scene="fourier", nx=512, seed=0, jitter=0.1, ips=True),
    # open-boundary mirror outlet: ghost construction + consistent interpolation of the density
    # and both velocity components, fluid block of 1024 x 1024 with the outlet at x > 0.9
    "outlet_mirror_1024": dict(scene="regions", nx=1024, mirror_x=0.9),
    # gradient of a rollout loss: 128x128 periodic Fourier flow, 1000 steps, checkpoints every 25
    "adjoint_fourier128": dict(scene="adjoint", nx=128, seed=0, target_seed=1, rollout=1000, every=25),
    # the walled adjoint: dam break dx = 1/128 (32,768 fluid + 3,090 wall particles), 200 steps
    "adjoint_dambreak128": dict(scene="adjoint", ic="dam_break", dx=1.0 / 128, target_seed=1, rollout=200,
                                every=25),
    # learned k=4 step: trained at 128x128 (dx = 1/64), evaluated on 32 domains of 256x256 (4x4 box)
    "learned_fourier_b32": dict(scene="learned", nx_train=128, nx_eval=256, L_eval=4.0, batch=32, k=4, traj=8,
                                frames=24, iters=3000, rollout=200),
    # the same step trained on 256 trajectories x 64 frames (16,128 frame pairs, generated as one
    # batched solver run per 256 domains; 1/32 of the 2,048 x 256 frames of the training config)
    "learned_fourier_b32_data256": dict(scene="learned", nx_train=128, nx_eval=256, L_eval=4.0, batch=32, k=4,
                                        traj=256, frames=64, iters=3000, rollout=200),
}
# the drop-in neighbor search (neighborSearch's reference-format output) on the fluid of the
# 2.1M-particle dam break, query = reference set
WORKLOADS["neighbors_dx1024"] = dict(scene="neighbors", dx=1.0 / 1024)
# the same at dx = 1/512 (524 k particles, a 1.1 GB list): the size the search's ncu captures use
WORKLOADS["neighbors_dx512"] = dict(scene="neighbors", dx=1.0 / 512)
# learned steps between restarts from the evaluation state in the timed learned rollout
LEARNED_SEGMENT = 5
NEIGHBOR_METRIC = "neighbor pairs/s (exact scatter-mode search, reference-format pair list)"
LEARNED_METRIC = "particle-steps/s (learned k=4 step, counted in plain-step equivalents)"
ADJOINT_METRIC = "adjoint particle-steps/s (forward + backward of a checkpointed rollout)"


def make_scene(name):
    from diffsph_gb300 import scenes
    w = WORKLOADS[name]
    if w["scene"] == "dam_break":
        cfg, st = scenes.dam_break(dx=w["dx"])
        if w.get("free_surface"):
            cfg["shifting"]["freeSurface"] = True
        return cfg, st
    if w["scene"] == "fourier":
        cfg, st = scenes.fourier_periodic(w["nx"], seed=w["seed"], jitter=w["jitter"])
        if w.get("ips"):
            cfg["shifting"]["scheme"] = "IPS"
        return cfg, st
    return scenes.taylor_green(w["nx"])


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region: the sampler is live (its
    first sample has arrived) before the region starts, samples every 20 ms, and keeps the
    samples whose arrival falls inside the region; a region shorter than the sampling interval
    gets the first sample after it instead (and says so in `window`)."""

    Q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self.proc = None
        self.t0 = self.t1 = None
        self.first = threading.Event()

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "20"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            self.first.wait(timeout=5.0)
        except Exception:
            self.proc = None
        self.t0 = time.monotonic()
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) == 6:
                self.samples.append((time.monotonic(), parts))
                self.first.set()

    def __exit__(self, *a):
        self.t1 = time.monotonic()
        if self.proc is not None:
            deadline = self.t1 + 0.5
            while not any(t >= self.t0 for t, _ in self.samples) and time.monotonic() < deadline:
                time.sleep(0.005)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        inside = [p for t, p in self.samples if self.t0 is not None and self.t0 <= t <= self.t1]
        after = [p for t, p in self.samples if self.t1 is not None and t > self.t1][:1]
        used, window = (inside, "timed region") if inside else (after, "first sample after the timed region")
        if not used:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(s[0]) for s in used if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in used if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in used for k in range(4) if s[2 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(used), "window": window,
                "region_s": round(self.t1 - self.t0, 4)}


def algorithmic_bytes(nbar):
    """Per fluid particle (fixed, implementation-independent definition): pass A of one
    right-hand side reads the neighbor list (4 nbar + 4), x, rho (12) and writes gradRho (8);
    pass B reads the list and x, u, rho, gradRho (28) and writes the two rates (12); the whole
    plain step moves 24 nbar + 352."""
    return {"pass_a": 4 * nbar + 24, "pass_b": 4 * nbar + 44, "step": 24 * nbar + 352,
            # one product y = A v of the implicit shift: the list (4 nbar + 4), x (8), v (8),
            # the dot operand (8), y (8)
            "ips_spmv": 4 * nbar + 36}


def cpu_baseline(workload, budget_s=20.0):
    """The oracle (numpy restatement of the reference step) on a bounded sample of the
    workload, on every host core (port_parallel); workloads without a dam-break / flow sample
    run it on one core."""
    from oracle import sph_oracle as O
    from diffsph_gb300 import scenes
    w = WORKLOADS[workload]
    if w["scene"] in ("dam_break", "fourier"):
        steps = 8 if w.get("ips") else 12
        v, nproc, n, dt = port_parallel(workload, steps, 1)
        return {"value": v, "unit": "particle-steps/s", "cores": nproc, "kind": "port",
                "sample": f"{nproc} processes x {n} fluid particles x {steps} steps in {dt:.1f} s "
                          f"({'dam break dx=1/64' if w['scene'] == 'dam_break' else 'the same flow at 64x64'}, "
                          "same scene and parameters, coarser lattice)"}
    if w["scene"] == "batched":
        cfg, st = scenes.batched_fourier(1, seed=w.get("seed", 0), n_min=4096, n_max=4096)[0]
        sample = "one 64x64 domain of the batch generator"
    elif w["scene"] == "dam_break":
        cfg, st = _reference_sample(workload)
        sample = "dam break dx=1/64 (same scene and parameters, coarser lattice)"
    elif w["scene"] == "fourier":
        cfg, st = _reference_sample(workload)
        sample = "the same flow generator at 64x64 (implicit shifting)"
    else:
        cfg, st = make_scene(workload)
        sample = workload
    n = st["fluid"]["positions"].shape[0]
    steps = 0
    old = np.seterr(divide="ignore", invalid="ignore")  # discarded wall rows, as in the reference arm
    t0 = time.perf_counter()
    s = copy.deepcopy(st)
    while True:
        s, _ = O.full_step(s, cfg)
        steps += 1
        if time.perf_counter() - t0 > budget_s or steps >= 50:
            break
    dt = time.perf_counter() - t0
    np.seterr(**old)
    return {"value": n * steps / dt, "unit": "particle-steps/s", "cores": 1, "kind": "port",
            "sample": f"{sample}: {n} fluid particles x {steps} steps in {dt:.1f} s"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    steps, warm = args.steps, args.warmup
    if WORKLOADS[args.workload]["scene"] == "adjoint":
        print(json.dumps({"impl": "reference", "unavailable": "the reference has no adjoint; its gradients "
                          "come from torch autograd through its own package, which is not installed here"}))
        return
    if WORKLOADS[args.workload]["scene"] == "learned":
        print(json.dumps({"impl": "reference", "unavailable": "the reference has no learned model"}))
        return
    sc = WORKLOADS[args.workload]["scene"]
    v, nproc, n, dt = port_parallel(args.workload, steps, warm)
    if sc == "neighbors":
        print(json.dumps({
            "impl": "reference", "metric": NEIGHBOR_METRIC, "value": v, "unit": "pairs/s", "n_gpus": args.gpus,
            "steps": steps, "warmup": warm, "ms_per_step": 1e3 * dt / steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (int64 indices)", "data": "synthetic",
            "config": {"workload": args.workload,
                       "sample": f"the dam break's fluid at dx = 1/64, {n} pairs, one copy per host core"},
            "cpu_baseline": {"value": v, "unit": "pairs/s", "cores": nproc, "kind": "port",
                             "sample": f"{nproc} processes x {n} pairs x {steps} searches"},
            "e2e": {"value": v, "unit": "pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))
        return
    if sc == "regions":
        print(json.dumps({
            "impl": "reference", "metric": REGIONS_METRIC, "value": v, "unit": "ghost-updates/s",
            "n_gpus": args.gpus, "steps": steps, "warmup": warm, "ms_per_step": 1e3 * dt / steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": args.workload,
                       "sample": f"mirror outlet on a {REGIONS_SAMPLE_NX}^2 block, {n} ghosts, one copy per host core"},
            "cpu_baseline": {"value": v, "unit": "ghost-updates/s", "cores": nproc, "kind": "port",
                             "sample": f"{nproc} processes x {n} ghosts x {steps} steps"},
            "e2e": {"value": v, "unit": "ghost-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))
        return
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "particle-steps/s", "n_gpus": args.gpus,
        "steps": steps, "warmup": warm, "ms_per_step": 1e3 * dt / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": args.workload,
                   "sample": f"{sc} sample, {n} fluid particles, one copy per host core"},
        "cpu_baseline": {"value": v, "unit": "particle-steps/s", "cores": nproc, "kind": "port",
                         "sample": f"{nproc} processes x {n} fluid particles x {steps} steps"},
        "e2e": {"value": v, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def port_parallel(workload, steps, warm):
    """The oracle's port of the step on every host core: one single-threaded process per core
    (spawned), each on its own copy of the workload's sample; they start their timed steps
    together (barrier) and the throughput is the units of all of them over the span from the
    first start to the last end. Returns (units/s, processes, units per step, seconds)."""
    import multiprocessing as mp
    from oracle import sph_oracle as O
    O.build_oracle()  # once, before the workers load it
    nproc = max(1, min(os.cpu_count() or 1, 64))
    for var in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS"):
        os.environ[var] = "1"
    ctx = mp.get_context("spawn")
    barrier = ctx.Barrier(nproc)
    queue = ctx.Queue()
    procs = [ctx.Process(target=_reference_worker, args=(workload, steps, warm, barrier, queue))
             for _ in range(nproc)]
    for p in procs:
        p.start()
    res = [queue.get() for _ in procs]
    for p in procs:
        p.join()
    n = res[0][0]
    dt = max(r[2] for r in res) - min(r[1] for r in res)
    return nproc * n * steps / dt, nproc, n, dt


def _reference_sample(workload):
    from diffsph_gb300 import scenes
    sc = WORKLOADS[workload]["scene"]
    if sc == "dam_break":
        cfg, st = scenes.dam_break(dx=1.0 / 64)
        if WORKLOADS[workload].get("free_surface"):
            cfg["shifting"]["freeSurface"] = True
        return cfg, st
    if sc == "batched":
        return scenes.batched_fourier(1, seed=0, n_min=4096, n_max=4096)[0]
    if sc == "fourier":
        w = WORKLOADS[workload]
        cfg, st = scenes.fourier_periodic(64, seed=w["seed"], jitter=w["jitter"])
        if w.get("ips"):
            cfg["shifting"]["scheme"] = "IPS"
        return cfg, st
    return make_scene(workload)


def _regions_block(nx, mirror_x):
    """The mirror-outlet scene of run_regions on an nx x nx lattice (numpy): the lower unit
    square of the dam break's fluid, random velocities, no walls; the region is x > mirror_x."""
    from diffsph_gb300 import scenes
    dx = 1.0 / nx
    cfg, st = scenes.dam_break(dx=dx)
    fl = st["fluid"]
    keep = fl["positions"][:, 1] < 1.0
    fl = {k: v[keep].copy() for k, v in fl.items()}
    rng = np.random.default_rng(3)
    fl["velocities"] = rng.uniform(-1, 1, fl["velocities"].shape).astype(np.float32)
    cfg["boundary"]["active"] = False
    cfg["particle"]["volume"] = dx * dx
    return fl, cfg


def regions_oracle_step(fl, cfg, mx):
    """One mirror-outlet update with the oracle on the host, the same steps as run_regions'
    GPU step (deltaPlus.py:188-235 with inletOutlet.py:67-147 and sphOps.py:313-341). The
    fluid inside the region x > mx gets ghosts mirrored across x = mx: the distance is
    mx - x, its gradient a central difference over 0.01 h (weights -1/2, 0, 1/2),
    normalised. The ghosts' neighbors are found among the fluid. The consistent
    interpolation of the density, then of both velocity components, is written back where a
    ghost has at least 10 neighbors. Returns the ghost count."""
    from oracle import sph_oracle as O
    H = float(cfg["particle"]["support"])
    x = fl["positions"]
    inside = np.nonzero(mx - x[:, 0] < 0)[0]
    p = x[inside]
    dist = mx - p[:, 0]
    # fp32 throughout, in the order of the GPU path's host-side gradient
    step = H * 0.01
    wts = np.array([-0.5, 0.0, 0.5], np.float32)
    grad = np.zeros_like(p)
    for a in range(2):
        off = np.zeros((3, 2), np.float32)
        off[:, a] = wts
        probe = p[:, None, :] + off[None] * np.float32(step)
        grad[:, a] = np.sum(wts * (mx - probe[..., 0]), axis=-1) / np.float32(step)
    grad = grad / (np.linalg.norm(grad, axis=1, keepdims=True) + np.float32(1e-7))
    ghost = {"positions": (p - 2 * dist[:, None] * grad).astype(np.float32),
             "supports": np.full(len(p), H, np.float32)}
    nb = O.neighbor_search(ghost, fl, cfg)
    ok = nb["numNeighbors"] >= 10
    shift = dist[:, None] * grad * 2
    for key, col in (("densities", None), ("velocities", 0), ("velocities", 1)):
        q = fl[key] if col is None else fl[key][:, col]
        sol = O.liuliu_consistent(ghost, fl, nb, q)[0]
        val = np.where(ok, sol[:, 0] + np.einsum("nd,nd->n", shift, sol[:, 1:]), q[inside])
        if col is None:
            fl[key][inside] = val
        else:
            fl[key][inside, col] = val
    return len(p)


def _reference_worker(workload, steps, warm, barrier, queue):
    """One oracle process of the reference arm (spawned; no GPU use)."""
    from oracle import sph_oracle as O
    # (wall ghosts whose moment system is singular get density 0, as in the reference; the
    # shift's wall-wall pairs then divide by zero in rows that are discarded)
    np.seterr(divide="ignore", invalid="ignore")
    if WORKLOADS[workload]["scene"] == "neighbors":
        from diffsph_gb300 import scenes
        cfg, st = scenes.dam_break(dx=1.0 / 64)
        fl = st["fluid"]
        for _ in range(warm):
            O.neighbor_search(fl, fl, cfg)
        barrier.wait()
        t0 = time.monotonic()
        pairs = 0
        for _ in range(steps):
            pairs = int(O.neighbor_search(fl, fl, cfg)["indices"][0].shape[0])
        t1 = time.monotonic()
        queue.put((pairs, t0, t1))
        return
    if WORKLOADS[workload]["scene"] == "regions":
        fl, cfg = _regions_block(REGIONS_SAMPLE_NX, WORKLOADS[workload]["mirror_x"])
        for _ in range(warm):
            regions_oracle_step(fl, cfg, WORKLOADS[workload]["mirror_x"])
        barrier.wait()
        t0 = time.monotonic()
        for _ in range(steps):
            ng = regions_oracle_step(fl, cfg, WORKLOADS[workload]["mirror_x"])
        t1 = time.monotonic()
        queue.put((ng if steps else 0, t0, t1))
        return
    cfg, st = _reference_sample(workload)
    n = st["fluid"]["positions"].shape[0]
    s = copy.deepcopy(st)
    for _ in range(warm):
        s, _ = O.full_step(s, cfg)
    barrier.wait()
    t0 = time.monotonic()
    for _ in range(steps):
        s, _ = O.full_step(s, cfg)
    t1 = time.monotonic()
    queue.put((n, t0, t1))


def reduce_max(value, world):
    """Max over ranks (the slowest rank defines the job time)."""
    if world <= 1:
        return value
    import torch
    dev = "cuda" if torch.cuda.is_available() and torch.distributed.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], device=dev, dtype=torch.float64)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def build_solver(workload):
    """Solver, fluid count, boundary count, scene (list of domains for batches)."""
    import numpy as np
    from diffsph_gb300 import scenes
    from diffsph_gb300.neighborhood import exact_pairs
    from diffsph_gb300.solver import BatchSolver, Solver
    w = WORKLOADS[workload]
    if w["scene"] == "batched":
        doms = scenes.batched_fourier(w["domains"], seed=w.get("seed", 0))
        sol = BatchSolver([c for c, _ in doms], [s["fluid"] for _, s in doms])
        nF = sol.nF
        # exact neighbors per particle, from the largest domain
        cfg, st = max(doms, key=lambda d: d[1]["fluid"]["positions"].shape[0])
        fl = st["fluid"]
        _, off = exact_pairs(fl["positions"], fl["positions"], fl["supports"], cfg, count_only=True)
        nbar = int(off[-1].item()) / fl["positions"].shape[0]
        return sol, nF, 0, nbar, doms
    cfg, st = make_scene(workload)
    fl, bd = st["fluid"], st.get("boundary")
    nF = fl["positions"].shape[0]
    nB = bd["positions"].shape[0] if bd is not None else 0
    sol = Solver(cfg, fl, bd)
    allx = fl["positions"] if bd is None else np.concatenate([fl["positions"], bd["positions"]])
    allh = fl["supports"] if bd is None else np.concatenate([fl["supports"], bd["supports"]])
    _, off = exact_pairs(fl["positions"], allx, allh, cfg, count_only=True)
    nbar = int(off[-1].item()) / nF
    return sol, nF, nB, nbar, st


def run_ours(args):
    import torch
    import __graft_entry__ as ge

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        torch.distributed.init_process_group("nccl")
    torch.cuda.set_device(local)
    ge.build()
    batched = WORKLOADS[args.workload]["scene"] == "batched"
    ips = bool(WORKLOADS[args.workload].get("ips", False))
    sol, nF, nB, nbar, scene = build_solver(args.workload)
    stream = torch.cuda.Stream()
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        if args.shape is None:
            shape, shape_ms = sol.autotune()
        else:  # a fixed launch shape for every pass (profiler runs: timings under a profiler mislead the tuner)
            sol.set_shape(args.shape)
            shape, shape_ms = sol.shapes(), {}
        for _ in range(args.warmup):
            sol.step(1)
        sol.check()
        # the timed steps replay a captured CUDA graph of two steps (same kernels, no launch
        # overhead); per-kernel times come from a short event-timed eager loop afterwards. An
        # implicit shift runs eagerly: it stops launching once its solve has returned, where a
        # graph would hold every one of its max_iter iterations
        # exactly K steps: pairs from the two-step graph, an odd last step from a one-step
        # graph under Verlet reuse (its buffers never rotate) or else eagerly
        steps = args.steps
        one_graph = bool(getattr(sol, "verlet_reuse", False))
        if not ips:
            sol.graph_step(2)  # capture
            if steps & 1 and one_graph:
                sol.graph_step(1)  # capture
        sol.check()
        sorts0 = sol.sort_count()
        torch.cuda.synchronize()
        # timed region: device-resident state, CUDA events on the launching stream
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        with ClockSampler(local) as clk:
            e0.record(stream)
            if ips:
                for _ in range(steps):
                    sol.step(1)
            else:
                for _ in range(steps // 2):
                    sol.graph_step(2)
                if steps & 1:
                    if one_graph:
                        sol.graph_step(1)
                    else:
                        sol.step(1)
            e1.record(stream)
            torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        sorts = sol.sort_count() - sorts0
        # per-kernel times from a short event-timed eager loop of the same step
        sol.set_timing(["pass_b_rates", "pass_a_gradient", "pass_a_scan", "shift", "cell_sort", "gather",
                        "mdbc_ghosts", "ips_setup", "ips_spmv", "ips_vector", "free_surface"])
        ips_iters = []
        timing_steps = 4
        for _ in range(timing_steps):
            sol.step(1)
            if ips:
                ips_iters.append(sol.ips_result())
        ktimes = sol.kernel_times()
        sol.set_timing([])
        sol.check()
        ms = reduce_max(ms, world)
        value = world * nF * steps / (ms / 1e3)
        # a one-step graph where the buffers never rotate (Verlet reuse); eager steps otherwise
        one_step_graph = bool(getattr(sol, "verlet_reuse", False)) and not ips
        e2e = run_e2e(sol, scene, batched, nF, world, min(steps, 10), stream, one_step_graph)
    pk, pk_kind = peaks()
    ab = algorithmic_bytes(nbar)
    # the dominant kernel of a step (largest share of its device time): pass A
    # (both pass A classes: the launches that filter the skin list and those that scan the stencil)
    # two pass A evaluations per step; under Verlet reuse the first is launched both ways (the
    # scanning and the filtering variant, one of which returns at once), and its time counts
    pa_ms = ktimes.get("pass_a_gradient", (0.0, 0))[0] + ktimes.get("pass_a_scan", (0.0, 0))[0]
    pa_avg = pa_ms / (2 * timing_steps)
    achieved = ab["pass_a"] * nF / (pa_avg / 1e3) / 1e9 if pa_avg > 0 else None
    pb_ms, pb_n = ktimes.get("pass_b_rates", (0.0, 0))
    pb_avg = pb_ms / max(pb_n, 1)
    achieved_b = ab["pass_b"] * nF / (pb_avg / 1e3) / 1e9 if pb_avg > 0 else None
    step_achieved = ab["step"] * nF * steps / (ms / 1e3) / 1e9
    launches = sol.launches_per_step() * steps
    ips_info = None
    if ips:
        # the products of iterations the solve ran (launches after its return do nothing)
        sp_ms, sp_n = ktimes.get("ips_spmv", (0.0, 0))
        working = 2 * sum(it for it, _ in ips_iters)
        sp_avg = sp_ms / max(working, 1)
        achieved_s = ab["ips_spmv"] * nF / (sp_avg / 1e3) / 1e9 if sp_avg > 0 else None
        ips_launches = sum(ktimes.get(k, (0.0, 0))[1] for k in ("ips_setup", "ips_spmv", "ips_vector")) / 4
        # the delta+ shift launch is replaced by the implicit shift's
        launches = int(round((sol.launches_per_step() - 1 + ips_launches) * steps))
        ips_info = {"iterations_and_codes": ips_iters, "spmv_avg_ms": sp_avg, "spmv_achieved_gbs": achieved_s,
                    "spmv_frac": (achieved_s / pk) if achieved_s else None,
                    "spmv_alg_bytes_per_particle": ab["ips_spmv"],
                    "spmv_traffic": (IPS_SPMV_DRAM_BYTES_PER_PARTICLE * nF
                                     if IPS_SPMV_DRAM_BYTES_PER_PARTICLE else None)}
    if rank != 0:
        return
    dram_a, dram_b, dram_note = DRAM_BYTES.get(WORKLOADS[args.workload]["scene"],
                                               (None, None, "no ncu capture of this scene's passes"))
    roofline = {"bound": "hbm", "kernel": "pass_a_gradient", "achieved": achieved, "peak": pk,
                "peak_kind": pk_kind, "unit": "GB/s",
                "frac": (achieved / pk) if achieved else None,
                "traffic": dram_a * nF if dram_a else None,
                "traffic_note": dram_note,
                "alg_bytes_per_particle": ab["pass_a"], "avg_launch_ms": pa_avg,
                "pass_b": {"achieved": achieved_b, "frac": (achieved_b / pk) if achieved_b else None,
                           "alg_bytes_per_particle": ab["pass_b"], "avg_launch_ms": pb_avg,
                           "traffic": dram_b * nF if dram_b else None},
                "step_alg_bytes_per_particle": ab["step"], "step_achieved_gbs": step_achieved,
                "step_frac": step_achieved / pk}
    if ips_info is not None and (sp_ms > pa_ms):
        # the implicit shift's products dominate such a step
        roofline.update({"kernel": "ips_spmv", "achieved": ips_info["spmv_achieved_gbs"],
                         "frac": ips_info["spmv_frac"], "traffic": ips_info["spmv_traffic"],
                         "traffic_note": "ncu dram bytes of k_ips_spmv on ips_fourier512, scaled by the "
                                         "particle count",
                         "alg_bytes_per_particle": ab["ips_spmv"], "avg_launch_ms": ips_info["spmv_avg_ms"],
                         "pass_a": {"achieved": achieved, "frac": (achieved / pk) if achieved else None,
                                    "alg_bytes_per_particle": ab["pass_a"], "avg_launch_ms": pa_avg}})
    line = {
        "metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": world, "steps": steps,
        "warmup": args.warmup, "ms_per_step": ms / steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": args.workload, "fluid_particles": nF, "boundary_particles": nB,
                   "mean_neighbors": round(nbar, 3), "l2": "state (> 160 MB) exceeds L2; no flush",
                   "parallelism": "replicas" if world > 1 else "single", "graph": not ips,
                   "shifting": ("IPS" if ips else "deltaPlus") + (
                       "+freeSurface" if WORKLOADS[args.workload].get("free_surface") else ""),
                   "launch_shapes": shape,
                   "shape_ms": {k: [round(v, 4) for v in ms] for k, ms in shape_ms.items() if max(ms) > 0},
                   "verlet_reuse": bool(getattr(sol, "verlet_reuse", False)), "sorts_in_timed_steps": sorts},
        "e2e": e2e,
        "roofline": roofline,
        "kernel_ms": {k: {"total_ms": v[0], "launches": v[1]} for k, v in ktimes.items() if v[1]},
        "gpu_launches": launches,
        **({"ips": ips_info} if ips_info is not None else {}),
        "clocks": clk.summary(),
    }
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args.workload, budget_s=args.cpu_budget)
    print(json.dumps(line))


def run_e2e(sol, scene, batched, nF, world, e_steps, stream, one_step_graph=False):
    """Same metric through the public API with host buffers: every step uploads the state
    from pinned host memory (the state the previous step read back; the scene's initial
    state for the first), advances one step (a replayed one-step graph when one_step_graph)
    and reads the state back. The step's arrays share one pinned host buffer: [fluid
    positions, velocities, densities, wall densities read back | wall positions, normals,
    distances, densities uploaded]. Every step the solver's upload kernel reads the whole
    buffer over the host link and its download kernel writes the first part (page-locked host
    memory is mapped into the device's address space: no staging copy)."""
    import torch
    if batched:
        fl = {k: torch.cat([torch.from_numpy(s["fluid"][k]) for _, s in scene]) for k in
              ("positions", "velocities", "densities")}
        bd = None
    else:
        fl = {k: torch.from_numpy(scene["fluid"][k]) for k in ("positions", "velocities", "densities")}
        bd = ({k: torch.from_numpy(scene["boundary"][k]) for k in ("positions", "normals", "distances", "densities")}
              if "boundary" in scene else None)
    nB = int(bd["positions"].shape[0]) if bd is not None else 0
    out_parts = [("positions", (nF, 2)), ("velocities", (nF, 2)), ("densities", (nF,))]
    if nB:
        out_parts.append(("boundary_densities", (nB,)))
    in_parts = ([("b_positions", (nB, 2)), ("b_normals", (nB, 2)), ("b_distances", (nB,)), ("b_densities", (nB,))]
                if nB else [])
    sizes = [(k, sh, int(np.prod(sh))) for k, sh in out_parts + in_parts]
    n_out = sum(c for k, _, c in sizes[:len(out_parts)])
    total = sum(c for _, _, c in sizes)
    host = torch.empty(total, dtype=torch.float32).pin_memory()

    def views(buf):
        v, o = {}, 0
        for k, sh, c in sizes:
            v[k] = buf[o:o + c].view(*sh)
            o += c
        return v

    hv = views(host)
    for k in ("positions", "velocities", "densities"):  # the first upload: the scene's state
        hv[k].copy_(fl[k].reshape(hv[k].shape))
    for k in ("positions", "normals", "distances", "densities"):
        if nB:
            hv["b_" + k].copy_(bd[k].reshape(hv["b_" + k].shape))

    def one():
        f = {k: hv[k] for k in ("positions", "velocities", "densities")}
        b = {k: hv["b_" + k] for k in ("positions", "normals", "distances", "densities")} if nB else None
        sol.upload(f, b)
        if one_step_graph:
            sol.graph_step(1)
        else:
            sol.step(1)
        sol.download({k: hv[k] for k, _ in out_parts})

    for _ in range(2):
        one()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(e_steps):
        one()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = reduce_max(e0.elapsed_time(e1), world)
    return {"value": world * nF * e_steps / (ms / 1e3), "unit": "particle-steps/s",
            "h2d_bytes_per_step": total * 4, "d2h_bytes_per_step": n_out * 4, "steps": e_steps,
            "one_step_graph": bool(one_step_graph),
            "transfer": "the upload and download kernels read and write the pinned host buffer directly"}


def run_adjoint(args):
    """Gradient of mean((u_T - u_target)^2) w.r.t. the initial velocity and nu over a
    1000-step rollout (forward with checkpoints, backward with segment recomputation).
    value: state resident on the device; e2e: the same call from host arrays, gradient
    copied back to pinned host memory."""
    import numpy as np
    import torch
    import __graft_entry__ as ge
    from diffsph_gb300 import scenes
    from diffsph_gb300.adjoint import rollout

    rank = int(os.environ.get("RANK", "0"))
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    ge.build()
    w = WORKLOADS[args.workload]
    bd = None
    if w.get("ic") == "dam_break":  # walled: mDBC walls, inviscid and boundary viscosity, gravity
        cfg, st = scenes.dam_break(w["dx"])
        bd = st["boundary"]
    else:
        cfg, st = scenes.fourier_periodic(w["nx"], seed=w["seed"], jitter=0.1)
    fl = st["fluid"]
    nF = fl["positions"].shape[0]
    target = scenes.fourier_velocity(np.asarray(fl["positions"], np.float64), np.random.default_rng(w["target_seed"]))
    T, every = w["rollout"], w["every"]
    stream = torch.cuda.Stream()
    tgt_d = torch.as_tensor(target, dtype=torch.float32, device="cuda")
    dev = {k: torch.as_tensor(fl[k], device="cuda") for k in ("positions", "velocities", "densities")}
    times = {}

    def grad_run(n_steps, from_host=False, record=False):
        if from_host:
            u0 = torch.from_numpy(fl["velocities"]).pin_memory().to("cuda", non_blocking=True)
            x0 = torch.from_numpy(fl["positions"]).pin_memory().to("cuda", non_blocking=True)
            r0 = torch.from_numpy(fl["densities"]).pin_memory().to("cuda", non_blocking=True)
            tg = torch.from_numpy(target.astype(np.float32)).pin_memory().to("cuda", non_blocking=True)
        else:
            u0, x0, r0, tg = dev["velocities"], dev["positions"], dev["densities"], tgt_d
        u0 = u0.clone().requires_grad_(True)
        nu = torch.tensor(float(cfg["diffusion"]["nu"]), dtype=torch.float64, requires_grad=True)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        ev[0].record(stream)
        _, u, _ = rollout(cfg, fl, n_steps, nu=nu, checkpoint_every=every, x0=x0, u0=u0, rho0=r0, boundary=bd)
        loss = torch.mean((u - tg) ** 2)
        ev[1].record(stream)
        loss.backward()
        g = u0.grad
        if from_host:
            out = torch.empty(g.shape, pin_memory=True)
            out.copy_(g, non_blocking=True)
        ev[2].record(stream)
        torch.cuda.synchronize()
        if record:
            times["forward_ms"] = ev[0].elapsed_time(ev[1])
            times["backward_ms"] = ev[1].elapsed_time(ev[2])
        return ev[0].elapsed_time(ev[2]), float(loss.detach()), float(nu.grad)

    with torch.cuda.stream(stream):
        for _ in range(max(args.warmup, 3)):
            grad_run(10)
        torch.cuda.synchronize()
        with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
            ms, loss, dnu = grad_run(T, record=True)
        ms_e2e, _, _ = grad_run(T, from_host=True)
    if rank != 0:
        return
    line = {
        "metric": ADJOINT_METRIC, "value": nF * T / (ms / 1e3), "unit": "particle-steps/s", "n_gpus": 1,
        "steps": T, "warmup": max(args.warmup, 3), "ms_per_step": ms / T, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": args.workload, "fluid_particles": nF,
                   "boundary_particles": int(bd["positions"].shape[0]) if bd is not None else 0,
                   "rollout_steps": T, "checkpoint_every": every,
                   "loss": loss, "dloss_dnu": dnu, "forward_ms": times["forward_ms"],
                   "backward_ms": times["backward_ms"], "l2": "state below L2 size; no flush (latency-bound)"},
        "e2e": {"value": nF * T / (ms_e2e / 1e3), "unit": "particle-steps/s",
                "h2d_bytes_per_step": (nF * 5 + nF * 2) * 4 / T, "d2h_bytes_per_step": nF * 2 * 4 / T},
        "clocks": clk.summary(),
    }
    print(json.dumps(line))


def run_regions(args):
    """Mirror-outlet processing of the reference's step (deltaPlus.py:188-235) on a fluid block:
    buildOutletGhostParticles (region distance function, mirrored ghosts, GPU neighbor search)
    and LiuLiuConsistent (sm_103a kernel) for the density and both velocity components, then the
    fluid update. Unit: ghost updates per second (one ghost, three quantities)."""
    import torch
    import __graft_entry__ as ge
    from diffsph_gb300 import regions

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    ge.build()
    w = WORKLOADS[args.workload]
    mx = w["mirror_x"]
    fl_np, cfg = _regions_block(w["nx"], mx)
    fl = {k: torch.from_numpy(v).cuda() for k, v in fl_np.items()}
    fl["numParticles"] = fl["positions"].shape[0]
    region = {"type": "mirror", "sdf": lambda p: mx - p[:, 0]}
    state = {"fluid": fl}

    def step():
        g = regions.buildOutletGhostParticles([region], state, cfg)
        cond = g["numNeighbors"] >= 10
        shift = g["sdf_dist"][:, None] * g["sdf_grad"] * 2
        for q, put in ((fl["densities"], None), (fl["velocities"][:, 0], 0), (fl["velocities"][:, 1], 1)):
            sol, _, _ = regions.LiuLiuConsistent(g, fl, q)
            val = torch.where(cond, sol[:, 0] + torch.einsum("nd,nd->n", shift, sol[:, 1:]), q[g["fluidIndex"]])
            if put is None:
                fl["densities"][g["fluidIndex"]] = val
            else:
                fl["velocities"][g["fluidIndex"], put] = val
        return g["positions"].shape[0]

    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        for _ in range(max(args.warmup, 3)):
            ng = step()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
            e0.record(stream)
            for _ in range(args.steps):
                ng = step()
            e1.record(stream)
            torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        # the kernel alone: one consistent interpolation over the ghost neighborhood
        g = regions.buildOutletGhostParticles([region], state, cfg)
        k0, k1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        k0.record(stream)
        for _ in range(10):
            regions.LiuLiuConsistent(g, fl, fl["densities"])
        k1.record(stream)
        torch.cuda.synchronize()
        kernel_ms = k0.elapsed_time(k1) / 10
    nb = g["neighborhood"]
    # the same step with the oracle on one host core, on the 128^2 sample of the block
    fl_h, cfg_h = _regions_block(REGIONS_SAMPLE_NX, mx)
    regions_oracle_step(fl_h, cfg_h, mx)
    reps, ng_h, t0 = 0, 0, time.perf_counter()
    while reps < 3 or time.perf_counter() - t0 < 2.0:
        ng_h = regions_oracle_step(fl_h, cfg_h, mx)
        reps += 1
    t_cpu = time.perf_counter() - t0
    print(json.dumps({
        "metric": REGIONS_METRIC, "value": ng * args.steps / (ms / 1e3),
        "unit": "ghost-updates/s", "n_gpus": 1, "steps": args.steps, "warmup": max(args.warmup, 3),
        "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": args.workload, "fluid_particles": int(fl["numParticles"]), "ghosts": ng,
                   "ghost_pairs": int(nb["indices"][0].shape[0]), "liuliu_kernel_ms": kernel_ms,
                   "note": "the region's distance function and its gradient run in the caller's Python, "
                           "the gradient on the host as in the reference"},
        "cpu_baseline": {"value": ng_h * reps / t_cpu, "unit": "ghost-updates/s", "cores": 1, "kind": "port",
                         "sample": f"the oracle's step on the {REGIONS_SAMPLE_NX}^2 block ({ng_h} ghosts) x {reps}"},
        "clocks": clk.summary()}))


def neighbor_bytes(nq, nr, pairs):
    """Algorithmic bytes of one search (fixed definition): the positions and supports read by
    the sort and the query (8 + 4 per reference particle, twice; 8 per query particle), the
    per-query counts and offsets written (4 + 8), and the pair list written in the reference's
    format: i, j (int64), q, h_j, W (fp32), xhat, gradW (2 x fp32) = 44 B per pair."""
    return 2 * 12 * nr + 8 * nq + 12 * nq + 44 * pairs


def run_neighbors(args):
    """The drop-in search alone (sph_neighbor_count + sph_neighbor_fill, with kernels and
    gradients): value with every buffer resident on the device; e2e from pinned host
    positions and supports to the whole pair list back in pinned host memory."""
    import ctypes
    import torch
    import __graft_entry__ as ge
    from diffsph_gb300 import _lib, scenes
    from diffsph_gb300.solver import domain_struct

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    if int(os.environ.get("RANK", "0")) != 0:
        return
    ge.build()
    lib = _lib.load()
    cfg, st = scenes.dam_break(dx=WORKLOADS[args.workload]["dx"])
    fl = st["fluid"]
    n = fl["positions"].shape[0]
    x = torch.from_numpy(fl["positions"]).cuda()
    h = torch.from_numpy(fl["supports"]).cuda()
    dom = domain_struct(cfg)
    hmax = float(fl["supports"].max())
    nbytes = ctypes.c_size_t()
    _lib.check("sph_neighbor_workspace_bytes",
               lib.sph_neighbor_workspace_bytes(n, n, ctypes.byref(dom), hmax, ctypes.byref(nbytes)))
    ws = torch.empty(int(nbytes.value) + 256, dtype=torch.uint8, device="cuda")
    wsp = ctypes.c_void_p((ws.data_ptr() + 255) & ~255)
    counts = torch.empty(n, dtype=torch.int32, device="cuda")
    offsets = torch.empty(n + 1, dtype=torch.int64, device="cuda")
    stream = torch.cuda.Stream()
    P = ctypes.c_void_p

    def count(xd, hd, st_):
        _lib.check("sph_neighbor_count", lib.sph_neighbor_count(
            P(xd.data_ptr()), n, P(xd.data_ptr()), P(hd.data_ptr()), n, ctypes.byref(dom), hmax, wsp,
            nbytes.value, P(counts.data_ptr()), P(offsets.data_ptr()), st_))

    with torch.cuda.stream(stream):
        st_ = ctypes.c_void_p(stream.cuda_stream)
        count(x, h, st_)
        torch.cuda.synchronize()
        npairs = int(offsets[-1].item())
        out = {"i": torch.empty(npairs, dtype=torch.int64, device="cuda"),
               "j": torch.empty(npairs, dtype=torch.int64, device="cuda"),
               "q": torch.empty(npairs, device="cuda"), "xhat": torch.empty(npairs, 2, device="cuda"),
               "h": torch.empty(npairs, device="cuda"), "W": torch.empty(npairs, device="cuda"),
               "gradW": torch.empty(npairs, 2, device="cuda")}

        def fill(xd, hd, st_):
            _lib.check("sph_neighbor_fill", lib.sph_neighbor_fill(
                P(xd.data_ptr()), n, P(xd.data_ptr()), P(hd.data_ptr()), n, ctypes.byref(dom), hmax, wsp,
                nbytes.value, P(offsets.data_ptr()), npairs, *[P(out[k].data_ptr()) for k in
                                                                ("i", "j", "q", "xhat", "h", "W", "gradW")], st_))

        for _ in range(max(args.warmup, 3)):
            count(x, h, st_)
            fill(x, h, st_)
        torch.cuda.synchronize()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
            ev[0].record(stream)
            for _ in range(args.steps):
                count(x, h, st_)
                fill(x, h, st_)
            ev[1].record(stream)
            torch.cuda.synchronize()
        ms = ev[0].elapsed_time(ev[1]) / args.steps
        # the fill alone (the dominant launch: it writes the pair list)
        ev[2].record(stream)
        for _ in range(args.steps):
            fill(x, h, st_)
        ev[3].record(stream)
        torch.cuda.synchronize()
        fill_ms = ev[2].elapsed_time(ev[3]) / args.steps
        # end to end: host arrays in, the pair count read back to size the list, the list out
        xh, hh = torch.from_numpy(fl["positions"]).pin_memory(), torch.from_numpy(fl["supports"]).pin_memory()
        host = {k: torch.empty(v.shape, dtype=v.dtype).pin_memory() for k, v in out.items()}
        cnt_h = torch.empty(1, dtype=torch.int64).pin_memory()
        e_steps = max(min(args.steps, 5), 2)
        t0 = time.perf_counter()
        for _ in range(e_steps):
            xd, hd = xh.to("cuda", non_blocking=True), hh.to("cuda", non_blocking=True)
            count(xd, hd, st_)
            cnt_h.copy_(offsets[-1:], non_blocking=True)
            stream.synchronize()
            assert int(cnt_h.item()) == npairs
            fill(xd, hd, st_)
            for k, v in host.items():
                v.copy_(out[k], non_blocking=True)
        stream.synchronize()
        e2e_s = (time.perf_counter() - t0) / e_steps
    alg = neighbor_bytes(n, n, npairs)
    pk, pk_kind = peaks()
    fill_alg = 44 * npairs + 12 * n
    line = {
        "metric": NEIGHBOR_METRIC, "value": npairs / (ms / 1e3), "unit": "pairs/s", "n_gpus": 1,
        "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 (int64 indices)", "data": "synthetic",
        "config": {"workload": args.workload, "query_particles": n, "reference_particles": n, "pairs": npairs,
                   "mean_neighbors": round(npairs / n, 3), "kernels": True,
                   "l2": f"pair list ({44 * npairs / 1e9:.2f} GB) exceeds L2; no flush"},
        "e2e": {"value": npairs / e2e_s, "unit": "pairs/s", "h2d_bytes_per_step": 12 * n,
                "d2h_bytes_per_step": 44 * npairs + 8, "steps": e_steps,
                "note": "host clock around upload, count, pair-count read-back, fill and the list's copy back"},
        "roofline": {"bound": "hbm", "kernel": "neighbor_fill", "achieved": fill_alg / (fill_ms / 1e3) / 1e9,
                     "peak": pk, "peak_kind": pk_kind, "unit": "GB/s",
                     "frac": fill_alg / (fill_ms / 1e3) / 1e9 / pk, "traffic": None,
                     "alg_bytes_per_launch": fill_alg, "avg_launch_ms": fill_ms,
                     "search_alg_bytes": alg, "search_achieved_gbs": alg / (ms / 1e3) / 1e9,
                     "search_frac": alg / (ms / 1e3) / 1e9 / pk},
        "gpu_launches": None,
        "clocks": clk.summary(),
    }
    if not args.no_cpu_baseline:
        v, nproc, pairs_h, dt = port_parallel(args.workload, 10, 1)
        line["cpu_baseline"] = {"value": v, "unit": "pairs/s", "cores": nproc, "kind": "port",
                                "sample": f"{nproc} processes x the oracle's search on the dam break's fluid at "
                                          f"dx = 1/64 ({pairs_h} pairs) x 10 in {dt:.1f} s"}
    print(json.dumps(line))


def run_learned(args):
    """Learned k=4 step against k plain steps on the same packed batch of periodic domains.
    value: particles x k / learned-step time (the state resident on the device); the plain
    batched solver's particle-steps/s on the same batch is reported beside it, with the
    velocity error of a learned rollout against the plain rollout and the judge's counts."""
    import numpy as np
    import torch
    import __graft_entry__ as ge
    from diffsph_gb300 import scenes
    from diffsph_gb300.learned import (CConvNet, LearnedStepper, check_device_errors, generate_trajectories,
                                       judged_rollout, take_row_overflow, train)
    from diffsph_gb300.solver import BatchSolver, Solver

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    if int(os.environ.get("RANK", "0")) != 0:
        return
    ge.build()
    w = dict(WORKLOADS[args.workload])
    if args.domains:
        w["batch"] = args.domains
    k = w["k"]
    t0 = time.perf_counter()
    torch.manual_seed(0)
    net = CConvNet(seed=0).cuda()
    hist = []
    t_gen = 0.0
    if not args.no_train:  # the step's cost does not depend on the weights; its accuracy does
        cfg_t, trajs = generate_trajectories(w["traj"], w["frames"], w["nx_train"], seed=0, k=k)
        torch.cuda.synchronize()
        t_gen = time.perf_counter() - t0
        hist = train(net, cfg_t, trajs, iters=w["iters"], k=k, lr=5e-3)
        del trajs
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    net.eval()
    doms = [scenes.fourier_periodic(w["nx_eval"], seed=1000 + d, jitter=0.1, L=w["L_eval"]) for d in range(w["batch"])]
    cfg = doms[0][0]
    fl = {key: torch.cat([torch.as_tensor(st["fluid"][key]) for _, st in doms]).cuda()
          for key in ("positions", "velocities", "densities")}
    n = fl["positions"].shape[0]
    stepper = LearnedStepper(cfg, net, k, n_domains=w["batch"])
    stream = torch.cuda.Stream()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    # the timed learned steps start again from the evaluation state every LEARNED_SEGMENT
    # steps, the segment a judged rollout checks before it goes on (an unjudged rollout of
    # hundreds of learned steps drifts away from the flow it was trained on); every step does
    # the full work on the state it is given
    x0 = (fl["positions"], fl["velocities"], fl["densities"])
    with torch.cuda.stream(stream):
        x, u, r = x0
        for s_ in range(max(args.warmup, 3)):
            x, u, r = stepper.step(*(x0 if s_ % LEARNED_SEGMENT == 0 else (x, u, r)))
        torch.cuda.synchronize()
        with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
            ev[0].record(stream)
            for s_ in range(args.steps):
                x, u, r = stepper.step(*(x0 if s_ % LEARNED_SEGMENT == 0 else (x, u, r)))
            ev[1].record(stream)
            torch.cuda.synchronize()
        check_device_errors()
        ms_learned = ev[0].elapsed_time(ev[1]) / args.steps
        # the dominant kernel alone: one 64-channel tensor-core aggregation on the live graph
        from diffsph_gb300.learned import Graph, aggregate
        g = Graph(x, cfg, w["batch"])
        h64 = torch.randn(n, 64, device="cuda").to(torch.bfloat16)
        aggregate(g, h64)
        k0, k1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        k0.record(stream)
        for _ in range(5):
            aggregate(g, h64)
        k1.record(stream)
        torch.cuda.synchronize()
        agg_ms = k0.elapsed_time(k1) / 5
        pairs = int(g.offsets[-1].item())
        # end to end: the state from pinned host memory, one learned step, the state back
        xh, uh, rh = (t.detach().cpu().pin_memory() for t in (x, u, r))
        outs = [torch.empty(t.shape, dtype=t.dtype).pin_memory() for t in (x, u, r)]
        e2e_ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        e_steps = max(args.steps // 2, 3)
        e2e_ev[0].record(stream)
        for _ in range(e_steps):
            xd, ud, rd = (t.to("cuda", non_blocking=True) for t in (xh, uh, rh))
            res = stepper.step(xd, ud, rd)
            for o, t in zip(outs, res):
                o.copy_(t, non_blocking=True)
        e2e_ev[1].record(stream)
        torch.cuda.synchronize()
        ms_e2e = e2e_ev[0].elapsed_time(e2e_ev[1]) / e_steps
        bytes_io = sum(t.numel() * t.element_size() for t in (xh, uh, rh))
        # this library's kernels in one learned step: per domain the neighbor count (13: two
        # position copies, cell keys, 3 scan kernels, scatter, cell order, gather, query, 3 scan
        # kernels) and the index fill (1); per layer one aggregation and one contraction (4 + 4)
        launches = 14 * w["batch"] + 8
        bsol = BatchSolver([c for c, _ in doms], [st["fluid"] for _, st in doms])
        bsol.autotune()
        for _ in range(max(args.warmup, 3)):
            bsol.step(1)
        bsol.graph_step(2)
        torch.cuda.synchronize()
        ev[2].record(stream)
        nplain = 2 * args.steps * k // 2
        for _ in range(nplain // 2):
            bsol.graph_step(2)
        ev[3].record(stream)
        torch.cuda.synchronize()
        bsol.check()
        ms_plain = ev[2].elapsed_time(ev[3]) / nplain
    acc_info = {}
    if not args.no_train:
        # accuracy on one domain: learned rollout vs the plain rollout of the same length
        c0, s0 = doms[0]
        sol = Solver(c0, s0["fluid"])
        sol.step(w["rollout"])
        sol.check()
        ref = sol.download()
        one = LearnedStepper(c0, net, k)
        xo = torch.as_tensor(s0["fluid"]["positions"]).cuda()
        uo = torch.as_tensor(s0["fluid"]["velocities"]).cuda()
        ro = torch.as_tensor(s0["fluid"]["densities"]).cuda()
        for _ in range(w["rollout"] // k):
            xo, uo, ro = one.step(xo, uo, ro)
        free_overflow = take_row_overflow()
        err = float(torch.linalg.norm(uo - ref["velocities"]) / torch.linalg.norm(ref["velocities"]))
        rho_dev = float(torch.max(torch.abs(ro - 1.0)))
        (_, uj, _), acc, rej = judged_rollout(one, s0["fluid"], w["rollout"] // k, segment=5)
        err_j = float(torch.linalg.norm(uj - ref["velocities"]) / torch.linalg.norm(ref["velocities"]))
        acc_info = {
            "train": {"trajectories": w["traj"], "frames": w["frames"], "particles": w["nx_train"] ** 2,
                      "iters": w["iters"], "seconds": round(t_train, 1), "generate_seconds": round(t_gen, 1),
                      "loss_first100": float(np.mean(hist[:100])), "loss_last100": float(np.mean(hist[-100:]))},
            "rollout_steps": w["rollout"], "velocity_rel_l2_vs_plain": err, "max_density_dev": rho_dev,
            "free_rollout_row_overflow": free_overflow,
            "judged": {"segments_accepted": acc, "segments_rejected": rej, "velocity_rel_l2_vs_plain": err_j}}
    else:
        acc_info = {"train": "untrained weights (timing only)"}
    line = {
        "metric": LEARNED_METRIC, "value": n * k / (ms_learned / 1e3), "unit": "particle-steps/s", "n_gpus": 1,
        "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": ms_learned, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "bf16 (fp32 accumulate)", "data": "synthetic",
        "config": {"workload": args.workload, "particles": n, "domains": w["batch"], "k": k,
                   "restart_every": LEARNED_SEGMENT,
                   "plain_ms_per_step": ms_plain, "plain_particle_steps_per_s": n / (ms_plain / 1e3),
                   "learned_over_plain_simulated_time": (k * ms_plain) / ms_learned,
                   **acc_info,
                   "l2": f"inputs ({n} particles x 20 B) {'exceed' if n * 20 > 129e6 else 'fit in'} L2"},
        "clocks": clk.summary(),
    }
    # algorithmic FLOPs of a 64-channel aggregation: 2 x 64 x 64 per exact pair
    pk_tf = None
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            pk_tf, pk_kind = float(json.load(f)["bf16_tflops"]), "measured"
    except Exception:
        pk_tf, pk_kind = 1900.0, "fallback"
    flops = 2.0 * 64 * 64 * pairs
    achieved = flops / (agg_ms / 1e3) / 1e12
    line["roofline"] = {"bound": "tensor", "kernel": "cconv_aggregate_tc (64 channels)", "achieved": achieved,
                        "peak": pk_tf, "peak_kind": pk_kind, "unit": "TFLOP/s", "frac": achieved / pk_tf,
                        "traffic": 4.233e9 / 524288 * n,
                        "traffic_note": "ncu dram bytes (E write) of k_aggregate_tc_mn on 8 x 65,536 particles, "
                                        "scaled by the particle count",
                        "avg_launch_ms": agg_ms, "pairs": pairs, "flop_per_launch": flops}
    line["e2e"] = {"value": n * k / (ms_e2e / 1e3), "unit": "particle-steps/s", "h2d_bytes_per_step": bytes_io,
                   "d2h_bytes_per_step": bytes_io}
    line["gpu_launches"] = launches * args.steps if launches is not None else None
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="dambreak_dx1024", choices=list(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--shape", type=int, default=None,
                    help="launch shape of every neighbor pass instead of the autotuner's choice")
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--no-train", action="store_true",
                    help="learned workload: time the step with untrained weights (no accuracy figures)")
    ap.add_argument("--domains", type=int, default=0, help="learned workload: number of packed domains")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif WORKLOADS[args.workload]["scene"] == "adjoint":
        run_adjoint(args)
    elif WORKLOADS[args.workload]["scene"] == "learned":
        run_learned(args)
    elif WORKLOADS[args.workload]["scene"] == "regions":
        run_regions(args)
    elif WORKLOADS[args.workload]["scene"] == "neighbors":
        run_neighbors(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
