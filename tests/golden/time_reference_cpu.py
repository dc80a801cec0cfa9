"""Times the reference's own CPU step next to the oracle's port of it, on the same sample.

The benchmark's reference arm and CPU baseline run the oracle (numpy + C restatement of the
reference's step), because the reference itself (plain Python on torch) is not installed on
the GPU machine. This script calibrates that stand-in in the development container: it runs
the reference runner's step (integrate with symplecticEuler, then solveShifting; src/diffSPH/
v2/runner.py:37-42) through tests/golden/ref_harness.py on the dam break at dx = 1/64 (8,192
fluid particles) with torch on every host core, and the oracle's full_step on the same
scene on one core. The harness's candidate search (a brute-force stand-in for the external
torchCompactRadius package) is timed separately and excluded from the reference's figure.

    DIFFSPH_REF_SRC=<reference checkout>/src python tests/golden/time_reference_cpu.py

Prints one JSON line.
"""
import copy
import json
import os
import sys
import time

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from make_golden import reference_config, to_torch_state  # noqa: E402
from ref_harness import load_reference  # noqa: E402
from diffsph_gb300 import scenes  # noqa: E402
from oracle import sph_oracle as O  # noqa: E402


def main(steps=5):
    torch.set_num_threads(os.cpu_count() or 1)
    R = load_reference()
    shim = sys.modules["torchCompactRadius.neighborhood"]
    search_s = [0.0]
    inner = shim.neighborSearchExisting

    def timed(*a, **k):
        t0 = time.perf_counter()
        r = inner(*a, **k)
        search_s[0] += time.perf_counter() - t0
        return r

    shim.neighborSearchExisting = timed
    R.neighborhood.neighborSearchExisting = timed  # the reference's by-name copy (neighborhood.py:350)
    cfg, st = scenes.dam_break(dx=1.0 / 64)
    n = st["fluid"]["positions"].shape[0]
    rc = reference_config(R, cfg)
    state = {p: to_torch_state(v) for p, v in st.items()}
    perennial = dict(state)
    perennial.update(time=0.0, timestep=0, dt=rc["timestep"]["dt"])

    def step(p):
        p, *_ = R.integration.integrate(R.deltaPlus.simulationStep, p, rc, None)
        dx, _ = R.shifting.solveShifting(p, rc)
        p["fluid"]["positions"] = p["fluid"]["positions"] + dx
        return p

    perennial = step(perennial)  # warm-up
    search_s[0] = 0.0
    t0 = time.perf_counter()
    for _ in range(steps):
        perennial = step(perennial)
    total = time.perf_counter() - t0
    ref_s = total - search_s[0]
    # the oracle's port on the same scene, one core
    np.seterr(divide="ignore", invalid="ignore")
    s = copy.deepcopy(st)
    s, _ = O.full_step(s, cfg)
    t0 = time.perf_counter()
    for _ in range(steps):
        s, _ = O.full_step(s, cfg)
    port_s = time.perf_counter() - t0
    print(json.dumps({
        "sample": f"dam break dx=1/64, {n} fluid particles, {steps} steps",
        "reference_torch": {"threads": torch.get_num_threads(), "seconds": round(ref_s, 3),
                            "particle_steps_per_s": n * steps / ref_s,
                            "candidate_search_excluded_s": round(search_s[0], 3)},
        "oracle_port": {"cores": 1, "seconds": round(port_s, 3), "particle_steps_per_s": n * steps / port_s},
        "port_over_reference": (n * steps / port_s) / (n * steps / ref_s),
    }))


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else 5)
