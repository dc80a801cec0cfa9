"""GPU parity: the sm_103a library (through its C ABI) against the CPU oracle.

Tolerances (stated per check):
* neighbor sets bit-exact: identical (i, j) lists, q = r/h and the unit vectors bit-exact;
* per-particle fields: 1e-5 of the field's magnitude for densities and density rates,
  1e-4 for accelerations and velocities. Several fields are near-cancelling pair sums
  (the continuity rate of a divergence-free lattice flow, gradients downstream of the
  ill-conditioned mDBC moment solve), where any fp32 evaluation, the reference's included,
  carries rounding noise well above those bounds. Every field is therefore compared with
  an fp64 run of the oracle: the GPU error must stay within 4x the error of the fp32
  oracle (the reference's operation order) plus the stated tolerance times the magnitude.
"""
import copy

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from golden_io import CASES, load_case, rel_max  # noqa: E402
from oracle import sph_oracle as O  # noqa: E402
from diffsph_gb300 import scenes  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _lib_built():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from diffsph_gb300 import _lib
    _lib.load()


def _np(t):
    return t.detach().cpu().numpy()


def _as64(st):
    return {p: {k: (v.astype(np.float64) if v.dtype == np.float32 else v.copy()) for k, v in a.items()}
            for p, a in st.items()}


def assert_fp32_parity(gpu, o32, o64, tol, what=""):
    """|gpu - o64| <= 4 |o32 - o64| + tol * max|o64| (element-wise maxima)."""
    gpu, o32, o64 = (np.asarray(a, np.float64) for a in (gpu, o32, o64))
    e_gpu = float(np.max(np.abs(gpu - o64)))
    e_32 = float(np.max(np.abs(o32 - o64)))
    scale = float(np.max(np.abs(o64)))
    assert e_gpu <= 4 * e_32 + tol * scale, f"{what}: gpu err {e_gpu:.3e}, fp32 err {e_32:.3e}, scale {scale:.3e}"


def _cfg32(cfg):
    c = copy.deepcopy(cfg)
    c["oracle"] = {"pinv": "torch"}  # the reference's own fp32 moment solve
    return c


def _case_list():
    out = []
    for c in CASES:
        z, cfg, st = load_case(c)
        out.append((c, cfg, st))
    cfg, st = scenes.taylor_green(64)
    out.append(("tgv64_lattice", cfg, st))
    cfg, st = scenes.fourier_periodic(96, seed=5)
    out.append(("fourier96", cfg, st))
    cfg, st = scenes.dam_break(dx=1.0 / 32)
    out.append(("dambreak32", cfg, st))
    return out


CASE_LIST = _case_list()
IDS = [c[0] for c in CASE_LIST]


@pytest.mark.parametrize("name,cfg,st", CASE_LIST, ids=IDS)
def test_neighbor_search_bit_exact(name, cfg, st):
    from diffsph_gb300.neighborhood import neighborSearch
    fl = st["fluid"]
    ref = O.neighbor_search(fl, fl, cfg)
    _, nb = neighborSearch({k: torch.from_numpy(v) for k, v in fl.items()},
                           {k: torch.from_numpy(v) for k, v in fl.items()}, cfg)
    i, j = _np(nb["indices"][0]), _np(nb["indices"][1])
    assert np.array_equal(i, ref["indices"][0]) and np.array_equal(j, ref["indices"][1])
    assert np.array_equal(_np(nb["distances"]), ref["distances"])
    assert np.array_equal(_np(nb["vectors"]), ref["vectors"])
    assert np.array_equal(_np(nb["numNeighbors"]), ref["numNeighbors"])
    assert rel_max(_np(nb["kernels"]), ref["kernels"]) < 1e-6
    assert rel_max(_np(nb["gradients"]), ref["gradients"]) < 1e-6


def test_neighbor_search_query_vs_reference_sets():
    """Boundary -> fluid style search: separate query and reference sets, per-particle h."""
    from diffsph_gb300.neighborhood import neighborSearch
    cfg, st = scenes.dam_break(dx=1.0 / 32)
    fl, bd = st["fluid"], st["boundary"]
    ref = O.neighbor_search(fl, bd, cfg)
    _, nb = neighborSearch({k: torch.from_numpy(v) for k, v in fl.items()},
                           {k: torch.from_numpy(v) for k, v in bd.items()}, cfg)
    assert np.array_equal(_np(nb["indices"][0]), ref["indices"][0])
    assert np.array_equal(_np(nb["indices"][1]), ref["indices"][1])
    assert np.array_equal(_np(nb["distances"]), ref["distances"])


@pytest.mark.parametrize("scene", ["fourier_periodic", "dam_break"])
def test_neighbor_search_variable_supports(scene):
    """Scatter mode with a different support per reference particle (uniform in 0.5 H ..
    1.5 H): pairs, q = r/h_j, unit vectors and supports bit-exact; kernel values and
    gradients within 1e-6 relative (as for uniform supports: the reference's fp32 power
    (1 - q)**4 is not pinned to the last ulp)."""
    from diffsph_gb300.neighborhood import neighborSearch
    if scene == "fourier_periodic":
        cfg, st = scenes.fourier_periodic(40, seed=12, jitter=0.3)
        fl = st["fluid"]
        qs, rs = fl, dict(fl)
    else:
        cfg, st = scenes.dam_break(dx=1.0 / 32)
        qs, rs = st["fluid"], dict(st["boundary"])
    rng = np.random.default_rng(3)
    H = float(cfg["particle"]["support"])
    rs["supports"] = (H * rng.uniform(0.5, 1.5, rs["positions"].shape[0])).astype(np.float32)
    ref = O.neighbor_search(qs, rs, cfg)
    _, nb = neighborSearch({k: torch.from_numpy(np.asarray(v)) for k, v in qs.items()},
                           {k: torch.from_numpy(np.asarray(v)) for k, v in rs.items()}, cfg)
    assert np.array_equal(_np(nb["indices"][0]), ref["indices"][0])
    assert np.array_equal(_np(nb["indices"][1]), ref["indices"][1])
    for key in ("distances", "vectors", "supports"):
        assert np.array_equal(_np(nb[key]), ref[key]), key
    assert rel_max(_np(nb["kernels"]), ref["kernels"]) < 1e-6
    assert rel_max(_np(nb["gradients"]), ref["gradients"]) < 1e-6


def test_neighbor_search_rows_longer_than_the_warp_buffer():
    """Supports of 1.6-2.2 H give rows of ~120-240 pairs: those over the warp fill's shared
    buffer (128) take the one-thread path; all rows bit-exact against the oracle."""
    from diffsph_gb300.neighborhood import neighborSearch
    cfg, st = scenes.fourier_periodic(40, seed=13, jitter=0.2)
    qs, rs = st["fluid"], dict(st["fluid"])
    rng = np.random.default_rng(4)
    H = float(cfg["particle"]["support"])
    rs["supports"] = (H * rng.uniform(1.6, 2.2, rs["positions"].shape[0])).astype(np.float32)
    ref = O.neighbor_search(qs, rs, cfg)
    assert int(np.max(ref["numNeighbors"])) > 128
    _, nb = neighborSearch({k: torch.from_numpy(np.asarray(v)) for k, v in qs.items()},
                           {k: torch.from_numpy(np.asarray(v)) for k, v in rs.items()}, cfg)
    assert np.array_equal(_np(nb["indices"][0]), ref["indices"][0])
    assert np.array_equal(_np(nb["indices"][1]), ref["indices"][1])
    for key in ("distances", "vectors", "supports"):
        assert np.array_equal(_np(nb[key]), ref[key]), key


def test_neighbor_search_empty_and_isolated():
    from diffsph_gb300.neighborhood import exact_pairs
    cfg, _ = scenes.taylor_green(16)
    x = np.array([[0.0, 0.0], [0.9, 0.9]], np.float32)  # farther apart than h = 0.5
    h = np.full(2, 0.5, np.float32)
    i, j, *_ = exact_pairs(x, x, h, cfg)
    assert _np(i).tolist() == [0, 1] and _np(j).tolist() == [0, 1]
    i, j, *_ = exact_pairs(np.zeros((0, 2), np.float32), x, h, cfg)
    assert i.numel() == 0


def _solver(cfg, st):
    from diffsph_gb300.solver import Solver
    b = st.get("boundary")
    return Solver(cfg, st["fluid"], b)


@pytest.mark.parametrize("name,cfg,st", CASE_LIST, ids=IDS)
def test_rhs_matches_oracle(name, cfg, st):
    s32 = copy.deepcopy(st)
    (_, dudt32, drhodt32), _ = O.simulation_step(s32, _cfg32(cfg))
    s64 = _as64(st)
    (_, dudt64, drhodt64), _ = O.simulation_step(s64, cfg)
    sol = _solver(cfg, st)
    out = sol.rhs()
    torch.cuda.synchronize()
    f32, f64 = s32["fluid"], s64["fluid"]
    # the fused passes select exactly the reference's pairs
    nn = _np(out["numNeighbors"])
    assert np.array_equal(nn[:, 0], f32["neighborhood"]["numNeighbors"])
    if "boundary" in st:
        assert np.array_equal(nn[:, 1], s32["boundaryToFluidNeighborhood"]["numNeighbors"])
    assert_fp32_parity(_np(out["pressures"]), f32["pressures"], f64["pressures"], 1e-5, "pressures")
    assert_fp32_parity(_np(out["gradRho^L"]), f32["gradRho^L"], f64["gradRho^L"], 1e-5, "gradRho^L")
    assert_fp32_parity(_np(out["drhodt"]), drhodt32, drhodt64, 1e-5, "drhodt")
    assert_fp32_parity(_np(out["dudt"]), dudt32, dudt64, 1e-4, "dudt")
    if "boundary" in st:
        assert_fp32_parity(_np(out["boundary_densities"]), s32["boundary"]["densities"],
                           s64["boundary"]["densities"], 1e-5, "boundary densities")
    else:
        # fluid-only: the direct bound holds as well
        assert rel_max(_np(out["dudt"]), dudt32) < 1e-4


@pytest.mark.parametrize("name,cfg,st", CASE_LIST, ids=IDS)
def test_full_step_matches_oracle(name, cfg, st):
    r32, _ = O.full_step(copy.deepcopy(st), _cfg32(cfg))
    r64, _ = O.full_step(_as64(st), cfg)
    sol = _solver(cfg, st)
    sol.step(1)
    sol.check()
    got = sol.download()
    a, b = r32["fluid"], r64["fluid"]
    assert_fp32_parity(_np(got["velocities"]), a["velocities"], b["velocities"], 1e-4, "velocities")
    assert_fp32_parity(_np(got["densities"]), a["densities"], b["densities"], 1e-5, "densities")
    dx = float(cfg["particle"]["dx"])
    # positions: the shift is clamped to 0.05 dx; compare the increment x' - x^n
    x0 = st["fluid"]["positions"]
    assert_fp32_parity(_np(got["positions"]) - x0, a["positions"] - x0, b["positions"] - x0, 1e-4, "dx")
    if "boundary" not in st:
        # fluid-only: the direct bounds against the reference-order fp32 run hold as well
        assert rel_max(_np(got["velocities"]), a["velocities"]) < 1e-4
        assert rel_max(_np(got["densities"]), a["densities"]) < 1e-5
    if "boundary" in st:
        assert_fp32_parity(_np(got["boundary_densities"]), r32["boundary"]["densities"],
                           r64["boundary"]["densities"], 1e-5, "boundary densities")


@pytest.mark.parametrize("speed", [30.0, 45.0])
def test_fast_flow_falls_back_from_the_skin_list(speed):
    """Particles that move farther than the skin list allows (0.049 h since the sort) make
    the passes that would filter it scan the stencil instead, inside the sort's 0.13 h bound:
    at 30 m/s the step moves them about 0.07 h (the shift falls back), at 45 m/s the half step
    already moves them 0.054 h (the second pass A falls back too). The step still matches
    the oracle."""
    cfg, st = scenes.dam_break(dx=1.0 / 32)
    st = copy.deepcopy(st)
    st["fluid"]["velocities"][:, 0] = np.float32(speed)
    h = float(cfg["particle"]["support"])
    assert 0.05 * h < speed * float(cfg["timestep"]["dt"]) < 0.125 * h
    r32, _ = O.full_step(copy.deepcopy(st), _cfg32(cfg))
    r64, _ = O.full_step(_as64(st), cfg)
    sol = _solver(cfg, st)
    sol.step(1)
    sol.check()
    got = sol.download()
    a, b = r32["fluid"], r64["fluid"]
    assert_fp32_parity(_np(got["velocities"]), a["velocities"], b["velocities"], 1e-4, "velocities")
    assert_fp32_parity(_np(got["densities"]), a["densities"], b["densities"], 1e-5, "densities")
    x0 = st["fluid"]["positions"]
    assert_fp32_parity(_np(got["positions"]) - x0, a["positions"] - x0, b["positions"] - x0, 1e-4, "dx")


def test_integrate_then_shift_equals_step():
    """The runner's two calls (integrate, solveShifting) give the fused step's result; the
    standalone shift re-sorts the particles, so sums differ only in summation order."""
    cfg, st = scenes.fourier_periodic(64, seed=2)
    a = _solver(cfg, st)
    a.step(1)
    b = _solver(cfg, st)
    b.integrate()
    dx = b.shift()
    ga, gb = a.download(), b.download()
    assert torch.equal(ga["velocities"], gb["velocities"])
    assert torch.equal(ga["densities"], gb["densities"])
    d = float(cfg["particle"]["dx"])
    assert float((ga["positions"] - gb["positions"]).abs().max()) < 1e-6 * d + 2.5e-7
    # clamp at 0.05 dx per component, plus one fp32 rounding of x_new - x (|x| <= 1)
    assert float(dx.abs().max()) <= 0.05 * d + 1.2e-7


def test_ten_steps_track_oracle():
    cfg, st = scenes.taylor_green(32)
    s = copy.deepcopy(st)
    for _ in range(10):
        s, _ = O.full_step(s, cfg)
    sol = _solver(cfg, st)
    sol.step(10)
    sol.check()
    got = sol.download()
    assert rel_max(_np(got["velocities"]), s["fluid"]["velocities"]) < 1e-4
    assert rel_max(_np(got["densities"]) - 1.0, s["fluid"]["densities"] - 1.0) < 1e-3


@pytest.mark.parametrize("shape", list(range(5)))
def test_every_launch_shape_gives_the_same_step(shape):
    """All launch shapes of the autotuner (4, 8, 16 warps; 32- or 16-bit lists; one block
    per tile or a persistent grid) evaluate the same pairs in the same order."""
    cfg, st = scenes.dam_break(dx=1.0 / 32)
    a = _solver(cfg, st)
    a.step(2)
    b = _solver(cfg, st)
    b.set_shape(shape)
    b.step(2)
    b.check()
    ga, gb = a.download(), b.download()
    for k in ("positions", "velocities", "densities", "boundary_densities"):
        assert torch.equal(ga[k], gb[k]), k


def test_autotune_picks_a_shape_and_keeps_parity():
    cfg, st = scenes.fourier_periodic(64, seed=4)
    a = _solver(cfg, st)
    shapes, ms = a.autotune()
    assert shapes == a.shapes()
    for p in ("pass_a_scan", "pass_b", "shift"):
        assert 0 <= shapes[p] < len(ms[p]) and ms[p][shapes[p]] > 0
        assert ms[p][shapes[p]] == min(v for v in ms[p] if v > 0)
    # under Verlet reuse (the default at verletScale 1.5) a periodic domain filters a skin
    # list too; the continuity scheme sums no densities
    assert a.verlet_reuse and max(ms["pass_a_filter"]) > 0 and max(ms["density_sum"]) < 0
    a.step(1)
    b = _solver(cfg, st)
    b.step(1)
    ga, gb = a.download(), b.download()
    assert torch.equal(ga["velocities"], gb["velocities"])


def test_autotune_per_pass_on_the_dam_break_leaves_the_state_and_the_steps_unchanged():
    """The tuner runs every pass (the shift too) on the current state without moving it, and
    a Verlet-reuse solver steps on like an untuned one (up to the order of the pair sums:
    the tuner sorts at the current positions, the untuned solver keeps its older order)."""
    cfg, st = scenes.dam_break(dx=1.0 / 64)
    a = _solver(cfg, st)
    a.set_verlet_reuse(True)
    a.step(2)
    before = a.download()
    shapes, ms = a.autotune()
    after = a.download()
    for k in ("positions", "velocities", "densities"):
        assert torch.equal(before[k], after[k]), k
    assert max(ms["pass_a_filter"]) > 0 and max(ms["shift"]) > 0
    a.step(3)
    a.check()
    b = _solver(cfg, st)
    b.set_verlet_reuse(True)
    b.step(5)
    ga, gb = a.download(), b.download()
    d = float(cfg["particle"]["dx"])
    assert float((ga["positions"] - gb["positions"]).abs().max()) < 1e-5 * d
    assert rel_max(_np(ga["velocities"]), _np(gb["velocities"])) < 1e-5
    assert rel_max(_np(ga["densities"]), _np(gb["densities"])) < 1e-6


def test_reupload_keeps_the_order_under_verlet_reuse():
    """A state read back and uploaded again keeps the particles' slots: no sort is forced,
    and the run continues bit for bit as if it had never left the device."""
    cfg, st = scenes.dam_break(dx=1.0 / 64)
    a = _solver(cfg, st)
    a.set_verlet_reuse(True)
    b = _solver(cfg, st)
    b.set_verlet_reuse(True)
    a.step(4)
    b.step(4)
    got = b.download()
    b.upload({k: got[k] for k in ("positions", "velocities", "densities")}, st["boundary"])
    b.step(1)
    s0 = a.sort_count()
    a.step(1)
    assert b.sort_count() == a.sort_count() - s0  # the same sorts as the run that stayed
    a.step(3)
    b.step(3)
    b.check()
    ga, gb = a.download(), b.download()
    for k in ("positions", "velocities", "densities", "boundary_densities"):
        assert torch.equal(ga[k], gb[k]), k


def test_page_locked_host_state_round_trip_equals_the_device_path():
    """Upload from and download into page-locked host tensors (read and written by the
    solver's kernels over the host link, no staging copy) give the device path's state bit
    for bit, through a re-upload that keeps the order under Verlet reuse and through a sort."""
    cfg, st = scenes.dam_break(dx=1.0 / 64)
    a = _solver(cfg, st)
    b = _solver(cfg, st)
    nF, nB = st["fluid"]["positions"].shape[0], st["boundary"]["positions"].shape[0]
    host = {"positions": torch.empty(nF, 2).pin_memory(), "velocities": torch.empty(nF, 2).pin_memory(),
            "densities": torch.empty(nF).pin_memory(), "boundary_densities": torch.empty(nB).pin_memory()}
    bnd = {k: torch.from_numpy(np.ascontiguousarray(st["boundary"][k], np.float32)).pin_memory()
           for k in ("positions", "normals", "distances")}
    for _ in range(3):
        a.step(2)
        b.step(2)
        got = b.download(host)
        torch.cuda.synchronize()
        ref = a.download()
        for k in host:
            assert torch.equal(got[k], ref[k].cpu()), k
        b.upload({k: host[k] for k in ("positions", "velocities", "densities")},
                 dict(bnd, densities=host["boundary_densities"]))
        dev = {k: ref[k] for k in ("positions", "velocities", "densities")}
        a.upload(dev, dict({k: torch.from_numpy(np.ascontiguousarray(st["boundary"][k], np.float32)).cuda()
                            for k in ("positions", "normals", "distances")}, densities=ref["boundary_densities"]))
    a.step(3)
    b.step(3)
    b.check()
    assert a.sort_count() == b.sort_count()
    ga, gb = a.download(), b.download()
    for k in ("positions", "velocities", "densities", "boundary_densities"):
        assert torch.equal(ga[k], gb[k]), k
    with pytest.raises(ValueError):
        b.download({"positions": torch.empty(nF, 2), "velocities": host["velocities"],
                    "densities": host["densities"], "boundary_densities": host["boundary_densities"]})


def test_per_pass_shapes_mix_in_one_batched_step():
    """Different shapes per pass (persistent and one-block-per-tile grids mixed) on a packed
    batch give the same state as the default shape."""
    from diffsph_gb300.solver import BatchSolver
    doms = [scenes.fourier_periodic(nx, seed=20 + nx, jitter=0.1) for nx in (24, 40, 33)]
    a = BatchSolver([c for c, _ in doms], [s["fluid"] for _, s in doms])
    b = BatchSolver([c for c, _ in doms], [s["fluid"] for _, s in doms])
    b.set_shape(4, "pass_a_scan")
    b.set_shape(3, "pass_b")
    b.set_shape(4, "shift")
    assert b.shapes()["pass_b"] == 3 and b.shapes()["shift"] == 4
    a.step(3)
    b.step(3)
    b.check()
    ga, gb = a.download(), b.download()
    for k in ("positions", "velocities", "densities"):
        assert torch.equal(ga[k], gb[k]), k


def test_reference_runner_loop_with_dropins():
    """The reference runner's loop body (integrate -> solveShifting -> positions += dx)
    with the drop-in functions, against the fused step."""
    from diffsph_gb300 import scheme
    cfg, st = scenes.dam_break(dx=1.0 / 32)
    state = {p: {k: torch.from_numpy(v).cuda() for k, v in a.items()} for p, a in st.items()}
    for _ in range(3):
        state, *_ = scheme.integrate(scheme.simulationStep, state, cfg)
        dx, _ = scheme.solveShifting(state, cfg)
        state["fluid"]["positions"] = state["fluid"]["positions"] + dx
    ref = _solver(cfg, st)
    ref.step(3)
    got = ref.download()
    d = float(cfg["particle"]["dx"])
    assert float((state["fluid"]["positions"] - got["positions"]).abs().max()) < 1e-4 * d
    assert rel_max(_np(state["fluid"]["velocities"]), _np(got["velocities"])) < 1e-4
    assert rel_max(_np(state["fluid"]["densities"]), _np(got["densities"])) < 1e-6


def test_simulation_step_dropin_matches_oracle():
    from diffsph_gb300 import scheme
    cfg, st = scenes.taylor_green(32)
    s32 = copy.deepcopy(st)
    (_, dudt32, drhodt32), _ = O.simulation_step(s32, cfg)
    state = {p: {k: torch.from_numpy(v).cuda() for k, v in a.items()} for p, a in st.items()}
    (u, dudt, drhodt), (ub, _, _) = scheme.simulationStep(state, cfg)
    assert ub is None
    assert rel_max(_np(dudt), dudt32) < 1e-4
    assert np.array_equal(_np(state["fluid"]["numNeighbors"]), s32["fluid"]["numNeighbors"])
    assert rel_max(_np(state["fluid"]["L"]).reshape(-1, 2, 2), s32["fluid"]["L"]) < 1e-4



def test_batched_domains_equal_single_domain_solvers():
    """Packed batch of uneven periodic domains == one solver per domain, bit for bit."""
    from diffsph_gb300.solver import BatchSolver
    doms = scenes.batched_fourier(5, seed=11, n_min=256, n_max=4096)
    batch = BatchSolver([c for c, _ in doms], [s["fluid"] for _, s in doms])
    # sorting every step (under Verlet reuse the batch sorts when any domain needs it, a
    # solver of one domain when that domain does: the pair sums' order would differ)
    batch.set_verlet_reuse(False)
    batch.step(3)
    batch.check()
    got = batch.download()
    parts = {k: batch.split(got[k]) for k in ("positions", "velocities", "densities")}
    for d, (cfg, st) in enumerate(doms):
        one = _solver(cfg, st)
        one.set_verlet_reuse(False)
        one.step(3)
        ref = one.download()
        for k in ("positions", "velocities", "densities"):
            assert torch.equal(parts[k][d], ref[k]), (d, k)


def test_batched_domain_matches_oracle():
    from diffsph_gb300.solver import BatchSolver
    doms = scenes.batched_fourier(3, seed=2, n_min=256, n_max=1024)
    batch = BatchSolver([c for c, _ in doms], [s["fluid"] for _, s in doms])
    batch.step(1)
    got = batch.download()
    vel = batch.split(got["velocities"])
    for d, (cfg, st) in enumerate(doms):
        ref, _ = O.full_step(copy.deepcopy(st), cfg)
        assert rel_max(_np(vel[d]), ref["fluid"]["velocities"]) < 1e-4


def test_graph_replay_equals_plain_steps():
    cfg, st = scenes.fourier_periodic(48, seed=9)
    a = _solver(cfg, st)
    a.step(4)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        b = _solver(cfg, st)
        b.graph_step(2)
        b.graph_step(2)
        gb = b.download()
    s.synchronize()
    ga = a.download()
    for k in ("positions", "velocities", "densities"):
        assert torch.equal(ga[k], gb[k]), k


@pytest.mark.parametrize("scene", ["fourier_periodic", "dam_break"])
def test_graph_replay_interleaved_with_eager_steps(scene):
    """Eager steps between replays rotate the solver's buffers; the replays must follow
    (graphs are keyed by the buffer assignment): 1 + 2 + 1 + 2 + 2 steps equal 8 plain steps."""
    cfg, st = scenes.fourier_periodic(48, seed=9) if scene == "fourier_periodic" else scenes.dam_break(dx=1.0 / 32)
    a = _solver(cfg, st)
    a.step(8)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        b = _solver(cfg, st)
        b.step(1)
        b.graph_step(2)
        b.step(1)
        b.graph_step(2)
        b.graph_step(2)
        gb = b.download()
    s.synchronize()
    ga = a.download()
    for k in ("positions", "velocities", "densities"):
        assert torch.equal(ga[k], gb[k]), k


def test_taylor_green_decays_at_the_viscous_rate():
    """Accuracy (not parity): the Taylor-Green vortex u = (-cos(pi x) sin(pi y),
    sin(pi x) cos(pi y)) of viscosity nu = 0.01 decays as exp(-2 pi^2 nu t). Its amplitude
    A(t) = sum u . u_exact(x) / sum u_exact(x)^2 after 500 steps (t = 0.9375) on the 64^2
    lattice stays within 0.5 % of that: the fp32 oracle's A is 0.83135 there, 1.0004 times
    exp(-2 pi^2 nu t) = 0.83106."""
    cfg, st = scenes.taylor_green(64)
    sol = _solver(cfg, st)
    steps = 500
    sol.step(steps)
    sol.check()
    got = sol.download()
    x = _np(got["positions"]).astype(np.float64)
    u = _np(got["velocities"]).astype(np.float64)
    ue = np.stack([-np.cos(np.pi * x[:, 0]) * np.sin(np.pi * x[:, 1]),
                   np.sin(np.pi * x[:, 0]) * np.cos(np.pi * x[:, 1])], -1)
    amp = float(np.sum(u * ue) / np.sum(ue * ue))
    t = steps * float(cfg["timestep"]["dt"])
    assert abs(t - 0.9375) < 1e-9
    nu = float(cfg["diffusion"]["nu"])
    assert abs(amp / np.exp(-2 * np.pi ** 2 * nu * t) - 1) < 5e-3, amp


def test_verlet_reuse_skips_sorts_and_matches_sorting_every_step():
    """Verlet reuse (on by default, as the reference reuses its neighbor structure at
    neighborhood.verletScale = 1.5): in the dam break's first steps the
    column's foot moves 0.002-0.013 h per step, so only some steps sort (about one in three).
    The state equals that of a solver sorting every step up to the order of each particle's
    pair sums; a graph replay equals the eager steps bit for bit."""
    cfg, st = scenes.dam_break(dx=1.0 / 32)
    a = _solver(cfg, st)
    assert a.verlet_reuse
    b = _solver(cfg, st)
    b.set_verlet_reuse(False)
    a.step(12)
    b.step(12)
    a.check()
    b.check()
    assert b.sort_count() == 12
    assert 2 <= a.sort_count() < 12
    ga, gb = a.download(), b.download()
    assert rel_max(_np(ga["velocities"]), _np(gb["velocities"])) < 1e-4
    assert rel_max(_np(ga["densities"]), _np(gb["densities"])) < 1e-5
    assert float((ga["positions"] - gb["positions"]).abs().max()) < 1e-6
    c = _solver(cfg, st)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        for _ in range(6):
            c.graph_step(2)
        gc = c.download()
    s.synchronize()
    assert c.sort_count() == a.sort_count()
    for k in ("positions", "velocities", "densities", "boundary_densities"):
        assert torch.equal(ga[k], gc[k]), k
    # the buffers never rotate under reuse, so one-step graphs replay too
    d = _solver(cfg, st)
    with torch.cuda.stream(s):
        for _ in range(12):
            d.graph_step(1)
        gd = d.download()
    s.synchronize()
    for k in ("positions", "velocities", "densities", "boundary_densities"):
        assert torch.equal(ga[k], gd[k]), k


def test_verlet_reuse_sorts_every_step_of_a_fast_flow():
    """At 20 m/s a step moves every particle 0.048 h, past the 0.034 h reuse limit: each step
    sorts, and the result equals sorting every step bit for bit."""
    cfg, st = scenes.dam_break(dx=1.0 / 32)
    st = copy.deepcopy(st)
    st["fluid"]["velocities"][:, 0] = np.float32(20.0)
    a = _solver(cfg, st)
    b = _solver(cfg, st)
    b.set_verlet_reuse(False)
    a.step(3)
    b.step(3)
    a.check()
    b.check()
    assert a.sort_count() == 3
    ga, gb = a.download(), b.download()
    for k in ("positions", "velocities", "densities", "boundary_densities"):
        assert torch.equal(ga[k], gb[k]), k


def _drifting_fourier(nx, seed):
    """A jittered periodic Fourier flow at 0.3 of its speed plus a drift of (0.6, 0.35): about
    0.015 h per step, so particles cross the periodic boundary between Verlet sorts."""
    cfg, st = scenes.fourier_periodic(nx, seed=seed, jitter=0.1)
    st = copy.deepcopy(st)
    v = st["fluid"]["velocities"]
    st["fluid"]["velocities"] = (np.float32(0.3) * v + np.array([0.6, 0.35], np.float32)).astype(np.float32)
    return cfg, st


def test_verlet_reuse_on_periodic_domains():
    """Verlet reuse on a periodic domain (on by default at verletScale 1.5, as the reference
    reuses its neighborhood on any domain): fewer sorts than steps while particles cross the
    periodic boundary between sorts; the state equals that of a solver sorting every step up
    to the order of each particle's pair sums, and one-step graph replays equal the eager
    steps bit for bit. Rows away from the wrap filter the skin list without the minimum
    image: a pair that needed it there would be lost and move the state by far more."""
    from diffsph_gb300._lib import SphError
    cfg, st = _drifting_fourier(48, seed=9)
    a = _solver(cfg, st)
    assert a.verlet_reuse
    b = _solver(cfg, st)
    b.set_verlet_reuse(False)
    a.step(40)
    b.step(40)
    a.check()
    b.check()
    assert b.sort_count() == 40
    assert 2 <= a.sort_count() <= 30, a.sort_count()
    ga, gb = a.download(), b.download()
    hi = torch.tensor(cfg["domain"]["maxExtent"], dtype=torch.float32)
    assert bool((ga["positions"].cpu() > hi).any())  # raw positions past the wrap
    assert rel_max(_np(ga["velocities"]), _np(gb["velocities"])) < 1e-3
    assert rel_max(_np(ga["densities"]), _np(gb["densities"])) < 1e-5
    assert float((ga["positions"] - gb["positions"]).abs().max()) < 1e-5
    s = torch.cuda.Stream()
    c = _solver(cfg, st)
    with torch.cuda.stream(s):
        for _ in range(40):
            c.graph_step(1)
        gc = c.download()
    s.synchronize()
    assert c.sort_count() == a.sort_count()
    for k in ("positions", "velocities", "densities"):
        assert torch.equal(ga[k], gc[k]), k
    # without reuse every step rotates the buffers: graphs hold an even number of steps
    with torch.cuda.stream(s):
        with pytest.raises(SphError):
            b.graph_step(1)
    s.synchronize()


def test_batched_verlet_reuse_matches_sorting_every_step():
    """A packed batch under Verlet reuse (domains of different dx: each particle against its
    own domain's limit; any domain past it sorts the batch) equals the batch sorting every
    step up to the order of each particle's pair sums, with fewer sorts."""
    from diffsph_gb300.solver import BatchSolver
    doms = [_drifting_fourier(nx, seed=30 + nx) for nx in (20, 33, 48)]
    a = BatchSolver([c for c, _ in doms], [s["fluid"] for _, s in doms])
    assert a.verlet_reuse
    b = BatchSolver([c for c, _ in doms], [s["fluid"] for _, s in doms])
    b.set_verlet_reuse(False)
    a.step(30)
    b.step(30)
    a.check()
    b.check()
    assert b.sort_count() == 30
    assert 2 <= a.sort_count() < 30, a.sort_count()
    ga, gb = a.download(), b.download()
    assert rel_max(_np(ga["velocities"]), _np(gb["velocities"])) < 1e-3
    assert rel_max(_np(ga["densities"]), _np(gb["densities"])) < 1e-5
    assert float((ga["positions"] - gb["positions"]).abs().max()) < 1e-5
