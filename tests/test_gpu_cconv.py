"""Learned continuous-convolution path: kernels against the CPU oracle and the trained gain.

* tcgen05 GEMM: against an FP32 matmul of the same BF16 operands, relative error <= 1e-5
  of the output's magnitude (only the FP32 summation order differs).
* aggregation: against the oracle's float64 sums of the same BF16 features; the kernel
  rounds E to BF16, so |gpu - oracle| <= 2^-8 |oracle| + 1e-5 max|oracle|.
* transposed aggregation (FP32 in and out): <= 1e-5 of the magnitude.
* layer gradients dW and dh: against the oracle's backward with the same BF16 roundings,
  relative L2 error <= 1e-4.
* gain: a network trained here (3000 Adam iterations on 8 small solver trajectories)
  predicts 4 solver steps better than the method without it (persistence, or one plain
  step of 4 dt), for the velocity and the density increments.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import cconv_oracle as CO  # noqa: E402
from diffsph_gb300 import scenes  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _lib_built():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from diffsph_gb300 import _lib
    _lib.load()


def _np(t):
    return t.detach().float().cpu().numpy()


@pytest.mark.parametrize("M,N,K", [(128, 64, 64), (256, 64, 1024), (384, 128, 4096), (128, 256, 192),
                                   (1024, 4096, 64), (4096, 64, 1024)])
def test_gemm_matches_fp32_matmul(M, N, K):
    from diffsph_gb300.learned import check_device_errors, gemm_tn
    g = torch.Generator(device="cuda").manual_seed(M + N + K)
    A = torch.randn(M, K, device="cuda", generator=g).to(torch.bfloat16)
    Bt = torch.randn(N, K, device="cuda", generator=g).to(torch.bfloat16)
    D = gemm_tn(A, Bt)
    ref = A.float() @ Bt.float().t()
    torch.cuda.synchronize()
    check_device_errors()
    err = float((D - ref).abs().max())
    assert err <= 1e-5 * float(ref.abs().max()) + 1e-6, err
    # accumulate into an existing output
    D2 = gemm_tn(A, Bt, out=D.clone(), accumulate=True)
    assert float((D2 - 2 * ref).abs().max()) <= 2e-5 * float(ref.abs().max()) + 1e-6


def test_gemm_strided_operands():
    from diffsph_gb300.learned import gemm_tn
    A_full = torch.randn(256, 192, device="cuda").to(torch.bfloat16)
    Bt_full = torch.randn(64, 256, device="cuda").to(torch.bfloat16)
    A, Bt = A_full[:, :128], Bt_full[:, 64:192]
    D = gemm_tn(A, Bt)
    ref = A.float() @ Bt.float().t()
    assert float((D - ref).abs().max()) <= 1e-5 * float(ref.abs().max())


def test_gemm_wait_timeout_sets_the_error_word_and_the_context_stays_usable():
    """Every mbarrier wait of the tensor-core GEMM is bounded. With the poll limit at 0 every
    wait fails at once (no load and no MMA is issued): the kernel sets its error bits (free
    stage 1, loaded stage 2, completion 4), releases its tensor memory and returns, and
    check_device_errors raises. The limit restored, the next GEMM in the same context is
    correct."""
    import ctypes

    from diffsph_gb300 import _lib
    from diffsph_gb300.learned import check_device_errors, gemm_tn
    lib = _lib.load()
    A = torch.randn(256, 128, device="cuda").to(torch.bfloat16)
    Bt = torch.randn(64, 128, device="cuda").to(torch.bfloat16)
    check_device_errors()
    prev = ctypes.c_uint32()
    _lib.check("sph_set_gemm_wait_limit", lib.sph_set_gemm_wait_limit(0, ctypes.byref(prev)))
    try:
        gemm_tn(A, Bt)
        torch.cuda.synchronize()
    finally:
        lib.sph_set_gemm_wait_limit(prev.value, None)
    assert prev.value > 0
    with pytest.raises(RuntimeError, match="0x7"):
        check_device_errors()
    D = gemm_tn(A, Bt)
    ref = A.float() @ Bt.float().t()
    torch.cuda.synchronize()
    check_device_errors()
    assert float((D - ref).abs().max()) <= 1e-5 * float(ref.abs().max()) + 1e-6


def test_gemm_rejects_bad_shapes():
    from diffsph_gb300 import _lib
    from diffsph_gb300.learned import gemm_tn
    A = torch.zeros(100, 64, device="cuda", dtype=torch.bfloat16)
    Bt = torch.zeros(64, 64, device="cuda", dtype=torch.bfloat16)
    with pytest.raises(_lib.SphError):
        gemm_tn(A, Bt)


def _graph_case(nx=24, seed=4, C=16):
    from diffsph_gb300.learned import Graph
    cfg, st = scenes.fourier_periodic(nx, seed=seed, jitter=0.3)
    x = torch.as_tensor(st["fluid"]["positions"], device="cuda")
    g = Graph(x, cfg)
    rng = np.random.default_rng(seed)
    h = CO.bf16(rng.standard_normal((g.n, C)).astype(np.float32))
    dom = {"min": cfg["domain"]["minExtent"], "max": cfg["domain"]["maxExtent"], "periodic": [True, True]}
    return cfg, g, h, dom


@pytest.mark.parametrize("C,rel", [(16, False), (32, False), (64, False), (16, True), (64, True)])
def test_aggregate_matches_oracle(C, rel):
    from diffsph_gb300.learned import aggregate
    cfg, g, h, dom = _graph_case(C=C)
    E = aggregate(g, torch.as_tensor(h, device="cuda").to(torch.bfloat16), rel, tensor_cores=False)
    Eo = CO.aggregate(_np(g.x), _np(g.offsets).astype(np.int64), _np(g.nbr).astype(np.int64), dom, g.H, g.inv_norm,
                      h.astype(np.float64), rel)
    Eg = _np(E[:g.n]).astype(np.float64)
    assert np.all(np.abs(Eg - Eo) <= 2.0 ** -8 * np.abs(Eo) + 1e-5 * np.abs(Eo).max())
    assert float(E[g.n:].abs().max()) == 0.0 if g.npad > g.n else True


@pytest.mark.parametrize("C,rel", [(16, False), (32, False), (64, False), (16, True), (64, True)])
def test_tensor_core_aggregate_matches_oracle(C, rel):
    """The tcgen05 aggregation against the oracle with the same BF16 operand roundings:
    only the FP32 accumulation order and the final BF16 rounding differ."""
    from diffsph_gb300.learned import aggregate, check_device_errors
    cfg, g, h, dom = _graph_case(C=C)
    E = aggregate(g, torch.as_tensor(h, device="cuda").to(torch.bfloat16), rel, tensor_cores=True)
    torch.cuda.synchronize()
    check_device_errors()
    x, off, nbr = _np(g.x), _np(g.offsets).astype(np.int64), _np(g.nbr).astype(np.int64)
    Eo = CO.aggregate(x, off, nbr, dom, g.H, g.inv_norm, h.astype(np.float64), rel, round_operands=True)
    Eg = _np(E[:g.n]).astype(np.float64)
    # the kernel rounds an fp32 basis value to bf16, the oracle an fp64 one: a term may land
    # one bf16 ulp (2^-8 relative) apart, so the bound scales with the sum of |terms|
    rows, cols, d = CO.edges(x, off, nbr, dom)
    hh = h.astype(np.float64)
    hv = np.abs(hh[cols] - hh[rows]) if rel else np.abs(hh[cols])
    S = np.zeros((g.n, 64, C))
    np.add.at(S, rows, np.abs(CO.basis(d, g.H))[:, :, None] * hv[:, None, :])
    S = S.reshape(g.n, 64 * C) * g.inv_norm
    assert np.all(np.abs(Eg - Eo) <= 2.0 ** -8 * np.abs(Eo) + 2.0 ** -7 * S + 1e-7)
    assert np.linalg.norm(Eg - Eo) <= 2e-3 * np.linalg.norm(Eo)
    # and against the exact (fp32-basis) CUDA-core kernel: BF16 basis rounding only
    Ec = _np(aggregate(g, torch.as_tensor(h, device="cuda").to(torch.bfloat16), rel, tensor_cores=False)[:g.n])
    assert np.linalg.norm(Eg - Ec) <= 5e-3 * np.linalg.norm(Ec)


@pytest.mark.parametrize("C,rel", [(16, False), (64, False), (16, True), (64, True)])
def test_aggregate_transpose_matches_oracle(C, rel):
    from diffsph_gb300.learned import aggregate_t
    cfg, g, _, dom = _graph_case(C=C)
    rng = np.random.default_rng(7)
    dE = rng.standard_normal((g.n, 64 * C)).astype(np.float32)
    dh = aggregate_t(g, torch.as_tensor(dE, device="cuda"), C, rel)
    ref = CO.aggregate_t(_np(g.x), _np(g.offsets).astype(np.int64), _np(g.nbr).astype(np.int64), dom, g.H,
                         g.inv_norm, dE.astype(np.float64), C, rel)
    assert np.max(np.abs(_np(dh) - ref)) <= 1e-5 * np.abs(ref).max()


@pytest.mark.parametrize("C,rel", [(64, False), (16, True)])
def test_layer_gradients_match_oracle(C, rel):
    from diffsph_gb300.learned import ConvFn
    cfg, g, h, dom = _graph_case(C=C, nx=20)
    rng = np.random.default_rng(3)
    W = (rng.standard_normal((64 * C, 64)) * 0.05).astype(np.float32)
    G = rng.standard_normal((g.n, 64)).astype(np.float32)
    ht = torch.as_tensor(h, device="cuda").requires_grad_(True)
    Wt = torch.as_tensor(W, device="cuda").requires_grad_(True)
    y = ConvFn.apply(ht, Wt, g, rel)
    (y * torch.as_tensor(G, device="cuda")).sum().backward()
    args = (_np(g.x), _np(g.offsets).astype(np.int64), _np(g.nbr).astype(np.int64), dom, g.H, g.inv_norm)
    yo, Eq = CO.layer_forward(*args, h, W, relative=rel)
    dho, dWo = CO.layer_backward(*args, Eq, W, G, C, relative=rel)

    def rel(a, b):
        return float(np.linalg.norm(a - b) / np.linalg.norm(b))

    # y: FP32 sums of identical BF16 products
    assert rel(_np(y), yo) < 1e-4
    assert rel(_np(Wt.grad), dWo) < 1e-4
    assert rel(_np(ht.grad), dho) < 1e-4


def test_training_data_comes_from_the_batched_solver():
    """generate_trajectories packs its trajectories into one batched solver (graph replays of
    k steps); every frame equals a single-domain solver's run of the same initial condition,
    the first bit for bit, the later ones up to the order of each particle's pair sums (under
    Verlet reuse the batch sorts when any of its domains needs it)."""
    from diffsph_gb300 import scenes
    from diffsph_gb300.learned import _wrap, generate_trajectories
    from diffsph_gb300.solver import Solver
    cfg, trajs = generate_trajectories(3, 3, 24, seed=5, k=4, chunk=2)
    rng = np.random.default_rng(5)
    assert len(trajs) == 3 and all(len(t) == 3 for t in trajs)
    for t in range(3):
        c, st = scenes.fourier_periodic(24, seed=int(rng.integers(0, 2 ** 31 - 1)), jitter=0.1)
        sol = Solver(c, st["fluid"])
        for f in range(3):
            got = sol.download()
            x, u, r = _wrap(got["positions"], c), got["velocities"], got["densities"]
            if f == 0:
                assert torch.equal(x, trajs[t][f][0]) and torch.equal(u, trajs[t][f][1]), t
                assert torch.equal(r, trajs[t][f][2]), t
            else:
                # (wrapped positions: a particle on the wrap may land on either side)
                dxw = (x - trajs[t][f][0]).abs()
                dxw = torch.minimum(dxw, 2.0 - dxw)
                assert float(dxw.max()) < 1e-5, (t, f)
                assert float((u - trajs[t][f][1]).abs().max()) < 1e-4 * float(u.abs().max()), (t, f)
                assert float((r - trajs[t][f][2]).abs().max()) < 1e-5, (t, f)
            sol.step(4)


def test_trained_network_beats_the_method_without_it():
    """Trains on 8 solver trajectories of 32^2-particle periodic Fourier flows (24 frames,
    one every 4 steps) and evaluates on a held-out trajectory: the learned 4-step update
    must be closer to the solver's 4 steps than persistence (u, rho unchanged) and than one
    plain step of 4 dt (the solver taking the learned step's time step directly)."""
    import copy

    from diffsph_gb300.learned import (CConvNet, LearnedStepper, check_device_errors, generate_trajectories,
                                       train)
    from diffsph_gb300.solver import Solver
    k = 4
    cfg, trajs = generate_trajectories(9, 24, 32, seed=11, k=k)
    train_set, held = trajs[:8], trajs[8]
    torch.manual_seed(0)
    net = CConvNet().cuda()
    hist = train(net, cfg, train_set, iters=3000, k=k, lr=5e-3)
    check_device_errors()
    assert np.mean(hist[-50:]) < 0.5 * np.mean(hist[:50])
    stepper = LearnedStepper(cfg, net, k)
    cfg4 = copy.deepcopy(cfg)
    cfg4["timestep"]["dt"] = k * float(cfg["timestep"]["dt"])
    e_net, e_pers, e_big, e_rho = [], [], [], []
    for i in range(len(held) - 1):
        a, b = held[i], held[i + 1]
        with torch.no_grad():
            _, u_net, r_net = stepper.step(*a)
        e_rho.append(float(torch.linalg.norm(r_net - b[2]) / torch.linalg.norm(b[2] - a[2])))
        sol = Solver(cfg4, {"positions": a[0], "velocities": a[1], "densities": a[2],
                            "masses": np.full(a[0].shape[0], float(cfg["particle"]["dx"]) ** 2),
                            "supports": np.full(a[0].shape[0], float(cfg["particle"]["support"]))})
        sol.step(1)
        big = sol.download()
        du = b[1] - a[1]
        scale = float(torch.linalg.norm(du))
        e_net.append(float(torch.linalg.norm(u_net - b[1])) / scale)
        e_pers.append(float(torch.linalg.norm(a[1] - b[1])) / scale)
        e_big.append(float(torch.linalg.norm(big["velocities"] - b[1])) / scale)
    m_net, m_pers, m_big = np.mean(e_net), np.mean(e_pers), np.mean(e_big)
    print(f"relative velocity-increment error: learned {m_net:.3f}, persistence {m_pers:.3f}, "
          f"one 4dt step {m_big:.3f}; density increment: learned {np.mean(e_rho):.3f}, persistence 1")
    assert m_net < m_pers
    assert m_net < m_big
    assert np.mean(e_rho) < 0.5


@pytest.mark.parametrize("bad", ["density", "velocity"])
def test_judge_rejects_a_bad_network_and_falls_back_to_the_solver(bad):
    """A network whose output is biased breaks the density bound (+0.05 rho0 per learned
    step) or the kinetic-energy bound (+0.2 on every velocity): every segment is rejected
    and re-run by the solver, so the rollout equals the plain solver's (up to the summation
    order of the re-sorted restarts)."""
    from diffsph_gb300.learned import CConvNet, LearnedStepper, judged_rollout
    from diffsph_gb300.solver import Solver
    cfg, st = scenes.fourier_periodic(32, seed=21, jitter=0.1)
    net = CConvNet(seed=5).cuda()
    with torch.no_grad():
        net.dec2.weight.zero_()
        if bad == "density":
            net.dec2.bias[2] = 0.05
        else:
            net.dec2.bias[0:2] = 0.2
    stepper = LearnedStepper(cfg, net, 4)
    (x, u, r), acc, rej = judged_rollout(stepper, st["fluid"], 6, segment=2)
    assert acc == 0 and rej == 3
    sol = Solver(cfg, st["fluid"])
    sol.step(24)
    ref = sol.download()
    assert float(torch.linalg.norm(u - ref["velocities"]) / torch.linalg.norm(ref["velocities"])) < 1e-5
    assert float(torch.max(torch.abs(r - ref["densities"]))) < 1e-5


@pytest.mark.parametrize("n_domains", [1, 3])
def test_graph_lists_equal_the_exact_neighbor_sets(n_domains):
    """The CSR-only fill (cell order) holds exactly the pairs of the reference-format
    search (sorted rows), domain by domain, with global indices for packed domains."""
    from diffsph_gb300.learned import Graph
    from diffsph_gb300.neighborhood import exact_pairs
    doms = [scenes.fourier_periodic(24, seed=30 + d, jitter=0.3) for d in range(n_domains)]
    cfg = doms[0][0]
    x = torch.cat([torch.as_tensor(st["fluid"]["positions"]) for _, st in doms]).cuda()
    g = Graph(x, cfg, n_domains)
    per = x.shape[0] // n_domains
    off = _np(g.offsets).astype(np.int64)
    nbr = g.nbr.cpu().numpy().astype(np.int64)
    for d in range(n_domains):
        xd = x[d * per:(d + 1) * per]
        _, j, _, _, _, _, _, _, o = exact_pairs(xd, xd, torch.full((per,), g.H, device="cuda"), cfg,
                                                compute_kernels=False)
        j, o = j.cpu().numpy(), o.cpu().numpy()
        for i in range(per):
            row = np.sort(nbr[off[d * per + i]:off[d * per + i + 1]]) - d * per
            assert np.array_equal(row, j[o[i]:o[i + 1]]), (d, i)


def test_row_over_the_aggregation_capacity_is_flagged_and_taken():
    """A particle with more than 64 neighbors within the learned support (a cluster the
    learned steps can bring about) is truncated to its first 64 edges by the tensor-core
    aggregation, which sets the row-capacity flag: take_row_overflow reports it once and
    clears it (a judged rollout then rejects the segment), and no other flag is left."""
    from diffsph_gb300.learned import Graph, aggregate, check_device_errors, take_row_overflow
    cfg, st = scenes.fourier_periodic(32, seed=3, jitter=0.0)
    x = torch.as_tensor(st["fluid"]["positions"]).clone()
    H = float(cfg["particle"]["support"])
    gen = torch.Generator().manual_seed(0)
    x[:80] = torch.tensor([0.1, 0.2]) + 0.05 * H * torch.rand(80, 2, generator=gen)
    g = Graph(x.cuda(), cfg)
    assert int((g.offsets[1:] - g.offsets[:-1]).max()) > 64
    h = torch.randn(g.n, 16, device="cuda").to(torch.bfloat16)
    assert not take_row_overflow()
    aggregate(g, h)
    assert take_row_overflow()
    assert not take_row_overflow()
    check_device_errors()
