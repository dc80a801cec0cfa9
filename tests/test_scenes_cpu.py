"""The seeded scene generators: the Fourier-mode initial field of the batched, adjoint and
learned workloads (a stream function of 16 random modes with |k| <= 4, amplitudes |k|^-2,
uniform phases, normalised to a maximum speed of 1)."""
import numpy as np

from diffsph_gb300 import scenes


def _grid(n, L=2.0):
    g = (np.arange(n) + 0.5) * (L / n) - L / 2
    X, Y = np.meshgrid(g, g, indexing="ij")
    return np.stack([X.ravel(), Y.ravel()], -1)


def test_modes_are_distinct_up_to_sign():
    for seed in range(20):
        k, ph = scenes.fourier_modes(np.random.default_rng(seed))
        assert k.shape == (16, 2) and ph.shape == (16,)
        norms = np.hypot(k[:, 0], k[:, 1])
        assert np.all((norms > 0) & (norms <= 4))
        keys = {tuple(v) for v in k} | {tuple(-v) for v in k}
        assert len(keys) == 32  # no repeat, no pair k, -k
        assert np.all((ph >= 0) & (ph < 2 * np.pi))


def test_field_is_divergence_free_spectrally():
    """Sampled on a periodic 32 x 32 grid (above twice the largest wavenumber), the field's
    discrete Fourier transform has k . u_hat = 0 to rounding at every wave vector."""
    n, L = 32, 2.0
    x = _grid(n, L)
    u = scenes.fourier_velocity(x, np.random.default_rng(3), L=L)
    uh = [np.fft.fft2(u[:, a].reshape(n, n)) for a in range(2)]
    kk = np.fft.fftfreq(n, d=L / n) * 2 * np.pi
    KX, KY = np.meshgrid(kk, kk, indexing="ij")
    div = KX * uh[0] + KY * uh[1]
    scale = np.max(np.hypot(KX, KY) * np.hypot(np.abs(uh[0]), np.abs(uh[1])))
    assert np.max(np.abs(div)) <= 1e-12 * scale


def test_spectrum_follows_k_to_the_minus_two():
    """The stream function's amplitude |psi_hat(k)| = |u_hat(k)| / |k| times |k|^2 is the same
    for every drawn mode, and the field holds no other mode."""
    n, L = 32, 2.0
    rng = np.random.default_rng(5)
    x = _grid(n, L)
    k_int, _ = scenes.fourier_modes(np.random.default_rng(5))
    u = scenes.fourier_velocity(x, rng, L=L)
    uh = [np.fft.fft2(u[:, a].reshape(n, n)) for a in range(2)]
    mag = np.hypot(np.abs(uh[0]), np.abs(uh[1]))
    vals = []
    for kx, ky in k_int:
        k2 = (2 * np.pi / L) ** 2 * (kx * kx + ky * ky)
        vals.append(mag[kx % n, ky % n] / np.sqrt(k2) * k2)
    vals = np.asarray(vals)
    assert np.max(np.abs(vals - vals.mean())) <= 1e-9 * vals.mean()
    active = np.zeros((n, n), bool)
    for kx, ky in k_int:
        active[kx % n, ky % n] = active[-kx % n, -ky % n] = True
    assert np.max(mag[~active]) <= 1e-9 * np.max(mag)


def test_seed_reproduces_the_field_and_max_speed_is_one():
    a = scenes.fourier_periodic(24, seed=11, jitter=0.1)[1]["fluid"]
    b = scenes.fourier_periodic(24, seed=11, jitter=0.1)[1]["fluid"]
    c = scenes.fourier_periodic(24, seed=12, jitter=0.1)[1]["fluid"]
    for key in ("positions", "velocities", "densities"):
        assert np.array_equal(a[key], b[key])
    assert not np.array_equal(a["velocities"], c["velocities"])
    assert abs(float(np.max(np.linalg.norm(a["velocities"].astype(np.float64), axis=1))) - 1.0) < 1e-6


def test_batched_counts_are_log_uniform_squares_in_range():
    doms = scenes.batched_fourier(64, seed=0, n_min=1024, n_max=65536)
    counts = np.asarray([s["fluid"]["positions"].shape[0] for _, s in doms])
    roots = np.sqrt(counts)
    assert np.all(roots == np.round(roots))
    assert counts.min() >= 900 and counts.max() <= 66000
    # log-uniform: the median near the geometric mean of the range
    assert 0.5 < np.median(counts) / np.sqrt(1024 * 65536) < 2.0
