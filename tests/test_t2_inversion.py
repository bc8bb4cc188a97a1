"""T2 (inverse Laplace) inversion of CPMG decays on the host, against the oracle's numpy restatement
of the reference's NMRInverter (L-curve on numpy's SVD), scipy's NNLS, and decays built from known
T2 distributions. CPU only."""
import numpy as np
import pytest

from oracle import laplace as L
from randomwalk_nmr_gb300 import host

DECAYS = [(0.2, 15000), (0.2, 2000), (0.1, 20000), (1.0, 600), (0.2, 1000)]


def bimodal(te, n, w=(0.6, 0.4), t2=(20.0, 300.0)):
    t = np.arange(n + 1) * te
    return t, w[0] * np.exp(-t / t2[0]) + w[1] * np.exp(-t / t2[1])


def assert_same_lcurve_choice(lam, r):
    """lam is the oracle's L-curve choice or a grid neighbour whose curvature is within 1 % of the
    maximum. With noisy data the residual norm takes the data's projections on singular directions
    near eps * s_max, which rounding fixes differently in every SVD (the reference's Eigen
    JacobiSVD included), so the curvature agrees to ~1e-3 and its flat maximum can move a step."""
    k = int(np.argmin(np.abs(r["lambdas"] - lam)))
    assert r["lambdas"][k] == lam and abs(k - r["best"]) <= 2
    c = r["curvature"]
    assert c[k] >= c[r["best"]] - 1e-2 * abs(c[r["best"]])


def test_t2_bins_match_reference_accumulation():
    for lo, hi, n in [(0.1, 1e4, 128), (0.5, 2000.0, 64), (1.0, 10.0, 7)]:
        b, _, _, _ = host.invert_t2(*bimodal(0.2, 300), min_t2=lo, max_t2=hi, num_t2_bins=n)
        assert np.array_equal(b, L.t2_bins(lo, hi, n))
    b, _, _, _ = host.invert_t2(*bimodal(0.2, 300), min_t2=1.0, max_t2=500.0, num_t2_bins=32, use_logspace=False)
    assert np.array_equal(b, L.t2_bins(1.0, 500.0, 32, use_log=False))


@pytest.mark.parametrize("te,n", DECAYS)
def test_prune_averaging_is_bit_identical(te, n):
    t, a = bimodal(te, n)
    t, a = t[1:], a[1:]
    got = host.prune_decay(t, a, 512)
    sl = L.pruning_slices(t, 512)
    assert got is not None and sl is not None
    assert np.array_equal(got[0], L.prune(t, sl, 512, True))
    assert np.array_equal(got[1], L.prune(a, sl, 512, False))
    # the leading points are copied and the last one kept; the first averaged slice starts a few
    # points before the copied prefix ends (the reference's grid search), so times dip once there
    ps = sl[0][0]
    assert np.array_equal(got[0][:ps], t[:ps]) and got[0][-1] == t[-1] and got[1][-1] == a[-1]
    assert np.sum(np.diff(got[0]) <= 0) <= 1


def test_short_decays_are_not_pruned():
    t, a = bimodal(0.2, 512)
    assert host.prune_decay(t[1:], a[1:], 512) is None and L.pruning_slices(t[1:], 512) is None
    assert host.prune_decay(t[1:], a[1:], 0) is None


@pytest.mark.parametrize("te,n,prune", [(0.2, 15000, 512), (0.2, 2000, 512), (0.2, 60, 512), (0.5, 400, 0)])
def test_lcurve_matches_svd_restatement(te, n, prune):
    t, a = bimodal(te, n)
    t, a = t[1:], a[1:]
    if prune and len(t) > prune:
        sl = L.pruning_slices(t, prune)
        t, a = L.prune(t, sl, prune, True), L.prune(a, sl, prune, False)
    A = L.kernel(t, L.t2_bins(0.1, 1e4, 128))
    best, curv, sv = host.lcurve(A, a)
    ob, _, ocurv, _, _, osv = L.lcurve(A, a, -4.0, 2.0, 512)
    assert best == ob
    np.testing.assert_allclose(curv, ocurv, rtol=0, atol=1e-9 * np.max(np.abs(ocurv)))
    big = osv > 1e-8 * osv[0]
    assert len(sv) == min(A.shape)
    # LAPACK's singular values carry absolute errors of order eps * s_max
    np.testing.assert_allclose(sv[big], osv[big], rtol=1e-12, atol=1e-13 * osv[0])


def test_nnls_matches_scipy_and_oracle():
    scipy_opt = pytest.importorskip("scipy.optimize")
    rng = np.random.default_rng(3)
    for m, n in [(40, 12), (200, 64), (30, 30), (8, 20)]:
        A = rng.normal(size=(m, n))
        b = rng.normal(size=m)
        x, solves = host.nnls(A, b)
        xs, _ = scipy_opt.nnls(A, b, maxiter=50 * n)
        assert np.all(x >= 0) and solves > 0
        if m >= n:  # unique minimiser
            np.testing.assert_allclose(x, xs, rtol=0, atol=1e-10 * max(1.0, np.max(np.abs(xs))))
            np.testing.assert_allclose(x, L.nnls(A, b), rtol=0, atol=1e-10 * max(1.0, np.max(np.abs(xs))))
        r, rs = np.linalg.norm(A @ x - b), np.linalg.norm(A @ xs - b)
        assert r <= rs * (1 + 1e-10) + 1e-12
    # a Tikhonov-augmented exponential kernel, the inversion's own system
    t, a = bimodal(0.2, 2000)
    A = L.kernel(t[1:], L.t2_bins(0.1, 1e4, 128))
    Aa = np.vstack([A, 0.05 * np.eye(128)])
    ba = np.concatenate([a[1:], np.zeros(128)])
    x, _ = host.nnls(Aa, ba)
    xs, _ = scipy_opt.nnls(Aa, ba, maxiter=10000)
    np.testing.assert_allclose(x, xs, rtol=0, atol=1e-10 * np.max(xs))


@pytest.mark.parametrize("te,n,prune", [(0.2, 15000, 512), (0.2, 2000, 512), (0.2, 60, 512), (1.0, 600, 0)])
def test_inversion_matches_oracle(te, n, prune):
    t, a = bimodal(te, n)
    bins, x, lam, noise = host.invert_t2(t, a, prune_num=prune)
    r = L.invert(t, a, prune_num=prune)
    assert np.array_equal(bins, r["bins"]) and lam == r["lam"]
    np.testing.assert_allclose(x, r["amps"], rtol=0, atol=1e-9 * np.max(r["amps"]))
    assert np.all(x >= 0) and not np.any(noise)


def test_recovers_known_distribution():
    """Decay from a log-normal T2 distribution on the inversion's own bins, observed until it has
    died out: the recovered distribution reproduces the decay and its log-mean T2. (With a window
    shorter than the slowest T2 the L-curve criterion can pick a large lambda; that is the
    criterion's behaviour, kept as in the reference.)"""
    bins = L.t2_bins(0.1, 1e4, 128)
    lb = np.log10(bins)
    for centre in (1.0, 1.8, 2.6):
        w = np.exp(-0.5 * ((lb - centre) / 0.15) ** 2)
        w /= w.sum()
        t = np.arange(6001) * 1.0
        a = np.exp(-t[:, None] / bins[None, :]) @ w
        _, x, _, _ = host.invert_t2(t, a)
        assert abs(np.sum(x * lb) / np.sum(x) - centre) < 0.02 and abs(x.sum() - 1.0) < 1e-3
        fit = np.exp(-t[1:, None] / bins[None, :]) @ x
        assert np.max(np.abs(fit - a[1:])) < 1e-4


def test_noise_is_seeded_and_inverted_with_the_decay():
    t, a = bimodal(0.2, 3000)
    b1, x1, l1, n1 = host.invert_t2(t, a, noise_amp=0.01, noise_seed=9)
    b2, x2, l2, n2 = host.invert_t2(t, a, noise_amp=0.01, noise_seed=9)
    assert np.array_equal(x1, x2) and np.array_equal(n1, n2) and l1 == l2
    assert n1[0] == 0.0 and abs(np.std(n1[1:]) - 0.01) < 1e-3
    r = L.invert(t, a, noise=n1[1:])
    assert_same_lcurve_choice(l1, r)
    r = L.invert(t, a, noise=n1[1:], force_lambda=l1)
    np.testing.assert_allclose(x1, r["amps"], rtol=0, atol=1e-9 * np.max(r["amps"]))
    _, x3, _, n3 = host.invert_t2(t, a, noise_amp=0.01, noise_seed=10)
    assert not np.array_equal(n1, n3)


def test_bad_inputs_are_rejected():
    t, a = bimodal(0.2, 100)
    with pytest.raises(ValueError):
        host.invert_t2(t[:2], a[:2])
    with pytest.raises(ValueError):
        host.invert_t2(t, a, min_t2=0.0)
    with pytest.raises(ValueError):
        host.invert_t2(t, a[:-1])
    with pytest.raises(ValueError):
        host.invert_t2(t, a, num_t2_bins=0)
