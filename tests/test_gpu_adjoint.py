"""The seed-replay adjoint kernel against (1) an FP64 CPU pathwise gradient built from the
oracle's per-walker collision histories and (2) central finite differences under common random
numbers (same seeds, so the trajectories are fixed and the echo train is smooth in f)."""
import numpy as np
import pytest

from conftest import dfactor
from randomwalk_nmr_gb300 import host

pytestmark = pytest.mark.gpu


def setup(engine, n_phases, seed=12, n=3000, morton=True):
    lab, _ = host.synth_spheres((24, 28, 22), 2.0, 5.0, 0.4, n_phases, seed=seed)
    blocks, _ = host.pack_blocks(lab)
    x, y, z, s, _ = host.place_walkers(blocks, lab.shape, n, seed)
    engine.allow_morton(morton)
    engine.upload_labels(lab, n_phases)
    engine.upload_walkers(x, y, z, s)
    return lab, (x, y, z, s)


def pathwise_gradient(oracle, lab, w, n_echoes, spe, f, grad, n_phases):
    """sum_e g_e sum_w dE_w(e)/df_q from per-walker, per-echo collision counts (CPU, FP64)."""
    f = np.asarray(f, np.float64)
    P = n_phases
    counts = np.zeros((n_echoes + 1, len(w[0]), P), np.int64)
    state = [np.array(a) for a in w]
    for e in range(n_echoes):
        o = oracle.cpmg(lab, tuple(state), 1, spe, f, n_phases=n_phases, threads=4)
        counts[e + 1] = counts[e] + o["collf"].astype(np.int64)
        state = [o["xf"], o["yf"], o["zf"], o["seedf"]]
    out = np.zeros(P)
    for q in range(P):
        c = counts[..., q].astype(np.float64)
        dq = np.where(c > 0, c * f[q] ** np.maximum(c - 1, 0), 0.0)
        other = np.ones_like(c)
        for r in range(P):
            if r != q:
                other *= f[r] ** counts[..., r]
        out[q] = np.sum(grad[:, None] * dq * other)
    return out


@pytest.mark.parametrize("n_phases,morton", [(1, True), (2, True), (2, False)])
def test_adjoint_matches_pathwise_and_finite_differences(engine, oracle, n_phases, morton):
    lab, w = setup(engine, n_phases, morton=morton)
    n_echoes, spe = 60, 2
    f = dfactor([10.0, 30.0][:n_phases])
    rng = np.random.default_rng(0)
    grad = rng.normal(size=n_echoes + 1)
    adj = engine.cpmg_adjoint(n_echoes, spe, f, grad)
    ref = pathwise_gradient(oracle, lab, w, n_echoes, spe, f, grad, n_phases)
    np.testing.assert_allclose(adj, ref, rtol=1e-10)
    h = 1e-6
    for q in range(n_phases):
        fp, fm = f.copy(), f.copy()
        fp[q] += h
        fm[q] -= h
        Lp = grad @ engine.cpmg(n_echoes, spe, fp)["echo_sum"]
        Lm = grad @ engine.cpmg(n_echoes, spe, fm)["echo_sum"]
        np.testing.assert_allclose(adj[q], (Lp - Lm) / (2 * h), rtol=1e-5)


def test_adjoint_zero_gradient_is_zero(engine):
    setup(engine, 1)
    adj = engine.cpmg_adjoint(20, 1, dfactor(10.0), np.zeros(21))
    assert np.all(adj == 0.0)


@pytest.mark.parametrize("f", [[0.0, 0.97], [0.55, 0.0, 0.9, 0.999]])
def test_adjoint_with_a_zero_decrease_factor(engine, oracle, f):
    """With every f_q > 0 the kernel sums g E c_q and divides by f_q; a zero factor takes the
    direct derivative (c_q f_q^(c_q - 1) is 1 at c_q = 1 while E is 0). Both against the pathwise
    gradient."""
    n_phases = len(f)
    lab, w = setup(engine, n_phases, seed=5, n=1500)
    n_echoes, spe = 25, 2
    rng = np.random.default_rng(2)
    grad = rng.normal(size=n_echoes + 1)
    ref = pathwise_gradient(oracle, lab, w, n_echoes, spe, f, grad, n_phases)
    adj = engine.cpmg_adjoint(n_echoes, spe, np.array(f), grad)
    np.testing.assert_allclose(adj, ref, rtol=1e-10, atol=1e-12 * np.max(np.abs(ref)))
    g2 = engine.cpmg_adjoint(n_echoes, spe, np.array([v if v > 0 else 0.5 for v in f]), grad)
    ref2 = pathwise_gradient(oracle, lab, w, n_echoes, spe, [v if v > 0 else 0.5 for v in f], grad, n_phases)
    np.testing.assert_allclose(g2, ref2, rtol=1e-10, atol=1e-12 * np.max(np.abs(ref2)))


def _tables_fx(f, kmax):
    """round(f^k * 2^63), f^k the FP64 repeated product: the engine's fixed-point survival tables."""
    from fractions import Fraction
    out, v = [], 1.0
    for _ in range(kmax + 1):
        out.append(round(Fraction(v) * 2 ** 63))
        v = v * f
    return out


def _fx_mul(a, b):
    return b if a >> 63 else ((a << 1) * b) >> 64


def _collision_histories(oracle, lab, w, n_echoes, spe, f, n_phases, bc):
    """Per-walker collision counts after every echo [n_echoes+1][n][phases], from the oracle."""
    counts = np.zeros((n_echoes + 1, len(w[0]), n_phases), np.int64)
    state = [np.array(a) for a in w]
    for e in range(n_echoes):
        o = oracle.cpmg(lab, tuple(state), 1, spe, f, n_phases=n_phases, bc=bc, threads=4)
        counts[e + 1] = counts[e] + o["collf"].astype(np.int64)
        state = [o["xf"], o["yf"], o["zf"], o["seedf"]]
    return counts


@pytest.mark.parametrize("n_phases,morton,bc,spe", [(1, True, "noflux", 3), (2, True, "noflux", 3),
                                                    (4, True, "noflux", 3), (3, True, "noflux", 1),
                                                    (4, True, "noflux", 2), (2, True, "noflux", 1),
                                                    (2, False, "noflux", 3), (3, False, "periodic", 3),
                                                    (1, False, "mirror", 3)])
def test_sensitivities_exact(engine, oracle, n_phases, morton, bc, spe):
    """rwnmr_cpmg_run_sens: the same echo train as rwnmr_cpmg_run, and per-echo sums of E * c_q that
    equal, exactly, the sums formed from the oracle's per-walker collision histories and the engine's
    fixed-point tables; their gradient equals the seed-replay adjoint's. The Morton walk replays each
    window's collisions (1, 2 or 3 steps per echo; launches of 32 echoes split the windows)."""
    lab, w = setup(engine, n_phases, n=1500, morton=morton)
    assert engine.morton_layout == morton
    n_echoes = 40
    f = dfactor([10.0, 30.0, 5.0, 60.0][:n_phases])
    out = engine.cpmg_sens(n_echoes, spe, f, bc=bc, echoes_per_launch=32)
    plain = engine.cpmg(n_echoes, spe, f, bc=bc)
    assert np.array_equal(out["echo_sum"], plain["echo_sum"])
    counts = _collision_histories(oracle, lab, w, n_echoes, spe, f, n_phases, bc)
    tabs = [_tables_fx(f[q], int(counts[..., q].max())) for q in range(n_phases)]
    for e in range(n_echoes + 1):
        ce = counts[e]
        efx = []
        for k in range(len(ce)):
            v = tabs[0][ce[k, 0]]
            for q in range(1, n_phases):
                v = _fx_mul(v, tabs[q][ce[k, q]])
            efx.append(v)
        for q in range(n_phases):
            assert out["sens_fx"][e][q] == sum(v * int(c) for v, c in zip(efx, ce[:, q])), (e, q)
    rng = np.random.default_rng(1)
    grad = rng.normal(size=n_echoes + 1)
    np.testing.assert_allclose(grad @ out["sens"] / f, engine.cpmg_adjoint(n_echoes, spe, f, grad, bc=bc), rtol=1e-11)


def test_sensitivities_need_per_phase_factors(engine):
    setup(engine, 1, n=200)
    engine.set_walker_dfactor(np.full(engine.n, 0.99))
    with pytest.raises(Exception, match="per-phase decrease factors"):
        engine.cpmg_sens(5, 2, None)


@pytest.mark.parametrize("f", [[0.995, 0.98], [0.0, 0.98]])
def test_adjoint_leaves_the_walkers(engine, f):
    """Both adjoint paths (the integer sensitivity walk on scratch state, and the FP64 replay for a
    zero factor) leave the context's walker state as the last walk left it."""
    setup(engine, 2, n=500)
    engine.cpmg(20, 2, [0.99, 0.97])
    before = engine.download_walkers()
    engine.cpmg_adjoint(35, 3, np.asarray(f), np.ones(36))
    after = engine.download_walkers()
    for key in before:
        assert np.array_equal(before[key], after[key])
