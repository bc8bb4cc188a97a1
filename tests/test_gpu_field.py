"""CPMG walk in an internal magnetic field (the reference's RESIDUAL_FIELD uniform / import paths)
against the CPU oracle: positions, RNG states, collision counts and final phases bit-exact (every
phase update is one fused multiply-add on both sides), echo sums within 1e-12 * n of the oracle's
FP64 sums (which carry the C library's cos), and the exact integer sums within 3 units of 2^-61 per
walker of values computed with a 256-bit cosine."""
from fractions import Fraction

import numpy as np
import pytest

from conftest import dfactor
from test_fixed_cos import exact_cos_q62
from randomwalk_nmr_gb300 import RwnmrError, host

pytestmark = pytest.mark.gpu

GAMMA = 1.0e6 * 42.576 * 2.0 * np.pi  # 1e6 * GIROMAGNETIC_RATIO with GIROMAGNETIC_UNIT: mhertz
D0, RES = 2.5, 1.0
TIME_INTERVAL = 1.0e-3 * RES * RES / (6.0 * D0)  # seconds per step
ECHO_ATOL_PER_WALKER = 1e-12


def image(shape=(24, 20, 28), seed=3, porosity=0.35, n_phases=1, rmin=2.0, rmax=5.0):
    lab, _ = host.synth_spheres(shape, rmin, rmax, porosity, n_phases, seed=seed)
    return lab


def walkers(lab, n, seed, shift=0):
    blocks, _ = host.pack_blocks(lab)
    x, y, z, s, _ = host.place_walkers(blocks, lab.shape, n, seed, "random", 0, shift)
    return x, y, z, s


def run_both(engine, oracle, lab, w, n_echoes, spe, df, gradient=2.0, direction=0, field=None, bc="noflux", shift=0,
             n_phases=None, chunk=0):
    engine.upload_labels(lab, n_phases)
    engine.upload_walkers(*w)
    dg = gradient * 1.0e-6 * RES
    if field is None:
        engine.set_field_uniform(gradient, direction, RES)
    else:
        engine.upload_field(field)
    g = engine.cpmg_field(n_echoes, spe, df, GAMMA, TIME_INTERVAL, bc=bc, shift=shift, echoes_per_launch=chunk)
    st = engine.download_walkers()
    gt = 0.5 * GAMMA * TIME_INTERVAL
    o = oracle.cpmg_field(lab, w, n_echoes, spe, df, gt, field=field, dg=dg, axis=direction, bc=bc, shift=shift,
                          n_phases=n_phases, threads=4)
    return g, st, o


def assert_parity(g, st, o, n):
    assert np.array_equal(st["x"], o["xf"])
    assert np.array_equal(st["y"], o["yf"])
    assert np.array_equal(st["z"], o["zf"])
    assert np.array_equal(st["seed"], o["seedf"])
    assert np.array_equal(st["collisions"], o["collf"])
    assert np.array_equal(g["phase"].view(np.uint64), o["phasef"].view(np.uint64))
    np.testing.assert_allclose(g["echo_sum"], o["echo_fp64"], rtol=0, atol=ECHO_ATOL_PER_WALKER * max(n, 1))


@pytest.mark.parametrize("bc", ["noflux", "periodic", "mirror"])
@pytest.mark.parametrize("shift", [0, 1])
def test_field_uniform_parity(engine, oracle, bc, shift):
    lab = image()
    w = walkers(lab, 2500, 7, shift=shift)
    g, st, o = run_both(engine, oracle, lab, w, 60, 4, dfactor(10.0), direction=shift + 1, bc=bc, shift=shift)
    assert_parity(g, st, o, len(w[0]))
    # the field dephases the walkers: the echo train falls below the pure relaxation decay
    assert g["echo_sum"][-1] < 0.99 * engine.cpmg(60, 4, dfactor(10.0), bc=bc, shift=shift)["echo_sum"][-1]


@pytest.mark.parametrize("n_phases", [2, 4])
def test_field_multiphase_parity(engine, oracle, n_phases):
    lab = image(n_phases=n_phases, seed=11)
    w = walkers(lab, 1800, 5)
    rho = [5.0, 25.0, 12.0, 40.0][:n_phases]
    g, st, o = run_both(engine, oracle, lab, w, 40, 6, dfactor(rho), direction=2, n_phases=n_phases)
    assert_parity(g, st, o, len(w[0]))
    assert np.all(st["collisions"].sum(axis=0) > 0)


def test_field_array_equals_uniform_and_imports_arbitrary_fields(engine, oracle):
    lab = image(seed=6)
    w = walkers(lab, 2000, 2)
    n = len(w[0])
    uni, st_u, _ = run_both(engine, oracle, lab, w, 50, 4, dfactor(15.0), gradient=3.0, direction=1)
    arr = oracle.uniform_field(lab, RES, 3.0, 1)
    g, st, o = run_both(engine, oracle, lab, w, 50, 4, dfactor(15.0), field=arr)
    assert np.array_equal(g["echo_sum"], uni["echo_sum"])
    assert np.array_equal(g["phase"], uni["phase"])
    assert_parity(g, st, o, n)
    # an arbitrary field, non-zero in solid voxels too (read as stored, like the reference)
    rng = np.random.default_rng(1)
    arb = rng.normal(0.0, 2e-5, lab.shape)
    g, st, o = run_both(engine, oracle, lab, w, 50, 4, dfactor(15.0), field=arb, bc="periodic")
    assert_parity(g, st, o, n)


def test_field_walkers_starting_in_solid(engine, oracle):
    """The uniform field is 0 in solid voxels; a walker placed on one sees 0 until it moves."""
    lab = image(shape=(14, 16, 18), seed=8, porosity=0.5)
    zz, yy, xx = np.nonzero(lab != 0)
    pick = np.arange(0, len(xx), max(1, len(xx) // 300))
    w = (xx[pick].astype(np.int32), yy[pick].astype(np.int32), zz[pick].astype(np.int32),
         (np.arange(len(pick), dtype=np.uint64) + np.uint64(1)) * np.uint64(0x9E3779B97F4A7C15))
    pw = walkers(lab, 300, 4)
    w = tuple(np.concatenate([a, b]) for a, b in zip(w, pw))
    g, st, o = run_both(engine, oracle, lab, w, 30, 2, dfactor(20.0), gradient=5.0, direction=0)
    assert_parity(g, st, o, len(w[0]))


def test_field_odd_steps_and_zero_field(engine, oracle):
    lab = image(seed=9)
    w = walkers(lab, 1500, 3)
    n = len(w[0])
    # odd steps per echo: each inversion takes steps_per_echo // 2 steps, as in the reference
    g, st, o = run_both(engine, oracle, lab, w, 40, 5, dfactor(8.0))
    assert_parity(g, st, o, n)
    plain = engine.cpmg(40, 4, dfactor(8.0))
    assert np.array_equal(engine.download_walkers()["seed"], st["seed"])
    # no field: phases stay zero and the echo train is the plain CPMG decay
    g0, st0, o0 = run_both(engine, oracle, lab, w, 40, 4, dfactor(8.0), gradient=0.0)
    assert np.all(g0["phase"] == 0.0)
    np.testing.assert_allclose(g0["echo_sum"], plain["echo_sum"], rtol=1e-15, atol=n * 2.0 ** -60)
    # one step per echo: no step at all
    g1, st1, _ = run_both(engine, oracle, lab, w, 10, 1, dfactor(8.0))
    assert np.array_equal(st1["x"], w[0]) and np.all(g1["echo_sum"] == n)


def test_field_chunking_determinism_and_errors(engine, oracle):
    lab = image(seed=5)
    w = walkers(lab, 1200, 1)
    engine.upload_labels(lab)
    engine.upload_walkers(*w)
    with pytest.raises(RwnmrError, match="no internal field"):
        engine.cpmg_field(10, 2, dfactor(5.0), GAMMA, TIME_INTERVAL)
    with pytest.raises(RwnmrError):
        engine.upload_field(np.zeros(7))
    with pytest.raises(RwnmrError):
        engine.set_field_uniform(1.0, 3, RES)
    engine.set_field_uniform(4.0, 2, RES)
    outs = [engine.cpmg_field(97, 2, dfactor(5.0), GAMMA, TIME_INTERVAL, echoes_per_launch=c) for c in (0, 7, 32)]
    for o in outs[1:]:
        assert np.array_equal(o["echo_sum"], outs[0]["echo_sum"])
        assert np.array_equal(o["phase"], outs[0]["phase"])
    # a new image drops the field
    engine.upload_labels(lab)
    with pytest.raises(RwnmrError, match="no internal field"):
        engine.cpmg_field(10, 2, dfactor(5.0), GAMMA, TIME_INTERVAL)


def test_field_per_walker_dfactor(engine, oracle):
    """Per-walker decrease factors in the field walk: pAlive *= f_w at every collision, as the
    reference's field kernels do with each walker's penalty."""
    lab = image(seed=14)
    w = walkers(lab, 1600, 6)
    n = len(w[0])
    rng = np.random.default_rng(3)
    f = dfactor(rng.uniform(2.0, 60.0, n))
    engine.upload_labels(lab)
    engine.upload_walkers(*w)
    engine.set_field_uniform(3.0, 0, RES)
    engine.set_walker_dfactor(f)
    g = engine.cpmg_field(45, 4, None, GAMMA, TIME_INTERVAL, bc="mirror", echoes_per_launch=8)
    st = engine.download_walkers()
    o = oracle.cpmg_field(lab, w, 45, 4, None, 0.5 * GAMMA * TIME_INTERVAL, dg=3.0 * 1.0e-6 * RES, axis=0, bc="mirror",
                          threads=4, walker_dfactor=f)
    assert_parity(g, st, o, n)
    # equal factors: the per-phase table path, bit for bit
    engine.set_walker_dfactor(np.full(n, f[0]))
    a = engine.cpmg_field(20, 2, None, GAMMA, TIME_INTERVAL)
    b = engine.cpmg_field(20, 2, f[0], GAMMA, TIME_INTERVAL)
    assert np.array_equal(a["echo_sum"], b["echo_sum"]) and np.array_equal(a["phase"], b["phase"])


def _fp64_powers(f, n):
    """f^k, k = 0..n, as the FP64 repeated product (the survival tables and the per-walker product)."""
    out = np.empty(n + 1)
    v = 1.0
    for k in range(n + 1):
        out[k] = v
        v = v * f
    return out


@pytest.mark.parametrize("bc", ["noflux", "periodic"])
@pytest.mark.parametrize("case", ["one_phase", "two_phases", "per_walker"])
def test_field_energies_within_fixed_point_bound(engine, oracle, case, bc):
    """The kernel's exact echo sums against exact values: every walker's E * 2^61 (pAlive from its
    collision counts, cos from its final phase, both downloaded) within 3 units of pAlive * cos(phase)
    * 2^61 computed with a 256-bit cosine, so the last echo's integer sum is within 3 n units. Both
    kernel families: the noflux walk on the Morton copy and the bit-block walk (periodic)."""
    n_phases = 2 if case == "two_phases" else 1
    lab = image(seed=21, n_phases=n_phases)
    w = walkers(lab, 900, 8)
    n = len(w[0])
    rho = [12.0, 40.0][:n_phases]
    engine.upload_labels(lab, n_phases)
    engine.upload_walkers(*w)
    engine.set_field_uniform(40.0, 2, RES)  # a strong gradient: phases over many radians
    if case == "per_walker":
        f = dfactor(np.random.default_rng(5).uniform(2.0, 60.0, n))
        engine.set_walker_dfactor(f)
        g = engine.cpmg_field(30, 4, None, GAMMA, TIME_INTERVAL, bc=bc)
    else:
        g = engine.cpmg_field(30, 4, dfactor(rho), GAMMA, TIME_INTERVAL, bc=bc)
    st = engine.download_walkers()
    assert engine.morton_layout
    assert g["echo_fx"][0] == n << 62  # phase 0, pAlive 1: every walker adds 2^61 + 2^61
    assert np.ptp(g["phase"]) > 10.0
    coll = st["collisions"]
    exact = Fraction(0)
    if case == "per_walker":
        for k in range(n):
            pal = Fraction(float(_fp64_powers(f[k], int(coll[k, 0]))[-1]))
            exact += pal * exact_cos_q62(float(g["phase"][k])) / 2
    else:
        tabs = [_fp64_powers(float(dfactor(r)), int(coll[:, q].max())) for q, r in enumerate(rho)]
        for k in range(n):
            pal = Fraction(1)
            for q in range(n_phases):
                pal *= Fraction(round(Fraction(float(tabs[q][coll[k, q]])) * 2 ** 63), 2 ** 63)
            exact += pal * exact_cos_q62(float(g["phase"][k])) / 2
    err = abs(Fraction(g["echo_fx"][-1] - (n << 61)) - exact)
    assert err < 3 * n, float(err / n)


@pytest.mark.parametrize("n_phases", [1, 2])
def test_field_walk_layouts_identical(engine, n_phases):
    """The uniform-field noflux walk on the image's Morton copy (gradient coordinate carried beside the
    Morton index) and on the bit blocks: positions, seeds, collisions, phases and exact sums equal,
    along every gradient axis."""
    lab = image(shape=(37, 22, 30), seed=9, n_phases=n_phases)
    w = walkers(lab, 2500, 13)
    rho = [8.0, 30.0][:n_phases]
    for axis in range(3):
        outs = []
        for morton in (True, False):
            engine.allow_morton(morton)
            engine.upload_labels(lab, n_phases)
            assert engine.morton_layout == morton
            engine.upload_walkers(*w)
            engine.set_field_uniform(15.0, axis, RES)
            g = engine.cpmg_field(40, 4, dfactor(rho), GAMMA, TIME_INTERVAL, echoes_per_launch=32)
            outs.append((g, engine.download_walkers()))
        (a, sa), (b, sb) = outs
        assert a["echo_fx"] == b["echo_fx"]
        assert np.array_equal(a["phase"].view(np.uint64), b["phase"].view(np.uint64))
        for key in ("x", "y", "z", "seed", "collisions"):
            assert np.array_equal(sa[key], sb[key])
    engine.allow_morton(True)


def test_field_huge_phases_take_the_fp64_cosine(engine, oracle):
    """Phases of 2^40 rad and more (a field far beyond any physical one) leave the fixed-point
    cosine's range; those walkers' energies take CUDA's FP64 cos, and the sums still match the
    oracle's."""
    lab = image(seed=17)
    w = walkers(lab, 1200, 3)
    n = len(w[0])
    engine.upload_labels(lab)
    engine.upload_walkers(*w)
    gradient = 1.0e15  # T/m: a move along x changes gammatau * B by ~2^43 rad
    engine.set_field_uniform(gradient, 0, RES)
    g = engine.cpmg_field(6, 2, dfactor(10.0), GAMMA, TIME_INTERVAL)
    assert np.mean(np.abs(g["phase"]) >= 2.0 ** 40) > 0.2
    st = engine.download_walkers()
    o = oracle.cpmg_field(lab, w, 6, 2, dfactor(10.0), 0.5 * GAMMA * TIME_INTERVAL, dg=gradient * 1.0e-6 * RES,
                          axis=0, threads=4)
    assert_parity(g, st, o, n)
