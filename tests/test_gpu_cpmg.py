"""GPU parity of the CPMG / mapping walk against the CPU oracle (bit-exact integers, exact
fixed-point echo sums, FP64 echo sums within 1e-12 relative of the oracle's serial FP64 sum)."""
import numpy as np
import pytest

from conftest import dfactor
from randomwalk_nmr_gb300 import Engine, fx_to_float, host

pytestmark = pytest.mark.gpu

# echo amplitudes: GPU fixed-point sum vs the oracle's serial FP64 sum of the same energies
ECHO_RTOL = 1e-12


def image(shape=(26, 22, 30), seed=3, porosity=0.35, n_phases=1, rmin=2.0, rmax=6.0):
    lab, _ = host.synth_spheres(shape, rmin, rmax, porosity, n_phases, seed=seed)
    return lab


def walkers(lab, n, seed, shift=0, mode="random", dev=0):
    blocks, _ = host.pack_blocks(lab)
    x, y, z, s, info = host.place_walkers(blocks, lab.shape, n, seed, mode, dev, shift)
    return x, y, z, s


def run_both(engine, oracle, lab, w, n_echoes, spe, df, bc="noflux", shift=0, n_phases=None, chunk=0):
    engine.upload_labels(lab, n_phases)
    engine.upload_walkers(*w)
    g = engine.cpmg(n_echoes, spe, df, bc=bc, shift=shift, echoes_per_launch=chunk)
    st = engine.download_walkers()
    o = oracle.cpmg(lab, w, n_echoes, spe, df, bc=bc, shift=shift, n_phases=n_phases, threads=4)
    return g, st, o


def assert_parity(g, st, o):
    assert np.array_equal(st["x"], o["xf"])
    assert np.array_equal(st["y"], o["yf"])
    assert np.array_equal(st["z"], o["zf"])
    assert np.array_equal(st["seed"], o["seedf"])
    assert np.array_equal(st["collisions"], o["collf"])
    assert np.array_equal(g["echo_coll"], o["echo_coll"])
    assert np.array_equal(g["echo_fx"], o["echo_fx"])
    np.testing.assert_allclose(g["echo_sum"], o["echo_fp64"], rtol=ECHO_RTOL, atol=0)
    np.testing.assert_allclose(g["echo_sum"], fx_to_float(g["echo_fx"]), rtol=1e-15)


@pytest.mark.parametrize("bc", ["noflux", "periodic", "mirror"])
@pytest.mark.parametrize("shift", [0, 1])
def test_cpmg_parity_bc_shift(engine, oracle, bc, shift):
    lab = image()
    w = walkers(lab, 3000, 7, shift=shift)
    g, st, o = run_both(engine, oracle, lab, w, 150, 2, dfactor(10.0), bc=bc, shift=shift)
    assert_parity(g, st, o)


@pytest.mark.parametrize("n_phases", [2, 3, 4])
def test_cpmg_parity_multiphase(engine, oracle, n_phases):
    lab = image(n_phases=n_phases, seed=11)
    w = walkers(lab, 2000, 5)
    rho = [5.0, 25.0, 12.0, 40.0][:n_phases]
    g, st, o = run_both(engine, oracle, lab, w, 120, 3, dfactor(rho), n_phases=n_phases)
    assert_parity(g, st, o)
    assert np.all(g["echo_coll"].sum(axis=0) > 0)


@pytest.mark.parametrize("spe", [2047, 2048, 3001])
def test_cpmg_two_phase_long_echoes(engine, oracle, spe):
    """Two phases count collisions in 16-bit halves of one word up to 2047 steps per echo and in
    separate words beyond; both sides of the switch agree with the oracle."""
    lab = image(shape=(20, 18, 22), n_phases=2, seed=13, rmin=1.5, rmax=3.0)
    w = walkers(lab, 700, 9)
    g, st, o = run_both(engine, oracle, lab, w, 4, spe, dfactor([3.0, 8.0]), n_phases=2)
    assert_parity(g, st, o)
    assert g["echo_coll"].max() > 32 * 256  # warp-wide sums well past 8 bits per phase


def test_cpmg_parity_reference_golden(engine, golden):
    """Against the reference's own per-echo walk outputs."""
    gd = golden
    lab = gd["img_a"]
    w = (gd["walk_x0"], gd["walk_y0"], gd["walk_z0"], gd["walk_seed0"])
    engine.upload_labels(lab)
    engine.upload_walkers(*w)
    g = engine.cpmg(200, 2, float(gd["walk_dfactor"][0]))
    st = engine.download_walkers()
    assert np.array_equal(st["x"], gd["walk_xf"])
    assert np.array_equal(st["y"], gd["walk_yf"])
    assert np.array_equal(st["z"], gd["walk_zf"])
    assert np.array_equal(st["seed"], gd["walk_seedf"])
    assert np.array_equal(st["collisions"][:, 0], gd["walk_coll"])
    assert np.array_equal(g["echo_coll"][:, 0], gd["walk_coll_per_echo"])
    np.testing.assert_allclose(g["echo_sum"], gd["walk_energy_sum"], rtol=ECHO_RTOL)


def test_cpmg_launch_chunking_is_invisible(engine, oracle):
    lab = image(seed=5)
    w = walkers(lab, 1500, 3)
    outs = []
    for chunk in (0, 7, 32, 500):
        engine.upload_labels(lab)
        engine.upload_walkers(*w)
        outs.append(engine.cpmg(257, 1, dfactor(30.0), echoes_per_launch=chunk))
    for o in outs[1:]:
        assert np.array_equal(o["echo_fx"], outs[0]["echo_fx"])
        assert np.array_equal(o["echo_coll"], outs[0]["echo_coll"])


def test_cpmg_deterministic_and_rerunnable(engine):
    lab = image(seed=9)
    w = walkers(lab, 4000, 1)
    engine.upload_labels(lab)
    engine.upload_walkers(*w)
    a = engine.cpmg(100, 2, dfactor(10.0))
    b = engine.cpmg(100, 2, dfactor(10.0))
    assert np.array_equal(a["echo_fx"], b["echo_fx"])
    assert np.array_equal(a["echo_sum"], b["echo_sum"])


def test_cpmg_edge_cases(engine, oracle):
    lab = image(shape=(5, 7, 9), seed=2, porosity=0.6, rmin=1.0, rmax=2.0)
    # walkers on every face of the image
    zz, yy, xx = np.nonzero(lab == 0)
    on_face = (xx == 0) | (yy == 0) | (zz == 0) | (xx == 8) | (yy == 6) | (zz == 4)
    idx = np.nonzero(on_face)[0]
    w = (xx[idx].astype(np.int32), yy[idx].astype(np.int32), zz[idx].astype(np.int32),
         np.arange(1, len(idx) + 1, dtype=np.uint64) * np.uint64(0x9E3779B97F4A7C15))
    for bc in ("noflux", "periodic", "mirror"):
        g, st, o = run_both(engine, oracle, lab, w, 64, 5, dfactor(20.0), bc=bc)
        assert_parity(g, st, o)
    # zero echoes, zero walkers
    engine.upload_walkers(*w)
    z = engine.cpmg(0, 1, dfactor(20.0))
    assert z["echo_sum"][0] == len(idx)
    engine.upload_walkers(*(a[:0] for a in w))
    e = engine.cpmg(10, 1, dfactor(20.0))
    assert np.all(e["echo_sum"] == 0) and np.all(e["echo_coll"] == 0)


def test_cpmg_rejects_bad_input(engine):
    from randomwalk_nmr_gb300 import RwnmrError

    lab = image()
    engine.upload_labels(lab)
    with pytest.raises(RwnmrError):
        engine.cpmg(10, 1, 0.5)  # walkers missing
    engine.upload_walkers(np.array([500], np.int32), np.array([0], np.int32), np.array([0], np.int32),
                          np.array([1], np.uint64))
    with pytest.raises(RwnmrError, match="outside the image"):
        engine.cpmg(10, 1, 0.5)
    with pytest.raises(RwnmrError):
        engine.cpmg(10, 1, 1.5)  # decrease factor outside [0, 1]


@pytest.mark.parametrize("n_phases", [2, 3])
def test_labels_beyond_the_phase_count_are_rejected(engine, n_phases):
    """A multi-phase upload whose labels name a phase beyond n_phases fails (the walks index the
    per-phase tables by the voxel's phase); single-phase images take any non-zero label as solid."""
    from randomwalk_nmr_gb300 import RwnmrError

    lab = image(n_phases=n_phases + 1)
    assert lab.max() == n_phases + 1
    with pytest.raises(RwnmrError, match="exceeds the phase count"):
        engine.upload_labels(lab, n_phases)
    engine.upload_labels(lab, n_phases + 1)
    engine.upload_labels(lab, 1)


@pytest.mark.parametrize("bc,n_phases", [("noflux", 1), ("periodic", 1), ("noflux", 2), ("mirror", 4)])
def test_map_walk_matches_oracle(engine, oracle, bc, n_phases):
    lab = image(seed=4, n_phases=n_phases)
    w = walkers(lab, 2500, 8)
    engine.upload_labels(lab, n_phases)
    engine.upload_walkers(*w)
    coll = engine.map(20000 + 17, bc=bc)  # two launches of up to 16384 steps
    d, oc = oracle.displacements(lab, w, 20000 + 17, bc=bc, threads=4, n_phases=n_phases)
    assert np.array_equal(coll, oc.sum(axis=1))
    assert np.array_equal(engine.download_walkers()["collisions"], oc)
    st = engine.download_walkers()
    assert np.array_equal(st["x"] - w[0], d[0])
    assert np.array_equal(st["z"] - w[2], d[2])


def test_cpmg_per_walker_dfactor_reference_golden(engine, golden):
    """RHO_TYPE sigmoid: every walker relaxes with its own decrease factor (the reference's, from
    the sigmoid of its collision rate); the echo sums are the reference's raw signal."""
    gd = golden
    engine.upload_labels(gd["img_a"])
    engine.upload_walkers(gd["cpmg_x0"], gd["cpmg_y0"], gd["cpmg_z0"], gd["cpmg_seed0"])
    engine.set_walker_dfactor(gd["cpmg_sig_dfactor"])
    n_echoes = len(gd["cpmg_sig_raw"]) - 1
    g = engine.cpmg(n_echoes, 3, None)
    np.testing.assert_allclose(g["echo_sum"], gd["cpmg_sig_raw"], rtol=1e-12)
    # launch chunks carry each walker's energy exactly
    g2 = engine.cpmg(n_echoes, 3, None, echoes_per_launch=7)
    assert np.array_equal(g2["echo_fx"], g["echo_fx"]) and np.array_equal(g2["echo_coll"], g["echo_coll"])


def test_cpmg_per_walker_dfactor_equal_factors_match_tables(engine):
    from randomwalk_nmr_gb300 import RwnmrError

    lab = image(seed=12)
    w = walkers(lab, 3000, 2)
    engine.upload_labels(lab)
    engine.upload_walkers(*w)
    f = dfactor(17.0)
    t = engine.cpmg(80, 2, f)
    engine.set_walker_dfactor(np.full(len(w[0]), f))
    p = engine.cpmg(80, 2, None)
    assert np.array_equal(p["echo_fx"], t["echo_fx"])
    assert np.array_equal(p["echo_coll"], t["echo_coll"])
    with pytest.raises(RwnmrError):
        engine.cpmg_adjoint(80, 2, None, np.ones(81))
    with pytest.raises(RwnmrError):
        engine.set_walker_dfactor(np.full(len(w[0]), 1.5))
    engine.upload_walkers(*w)  # new walkers drop the factors
    with pytest.raises(RwnmrError, match="per-walker"):
        engine.cpmg(10, 2, None)
    engine.upload_labels(image(n_phases=2, seed=12), 2)
    engine.upload_walkers(*w)
    engine.set_walker_dfactor(np.full(len(w[0]), f))
    with pytest.raises(RwnmrError, match="single-phase"):
        engine.cpmg(10, 2, None)


@pytest.mark.parametrize("n_phases", [1, 2, 3])
def test_image_upload_and_download_blocks(engine, golden, n_phases):
    """GPU packing of labels (with phase planes) returns the reference's bit-blocks as solid masks;
    blocks + labels are accepted when they agree and rejected when they do not."""
    from randomwalk_nmr_gb300 import RwnmrError

    lab = golden["img_a"].astype(np.uint8)
    if n_phases > 1:
        lab = image(shape=lab.shape, n_phases=n_phases, seed=17)
    blocks, _ = host.pack_blocks(lab)
    engine.upload_labels(lab, n_phases)
    assert np.array_equal(engine.download_blocks(), blocks)
    if n_phases == 1:
        assert np.array_equal(blocks, golden["img_a_blocks"])
    engine.upload_blocks(blocks, lab.shape, lab if n_phases > 1 else None, n_phases)
    assert np.array_equal(engine.download_blocks(), blocks)
    bad = blocks.copy()
    bad[len(bad) // 2] ^= np.uint64(1)
    with pytest.raises(RwnmrError, match="disagree"):
        engine.upload_blocks(bad, lab.shape, lab, n_phases)


@pytest.mark.parametrize("shape", [(26, 22, 30), (2, 3, 64), (40, 2, 5), (33, 17, 9)])
@pytest.mark.parametrize("n_phases", [1, 2, 4])
def test_cpmg_morton_and_block_layouts(engine, oracle, shape, n_phases):
    """The noflux walk runs on the image's Morton copy (built for these small images) or, with the
    copy switched off, on the bit-blocks; both are bit-exact against the oracle, including walkers
    reversing at every face of thin images, and identical to each other."""
    lab = image(shape=shape, seed=13, porosity=0.3, n_phases=n_phases, rmin=1.0, rmax=3.0)
    w = walkers(lab, 2500, 17)
    rho = [5.0, 25.0, 12.0, 40.0][:n_phases]
    df = dfactor(rho) if n_phases > 1 else dfactor(10.0)
    try:
        for morton in (True, False):
            engine.allow_morton(morton)
            g, st, o = run_both(engine, oracle, lab, w, 120, 3, df, n_phases=n_phases)
            assert engine.morton_layout == morton
            assert_parity(g, st, o)
            # one step per echo (the headline instance) and a runtime step count
            for spe in (1, 7):
                g, st, o = run_both(engine, oracle, lab, w, 60, spe, df, n_phases=n_phases)
                assert_parity(g, st, o)
    finally:
        engine.allow_morton(True)


def test_long_mapping_walk_with_walker_resorting(engine, oracle):
    """A mapping walk of many walkers (>= 2^16) over more than two 2048-step launches re-sorts the
    stored walkers by position between launches: collision counts, final positions and seeds still
    come back in upload order and equal the oracle's, and later walks on the context are unchanged."""
    lab, _ = host.synth_spheres((40, 36, 44), 2.0, 6.0, 0.35, 2, seed=21)
    blocks, _ = host.pack_blocks(lab)
    w = host.place_walkers(blocks, lab.shape, 70_000, 9)[:4]
    engine.upload_labels(lab, 2)
    engine.upload_walkers(*w)
    steps = 5000
    coll = engine.map(steps)
    st = engine.download_walkers()
    m = 3000
    sub = tuple(a[:m] for a in w)
    f = dfactor([10.0, 30.0])
    o = oracle.cpmg(lab, sub, 1, steps, f, n_phases=2, threads=4)
    assert np.array_equal(coll[:m], o["collf"].sum(axis=1))
    assert np.array_equal(st["x"][:m], o["xf"]) and np.array_equal(st["y"][:m], o["yf"])
    assert np.array_equal(st["z"][:m], o["zf"]) and np.array_equal(st["seed"][:m], o["seedf"])
    assert np.array_equal(st["collisions"][:m], o["collf"])
    # the re-sorted context walks from the same initial state as a fresh one
    a = engine.cpmg(60, 2, f)["echo_fx"]
    fresh = Engine(0)
    fresh.upload_labels(lab, 2)
    fresh.upload_walkers(*w)
    b = fresh.cpmg(60, 2, f)["echo_fx"]
    fresh.close()
    assert np.array_equal(a, b)


def test_checkpoint_and_resume_in_another_context(engine):
    """A mapping walk checkpointed after 700 steps (download_walkers), restored into a fresh context
    with the same uploaded walkers and continued for 900 steps equals an uninterrupted 1600-step walk:
    positions, RNG states and per-phase collision counts."""
    lab, _ = host.synth_spheres((30, 34, 28), 2.0, 5.0, 0.35, 2, seed=8)
    blocks, _ = host.pack_blocks(lab)
    w = host.place_walkers(blocks, lab.shape, 5000, 3)[:4]
    engine.upload_labels(lab, 2)
    engine.upload_walkers(*w)
    engine.map(1600)
    full = engine.download_walkers()
    engine.upload_walkers(*w)
    engine.map(700)
    ckpt = engine.download_walkers()
    other = Engine(0)
    other.upload_labels(lab, 2)
    other.upload_walkers(*w)
    other.restore_walkers(ckpt)
    other.map_continue(900)
    resumed = other.download_walkers()
    other.close()
    for key in ("x", "y", "z", "seed", "collisions"):
        assert np.array_equal(resumed[key], full[key]), key


@pytest.mark.parametrize("bc", ["noflux", "periodic", "mirror"])
@pytest.mark.parametrize("spe", [1, 2, 3])
@pytest.mark.parametrize("n_phases", [1, 2])
def test_cpmg_fixed_step_instances(engine, oracle, bc, spe, n_phases):
    """The instances with the steps per echo fixed at compile time (1-3), including the Morton walk's
    fast echo loop (noflux), for every boundary condition, against the oracle; 2600 walkers leave a
    partial last CTA, so both echo loops run."""
    lab = image(shape=(27, 31, 23), n_phases=n_phases, seed=17)
    w = walkers(lab, 2600, 21)
    g, st, o = run_both(engine, oracle, lab, w, 70, spe, dfactor([7.0, 30.0][:n_phases]), bc=bc, n_phases=n_phases)
    assert_parity(g, st, o)


@pytest.mark.parametrize("chunk", [45, 64, 1000])
@pytest.mark.parametrize("spe", [1, 2])
@pytest.mark.parametrize("n_phases", [1, 2])
def test_cpmg_collision_replay_across_launches(engine, oracle, chunk, spe, n_phases):
    """The collision replay (one or two steps per echo, Morton walk) split into launches of 45, 64 and
    1000 echoes: windows start at odd echoes, the last window of a launch is partial, and the counts
    and per-CTA limb sums restart from the stored walker state at each launch."""
    lab = image(shape=(40, 36, 44), n_phases=n_phases, seed=23)
    w = walkers(lab, 5000, 29)
    g, st, o = run_both(engine, oracle, lab, w, 230, spe, dfactor([12.0, 40.0][:n_phases]), n_phases=n_phases,
                        chunk=chunk)
    assert_parity(g, st, o)
