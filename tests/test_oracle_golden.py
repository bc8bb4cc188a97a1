"""Pins the CPU restatement (oracle/) and the host frontend against fixtures produced by the
reference's own CPU code (tests/golden/make_golden.py). Runs without a GPU."""
import numpy as np

from randomwalk_nmr_gb300 import host


def test_bitblock_packing_matches_reference(golden, oracle):
    lab = golden["img_a"]
    b, dims = oracle.pack_blocks(lab)
    assert np.array_equal(b, golden["img_a_blocks"])
    assert list(dims) == list(golden["img_a_bdims"])
    hb, hdims = host.pack_blocks(lab)
    assert np.array_equal(hb, golden["img_a_blocks"])
    assert list(hdims) == list(golden["img_a_bdims"])


def test_walk_matches_reference_bit_exact(golden, oracle):
    g = golden
    walkers = (g["walk_x0"], g["walk_y0"], g["walk_z0"], g["walk_seed0"])
    f = float(g["walk_dfactor"][0])
    assert np.all(g["walk_dfactor"] == f)
    out = oracle.cpmg(g["img_a"], walkers, 200, 2, f)
    # FP64 energy sums in the reference's serial walker order: bit-exact
    assert np.array_equal(out["echo_fp64"], g["walk_energy_sum"])
    assert np.array_equal(out["echo_coll"][:, 0], g["walk_coll_per_echo"])
    assert np.array_equal(out["xf"], g["walk_xf"])
    assert np.array_equal(out["yf"], g["walk_yf"])
    assert np.array_equal(out["zf"], g["walk_zf"])
    assert np.array_equal(out["seedf"], g["walk_seedf"])
    assert np.array_equal(out["collf"][:, 0], g["walk_coll"])


def test_oracle_threads_do_not_change_integers(golden, oracle):
    g = golden
    walkers = (g["walk_x0"], g["walk_y0"], g["walk_z0"], g["walk_seed0"])
    f = float(g["walk_dfactor"][0])
    a = oracle.cpmg(g["img_a"], walkers, 50, 2, f, threads=1)
    b = oracle.cpmg(g["img_a"], walkers, 50, 2, f, threads=4)
    assert np.array_equal(a["echo_fx"], b["echo_fx"])
    assert np.array_equal(a["echo_coll"], b["echo_coll"])
    np.testing.assert_allclose(a["echo_fp64"], b["echo_fp64"], rtol=1e-14)


def test_cpmg_sequence_raw_signal(golden, oracle):
    """The reference CPMG (map walk, relaxivity update, walk) raw echo sums."""
    g = golden
    walkers = (g["cpmg_x0"], g["cpmg_y0"], g["cpmg_z0"], g["cpmg_seed0"])
    n = len(g["cpmg_raw"]) - 1
    f = float(g["cpmg_dfactor"][0])
    out = oracle.cpmg(g["img_a"], walkers, n, 3, f)
    assert np.array_equal(out["echo_fp64"], g["cpmg_raw"])
    # the collision-mapping walk before it covers the same steps
    assert np.array_equal(out["collf"][:, 0], g["cpmg_map_collisions"])


def test_pfgse_matches_reference(golden, oracle):
    g = golden
    walkers = (g["pfgse_x0"], g["pfgse_y0"], g["pfgse_z0"], g["pfgse_seed0"])
    f = float(g["pfgse_dfactor"][0])
    out = oracle.pfgse(g["img_a"], walkers, f, g["pfgse_steps"], g["pfgse_kvec"], 1.0)
    Mkt = out["M"] / out["esum"][:, None]
    # same per-walker FP64 formula and serial order as NMR_PFGSE::simulation_omp: bit-exact
    assert np.array_equal(Mkt, g["pfgse_Mkt"])


def test_placement_matches_reference(golden):
    g = golden
    lab = g["img_p"]
    blocks, _ = host.pack_blocks(lab)
    k = 0
    while f"place{k}_args" in g:
        dev, shift, n, seed = (int(v) for v in g[f"place{k}_args"])
        mode = str(g[f"place{k}_mode"])
        x, y, z, s, info = host.place_walkers(blocks, lab.shape, n, seed, mode, dev, shift)
        assert info["clamped"] == 0
        assert np.array_equal(x, g[f"place{k}_x"]), mode
        assert np.array_equal(y, g[f"place{k}_y"]), mode
        assert np.array_equal(z, g[f"place{k}_z"]), mode
        assert np.array_equal(s, g[f"place{k}_seed"]), mode
        k += 1
    assert k >= 6


def test_mod6_and_xorshift_restatement(oracle):
    rng = np.random.default_rng(5)
    vals = list(rng.integers(0, 2**63, 2000, dtype=np.uint64) * np.uint64(2) + rng.integers(0, 2, 2000, dtype=np.uint64))
    vals += [0, 1, 5, 6, 11, 12, 2**64 - 1, 2**63, 2**32 - 1, 2**32, 2**32 + 1]
    for v in vals:
        assert oracle.lib.orc_mod6(int(v)) == int(v) % 6
    x = 88172645463325252
    for _ in range(100):
        y = oracle.lib.orc_xorshift64(x)
        e = x ^ ((x << 13) & (2**64 - 1))
        e ^= e >> 7
        e ^= (e << 17) & (2**64 - 1)
        assert y == e
        x = y


def test_energy_table_fixed_point(oracle):
    t, fx = oracle.energy_table(0.99, 500)
    assert t[0] == 1.0 and fx[0] == 2**63
    acc = 1.0
    for k in range(1, 501):
        acc = acc * 0.99
        assert t[k] == acc
        assert int(fx[k]) == round(acc * 2.0**63)


# -- full image sizes of the benchmark configurations (tests/golden/reference_c1.npz, reference_c3.npz)
import os  # noqa: E402

import pytest  # noqa: E402

from conftest import ROOT  # noqa: E402


@pytest.fixture(scope="module")
def c1():
    return dict(np.load(os.path.join(ROOT, "tests", "golden", "reference_c1.npz")))


@pytest.fixture(scope="module")
def c3():
    return dict(np.load(os.path.join(ROOT, "tests", "golden", "reference_c3.npz")))


def test_c1_full_size_walk_matches_reference(c1, oracle):
    """100^3 sphere pack, 10,000 walkers, 2000 echoes x 3 steps (6e7 walker-steps): the host's
    image and placement and the restated walk against the reference's own CPU walk."""
    lab, _ = host.synth_spheres((100, 100, 100), 4.0, 10.0, 0.30, 1, seed=1)
    blocks, dims = host.pack_blocks(lab)
    assert np.array_equal(blocks, c1["c1_blocks"]) and list(dims) == list(c1["c1_bdims"])
    x, y, z, s, info = host.place_walkers(blocks, lab.shape, 10_000, 7)
    for a, k in ((x, "x0"), (y, "y0"), (z, "z0"), (s, "seed0")):
        assert np.array_equal(a, c1["c1_" + k])
    f = float(c1["c1_dfactor"][0])
    out = oracle.cpmg(lab, (x, y, z, s), 2000, 3, f, threads=1)
    # one thread: the reference's serial walker order, so even the FP64 echo sums are bit-exact
    assert np.array_equal(out["echo_fp64"], c1["c1_energy_sum"])
    assert np.array_equal(out["echo_coll"][:, 0], c1["c1_coll_per_echo"])
    for a, k in (("xf", "xf"), ("yf", "yf"), ("zf", "zf"), ("seedf", "seedf")):
        assert np.array_equal(out[a], c1["c1_" + k])
    assert np.array_equal(out["collf"][:, 0], c1["c1_coll"])


def test_c3_full_size_pfgse_matches_reference(c3, oracle):
    """256^3 sphere pack, 64 gradients 0-100 G/cm along z, 10 exposure times 1-100 ms log-spaced
    (cumulative walk to 1500 steps), 16,384 walkers: the restated PFGSE sums against the reference's
    own CPU sequence: bit-exact in the reference's serial walker order."""
    import hashlib

    lab, _ = host.synth_spheres((256, 256, 256), 5.0, 15.0, 0.35, 1, seed=3)
    blocks, dims = host.pack_blocks(lab)
    assert hashlib.sha256(blocks.tobytes()).hexdigest() == str(c3["c3_blocks_sha256"])
    x, y, z, s, info = host.place_walkers(blocks, lab.shape, 16_384, 7)
    for a, k in ((x, "x0"), (y, "y0"), (z, "z0"), (s, "seed0")):
        assert np.array_equal(a, c3["c3_" + k])
    f = float(c3["c3_dfactor"][0])
    out = oracle.pfgse(lab, (x, y, z, s), f, c3["c3_steps"], c3["c3_kvec"], 1.0, threads=1)
    Mkt = out["M"] / out["esum"][:, None]
    assert np.array_equal(Mkt, c3["c3_Mkt"])


def test_oracle_inputs_match_reference_placement_and_library_generator(golden, c1, c3, oracle):
    """The oracle's own sphere packs and random placement (used by the benchmark's CPU reference
    arm, which loads no product code): the library's generator gives the same bytes, and the
    placement is the reference's, draw for draw (golden placement fixtures and the full-size sets)."""
    for args in (((20, 18, 22), 2.0, 5.0, 0.4, 4, 23), ((100, 100, 100), 4.0, 10.0, 0.30, 1, 1),
                 ((33, 17, 41), 1.0, 3.5, 0.2, 2, 9)):
        a, pa = oracle.synth_spheres(*args)
        b, pb = host.synth_spheres(*args[:5], seed=args[5])
        assert np.array_equal(a, b) and pa == pb
    lab = golden["img_p"]
    k = 0
    while f"place{k}_args" in golden:
        dev, shift, n, seed = (int(v) for v in golden[f"place{k}_args"])
        if str(golden[f"place{k}_mode"]) == "random":
            x, y, z, s, clamped = oracle.place_walkers(lab, n, seed, shift)
            assert clamped == 0
            for a, key in ((x, "x"), (y, "y"), (z, "z"), (s, "seed")):
                assert np.array_equal(a, golden[f"place{k}_{key}"]), (k, key)
        k += 1
    lab1, _ = oracle.synth_spheres((100, 100, 100), 4.0, 10.0, 0.30, 1, 1)
    assert np.array_equal(oracle.pack_blocks(lab1)[0], c1["c1_blocks"])
    x, y, z, s, _ = oracle.place_walkers(lab1, 10_000, 7)
    assert np.array_equal(x, c1["c1_x0"]) and np.array_equal(z, c1["c1_z0"]) and np.array_equal(s, c1["c1_seed0"])
    lab3, _ = oracle.synth_spheres((256, 256, 256), 5.0, 15.0, 0.35, 1, 3)
    x, y, z, s, _ = oracle.place_walkers(lab3, 16_384, 7)
    assert np.array_equal(y, c3["c3_y0"]) and np.array_equal(s, c3["c3_seed0"])
