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
