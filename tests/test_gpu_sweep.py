"""Seeded sweep of CPMG and PFGSE configurations against the oracle: random image shapes (thin and
odd ones included), 1-4 phases, every boundary condition, voxel division, 1-7 steps per echo, both
image layouts and walker counts that leave partial sort tiles. Every case bit-exact on positions,
RNG states, collision counts and fixed-point sums."""
import numpy as np
import pytest

from conftest import dfactor
from randomwalk_nmr_gb300 import host

pytestmark = pytest.mark.gpu

CASES = 24


def config(k):
    rng = np.random.default_rng(1000 + k)
    shape = tuple(int(v) for v in rng.integers(2, 41, 3))
    n_phases = int(rng.choice([1, 1, 2, 3, 4]))
    bc = str(rng.choice(["noflux", "noflux", "periodic", "mirror"]))
    shift = int(rng.choice([0, 0, 0, 1]))
    spe = int(rng.integers(1, 8))
    echoes = int(rng.integers(5, 41))
    n = int(rng.integers(1, 3000))
    morton = bool(rng.integers(0, 2))
    return dict(shape=shape, n_phases=n_phases, bc=bc, shift=shift, spe=spe, echoes=echoes, n=n, morton=morton,
                seed=int(rng.integers(1, 1 << 30)))


@pytest.mark.parametrize("k", range(CASES))
def test_cpmg_sweep(engine, oracle, k):
    c = config(k)
    lab, _ = host.synth_spheres(c["shape"], 1.0, 4.0, 0.35, c["n_phases"], seed=c["seed"])
    blocks, _ = host.pack_blocks(lab)
    try:
        w = host.place_walkers(blocks, lab.shape, c["n"], c["seed"] + 1, shift=c["shift"])[:4]
    except Exception:
        pytest.skip("no pore voxel to place walkers in")
    rho = [5.0, 25.0, 12.0, 40.0][: c["n_phases"]]
    df = dfactor(rho)
    engine.allow_morton(c["morton"])
    engine.upload_labels(lab, c["n_phases"])
    engine.upload_walkers(*w)
    g = engine.cpmg(c["echoes"], c["spe"], df, bc=c["bc"], shift=c["shift"])
    st = engine.download_walkers()
    o = oracle.cpmg(lab, w, c["echoes"], c["spe"], df, bc=c["bc"], shift=c["shift"], n_phases=c["n_phases"], threads=4)
    assert np.array_equal(st["x"], o["xf"]) and np.array_equal(st["y"], o["yf"]) and np.array_equal(st["z"], o["zf"])
    assert np.array_equal(st["seed"], o["seedf"])
    assert np.array_equal(st["collisions"], o["collf"])
    assert np.array_equal(g["echo_coll"], o["echo_coll"])
    assert np.array_equal(g["echo_fx"], o["echo_fx"])


@pytest.mark.parametrize("k", range(0, CASES, 3))
def test_pfgse_sweep(engine, oracle, k):
    c = config(k)
    lab, _ = host.synth_spheres(c["shape"], 1.0, 4.0, 0.35, 1, seed=c["seed"])
    blocks, _ = host.pack_blocks(lab)
    try:
        w = host.place_walkers(blocks, lab.shape, c["n"], c["seed"] + 1)[:4]
    except Exception:
        pytest.skip("no pore voxel to place walkers in")
    steps = np.array(sorted({1, 2 * c["spe"], 5 * c["spe"], 9 * c["spe"]}), np.int32)
    kv = np.zeros((6, 3))
    kv[:, 2] = np.linspace(0.0, 0.05, 6)
    f = dfactor(10.0)
    engine.allow_morton(c["morton"])
    engine.upload_labels(lab, 1)
    engine.upload_walkers(*w)
    out = engine.pfgse(steps, kv, 1.0, f, bc=c["bc"])
    o = oracle.pfgse(lab, w, f, steps, kv, 1.0, bc=c["bc"], threads=4)
    np.testing.assert_allclose(out["M"], o["M"], rtol=0, atol=1e-12 * max(1.0, float(np.max(np.abs(o["M"])))))
    assert np.array_equal(out["msd"], o["msd"])
