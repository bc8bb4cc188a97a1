"""Known-answer physics of the walk, independent of the oracle:
* no surface relaxation (decrease factor 1): every echo sum equals the walker count exactly;
* free diffusion (an image without solid, periodic boundary): the mean squared displacement after t steps
  is t voxels^2, i.e. D = D0 exactly in expectation (MSD = 6 D0 t);
* PFGSE in free space along z: M(k)/M(0) = (2/3 + cos(k res)/3)^t, the exact characteristic function of
  the lattice walk, whose small-k limit is the narrow-pulse exp(-k^2 D0 Delta)."""
import numpy as np
import pytest

from conftest import dfactor
from randomwalk_nmr_gb300 import host

pytestmark = pytest.mark.gpu

D0, RES = 2.5, 1.0


def test_no_relaxation_keeps_every_echo_at_the_walker_count(engine):
    lab, _ = host.synth_spheres((40, 36, 32), 2.0, 6.0, 0.35, 2, seed=12)
    blocks, _ = host.pack_blocks(lab)
    w = host.place_walkers(blocks, lab.shape, 20_000, 2)[:4]
    engine.upload_labels(lab, 2)
    engine.upload_walkers(*w)
    g = engine.cpmg(200, 3, [1.0, 1.0])
    assert np.all(g["echo_sum"] == len(w[0]))
    assert np.all(g["echo_coll"].sum(axis=1) > 0)  # the walkers do hit walls


def _free_space(engine, n=200_000, edge=64, seed=5):
    lab = np.zeros((edge, edge, edge), np.uint8)
    rng = np.random.default_rng(seed)
    x, y, z = (rng.integers(0, edge, n).astype(np.int32) for _ in range(3))
    s = rng.integers(1, 2**63, n, dtype=np.uint64)
    engine.upload_labels(lab, 1)
    engine.upload_walkers(x, y, z, s)
    return n


def test_free_diffusion_msd_is_six_d0_t(engine):
    n = _free_space(engine)
    steps = np.array([10, 100, 400], np.int32)
    out = engine.pfgse(steps, np.zeros((1, 3)), RES, 1.0, bc="periodic")
    msd = out["msd"].sum(axis=1) / n  # voxels^2
    rel = np.abs(msd / steps - 1.0)
    assert np.all(rel < 0.01), rel  # the mean of n walkers: relative error ~ sqrt(2/(3n)) = 0.2 %
    dt = RES * RES / (6.0 * D0)
    D = msd * RES * RES / (6.0 * steps * dt)
    np.testing.assert_allclose(D, D0, rtol=0.01)


def test_free_space_attenuation_is_the_lattice_characteristic_function(engine):
    n = _free_space(engine, seed=6)
    steps = np.array([50, 200], np.int32)
    k = np.linspace(0.0, 0.3, 16)  # rad per micrometre
    kv = np.zeros((len(k), 3))
    kv[:, 2] = k
    out = engine.pfgse(steps, kv, RES, 1.0, bc="periodic")
    att = out["M"] / out["M"][:, :1]
    for i, t in enumerate(steps):
        exact = (2.0 / 3.0 + np.cos(k * RES) / 3.0) ** t
        assert np.all(np.abs(att[i] - exact) < 6.0 / np.sqrt(2.0 * n)), np.max(np.abs(att[i] - exact))
        small = k * k * D0 * t * RES * RES / (6.0 * D0) < 0.5  # narrow-pulse limit, small k
        np.testing.assert_allclose(att[i][small], np.exp(-(k[small] ** 2) * D0 * t * RES * RES / (6.0 * D0)),
                                   atol=0.02)
