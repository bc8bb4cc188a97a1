"""Batched multi-image walk with relaxivity candidates: every (image, candidate) echo train
against the single-image engine on the same walkers, derivatives against the seed-replay
adjoint, graph replay and autotuning."""
import numpy as np
import pytest

from conftest import dfactor
from randomwalk_nmr_gb300 import Batch, Engine, host

pytestmark = pytest.mark.gpu


def make_images(n_images=5, seed=0):
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n_images):
        shape = tuple(int(v) for v in rng.integers(12, 40, 3))
        lab, _ = host.synth_spheres(shape, 1.5, 5.0, float(rng.uniform(0.25, 0.45)), 1, seed=100 + k)
        blocks, _ = host.pack_blocks(lab)
        n = int(rng.integers(0, 3000)) if k else 1  # uneven walker counts, one tiny image
        w = host.place_walkers(blocks, lab.shape, n, 500 + k)[:4]
        out.append((lab, blocks, w))
    return out


@pytest.mark.parametrize("bc", ["noflux", "periodic"])
def test_batch_matches_single_image_engine(bc):
    imgs = make_images()
    n_echoes, spe = 40, 3
    rng = np.random.default_rng(1)
    rho = rng.uniform(2.0, 50.0, (len(imgs), 16))
    f = dfactor(rho)
    b = Batch(0)
    for lab, blocks, w in imgs:
        b.add_image(blocks, lab.shape, *w)
    echo, decho = b.cpmg(f, n_echoes, spe, derivatives=True, bc=bc)
    echo2, decho2 = b.cpmg(f, n_echoes, spe, derivatives=True, bc=bc, use_graph=False)
    assert np.array_equal(echo, echo2) and np.array_equal(decho, decho2)
    # launch shape and walkers per thread do not change the exact sums
    for t, wpt in ((128, 2), (512, 1), (256, 2)):
        echo3, decho3 = b.cpmg(f, n_echoes, spe, derivatives=True, bc=bc, threads_per_block=t, walkers_per_thread=wpt)
        assert np.array_equal(echo3, echo) and np.array_equal(decho3, decho)
    eng = Engine(0)
    for k, (lab, blocks, w) in enumerate(imgs):
        eng.upload_labels(lab, 1)
        eng.upload_walkers(*w)
        for r in (0, 7, 15):
            ref = eng.cpmg(n_echoes, spe, f[k, r], bc=bc)["echo_sum"]
            np.testing.assert_allclose(echo[k, r], ref, rtol=1e-12, atol=1e-12)
            g = rng.normal(size=n_echoes + 1)
            adj = eng.cpmg_adjoint(n_echoes, spe, f[k, r], g, bc=bc)[0]
            np.testing.assert_allclose(g @ decho[k, r], adj, rtol=1e-10, atol=1e-9)
    eng.close()
    b.close()


def test_batch_autotune_and_fewer_candidates():
    imgs = make_images(3, seed=4)
    b = Batch(0)
    for lab, blocks, w in imgs:
        b.add_image(blocks, lab.shape, *w)
    t, wpt, ms = b.autotune(20, 2, 16)
    assert t in (128, 256, 512) and wpt in (1, 2) and ms > 0
    f = dfactor(np.array([[10.0, 20.0], [5.0, 30.0], [40.0, 2.0]]))
    echo, _ = b.cpmg(f, 20, 2, derivatives=False)
    assert echo.shape == (3, 2, 21)
    full, _ = b.cpmg(np.concatenate([f, np.ones((3, 14))], 1), 20, 2, derivatives=False)
    assert np.array_equal(full[:, :2], echo)
    b.close()
