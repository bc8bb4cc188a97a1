"""Batched multi-image walk with relaxivity candidates: every (image, candidate) echo train
against the single-image engine on the same walkers, derivatives against the seed-replay
adjoint, graph replay and autotuning; the per-echo collision histograms against the oracle's
per-walker collision counts, and histogram evaluation against the candidate walk (identical sums)."""
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


@pytest.mark.parametrize("bc,method", [("noflux", "walk"), ("periodic", "walk"), ("noflux", "histograms"),
                                       ("mirror", "histograms")])
def test_batch_matches_single_image_engine(bc, method):
    imgs = make_images()
    n_echoes, spe = 40, 3
    rng = np.random.default_rng(1)
    rho = rng.uniform(2.0, 50.0, (len(imgs), 16))
    f = dfactor(rho)
    b = Batch(0)
    for lab, blocks, w in imgs:
        b.add_image(blocks, lab.shape, *w)
    echo, decho = b.cpmg(f, n_echoes, spe, derivatives=True, bc=bc, method=method)
    echo2, decho2 = b.cpmg(f, n_echoes, spe, derivatives=True, bc=bc, use_graph=False, method=method)
    assert np.array_equal(echo, echo2) and np.array_equal(decho, decho2)
    # launch shape and walkers per thread do not change the exact sums
    for t, wpt in ((128, 2), (512, 1), (256, 2)):
        echo3, decho3 = b.cpmg(f, n_echoes, spe, derivatives=True, bc=bc, threads_per_block=t, walkers_per_thread=wpt,
                               method="walk")
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


@pytest.mark.parametrize("bc", ["noflux", "periodic", "mirror"])
def test_histograms_and_candidate_walk_agree_exactly(bc):
    """Sums evaluated from the per-echo collision histograms equal the candidate walk's sums bit for
    bit; a second candidate population is evaluated from the stored histograms without a walk."""
    imgs = make_images(4, seed=7)
    b = Batch(0)
    for lab, blocks, w in imgs:
        b.add_image(blocks, lab.shape, *w)
    rng = np.random.default_rng(3)
    for n_echoes, spe in ((30, 3), (17, 1), (9, 5)):
        f = dfactor(rng.uniform(2.0, 50.0, (4, 16)))
        eh, dh = b.cpmg(f, n_echoes, spe, bc=bc, method="histograms")
        assert b.histogram_walk_ms > 0
        ew, dw = b.cpmg(f, n_echoes, spe, bc=bc, method="walk")
        assert np.array_equal(eh, ew) and np.array_equal(dh, dw)
        f2 = dfactor(rng.uniform(2.0, 50.0, (4, 16)))
        launches = b.launch_count
        eh2, dh2 = b.cpmg(f2, n_echoes, spe, bc=bc, method="histograms")
        assert b.launch_count - launches == 2  # tables and evaluation: no walk
        ew2, dw2 = b.cpmg(f2, n_echoes, spe, bc=bc, method="walk")
        assert np.array_equal(eh2, ew2) and np.array_equal(dh2, dw2)
        e3, d3 = b.cpmg(f2[:, :5], n_echoes, spe, derivatives=False, bc=bc, method="histograms")
        assert d3 is None and np.array_equal(e3, eh2[:, :5])
    b.close()


def test_collision_histograms_match_oracle(oracle):
    """Row e of an image's histogram counts that image's walkers by their collision count after
    echo e, exactly as the oracle's per-walker counts after e echoes give."""
    imgs = make_images(3, seed=9)
    b = Batch(0)
    for lab, blocks, w in imgs:
        b.add_image(blocks, lab.shape, *w)
    spe, n_echoes = 2, 25
    b.cpmg(np.full((3, 1), 0.99), n_echoes, spe, derivatives=False, method="histograms")
    for k, (lab, blocks, w) in enumerate(imgs):
        n = len(w[0])
        for e in (0, 1, 7, n_echoes):
            h = b.collision_histogram(k, e)
            assert len(h) == spe * e + 1 and int(h.sum()) == n
            if e == 0 or n == 0:
                assert h[0] == n
                continue
            coll = oracle.cpmg(lab, w, e, spe, 0.99, threads=4)["collf"][:, 0]
            assert np.array_equal(h, np.bincount(coll, minlength=spe * e + 1))
    with pytest.raises(Exception):
        b.collision_histogram(0, n_echoes + 1)
    b.close()


def _big_batch():
    """Four images with 200k walkers each: more work items than resident CTAs."""
    b = Batch(0)
    for k in range(4):
        lab, _ = host.synth_spheres((48, 44, 40), 2.0, 6.0, 0.35, 1, seed=300 + k)
        blocks, _ = host.pack_blocks(lab)
        w = host.place_walkers(blocks, lab.shape, 200_000, 700 + k)[:4]
        b.add_image(blocks, lab.shape, *w)
    return b


@pytest.mark.parametrize("method", ["walk", "histograms"])
def test_batch_cancel_and_time_budget(method):
    """A cancelled walk and a walk past its time budget stop taking work items, end normally and
    raise RWNMR_ERR_CANCELLED / RWNMR_ERR_TIMEOUT; the batch then runs normally and gives the same
    sums as a batch that was never stopped."""
    from randomwalk_nmr_gb300 import RwnmrError
    f = dfactor(np.linspace(2.0, 50.0, 16))[None, :].repeat(4, axis=0)
    ref_b = _big_batch()
    ref = ref_b.cpmg(f, 40, 3, method=method)
    ref_b.close()
    b = _big_batch()
    b.cancel()
    with pytest.raises(RwnmrError) as e:
        b.cpmg(f, 40, 3, method=method)
    assert e.value.status == 7
    got = b.cpmg(f, 40, 3, method=method)  # the request was consumed
    assert np.array_equal(got[0], ref[0]) and np.array_equal(got[1], ref[1])
    b.set_time_budget(1e-9)
    with pytest.raises(RwnmrError) as e:
        b.cpmg(f, 40, 3, method="walk")  # walks again whatever the stored histograms
    assert e.value.status == 8
    b.set_time_budget(0.0)
    got = b.cpmg(f, 40, 3, method=method)
    assert np.array_equal(got[0], ref[0]) and np.array_equal(got[1], ref[1])
    b.set_time_budget(60.0)  # a generous budget changes nothing
    got = b.cpmg(f, 40, 3, method=method)
    assert np.array_equal(got[0], ref[0]) and np.array_equal(got[1], ref[1])
    b.close()


def test_batch_cancel_does_not_carry_over():
    """A cancel request made while no walk can see it -- here before a call that only evaluates the
    stored collision histograms -- is consumed when that call returns: the call succeeds and the
    next call, which walks again, is not cancelled."""
    f = dfactor(np.linspace(2.0, 50.0, 16))[None, :].repeat(4, axis=0)
    b = _big_batch()
    ref = b.cpmg(f, 40, 3, method="histograms")  # walks and stores the histograms
    b.cancel()
    got = b.cpmg(f, 40, 3, method="histograms")  # evaluates only: completes normally
    assert np.array_equal(got[0], ref[0]) and np.array_equal(got[1], ref[1])
    again = b.cpmg(f, 40, 3, method="walk")  # walks: must not see the earlier request
    assert np.array_equal(again[0], ref[0]) and np.array_equal(again[1], ref[1])
    b.close()
