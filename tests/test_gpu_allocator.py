"""Injectable device allocator (rwnmr_set_device_allocator): an allocator that fails makes the calls
that need memory return RWNMR_ERR_NOMEM and leaves the context usable; PyTorch's caching allocator
gives the same results as cudaMalloc; buffers are freed by the allocator that made them."""
import numpy as np
import pytest

from conftest import dfactor
from randomwalk_nmr_gb300 import Engine, RwnmrError, host, set_device_allocator, use_torch_allocator

pytestmark = pytest.mark.gpu


def _inputs(seed=4, n=3000):
    lab, _ = host.synth_spheres((30, 28, 26), 2.0, 5.0, 0.35, 2, seed=seed)
    blocks, _ = host.pack_blocks(lab)
    return lab, host.place_walkers(blocks, lab.shape, n, seed)[:4]


def _run(eng, lab, w):
    eng.upload_labels(lab, 2)
    eng.upload_walkers(*w)
    return eng.cpmg(30, 2, dfactor([10.0, 30.0]))["echo_fx"]


def test_failing_allocator_gives_nomem_and_the_context_recovers():
    lab, w = _inputs()
    ref_eng = Engine(0)
    ref = _run(ref_eng, lab, w)
    ref_eng.close()
    eng = Engine(0)
    calls = []
    try:
        set_device_allocator(lambda n: calls.append(n) or 0, lambda p: None)
        with pytest.raises(RwnmrError) as e:
            _run(eng, lab, w)
        assert e.value.status == 3 and calls  # RWNMR_ERR_NOMEM, from the injected allocator
    finally:
        set_device_allocator(None, None)
    assert np.array_equal(_run(eng, lab, w), ref)
    eng.close()


def test_allocator_failing_midway_through_a_run():
    """Every allocation succeeds through cudaMalloc-backed torch memory until the k-th, for each k:
    each failure is a clean RWNMR_ERR_NOMEM and the next run, with memory, matches."""
    torch = pytest.importorskip("torch")
    lab, w = _inputs(seed=5, n=1500)
    ref_eng = Engine(0)
    ref = _run(ref_eng, lab, w)
    ref_eng.close()
    for k in range(0, 12, 3):
        count = [0]

        def alloc(n, k=k):
            count[0] += 1
            return 0 if count[0] > k else torch.cuda.caching_allocator_alloc(n, 0)

        eng = Engine(0)
        try:
            set_device_allocator(alloc, torch.cuda.caching_allocator_delete)
            try:
                out = _run(eng, lab, w)
                assert np.array_equal(out, ref)  # k was past the run's last allocation
            except RwnmrError as e:
                assert e.status == 3
        finally:
            set_device_allocator(None, None)
        assert np.array_equal(_run(eng, lab, w), ref)
        eng.close()


def test_torch_caching_allocator_same_results():
    pytest.importorskip("torch")
    lab, w = _inputs(seed=6)
    ref_eng = Engine(0)
    ref = _run(ref_eng, lab, w)
    ref_eng.close()
    try:
        use_torch_allocator(0)
        eng = Engine(0)
        assert np.array_equal(_run(eng, lab, w), ref)
        eng.close()  # frees through the torch allocator
    finally:
        set_device_allocator(None, None)


def test_allocator_arguments_checked():
    with pytest.raises(ValueError):
        set_device_allocator(lambda n: 0, None)
