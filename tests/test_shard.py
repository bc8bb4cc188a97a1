"""Multi-rank walker sharding on CPU: two gloo ranks each walk half of the population (the oracle
stands in for each rank's GPU walk) and one integer all-reduce gives echo sums bit-identical to
the whole population walked at once."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from randomwalk_nmr_gb300 import host  # noqa: E402
from randomwalk_nmr_gb300.shard import allreduce_sum_int, combine_cpmg, shard_bounds  # noqa: E402


def test_shard_bounds_cover_the_population():
    for n in (0, 1, 7, 1000, 1001):
        for world in (1, 2, 3, 8):
            spans = [shard_bounds(n, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
            assert max(h - l for l, h in spans) - min(h - l for l, h in spans) <= 1
    with pytest.raises(ValueError):
        shard_bounds(10, 2, 2)


def test_no_process_group_is_identity():
    a = np.arange(12, dtype=np.uint64).reshape(4, 3)
    assert np.array_equal(allreduce_sum_int(a), a)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, lab, walkers, q):
    import torch.distributed as dist

    from oracle.pyoracle import Oracle

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    lo, hi = shard_bounds(len(walkers[0]), rank, world)
    o = Oracle().cpmg(lab, tuple(a[lo:hi] for a in walkers), 60, 2, 0.993, threads=1)
    out = combine_cpmg(dict(echo_fx=o["echo_fx"], echo_coll=o["echo_coll"]))
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, out["echo_fx"], out["echo_coll"], out["echo_sum"]))


@pytest.mark.parametrize("world", [2, 3])
def test_sharded_echo_sums_are_bit_identical(oracle, world):
    import torch.multiprocessing as mp

    lab, _ = host.synth_spheres((22, 18, 20), 2.0, 5.0, 0.35, 1, seed=6)
    blocks, _ = host.pack_blocks(lab)
    walkers = host.place_walkers(blocks, lab.shape, 1501, 3)[:4]
    full = oracle.cpmg(lab, walkers, 60, 2, 0.993, threads=1)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, lab, walkers, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, fx, coll, esum in res:
        assert np.array_equal(fx, full["echo_fx"])
        assert np.array_equal(coll, full["echo_coll"])
        np.testing.assert_allclose(esum, full["echo_fp64"], rtol=1e-12)
