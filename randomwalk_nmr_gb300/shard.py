"""Walker sharding across ranks (one process per GPU).

Walkers are independent, so a population splits into contiguous slices, one per rank, with no
communication during the walk. The only exchange is at the end: every rank holds the exact
fixed-point limb sums of its slice's energies per echo (``echo_fx``, three integer limbs per echo),
and one integer all-reduce adds them. Integer addition is exact and associative, so the combined
echo train is bit-identical to one GPU walking the whole population, for any number of ranks and
any split. The same holds for the per-echo per-phase collision counts.

Limb sums stay below 2^53 per rank (fewer than 2^31 walkers, limbs below 2^22), so up to 2^10 ranks
add without overflow in int64.
"""
from __future__ import annotations

import numpy as np

from .engine import fx_to_float


def shard_bounds(n: int, rank: int, world: int) -> tuple[int, int]:
    """Contiguous walker range [lo, hi) of `rank` among `world` ranks (sizes differ by at most 1)."""
    if not 0 <= rank < world:
        raise ValueError("rank out of range")
    return n * rank // world, n * (rank + 1) // world


def allreduce_sum_int(values: np.ndarray, group=None) -> np.ndarray:
    """Sums an integer array over the ranks of `group` (exact); a no-op without a process group."""
    import torch
    import torch.distributed as dist

    arr = np.ascontiguousarray(values)
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size(group) == 1:
        return arr.copy()
    t = torch.from_numpy(arr.astype(np.int64))
    if dist.get_backend(group) == "nccl":
        t = t.cuda()
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t.cpu().numpy().astype(arr.dtype)


def combine_cpmg(out: dict, group=None) -> dict:
    """Global echo train from one rank's `Engine.cpmg` output over its walker slice."""
    fx = allreduce_sum_int(out["echo_fx"], group)
    coll = allreduce_sum_int(out["echo_coll"], group)
    return dict(echo_sum=fx_to_float(fx), echo_fx=fx, echo_coll=coll)


def cpmg_sharded(engine, walkers, rank: int, world: int, n_echoes: int, steps_per_echo: int, dfactor,
                 bc: str = "noflux", shift: int = 0, group=None) -> dict:
    """Uploads this rank's slice of `walkers` (x0, y0, z0, seed0) to `engine`, walks it, and combines
    the echo trains of all ranks."""
    lo, hi = shard_bounds(len(walkers[0]), rank, world)
    engine.upload_walkers(*(np.ascontiguousarray(a[lo:hi]) for a in walkers))
    return combine_cpmg(engine.cpmg(n_echoes, steps_per_echo, dfactor, bc=bc, shift=shift), group)
