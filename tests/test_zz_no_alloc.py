"""rwnmr_cpmg_run_noalloc: the CPMG walk for callers that cannot let the library allocate device
memory (their own allocator owns the GPU's memory, or they run under a hard memory cap). The test
owns every device buffer (allocated here through torch), calls the entry point through the C ABI
twice in a row, and checks both calls against the regular context-based entry point (bit for bit)
and the CPU oracle, and that the device's free memory does not change during a call."""
import ctypes

import numpy as np
import pytest

from conftest import dfactor
from randomwalk_nmr_gb300 import Engine, host
from randomwalk_nmr_gb300.engine import CpmgParams, load_library

pytestmark = pytest.mark.gpu

ECHO_RTOL = 1e-12  # same tolerance as the other CPMG parity tests


class NoallocArgs(ctypes.Structure):
    _fields_ = [
        ("blocks", ctypes.c_void_p), ("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("nz", ctypes.c_int32),
        ("n_phases", ctypes.c_int32), ("n", ctypes.c_int64), ("x0", ctypes.c_void_p), ("y0", ctypes.c_void_p),
        ("z0", ctypes.c_void_p), ("seed0", ctypes.c_void_p), ("x", ctypes.c_void_p), ("y", ctypes.c_void_p),
        ("z", ctypes.c_void_p), ("seed", ctypes.c_void_p), ("collisions", ctypes.c_void_p),
        ("echo_sum", ctypes.c_void_p), ("echo_coll", ctypes.c_void_p), ("stream", ctypes.c_void_p),
    ]


def device_blocks(labels, n_phases):
    """Bit-blocks with phase bit-planes in the layout the entry point documents."""
    blocks, _ = host.pack_blocks(labels)
    if n_phases == 1:
        return blocks
    nz, ny, nx = labels.shape
    bc, br, bd = (nx + 3) // 4, (ny + 3) // 4, (nz + 3) // 4
    words = 2 if n_phases == 2 else 4
    out = np.zeros((len(blocks), words), np.uint64)
    out[:, 0] = blocks
    pad = np.zeros((bd * 4, br * 4, bc * 4), np.uint8)
    pad[:nz, :ny, :nx] = labels
    ph = np.where(pad > 0, pad.astype(np.int64) - 1, 0)
    z, y, x = np.meshgrid(np.arange(bd * 4), np.arange(br * 4), np.arange(bc * 4), indexing="ij")
    blk = (x // 4) + (y // 4) * bc + (z // 4) * bc * br
    bit = (x % 4) + 4 * (y % 4) + 16 * (z % 4)
    for plane in range(words - 1):
        sel = ((ph >> plane) & 1).astype(bool) & (pad > 0)
        vals = np.zeros(len(blocks), np.uint64)
        np.bitwise_or.at(vals, blk[sel], np.left_shift(np.uint64(1), bit[sel].astype(np.uint64)))
        out[:, plane + 1] = vals
    # each block as 2W uint32: the W words' low halves, then their high halves
    halves = np.concatenate([out & np.uint64(0xFFFFFFFF), out >> np.uint64(32)], axis=1).astype(np.uint32)
    return halves.reshape(-1).view(np.uint64)


def run_noalloc(lab, n_phases, walkers, n_echoes, spe, f, blocks=None, calls=2):
    """Owns every device buffer (allocated through torch before the calls), calls the entry point
    `calls` times in a row and yields (status, message, outputs, free bytes before, after) per call."""
    import torch

    fn = load_library().rwnmr_cpmg_run_noalloc
    x, y, z, s = walkers
    dev = torch.device("cuda:0")
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)  # noqa: E731
    d_blocks = t((device_blocks(lab, n_phases) if blocks is None else blocks).view(np.int64))
    d_in = [t(x), t(y), t(z), t(s.view(np.int64))]
    n = len(x)
    d_x, d_y, d_z = (torch.empty(n, dtype=torch.int32, device=dev) for _ in range(3))
    d_seed = torch.empty(n, dtype=torch.int64, device=dev)
    d_coll = torch.empty(n_phases * n, dtype=torch.int32, device=dev)
    d_sum = torch.empty(n_echoes + 1, dtype=torch.float64, device=dev)
    d_ecoll = torch.empty(n_echoes * n_phases, dtype=torch.int64, device=dev)
    stream = torch.cuda.current_stream(dev)
    nz, ny, nx = lab.shape
    args = NoallocArgs(d_blocks.data_ptr(), nx, ny, nz, n_phases, n, *[a.data_ptr() for a in d_in], d_x.data_ptr(),
                       d_y.data_ptr(), d_z.data_ptr(), d_seed.data_ptr(), d_coll.data_ptr(), d_sum.data_ptr(),
                       d_ecoll.data_ptr(), stream.cuda_stream)
    prm = CpmgParams(0, 0, spe, n_echoes, f.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), 0)
    err = ctypes.create_string_buffer(256)
    for _ in range(calls):
        d_sum.fill_(-1.0)
        d_ecoll.fill_(-1)
        d_x.fill_(-1)
        d_y.fill_(-1)
        d_z.fill_(-1)
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info(dev)[0]
        st = fn(ctypes.byref(prm), ctypes.byref(args), err, len(err))
        torch.cuda.synchronize()
        free1 = torch.cuda.mem_get_info(dev)[0]
        out = dict(echo_sum=d_sum.cpu().numpy(), echo_coll=d_ecoll.cpu().numpy().reshape(n_echoes, n_phases).astype(np.uint64),
                   x=d_x.cpu().numpy(), y=d_y.cpu().numpy(), z=d_z.cpu().numpy(),
                   seed=d_seed.cpu().numpy().view(np.uint64),
                   collisions=d_coll.cpu().numpy().view(np.uint32).reshape(n_phases, n).T)
        yield st, err.value.decode(), out, free0, free1


@pytest.mark.parametrize("n_phases", [1, 2, 3])
def test_noalloc_matches_context_entry_point_and_oracle_twice(n_phases, oracle):
    lab, _ = host.synth_spheres((30, 26, 34), 2.0, 6.0, 0.35, n_phases, seed=21)
    blocks, _ = host.pack_blocks(lab)
    x, y, z, s, _ = host.place_walkers(blocks, lab.shape, 5000, 9)
    n_echoes, spe = 300, 2
    f = np.ascontiguousarray(np.broadcast_to(dfactor([10.0, 30.0, 18.0][:n_phases]), (n_phases,)))

    eng = Engine(0)
    eng.upload_labels(lab, n_phases)
    eng.upload_walkers(x, y, z, s)
    ref = eng.cpmg(n_echoes, spe, f)
    ref_state = eng.download_walkers()
    eng.close()
    orc = oracle.cpmg(lab, (x, y, z, s), n_echoes, spe, f, n_phases=n_phases, threads=4)

    for call, (st, msg, out, free0, free1) in enumerate(run_noalloc(lab, n_phases, (x, y, z, s), n_echoes, spe, f)):
        assert st == 0, msg
        if call > 0:
            # nothing was allocated on the device during the call (the first call may still load the
            # library's kernels, which the CUDA driver does on first use)
            assert free1 == free0
        # the same exact sums as the context entry point, converted with the same single rounding
        assert np.array_equal(out["echo_sum"], ref["echo_sum"]), call
        assert np.array_equal(out["echo_coll"], ref["echo_coll"]), call
        for k in ("x", "y", "z", "seed", "collisions"):
            assert np.array_equal(out[k], ref_state[k]), (call, k)
        # and the CPU oracle: bit-exact integers, echo sums within the CPMG parity tolerance
        assert np.array_equal(out["x"], orc["xf"]) and np.array_equal(out["y"], orc["yf"])
        assert np.array_equal(out["z"], orc["zf"]) and np.array_equal(out["seed"], orc["seedf"])
        assert np.array_equal(out["collisions"], orc["collf"])
        assert np.array_equal(out["echo_coll"], orc["echo_coll"])
        np.testing.assert_allclose(out["echo_sum"], orc["echo_fp64"], rtol=ECHO_RTOL, atol=0)


def test_noalloc_rejects_phase_index_beyond_phase_count():
    """A 3-phase image whose bit-planes mark a solid voxel with phase index 3 is an error, not a
    walk that silently skips that voxel's relaxation."""
    lab, _ = host.synth_spheres((20, 18, 22), 2.0, 5.0, 0.4, 4, seed=23)
    assert lab.max() == 4
    blocks, _ = host.pack_blocks(lab)
    x, y, z, s, _ = host.place_walkers(blocks, lab.shape, 500, 3)
    f = dfactor([10.0, 30.0, 18.0])
    bad = device_blocks(lab, 4)  # planes of a 4-phase image passed as 3 phases
    st, msg, _, _, _ = next(run_noalloc(lab, 3, (x, y, z, s), 20, 1, f, blocks=bad, calls=1))
    assert st == 1 and "phase index" in msg  # RWNMR_ERR_INVALID


def test_noalloc_rejects_oversized_walk():
    lib = load_library()
    f = np.array([0.99])
    prm = CpmgParams(0, 0, 1, 2_000_000, f.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), 0)
    args = NoallocArgs(256, 8, 8, 8, 1, 0, None, None, None, None, None, None, None, None, None, 256, None, None)
    err = ctypes.create_string_buffer(256)
    st = lib.rwnmr_cpmg_run_noalloc(ctypes.byref(prm), ctypes.byref(args), err, len(err))
    assert st == 5  # RWNMR_ERR_UNSUPPORTED
    assert b"bytes of scratch" in err.value
