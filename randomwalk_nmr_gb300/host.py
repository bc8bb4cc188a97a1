"""Bindings of the host frontend C ABI (include/rwnmr_host.h): synthetic images, bit-block
packing and walker placement. These run on the CPU and need no GPU."""
from __future__ import annotations

import ctypes

import numpy as np

from .engine import load_library

_vp = ctypes.c_void_p

HOST_EXPORTS = ["rwnmr_synth_spheres", "rwnmr_pack_blocks", "rwnmr_place_walkers", "rwnmr_png_solid_mask",
                "rwnmr_config_json", "rwnmr_cli_main"]


class PlacementInfo(ctypes.Structure):
    _fields_ = [("pores", ctypes.c_uint32), ("porosity", ctypes.c_double), ("occupancy", ctypes.c_double),
                ("clamped", ctypes.c_uint32)]


def _lib():
    L = load_library()
    L.rwnmr_synth_spheres.restype = ctypes.c_int64
    L.rwnmr_pack_blocks.restype = ctypes.c_int64
    L.rwnmr_place_walkers.restype = ctypes.c_int
    L.rwnmr_png_solid_mask.restype = ctypes.c_int64
    return L


def _p(a):
    return None if a is None else a.ctypes.data_as(_vp)


def synth_spheres(shape, rmin: float, rmax: float, porosity: float, n_phases: int = 1, seed: int = 1):
    """Overlapping-sphere image [nz][ny][nx] (uint8 labels, 0 = pore). Returns (labels, porosity)."""
    nz, ny, nx = shape
    labels = np.zeros((nz, ny, nx), np.uint8)
    por = ctypes.c_double(0.0)
    n = _lib().rwnmr_synth_spheres(_p(labels), nx, ny, nz, ctypes.c_double(rmin), ctypes.c_double(rmax),
                                   ctypes.c_double(porosity), int(n_phases), ctypes.c_uint64(seed), ctypes.byref(por))
    if n < 0:
        raise ValueError("invalid sphere-pack parameters")
    return labels, por.value


def pack_blocks(labels: np.ndarray):
    """Bit-blocks of a label volume; returns (blocks uint64, (bcols, brows, bdepth))."""
    labels = np.ascontiguousarray(labels, dtype=np.uint8)
    nz, ny, nx = labels.shape
    dims = np.zeros(3, np.int32)
    L = _lib()
    nb = L.rwnmr_pack_blocks(None, nx, ny, nz, None, _p(dims))
    blocks = np.zeros(nb, np.uint64)
    L.rwnmr_pack_blocks(_p(labels), nx, ny, nz, _p(blocks), _p(dims))
    return blocks, tuple(int(d) for d in dims)


def place_walkers(blocks: np.ndarray, shape, n: int, seed: int, mode: str = "random", deviation: int = 0,
                  shift: int = 0):
    """Walker initial state as NMR_Simulation::setWalkers creates it: (x0, y0, z0, seed0, info)."""
    blocks = np.ascontiguousarray(blocks, dtype=np.uint64)
    nz, ny, nx = shape
    x0, y0, z0 = (np.zeros(n, np.int32) for _ in range(3))
    s0 = np.zeros(n, np.uint64)
    info = PlacementInfo()
    rc = _lib().rwnmr_place_walkers(_p(blocks), nx, ny, nz, mode.encode(), int(deviation), int(shift),
                                    ctypes.c_uint64(seed), ctypes.c_int64(n), _p(x0), _p(y0), _p(z0), _p(s0),
                                    ctypes.byref(info))
    if rc != 0:
        raise ValueError(f"walker placement failed (rc={rc})")
    return x0, y0, z0, s0, dict(pores=info.pores, porosity=info.porosity, occupancy=info.occupancy,
                                clamped=info.clamped)


def png_mask(path: str) -> np.ndarray:
    """Solid mask [height][width] of one PNG slice (1 = solid)."""
    L = _lib()
    w, h = ctypes.c_int32(), ctypes.c_int32()
    err = ctypes.create_string_buffer(512)
    n = L.rwnmr_png_solid_mask(path.encode(), ctypes.byref(w), ctypes.byref(h), None, err, len(err))
    if n < 0:
        raise ValueError(err.value.decode())
    out = np.zeros((h.value, w.value), np.uint8)
    L.rwnmr_png_solid_mask(path.encode(), None, None, _p(out), err, len(err))
    return out


def cli(args, cwd=None) -> int:
    """Runs the command-line driver in-process (argv without the program name)."""
    import os

    L = _lib()
    argv = [b"rwnmr_gb300"] + [str(a).encode() for a in args]
    arr = (ctypes.c_char_p * len(argv))(*argv)
    old = os.getcwd()
    try:
        if cwd:
            os.chdir(cwd)
        return int(L.rwnmr_cli_main(len(argv), arr))
    finally:
        os.chdir(old)
