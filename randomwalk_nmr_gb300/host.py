"""Bindings of the host frontend C ABI (include/rwnmr_host.h): synthetic images, bit-block
packing and walker placement. These run on the CPU and need no GPU."""
from __future__ import annotations

import ctypes

import numpy as np

from .engine import load_library

_vp = ctypes.c_void_p

HOST_EXPORTS = ["rwnmr_synth_spheres", "rwnmr_pack_blocks", "rwnmr_place_walkers", "rwnmr_png_solid_mask",
                "rwnmr_config_json", "rwnmr_cli_main", "rwnmr_t2_invert", "rwnmr_t2_prune", "rwnmr_t2_lcurve",
                "rwnmr_nnls"]


class T2Config(ctypes.Structure):
    """rwnmr_t2_config: the cpmg config's Laplace-inversion keys."""
    _fields_ = [("min_t2", ctypes.c_double), ("max_t2", ctypes.c_double), ("use_logspace", ctypes.c_int32),
                ("num_t2_bins", ctypes.c_int32), ("min_lambda", ctypes.c_double), ("max_lambda", ctypes.c_double),
                ("num_lambdas", ctypes.c_int32), ("prune_num", ctypes.c_int32), ("noise_amp", ctypes.c_double),
                ("noise_seed", ctypes.c_uint64)]


class PlacementInfo(ctypes.Structure):
    _fields_ = [("pores", ctypes.c_uint32), ("porosity", ctypes.c_double), ("occupancy", ctypes.c_double),
                ("clamped", ctypes.c_uint32)]


def _lib():
    L = load_library()
    L.rwnmr_synth_spheres.restype = ctypes.c_int64
    L.rwnmr_pack_blocks.restype = ctypes.c_int64
    L.rwnmr_place_walkers.restype = ctypes.c_int
    L.rwnmr_png_solid_mask.restype = ctypes.c_int64
    for name in ("rwnmr_t2_invert", "rwnmr_t2_prune", "rwnmr_t2_lcurve", "rwnmr_nnls"):
        getattr(L, name).restype = ctypes.c_int32
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


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def invert_t2(times, amps, min_t2=0.1, max_t2=10000.0, use_logspace=True, num_t2_bins=128, min_lambda=-4.0,
              max_lambda=2.0, num_lambdas=512, prune_num=512, noise_amp=0.0, noise_seed=0):
    """T2 distribution of a decay whose first point is t = 0 (rwnmr_t2_invert; the defaults are the
    reference's cpmg.config). Returns (bins, amps, lambda, noise per decay point)."""
    t, a = _f64(times), _f64(amps)
    if t.shape != a.shape or t.ndim != 1:
        raise ValueError("times and amps must be 1-D of equal length")
    cfg = T2Config(min_t2, max_t2, int(bool(use_logspace)), num_t2_bins, min_lambda, max_lambda, num_lambdas,
                   prune_num, noise_amp, noise_seed)
    bins = np.zeros(max(num_t2_bins, 0))
    out = np.zeros_like(bins)
    noise = np.zeros_like(t)
    lam = ctypes.c_double(0.0)
    err = ctypes.create_string_buffer(512)
    n = _lib().rwnmr_t2_invert(_p(t), _p(a), len(t), ctypes.byref(cfg), _p(bins), _p(out), ctypes.byref(lam),
                               _p(noise), err, 512)
    if n < 0:
        raise ValueError(err.value.decode())
    return bins, out, lam.value, noise


def prune_decay(times, amps, prune_num: int):
    """Prune-averaged (times, amps) of a decay (without its t = 0 point), or None when the decay is
    not longer than prune_num."""
    t, a = _f64(times), _f64(amps)
    ot, oa = np.zeros(max(prune_num, 0)), np.zeros(max(prune_num, 0))
    n = _lib().rwnmr_t2_prune(_p(t), _p(a), len(t), prune_num, _p(ot), _p(oa))
    if n < 0:
        raise ValueError("bad arguments")
    return None if n == 0 else (ot, oa)


def lcurve(A, b, min_lambda=-4.0, max_lambda=2.0, num_lambdas=512):
    """(best index, curvature per lambda, singular values) of the Tikhonov L-curve for kernel A."""
    A = np.asfortranarray(A, dtype=np.float64)
    m, n = A.shape
    curv = np.zeros(num_lambdas)
    sv = np.zeros(min(m, n))
    ns = ctypes.c_int32(0)
    best = _lib().rwnmr_t2_lcurve(A.ctypes.data_as(_vp), m, n, _p(_f64(b)), ctypes.c_double(min_lambda),
                                  ctypes.c_double(max_lambda), num_lambdas, _p(curv), _p(sv), ctypes.byref(ns))
    if best < 0:
        raise ValueError("bad arguments")
    return best, curv, sv[:ns.value]


def nnls(A, b, max_solves: int = 0):
    """x >= 0 minimising ||A x - b|| (rwnmr_nnls). Returns (x, least-squares solves)."""
    A = np.asfortranarray(A, dtype=np.float64)
    m, n = A.shape
    x = np.zeros(n)
    r = _lib().rwnmr_nnls(A.ctypes.data_as(_vp), m, n, _p(_f64(b)), _p(x), max_solves)
    if r < 0:
        raise ValueError("NNLS failed (bad arguments or no convergence)")
    return x, r
