"""Python binding of the GB300 walker engine's C ABI (include/rwnmr_gb300.h).

The engine is the CUDA library ``_build/librwnmr_gb300.so``. There is no CPU fallback: if the
library is missing or no CUDA device is usable, constructing an :class:`Engine` raises.
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

from . import build as _build

_vp = ctypes.c_void_p
_LOCK = threading.Lock()
_LIB = None

BC = {"noflux": 0, "periodic": 1, "mirror": 2}

STATUS = {
    0: "RWNMR_OK",
    1: "RWNMR_ERR_INVALID",
    2: "RWNMR_ERR_CUDA",
    3: "RWNMR_ERR_NOMEM",
    4: "RWNMR_ERR_STATE",
    5: "RWNMR_ERR_UNSUPPORTED",
    6: "RWNMR_ERR_DEVICE",
    7: "RWNMR_ERR_CANCELLED",
    8: "RWNMR_ERR_TIMEOUT",
}

# Every function the C header declares, for load checks.
EXPORTS = [
    "rwnmr_ctx_create", "rwnmr_ctx_destroy", "rwnmr_last_error", "rwnmr_version", "rwnmr_ctx_set_stream",
    "rwnmr_ctx_launch_count", "rwnmr_ctx_last_kernel_ms", "rwnmr_image_upload", "rwnmr_image_upload_labels",
    "rwnmr_image_download_blocks", "rwnmr_image_layout", "rwnmr_ctx_set_image_layout", "rwnmr_walkers_upload", "rwnmr_walkers_download", "rwnmr_cpmg_run",
    "rwnmr_cpmg_run_sens", "rwnmr_cpmg_adjoint", "rwnmr_map_run", "rwnmr_map_continue", "rwnmr_pfgse_run", "rwnmr_pfgse_grad_g",
    "rwnmr_cpmg_run_noalloc", "rwnmr_batch_create", "rwnmr_batch_destroy", "rwnmr_batch_last_error",
    "rwnmr_batch_cancel", "rwnmr_batch_set_time_budget", "rwnmr_set_device_allocator", "rwnmr_walkers_restore",
    "rwnmr_batch_last_kernel_ms", "rwnmr_batch_launch_count", "rwnmr_batch_add_image", "rwnmr_batch_cpmg",
    "rwnmr_batch_autotune", "rwnmr_batch_collision_histogram", "rwnmr_batch_histogram_walk_ms",
    "rwnmr_field_set_uniform", "rwnmr_field_upload", "rwnmr_field_clear",
    "rwnmr_cpmg_field_run", "rwnmr_walkers_set_dfactor",
]


class RwnmrError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


class CpmgParams(ctypes.Structure):
    _fields_ = [
        ("bc", ctypes.c_int32), ("shift", ctypes.c_int32), ("steps_per_echo", ctypes.c_int32),
        ("n_echoes", ctypes.c_int32), ("dfactor", ctypes.POINTER(ctypes.c_double)),
        ("echoes_per_launch", ctypes.c_int32),
    ]


class FieldCpmgParams(ctypes.Structure):
    _fields_ = [
        ("bc", ctypes.c_int32), ("shift", ctypes.c_int32), ("steps_per_echo", ctypes.c_int32),
        ("n_echoes", ctypes.c_int32), ("dfactor", ctypes.POINTER(ctypes.c_double)), ("gamma", ctypes.c_double),
        ("time_interval", ctypes.c_double), ("echoes_per_launch", ctypes.c_int32),
    ]


class PfgseParams(ctypes.Structure):
    _fields_ = [
        ("bc", ctypes.c_int32), ("shift", ctypes.c_int32), ("n_delta", ctypes.c_int32),
        ("steps", ctypes.POINTER(ctypes.c_int32)), ("n_g", ctypes.c_int32),
        ("kvec", ctypes.POINTER(ctypes.c_double)), ("res", ctypes.c_double),
        ("dfactor", ctypes.POINTER(ctypes.c_double)),
    ]


def library_path() -> str:
    return _build.LIB


_ALLOC_FN = ctypes.CFUNCTYPE(ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p)
_FREE_FN = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_void_p)
_ALLOC_KEEP = []  # every callback pair ever installed: buffers are freed by the allocator that made them


def set_device_allocator(alloc=None, free=None):
    """Route the engine contexts' device allocations through alloc(nbytes) -> device pointer (int;
    0 when it cannot allocate, which the calls report as RWNMR_ERR_NOMEM) and free(pointer).
    Both None restores cudaMalloc / cudaFree. Affects allocations made after the call."""
    lib = load_library()
    if alloc is None and free is None:
        st = lib.rwnmr_set_device_allocator(None, None, None)
    elif alloc is None or free is None:
        raise ValueError("give both alloc and free, or neither")
    else:
        a = _ALLOC_FN(lambda n, user: alloc(int(n)) or None)
        f = _FREE_FN(lambda ptr, user: free(int(ptr)))
        _ALLOC_KEEP.append((a, f))
        st = lib.rwnmr_set_device_allocator(a, f, None)
    if st != 0:
        raise RwnmrError(st, "rwnmr_set_device_allocator")


def use_torch_allocator(device: int = 0):
    """Allocate the engine contexts' device buffers from PyTorch's caching allocator."""
    import torch

    set_device_allocator(lambda n: torch.cuda.caching_allocator_alloc(n, device),
                         lambda ptr: torch.cuda.caching_allocator_delete(ptr))


def load_library(build_if_missing: bool = True) -> ctypes.CDLL:
    """Loads the engine library (building it first if asked and absent)."""
    global _LIB
    with _LOCK:
        if _LIB is not None:
            return _LIB
        path = _build.LIB
        if not os.path.exists(path):
            if not build_if_missing:
                raise FileNotFoundError(f"rwnmr_gb300 engine library not built: {path}")
            _build.build()
        lib = ctypes.CDLL(path)
        lib.rwnmr_last_error.restype = ctypes.c_char_p
        lib.rwnmr_last_error.argtypes = [_vp]
        lib.rwnmr_version.restype = ctypes.c_char_p
        lib.rwnmr_ctx_launch_count.restype = ctypes.c_int64
        lib.rwnmr_ctx_launch_count.argtypes = [_vp]
        lib.rwnmr_ctx_last_kernel_ms.restype = ctypes.c_double
        lib.rwnmr_ctx_last_kernel_ms.argtypes = [_vp]
        lib.rwnmr_ctx_destroy.argtypes = [_vp]
        lib.rwnmr_batch_last_error.restype = ctypes.c_char_p
        lib.rwnmr_batch_last_error.argtypes = [_vp]
        lib.rwnmr_batch_last_kernel_ms.restype = ctypes.c_double
        lib.rwnmr_batch_last_kernel_ms.argtypes = [_vp]
        lib.rwnmr_batch_launch_count.restype = ctypes.c_int64
        lib.rwnmr_batch_launch_count.argtypes = [_vp]
        lib.rwnmr_batch_histogram_walk_ms.restype = ctypes.c_double
        lib.rwnmr_batch_histogram_walk_ms.argtypes = [_vp]
        lib.rwnmr_batch_destroy.argtypes = [_vp]
        for name in EXPORTS:
            getattr(lib, name)  # raises AttributeError if a declared symbol is missing
        _LIB = lib
        return lib


def _p(a):
    return None if a is None else a.ctypes.data_as(_vp)


def _dptr(a):
    if a is None:
        return ctypes.POINTER(ctypes.c_double)()
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class Engine:
    """One rwnmr_ctx: an image, a walker population and the walks over them on one GPU."""

    def __init__(self, device: int = 0):
        self.lib = load_library()
        ctx = _vp()
        st = self.lib.rwnmr_ctx_create(ctypes.byref(ctx), int(device))
        if st != 0:
            raise RwnmrError(st, f"could not create a CUDA context on device {device}")
        self.ctx = ctx
        self.n_phases = 1
        self.shape = None
        self.n = 0

    def close(self):
        if getattr(self, "ctx", None):
            self.lib.rwnmr_ctx_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st: int):
        if st != 0:
            msg = self.lib.rwnmr_last_error(self.ctx)
            raise RwnmrError(st, msg.decode() if msg else "")

    @property
    def launch_count(self) -> int:
        return int(self.lib.rwnmr_ctx_launch_count(self.ctx))

    @property
    def last_kernel_ms(self) -> float:
        return float(self.lib.rwnmr_ctx_last_kernel_ms(self.ctx))

    @property
    def morton_layout(self) -> bool:
        """True if the uploaded image has the Morton copy the noflux walks use."""
        return bool(self.lib.rwnmr_image_layout(self.ctx))

    def allow_morton(self, allow: bool = True):
        """Whether later image uploads build the Morton copy (default True)."""
        self._check(self.lib.rwnmr_ctx_set_image_layout(self.ctx, int(bool(allow))))

    def set_stream(self, stream_ptr: int | None):
        self._check(self.lib.rwnmr_ctx_set_stream(self.ctx, _vp(stream_ptr or 0)))

    # -- image ------------------------------------------------------------------------------
    def upload_labels(self, labels: np.ndarray, n_phases: int | None = None):
        labels = np.ascontiguousarray(labels, dtype=np.uint8)
        nz, ny, nx = labels.shape
        if n_phases is None:
            n_phases = max(1, int(labels.max()))
        self._check(self.lib.rwnmr_image_upload_labels(self.ctx, _p(labels), nx, ny, nz, int(n_phases)))
        self.n_phases = int(n_phases)
        self.shape = (nz, ny, nx)

    def upload_blocks(self, blocks: np.ndarray, shape, labels: np.ndarray | None = None, n_phases: int = 1):
        blocks = np.ascontiguousarray(blocks, dtype=np.uint64)
        nz, ny, nx = shape
        lab = None if labels is None else np.ascontiguousarray(labels, dtype=np.uint8)
        self._check(self.lib.rwnmr_image_upload(self.ctx, _p(blocks), nx, ny, nz, _p(lab), int(n_phases)))
        self.n_phases = int(n_phases)
        self.shape = (nz, ny, nx)

    def download_blocks(self) -> np.ndarray:
        nz, ny, nx = self.shape
        nb = ((nx + 3) // 4) * ((ny + 3) // 4) * ((nz + 3) // 4)
        out = np.zeros(nb, np.uint64)
        self._check(self.lib.rwnmr_image_download_blocks(self.ctx, _p(out)))
        return out

    # -- walkers ----------------------------------------------------------------------------
    def upload_walkers(self, x0, y0, z0, seed0):
        arrs = [np.ascontiguousarray(a, dtype=t) for a, t in
                ((x0, np.int32), (y0, np.int32), (z0, np.int32), (seed0, np.uint64))]
        n = len(arrs[0])
        if any(len(a) != n for a in arrs):
            raise ValueError("walker arrays differ in length")
        self._check(self.lib.rwnmr_walkers_upload(self.ctx, ctypes.c_int64(n), *[_p(a) for a in arrs]))
        self.n = n

    def download_walkers(self):
        n, P = self.n, self.n_phases
        x, y, z = (np.zeros(n, np.int32) for _ in range(3))
        s = np.zeros(n, np.uint64)
        c = np.zeros((n, P), np.uint32)
        self._check(self.lib.rwnmr_walkers_download(self.ctx, _p(x), _p(y), _p(z), _p(s), _p(c)))
        return dict(x=x, y=y, z=z, seed=s, collisions=c)

    def restore_walkers(self, state):
        """Checkpoint / resume: set the current walker state from a download_walkers() dict."""
        x, y, z = (np.ascontiguousarray(state[k], np.int32) for k in ("x", "y", "z"))
        s = np.ascontiguousarray(state["seed"], np.uint64)
        c = np.ascontiguousarray(state["collisions"], np.uint32).reshape(self.n, self.n_phases)
        self._check(self.lib.rwnmr_walkers_restore(self.ctx, _p(x), _p(y), _p(z), _p(s), _p(c)))

    def set_walker_dfactor(self, dfactor):
        """Per-walker decrease factors (single-phase images); walks called with dfactor=None use them."""
        f = np.ascontiguousarray(dfactor, np.float64)
        if f.shape != (self.n,):
            raise ValueError("one decrease factor per walker")
        self._check(self.lib.rwnmr_walkers_set_dfactor(self.ctx, _p(f)))

    def _dfactor(self, dfactor):
        if dfactor is None:
            return None
        return np.ascontiguousarray(np.broadcast_to(np.asarray(dfactor, np.float64), (self.n_phases,)))

    # -- walks ------------------------------------------------------------------------------
    def cpmg(self, n_echoes: int, steps_per_echo: int, dfactor, bc: str = "noflux", shift: int = 0,
             echoes_per_launch: int = 0):
        df = self._dfactor(dfactor)
        prm = CpmgParams(BC[bc], int(shift), int(steps_per_echo), int(n_echoes), _dptr(df), int(echoes_per_launch))
        echo_sum = np.zeros(n_echoes + 1)
        echo_fx = np.zeros((n_echoes + 1, 3), np.uint64)
        echo_coll = np.zeros((n_echoes, self.n_phases), np.uint64)
        self._check(self.lib.rwnmr_cpmg_run(self.ctx, ctypes.byref(prm), _p(echo_sum), _p(echo_fx), _p(echo_coll)))
        return dict(echo_sum=echo_sum, echo_fx=echo_fx, echo_coll=echo_coll)

    def cpmg_sens(self, n_echoes: int, steps_per_echo: int, dfactor, bc: str = "noflux", shift: int = 0,
                  echoes_per_launch: int = 0):
        """The CPMG walk with forward sensitivities: echo_sum as cpmg(), sens [n_echoes+1][n_phases] =
        sum over walkers of E * c_q (d echo_sum / d dfactor_q = sens / dfactor_q), and sens_fx, the same
        sums as exact Python ints in units of 2^-63."""
        df = self._dfactor(dfactor)
        if df is None:
            raise ValueError("sensitivities are for per-phase decrease factors")
        prm = CpmgParams(BC[bc], int(shift), int(steps_per_echo), int(n_echoes), _dptr(df), int(echoes_per_launch))
        echo_sum = np.zeros(n_echoes + 1)
        sens = np.zeros((n_echoes + 1, self.n_phases))
        limbs = np.zeros((n_echoes + 1, self.n_phases, 4), np.uint64)
        self._check(self.lib.rwnmr_cpmg_run_sens(self.ctx, ctypes.byref(prm), _p(echo_sum), _p(sens), _p(limbs)))
        sens_fx = [[sum(int(v) << (24 * k) for k, v in enumerate(row)) for row in e] for e in limbs]
        return dict(echo_sum=echo_sum, sens=sens, sens_fx=sens_fx)

    def cpmg_adjoint(self, n_echoes: int, steps_per_echo: int, dfactor, grad_echo, bc: str = "noflux",
                     shift: int = 0):
        df = self._dfactor(dfactor)
        prm = CpmgParams(BC[bc], int(shift), int(steps_per_echo), int(n_echoes), _dptr(df), 0)
        g = np.ascontiguousarray(grad_echo, np.float64)
        if g.shape != (n_echoes + 1,):
            raise ValueError("grad_echo must have n_echoes + 1 entries")
        out = np.zeros(self.n_phases)
        self._check(self.lib.rwnmr_cpmg_adjoint(self.ctx, ctypes.byref(prm), _p(g), _p(out)))
        return out

    # -- internal field ---------------------------------------------------------------------
    def set_field_uniform(self, gradient: float, direction: int, resolution: float):
        """RESIDUAL_FIELD: uniform -- B = coord * gradient * 1e-6 * resolution in pores, 0 in solid."""
        self._check(self.lib.rwnmr_field_set_uniform(self.ctx, ctypes.c_double(gradient), int(direction),
                                                     ctypes.c_double(resolution)))

    def upload_field(self, values: np.ndarray):
        """RESIDUAL_FIELD: import -- one value per image voxel, shape (nz, ny, nx)."""
        v = np.ascontiguousarray(values, np.float64)
        self._check(self.lib.rwnmr_field_upload(self.ctx, _p(v), ctypes.c_int64(v.size)))

    def clear_field(self):
        self._check(self.lib.rwnmr_field_clear(self.ctx))

    def cpmg_field(self, n_echoes: int, steps_per_echo: int, dfactor, gamma: float, time_interval: float,
                   bc: str = "noflux", shift: int = 0, echoes_per_launch: int = 0):
        """CPMG walk in the internal field; returns the echo energy sums, their exact fixed-point
        form (echo_fx: sum over walkers of E * 2^61 + 2^61, Python ints) and final walker phases."""
        df = self._dfactor(dfactor)
        prm = FieldCpmgParams(BC[bc], int(shift), int(steps_per_echo), int(n_echoes), _dptr(df), float(gamma),
                              float(time_interval), int(echoes_per_launch))
        echo_sum = np.zeros(n_echoes + 1)
        limbs = np.zeros((n_echoes + 1, 3), np.uint64)
        phase = np.zeros(self.n)
        self._check(self.lib.rwnmr_cpmg_field_run(self.ctx, ctypes.byref(prm), _p(echo_sum), _p(limbs), _p(phase)))
        echo_fx = [int(a) + (int(b) << 21) + (int(c) << 42) for a, b, c in limbs]
        return dict(echo_sum=echo_sum, echo_fx=echo_fx, phase=phase)

    def map(self, steps: int, bc: str = "noflux", shift: int = 0) -> np.ndarray:
        out = np.zeros(self.n, np.uint32)
        self._check(self.lib.rwnmr_map_run(self.ctx, BC[bc], int(shift), ctypes.c_int64(steps), _p(out)))
        return out

    def map_continue(self, steps: int, bc: str = "noflux", shift: int = 0) -> np.ndarray:
        out = np.zeros(self.n, np.uint32)
        self._check(self.lib.rwnmr_map_continue(self.ctx, BC[bc], int(shift), ctypes.c_int64(steps), _p(out)))
        return out

    def _pfgse_params(self, steps, kvec, res, dfactor, bc, shift):
        steps = np.ascontiguousarray(steps, np.int32)
        kvec = np.ascontiguousarray(kvec, np.float64).reshape(-1, 3)
        df = self._dfactor(dfactor)
        prm = PfgseParams(BC[bc], int(shift), len(steps), steps.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                          len(kvec), _dptr(kvec), float(res), _dptr(df))
        return prm, (steps, kvec, df)

    def pfgse(self, steps, kvec, res: float, dfactor, bc: str = "noflux", shift: int = 0):
        prm, keep = self._pfgse_params(steps, kvec, res, dfactor, bc, shift)
        nd, ng = prm.n_delta, prm.n_g
        M = np.zeros((nd, ng))
        esum = np.zeros(nd)
        msd = np.zeros((nd, 3), np.uint64)
        self._check(self.lib.rwnmr_pfgse_run(self.ctx, ctypes.byref(prm), _p(M), _p(esum), _p(msd)))
        return dict(M=M, esum=esum, msd=msd)

    def pfgse_grad_g(self, steps, kvec, res: float, dfactor, kscale: float, direction, bc="noflux", shift=0):
        prm, keep = self._pfgse_params(steps, kvec, res, dfactor, bc, shift)
        d = np.ascontiguousarray(direction, np.float64)
        out = np.zeros((prm.n_delta, prm.n_g))
        self._check(self.lib.rwnmr_pfgse_grad_g(self.ctx, ctypes.byref(prm), ctypes.c_double(kscale), _p(d), _p(out)))
        return out


class BatchParams(ctypes.Structure):
    _fields_ = [("bc", ctypes.c_int32), ("steps_per_echo", ctypes.c_int32), ("n_echoes", ctypes.c_int32),
                ("n_candidates", ctypes.c_int32), ("derivatives", ctypes.c_int32),
                ("threads_per_block", ctypes.c_int32), ("use_graph", ctypes.c_int32),
                ("walkers_per_thread", ctypes.c_int32), ("method", ctypes.c_int32)]


BATCH_METHOD = {"auto": 0, "histograms": 1, "walk": 2}


class Batch:
    """Many images, each with its walkers and up to 16 relaxivity candidates, walked by one
    persistent launch (rwnmr_batch_*)."""

    def __init__(self, device: int = 0):
        self.lib = load_library()
        b = _vp()
        st = self.lib.rwnmr_batch_create(ctypes.byref(b), int(device))
        if st != 0:
            raise RwnmrError(st, f"could not create a batch on device {device}")
        self.b = b
        self.n_images = 0

    def close(self):
        if getattr(self, "b", None):
            self.lib.rwnmr_batch_destroy(self.b)
            self.b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st):
        if st != 0:
            raise RwnmrError(st, self.lib.rwnmr_batch_last_error(self.b).decode())

    def cancel(self):
        """Stop the batch walk in flight (or the next one): it raises RWNMR_ERR_CANCELLED. Callable from
        another thread while a batch call runs."""
        self._check(self.lib.rwnmr_batch_cancel(self.b))

    def set_time_budget(self, seconds: float):
        """Bound each persistent batch walk to about `seconds` (0: no bound); a walk that runs out
        raises RWNMR_ERR_TIMEOUT."""
        self._check(self.lib.rwnmr_batch_set_time_budget(self.b, ctypes.c_double(seconds)))

    def add_image(self, blocks, shape, x0, y0, z0, seed0) -> int:
        blocks = np.ascontiguousarray(blocks, np.uint64)
        nz, ny, nx = shape
        arrs = [np.ascontiguousarray(a, t) for a, t in ((x0, np.int32), (y0, np.int32), (z0, np.int32),
                                                          (seed0, np.uint64))]
        idx = ctypes.c_int32()
        self._check(self.lib.rwnmr_batch_add_image(self.b, _p(blocks), nx, ny, nz, ctypes.c_int64(len(arrs[0])),
                                                   *[_p(a) for a in arrs], ctypes.byref(idx)))
        self.n_images += 1
        return idx.value

    def cpmg(self, dfactor, n_echoes: int, steps_per_echo: int, derivatives: bool = True, bc: str = "noflux",
             threads_per_block: int = 0, use_graph: bool = True, walkers_per_thread: int = 0, method: str = "auto"):
        """Echo sums [image][candidate][echo] (and derivatives) for dfactor [image][candidate].
        method "histograms" walks once per (n_echoes, steps_per_echo, bc) and evaluates every later
        call from the stored per-echo collision histograms; "walk" walks on every call; "auto" picks
        histograms when they fit in half the free device memory. Both give identical sums."""
        f = np.ascontiguousarray(dfactor, np.float64)
        if f.ndim == 1:
            f = f[:, None]
        R = f.shape[1]
        prm = BatchParams(BC[bc], int(steps_per_echo), int(n_echoes), R, int(bool(derivatives)),
                          int(threads_per_block), int(bool(use_graph)), int(walkers_per_thread), BATCH_METHOD[method])
        echo = np.zeros((self.n_images, R, n_echoes + 1))
        decho = np.zeros_like(echo) if derivatives else None
        self._check(self.lib.rwnmr_batch_cpmg(self.b, ctypes.byref(prm), _p(f), _p(echo), _p(decho)))
        return echo, decho

    def autotune(self, n_echoes: int, steps_per_echo: int, n_candidates: int = 16, derivatives: bool = True,
                 bc: str = "noflux", method: str = "auto"):
        prm = BatchParams(BC[bc], int(steps_per_echo), int(n_echoes), int(n_candidates), int(bool(derivatives)), 0, 0, 0,
                          BATCH_METHOD[method])
        t = ctypes.c_int32()
        wpt = ctypes.c_int32()
        ms = ctypes.c_double()
        self._check(self.lib.rwnmr_batch_autotune(self.b, ctypes.byref(prm), ctypes.byref(t), ctypes.byref(wpt),
                                                  ctypes.byref(ms)))
        return t.value, wpt.value, ms.value

    @property
    def last_kernel_ms(self) -> float:
        return float(self.lib.rwnmr_batch_last_kernel_ms(self.b))

    @property
    def launch_count(self) -> int:
        return int(self.lib.rwnmr_batch_launch_count(self.b))

    @property
    def histogram_walk_ms(self) -> float:
        return float(self.lib.rwnmr_batch_histogram_walk_ms(self.b))

    def collision_histogram(self, image: int, echo: int) -> np.ndarray:
        """Walkers of `image` per collision count after `echo` (from the last histogram walk)."""
        n = ctypes.c_int32()
        self._check(self.lib.rwnmr_batch_collision_histogram(self.b, int(image), int(echo), None, ctypes.byref(n)))
        out = np.zeros(n.value, np.uint32)
        self._check(self.lib.rwnmr_batch_collision_histogram(self.b, int(image), int(echo), _p(out), ctypes.byref(n)))
        return out


def fx_to_float(limbs) -> np.ndarray:
    """Exact fixed-point limb sums ([..., 3], scale 2^63) to float64."""
    limbs = np.asarray(limbs, dtype=np.uint64)
    flat = limbs.reshape(-1, 3)
    vals = [(int(a) + (int(b) << 21) + (int(c) << 42)) / float(1 << 63) for a, b, c in flat]
    return np.array(vals).reshape(limbs.shape[:-1])
