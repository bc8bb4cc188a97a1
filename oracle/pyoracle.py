"""ctypes bindings for the test oracle -- TEST INFRASTRUCTURE ONLY.

Two libraries are wrapped:

* ``_build/librwnmr_oracle.so`` -- the CPU restatement of the walker path (rwnmr_oracle.cpp);
* ``_ref/librwnmr_ref.so`` -- the reference's own CPU code built from its sources by this
  directory's Makefile (available only where the reference sources exist).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU baseline / reference legs import this
module. The product package never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import tempfile
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "librwnmr_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "librwnmr_ref.so")
# Root of a RandomWalk_NMR checkout, given by the caller (build recipe or fixture script) through
# the environment; without it only the restatement is built.
REF_ENV = "RWNMR_REFERENCE"

BC = {"noflux": 0, "periodic": 1, "mirror": 2}

_vp = ctypes.c_void_p


def _ptr(a):
    return None if a is None else a.ctypes.data_as(_vp)


def ref_source_dir(ref_root: str | None = None) -> str | None:
    """The reference's backend source directory under ``ref_root`` (default: $RWNMR_REFERENCE),
    or None when no checkout is given or it is absent."""
    root = ref_root if ref_root is not None else os.environ.get(REF_ENV)
    if not root:
        return None
    src = os.path.join(root, "src", "backend")
    return src if os.path.isdir(src) else None


def build(with_ref: bool | None = None, ref_root: str | None = None) -> None:
    """Builds the restatement, and the reference library when a reference checkout is given
    (``ref_root`` or $RWNMR_REFERENCE) and present."""
    src = ref_source_dir(ref_root)
    if with_ref is None:
        with_ref = src is not None
    if with_ref and src is None:
        raise FileNotFoundError("reference sources not found: set %s to a RandomWalk_NMR checkout" % REF_ENV)
    cmd = ["make", "-s", "-C", HERE, "ref" if with_ref else "all", "-j8"]
    if with_ref:
        cmd.append("REF_SRC=" + src)
    subprocess.run(cmd, check=True)


class OrcImage(ctypes.Structure):
    _fields_ = [
        ("blocks", _vp),
        ("labels", _vp),
        ("nx", ctypes.c_int32),
        ("ny", ctypes.c_int32),
        ("nz", ctypes.c_int32),
        ("bcols", ctypes.c_int32),
        ("brows", ctypes.c_int32),
        ("bdepth", ctypes.c_int32),
        ("n_phases", ctypes.c_int32),
    ]


class Oracle:
    """CPU restatement of the reference walker path."""

    def __init__(self, path: str = ORACLE_SO):
        if not os.path.exists(path):
            build(with_ref=False)
        self.lib = ctypes.CDLL(path)
        L = self.lib
        L.orc_pack_blocks.restype = ctypes.c_int64
        L.orc_xorshift64.restype = ctypes.c_uint64
        L.orc_xorshift64.argtypes = [ctypes.c_uint64]
        L.orc_mod6.restype = ctypes.c_uint32
        L.orc_mod6.argtypes = [ctypes.c_uint64]

    # -- image ------------------------------------------------------------------------------
    def pack_blocks(self, labels: np.ndarray):
        labels = np.ascontiguousarray(labels, dtype=np.uint8)
        nz, ny, nx = labels.shape
        dims = np.zeros(3, np.int32)
        nb = self.lib.orc_pack_blocks(_ptr(labels), nx, ny, nz, None, _ptr(dims))
        blocks = np.zeros(nb, np.uint64)
        self.lib.orc_pack_blocks(_ptr(labels), nx, ny, nz, _ptr(blocks), _ptr(dims))
        return blocks, dims

    def image(self, labels: np.ndarray, n_phases: int | None = None):
        """Returns (OrcImage, keepalive) for a label volume [nz][ny][nx]. The packed blocks of the
        last volume are reused while its contents (CRC-32) are unchanged, so repeated walks over one
        large image are not timed with its packing."""
        labels = np.ascontiguousarray(labels, dtype=np.uint8)
        key = (labels.shape, zlib.crc32(labels))
        cache = getattr(self, "_packed", None)
        if cache is not None and cache[0] == key:
            blocks, dims = cache[1]
        else:
            blocks, dims = self.pack_blocks(labels)
            self._packed = (key, (blocks, dims))
        nz, ny, nx = labels.shape
        if n_phases is None:
            n_phases = max(1, int(labels.max()))
        lab = labels if n_phases > 1 else None
        im = OrcImage(blocks.ctypes.data, None if lab is None else lab.ctypes.data, nx, ny, nz,
                      int(dims[0]), int(dims[1]), int(dims[2]), n_phases)
        return im, (blocks, labels)

    def synth_spheres(self, shape, rmin, rmax, porosity, n_phases=1, seed=1):
        """The benchmark's sphere-pack labels [nz][ny][nx] (0 = pore); returns (labels, porosity)."""
        nz, ny, nx = shape
        lab = np.zeros((nz, ny, nx), np.uint8)
        por = ctypes.c_double(0.0)
        self.lib.orc_synth_spheres.restype = ctypes.c_int64
        n = self.lib.orc_synth_spheres(_ptr(lab), nx, ny, nz, ctypes.c_double(rmin), ctypes.c_double(rmax),
                                       ctypes.c_double(porosity), int(n_phases), ctypes.c_uint64(seed),
                                       ctypes.byref(por))
        if n < 0:
            raise ValueError("orc_synth_spheres rejected its arguments")
        return lab, por.value

    def place_walkers(self, labels, n, seed, shift=0):
        """The reference's random placement: (x0, y0, z0, seed0, clamped)."""
        labels = np.ascontiguousarray(labels, dtype=np.uint8)
        nz, ny, nx = labels.shape
        x, y, z = (np.zeros(n, np.int32) for _ in range(3))
        s = np.zeros(n, np.uint64)
        clamped = ctypes.c_int64(0)
        rc = self.lib.orc_place_walkers_random(_ptr(labels), nx, ny, nz, ctypes.c_uint64(seed), ctypes.c_int64(n),
                                               int(shift), _ptr(x), _ptr(y), _ptr(z), _ptr(s), ctypes.byref(clamped))
        if rc != 0:
            raise ValueError("orc_place_walkers_random failed (%d)" % rc)
        return x, y, z, s, clamped.value

    def energy_table(self, f: float, n_max: int):
        t = np.zeros(n_max + 1)
        fx = np.zeros(n_max + 1, np.uint64)
        self.lib.orc_energy_table(ctypes.c_double(f), n_max, _ptr(t), _ptr(fx))
        return t, fx

    # -- walks ------------------------------------------------------------------------------
    def cpmg(self, labels, walkers, n_echoes, steps_per_echo, dfactor, bc="noflux", shift=0, threads=1,
             n_phases=None):
        im, keep = self.image(labels, n_phases)
        x0, y0, z0, s0 = [np.ascontiguousarray(a) for a in walkers]
        n = len(x0)
        P = im.n_phases
        df = np.ascontiguousarray(np.broadcast_to(np.asarray(dfactor, np.float64), (P,)))
        out = dict(
            echo_fp64=np.zeros(n_echoes + 1),
            echo_fx=np.zeros((n_echoes + 1, 3), np.uint64),
            echo_coll=np.zeros((n_echoes, P), np.uint64),
            xf=np.zeros(n, np.int32), yf=np.zeros(n, np.int32), zf=np.zeros(n, np.int32),
            seedf=np.zeros(n, np.uint64), collf=np.zeros((n, P), np.uint32),
        )
        rc = self.lib.orc_cpmg(ctypes.byref(im), BC[bc], shift, ctypes.c_int64(n), _ptr(x0), _ptr(y0), _ptr(z0),
                               _ptr(s0), n_echoes, steps_per_echo, _ptr(df), _ptr(out["echo_fp64"]),
                               _ptr(out["echo_fx"]), _ptr(out["echo_coll"]), _ptr(out["xf"]), _ptr(out["yf"]),
                               _ptr(out["zf"]), _ptr(out["seedf"]), _ptr(out["collf"]), threads)
        if rc != 0:
            raise ValueError("orc_cpmg rejected its arguments")
        return out

    def uniform_field(self, labels, resolution, gradient, direction):
        im, keep = self.image(labels, 1)
        out = np.zeros(np.asarray(labels).shape, np.float64)
        self.lib.orc_uniform_field(ctypes.byref(im), ctypes.c_double(resolution), ctypes.c_double(gradient),
                                   int(direction), _ptr(out))
        return out

    def cpmg_field(self, labels, walkers, n_echoes, steps_per_echo, dfactor, gammatau, field=None, dg=0.0, axis=0,
                   bc="noflux", shift=0, threads=1, n_phases=None, walker_dfactor=None):
        """Internal-field CPMG walk; field is a [nz][ny][nx] array or None for the uniform field
        value = coord_axis * dg (0 in solid)."""
        im, keep = self.image(labels, n_phases)
        x0, y0, z0, s0 = [np.ascontiguousarray(a) for a in walkers]
        n = len(x0)
        P = im.n_phases
        df = None if dfactor is None else np.ascontiguousarray(np.broadcast_to(np.asarray(dfactor, np.float64), (P,)))
        wdf = None if walker_dfactor is None else np.ascontiguousarray(walker_dfactor, np.float64)
        fld = None if field is None else np.ascontiguousarray(field, np.float64)
        out = dict(
            echo_fp64=np.zeros(n_echoes + 1), echo_fx=np.zeros((n_echoes + 1, 3), np.uint64),
            xf=np.zeros(n, np.int32), yf=np.zeros(n, np.int32), zf=np.zeros(n, np.int32),
            seedf=np.zeros(n, np.uint64), collf=np.zeros((n, P), np.uint32), phasef=np.zeros(n),
        )
        rc = self.lib.orc_cpmg_field(ctypes.byref(im), BC[bc], shift, ctypes.c_int64(n), _ptr(x0), _ptr(y0),
                                     _ptr(z0), _ptr(s0), n_echoes, steps_per_echo,
                                     None if df is None else _ptr(df), None if wdf is None else _ptr(wdf),
                                     ctypes.c_double(gammatau), None if fld is None else _ptr(fld),
                                     ctypes.c_double(dg), axis, _ptr(out["echo_fp64"]), _ptr(out["echo_fx"]),
                                     _ptr(out["xf"]), _ptr(out["yf"]), _ptr(out["zf"]), _ptr(out["seedf"]),
                                     _ptr(out["collf"]), _ptr(out["phasef"]), threads)
        if rc != 0:
            raise ValueError("orc_cpmg_field rejected its arguments")
        return out

    def pfgse(self, labels, walkers, dfactor, steps, kvec, res, bc="noflux", shift=0, threads=1, n_phases=None):
        im, keep = self.image(labels, n_phases)
        x0, y0, z0, s0 = [np.ascontiguousarray(a) for a in walkers]
        n = len(x0)
        P = im.n_phases
        df = np.ascontiguousarray(np.broadcast_to(np.asarray(dfactor, np.float64), (P,)))
        steps = np.ascontiguousarray(steps, np.int32)
        kvec = np.ascontiguousarray(kvec, np.float64).reshape(-1, 3)
        nd, ng = len(steps), len(kvec)
        out = dict(M=np.zeros((nd, ng)), esum=np.zeros(nd), msd=np.zeros((nd, 3), np.uint64),
                   esum_fx=np.zeros((nd, 3), np.uint64))
        rc = self.lib.orc_pfgse(ctypes.byref(im), BC[bc], shift, ctypes.c_int64(n), _ptr(x0), _ptr(y0), _ptr(z0),
                                _ptr(s0), _ptr(df), nd, _ptr(steps), ng, _ptr(kvec), ctypes.c_double(res),
                                _ptr(out["M"]), _ptr(out["esum"]), _ptr(out["msd"]), _ptr(out["esum_fx"]), threads)
        if rc != 0:
            raise ValueError("orc_pfgse rejected its arguments")
        return out

    def pfgse_grad_g(self, labels, walkers, dfactor, steps, kvec, res, kscale, direction, bc="noflux", shift=0,
                     threads=1, n_phases=None):
        """FP64 pathwise dM/dg [n_delta][n_g] for k_j = kscale * g_j * direction (unit vector)."""
        im, keep = self.image(labels, n_phases)
        x0, y0, z0, s0 = [np.ascontiguousarray(a) for a in walkers]
        n = len(x0)
        P = im.n_phases
        df = np.ascontiguousarray(np.broadcast_to(np.asarray(dfactor, np.float64), (P,)))
        steps = np.ascontiguousarray(steps, np.int32)
        kvec = np.ascontiguousarray(kvec, np.float64).reshape(-1, 3)
        d = np.ascontiguousarray(direction, np.float64)
        nd, ng = len(steps), len(kvec)
        out = np.zeros((nd, ng))
        rc = self.lib.orc_pfgse_grad_g(ctypes.byref(im), BC[bc], shift, ctypes.c_int64(n), _ptr(x0), _ptr(y0),
                                       _ptr(z0), _ptr(s0), _ptr(df), nd, _ptr(steps), ng, _ptr(kvec),
                                       ctypes.c_double(res), ctypes.c_double(kscale), _ptr(d), _ptr(out), threads)
        if rc != 0:
            raise ValueError("orc_pfgse_grad_g rejected its arguments")
        return out

    def displacements(self, labels, walkers, steps, bc="noflux", shift=0, threads=1, n_phases=None):
        im, keep = self.image(labels, n_phases)
        x0, y0, z0, s0 = [np.ascontiguousarray(a) for a in walkers]
        n = len(x0)
        d = np.zeros((3, n), np.int32)
        coll = np.zeros((n, im.n_phases), np.uint32)
        rc = self.lib.orc_displacements(ctypes.byref(im), BC[bc], shift, ctypes.c_int64(n), _ptr(x0), _ptr(y0),
                                        _ptr(z0), _ptr(s0), steps, _ptr(d[0]), _ptr(d[1]), _ptr(d[2]), _ptr(coll),
                                        threads)
        if rc != 0:
            raise ValueError("orc_displacements rejected its arguments")
        return d, coll


def fx_to_float(limbs: np.ndarray) -> np.ndarray:
    """Converts [..., 3] fixed-point limb sums (scale 2^63) to float64 via exact integers."""
    limbs = np.asarray(limbs, dtype=np.uint64)
    flat = limbs.reshape(-1, 3)
    out = np.array([(int(a) + (int(b) << 21) + (int(c) << 42)) / float(1 << 63) for a, b, c in flat])
    return out.reshape(limbs.shape[:-1])


# -------------------------------------------------------------------------------------------------
class RefSimParams(ctypes.Structure):
    _fields_ = [
        ("walkers", ctypes.c_int32), ("seed", ctypes.c_uint64), ("placement", ctypes.c_char_p),
        ("deviation", ctypes.c_int32), ("rho_type", ctypes.c_char_p), ("rho", ctypes.POINTER(ctypes.c_double)),
        ("n_rho", ctypes.c_int32), ("d0", ctypes.c_double), ("bulk_time", ctypes.c_double),
        ("steps_per_echo", ctypes.c_int32), ("bc", ctypes.c_char_p), ("resolution", ctypes.c_double),
        ("voxel_division", ctypes.c_int32), ("gamma", ctypes.c_double), ("gamma_unit", ctypes.c_char_p),
        ("histograms", ctypes.c_int32), ("histogram_size", ctypes.c_int32), ("histogram_scale", ctypes.c_char_p),
    ]


def ref_available() -> bool:
    return os.path.exists(REF_SO)


class RefSim:
    """The reference's own NMR_Simulation (CPU) over a voxel image, via oracle/ref_driver.cpp."""

    _lib = None

    @classmethod
    def lib(cls):
        if cls._lib is None:
            if not os.path.exists(REF_SO):
                raise FileNotFoundError("reference oracle library not built (oracle/_ref)")
            L = ctypes.CDLL(REF_SO)
            L.ref_sim_create.restype = _vp
            L.ref_pfgse.restype = ctypes.c_int
            L.ref_cpmg.restype = ctypes.c_int
            L.ref_bitblock.restype = ctypes.c_int
            cls._lib = L
        return cls._lib

    def __init__(self, labels, walkers, seed, rho=(0.0,), d0=2.5, bulk_time=2800.0, steps_per_echo=1,
                 bc="noflux", resolution=1.0, voxel_division=0, placement="random", deviation=0,
                 rho_type="uniform", gamma=42.576, gamma_unit="mhertz", histograms=1, histogram_size=1024,
                 histogram_scale="linear"):
        L = self.lib()
        self.labels = np.ascontiguousarray(labels, dtype=np.uint8)
        nz, ny, nx = self.labels.shape
        self._rho = (ctypes.c_double * len(rho))(*rho)
        p = RefSimParams(int(walkers), int(seed), placement.encode(), int(deviation), rho_type.encode(), self._rho,
                         len(rho), float(d0), float(bulk_time), int(steps_per_echo), bc.encode(), float(resolution),
                         int(voxel_division), float(gamma), gamma_unit.encode(), int(histograms), int(histogram_size),
                         histogram_scale.encode())
        self.workdir = tempfile.mkdtemp(prefix="rwnmr_ref_")
        self.h = L.ref_sim_create(self.workdir.encode(), _ptr(self.labels), nx, ny, nz, ctypes.byref(p))
        info = np.zeros(12, np.int64)
        infod = np.zeros(5)
        L.ref_sim_info(_vp(self.h), _ptr(info), _ptr(infod))
        keys = ["pores", "interface", "bcols", "brows", "bdepth", "nblocks", "nx", "ny", "nz", "walkers",
                "voxel_division", "steps_per_echo"]
        self.info = {k: int(v) for k, v in zip(keys, info)}
        self.info.update(dict(zip(["porosity", "svp", "dt", "voxel_res", "gamma"], map(float, infod))))

    def __del__(self):
        try:
            self.lib().ref_sim_destroy(_vp(self.h))
        except Exception:
            pass

    def blocks(self):
        b = np.zeros(self.info["nblocks"], np.uint64)
        self.lib().ref_sim_blocks(_vp(self.h), _ptr(b))
        return b

    def walkers(self):
        n = self.info["walkers"]
        x, y, z = (np.zeros(n, np.int32) for _ in range(3))
        s = np.zeros(n, np.uint64)
        df = np.zeros(n)
        self.lib().ref_sim_walkers(_vp(self.h), _ptr(x), _ptr(y), _ptr(z), _ptr(s), _ptr(df))
        return x, y, z, s, df

    def set_dfactor(self, f):
        self.lib().ref_sim_set_dfactor(_vp(self.h), ctypes.c_double(f))

    def walk(self, mode, n_echoes, steps_per_echo):
        n = self.info["walkers"]
        per = np.zeros(n_echoes + 1, np.float64 if mode == 1 else np.uint64)
        xf, yf, zf = (np.zeros(n, np.int32) for _ in range(3))
        coll = np.zeros(n, np.uint32)
        en = np.zeros(n)
        sd = np.zeros(n, np.uint64)
        self.lib().ref_walk(_vp(self.h), mode, n_echoes, steps_per_echo, _ptr(per), _ptr(xf), _ptr(yf), _ptr(zf),
                            _ptr(coll), _ptr(en), _ptr(sd))
        if mode == 0:
            per = per[:n_echoes]
        return dict(per_echo=per, xf=xf, yf=yf, zf=zf, coll=coll, energy=en, seed=sd)

    def cpmg(self, obs_time, apply_bulk=True, cap=1 << 20):
        raw, out, times = np.zeros(cap), np.zeros(cap), np.zeros(cap)
        mc = np.zeros(self.info["walkers"], np.uint32)
        n = self.lib().ref_cpmg(_vp(self.h), ctypes.c_double(obs_time), int(apply_bulk), _ptr(raw), _ptr(out),
                                _ptr(times), cap, _ptr(mc))
        if n < 0:
            raise ValueError("cap too small")
        return dict(raw=raw[:n].copy(), signal=out[:n].copy(), times=times[:n].copy(), map_collisions=mc)

    def cpmg_method(self, method, obs_time, apply_bulk=True, cap=1 << 20, hcap=1 << 14):
        """NMR_cpmg::set + run_simulation with METHOD ``method`` ("image-based" | "histogram"):
        the decay (raw and normalised) and the xi-rate histograms of the collision-mapping walk."""
        L = self.lib()
        L.ref_cpmg_method.restype = ctypes.c_int
        raw, out, times = np.zeros(cap), np.zeros(cap), np.zeros(cap)
        hb, ha = np.zeros(hcap), np.zeros(hcap)
        nmax = 64
        lb, la = np.zeros(nmax * hcap), np.zeros(nmax * hcap)
        sizes = np.zeros(2, np.int32)
        n = L.ref_cpmg_method(_vp(self.h), method.encode(), ctypes.c_double(obs_time), int(apply_bulk), _ptr(raw),
                              _ptr(out), _ptr(times), cap, _ptr(hb), _ptr(ha), _ptr(lb), _ptr(la), hcap, _ptr(sizes))
        hs, nl = int(sizes[0]), int(sizes[1])
        if n < 0 or nl > nmax:
            raise ValueError("cap too small")
        return dict(raw=raw[:n].copy(), signal=out[:n].copy(), times=times[:n].copy(), hist_bins=hb[:hs].copy(),
                    hist_amps=ha[:hs].copy(), list_bins=lb[: nl * hs].reshape(nl, hs).copy(),
                    list_amps=la[: nl * hs].reshape(nl, hs).copy())

    def multitau(self, cpmg_text, multitau_text, cap=256):
        """The reference's NMR_multitau::run on CPU; returns steps per echo, echo times, first echoes."""
        L = self.lib()
        L.ref_multitau.restype = ctypes.c_int
        steps = np.zeros(cap, np.uint32)
        times, amps = np.zeros(cap), np.zeros(cap)
        n = L.ref_multitau(_vp(self.h), cpmg_text.encode(), multitau_text.encode(), cap, _ptr(steps), _ptr(times),
                           _ptr(amps))
        if n < 0:
            raise ValueError("ref_multitau failed")
        return dict(steps=steps[:n].copy(), times=times[:n].copy(), amps=amps[:n].copy())

    def pfgse(self, pulse_width, gmax, n_g, time_seq, n_t, t_min=0.0, t_max=1.0, t_values=None, apply_bulk=False,
              threshold_type="samples", threshold_value=None, threshold_window=1, cap=256):
        L = self.lib()
        tv = np.ascontiguousarray(t_values if t_values is not None else [1.0], np.float64)
        if threshold_value is None:
            threshold_value = n_g
        Mkt = np.zeros(cap * n_g)
        steps = np.zeros(cap, np.int32)
        dsat, dmsd, delta = np.zeros(cap), np.zeros(cap), np.zeros(cap)
        kvec = np.zeros(n_g * 3)
        nd = L.ref_pfgse(_vp(self.h), ctypes.c_double(pulse_width), ctypes.c_double(gmax[0]),
                         ctypes.c_double(gmax[1]), ctypes.c_double(gmax[2]), n_g, time_seq.encode(), n_t,
                         ctypes.c_double(t_min), ctypes.c_double(t_max), _ptr(tv), int(apply_bulk),
                         threshold_type.encode(), ctypes.c_double(threshold_value), threshold_window, cap, _ptr(Mkt),
                         _ptr(steps), _ptr(dsat), _ptr(dmsd), _ptr(kvec), _ptr(delta))
        if nd < 0:
            raise ValueError("cap too small")
        return dict(Mkt=Mkt[: nd * n_g].reshape(nd, n_g).copy(), steps=steps[:nd].copy(), dsat=dsat[:nd].copy(),
                    dmsd=dmsd[:nd].copy(), kvec=kvec.reshape(n_g, 3), delta=delta[:nd].copy())


def _ref_pfgse_sampling(sim, samples, pulse_width, gmax, n_g, t_values, apply_bulk=False, threshold_type="samples",
                        threshold_value=None, cap=64):
    L = sim.lib()
    L.ref_pfgse_sampling.restype = ctypes.c_int
    tv = np.ascontiguousarray(t_values, np.float64)
    if threshold_value is None:
        threshold_value = n_g
    Mkt, Mstd, lhs, lhs_std = (np.zeros(cap * n_g) for _ in range(4))
    steps = np.zeros(cap, np.int32)
    dsat, dmsd, delta, dsat_err, dsat_std, dmsd_std = (np.zeros(cap) for _ in range(6))
    kvec = np.zeros(n_g * 3)
    nd = L.ref_pfgse_sampling(_vp(sim.h), int(samples), ctypes.c_double(pulse_width), ctypes.c_double(gmax[0]),
                              ctypes.c_double(gmax[1]), ctypes.c_double(gmax[2]), n_g, b"manual", len(tv), _ptr(tv),
                              int(apply_bulk), threshold_type.encode(), ctypes.c_double(threshold_value), cap, _ptr(Mkt),
                              _ptr(steps), _ptr(dsat), _ptr(dmsd), _ptr(kvec), _ptr(delta), _ptr(Mstd), _ptr(lhs),
                              _ptr(lhs_std), _ptr(dsat_err), _ptr(dsat_std), _ptr(dmsd_std))
    if nd < 0:
        raise ValueError("cap too small")
    r = lambda a: a[: nd * n_g].reshape(nd, n_g).copy()  # noqa: E731
    return dict(Mkt=r(Mkt), Mstd=r(Mstd), lhs=r(lhs), lhs_std=r(lhs_std), steps=steps[:nd].copy(), dsat=dsat[:nd].copy(),
                dsat_err=dsat_err[:nd].copy(), dsat_std=dsat_std[:nd].copy(), dmsd=dmsd[:nd].copy(),
                dmsd_std=dmsd_std[:nd].copy(), delta=delta[:nd].copy())


RefSim.pfgse_sampling = _ref_pfgse_sampling


def ref_uniform_field(labels, resolution, gradient, direction):
    """The reference's own uniform internal field (InternalField.cpp) for a binary image."""
    lab = np.ascontiguousarray(np.asarray(labels) != 0, np.uint8)
    nz, ny, nx = lab.shape
    out = np.zeros(lab.shape, np.float64)
    L = RefSim.lib()
    L.ref_uniform_field.restype = ctypes.c_int
    rc = L.ref_uniform_field(_ptr(lab), nx, ny, nz, ctypes.c_double(resolution), ctypes.c_double(gradient),
                             int(direction), _ptr(out))
    if rc != 0:
        raise ValueError("ref_uniform_field failed")
    return out


def ref_bitblock(labels):
    L = RefSim.lib()
    labels = np.ascontiguousarray(labels, dtype=np.uint8)
    nz, ny, nx = labels.shape
    dims = np.zeros(3, np.int32)
    nb = L.ref_bitblock(_ptr(labels), nx, ny, nz, None, _ptr(dims))
    blocks = np.zeros(nb, np.uint64)
    L.ref_bitblock(_ptr(labels), nx, ny, nz, _ptr(blocks), _ptr(dims))
    return blocks, dims
