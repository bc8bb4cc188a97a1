"""Generates the golden fixtures in this directory from the reference's own CPU code.

The reference (RandomWalk_NMR) ships no tests or golden vectors, so the fixtures are produced by
running its unmodified CPU sources, compiled by oracle/Makefile into oracle/_ref/librwnmr_ref.so,
through oracle/ref_driver.cpp. Run from the repository root where the reference sources exist:

    RWNMR_REFERENCE=<RandomWalk_NMR checkout> python tests/golden/make_golden.py

(the checkout defaults to /root/reference, where this script was written against a read-only copy);
the script builds oracle/_ref from that checkout first.

Images come from the repository's sphere-pack generator (randomwalk_nmr_gb300.host), so the
fixtures pin the reference's setup, walk, CPMG and PFGSE outputs on fixed inputs.
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import pyoracle  # noqa: E402
from oracle.pyoracle import RefSim, ref_bitblock  # noqa: E402
from randomwalk_nmr_gb300 import host  # noqa: E402


def dfactor(rho, res=1.0, d0=2.5):
    # Walker::computeDecreaseFactor (Walker/walker.h:203-209)
    return 1.0 - (2.0 / 3.0) * ((rho * res) / (d0 * 1e03))


def image_a():
    lab, _ = host.synth_spheres((28, 20, 24), 2.0, 6.0, 0.35, 1, seed=3)
    return lab


def main():
    pyoracle.build(with_ref=True, ref_root=os.environ.get(pyoracle.REF_ENV, "/root/reference"))
    out = {}
    lab = image_a()
    out["img_a"] = lab
    blocks, dims = ref_bitblock(lab)
    out["img_a_blocks"] = blocks
    out["img_a_bdims"] = dims

    # walker setup + per-echo walks (energy and collision modes) at rho = 10 um/s
    rs = RefSim(lab, 300, 7, rho=(10.0,), steps_per_echo=2)
    x, y, z, s, df = rs.walkers()
    out.update(walk_x0=x, walk_y0=y, walk_z0=z, walk_seed0=s, walk_dfactor=df)
    r1 = rs.walk(1, 200, 2)
    r0 = rs.walk(0, 200, 2)
    out.update(walk_energy_sum=r1["per_echo"], walk_coll_per_echo=r0["per_echo"], walk_xf=r1["xf"],
               walk_yf=r1["yf"], walk_zf=r1["zf"], walk_seedf=r1["seed"], walk_energy=r1["energy"],
               walk_coll=r0["coll"])

    # CPMG sequence (NMR_cpmg::set + image_simulation_omp + bulk + normalize)
    rs2 = RefSim(lab, 400, 5, rho=(25.0,), steps_per_echo=3, bulk_time=800.0)
    c = rs2.cpmg(obs_time=12.0, apply_bulk=True)
    x, y, z, s, df = rs2.walkers()
    out.update(cpmg_x0=x, cpmg_y0=y, cpmg_z0=z, cpmg_seed0=s, cpmg_dfactor=df, cpmg_raw=c["raw"],
               cpmg_signal=c["signal"], cpmg_times=c["times"], cpmg_map_collisions=c["map_collisions"])

    # PFGSE sequence (NMR_PFGSE::run without file output), gradient along z
    rs3 = RefSim(lab, 500, 9, rho=(5.0,), steps_per_echo=1)
    pf = rs3.pfgse(pulse_width=0.5, gmax=(0.0, 0.0, 400.0), n_g=8, time_seq="manual", n_t=3,
                   t_values=[0.4, 1.0, 2.5], threshold_type="samples", threshold_value=8)
    x, y, z, s, df = rs3.walkers()
    out.update(pfgse_x0=x, pfgse_y0=y, pfgse_z0=z, pfgse_seed0=s, pfgse_dfactor=df, pfgse_Mkt=pf["Mkt"],
               pfgse_steps=pf["steps"], pfgse_dsat=pf["dsat"], pfgse_dmsd=pf["dmsd"], pfgse_kvec=pf["kvec"],
               pfgse_delta=pf["delta"], pfgse_gamma=np.array(rs3.info["gamma"]))

    # RHO_TYPE sigmoid: every walker's relaxivity from its collision rate in the mapping walk
    # (NMR_cpmg.cpp:132-146, Walker/walker.h:162-196), image-based CPMG and PFGSE
    sig = (40.0, 5.0, 0.1, 30.0, 10.0, 0.0, 0.25, 50.0)
    out["sigmoid_rho"] = np.array(sig)
    rs4 = RefSim(lab, 400, 5, rho=sig, rho_type="sigmoid", steps_per_echo=3, bulk_time=800.0)
    c = rs4.cpmg(obs_time=12.0, apply_bulk=True)
    x, y, z, s, df = rs4.walkers()
    out.update(cpmg_sig_raw=c["raw"], cpmg_sig_signal=c["signal"], cpmg_sig_dfactor=df,
               cpmg_sig_map_collisions=c["map_collisions"])
    del rs4
    rs5 = RefSim(lab, 500, 9, rho=sig, rho_type="sigmoid", steps_per_echo=1)
    pf = rs5.pfgse(pulse_width=0.5, gmax=(0.0, 0.0, 400.0), n_g=8, time_seq="manual", n_t=3,
                   t_values=[0.4, 1.0, 2.5], threshold_type="samples", threshold_value=8)
    x, y, z, s, df = rs5.walkers()
    out.update(pfgse_sig_Mkt=pf["Mkt"], pfgse_sig_dsat=pf["dsat"], pfgse_sig_dmsd=pf["dmsd"], pfgse_sig_dfactor=df)
    del rs5

    # PFGSE with walker sampling (ALLOW_WALKER_SAMPLING, 4 samples). rho = 0 keeps every walker's
    # energy at 1: the reference's CPU sampling sums weight sample s's walkers with the energies of
    # sample 0 (NMR_pfgse.cpp:818, walkers[idx] for walkers[offset + idx]); its GPU path does not.
    rs7 = RefSim(lab, 600, 11, rho=(0.0,), steps_per_echo=1, bulk_time=900.0)
    ps = rs7.pfgse_sampling(4, pulse_width=0.5, gmax=(0.0, 0.0, 400.0), n_g=8, t_values=[0.4, 1.0, 2.5],
                            apply_bulk=True, threshold_type="samples", threshold_value=6)
    out.update({f"pfgse_smp_{k}": v for k, v in ps.items()})
    del rs7

    # multitau (NMR_multitau::run): log-spaced echo times, one CPMG each, first echo kept
    rs6 = RefSim(lab, 400, 5, rho=(25.0,), steps_per_echo=3, bulk_time=800.0)
    mt = rs6.multitau("METHOD: image-based\nOBS_TIME: 12.0\nAPPLY_BULK: true\nSAVE_MODE: false\n",
                      "TAU_MIN: 0.1\nTAU_MAX: 3.0\nTAU_POINTS: 6\nTAU_SCALE: log\nSAVE_DECAY: true\n")
    out.update(multitau_steps=mt["steps"], multitau_times=mt["times"], multitau_amps=mt["amps"])
    del rs6

    # METHOD: histogram (createPenaltiesVector + histogram_simulation, NMR_cpmg.cpp:235-343) and the
    # xi-rate collision histograms of the mapping walk (CollisionHistogram.cpp:59-249), for uniform
    # and sigmoid relaxivity, linear and log bins, several histogram windows; plus the image-based
    # method on the same setup, whose histograms come from the same mapping walk.
    hm_cases = [("hm_u", (25.0,), "uniform", 4, 256, "linear", "histogram"),
                ("hm_s", sig, "sigmoid", 3, 128, "linear", "histogram"),
                ("hm_l", (25.0,), "uniform", 2, 64, "log", "histogram"),
                ("hm_i", (25.0,), "uniform", 4, 256, "linear", "image-based")]
    for key, rho, rtype, nh, hs, scale, method in hm_cases:
        r = RefSim(lab, 400, 5, rho=rho, rho_type=rtype, steps_per_echo=3, bulk_time=800.0, histograms=nh,
                   histogram_size=hs, histogram_scale=scale)
        c = r.cpmg_method(method, obs_time=12.0, apply_bulk=True)
        out[f"{key}_args"] = np.array([nh, hs], np.int64)
        out[f"{key}_scale"] = np.array(scale)
        out[f"{key}_method"] = np.array(method)
        out[f"{key}_rho"] = np.array(rho)
        out.update({f"{key}_{k}": v for k, v in c.items()})
        del r

    # walker placement modes (no one-past-the-end pore draws in these cases)
    lab_p = lab.copy()
    nz, ny, nx = lab_p.shape
    lab_p[nz // 2 - 3:nz // 2 + 3, ny // 2 - 3:ny // 2 + 3, nx // 2 - 3:nx // 2 + 3] = 0
    out["img_p"] = lab_p
    cases = [("random", 0, 0, 2000, 21), ("random", 0, 1, 500, 22), ("point", 0, 0, 100, 23),
             ("point", 0, 2, 100, 24), ("cubic", 3, 0, 20, 25), ("cubic", 3, 1, 20, 26)]
    for k, (mode, dev, shift, n, seed) in enumerate(cases):
        r = RefSim(lab_p, n, seed, rho=(1.0,), placement=mode, deviation=dev, voxel_division=shift)
        x, y, z, s, df = r.walkers()
        out[f"place{k}_args"] = np.array([dev, shift, n, seed], np.int64)
        out[f"place{k}_mode"] = np.array(mode)
        out.update({f"place{k}_x": x, f"place{k}_y": y, f"place{k}_z": z, f"place{k}_seed": s})
        out[f"place{k}_pores"] = np.array(r.info["pores"])
        del r

    np.savez_compressed(os.path.join(HERE, "reference_cpu.npz"), **out)
    print("wrote", os.path.join(HERE, "reference_cpu.npz"))
    full_size()


def full_size():
    """Fixtures at full image sizes of the benchmark configurations.

    * plain CPMG, 100^3 (spheres of radius 4-10 to porosity 0.30, seed 1), 10,000 walkers placed
      with SEED 7, rho 10 um/s, 2000 echoes x 3 steps: the reference's own walk (Walker::walk /
      Walker::map in the serial order of NMR_cpmg::image_simulation_omp, NMR_cpmg.cpp:177-233):
      echo sums, per-echo collisions, final positions, RNG states and collision counts;
    * PFGSE, 256^3 (radius 5-15, porosity 0.35, seed 3), 64 gradients 0-100 G/cm along z, pulse
      1 ms, 10 exposure times log-spaced 1-100 ms, rho 10 um/s: the reference's CPU sequence
      (NMR_PFGSE::run, NMR_pfgse.cpp:98-131, 1658-1806) on 16,384 walkers placed with SEED 7.
    """
    out = {}
    lab, _ = host.synth_spheres((100, 100, 100), 4.0, 10.0, 0.30, 1, seed=1)
    blocks, dims = ref_bitblock(lab)
    out.update(c1_blocks=blocks, c1_bdims=dims)
    rs = RefSim(lab, 10_000, 7, rho=(10.0,), steps_per_echo=3, bulk_time=2800.0)
    x, y, z, s, df = rs.walkers()
    out.update(c1_x0=x, c1_y0=y, c1_z0=z, c1_seed0=s, c1_dfactor=df)
    r1 = rs.walk(1, 2000, 3)
    r0 = rs.walk(0, 2000, 3)
    out.update(c1_energy_sum=r1["per_echo"], c1_coll_per_echo=r0["per_echo"], c1_xf=r1["xf"], c1_yf=r1["yf"],
               c1_zf=r1["zf"], c1_seedf=r1["seed"], c1_coll=r0["coll"], c1_energy=r1["energy"])
    del rs
    np.savez_compressed(os.path.join(HERE, "reference_c1.npz"), **out)
    print("wrote", os.path.join(HERE, "reference_c1.npz"))

    out = {}
    lab, _ = host.synth_spheres((256, 256, 256), 5.0, 15.0, 0.35, 1, seed=3)
    blocks, dims = ref_bitblock(lab)
    out["c3_blocks_sha256"] = np.array(hashlib.sha256(blocks.tobytes()).hexdigest())
    out["c3_bdims"] = dims
    rs = RefSim(lab, 16_384, 7, rho=(10.0,), steps_per_echo=1, bulk_time=2800.0)
    pf = rs.pfgse(pulse_width=1.0, gmax=(0.0, 0.0, 100.0), n_g=64, time_seq="log", n_t=10, t_min=0.0, t_max=2.0,
                  threshold_type="samples", threshold_value=64)
    x, y, z, s, df = rs.walkers()
    out.update(c3_x0=x, c3_y0=y, c3_z0=z, c3_seed0=s, c3_dfactor=df, c3_Mkt=pf["Mkt"], c3_steps=pf["steps"],
               c3_dsat=pf["dsat"], c3_dmsd=pf["dmsd"], c3_kvec=pf["kvec"], c3_delta=pf["delta"],
               c3_gamma=np.array(rs.info["gamma"]), c3_dt=np.array(rs.info["dt"]))
    del rs
    np.savez_compressed(os.path.join(HERE, "reference_c3.npz"), **out)
    print("wrote", os.path.join(HERE, "reference_c3.npz"))


if __name__ == "__main__":
    # The reference's CPU PFGSE sums into malloc'd memory it never zeroes (NMR_pfgse.cpp:1673-1680).
    # oracle/ref_driver.cpp asks glibc for zero-filled allocations (M_PERTURB); glibc's per-thread
    # cache bypasses that, so this process runs with the cache disabled (read at process start).
    tun = "glibc.malloc.tcache_count=0"
    if tun not in os.environ.get("GLIBC_TUNABLES", ""):
        os.environ["GLIBC_TUNABLES"] = tun
        os.execv(sys.executable, [sys.executable] + sys.argv)
    main()
