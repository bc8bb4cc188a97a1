"""Generates the golden fixtures in this directory from the reference's own CPU code.

The reference (RandomWalk_NMR) ships no tests or golden vectors, so the fixtures are produced by
running its unmodified CPU sources, compiled by oracle/Makefile into oracle/_ref/librwnmr_ref.so,
through oracle/ref_driver.cpp. Run from the repository root where the reference sources exist:

    make -C oracle ref && python tests/golden/make_golden.py

Images come from the repository's sphere-pack generator (randomwalk_nmr_gb300.host), so the
fixtures pin the reference's setup, walk, CPMG and PFGSE outputs on fixed inputs.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.pyoracle import RefSim, ref_bitblock  # noqa: E402
from randomwalk_nmr_gb300 import host  # noqa: E402


def dfactor(rho, res=1.0, d0=2.5):
    # Walker::computeDecreaseFactor (Walker/walker.h:203-209)
    return 1.0 - (2.0 / 3.0) * ((rho * res) / (d0 * 1e03))


def image_a():
    lab, _ = host.synth_spheres((28, 20, 24), 2.0, 6.0, 0.35, 1, seed=3)
    return lab


def main():
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


if __name__ == "__main__":
    # The reference's CPU PFGSE sums into malloc'd memory it never zeroes (NMR_pfgse.cpp:1673-1680).
    # oracle/ref_driver.cpp asks glibc for zero-filled allocations (M_PERTURB); glibc's per-thread
    # cache bypasses that, so this process runs with the cache disabled (read at process start).
    tun = "glibc.malloc.tcache_count=0"
    if tun not in os.environ.get("GLIBC_TUNABLES", ""):
        os.environ["GLIBC_TUNABLES"] = tun
        os.execv(sys.executable, [sys.executable] + sys.argv)
    main()
