"""The command-line driver end to end (config files -> image -> walkers -> GPU walk -> output
files), checked against the reference's own CPU sequences on the same inputs (golden fixtures)."""
import os

import numpy as np
import pytest

from randomwalk_nmr_gb300 import host

pytestmark = pytest.mark.gpu


def write(path, text):
    os.makedirs(os.path.dirname(path), exist_ok=True)
    with open(path, "w") as f:
        f.write(text)


RW = ("NAME: t\nD0: 2.5\nBULK_TIME: {bulk}\nRHO_TYPE: uniform\nRHO: {{{rho}}}\nWALKERS: {n}\n"
      "WALKERS_PLACEMENT: random\nSTEPS_PER_ECHO: {spe}\nSEED: {seed}\nBC: noflux\n"
      "GIROMAGNETIC_RATIO: 42.576\nGIROMAGNETIC_UNIT: mhertz\nHISTOGRAMS: 1\nHISTOGRAM_SIZE: 1024\n")
IMG_A = "24,20,28,2,6,0.35,1,3"  # the sphere pack of the golden fixtures (nx, ny, nz, rmin, rmax, porosity, phases, seed)


def test_cli_cpmg_matches_reference_sequence(tmp_path, golden):
    root = str(tmp_path / "config") + "/"
    write(root + "default/rwnmr.config", RW.format(bulk=800.0, rho=25.0, n=400, spe=3, seed=5))
    write(root + "default/uct.config", "RESOLUTION: 1.0\nVOXEL_DIVISION: 0\n")
    write(root + "default/cpmg.config", "METHOD: image-based\nOBS_TIME: 12.0\nAPPLY_BULK: true\nSAVE_MODE: true\n"
                                        "SAVE_DECAY: true\nSAVE_HISTOGRAM: true\nSAVE_WALKERS: true\n")
    rc = host.cli(["--config-root", root, "--synthetic", IMG_A, "--quiet", "cpmg"], cwd=str(tmp_path))
    assert rc == 0
    d = str(tmp_path / "db" / "t") + "//NMR_cpmg_t=12.00ms"
    decay = np.loadtxt(d + "/cpmg_decay.csv", delimiter=",", skiprows=1)
    assert np.array_equal(decay[:, 0], golden["cpmg_times"])
    np.testing.assert_allclose(decay[:, 3], golden["cpmg_signal"], rtol=1e-12)
    np.testing.assert_allclose(decay[:, 1], golden["cpmg_signal"], rtol=1e-12)
    coll = np.loadtxt(d + "/cpmg_echo_collisions.csv", delimiter=",", skiprows=1)
    assert coll.shape == (len(golden["cpmg_times"]) - 1, 2)
    hist = np.loadtxt(d + "/cpmg_histogram.csv", delimiter=",", skiprows=1)
    assert hist.shape == (1024, 2) and abs(hist[:, 1].sum() - 1.0) < 1e-12
    walkers = np.loadtxt(d + "/cpmg_walkers.csv", delimiter=",", skiprows=1)
    assert np.array_equal(walkers[:, 6].astype(np.int64), golden["cpmg_map_collisions"].astype(np.int64))
    assert os.path.exists(str(tmp_path / "db" / "t" / "SimInfo.txt"))
    check_t2_file(d, decay)


@pytest.mark.parametrize("case", ["hm_u", "hm_s", "hm_l", "hm_i"])
def test_cli_histogram_method_and_xi_rate_histograms_match_reference(tmp_path, golden, case):
    """METHOD: histogram (penalty per xi-rate bin applied window by window, NMR_cpmg.cpp:235-343)
    and the xi-rate collision histograms of the mapping walk (CollisionHistogram.cpp:59-249) --
    global and per window, linear and log bins, uniform and sigmoid relaxivity -- against the
    reference's own CPU sequence on the same image and walkers. The image-based case checks the
    histogram outputs of an image-based run. Decay within 1e-12 relative; histogram bins and
    amplitudes exact (written with 17 significant digits)."""
    nh, hs = (int(v) for v in golden[f"{case}_args"])
    scale, method = str(golden[f"{case}_scale"]), str(golden[f"{case}_method"])
    rho = ", ".join(repr(float(v)) for v in golden[f"{case}_rho"])
    rtype = "sigmoid" if len(golden[f"{case}_rho"]) == 8 else "uniform"
    rw = RW.replace("RHO_TYPE: uniform", f"RHO_TYPE: {rtype}").replace(
        "HISTOGRAMS: 1\nHISTOGRAM_SIZE: 1024\n", f"HISTOGRAMS: {nh}\nHISTOGRAM_SIZE: {hs}\nHISTOGRAM_SCALE: {scale}\n")
    root = str(tmp_path / "config") + "/"
    write(root + "default/rwnmr.config", rw.format(bulk=800.0, rho=rho, n=400, spe=3, seed=5))
    write(root + "default/uct.config", "RESOLUTION: 1.0\nVOXEL_DIVISION: 0\n")
    write(root + "default/cpmg.config", f"METHOD: {method}\nOBS_TIME: 12.0\nAPPLY_BULK: true\nSAVE_MODE: true\n"
                                        "SAVE_DECAY: true\nSAVE_HISTOGRAM: true\nSAVE_HISTOGRAM_LIST: true\n")
    rc = host.cli(["--config-root", root, "--synthetic", IMG_A, "--quiet", "cpmg"], cwd=str(tmp_path))
    assert rc == 0
    d = str(tmp_path / "db" / "t") + "//NMR_cpmg_t=12.00ms"
    decay = np.loadtxt(d + "/cpmg_decay.csv", delimiter=",", skiprows=1)
    assert np.array_equal(decay[:, 0], golden[f"{case}_times"])
    np.testing.assert_allclose(decay[:, 3], golden[f"{case}_signal"], rtol=1e-12)
    hist = np.loadtxt(d + "/cpmg_histogram.csv", delimiter=",", skiprows=1)
    assert np.array_equal(hist[:, 0], golden[f"{case}_hist_bins"])
    assert np.array_equal(hist[:, 1], golden[f"{case}_hist_amps"])
    hl = np.genfromtxt(d + "/cpmg_histList.csv", delimiter=",", skip_header=1)[:, : 2 * nh]
    assert hl.shape == (golden[f"{case}_list_bins"].shape[1], 2 * nh)
    assert np.array_equal(hl[:, 0::2].T, golden[f"{case}_list_bins"])
    assert np.array_equal(hl[:, 1::2].T, golden[f"{case}_list_amps"])


def check_t2_file(d, decay, bins=128):
    """cpmg_T2.csv is the T2 inversion of the decay beside it (default cpmg.config settings): the
    oracle's restatement at the oracle's L-curve choice or at a grid neighbour (the curvature's
    flat maximum moves a step between SVD implementations on noisy decays)."""
    from oracle import laplace

    t2 = np.loadtxt(d + "/cpmg_T2.csv", delimiter=",", skiprows=1)
    assert t2.shape == (bins, 2) and np.all(t2[:, 1] >= 0)
    r = laplace.invert(decay[:, 0], decay[:, 3], num_t2_bins=bins)
    assert np.array_equal(t2[:, 0], r["bins"])
    near = range(max(0, r["best"] - 2), min(len(r["lambdas"]), r["best"] + 3))
    cands = [laplace.invert(decay[:, 0], decay[:, 3], num_t2_bins=bins, force_lambda=r["lambdas"][k])["amps"]
             for k in near]
    assert min(np.max(np.abs(t2[:, 1] - c)) / np.max(c) for c in cands) <= 1e-8


def test_cli_cpmg_internal_field(tmp_path, golden, oracle):
    """RESIDUAL_FIELD uniform / import through the config files: a zero field reproduces the
    plain decay, an imported copy of the uniform field reproduces the uniform run, a field file
    of the wrong size is rejected."""
    def run(name, extra):
        root = str(tmp_path / name / "config") + "/"
        write(root + "default/rwnmr.config", RW.format(bulk=800.0, rho=25.0, n=400, spe=4, seed=5))
        write(root + "default/uct.config", "RESOLUTION: 1.0\nVOXEL_DIVISION: 0\n")
        write(root + "default/cpmg.config", "METHOD: image-based\nOBS_TIME: 6.0\nAPPLY_BULK: true\nSAVE_MODE: true\n"
                                            "SAVE_DECAY: true\n" + extra)
        rc = host.cli(["--config-root", root, "--synthetic", IMG_A, "--quiet", "cpmg"], cwd=str(tmp_path / name))
        if rc != 0:
            return None
        d = str(tmp_path / name / "db" / "t") + "//NMR_cpmg_t=6.00ms"
        return np.loadtxt(d + "/cpmg_decay.csv", delimiter=",", skiprows=1)

    plain = run("plain", "")
    zero = run("zero", "RESIDUAL_FIELD: uniform\nGRADIENT_VALUE: 0.0\nGRADIENT_DIRECTION: z\n")
    np.testing.assert_allclose(zero[:, 1], plain[:, 1], rtol=1e-14)
    uni = run("uni", "RESIDUAL_FIELD: uniform\nGRADIENT_VALUE: 8.0\nGRADIENT_DIRECTION: y\n")
    assert uni[-1, 1] < 0.98 * plain[-1, 1]
    field = oracle.uniform_field(golden["img_a"], 1.0, 8.0, 1)
    path = str(tmp_path / "field.raw")
    field.tofile(path)
    imp = run("imp", f"RESIDUAL_FIELD: import\nPATH_TO_FIELD: {path}\n")
    assert np.array_equal(imp, uni)
    field[:-1].tofile(path)
    assert run("bad", f"RESIDUAL_FIELD: import\nPATH_TO_FIELD: {path}\n") is None


def test_cli_sigmoid_relaxivity_matches_reference(tmp_path, golden):
    """RHO_TYPE sigmoid: a relaxivity per walker from its collision rate in the mapping walk, for
    image-based CPMG and for PFGSE, against the reference's own CPU sequences."""
    sig = ", ".join(repr(float(v)) for v in golden["sigmoid_rho"])
    rw_sig = RW.replace("RHO_TYPE: uniform", "RHO_TYPE: sigmoid")
    root = str(tmp_path / "c" / "config") + "/"
    write(root + "default/rwnmr.config", rw_sig.format(bulk=800.0, rho=sig, n=400, spe=3, seed=5))
    write(root + "default/uct.config", "RESOLUTION: 1.0\nVOXEL_DIVISION: 0\n")
    write(root + "default/cpmg.config", "METHOD: image-based\nOBS_TIME: 12.0\nAPPLY_BULK: true\nSAVE_MODE: true\n"
                                        "SAVE_DECAY: true\n")
    assert host.cli(["--config-root", root, "--synthetic", IMG_A, "--quiet", "cpmg"], cwd=str(tmp_path / "c")) == 0
    d = str(tmp_path / "c" / "db" / "t") + "//NMR_cpmg_t=12.00ms"
    decay = np.loadtxt(d + "/cpmg_decay.csv", delimiter=",", skiprows=1)
    np.testing.assert_allclose(decay[:, 1], golden["cpmg_sig_signal"], rtol=1e-12)

    root = str(tmp_path / "p" / "config") + "/"
    write(root + "default/rwnmr.config", rw_sig.format(bulk=2800.0, rho=sig, n=500, spe=1, seed=9))
    write(root + "default/uct.config", "RESOLUTION: 1.0\nVOXEL_DIVISION: 0\n")
    write(root + "default/pfgse.config",
          "APPLY_BULK: false\nPULSE_WIDTH: 0.5\nMAX_GRADIENT: {0.0, 0.0, 400.0}\nGRADIENT_SAMPLES: 8\n"
          "TIME_SEQ: manual\nTIME_SAMPLES: 3\nTIME_VALUES: {0.4, 1.0, 2.5}\nAPPLY_SCALE_FACTOR: false\n"
          "THRESHOLD_TYPE: samples\nTHRESHOLD_VALUE: 8\nALLOW_WALKER_SAMPLING: false\nSAVE_MODE: true\n"
          "SAVE_PFGSE: true\n")
    assert host.cli(["--config-root", root, "--synthetic", IMG_A, "--quiet", "pfgse"], cwd=str(tmp_path / "p")) == 0
    d = str(tmp_path / "p" / "db" / "t") + "//NMR_pfgse"
    res = np.loadtxt(d + "/PFGSE_results.csv", delimiter=",", skiprows=1, ndmin=2)
    np.testing.assert_allclose(res[:, 1], golden["pfgse_sig_dsat"], rtol=1e-10)
    np.testing.assert_allclose(res[:, 5], golden["pfgse_sig_dmsd"], rtol=1e-12)
    for i in range(3):
        e = np.loadtxt(d + f"/timesamples/echoes_{i}.csv", delimiter=",", skiprows=1)
        assert np.all(np.abs(e[:, 2] / e[0, 2] - golden["pfgse_sig_Mkt"][i]) <= 1e-12)


@pytest.mark.parametrize("complete", [False, True])
def test_cli_multitau_matches_reference(tmp_path, golden, complete):
    """multitau: one CPMG per echo time (log-spaced te, whole even step counts), first echo of each,
    against the reference's own NMR_multitau run; COMPLETE_DECAY also writes each full decay."""
    root = str(tmp_path / "config") + "/"
    write(root + "default/rwnmr.config", RW.format(bulk=800.0, rho=25.0, n=400, spe=3, seed=5))
    write(root + "default/uct.config", "RESOLUTION: 1.0\nVOXEL_DIVISION: 0\n")
    write(root + "default/cpmg.config", "METHOD: image-based\nOBS_TIME: 12.0\nAPPLY_BULK: true\nSAVE_MODE: false\n")
    write(root + "default/multitau.config", "TAU_MIN: 0.1\nTAU_MAX: 3.0\nTAU_POINTS: 6\nTAU_SCALE: log\nSAVE_DECAY: true\n"
                                            + ("COMPLETE_DECAY: true\n" if complete else ""))
    assert host.cli(["--config-root", root, "--synthetic", IMG_A, "--quiet", "multitau"], cwd=str(tmp_path)) == 0
    d = str(tmp_path / "db" / "t") + "//NMR_multitau_min=0.10ms_max=3.00ms_pts=6_scale=log"
    mt = np.loadtxt(d + "/multitau_decay.csv", delimiter=",", skiprows=1)
    np.testing.assert_allclose(mt[:, 0], golden["multitau_times"], rtol=1e-15)
    np.testing.assert_allclose(mt[:, 1], golden["multitau_amps"], rtol=1e-12)
    te0 = d + "/NMR_cpmg_t=" + ("12.00" if complete else "0.13") + "ms_te=0.133"
    if complete:
        decay = np.loadtxt(te0 + "/cpmg_decay.csv", delimiter=",", skiprows=1)
        assert len(decay) == 91 and decay[1, 1] == mt[0, 1]  # 12 ms / (2 steps x 1/15 ms) echoes + t = 0
        check_t2_file(te0, decay)
    else:
        assert os.path.isdir(te0) and not os.path.exists(te0 + "/cpmg_decay.csv")


def test_cli_pfgse_walker_sampling_matches_reference(tmp_path, golden):
    """ALLOW_WALKER_SAMPLING with WALKER_SAMPLES 4: per-sample magnitudes, LHS and least-squares fits,
    their means and population deviations, per-sample mean squared displacements."""
    root = str(tmp_path / "config") + "/"
    write(root + "default/rwnmr.config", RW.format(bulk=900.0, rho=0.0, n=600, spe=1, seed=11) + "WALKER_SAMPLES: 4\n")
    write(root + "default/uct.config", "RESOLUTION: 1.0\nVOXEL_DIVISION: 0\n")
    write(root + "default/pfgse.config",
          "APPLY_BULK: true\nPULSE_WIDTH: 0.5\nMAX_GRADIENT: {0.0, 0.0, 400.0}\nGRADIENT_SAMPLES: 8\n"
          "TIME_SEQ: manual\nTIME_SAMPLES: 3\nTIME_VALUES: {0.4, 1.0, 2.5}\nAPPLY_SCALE_FACTOR: false\n"
          "THRESHOLD_TYPE: samples\nTHRESHOLD_VALUE: 6\nALLOW_WALKER_SAMPLING: true\nSAVE_MODE: true\n"
          "SAVE_PFGSE: true\n")
    assert host.cli(["--config-root", root, "--synthetic", IMG_A, "--quiet", "pfgse"], cwd=str(tmp_path)) == 0
    d = str(tmp_path / "db" / "t") + "//NMR_pfgse"
    res = np.loadtxt(d + "/PFGSE_results.csv", delimiter=",", skiprows=1, ndmin=2)
    g = {k[len("pfgse_smp_"):]: golden[k] for k in golden if k.startswith("pfgse_smp_")}
    np.testing.assert_allclose(res[:, 0], g["delta"], rtol=0)
    np.testing.assert_allclose(res[:, 1], g["dsat"], rtol=1e-10)
    np.testing.assert_allclose(res[:, 2], g["dsat_err"], rtol=1e-8, atol=1e-15)
    np.testing.assert_allclose(res[:, 3], g["dsat_std"], rtol=1e-8)
    assert np.all(res[:, 4] == 6)
    np.testing.assert_allclose(res[:, 5], g["dmsd"], rtol=1e-12)
    np.testing.assert_allclose(res[:, 6], g["dmsd_std"], rtol=1e-10)
    for i in range(3):
        e = np.loadtxt(d + f"/timesamples/echoes_{i}.csv", delimiter=",", skiprows=1)
        np.testing.assert_allclose(e[:, 2], g["Mkt"][i], rtol=1e-12)
        np.testing.assert_allclose(e[:, 4], g["Mstd"][i], rtol=1e-9, atol=1e-12)
        np.testing.assert_allclose(e[:, 5], g["lhs"][i], rtol=1e-10, atol=1e-13)
        np.testing.assert_allclose(e[:, 6], g["lhs_std"][i], rtol=1e-8, atol=1e-13)


def test_cli_saves_bit_block_image_and_walkers(tmp_path, golden):
    """SAVE_BINIMG writes NMR_binImage.txt in the reference's layout (fileHandler::writeBitBlockObject3D)
    with the reference's own bit-blocks; SAVE_WALKERS writes the walkers as created."""
    root = str(tmp_path / "config") + "/"
    write(root + "default/rwnmr.config", RW.format(bulk=800.0, rho=25.0, n=400, spe=3, seed=5)
          + "SAVE_BINIMG: true\nSAVE_WALKERS: true\n")
    write(root + "default/uct.config", "RESOLUTION: 1.0\nVOXEL_DIVISION: 0\n")
    assert host.cli(["--config-root", root, "--synthetic", IMG_A, "--quiet"], cwd=str(tmp_path)) == 0
    lines = open(str(tmp_path / "db" / "t" / "NMR_binImage.txt")).read().split("\n")
    assert lines[0] == "blocks, bRows, bColumns, bDepth, imgRows, imgColumns, imgDepth, "
    nb = len(golden["img_a_blocks"])
    bc, br, bd = (int(v) for v in golden["img_a_bdims"])
    assert lines[1] == f"{nb}, {br}, {bc}, {bd}, 20, 24, 28" and lines[2] == "" and lines[3] == "blockID, blockData"
    data = np.array([int(l.split(", ")[1]) for l in lines[4:4 + nb]], np.uint64)
    assert np.array_equal(data, golden["img_a_blocks"])
    w = np.loadtxt(str(tmp_path / "db" / "t" / "walkers.csv"), delimiter=",", skiprows=1)
    assert np.array_equal(w[:, 0], golden["cpmg_x0"]) and np.array_equal(w[:, 5], golden["cpmg_z0"])
    assert np.all(w[:, 6] == 0) and np.all(w[:, 8] == 1)


def test_cli_pfgse_matches_reference_sequence(tmp_path, golden):
    root = str(tmp_path / "config") + "/"
    write(root + "default/rwnmr.config", RW.format(bulk=2800.0, rho=5.0, n=500, spe=1, seed=9))
    write(root + "default/uct.config", "RESOLUTION: 1.0\nVOXEL_DIVISION: 0\n")
    write(root + "default/pfgse.config",
          "APPLY_BULK: false\nPULSE_WIDTH: 0.5\nMAX_GRADIENT: {0.0, 0.0, 400.0}\nGRADIENT_SAMPLES: 8\n"
          "TIME_SEQ: manual\nTIME_SAMPLES: 3\nTIME_VALUES: {0.4, 1.0, 2.5}\nAPPLY_SCALE_FACTOR: false\n"
          "THRESHOLD_TYPE: samples\nTHRESHOLD_VALUE: 8\nALLOW_WALKER_SAMPLING: false\nSAVE_MODE: true\n"
          "SAVE_PFGSE: true\n")
    rc = host.cli(["--config-root", root, "--synthetic", IMG_A, "--quiet", "pfgse"], cwd=str(tmp_path))
    assert rc == 0
    d = str(tmp_path / "db" / "t") + "//NMR_pfgse"
    res = np.loadtxt(d + "/PFGSE_results.csv", delimiter=",", skiprows=1, ndmin=2)
    np.testing.assert_allclose(res[:, 0], golden["pfgse_delta"], rtol=0)
    np.testing.assert_allclose(res[:, 1], golden["pfgse_dsat"], rtol=1e-10)
    np.testing.assert_allclose(res[:, 5], golden["pfgse_dmsd"], rtol=1e-12)
    for i in range(3):
        e = np.loadtxt(d + f"/timesamples/echoes_{i}.csv", delimiter=",", skiprows=1)
        att = e[:, 2] / e[0, 2]
        assert np.all(np.abs(att - golden["pfgse_Mkt"][i]) <= 1e-12)
    g = np.loadtxt(d + "/PFGSE_gradient.csv", delimiter=",", skiprows=1)
    np.testing.assert_allclose(g[:, 4:7], golden["pfgse_kvec"], rtol=1e-15, atol=0)


def test_cli_reads_png_stack(tmp_path, golden):
    """uct-config PNG slices -> same walk as the label volume they encode."""
    import struct
    import zlib

    lab = golden["img_a"]
    nz, ny, nx = lab.shape
    img_dir = tmp_path / "imgs"
    img_dir.mkdir()
    for z in range(nz):
        raw = b"".join(b"\x00" + bytes((lab[z, y] * 255).astype(np.uint8)) for y in range(ny))

        def chunk(t, dat):
            return struct.pack(">I", len(dat)) + t + dat + struct.pack(">I", zlib.crc32(t + dat) & 0xFFFFFFFF)

        png = (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", nx, ny, 8, 0, 0, 0, 0)) +
               chunk(b"IDAT", zlib.compress(raw)) + chunk(b"IEND", b""))
        (img_dir / f"slice_{z:03d}.png").write_bytes(png)
    root = str(tmp_path / "config") + "/"
    write(root + "default/rwnmr.config", RW.format(bulk=800.0, rho=25.0, n=400, spe=3, seed=5))
    write(root + "default/uct.config", f"DIR_PATH: {img_dir}/\nFILENAME: slice_\nFIRST_IDX: 0\nDIGITS: 3\n"
                                       f"EXTENSION: .png\nSLICES: {nz}\nRESOLUTION: 1.0\nVOXEL_DIVISION: 0\n")
    write(root + "default/cpmg.config", "OBS_TIME: 12.0\nAPPLY_BULK: true\nSAVE_HISTOGRAM: false\n")
    assert host.cli(["--config-root", root, "--quiet", "cpmg"], cwd=str(tmp_path)) == 0
    decay = np.loadtxt(str(tmp_path / "db" / "t") + "//NMR_cpmg_t=12.00ms/cpmg_decay.csv", delimiter=",",
                       skiprows=1)
    np.testing.assert_allclose(decay[:, 3], golden["cpmg_signal"], rtol=1e-12)
