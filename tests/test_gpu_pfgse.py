"""GPU parity of the PFGSE walk and its gradient-strength derivative against the CPU oracle."""
import numpy as np
import pytest

from conftest import dfactor
from randomwalk_nmr_gb300 import fx_to_float, host

pytestmark = pytest.mark.gpu

# |M_gpu - M_oracle| <= ATT_TOL * M(k=0): attenuations agree to 1e-12 of the unattenuated signal
ATT_TOL = 1e-12


def setup(engine, seed=3, n=4000, shape=(30, 26, 28), n_phases=1, morton=True):
    lab, _ = host.synth_spheres(shape, 2.0, 6.0, 0.4, n_phases, seed=seed)
    blocks, _ = host.pack_blocks(lab)
    x, y, z, s, _ = host.place_walkers(blocks, lab.shape, n, seed + 100)
    engine.allow_morton(morton)
    engine.upload_labels(lab, n_phases)
    assert engine.morton_layout == morton
    engine.upload_walkers(x, y, z, s)
    return lab, (x, y, z, s)


def kvecs(n_g, gmax, pulse_ms=1.0, gamma=42.576 * 2 * np.pi):
    """k_j as NMR_PFGSE builds them (NMR_pfgse.cpp:272-313,483-486): accumulated gradient steps."""
    gap = np.asarray(gmax, np.float64) / (n_g - 1)
    g = np.zeros(3)
    out = []
    for _ in range(n_g):
        out.append([(pulse_ms * 1e-3) * (gamma * 1e6) * (gi * 1e-8) for gi in g])
        g = g + gap
    return np.array(out)


@pytest.mark.parametrize("bc,morton", [("noflux", True), ("noflux", False), ("periodic", True), ("mirror", True)])
@pytest.mark.parametrize("gdir", [(0, 0, 100.0), (60.0, 0, 0), (30.0, 40.0, 20.0)])
def test_pfgse_parity(engine, oracle, bc, morton, gdir):
    lab, w = setup(engine, morton=morton)
    steps = np.array([15, 40, 100, 250], np.int32)
    kv = kvecs(16, gdir)
    f = dfactor(10.0)
    g = engine.pfgse(steps, kv, 1.0, f, bc=bc)
    o = oracle.pfgse(lab, w, f, steps, kv, 1.0, bc=bc, threads=4)
    assert np.array_equal(g["msd"], o["msd"])
    assert np.array_equal(fx_to_float(o["esum_fx"]), g["esum"])
    np.testing.assert_allclose(g["esum"], o["esum"], rtol=1e-12)
    scale = o["M"][:, :1]
    assert np.all(np.abs(g["M"] - o["M"]) <= ATT_TOL * scale)
    # attenuation decreases from 1 at k = 0
    att = g["M"] / g["M"][:, :1]
    assert np.allclose(att[:, 0], 1.0)


def test_pfgse_reference_golden(engine, golden):
    gd = golden
    lab = gd["img_a"]
    engine.upload_labels(lab)
    engine.upload_walkers(gd["pfgse_x0"], gd["pfgse_y0"], gd["pfgse_z0"], gd["pfgse_seed0"])
    g = engine.pfgse(gd["pfgse_steps"], gd["pfgse_kvec"], 1.0, float(gd["pfgse_dfactor"][0]))
    Mkt = g["M"] / g["esum"][:, None]
    assert np.all(np.abs(Mkt - gd["pfgse_Mkt"]) <= ATT_TOL)


def test_pfgse_multiphase(engine, oracle):
    lab, w = setup(engine, seed=8, n_phases=3)
    steps = np.array([10, 60, 200], np.int32)
    kv = kvecs(8, (0, 0, 80.0))
    f = dfactor([4.0, 20.0, 35.0])
    g = engine.pfgse(steps, kv, 1.0, f)
    o = oracle.pfgse(lab, w, f, steps, kv, 1.0, threads=4, n_phases=3)
    assert np.all(np.abs(g["M"] - o["M"]) <= ATT_TOL * o["M"][:, :1])


@pytest.mark.parametrize("bc", ["noflux", "periodic", "mirror"])
def test_pfgse_voxel_division(engine, oracle, bc):
    """Voxel division (walk grid 2x finer than the image): axis and oblique gradients."""
    lab, _ = host.synth_spheres((24, 22, 26), 2.0, 6.0, 0.4, 1, seed=12)
    blocks, _ = host.pack_blocks(lab)
    w = host.place_walkers(blocks, lab.shape, 3000, 77, "random", 0, 1)[:4]
    engine.upload_labels(lab, 1)
    engine.upload_walkers(*w)
    steps = np.array([30, 80, 200], np.int32)
    f = dfactor(15.0, res=0.5)
    for gdir in ((0, 0, 150.0), (40.0, 30.0, 60.0)):
        kv = kvecs(12, gdir)
        g = engine.pfgse(steps, kv, 0.5, f, bc=bc, shift=1)
        o = oracle.pfgse(lab, w, f, steps, kv, 0.5, bc=bc, shift=1, threads=4)
        assert np.array_equal(g["msd"], o["msd"])
        assert np.all(np.abs(g["M"] - o["M"]) <= ATT_TOL * o["M"][:, :1])


@pytest.mark.parametrize("gdir", [(0, 0, 1.0), (0.6, 0.0, 0.8)])
def test_pfgse_grad_g_matches_finite_differences(engine, gdir):
    lab, w = setup(engine, seed=5)
    steps = np.array([30, 120], np.int32)
    d = np.asarray(gdir, np.float64)
    d = d / np.linalg.norm(d)
    kscale = (1.0 * 1e-3) * (42.576 * 2 * np.pi * 1e6) * 1e-8  # dk/dg per G/cm, pulse 1 ms
    gvals = np.linspace(0.0, 120.0, 9)
    kv = np.outer(gvals * kscale, d)
    f = dfactor(10.0)
    dM = engine.pfgse_grad_g(steps, kv, 1.0, f, kscale, d)
    h = 1e-3
    Mp = engine.pfgse(steps, np.outer((gvals + h) * kscale, d), 1.0, f)["M"]
    Mm = engine.pfgse(steps, np.outer((gvals - h) * kscale, d), 1.0, f)["M"]
    fd = (Mp - Mm) / (2 * h)
    np.testing.assert_allclose(dM, fd, rtol=1e-5, atol=1e-7 * len(w[0]))


@pytest.mark.parametrize("gdir", [(0, 0, 1.0), (1.0, 0, 0), (0.6, 0.0, 0.8), (1.0, 1.0, 1.0)])
@pytest.mark.parametrize("bc", ["noflux", "periodic"])
def test_pfgse_grad_g_matches_fp64_pathwise_oracle(engine, oracle, gdir, bc):
    """rwnmr_pfgse_grad_g against the oracle's FP64 pathwise dM/dg on the same trajectories:
    relative 1e-10 (the GPU's energies are rounded once to 2^-63, its sines to 2^-61), with an
    absolute floor of 1e-12 of the largest derivative for entries that cancel to near zero."""
    lab, w = setup(engine, seed=5)
    steps = np.array([30, 120, 400], np.int32)
    d = np.asarray(gdir, np.float64)
    d = d / np.linalg.norm(d)
    kscale = (1.0 * 1e-3) * (42.576 * 2 * np.pi * 1e6) * 1e-8
    gvals = np.linspace(0.0, 120.0, 9)
    kv = np.outer(gvals * kscale, d)
    f = dfactor(10.0)
    dM = engine.pfgse_grad_g(steps, kv, 1.0, f, kscale, d, bc=bc)
    o = oracle.pfgse_grad_g(lab, w, f, steps, kv, 1.0, kscale, d, bc=bc, threads=4)
    assert np.all(dM[:, 0] == 0.0)
    np.testing.assert_allclose(dM, o, rtol=1e-10, atol=1e-12 * np.abs(o).max())


def test_pfgse_per_walker_dfactor(engine, golden):
    """RHO_TYPE sigmoid: the reference's per-walker decrease factors give its attenuations; equal
    per-walker factors reproduce the per-phase tables on both the axis and the general path."""
    gd = golden
    engine.upload_labels(gd["img_a"])
    engine.upload_walkers(gd["pfgse_x0"], gd["pfgse_y0"], gd["pfgse_z0"], gd["pfgse_seed0"])
    engine.set_walker_dfactor(gd["pfgse_sig_dfactor"])
    g = engine.pfgse(gd["pfgse_steps"], gd["pfgse_kvec"], 1.0, None)
    Mkt = g["M"] / g["esum"][:, None]
    assert np.all(np.abs(Mkt - gd["pfgse_sig_Mkt"]) <= ATT_TOL)
    lab, w = setup(engine, seed=6)
    steps = np.array([20, 90, 300], np.int32)
    f = dfactor(12.0)
    engine.set_walker_dfactor(np.full(len(w[0]), f))
    for gdir in ((0, 0, 90.0), (30.0, 40.0, 20.0)):
        kv = kvecs(8, gdir)
        a = engine.pfgse(steps, kv, 1.0, f)
        b = engine.pfgse(steps, kv, 1.0, None)
        assert np.array_equal(a["esum"], b["esum"]) and np.array_equal(a["M"], b["M"])


def test_pfgse_general_direction_rejects_huge_wavevectors(engine):
    setup(engine)
    kv = kvecs(4, (30.0, 40.0, 20.0))
    kv[-1] *= 1e16
    with pytest.raises(Exception, match="k res"):
        engine.pfgse(np.array([10, 20], np.int32), kv, 1.0, dfactor(10.0))
