"""GPU parity at the full image sizes of the benchmark configurations, through the C ABI.

* plain CPMG, 100^3 sphere pack, 10,000 walkers, 2000 echoes x 3 steps: against the reference's own
  CPU walk (tests/golden/reference_c1.npz);
* two-phase CPMG, 400^3 labels, 20,000 echoes at one step per echo: the headline image and echo count
  on a 65,536-walker population against the CPU oracle;
* PFGSE, 256^3 sphere pack, 64 gradients x 10 exposure times (walk to 1500 steps): against the
  reference's own CPU sequence on 16,384 walkers (tests/golden/reference_c3.npz) and against the
  oracle on 65,536 walkers.

Integers (positions, RNG states, collision counts, fixed-point sums) must be bit-exact, echo sums
within 1e-12 relative, attenuations within 1e-12 of M(0).
"""
import hashlib
import os

import numpy as np
import pytest

from conftest import ROOT, dfactor
from randomwalk_nmr_gb300 import fx_to_float, host

pytestmark = pytest.mark.gpu

ECHO_RTOL = 1e-12  # echo amplitudes relative to the reference's / oracle's FP64 sums
ATT_TOL = 1e-12  # |M_gpu - M_ref| <= ATT_TOL * M(k=0)
THREADS = os.cpu_count() or 1


def golden_file(name):
    return dict(np.load(os.path.join(ROOT, "tests", "golden", name)))


def kvecs(n_g, gmax, pulse_ms=1.0, gamma=42.576 * 2 * np.pi):
    """k_j as NMR_PFGSE builds them (NMR_pfgse.cpp:272-313, 483-486): accumulated gradient steps."""
    gap = np.asarray(gmax, np.float64) / (n_g - 1)
    g = np.zeros(3)
    out = []
    for _ in range(n_g):
        out.append([(pulse_ms * 1e-3) * (gamma * 1e6) * (gi * 1e-8) for gi in g])
        g = g + gap
    return np.array(out)


def test_c1_plain_cpmg_full_size_matches_reference(engine):
    c1 = golden_file("reference_c1.npz")
    lab, _ = host.synth_spheres((100, 100, 100), 4.0, 10.0, 0.30, 1, seed=1)
    blocks, _ = host.pack_blocks(lab)
    assert np.array_equal(blocks, c1["c1_blocks"])
    engine.upload_labels(lab, 1)
    engine.upload_walkers(c1["c1_x0"], c1["c1_y0"], c1["c1_z0"], c1["c1_seed0"])
    f = float(c1["c1_dfactor"][0])
    g = engine.cpmg(2000, 3, f)
    st = engine.download_walkers()
    assert np.array_equal(st["x"], c1["c1_xf"])
    assert np.array_equal(st["y"], c1["c1_yf"])
    assert np.array_equal(st["z"], c1["c1_zf"])
    assert np.array_equal(st["seed"], c1["c1_seedf"])
    assert np.array_equal(st["collisions"][:, 0], c1["c1_coll"])
    assert np.array_equal(g["echo_coll"][:, 0], c1["c1_coll_per_echo"])
    np.testing.assert_allclose(g["echo_sum"], c1["c1_energy_sum"], rtol=ECHO_RTOL, atol=0)
    # the last echo's exact sum equals the reference's per-walker energies rounded to 2^-63 each
    fx_last = sum(int(round(e * 2.0**63)) for e in c1["c1_energy"])
    l0, l1, l2 = (int(v) for v in g["echo_fx"][-1])
    assert l0 + (l1 << 21) + (l2 << 42) == fx_last


def test_c2_two_phase_full_image_and_echo_count(engine, oracle):
    lab, _ = host.synth_spheres((400, 400, 400), 6.0, 20.0, 0.25, 2, seed=2)
    blocks, _ = host.pack_blocks(lab)
    x, y, z, s, _ = host.place_walkers(blocks, lab.shape, 65_536, 7)
    res = float(np.sqrt(6.0 * 2.5 * 0.1))  # one step per 0.1 ms echo
    f = dfactor([5.0, 25.0], res=res)
    engine.upload_labels(lab, 2)
    engine.upload_walkers(x, y, z, s)
    g = engine.cpmg(20_000, 1, f)
    st = engine.download_walkers()
    o = oracle.cpmg(lab, (x, y, z, s), 20_000, 1, f, n_phases=2, threads=THREADS)
    assert np.array_equal(st["x"], o["xf"]) and np.array_equal(st["y"], o["yf"]) and np.array_equal(st["z"], o["zf"])
    assert np.array_equal(st["seed"], o["seedf"])
    assert np.array_equal(st["collisions"], o["collf"])
    assert np.array_equal(g["echo_coll"], o["echo_coll"])
    assert np.array_equal(g["echo_fx"], o["echo_fx"])
    np.testing.assert_allclose(g["echo_sum"], o["echo_fp64"], rtol=ECHO_RTOL, atol=0)


def c3_image():
    lab, _ = host.synth_spheres((256, 256, 256), 5.0, 15.0, 0.35, 1, seed=3)
    return lab


def test_c3_pfgse_full_size_matches_reference(engine):
    c3 = golden_file("reference_c3.npz")
    lab = c3_image()
    blocks, _ = host.pack_blocks(lab)
    assert hashlib.sha256(blocks.tobytes()).hexdigest() == str(c3["c3_blocks_sha256"])
    engine.upload_labels(lab, 1)
    engine.upload_walkers(c3["c3_x0"], c3["c3_y0"], c3["c3_z0"], c3["c3_seed0"])
    g = engine.pfgse(c3["c3_steps"], c3["c3_kvec"], 1.0, float(c3["c3_dfactor"][0]))
    Mkt = g["M"] / g["esum"][:, None]
    assert np.all(np.abs(Mkt - c3["c3_Mkt"]) <= ATT_TOL)


def test_c3_pfgse_full_size_matches_oracle(engine, oracle):
    c3 = golden_file("reference_c3.npz")
    lab = c3_image()
    blocks, _ = host.pack_blocks(lab)
    x, y, z, s, _ = host.place_walkers(blocks, lab.shape, 65_536, 7)
    steps = c3["c3_steps"]  # the reference's step counts for Delta = 1-100 ms log-spaced
    assert steps[-1] == 1500
    kv = kvecs(64, (0.0, 0.0, 100.0))
    np.testing.assert_allclose(kv, c3["c3_kvec"], rtol=1e-15)
    f = dfactor(10.0)
    engine.upload_labels(lab, 1)
    engine.upload_walkers(x, y, z, s)
    g = engine.pfgse(steps, kv, 1.0, f)
    o = oracle.pfgse(lab, (x, y, z, s), f, steps, kv, 1.0, threads=THREADS)
    assert np.array_equal(g["msd"], o["msd"])
    assert np.array_equal(fx_to_float(o["esum_fx"]), g["esum"])
    assert np.all(np.abs(g["M"] - o["M"]) <= ATT_TOL * o["M"][:, :1])
