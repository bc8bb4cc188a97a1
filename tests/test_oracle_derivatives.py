"""The oracle's FP64 pathwise PFGSE derivative dM/dg against central finite differences of the
oracle's own phase sums (common random numbers: the trajectories do not depend on g). Runs
without a GPU; the GPU derivative is checked against this pathwise form in test_gpu_pfgse.py."""
import numpy as np
import pytest

from conftest import dfactor
from randomwalk_nmr_gb300 import host

KSCALE = (1.0 * 1e-3) * (42.576 * 2 * np.pi * 1e6) * 1e-8  # dk/dg per G/cm at a 1 ms pulse


@pytest.mark.parametrize("gdir", [(0.0, 0.0, 1.0), (0.6, 0.0, 0.8), (1.0, 1.0, 1.0)])
def test_oracle_pathwise_dMdg_matches_finite_differences(oracle, gdir):
    lab, _ = host.synth_spheres((30, 26, 28), 2.0, 6.0, 0.4, 1, seed=5)
    blocks, _ = host.pack_blocks(lab)
    w = host.place_walkers(blocks, lab.shape, 3000, 105)[:4]
    d = np.asarray(gdir, np.float64)
    d = d / np.linalg.norm(d)
    steps = np.array([30, 120], np.int32)
    g = np.linspace(0.0, 120.0, 7)
    f = dfactor(10.0)
    dM = oracle.pfgse_grad_g(lab, w, f, steps, np.outer(g * KSCALE, d), 1.0, KSCALE, d, threads=4)
    h = 1e-2
    Mp = oracle.pfgse(lab, w, f, steps, np.outer((g + h) * KSCALE, d), 1.0, threads=4)["M"]
    Mm = oracle.pfgse(lab, w, f, steps, np.outer((g - h) * KSCALE, d), 1.0, threads=4)["M"]
    fd = (Mp - Mm) / (2 * h)
    assert np.all(dM[:, 0] == 0.0)  # sin(0) = 0: no first-order change at g = 0
    # truncation error of the central difference is O(h^2 k'^2 <dR^2>) relative: well below 1e-6 here
    np.testing.assert_allclose(dM, fd, rtol=1e-6, atol=1e-9 * len(w[0]))
