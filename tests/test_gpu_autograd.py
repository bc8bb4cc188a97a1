"""torch.autograd wrappers: gradients against central finite differences under common random
numbers (the same seeds, so the trajectories are fixed)."""
import numpy as np
import pytest
import torch

from randomwalk_nmr_gb300 import Engine, host
from randomwalk_nmr_gb300.autograd import cpmg_decay, pfgse_attenuation

pytestmark = pytest.mark.gpu


def engine_for(n_phases, seed=3, n=4000):
    lab, _ = host.synth_spheres((26, 24, 28), 2.0, 5.0, 0.4, n_phases, seed=seed)
    blocks, _ = host.pack_blocks(lab)
    x, y, z, s, _ = host.place_walkers(blocks, lab.shape, n, seed)
    e = Engine(0)
    e.upload_labels(lab, n_phases)
    e.upload_walkers(x, y, z, s)
    return e


@pytest.mark.parametrize("n_phases", [1, 3])
def test_cpmg_decay_gradients(n_phases):
    eng = engine_for(n_phases)
    rho = torch.tensor([12.0, 30.0, 4.0][:n_phases], dtype=torch.float64, requires_grad=True)
    t2b = torch.tensor(900.0, dtype=torch.float64, requires_grad=True)
    w = torch.linspace(0.0, 1.0, 81, dtype=torch.float64) ** 2
    M = cpmg_decay(rho, t2b, eng, 80, 2)
    assert abs(float(M[0].detach()) - 1.0) < 1e-15
    loss = (w * M).sum()
    launches = eng.launch_count
    loss.backward()
    assert eng.launch_count == launches  # the forward walk's sensitivities: no second walk

    def L(r, T):
        with torch.no_grad():
            return float((w * cpmg_decay(torch.tensor(r, dtype=torch.float64), torch.tensor(T, dtype=torch.float64),
                                         eng, 80, 2)).sum())

    base = rho.detach().numpy()
    for q in range(n_phases):
        h = 1e-3
        rp, rm = base.copy(), base.copy()
        rp[q] += h
        rm[q] -= h
        fd = (L(rp, 900.0) - L(rm, 900.0)) / (2 * h)
        np.testing.assert_allclose(rho.grad[q].item(), fd, rtol=1e-6)
    fdT = (L(base, 900.0 + 1e-2) - L(base, 900.0 - 1e-2)) / 2e-2
    np.testing.assert_allclose(t2b.grad.item(), fdT, rtol=1e-6)
    eng.close()


def test_pfgse_attenuation_gradient():
    eng = engine_for(1, seed=6)
    kscale = (1.0 * 1e-3) * (42.576 * 2 * np.pi * 1e6) * 1e-8
    steps = np.array([30, 90], np.int32)
    g = torch.linspace(0.0, 80.0, 9, dtype=torch.float64).requires_grad_(True)
    A = pfgse_attenuation(g, eng, steps, (0, 0, 1), kscale, dfactor=0.995)
    wts = torch.rand(A.shape, dtype=torch.float64, generator=torch.Generator().manual_seed(0))
    (wts * A).sum().backward()
    h = 1e-4
    for j in range(1, 9):
        gp = g.detach().clone()
        gm = g.detach().clone()
        gp[j] += h
        gm[j] -= h
        with torch.no_grad():
            fd = float(((wts * pfgse_attenuation(gp, eng, steps, (0, 0, 1), kscale, dfactor=0.995)).sum() -
                        (wts * pfgse_attenuation(gm, eng, steps, (0, 0, 1), kscale, dfactor=0.995)).sum()) / (2 * h))
        np.testing.assert_allclose(g.grad[j].item(), fd, rtol=1e-5, atol=1e-9)
    eng.close()
