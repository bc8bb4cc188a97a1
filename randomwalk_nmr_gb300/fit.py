"""Surface-relaxivity fits on the GPU walk.

* :func:`fit_rho_batch` -- many single-phase images at once: every image carries 16 relaxivity
  candidates (a multi-start population); each iteration is one batched walk (``Batch.cpmg``) that
  returns every candidate's echo train and its exact derivative, and each candidate takes a
  Gauss-Newton step on its own least-squares misfit. The best candidate per image wins.
* :func:`fit_rho_adjoint` -- one image with several material phases: L-BFGS on the relaxivity
  vector through ``cpmg_decay``, one walk per evaluation: the walk returns the echo train and its
  exact forward sensitivities (``rwnmr_cpmg_run_sens``), so the gradient needs no second walk (the
  seed-replay adjoint ``rwnmr_cpmg_adjoint`` covers a zero decrease factor).

Both report the GPU time they spent (sum of the walk kernels' device time).
"""
from __future__ import annotations

import time

import numpy as np
import torch

from .autograd import cpmg_decay, echo_times


def decrease_factor(rho, res=1.0, d0=2.5):
    """Walker::computeDecreaseFactor (Walker/walker.h:203-209)."""
    return 1.0 - (2.0 / 3.0) * (np.asarray(rho, np.float64) * res) / (d0 * 1e3)


def fit_rho_batch(batch, targets, n_walkers, n_echoes, steps_per_echo, t2b, rho_init, res=1.0, d0=2.5,
                  bounds=(0.5, 100.0), iters=8, bc="noflux", method="auto"):
    """Fits one relaxivity per image. targets [n_images][n_echoes+1] normalised echo trains;
    n_walkers [n_images]; rho_init [n_images][16] starting candidates; method as for Batch.cpmg
    (with histograms the walk happens once, in the first iteration). Returns a dict with the best
    relaxivity and misfit per image, the candidate history and the GPU seconds spent."""
    targets = np.asarray(targets, np.float64)
    rho = np.array(rho_init, np.float64, copy=True)
    nw = np.asarray(n_walkers, np.float64)[:, None, None]
    dt = res * res / (6.0 * d0)
    bulk = np.exp(-echo_times(n_echoes, steps_per_echo, dt) / t2b)[None, None, :]
    dfdrho = -(2.0 / 3.0) * res / (d0 * 1e3)
    gpu_s = 0.0
    history = []
    loss = None
    for it in range(iters + 1):
        echo, decho = batch.cpmg(decrease_factor(rho, res, d0), n_echoes, steps_per_echo, derivatives=True, bc=bc,
                                 method=method)
        gpu_s += batch.last_kernel_ms * 1e-3
        M = echo / nw * bulk
        J = decho / nw * bulk * dfdrho
        r = M - targets[:, None, :]
        loss = np.sum(r * r, axis=2)
        history.append((rho.copy(), loss.copy()))
        if it == iters:
            break
        # Gauss-Newton step per candidate, clipped to the bounds
        step = -np.sum(r * J, axis=2) / np.maximum(np.sum(J * J, axis=2), 1e-300)
        rho = np.clip(rho + step, bounds[0], bounds[1])
    best = np.argmin(loss, axis=1)
    idx = np.arange(len(rho))
    return dict(rho=rho[idx, best], loss=loss[idx, best], candidates=rho, candidate_loss=loss, history=history,
                gpu_seconds=gpu_s, walks=iters + 1)


def fit_rho_adjoint(engine, target, rho0, n_echoes, steps_per_echo, t2b, res=1.0, d0=2.5, max_evals=40,
                    bounds=(0.5, 100.0)):
    """L-BFGS fit of a relaxivity vector (one per material phase) to a normalised echo train,
    gradients from the walk's forward sensitivities (or the seed-replay adjoint for a zero decrease
    factor). Returns a dict with rho, loss, GPU seconds and the number of walks."""
    tgt = torch.as_tensor(np.asarray(target, np.float64))
    scale = float(tgt.abs().max())
    # optimise in a bounded reparametrisation rho = lo + (hi - lo) * sigmoid(u)
    lo, hi = bounds
    r0 = np.clip(np.asarray(rho0, np.float64), lo + 1e-6, hi - 1e-6)
    u = torch.tensor(np.log((r0 - lo) / (hi - r0)), dtype=torch.float64, requires_grad=True)
    t2 = torch.tensor(float(t2b), dtype=torch.float64)
    opt = torch.optim.LBFGS([u], lr=1.0, max_iter=max_evals, max_eval=max_evals, tolerance_grad=1e-12,
                            tolerance_change=1e-15, history_size=10, line_search_fn="strong_wolfe")
    stats = dict(gpu_seconds=0.0, evals=0, walks=0)

    def closure():
        opt.zero_grad()
        rho = lo + (hi - lo) * torch.sigmoid(u)
        M = cpmg_decay(rho, t2, engine, n_echoes, steps_per_echo, res, d0)
        stats["gpu_seconds"] += engine.last_kernel_ms * 1e-3
        stats["walks"] += 1
        loss = torch.sum(((M - tgt) / scale) ** 2)
        launches = engine.launch_count
        loss.backward()
        if engine.launch_count != launches:  # an adjoint walk (the sensitivities need none)
            stats["gpu_seconds"] += engine.last_kernel_ms * 1e-3
            stats["walks"] += 1
        stats["evals"] += 1
        return loss

    t0 = time.perf_counter()
    opt.step(closure)
    with torch.no_grad():
        rho = (lo + (hi - lo) * torch.sigmoid(u)).numpy()
        M = cpmg_decay(torch.tensor(rho), t2, engine, n_echoes, steps_per_echo, res, d0)
        stats["gpu_seconds"] += engine.last_kernel_ms * 1e-3
        loss = float(torch.sum(((M - tgt) / scale) ** 2))
    return dict(rho=rho, loss=loss, gpu_seconds=stats["gpu_seconds"], evals=stats["evals"],
                walks=stats["walks"] + 1, wall_seconds=time.perf_counter() - t0)
