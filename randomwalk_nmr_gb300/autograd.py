"""torch.autograd wrappers of the GPU walks.

* :func:`cpmg_decay` -- the CPMG echo train ``M(t_e) = exp(-t_e/T2b) * sum_w E_w(e) / N`` as a
  differentiable function of the surface relaxivity of each material phase and of the bulk T2.
  Forward is one GPU walk. When rho needs a gradient and every decrease factor is positive, that
  walk also sums the forward sensitivities sum_w E_w(e) c_wq(e) exactly (``rwnmr_cpmg_run_sens``)
  and backward is host arithmetic, d echo_sum / d f_q = sens_q / f_q; otherwise forward is
  ``rwnmr_cpmg_run`` and backward the seed-replay adjoint kernel (``rwnmr_cpmg_adjoint``), which
  replays every trajectory from its stored RNG seed. For fixed trajectories the echo train is
  smooth in rho and T2b, which is what these derivatives are (pathwise derivatives under common
  random numbers).
* :func:`pfgse_attenuation` -- PFGSE attenuation ``M(g_j, Delta)/M(0, Delta)`` as a function of the
  gradient strengths g_j along a fixed direction, backward through ``rwnmr_pfgse_grad_g``.

The relaxivity-to-collision-factor map is the reference's Walker::computeDecreaseFactor
(Walker/walker.h:203-209): f = 1 - (2/3) rho res / (D0 1e3); bulk relaxation and normalisation
follow NMR_cpmg::applyBulk / normalizeSignal (NMR_cpmg.cpp:346-384).
"""
from __future__ import annotations

import numpy as np
import torch

from .engine import Engine


def echo_times(n_echoes: int, steps_per_echo: int, dt: float) -> np.ndarray:
    """Signal times as NMR_cpmg builds them (NMR_cpmg.cpp:121-130): accumulated echo spacing."""
    out = np.zeros(n_echoes + 1)
    t = 0.0
    for e in range(n_echoes):
        t += steps_per_echo * dt
        out[e + 1] = t
    return out


class _CpmgDecay(torch.autograd.Function):
    @staticmethod
    def forward(ctx, rho, t2b, engine, n_echoes, steps_per_echo, res, d0, bc, shift):
        rho_np = rho.detach().cpu().double().numpy().reshape(-1)
        dfdrho = -(2.0 / 3.0) * res / (d0 * 1e3)
        f = 1.0 + dfdrho * rho_np
        ctx.sens = None
        if ctx.needs_input_grad[0] and np.all(f > 0.0):
            out = engine.cpmg_sens(n_echoes, steps_per_echo, f, bc=bc, shift=shift)
            raw, ctx.sens = out["echo_sum"], out["sens"]
        else:
            raw = engine.cpmg(n_echoes, steps_per_echo, f, bc=bc, shift=shift)["echo_sum"]
        dt = res * res / (6.0 * d0)
        t = echo_times(n_echoes, steps_per_echo, dt)
        T2 = float(t2b.detach().cpu())
        bulk = np.exp(-t / T2)
        n0 = raw[0]
        M = raw * bulk / n0
        ctx.engine = engine
        ctx.args = (n_echoes, steps_per_echo, bc, shift, f, dfdrho, T2, n0)
        ctx.save_for_backward(torch.from_numpy(t), torch.from_numpy(bulk), torch.from_numpy(M))
        ctx.rho_meta = (rho.dtype, rho.device, rho.shape)
        ctx.t2b_meta = (t2b.dtype, t2b.device, t2b.shape)
        return torch.from_numpy(M).to(device=rho.device)

    @staticmethod
    def backward(ctx, gM):
        t, bulk, M = ctx.saved_tensors
        n_echoes, spe, bc, shift, f, dfdrho, T2, n0 = ctx.args
        g = gM.detach().cpu().double().numpy()
        grad_rho = grad_t2 = None
        if ctx.needs_input_grad[0]:
            g_raw = g * bulk.numpy() / n0
            if ctx.sens is not None:
                gf = (g_raw @ ctx.sens) / f  # no walk: the forward sensitivities
            else:
                gf = ctx.engine.cpmg_adjoint(n_echoes, spe, f, g_raw, bc=bc, shift=shift)
            dt_, dev, shape = ctx.rho_meta
            grad_rho = torch.from_numpy(gf * dfdrho).to(dtype=dt_, device=dev).reshape(shape)
        if ctx.needs_input_grad[1]:
            # d exp(-t/T2)/dT2 = exp(-t/T2) t / T2^2
            val = float(np.sum(g * M.numpy() * t.numpy() / (T2 * T2)))
            dt_, dev, shape = ctx.t2b_meta
            grad_t2 = torch.full(shape, val, dtype=dt_, device=dev)
        return grad_rho, grad_t2, None, None, None, None, None, None, None


def cpmg_decay(rho: torch.Tensor, t2b: torch.Tensor, engine: Engine, n_echoes: int, steps_per_echo: int,
               res: float = 1.0, d0: float = 2.5, bc: str = "noflux", shift: int = 0) -> torch.Tensor:
    """Normalised CPMG echo train [n_echoes+1] of the engine's image and walkers; differentiable in
    rho (one relaxivity per material phase, um/s) and t2b (bulk T2, ms)."""
    return _CpmgDecay.apply(rho, t2b, engine, n_echoes, steps_per_echo, res, d0, bc, shift)


class _PfgseAttenuation(torch.autograd.Function):
    @staticmethod
    def forward(ctx, g, engine, steps, direction, kscale, res, dfactor, bc, shift):
        gnp = g.detach().cpu().double().numpy().reshape(-1)
        d = np.asarray(direction, np.float64)
        d = d / np.linalg.norm(d)
        kv = np.outer(gnp * kscale, d)
        out = engine.pfgse(steps, kv, res, dfactor, bc=bc, shift=shift)
        A = out["M"] / out["esum"][:, None]
        ctx.engine = engine
        ctx.args = (steps, kv, res, dfactor, kscale, d, bc, shift, out["esum"])
        ctx.meta = (g.dtype, g.device, g.shape)
        return torch.from_numpy(A).to(device=g.device)

    @staticmethod
    def backward(ctx, gA):
        steps, kv, res, dfactor, kscale, d, bc, shift, esum = ctx.args
        dM = ctx.engine.pfgse_grad_g(steps, kv, res, dfactor, kscale, d, bc=bc, shift=shift)
        gnp = gA.detach().cpu().double().numpy()
        grad = np.sum(gnp * dM / esum[:, None], axis=0)
        dt_, dev, shape = ctx.meta
        return torch.from_numpy(grad).to(dtype=dt_, device=dev).reshape(shape), None, None, None, None, None, None, None, None


def pfgse_attenuation(g: torch.Tensor, engine: Engine, steps, direction, kscale: float, res: float = 1.0,
                      dfactor=1.0, bc: str = "noflux", shift: int = 0) -> torch.Tensor:
    """Attenuation [n_delta][n_g] for gradient strengths g [n_g] (G/cm) along `direction`; k = kscale * g.
    kscale = pulse_width[ms] 1e-3 * gamma[rad/(s T)] 1e6 * 1e-8 (NMR_pfgse.cpp:483-486)."""
    return _PfgseAttenuation.apply(g, engine, steps, direction, kscale, res, dfactor, bc, shift)
