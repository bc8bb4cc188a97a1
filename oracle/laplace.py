"""Oracle: CPU restatement of the reference's T2 (Laplace) inversion, in numpy.

TEST INFRASTRUCTURE ONLY: the tests use it as the checker of the library's T2 inversion
(rwnmr_t2_* in the host library). Nothing in the product imports it.

Restated from the reference's Laplace module (src/backend/Laplace), which needs Eigen and does not
compile here, so parity is pinned on independent implementations of the same published
algorithms (numpy's LAPACK SVD for the L-curve, scipy's Lawson-Hanson NNLS for the solve) and on
synthetic decays with known T2 distributions, not on outputs of the reference's own build.

Steps (NMR_cpmg::applyLaplace, NMR_Simulation/NMR_cpmg.cpp:387-453):
  1. drop the t = 0 point of the decay;
  2. optional Gaussian noise (NOISE_AMP), added before pruning (nmrinv_core.cpp:357-391);
  3. log-spaced prune-averaging of the times (geometric means) and amplitudes (arithmetic
     means) to PRUNE_NUM points (nmrinv_core.cpp:145-239);
  4. kernel A[i, j] = exp(-t_i / T2_j) over log-spaced T2 bins (nmrinv_core.cpp:99-142);
  5. Tikhonov lambda = the L-curve corner: thin SVD of A, curvature of (||x||, ||r||) over
     NUM_LAMBDAS log-spaced lambdas, the first maximum (TikhonovSolver.cpp:14-116);
  6. non-negative least squares on [A; lambda I] x = [b; 0] (Lawson-Hanson active set,
     Laplace/include/NNLS.hpp:289-406; nmrinv_core.cpp:317-336, 402-481).
"""
from __future__ import annotations

import math

import numpy as np


def linspace(start: float, end: float, size: int) -> list[float]:
    """Incremental linspace with the final point (vector_funcs.cpp:85-100): value += step."""
    step = (end - start) / (size - 1)
    out, v = [], start
    for _ in range(size):
        out.append(v)
        v += step
    return out


def logspace(start: float, end: float, size: int) -> np.ndarray:
    """10 ** linspace (vector_funcs.cpp:102-107)."""
    return np.array([math.pow(10.0, v) for v in linspace(start, end, size)])


def t2_bins(min_t2: float, max_t2: float, n: int, use_log: bool = True) -> np.ndarray:
    """get_t2_bins (nmrinv_core.cpp:129-142)."""
    if use_log:
        return logspace(math.log10(min_t2), math.log10(max_t2), n)
    return np.array(linspace(min_t2, max_t2, n))


def pruning_slices(times, num_pruning: int):
    """get_nmr_pruning_slices (nmrinv_core.cpp:145-179): (pruned index, raw begin, raw end) per
    log-spaced slice, after the leading points that stay as they are."""
    t = [float(v) for v in times]
    n = len(t)
    if num_pruning < 3 or n <= num_pruning:
        return None  # nothing to prune (the reference reads past the times here)
    lg = [math.log10(v) for v in t]
    d = (lg[n - 1] - lg[0]) / (num_pruning - 1)
    nl = [lg[0] + d * i for i in range(num_pruning)]
    ps = 1
    while ps < num_pruning - 1 and math.pow(10.0, nl[ps]) - t[ps] <= 0.0:
        ps += 1
    ps -= 1
    ib = 0
    while ib < n and lg[ib] - nl[ps] <= 0.0:
        ib += 1
    if ib >= n:
        return None
    out = []
    for pi in range(ps, num_pruning - 1):
        b0, lo, hi = ib, nl[pi], nl[pi + 1]
        while ib < n and lo <= lg[ib] < hi:
            ib += 1
        out.append((pi, b0, ib))
    return out


def prune(data, slices, num_pruning: int, use_log: bool) -> np.ndarray:
    """prune_nmr_data_from_slices for one curve (nmrinv_core.cpp:182-239)."""
    data = [float(v) for v in data]
    out = np.zeros(num_pruning)
    ps = slices[0][0]
    out[:ps] = data[:ps]
    for pi, b0, b1 in slices:
        if use_log:
            s = 0.0
            for v in data[b0:b1]:
                s += math.log10(v)
            out[pi] = math.pow(10.0, s / (b1 - b0)) if b1 > b0 else float("nan")
        else:
            s = 0.0
            for v in data[b0:b1]:
                s += v
            out[pi] = s / (b1 - b0) if b1 > b0 else float("nan")
    out[num_pruning - 1] = data[-1]
    return out


def kernel(times, bins) -> np.ndarray:
    """create_nmr_inversion_matrix without the Tikhonov rows (nmrinv_core.cpp:99-126)."""
    t = np.asarray(times, np.float64)[:, None]
    return np.exp(-t / np.asarray(bins, np.float64)[None, :])


def lcurve(A: np.ndarray, b: np.ndarray, min_lambda: float, max_lambda: float, num_lambdas: int):
    """TikhonovSolver::find_best_lambda + set_Lcurve_values_from_lambda (TikhonovSolver.cpp:14-116).
    Returns (best index, lambdas, curvature, solution norms, residual norms, singular values)."""
    U, s, _ = np.linalg.svd(A, full_matrices=False)
    keep = 0
    while keep < len(s) and s[keep] != 0.0:
        keep += 1
    s = s[:keep]
    uatb = U[:, :keep].T @ b
    d = uatb / s
    d2 = d * d
    lambdas = logspace(min_lambda, max_lambda, num_lambdas)
    curv = np.empty(num_lambdas)
    sn = np.empty(num_lambdas)
    rn = np.empty(num_lambdas)
    for k, lam in enumerate(lambdas):
        sql = lam * lam
        s2 = s * s
        ft = s2 / (s2 + sql)
        om = 1.0 - ft
        eta = float(np.sum((ft * d) ** 2))
        rho = float(np.sum((om * uatb) ** 2))
        deta = float(np.sum(om * ft * ft * d2)) * (-4.0 / lam)
        mult = -2.0 * eta * rho / deta
        num = sql * deta * rho + 2.0 * lam * eta * rho + sql * sql * eta * deta
        den = (sql * eta * eta + rho * rho) ** 1.5
        curv[k] = mult * num / den
        sn[k] = math.sqrt(eta)
        rn[k] = math.sqrt(rho)
    best = int(np.argmax(curv))
    return best, lambdas, curv, sn, rn, s


def nnls(A: np.ndarray, b: np.ndarray, eps: float = 1e-10, max_solves: int | None = None) -> np.ndarray:
    """Lawson-Hanson NNLS with the reference's choices (NNLS.hpp:289-406): the passive set grows
    by the free index of largest gradient until no gradient exceeds eps; an infeasible
    least-squares step moves to the boundary and drops the one passive index that hits zero
    first. Least squares on the passive columns by numpy lstsq."""
    m, n = A.shape
    AtA = A.T @ A
    Atb = A.T @ b
    x = np.zeros(n)
    perm = list(range(n))
    npas = 0
    solves = 0
    max_solves = max_solves or 30 * n
    while True:
        w = Atb - AtA @ x
        if npas == n:
            return x
        zi = max(range(npas, n), key=lambda i: (w[perm[i]], -i))
        if w[perm[zi]] - eps < 0 or npas >= m:
            return x
        perm[zi], perm[npas] = perm[npas], perm[zi]
        npas += 1
        while True:
            if solves >= max_solves:
                raise RuntimeError("NNLS did not converge")
            cols = perm[:npas]
            z, *_ = np.linalg.lstsq(A[:, cols], b, rcond=None)
            solves += 1
            y = np.zeros(n)
            y[cols] = z
            alpha, rem = np.inf, -1
            for i in range(npas):
                j = perm[i]
                if y[j] <= 0:
                    t = -x[j] / (y[j] - x[j])
                    if alpha > t:
                        alpha, rem = t, i
            if rem < 0:
                x = y
                break
            for i in range(npas):
                j = perm[i]
                x[j] += alpha * (y[j] - x[j])
            perm[rem], perm[npas - 1] = perm[npas - 1], perm[rem]
            npas -= 1


def invert(times, amps, min_t2=0.1, max_t2=10000.0, use_log=True, num_t2_bins=128, min_lambda=-4.0,
           max_lambda=2.0, num_lambdas=512, prune_num=512, noise=None, force_lambda=None):
    """NMR_cpmg::applyLaplace on a decay whose first point is t = 0 (NMR_cpmg.cpp:387-453).
    noise: the Gaussian draws to add (length len(times) - 1) or None; force_lambda: solve at this
    lambda instead of the L-curve's (for comparing solves when two curvatures tie). Returns a dict."""
    t = np.asarray(times, np.float64)[1:]
    a = np.asarray(amps, np.float64)[1:]
    if noise is not None:
        a = a + np.asarray(noise, np.float64)
    bins = t2_bins(min_t2, max_t2, num_t2_bins, use_log)
    sl = pruning_slices(t, prune_num) if prune_num > 0 else None
    if sl is not None:
        tu = prune(t, sl, prune_num, True)
        au = prune(a, sl, prune_num, False)
    else:
        tu, au = t, a
    A = kernel(tu, bins)
    best, lambdas, curv, sn, rn, s = lcurve(A, au, min_lambda, max_lambda, num_lambdas)
    lam = lambdas[best] if force_lambda is None else force_lambda
    Aa = np.vstack([A, lam * np.eye(num_t2_bins)]) if lam else A
    ba = np.concatenate([au, np.zeros(num_t2_bins)]) if lam else au
    x = nnls(Aa, ba)
    return dict(bins=bins, amps=x, lam=lam, best=best, used_times=tu, used_amps=au, curvature=curv,
                singular_values=s, lambdas=lambdas)
