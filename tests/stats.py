"""Statistical comparison of two batch-tallied dose runs."""

from __future__ import annotations

import numpy as np


def batch_mean_sigma(acc, acc2, nbatch):
    """Per-region batch mean and its standard error (the reference's batch
    method, omc_dosxyz.c:739-751), without the relative scaling."""
    m = acc / nbatch
    m2 = acc2 / nbatch
    var = np.maximum(m2 - m * m, 0.0) / (nbatch - 1)
    return m, np.sqrt(var)


def compare(acc_a, acc2_a, acc_b, acc2_b, nbatch, dmax_frac=0.2):
    """z-scores of run a against run b over regions above dmax_frac of the
    maximum of b (region 0, outside the phantom, excluded).  With the
    uncertainties estimated from nbatch batches per run, the difference over
    its estimated sigma follows a t distribution of 2(nbatch-1) degrees of
    freedom; it is mapped to a standard normal so that `consistent`
    applies."""
    from scipy import stats as S

    ma, sa = batch_mean_sigma(acc_a[1:], acc2_a[1:], nbatch)
    mb, sb = batch_mean_sigma(acc_b[1:], acc2_b[1:], nbatch)
    sel = mb > dmax_frac * mb.max()
    sig = np.sqrt(sa[sel] ** 2 + sb[sel] ** 2)
    t = (ma[sel] - mb[sel]) / np.where(sig > 0, sig, np.inf)
    z = S.norm.ppf(np.clip(S.t.cdf(t, 2 * (nbatch - 1)), 1e-300, 1 - 1e-16))
    return {
        "n": int(sel.sum()),
        "frac_2sigma": float(np.mean(np.abs(z) <= 2.0)),
        "mean_z2": float(np.mean(z * z)),
        "mean_z": float(np.mean(z)),
        "etot_a": float(acc_a[1:].sum()),
        "etot_b": float(acc_b[1:].sum()),
        "etot_rel": float((acc_a[1:].sum() - acc_b[1:].sum()) / acc_b[1:].sum()),
    }


def consistent(c, p_min=1e-4):
    """Two runs are statistically identical if the number of voxels with
    |z| > 2 is plausible under Binomial(n, 0.0455) and sum z^2 under
    chi^2(n), both at tail probability p_min (voxels are treated as
    independent)."""
    from scipy import stats as S

    n = c["n"]
    k_out = int(round((1.0 - c["frac_2sigma"]) * n))
    p_binom = float(S.binom.sf(k_out - 1, n, 0.0455)) if k_out > 0 else 1.0
    q = c["mean_z2"] * n
    p_chi2 = float(min(S.chi2.cdf(q, n), S.chi2.sf(q, n)))
    c["p_binom"], c["p_chi2"] = p_binom, p_chi2
    return p_binom > p_min and p_chi2 > p_min


def compare_runs(runs_a, runs_b, dmax_frac=0.2):
    """Two sets of K independent repeats of a per-row/per-voxel quantity
    (arrays [K, rows, voxels] or [K, voxels]).  Per entry above dmax_frac of
    its row maximum (of b's mean): the Welch statistic of the two means,
    which with K repeats per side follows a t distribution of 2(K-1)
    degrees of freedom, mapped to a standard normal so that `consistent`
    applies; plus a t statistic of the total over all entries."""
    from scipy import stats as S

    a = np.asarray(runs_a, dtype=np.float64)
    b = np.asarray(runs_b, dtype=np.float64)
    k = a.shape[0]
    ma, mb = a.mean(0), b.mean(0)
    va, vb = a.var(0, ddof=1) / k, b.var(0, ddof=1) / b.shape[0]
    sel = mb > dmax_frac * mb.max(axis=-1, keepdims=True)
    sig = np.sqrt(va[sel] + vb[sel])
    t = (ma[sel] - mb[sel]) / np.where(sig > 0, sig, np.inf)
    dof = k + b.shape[0] - 2
    z = S.norm.ppf(np.clip(S.t.cdf(t, dof), 1e-300, 1 - 1e-16))
    ta = a.reshape(k, -1).sum(1)
    tb = b.reshape(b.shape[0], -1).sum(1)
    t_tot = (ta.mean() - tb.mean()) / np.sqrt(ta.var(ddof=1) / k + tb.var(ddof=1) / b.shape[0])
    return {"n": int(sel.sum()), "frac_2sigma": float(np.mean(np.abs(z) <= 2.0)), "mean_z2": float(np.mean(z * z)),
            "etot_rel": float(ta.mean() / tb.mean() - 1), "t_total": float(t_tot)}
