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
    maximum of b (region 0, outside the phantom, excluded)."""
    ma, sa = batch_mean_sigma(acc_a[1:], acc2_a[1:], nbatch)
    mb, sb = batch_mean_sigma(acc_b[1:], acc2_b[1:], nbatch)
    sel = mb > dmax_frac * mb.max()
    sig = np.sqrt(sa[sel] ** 2 + sb[sel] ** 2)
    z = (ma[sel] - mb[sel]) / np.where(sig > 0, sig, np.inf)
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
