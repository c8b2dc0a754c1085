"""Statistical comparison of two independent tally estimates."""
import numpy as np
from scipy import stats as sst


def compare(m1, s1, m2, s2, z=3.0):
    """Per-bin combined-sigma test and chi-square over the bins whose
    combined variance is positive.  Returns (frac_within_z, chi2, dof, p)."""
    m1, s1, m2, s2 = (np.asarray(a, np.float64) for a in (m1, s1, m2, s2))
    var = s1 ** 2 + s2 ** 2
    both_zero = (m1 == 0) & (m2 == 0)
    ok = var > 0
    d = m1 - m2
    within = np.where(ok, np.abs(d) <= z * np.sqrt(np.where(ok, var, 1.0)), both_zero | (d == 0))
    chi2 = float(np.sum(d[ok] ** 2 / var[ok]))
    dof = int(ok.sum())
    p = float(sst.chi2.sf(chi2, dof)) if dof > 0 else 1.0
    return float(within.mean()) if within.size else 1.0, chi2, dof, p


def assert_agree(m1, s1, m2, s2, what="", p_min=1e-4, frac_min=0.98):
    frac, chi2, dof, p = compare(m1, s1, m2, s2)
    assert frac >= frac_min and p >= p_min, \
        f"{what}: {frac:.3f} of bins within 3 sigma, chi2 {chi2:.1f} / {dof} dof, p = {p:.2e}"
    return frac, chi2, dof, p


def resolved(m1, s1, m2, s2, r_max=0.2):
    """Bins that both estimates resolve: nonzero means with relative error
    R <= r_max.  A rare-event bin scored by a few histories has a
    heavy-tailed estimate whose standard error is itself unreliable (a run
    may score it zero times and report sigma = 0), so a combined-sigma test
    there measures luck, not agreement."""
    m1, s1, m2, s2 = (np.asarray(a, np.float64) for a in (m1, s1, m2, s2))
    return (m1 != 0) & (m2 != 0) & (s1 <= r_max * np.abs(m1)) & (s2 <= r_max * np.abs(m2))
