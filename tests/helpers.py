"""Shared set-up for the parity tests: one lattice, fed to the GPU library and the oracle."""
import numpy as np

import ether_gb300 as eg
from oracle import pyoracle as po

KB = eg.KB_EV


def beta_of(kT_over_J, J_mev=1.0):
    """beta (1/eV) at k_B T = kT_over_J * |J| with J in meV."""
    return 1.0 / (kT_over_J * abs(J_mev) * 1e-3)


def random_ising(lat, seed):
    rng = np.random.default_rng(seed)
    ion = lat.ion.copy()
    ion[:, 1:3] = 0.0
    ion[:, 3] = rng.choice([-1.0, 1.0], size=lat.N)
    return ion


def random_xyz(lat, seed):
    rng = np.random.default_rng(seed)
    ion = lat.ion.copy()
    v = rng.normal(size=(lat.N, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    v = v.astype(np.float32).astype(np.float64)
    ion[:, 1:4] = v
    ion[:, 5] = rng.uniform(-np.pi, np.pi, size=lat.N).astype(np.float32)
    return ion


def make_pair(lat, model, shells_J, s=(1.0,), replicas=1, seed=1992, flags=0, para=None,
              **kw):
    """GPU Sweep and oracle System on the same lattice and couplings."""
    nsp = lat.n_species
    j = eg.couplings(nsp, shells_J, list(s), para=para)
    sw = eg.Sweep.from_lattice(lat, j, np.asarray(s, float), model, replicas=replicas,
                               seed=seed, flags=flags, **kw)
    osys = po.System.from_lattice(lat, j, np.asarray(s, float), model, **kw)
    return sw, osys


OBSERVABLES = ("E", "U_E", "C_v", "|M|", "U_M", "chi")


def assert_means_agree(mean, err, ref_mean, ref_err, n, ref_n, family_p=0.01):
    """Two runs' per-temperature observables (E, U_E, C_v, |M|, U_M, chi:
    src/observables_per_repeat.f90:29-69), each given as the mean over n (ref_n) REPEATs and
    its REPEAT error bar sqrt(sum (x - mean)^2 / (m (m - 1))), agree when every one of the K
    differences z = (mean - ref_mean) / sqrt(err^2 + ref_err^2) has a two-sided p-value (Welch:
    Student's t with the Welch-Satterthwaite degrees of freedom, since the error bars are
    themselves estimated from the REPEATs) of at least family_p / K: Bonferroni, a family-wise
    false-alarm rate of family_p (1%) whatever the correlation between the comparisons.
    Asking every z to lie within 2 sigma would fail about K/20 comparisons by chance alone."""
    from scipy import stats
    e1, e2 = np.asarray(err, dtype=np.float64), np.asarray(ref_err, dtype=np.float64)
    z = (np.asarray(mean) - np.asarray(ref_mean)) / np.sqrt(e1 ** 2 + e2 ** 2)
    assert np.all(np.isfinite(z)), z
    df = (e1 ** 2 + e2 ** 2) ** 2 / (e1 ** 4 / (n - 1) + e2 ** 4 / (ref_n - 1))
    pv = 2.0 * stats.t.sf(np.abs(z), df)
    print("MEANS K=%d max|z|=%.2f min p=%.4f (bound %.4f)" % (z.size, np.abs(z).max(), pv.min(),
                                                             family_p / z.size))
    assert np.all(pv >= family_p / z.size), (z, pv)
    return z


def assert_same_ensemble(vals, ref_vals, family_p=0.01):
    """Statistical parity of two runs from their per-REPEAT values vals, ref_vals of shape
    (T temperatures, REPEATs, 6 observables: E, U_E, C_v, |M|, U_M, chi).

    The six observables of one temperature come from the same samples and are strongly
    correlated, so they are tested jointly: per temperature, Hotelling's two-sample T^2 on the
    six REPEAT means with the pooled covariance estimated from the REPEATs,
    F = (n1 + n2 - p - 1) / (p (n1 + n2 - 2)) T^2 ~ F(p, n1 + n2 - p - 1) under equal means.
    The T tests are held to a family-wise false-alarm rate of family_p (1%) by Bonferroni:
    every p-value >= family_p / T, which holds whatever the dependence between temperatures
    (parallel tempering couples them).  Also checks each observable against the REPEAT error
    bars the reference reports (assert_means_agree): at most 2% false alarms in all."""
    from scipy import stats
    a = np.asarray(vals, dtype=np.float64)
    b = np.asarray(ref_vals, dtype=np.float64)
    T, n1, p = a.shape
    n2 = b.shape[1]
    pv = []
    for t in range(T):
        x, y = a[t], b[t]
        d = x.mean(0) - y.mean(0)
        Sp = ((n1 - 1) * np.cov(x, rowvar=False) + (n2 - 1) * np.cov(y, rowvar=False)) / (n1 + n2 - 2)
        sd = np.sqrt(np.diag(Sp))
        keep = sd > 0
        k = int(keep.sum())
        dn = d[keep] / sd[keep]
        Rn = Sp[np.ix_(keep, keep)] / np.outer(sd[keep], sd[keep])  # correlation matrix
        T2 = (n1 * n2 / (n1 + n2)) * float(dn @ np.linalg.solve(Rn, dn))
        F = (n1 + n2 - k - 1) / (k * (n1 + n2 - 2)) * T2
        pv.append(float(stats.f.sf(F, k, n1 + n2 - k - 1)))
    pv = np.array(pv)
    print("ENSEMBLE T=%d Hotelling p-values %s (bound %.4f)" %
          (T, " ".join("%.3f" % q for q in pv), family_p / T))
    assert np.all(pv >= family_p / T), pv
    err = lambda v: v.std(1, ddof=1) / np.sqrt(v.shape[1])
    assert_means_agree(a.mean(1), err(a), b.mean(1), err(b), n1, n2, family_p)
    return pv
