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


def assert_same_ensemble(mean, err, ref_mean, ref_err, family_p=0.01):
    """Statistical parity of two runs' per-temperature observables (E, U_E, C_v, |M|, U_M,
    chi: src/observables_per_repeat.f90:29-69), each given as the mean over REPEATs and its
    REPEAT error bar sqrt(sum (x - mean)^2 / (m (m - 1))).

    z = (mean - ref_mean) / sqrt(err^2 + ref_err^2) for each of the K comparisons.  The rule,
    at a family-wise false-alarm rate of `family_p` (1%):
      * every |z| <= z*, the two-sided Bonferroni bound Phi^-1(1 - family_p / (2K)), which
        holds whatever the correlation between the comparisons (the six observables of one
        temperature share their samples);
      * sum z^2 <= the (1 - family_p) quantile of chi^2 with K degrees of freedom: a check
        that no small systematic offset is spread over many comparisons (exact for
        independent comparisons).
    Asking every z to lie within 2 sigma would fail about K/20 comparisons by chance alone."""
    from scipy import stats
    z = (np.asarray(mean) - np.asarray(ref_mean)) / np.sqrt(np.asarray(err) ** 2 + np.asarray(ref_err) ** 2)
    assert np.all(np.isfinite(z)), z
    K = z.size
    zmax = stats.norm.isf(family_p / (2 * K))
    chi2 = float((z ** 2).sum())
    chi2_max = stats.chi2.isf(family_p, K)
    print("ENSEMBLE K=%d max|z|=%.2f (bound %.2f) chi2=%.1f (bound %.1f)" %
          (K, np.abs(z).max(), zmax, chi2, chi2_max))
    assert np.abs(z).max() <= zmax, z
    assert chi2 <= chi2_max, (chi2, chi2_max, z)
    return z
