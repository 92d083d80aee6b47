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
