"""Exact thermodynamics of the nearest-neighbour Ising model on a finite m x n square torus.

Test infrastructure.  The partition function is Kaufman's closed form (B. Kaufman, Phys. Rev.
76, 1232 (1949); with the sign convention for gamma_0 of A. E. Ferdinand and M. E. Fisher,
Phys. Rev. 185, 832 (1969)), for H = -J sum_<ij> s_i s_j and K = J / kT:

    Z = 1/2 (2 sinh 2K)^(mn/2) (Z1 + Z2 + Z3 + Z4)
    Z1 = prod_{r<n} 2 cosh(m g_{2r+1} / 2)     Z2 = prod_{r<n} 2 sinh(m g_{2r+1} / 2)
    Z3 = prod_{r<n} 2 cosh(m g_{2r} / 2)       Z4 = prod_{r<n} 2 sinh(m g_{2r} / 2)
    cosh g_l = cosh 2K coth 2K - cos(pi l / n)  (l >= 1),   g_0 = 2K + ln tanh K.

The energy and heat capacity per site follow as derivatives of ln Z in K (mpmath at 60
digits).  brute_force_ln_z enumerates all 2^(mn) states of a small torus and pins the formula.
"""
import mpmath as mp
import numpy as np

mp.mp.dps = 60


def ln_z(K, m, n):
    K = mp.mpf(K)
    c = mp.cosh(2 * K) / mp.tanh(2 * K)

    def gamma(l):
        if l == 0:
            return 2 * K + mp.log(mp.tanh(K))
        return mp.acosh(c - mp.cos(mp.pi * l / n))

    odd = [gamma(2 * r + 1) for r in range(n)]
    even = [gamma(2 * r) for r in range(n)]
    z1 = mp.fprod(2 * mp.cosh(m * g / 2) for g in odd)
    z2 = mp.fprod(2 * mp.sinh(m * g / 2) for g in odd)
    z3 = mp.fprod(2 * mp.cosh(m * g / 2) for g in even)
    z4 = mp.fprod(2 * mp.sinh(m * g / 2) for g in even)
    return mp.log(mp.mpf(1) / 2) + (m * n / mp.mpf(2)) * mp.log(2 * mp.sinh(2 * K)) + mp.log(z1 + z2 + z3 + z4)


def energy_cv(K, m, n):
    """Mean energy per site in units of J and heat capacity per site in units of k_B."""
    N = m * n
    d1 = mp.diff(lambda k: ln_z(k, m, n), K, 1)
    d2 = mp.diff(lambda k: ln_z(k, m, n), K, 2)
    e = -d1 / N                       # <H> / (N J)
    cv = mp.mpf(K) ** 2 * d2 / N      # Var(H) / (N k_B^2 T^2)
    return float(e), float(cv)


def brute_force_ln_z(K, m, n):
    N = m * n
    states = np.arange(1 << N, dtype=np.int64)
    s = 1 - 2 * ((states[:, None] >> np.arange(N)) & 1).astype(np.int64)  # (2^N, N) of +-1
    g = s.reshape(-1, m, n)
    bonds = (g * np.roll(g, 1, axis=1)).sum(axis=(1, 2)) + (g * np.roll(g, 1, axis=2)).sum(axis=(1, 2))
    vals, counts = np.unique(bonds, return_counts=True)
    return mp.log(mp.fsum(int(c) * mp.exp(mp.mpf(K) * int(v)) for v, c in zip(vals, counts)))
