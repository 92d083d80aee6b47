"""Integrated autocorrelation time with Sokal's automatic windowing.

tau_int(W) = 1/2 + sum_{t=1..W} rho(t); the window W is the smallest with W >= c tau_int(W)
(c = 6 by default).  Error: tau sqrt(2 (2W + 1) / n) (Madras & Sokal, J. Stat. Phys. 50 (1988)
109; Sokal, "Monte Carlo methods in statistical mechanics", Cargese lectures 1996).

For R independent replicas of the same chain the autocovariance is averaged over replicas
before normalising, which is what a batched GPU run provides.
"""
import numpy as np


def autocorrelation(series):
    """Normalised autocorrelation rho(t), t = 0..n-1, of series (R, n) or (n,), averaged over
    replicas (FFT-based, each replica's own mean removed)."""
    x = np.atleast_2d(np.asarray(series, dtype=np.float64))
    x = x - x.mean(axis=1, keepdims=True)
    n = x.shape[1]
    nfft = 1 << (2 * n - 1).bit_length()
    f = np.fft.rfft(x, nfft, axis=1)
    acov = np.fft.irfft(f * np.conj(f), nfft, axis=1)[:, :n].mean(axis=0)
    acov /= np.arange(n, 0, -1)
    if acov[0] <= 0:
        return np.zeros(n)
    return acov / acov[0]


def tau_int(series, c=6.0):
    """(tau_int, error, window) of series (R, n) or (n,)."""
    x = np.atleast_2d(np.asarray(series, dtype=np.float64))
    n = x.shape[1]
    rho = autocorrelation(x)
    tau = 0.5
    W = 0
    for W in range(1, n):
        tau += rho[W]
        if W >= c * tau:
            break
    err = tau * np.sqrt(2.0 * (2 * W + 1) / (n * x.shape[0]))
    return float(tau), float(err), int(W)


def independent_samples_per_second(n_replicas, sweeps_per_second, tau, stride=1):
    """Independent samples per second of the whole batch: every replica yields one
    independent sample per 2 tau_int sweeps (tau measured in units of `stride` sweeps)."""
    return n_replicas * sweeps_per_second / (2.0 * tau * stride)
