"""Sokal automatic-windowing tau_int on processes with a known answer."""
import numpy as np
import pytest

from ether_gb300.analysis import autocorrelation, independent_samples_per_second, tau_int


@pytest.mark.parametrize("phi", [0.0, 0.5, 0.9, 0.97])
def test_tau_int_of_ar1(phi):
    """AR(1) x_t = phi x_{t-1} + e_t: rho(t) = phi^t, tau_int = (1 + phi) / (2 (1 - phi))."""
    rng = np.random.default_rng(1)
    R, n = 32, 20000
    x = np.zeros((R, n))
    e = rng.normal(size=(R, n))
    x[:, 0] = e[:, 0] / np.sqrt(1 - phi ** 2)
    for t in range(1, n):
        x[:, t] = phi * x[:, t - 1] + e[:, t]
    tau, err, W = tau_int(x)
    want = (1 + phi) / (2 * (1 - phi))
    assert abs(tau - want) < max(4 * err, 0.02 * want)
    rho = autocorrelation(x)
    assert abs(rho[1] - phi) < 0.02


def test_independent_samples_per_second():
    assert independent_samples_per_second(10, 100.0, 5.0) == pytest.approx(100.0)
    assert independent_samples_per_second(10, 100.0, 5.0, stride=2) == pytest.approx(50.0)
