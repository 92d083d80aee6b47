"""ether_sc_energy_noalloc: the energy / magnetisation entry point that allocates nothing,
for callers that cannot allocate device memory where they need an energy (their memory is
owned by a host framework's pool or an OpenACC/OpenMP-target runtime, or a fixed budget is
spent).  Checked through the C-ABI against the context-based ether_tot_energy /
ether_tot_magnetisation on the same configurations, on two calls in a row.  This file is
collected last so that a stop-at-first-failure run has run every other test before it."""
import ctypes as C

import numpy as np
import pytest

import ether_gb300 as eg
from ether_gb300 import abi
from tests.helpers import make_pair, random_ising, random_xyz

pytestmark = pytest.mark.gpu

FM = [[(1, 1, (-1.0, -1.0, -1.0))]]


def _device_copy(host):
    """Caller-owned device buffer (the test is the caller and may allocate)."""
    torch = pytest.importorskip("torch")
    t = torch.from_numpy(np.ascontiguousarray(host)).to("cuda")
    torch.cuda.synchronize()
    return t


def _natural_order_spins(ions, model):
    if model == eg.MODEL_ISING:
        return np.stack([ion[:, 3] for ion in ions]).astype(np.int8)
    return np.stack([np.concatenate([ion[:, 1:4], ion[:, 5:6]], axis=1) for ion in ions]).astype(np.float32)


@pytest.mark.parametrize("model", [eg.MODEL_ISING, eg.MODEL_XYZ])
def test_noalloc_matches_context_energy_two_calls(model):
    lib = abi.load()
    L = 12
    R = 3
    lat = eg.simple_cubic(L)
    h = (0.3, -0.2, 1.0)
    sw, _ = make_pair(lat, model, FM, replicas=R, zeeman=True, h=h, g_factor=2.0)
    ions = [random_ising(lat, 20 + r) if model == eg.MODEL_ISING else random_xyz(lat, 20 + r)
            for r in range(R)]
    for r in range(R):
        sw.set_spins(ions[r], replica=r)
    E_ref = sw.tot_energy()
    M_ref = sw.tot_magnetisation()
    dev = _device_copy(_natural_order_spins(ions, model))
    Lv = np.array([L, L, L], dtype=np.int32)
    J = np.array([-1e-3, -1e-3, -1e-3])
    zee = -(2.0 * eg.MB_EV * 1.0) * np.array(h)
    rtol = 1e-12 if model == eg.MODEL_ISING else 1e-6
    for call in range(2):
        E = np.full(R, np.nan)
        M = np.full((R, 3), np.nan)
        rc = lib.ether_sc_energy_noalloc(model, C.c_void_p(dev.data_ptr()), abi.iptr(Lv), R,
                                         abi.dptr(J), abi.dptr(zee), abi.dptr(E), abi.dptr(M), None)
        assert rc == 0, lib.ether_last_error()
        np.testing.assert_allclose(E, E_ref, rtol=rtol, atol=1e-12)
        np.testing.assert_allclose(M, M_ref, rtol=rtol, atol=1e-9)


def test_noalloc_rejects_more_replicas_than_its_scratch():
    lib = abi.load()
    R = 993  # one more than the 992 the static scratch takes
    dev = _device_copy(np.ones(64 * R, dtype=np.int8))  # sized for the request all the same
    Lv = np.array([4, 4, 4], dtype=np.int32)
    J = np.zeros(3)
    E = np.zeros(R)
    M = np.zeros(3 * R)
    rc = lib.ether_sc_energy_noalloc(eg.MODEL_ISING, C.c_void_p(dev.data_ptr()), abi.iptr(Lv),
                                     R, abi.dptr(J), abi.dptr(J), abi.dptr(E), abi.dptr(M), None)
    assert rc == -5
    assert b"at most 992" in lib.ether_last_error()
