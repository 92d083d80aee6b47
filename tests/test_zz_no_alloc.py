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


def _numpy_energy(spins, L, J, zee, model):
    """get_tot_energy / get_tot_magnetisation of periodic simple-cubic configurations in the
    reference's site order (x fastest), computed by array rolls: E = sum_i S_i . (J o h_i + z)
    with h_i the sum of the six neighbours."""
    R = spins.shape[0]
    L1, L2, L3 = L
    if model == eg.MODEL_ISING:
        s = spins.reshape(R, L3, L2, L1)
        nb = np.zeros_like(s)
        for ax in (1, 2, 3):
            nb += np.roll(s, 1, axis=ax)
            nb += np.roll(s, -1, axis=ax)
        bonds = (s.astype(np.int32) * nb).reshape(R, -1).sum(axis=1, dtype=np.int64)
        tot = s.reshape(R, -1).sum(axis=1, dtype=np.int64)
        E = J[2] * bonds.astype(np.float64) + zee[2] * tot.astype(np.float64)
        M = np.zeros((R, 3))
        M[:, 2] = tot
        return E, M
    s = spins[..., :3].astype(np.float64).reshape(R, L3, L2, L1, 3)
    h = np.zeros_like(s)
    for ax in (1, 2, 3):
        h += np.roll(s, 1, axis=ax) + np.roll(s, -1, axis=ax)
    E = (s * (h * np.asarray(J) + np.asarray(zee))).reshape(R, -1).sum(axis=1)
    return E, s.reshape(R, -1, 3).sum(axis=1)


@pytest.mark.parametrize("model,R", [(eg.MODEL_ISING, 992), (eg.MODEL_XYZ, 5)])
def test_noalloc_unequal_sides_at_the_block_clamp(model, R):
    """(40, 36, 50) = 72000 sites: more than 32 blocks of 2048 sites, so the partials use the
    32-block clamp; for Ising the 992 replicas fill the scratch array to its limit."""
    lib = abi.load()
    L = (40, 36, 50)
    N = int(np.prod(L))
    rng = np.random.default_rng(5)
    if model == eg.MODEL_ISING:
        # biased towards +1 so that E and M are far from zero
        host = np.where(rng.random((R, N)) < 0.7, 1, -1).astype(np.int8)
    else:
        v = rng.normal(size=(R, N, 3)) + np.array([0.0, 0.0, 1.5])
        v /= np.linalg.norm(v, axis=2, keepdims=True)
        host = np.concatenate([v, np.zeros((R, N, 1))], axis=2).astype(np.float32)
    J = np.array([-1e-3, -0.8e-3, -1.2e-3])
    zee = np.array([0.1e-3, -0.2e-3, 0.3e-3])
    E_ref, M_ref = _numpy_energy(host, L, J, zee, model)
    dev = _device_copy(host)
    Lv = np.array(L, dtype=np.int32)
    for call in range(2):
        E = np.full(R, np.nan)
        M = np.full((R, 3), np.nan)
        rc = lib.ether_sc_energy_noalloc(model, C.c_void_p(dev.data_ptr()), abi.iptr(Lv), R,
                                         abi.dptr(J), abi.dptr(zee), abi.dptr(E), abi.dptr(M), None)
        assert rc == 0, lib.ether_last_error()
        np.testing.assert_allclose(E, E_ref, rtol=1e-9, atol=1e-8)
        np.testing.assert_allclose(M, M_ref, rtol=1e-9, atol=1e-6)


def test_noalloc_rejects_pageable_host_memory_without_launching():
    """A host array that was never registered with CUDA is refused by the pointer check that
    runs before any launch; the call returns ETHER_ERR_ARG and the device stays usable."""
    lib = abi.load()
    host = np.ones(4 * 4 * 4, dtype=np.int8)
    Lv = np.array([4, 4, 4], dtype=np.int32)
    J = np.zeros(3)
    E = np.zeros(1)
    M = np.zeros(3)
    rc = lib.ether_sc_energy_noalloc(eg.MODEL_ISING, C.c_void_p(host.ctypes.data), abi.iptr(Lv),
                                     1, abi.dptr(J), abi.dptr(J), abi.dptr(E), abi.dptr(M), None)
    assert rc == -1
    assert b"pageable host memory" in lib.ether_last_error()
    # the library keeps working after the refusal
    dev = _device_copy(host)
    rc = lib.ether_sc_energy_noalloc(eg.MODEL_ISING, C.c_void_p(dev.data_ptr()), abi.iptr(Lv),
                                     1, abi.dptr(J), abi.dptr(J), abi.dptr(E), abi.dptr(M), None)
    assert rc == 0, lib.ether_last_error()
    assert M[2] == 64.0
