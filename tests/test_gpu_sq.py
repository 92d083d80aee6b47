"""Structure factor on the tensor cores (BF16 high/low split, FP32 accumulation) against the
oracle's FP64 restatement of utility/Structure_Factor/structure_factor.f90:131-183.

Tolerance: |S_a(q)|/N within 3e-4 absolute and |S(q)|^2/N^2 within 1e-3 of the largest value
(the split keeps about 16 significant bits per product; sums run over N sites)."""
import ctypes as C

import numpy as np
import pytest

import ether_gb300 as eg
from ether_gb300 import abi
from oracle import pyoracle as po
from tests.helpers import make_pair, random_ising, random_xyz

pytestmark = pytest.mark.gpu

FM = [[(1, 1, (-1.0, -1.0, -1.0))]]


def _gpu_sq(sw, abc, nq, q0, dq):
    Q = int(np.prod(nq))
    sq = np.zeros(sw.R * Q, dtype=np.float32)
    comp = np.zeros(sw.R * Q * 3, dtype=np.float32)
    a = np.ascontiguousarray(abc, dtype=np.float64).ravel()
    n = np.ascontiguousarray(nq, dtype=np.int32)
    abi.check(sw.lib.ether_structure_factor(
        sw.h, abi.dptr(a), abi.iptr(n), abi.dptr(np.asarray(q0, float)), abi.dptr(np.asarray(dq, float)),
        sq.ctypes.data_as(C.POINTER(C.c_float)), comp.ctypes.data_as(C.POINTER(C.c_float))))
    return sq.reshape(sw.R, Q), comp.reshape(sw.R, Q, 3)


def _oracle_sq(lat, spins, abc, nq, q0, dq, qidx):
    """FP64 direct sums for the q-points qidx (flat index h1 + n0 (h2 + n1 h3))."""
    abc = np.asarray(abc, float)
    vol = np.dot(abc[0], np.cross(abc[1], abc[2]))
    b = 2 * np.pi * np.array([np.cross(abc[1], abc[2]), np.cross(abc[2], abc[0]),
                              np.cross(abc[0], abc[1])]) / vol
    h1 = qidx % nq[0]
    h2 = (qidx // nq[0]) % nq[1]
    h3 = qidx // (nq[0] * nq[1])
    coef = np.stack([q0[0] + h1 * dq[0], q0[1] + h2 * dq[1], q0[2] + h3 * dq[2]], axis=1)
    qv = np.ascontiguousarray(coef @ b)
    pos = np.ascontiguousarray(lat.ion[:, 6:9])
    N = lat.N
    sq, comp = [], []
    for S in spins:
        out = np.zeros(6 * len(qidx))
        po.lib().orc_structure_factor(N, pos.ctypes.data_as(po.PD),
                                      np.ascontiguousarray(S).ctypes.data_as(po.PD), len(qidx),
                                      qv.ctypes.data_as(po.PD), out.ctypes.data_as(po.PD))
        out = out.reshape(-1, 3, 2)
        m2 = (out ** 2).sum(axis=2)
        sq.append(m2.sum(axis=1) / N ** 2)
        comp.append(np.sqrt(m2) / N)
    return np.array(sq), np.array(comp)


def _check(lat, model, R, nq, q0, dq, abc, seed=1):
    sw, _ = make_pair(lat, model, FM, replicas=R)
    spins = []
    for r in range(R):
        ion = random_ising(lat, seed + r) if model == eg.MODEL_ISING else random_xyz(lat, seed + r)
        sw.set_spins(ion, replica=r)
        g = sw.get_spins(lat.ion, r)
        spins.append(g[:, 1:4] if model == eg.MODEL_XYZ else np.stack([0 * g[:, 3], 0 * g[:, 3], g[:, 3]], 1))
    sq, comp = _gpu_sq(sw, abc, nq, q0, dq)
    Q = int(np.prod(nq))
    qidx = np.arange(Q) if Q <= 512 else np.random.default_rng(0).choice(Q, 512, replace=False)
    ref_sq, ref_comp = _oracle_sq(lat, spins, abc, nq, q0, dq, qidx)
    assert np.all(np.isfinite(sq))
    np.testing.assert_allclose(comp[:, qidx, :], ref_comp, atol=3e-4, rtol=0)
    np.testing.assert_allclose(sq[:, qidx], ref_sq, atol=1e-3 * max(ref_sq.max(), 1e-6), rtol=0)
    return sq, ref_sq


def test_sq_tiny_single_block():
    lat = eg.simple_cubic(4)
    _check(lat, eg.MODEL_XYZ, 1, (64, 1, 1), (0.0, 0.0, 0.0), (1.0 / 16, 0.0, 0.0), np.eye(3))


def test_sq_ising_many_blocks_and_replicas():
    lat = eg.simple_cubic(8)
    _check(lat, eg.MODEL_ISING, 3, (64, 2, 3), (-1.0, 0.0, 0.25), (1.0 / 32, 0.5, 0.125), np.eye(3))


def test_sq_pyrochlore_offset_grid():
    lat = eg.pyrochlore(2)
    abc = np.eye(3) * eg.model.PYROCHLORE_A
    _check(lat, eg.MODEL_XYZ, 2, (64, 3, 2), (-0.5, -0.25, 0.1), (1.0 / 64, 0.3, 0.7), abc)


def test_sq_ordered_state_bragg_peak():
    """All spins up on 8^3: along q = (h/64) b1, |S|/N is the Dirichlet kernel
    |sin(8 pi q) / (8 sin(pi q))|: 1 at q = 0, 0 at q = k/8."""
    lat = eg.simple_cubic(8)
    sw, _ = make_pair(lat, eg.MODEL_ISING, FM, replicas=1)
    ion = lat.ion.copy()
    ion[:, 3] = 1.0
    sw.set_spins(ion)
    sq, comp = _gpu_sq(sw, np.eye(3), (64, 1, 1), (0.0, 0.0, 0.0), (1.0 / 64, 0.0, 0.0))
    q = np.arange(1, 64) / 64.0
    want = (np.sin(8 * np.pi * q) / (8 * np.sin(np.pi * q))) ** 2
    assert abs(sq[0, 0] - 1.0) < 1e-3
    np.testing.assert_allclose(sq[0, 1:], want, atol=1e-3)
    assert np.all(sq[0, 8::8] < 1e-5)
    assert abs(comp[0, 0, 2] - 1.0) < 1e-3
