"""Learned patch proposal for the Heisenberg (XYZ) model on the GPU (ether_learn_* of an XYZ
context), against the oracle.

* training kernels: the von Mises-Fisher loss and its gradient equal the oracle's FP64
  forward/backward (same BF16 rounding points);
* inference network (FP32 GEMM): its outputs equal the oracle's forward;
* Metropolis-Hastings step: given the vMF parameters the GPU used, the oracle replays every
  learned sweep bit for bit (spins and accepted patches);
* exactness: interleaving learned sweeps leaves <e> and <|m|> unchanged;
* the gain: after training on configurations of the plain sweep, the network's proposals are
  accepted far more often than the untrained network's.
"""
import numpy as np
import pytest

import ether_gb300 as eg
from oracle import pyoracle as po
from tests.helpers import beta_of

pytestmark = pytest.mark.gpu

FM = [[(1, 1, (-1.0, -1.0, -1.0))]]
KTC = 1.443
J_EV = np.float32(-1.0 / 1000.0)  # the context's FP32 coupling (FM, 1 meV)


def heis(L, R, kT, seed=1992, spins_seed=3):
    lat = eg.simple_cubic(L)
    j = eg.couplings(1, FM, [1.0])
    sw = eg.Sweep.from_lattice(lat, j, np.array([1.0]), eg.MODEL_XYZ, replicas=R, seed=seed)
    kT = np.broadcast_to(np.asarray(kT, float), (R,))
    sw.set_beta([beta_of(k) for k in kT])
    rng = np.random.default_rng(spins_seed)
    for r in range(R):
        ion = lat.ion.copy()
        v = rng.normal(size=(lat.N, 3))
        ion[:, 1:4] = v / np.linalg.norm(v, axis=1, keepdims=True)
        sw.set_spins(ion, r)
    return lat, sw, kT


def storage_spins(lat, sw, r):
    """Replica r as the oracle's colour-split (N, 4) float32 array (x, y, z, phi)."""
    col, rank = sw.colouring()
    g = sw.get_spins(lat.ion, r)
    sp = np.zeros((lat.N, 4), np.float32)
    sp[col * (lat.N // 2) + rank] = g[:, [1, 2, 3, 5]].astype(np.float32)
    return sp


def random_params(seed, scale=1.0):
    rng = np.random.default_rng(seed)
    n = po.xmlp_n_params()
    o = [0, 38912, 39040, 55424, 55552, 67840, 67936]
    p = np.zeros(n, np.float32)
    p[o[0]:o[1]] = rng.normal(size=o[1] - o[0]) * np.sqrt(2 / 304)
    p[o[1]:o[2]] = rng.normal(size=o[2] - o[1]) * 0.1
    p[o[2]:o[3]] = rng.normal(size=o[3] - o[2]) * np.sqrt(2 / 128)
    p[o[3]:o[4]] = rng.normal(size=o[4] - o[3]) * 0.1
    p[o[4]:o[5]] = rng.normal(size=o[5] - o[4]) * 0.3 * scale
    p[o[5]:] = rng.normal(size=o[6] - o[5]) * 0.3 * scale
    return p


def random_inputs(rng, B):
    v = rng.normal(size=(B, 96, 3))
    v /= np.linalg.norm(v, axis=2, keepdims=True)
    x = np.zeros((B, 304), np.float32)
    bf = np.vectorize(lambda c: po.lib().orc_bf16_round(float(c)))
    x[:, :288] = bf(v.reshape(B, 288))
    x[:, 288:291] = bf(rng.uniform(-1.0, 1.0, size=(B, 1)) * np.ones((1, 3)))
    return x


def test_shape_and_unsupported_contexts():
    lat, sw, _ = heis(8, 1, KTC)
    lr = eg.Learned(sw, seed=1, capacity=4096)
    assert (lr.n_in, lr.n_out, lr.n_params) == (304, 96, po.xmlp_n_params())
    assert lr.params().size == lr.n_params
    lr.close()
    j = eg.couplings(1, FM, [1.0])
    ang = eg.Sweep.from_lattice(lat, j, np.array([1.0]), eg.MODEL_XYZ, replicas=1, seed=1, angle=True,
                                dphi=0.5)
    with pytest.raises(eg.EtherError):
        eg.Learned(ang, seed=1, capacity=4096)


def test_training_gradient_matches_oracle():
    lat, sw, _ = heis(8, 1, KTC)
    lr = eg.Learned(sw, seed=1, capacity=4096)
    p = random_params(2)
    lr.set_params(p)
    rng = np.random.default_rng(3)
    x = random_inputs(rng, 64)
    y = rng.normal(size=(64, 32, 3))
    y = (y / np.linalg.norm(y, axis=2, keepdims=True)).reshape(64, 96).astype(np.float32)
    loss_g, g = lr.loss_grad(x, y)
    loss_o, go = po.xmlp_loss_grad(p, x, y, quant=True)
    assert loss_g == pytest.approx(loss_o, rel=1e-5)
    o = [0, 38912, 39040, 55424, 55552, 67840, 67936]
    for a, b in zip(o[:-1], o[1:]):
        assert np.linalg.norm(g[a:b] - go[a:b]) <= 1e-3 * np.linalg.norm(go[a:b]) + 1e-9, (a, b)
    lr.close()


@pytest.mark.parametrize("B", [1, 200])
def test_forward_matches_oracle(B):
    lat, sw, _ = heis(8, 1, KTC)
    lr = eg.Learned(sw, seed=1, capacity=4096)
    p = random_params(4, scale=3.0)
    lr.set_params(p)
    x = random_inputs(np.random.default_rng(B), B)
    z = lr.forward(x)
    zo = po.xmlp_forward(p, x, quant=2)  # inference: hidden biases in BF16 as well
    err = np.abs(z - zo)
    # FP32 accumulation vs FP64: equal unless a BF16 rounding of a hidden unit flips
    assert np.mean(err) < 1e-3 * max(1.0, np.abs(zo).mean())
    assert np.max(err) < 0.05 * max(1.0, np.abs(zo).max())
    lr.close()


@pytest.mark.parametrize("L", [8, (8, 16, 8)])
def test_learned_sweep_replays_bit_exact(L):
    kT = [20.0, 2.0 * KTC, KTC, 0.7 * KTC]
    lat, sw, kT = heis(L, 4, kT)
    sw.set_streams(stream=[11, 12, 13, 14], step=[0, 0, 0, 0])
    lr = eg.Learned(sw, seed=9, capacity=4096)
    # a weak network: concentrations from below 1e-3 (uniform) to O(1), so that moves are
    # accepted and both forms of the vMF sampler and density run
    lr.set_params(random_params(5, scale=0.1))
    lr.set_dump(True)
    Ls = [L] * 3 if np.isscalar(L) else list(L)
    tot_acc = 0
    for t in range(5):
        before = [storage_spins(lat, sw, r) for r in range(4)]
        acc0 = lr.accepts().copy()
        lr.sweep_(1)
        dump = lr.dump()
        acc1 = lr.accepts()
        for r in range(4):
            sp = before[r].copy()
            beta = np.float32(beta_of(kT[r]))
            a = po.xpatch_sweep(sp, Ls, beta, [J_EV] * 3, np.ascontiguousarray(dump[:, r]), 1992, 11 + r, t)
            np.testing.assert_array_equal(sp, storage_spins(lat, sw, r))
            assert a == int(acc1[r] - acc0[r])
            tot_acc += a
    assert tot_acc > 0  # the replay exercised accepted moves
    lr.close()


def _chain(L, R, kT, steps, equil, learned, seed):
    lat, sw, _ = heis(L, R, kT, seed=seed, spins_seed=seed)
    lr = eg.Learned(sw, seed=seed, capacity=4096) if learned else None
    if lr is not None:
        lr.set_params(random_params(seed, scale=0.1))
    es, ms = [], []
    for s in range(equil + steps):
        sw.metropolis(1, accept=False)
        if lr is not None:
            lr.sweep_(1)
        if s >= equil and (s - equil) % 10 == 0:
            E = sw.tot_energy()
            M = sw.tot_magnetisation()
            es.append(np.asarray(E[:, 0] if np.ndim(E) == 2 else E) / lat.N)
            ms.append(np.linalg.norm(np.asarray(M).reshape(R, 3), axis=1) / lat.N)
    es = np.mean(es, axis=0)
    ms = np.mean(ms, axis=0)
    acc = lr.accepts().sum() / max(1, lr.info().proposed) if lr is not None else 0.0
    return es.mean(), es.std(ddof=1) / np.sqrt(R), ms.mean(), ms.std(ddof=1) / np.sqrt(R), acc


def test_learned_sweeps_leave_the_distribution_unchanged():
    """An untrained network is a poor proposal, but any proposal keeps the distribution."""
    a = _chain(8, 64, 1.5 * KTC, 1200, 300, False, 21)
    b = _chain(8, 64, 1.5 * KTC, 1200, 300, True, 22)
    assert b[4] > 0.002, b
    assert abs(a[0] - b[0]) < 4 * np.hypot(a[1], b[1]) + 1e-12
    assert abs(a[2] - b[2]) < 4 * np.hypot(a[3], b[3]) + 1e-12


def test_training_raises_acceptance():
    """Train on plain-sweep configurations at 8 temperatures around T_c; the trained network
    is accepted far more often than the untrained one on the same configurations."""
    R = 64
    kT = np.repeat(KTC * np.linspace(0.9, 1.1, 8), R // 8)
    lat, sw, _ = heis(16, R, kT, seed=31)
    sw.metropolis(500, accept=False)
    trained = eg.Learned(sw, seed=5, capacity=1 << 18)
    for _ in range(40):
        sw.metropolis(10, accept=False)
        trained.collect(64)
    loss0 = trained.train(1, batch=1024, lr=1e-3)
    loss1 = trained.train(1500, batch=1024, lr=1e-3)
    assert loss1 < loss0
    untrained = eg.Learned(sw, seed=5, capacity=4096)
    rates = []
    for lr in (untrained, trained):
        a0 = lr.accepts().sum()
        p0 = lr.info().proposed
        for _ in range(20):
            sw.metropolis(1, accept=False)
            lr.sweep_(1)
        rates.append((lr.accepts().sum() - a0) / (lr.info().proposed - p0))
    assert rates[1] > 3.0 * rates[0] and rates[1] > 0.01, rates
    trained.close()
    untrained.close()


def test_learned_series_recorder():
    lat, sw, _ = heis(16, 8, KTC, seed=41)
    lr = eg.Learned(sw, seed=3, capacity=4096)
    m = lr.record_series(10, 1, 1)
    assert m.shape == (8, 10)
    np.testing.assert_allclose(m[:, -1], np.linalg.norm(sw.tot_magnetisation(), axis=1), rtol=1e-12)
    assert lr.info().proposed == 10 * 2 * 8 * lr.info().patches_per_class
    m3 = lr.record_series(9, 0, 1, stride=3)
    assert m3.shape == (8, 3)
    np.testing.assert_allclose(m3[:, -1], np.linalg.norm(sw.tot_magnetisation(), axis=1), rtol=1e-12)
    lr.close()


def test_learn_batch_sweep_equals_each_contexts_own_calls():
    """ether_learn_batch_sweep over an Ising and a Heisenberg context (different sizes):
    spins and accepted patches as each context's own ether_metropolis + ether_learn_sweep."""
    def pair():
        out = []
        for model, L, kT, seed in ((eg.MODEL_ISING, 16, 4.511, 3), (eg.MODEL_XYZ, 8, KTC, 4)):
            lat = eg.simple_cubic(L)
            sw = eg.Sweep.from_lattice(lat, eg.couplings(1, FM, [1.0]), np.array([1.0]), model, replicas=3,
                                       seed=seed)
            sw.set_beta([beta_of(kT)] * 3)
            ion = lat.ion.copy()
            rng = np.random.default_rng(seed)
            if model == eg.MODEL_ISING:
                ion[:, 3] = rng.choice([-1.0, 1.0], size=lat.N)
            else:
                v = rng.normal(size=(lat.N, 3))
                ion[:, 1:4] = v / np.linalg.norm(v, axis=1, keepdims=True)
            sw.set_spins(ion)
            lr = eg.Learned(sw, seed=seed, capacity=4096)
            if model == eg.MODEL_XYZ:
                lr.set_params(random_params(6, scale=0.1))
            out.append((lat, sw, lr))
        return out
    A, B = pair(), pair()
    eg.learn_batch_sweep([lr for _, _, lr in A], nsweeps=4, plain_per_sweep=1)
    for _ in range(4):
        for _, sw, lr in B:
            sw.metropolis(1, accept=False)
            lr.sweep_(1)
    for (lat, sa, la), (_, sb, lb) in zip(A, B):
        for r in range(3):
            np.testing.assert_array_equal(sa.get_spins(lat.ion, r), sb.get_spins(lat.ion, r))
        np.testing.assert_array_equal(la.accepts(), lb.accepts())
    for (_, sa, la), (_, sb, lb) in zip(A, B):
        la.close(); lb.close(); sa.close(); sb.close()
