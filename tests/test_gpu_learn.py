"""Learned patch proposal on the GPU (ether_learn_*), against the oracle.

* training kernels: loss and gradient equal the oracle's FP64 forward/backward (same BF16
  rounding points);
* inference network on the tensor cores: logits equal the oracle's forward;
* Metropolis-Hastings step: given the logits the GPU used, the oracle replays every learned
  sweep bit for bit (spins and accepted patches);
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
KTC = 4.511


def ising(L, R, kT, seed=1992, spins_seed=3):
    lat = eg.simple_cubic(L)
    j = eg.couplings(1, FM, [1.0])
    sw = eg.Sweep.from_lattice(lat, j, np.array([1.0]), eg.MODEL_ISING, replicas=R, seed=seed)
    kT = np.broadcast_to(np.asarray(kT, float), (R,))
    sw.set_beta([beta_of(k) for k in kT])
    rng = np.random.default_rng(spins_seed)
    for r in range(R):
        ion = lat.ion.copy()
        ion[:, 3] = rng.choice([-1.0, 1.0], size=lat.N)
        sw.set_spins(ion, r)
    return lat, sw, kT


def storage_spins(lat, sw, r):
    """Replica r as the oracle's colour-split uint8 array."""
    col, rank = sw.colouring()
    g = sw.get_spins(lat.ion, r)
    sp = np.zeros(lat.N, np.uint8)
    sp[col * (lat.N // 2) + rank] = (g[:, 3] > 0).astype(np.uint8)
    return sp


def random_params(seed, scale=1.0):
    rng = np.random.default_rng(seed)
    n = eg.model.N_LEARN_PARAMS
    p = np.zeros(n, np.float32)
    p[:16384] = rng.normal(size=16384) * np.sqrt(2 / 128)
    p[16384:16512] = rng.normal(size=128) * 0.1
    p[16512:32896] = rng.normal(size=16384) * np.sqrt(2 / 128)
    p[32896:33024] = rng.normal(size=128) * 0.1
    p[33024:37120] = rng.normal(size=4096) * 0.1 * scale
    p[37120:] = rng.normal(size=32) * 0.1 * scale
    return p


def random_inputs(rng, B):
    x = np.where(rng.random((B, 128)) < 0.5, -1.0, 1.0).astype(np.float32)
    x[:, 96] = [po.lib().orc_bf16_round(float(v)) for v in rng.uniform(-1.0, 1.0, size=B)]
    x[:, 97:] = 0.0
    return x


def test_training_gradient_matches_oracle():
    lat, sw, _ = ising(8, 1, KTC)
    lr = eg.Learned(sw, seed=1, capacity=4096)
    p = random_params(2)
    lr.set_params(p)
    rng = np.random.default_rng(3)
    x = random_inputs(rng, 96)
    y = rng.integers(0, 2 ** 32, size=96, dtype=np.uint64).astype(np.uint32)
    loss_g, g = lr.loss_grad(x, y)
    loss_o, go = po.mlp_loss_grad(p, x, y, quant=True)
    assert loss_g == pytest.approx(loss_o, rel=1e-5)
    rel = np.linalg.norm(g - go) / np.linalg.norm(go)
    assert rel < 1e-4, rel
    # every block of the gradient, not just the norm
    for a, b in [(0, 16384), (16384, 16512), (16512, 32896), (32896, 33024), (33024, 37120), (37120, 37152)]:
        assert np.linalg.norm(g[a:b] - go[a:b]) <= 1e-3 * np.linalg.norm(go[a:b]) + 1e-9
    lr.close()


@pytest.mark.parametrize("B", [1, 128, 1000])
def test_tensor_core_forward_matches_oracle(B):
    lat, sw, _ = ising(8, 1, KTC)
    lr = eg.Learned(sw, seed=1, capacity=4096)
    p = random_params(4, scale=10.0)
    lr.set_params(p)
    x = random_inputs(np.random.default_rng(B), B)
    z = lr.forward(x)
    zo = po.mlp_forward(p, x, quant=True)
    err = np.abs(z - zo)
    # FP32 tensor-core accumulation vs FP64: equal unless a BF16 rounding of a hidden unit flips
    assert np.mean(err) < 1e-3 * max(1.0, np.abs(zo).mean())
    assert np.max(err) < 0.05 * max(1.0, np.abs(zo).max())
    lr.close()


@pytest.mark.parametrize("L", [8, 16, (8, 16, 24)])
def test_learned_sweep_replays_bit_exact(L):
    kT = [50.0, 2.0 * KTC, KTC, 0.8 * KTC]
    lat, sw, kT = ising(L, 4, kT)
    sw.set_streams(stream=[11, 12, 13, 14], step=[0, 0, 0, 0])
    lr = eg.Learned(sw, seed=9, capacity=4096)
    lr.set_params(random_params(5, scale=1.0))
    lr.set_dump(True)
    Ls = [L] * 3 if np.isscalar(L) else list(L)
    tot_acc = 0
    for t in range(3):
        before = [storage_spins(lat, sw, r) for r in range(4)]
        acc0 = lr.accepts().copy()
        lr.sweep_(1)
        dump = lr.dump()
        acc1 = lr.accepts()
        for r in range(4):
            sp = before[r].copy()
            bj = -1.0 / kT[r]
            a = po.patch_sweep(sp, Ls, bj, np.ascontiguousarray(dump[:, r]), 1992, 11 + r, t)
            np.testing.assert_array_equal(sp, storage_spins(lat, sw, r))
            assert a == int(acc1[r] - acc0[r])
            tot_acc += a
    assert tot_acc > 0  # the replay exercised accepted moves
    lr.close()


def _chain(L, R, kT, steps, equil, learned, seed):
    lat, sw, _ = ising(L, R, kT, seed=seed, spins_seed=seed)
    lr = eg.Learned(sw, seed=seed, capacity=4096) if learned else None
    if lr is not None:
        lr.set_params(random_params(seed, scale=1.0))
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
    a = _chain(8, 64, 1.5 * KTC, 1500, 300, False, 21)
    b = _chain(8, 64, 1.5 * KTC, 1500, 300, True, 22)
    assert b[4] > 0.005, b
    assert abs(a[0] - b[0]) < 4 * np.hypot(a[1], b[1]) + 1e-12
    assert abs(a[2] - b[2]) < 4 * np.hypot(a[3], b[3]) + 1e-12


def test_training_raises_acceptance():
    """Train on plain-sweep configurations at 8 temperatures around T_c; the trained network
    is accepted far more often than the untrained one on the same configurations."""
    R = 64
    kT = np.repeat(KTC * np.linspace(0.9, 1.1, 8), R // 8)
    lat, sw, _ = ising(16, R, kT, seed=31)
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
    assert rates[1] > 3.0 * rates[0] and rates[1] > 0.02, rates
    trained.close()
    untrained.close()


def test_learned_series_recorder():
    """The device-side series ends at the configuration the context holds afterwards."""
    lat, sw, _ = ising(16, 8, KTC, seed=41)
    lr = eg.Learned(sw, seed=3, capacity=4096)
    m = lr.record_series(25, 1, 1)
    assert m.shape == (8, 25)
    np.testing.assert_allclose(m[:, -1], np.linalg.norm(sw.tot_magnetisation(), axis=1), rtol=1e-12)
    assert lr.info().proposed == 25 * 2 * 8 * lr.info().patches_per_class
    m2 = lr.record_series(5, 0, 2)
    assert m2.shape == (8, 5)
    m3 = lr.record_series(12, 1, 1, stride=4)  # |M| after steps 4, 8, 12
    assert m3.shape == (8, 3)
    np.testing.assert_allclose(m3[:, -1], np.linalg.norm(sw.tot_magnetisation(), axis=1), rtol=1e-12)
    lr.close()
