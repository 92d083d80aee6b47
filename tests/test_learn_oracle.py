"""The learned patch proposal's oracle (oracle/learn_oracle.c), on the CPU.

* the MLP gradient equals central finite differences (FP64, no BF16 rounding);
* the BF16 rounding and the FP32 log used in the acceptance behave as specified;
* the patch geometry covers every boundary site exactly once;
* exact Metropolis-Hastings: a chain that interleaves learned-patch sweeps (driven by
  stand-in proposals, good and bad) with Metropolis sweeps has the same <e> and <|m|> as
  Metropolis alone -- the stationary distribution is unchanged whatever the proposal;
* the XYZ learner: its MLP gradient (von Mises-Fisher loss) equals central finite
  differences, and its vMF sampler and density agree (normalised density, the sampler's
  mean cosine coth(kappa) - 1/kappa, unit vectors).
"""
import numpy as np
import pytest

from oracle import pyoracle as po


def _random_batch(rng, B):
    x = np.where(rng.random((B, 128)) < 0.5, -1.0, 1.0).astype(np.float32)
    x[:, 96] = rng.uniform(-1.2, 1.2, size=B)
    x[:, 97:] = 0.0
    y = rng.integers(0, 2 ** 32, size=B, dtype=np.uint64).astype(np.uint32)
    return x, y


def test_mlp_gradient_matches_finite_differences():
    rng = np.random.default_rng(5)
    n = po.mlp_n_params()
    assert n == 128 * 128 + 128 + 128 * 128 + 128 + 32 * 128 + 32
    p = (rng.normal(size=n) * 0.15).astype(np.float32)
    x, y = _random_batch(rng, 6)
    loss, g = po.mlp_loss_grad(p, x, y, quant=False)
    assert np.isfinite(loss) and loss > 0
    # parameters with non-negligible gradient in every block
    blocks = [(0, 16384), (16384, 16512), (16512, 32896), (32896, 33024), (33024, 37120),
              (37120, 37152)]
    idx = []
    for a, b in blocks:
        seg = np.abs(g[a:b])
        idx += list(a + np.argsort(seg)[-4:])
    h = 1e-3
    for i in idx:
        pp = p.copy()
        pp[i] = p[i] + h
        lp, _ = po.mlp_loss_grad(pp, x, y, quant=False)
        pp[i] = p[i] - h
        lm, _ = po.mlp_loss_grad(pp, x, y, quant=False)
        fd = (lp - lm) / (float(np.float32(p[i] + h)) - float(np.float32(p[i] - h)))
        assert fd == pytest.approx(g[i], rel=2e-3, abs=1e-7), i


def test_bf16_rounding_is_round_to_nearest_even():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(1)
    v = np.concatenate([rng.normal(size=2000).astype(np.float32),
                        np.float32([1.0, -1.0, 0.0, 1.00390625, 1.01171875, 3.3e-30])])
    ours = np.array([po.lib().orc_bf16_round(float(f)) for f in v], dtype=np.float32)
    ref = torch.from_numpy(v).to(torch.bfloat16).to(torch.float32).numpy()
    np.testing.assert_array_equal(ours, ref)


def test_logf_own_accuracy():
    xs = np.concatenate([np.geomspace(2.0 ** -32, 1.0, 3000), [1.0, 0.5, 0.999999]]).astype(np.float32)
    ours = np.array([po.lib().orc_logf_own(float(x)) for x in xs])
    ref = np.log(xs.astype(np.float64))
    err = np.abs(ours - ref) / np.maximum(np.abs(ref), 1e-3)
    assert err.max() < 3e-7


def test_patch_geometry():
    A, B, Bn, Ab = po.patch_tables()
    assert all((a.sum() % 2) == 0 for a in A) and all((b.sum() % 2) == 1 for b in B)
    cover = np.zeros(96, int)
    for m in range(32):
        for c in Bn[m]:
            if c < 0:
                cover[-c - 1] += 1
            else:
                # an A neighbour is one lattice step away
                assert np.abs(A[c] - B[m]).sum() == 1
    for k in range(32):
        for c in Ab[k]:
            if c >= 0:
                cover[c] += 1
    np.testing.assert_array_equal(cover, np.ones(96, int))
    # every internal A-B bond appears once
    assert sum(int((Bn[m] >= 0).sum()) for m in range(32)) == 144


def test_patch_gather_canonical_frame():
    """A-sites are colour 0 whatever the offset parity; gathered bits match the lattice."""
    L = [8, 8, 8]
    rng = np.random.default_rng(2)
    sp = rng.integers(0, 2, size=512).astype(np.uint8)
    A, B, _, _ = po.patch_tables()
    half = 256
    for off in ([0, 0, 0], [1, 0, 0], [1, 2, 3], [3, 3, 3]):
        x, bnd, ab, bb = po.patch_gather(sp, L, off, 1, 0, 1, 0.5)
        par = sum(off) & 1
        for k in range(32):
            a, b, c = A[k]
            X = (4 * 1 + off[0] + (3 - a if par else a)) % 8
            Y = (off[1] + b) % 8
            Z = (4 * 1 + off[2] + c) % 8
            assert (X + Y + Z) % 2 == 0
            s = sp[((X + Y + Z) & 1) * half + (Z * 8 + Y) * 4 + X // 2]
            assert ((ab >> k) & 1) == s
        assert np.all(np.abs(x[:96]) == 1.0) and x[96] == 0.5 and np.all(x[97:] == 0)


@pytest.mark.parametrize("zscale,zbias,kT", [(2.0 / 4.511, 0.0, 4.511), (0.0, 2.5, 4.511),
                                             (2.0 / 3.5, 0.0, 3.5)])
def test_patch_chain_is_unbiased(zscale, zbias, kT):
    bj = -1.0 / kT  # ferromagnet in ETHER's sign
    steps = 12000
    a = po.patch_chain([8, 8, 8], bj, steps, 400, False, seed=11)
    b = po.patch_chain([8, 8, 8], bj, steps, 400, True, zscale=zscale, zbias=zbias, seed=12)
    assert b["accept"] > 0.0
    for key in ("e", "m"):
        err = np.hypot(a[key + "_err"], b[key + "_err"])
        assert abs(a[key] - b[key]) < 4.0 * err + 1e-9, (key, a, b)


def _xyz_batch(rng, B):
    """Boundary spins (unit vectors, BF16-rounded), beta J features, unit-vector targets."""
    v = rng.normal(size=(B, 96, 3))
    v /= np.linalg.norm(v, axis=2, keepdims=True)
    x = np.zeros((B, 304), np.float32)
    x[:, :288] = [[po.lib().orc_bf16_round(float(c)) for c in row] for row in v.reshape(B, 288)]
    x[:, 288:291] = rng.uniform(-2.0, 2.0, size=(B, 1))
    y = rng.normal(size=(B, 32, 3))
    y /= np.linalg.norm(y, axis=2, keepdims=True)
    return x, y.reshape(B, 96).astype(np.float32)


def test_xyz_mlp_gradient_matches_finite_differences():
    rng = np.random.default_rng(8)
    n = po.xmlp_n_params()
    assert n == 128 * 304 + 128 + 128 * 128 + 128 + 96 * 128 + 96
    p = (rng.normal(size=n) * 0.1).astype(np.float32)
    x, y = _xyz_batch(rng, 5)
    loss, g = po.xmlp_loss_grad(p, x, y, quant=False)
    assert np.isfinite(loss)
    o = [0, 38912, 39040, 55424, 55552, 67840, 67936]
    idx = []
    for a, b in zip(o[:-1], o[1:]):
        idx += list(a + np.argsort(np.abs(g[a:b]))[-4:])
    h = 1e-3
    for i in idx:
        pp = p.copy()
        pp[i] = p[i] + h
        lp, _ = po.xmlp_loss_grad(pp, x, y, quant=False)
        pp[i] = p[i] - h
        lm, _ = po.xmlp_loss_grad(pp, x, y, quant=False)
        fd = (lp - lm) / (float(np.float32(p[i] + h)) - float(np.float32(p[i] - h)))
        assert fd == pytest.approx(g[i], rel=2e-3, abs=1e-7), i


@pytest.mark.parametrize("kappa", [5e-4, 0.05, 0.7, 3.0, 40.0])
def test_vmf_sampler_and_density_agree(kappa):
    rng = np.random.default_rng(int(kappa * 1000) + 1)
    mu = np.array([0.2, -0.6, 0.77])
    mu /= np.linalg.norm(mu)
    m = (mu * kappa).astype(np.float32)
    n = 20000
    u = rng.integers(0, 2 ** 24, n) / 2 ** 24
    v = rng.integers(0, 2 ** 24, n) / 2 ** 23 - 1.0
    xs = np.array([po.vmf_sample(m, a, b) for a, b in zip(u, v)], dtype=np.float64)
    assert np.abs(np.linalg.norm(xs, axis=1) - 1.0).max() < 3e-7
    c = xs @ mu
    want = 0.0 if kappa < 1e-3 else 1.0 / np.tanh(kappa) - 1.0 / kappa
    assert abs(c.mean() - want) < 5.0 * c.std() / np.sqrt(n) + 1e-6
    # the FP32 density equals the FP64 formula, and (where uniform points see its mass)
    # integrates to one
    for x in xs[:200]:
        dot = float(np.float32(m) @ x)
        ref = -np.log(4 * np.pi) if kappa < 1e-3 else (
            np.log(kappa) - np.log(2 * np.pi) - np.log(-np.expm1(-2 * kappa)) + dot - kappa)
        assert po.vmf_logpdf(m, x) == pytest.approx(ref, abs=2e-5 * max(1.0, kappa))
    if kappa <= 3.0:
        g = rng.normal(size=(20000, 3))
        g /= np.linalg.norm(g, axis=1, keepdims=True)
        pdf = np.exp([po.vmf_logpdf(m, x) for x in g])
        assert abs(4 * np.pi * pdf.mean() - 1.0) < 5.0 * 4 * np.pi * pdf.std() / np.sqrt(len(g)) + 1e-6
