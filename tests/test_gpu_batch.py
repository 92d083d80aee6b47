"""Batched sweeps (ether_batch_*): kernels per member group, colour phase and member class over
many contexts leave every member exactly as its own ether_metropolis would -- spins bit for bit and the
acceptance counters -- for mixed sizes and models (simple-cubic Ising with 16-, 8- and 4-byte
vectors, general Ising, simple-cubic XYZ, general XYZ and Ising on the pyrochlore lattice,
whose colourings have more than two classes), for every tile shape and walk and after the
autotuner."""
import numpy as np
import pytest

import ether_gb300 as eg
from tests.helpers import beta_of, random_ising, random_xyz

pytestmark = pytest.mark.gpu

FM = [[(1, 1, (-1.0, -1.0, -1.0))]]
AFM = [[(1, 1, (1.0, 1.0, 1.0))]]

# (lattice, model, couplings, replicas, flags)
SPECS = [
    (lambda: eg.simple_cubic((32, 8, 6)), eg.MODEL_ISING, FM, 3, 0),       # 16-byte vectors
    (lambda: eg.simple_cubic(16), eg.MODEL_ISING, AFM, 2, 0),              # 8-byte vectors
    (lambda: eg.simple_cubic((8, 6, 4)), eg.MODEL_ISING, FM, 3, 0),        # 4-byte vectors
    (lambda: eg.simple_cubic(12), eg.MODEL_ISING, FM, 2, 0),               # H = 6: general path
    (lambda: eg.simple_cubic(8), eg.MODEL_ISING, FM, 2, eg.FLAG_FORCE_GENERAL),
    (lambda: eg.pyrochlore(2), eg.MODEL_ISING, AFM, 2, 0),
    (lambda: eg.simple_cubic(12), eg.MODEL_XYZ, FM, 2, 0),
    (lambda: eg.simple_cubic((6, 8, 10)), eg.MODEL_XYZ, AFM, 3, 0),
    (lambda: eg.pyrochlore(2), eg.MODEL_XYZ, AFM, 2, 0),
]


def build_members(specs=SPECS, seed0=11):
    """Member contexts of the specs (lattice, model, couplings, replicas, flags[, options])."""
    out = []
    for k, spec in enumerate(specs):
        mk, model, shells, R, flags = spec[:5]
        opts = spec[5] if len(spec) > 5 else {}
        lat = mk()
        j = eg.couplings(lat.n_species, shells, [1.0])
        sw = eg.Sweep.from_lattice(lat, j, np.asarray([1.0]), model, replicas=R,
                                   seed=1992 + 7 * k, flags=flags, **opts)
        sw.set_ladder([beta_of(3.0 + 1.5 * i) for i in range(R)])
        ion = random_ising(lat, seed0 + k) if model == eg.MODEL_ISING else random_xyz(lat, seed0 + k)
        sw.set_spins(ion)
        sw.set_streams(stream=[100 * k + r for r in range(R)], step=[3 * r for r in range(R)])
        out.append((lat, sw))
    return out


def member_class(lat, sw):
    """The batch kernel class of a member: model, fast path and, for simple-cubic Ising, the
    vector width (the largest of 16, 8 and 4 bytes that divides L1/2).  The members here have
    no Zeeman, SIA or ANGLE options."""
    info = sw.info()
    vec = 0
    if info.fast_path and sw.model == eg.MODEL_ISING:
        H = int(lat.sc[0]) // 2
        vec = 16 if H % 16 == 0 else 8 if H % 8 == 0 else 4
    return (sw.model, info.fast_path, vec)


def states(members):
    res = []
    for lat, sw in members:
        for r in range(sw.R):
            g = sw.get_spins(lat.ion, r)
            res.append(g[:, [1, 2, 3, 5]].copy())
        res.append(sw.accept_counts().astype(np.float64))
    return res


def assert_same(a, b):
    assert len(a) == len(b)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)


@pytest.mark.parametrize("config", [(256, 2, 0, 0), (128, 1, 1, 1), (64, 8, 2, 0), (256, 64, 0, 1),
                                    (128, 4, 0, 1), (128, 2, 0, 2), (64, 1, 0, 2)])
def test_batch_equals_member_sweeps(config):
    A = build_members()
    B = build_members()
    batch = eg.Batch([sw for _, sw in A])
    batch.set_config(*config)
    batch.metropolis(4)
    for _, sw in B:
        sw.metropolis(4)
    assert_same(states(A), states(B))
    info = batch.info()
    assert info.n_members == len(SPECS)
    assert info.n_replicas == sum(s[3] for s in SPECS)
    # one kernel per (colour phase, member class) with work, and the sweep-counter advance
    assert info.kernels_per_sweep == 1 + sum(
        len({member_class(lat, sw) for lat, sw in A if sw.info().n_colours > p})
        for p in range(max(sw.info().n_colours for _, sw in A)))
    assert info.site_updates_per_sweep == sum(sw.N * sw.R for _, sw in A)
    assert info.kernel_launches == 4 * info.kernels_per_sweep
    assert info.last_sweep_ms > 0.0
    batch.close()


def test_batch_interleaves_with_member_calls():
    """Stream ordering: batch sweeps, a member's own sweep, more batch sweeps."""
    A = build_members()
    B = build_members()
    batch = eg.Batch([sw for _, sw in A])
    batch.metropolis(2)
    A[0][1].metropolis(1)
    A[5][1].metropolis(1)
    batch.metropolis(1)
    for k, (_, sw) in enumerate(B):
        sw.metropolis(2)
        if k in (0, 5):
            sw.metropolis(1)
        sw.metropolis(1)
    assert_same(states(A), states(B))
    batch.close()


def test_batch_autotune_restores_state_and_keeps_parity():
    A = build_members()
    B = build_members()
    batch = eg.Batch([sw for _, sw in A])
    before = states(A)
    cfg, ms = batch.autotune()
    # walk 2 (one block per tile) ignores the blocks per SM, reported as 0
    assert cfg[0] in (128, 256) and cfg[1] in (1, 2, 4, 8, 16, 32) and cfg[3] in (0, 1, 2)
    assert cfg[2] >= 1 or cfg[3] == 2
    assert ms > 0.0
    assert_same(states(A), before)
    batch.metropolis(3)
    for _, sw in B:
        sw.metropolis(3)
    assert_same(states(A), states(B))
    batch.close()


def test_batch_members_with_variants():
    """Members on other Ising kernel variants (8-byte vectors, several per thread)."""
    specs = [SPECS[0], SPECS[1], SPECS[6]]
    A = build_members(specs)
    B = build_members(specs)
    A[0][1].set_variant(84)
    B[0][1].set_variant(161)
    batch = eg.Batch([sw for _, sw in A])
    batch.metropolis(3)
    for _, sw in B:
        sw.metropolis(3)
    assert_same(states(A), states(B))
    batch.close()


def test_batch_rejects_bad_input():
    A = build_members(SPECS[:2])
    with pytest.raises(eg.EtherError):
        eg.Batch([A[0][1], A[0][1]])
    batch = eg.Batch([sw for _, sw in A])
    with pytest.raises(eg.EtherError):
        batch.set_config(96, 1, 0)
    with pytest.raises(eg.EtherError):
        batch.set_config(128, 1, 0, walk=3)
    with pytest.raises(eg.EtherError):
        batch.metropolis(-1)
    batch.close()


def test_batch_members_with_field_anisotropy_and_angle_proposals():
    """The XYZ classes with options (Zeeman, SIA, ANGLE proposals) on simple-cubic and general
    lattices, beside exchange-only members: spins and counters as the members' own sweeps."""
    zs = {"zeeman": True, "h": (0.0, 0.3, 1.0), "g_factor": 2.0, "sia": True,
          "sia_vec": np.array([[0.0, 0.0, -0.3e-3]])}
    specs = [
        (lambda: eg.simple_cubic(12), eg.MODEL_XYZ, FM, 2, 0, zs),
        (lambda: eg.simple_cubic((6, 8, 10)), eg.MODEL_XYZ, AFM, 2, 0, {"angle": True, "dphi": 0.6}),
        (lambda: eg.pyrochlore(2), eg.MODEL_XYZ, AFM, 2, 0, zs),
        (lambda: eg.simple_cubic(8), eg.MODEL_XYZ, FM, 2, 0),
        (lambda: eg.simple_cubic(16), eg.MODEL_ISING, AFM, 2, 0),
    ]
    A = build_members(specs)
    B = build_members(specs)
    batch = eg.Batch([sw for _, sw in A])
    batch.metropolis(4)
    for _, sw in B:
        sw.metropolis(4)
    assert_same(states(A), states(B))
    batch.close()


def test_batch_large_member_runs_its_own_kernels():
    """A member above the L2 group budget of half the L2 (64^3 x 48 XYZ replicas = 201 MB,
    beside smaller members) runs its own phase kernels inside the batch graph: the same spins
    and counters as the members' own sweeps."""
    specs = [
        (lambda: eg.simple_cubic(16), eg.MODEL_ISING, AFM, 2, 0),
        (lambda: eg.simple_cubic(64), eg.MODEL_XYZ, FM, 48, 0),
        (lambda: eg.simple_cubic(12), eg.MODEL_XYZ, FM, 2, 0),
    ]
    A = build_members(specs)
    B = build_members(specs)
    batch = eg.Batch([sw for _, sw in A])
    batch.metropolis(3)
    for _, sw in B:
        sw.metropolis(3)
    assert_same(states(A), states(B))
    info = batch.info()
    assert info.site_updates_per_sweep == sum(sw.N * sw.R for _, sw in A)
    # groups: the Ising member, the large member alone, the small XYZ member; per sweep the
    # large member's two phase kernels, one class kernel per phase for each small member's
    # group, and the counter advance
    assert info.kernels_per_sweep == 2 + 2 * 2 + 1
    batch.close()


def test_batch_members_with_local_axis_anisotropy():
    """Members with per-site local-axis anisotropy (pyrochlore <111> axes; a simple-cubic
    lattice with two axis classes) in the XYZ option classes: as their own sweeps."""
    def members():
        out = []
        lat = eg.pyrochlore(2)
        ax = eg.local_111_axes(lat)
        sl = np.concatenate([ax, np.full((lat.N, 1), -0.2e-3)], axis=1)
        sc = eg.simple_cubic(12)
        par = (np.arange(sc.N) % 12 + (np.arange(sc.N) // 12) % 12 + np.arange(sc.N) // 144) % 2
        sl2 = np.where(par[:, None] == 0, [[0.0, 0.0, 1.0, -0.3e-3]], [[0.6, 0.8, 0.0, 0.1e-3]])
        for k, (l, shells, s) in enumerate(((lat, AFM, sl), (sc, FM, sl2))):
            j = eg.couplings(1, shells, [1.0])
            sw = eg.Sweep.from_lattice(l, j, np.asarray([1.0]), eg.MODEL_XYZ, replicas=2, seed=5 + k,
                                       sia_local=s)
            sw.set_ladder([beta_of(1.0), beta_of(2.5)])
            sw.set_spins(random_xyz(l, 40 + k))
            out.append((l, sw))
        lat3 = eg.simple_cubic(8)
        sw3 = eg.Sweep.from_lattice(lat3, eg.couplings(1, FM, [1.0]), np.asarray([1.0]), eg.MODEL_XYZ, replicas=2)
        sw3.set_ladder([beta_of(1.0), beta_of(2.5)])
        sw3.set_spins(random_xyz(lat3, 9))
        out.append((lat3, sw3))
        return out
    A, B = members(), members()
    batch = eg.Batch([sw for _, sw in A])
    batch.metropolis(4)
    for _, sw in B:
        sw.metropolis(4)
    assert_same(states(A), states(B))
    batch.close()


def test_batch_mcs_equals_each_members_own_mcs():
    """ether_batch_mcs against every member's own ether_mcs under one schedule (overrelaxation
    every 3 steps, PT every 2, measurement every 4 after 6 equilibration steps): spins,
    acceptance counters, per-temperature acceptance, slot permutations, measurement sums,
    spiral sums and swap counters bit for bit, over a captured chunk (24 steps) and a short
    direct one (3 steps).  Members: Ising and XYZ on simple-cubic and pyrochlore lattices
    (PT and measurement in the batched launches, one of them also sampling the spiral state
    per member), an XYZ member with a field, which does not overrelax, and a member in the
    reference-copy PT mode, which keeps its own PT and measurement kernels."""
    zs = {"zeeman": True, "h": (0.0, 0.3, 1.0), "g_factor": 2.0}
    specs = [SPECS[0], SPECS[2], SPECS[5], SPECS[6], SPECS[8],
             (lambda: eg.simple_cubic(8), eg.MODEL_XYZ, FM, 2, 0, zs),
             (lambda: eg.simple_cubic(6), eg.MODEL_XYZ, AFM, 3, eg.FLAG_PT_REFERENCE_COPY)]
    sch = dict(tmcs_eq=6, coa=4, ovrr=True, ovrr_para=0.5, ovrr_mcs=3, pt=True, exchange_interval=2)
    A = build_members(specs)
    B = build_members(specs)
    for X in (A, B):
        assert X[3][1].spiral_setup(1.01) > 0
    for _, sw in A + B:
        sw.zero_avg()
    batch = eg.Batch([sw for _, sw in A])
    swaps = batch.mcs(0, 24, swap_counts=[5 * k for k in range(len(specs))], **sch)
    swaps = batch.mcs(24, 3, swap_counts=swaps, **sch)
    own = []
    for k, (_, sw) in enumerate(B):
        s = sw.mcs(0, 24, swap_count=5 * k, **sch)
        own.append(sw.mcs(24, 3, swap_count=s, **sch))
    np.testing.assert_array_equal(swaps, own)
    assert_same(states(A), states(B))
    for (_, a), (_, b) in zip(A, B):
        np.testing.assert_array_equal(a.slots(), b.slots())
        np.testing.assert_array_equal(a.sums(), b.sums())
        np.testing.assert_array_equal(a.slot_accept_counts(), b.slot_accept_counts())
    np.testing.assert_array_equal(A[3][1].spiral_avg(), B[3][1].spiral_avg())
    assert all(b_.sums()[:, 0].max() > 0 for _, b_ in B)  # measurements happened
    assert batch.info().last_sweep_ms > 0.0
    batch.close()
