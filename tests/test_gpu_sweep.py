"""GPU parity of the Metropolis colour phases against the oracle's Checkerboard mode.

Ising: bit-exact spin trajectories (fixed-stream replay).  XYZ: the GPU's FP32 state equals
the oracle's FP32 mirror bit for bit, and its observables stay within 1e-5 relative of the
oracle's FP64 replay over the first 100 sweeps.
"""
import ctypes as C

import numpy as np
import pytest

import ether_gb300 as eg
from tests.helpers import beta_of, make_pair, random_ising, random_xyz

pytestmark = pytest.mark.gpu

FM = [[(1, 1, (-1.0, -1.0, -1.0))]]       # ETHER's sign: J < 0 is ferromagnetic
AFM_J1_J2 = [[(1, 1, (1.0, 1.0, 1.0))], [(1, 1, (-0.1, -0.1, -0.1))]]


def ising_replay(lat, shells, kT, sweeps, flags=0, seed=1992, stream=0, variant=None,
                 autotune=False, **kw):
    sw, osys = make_pair(lat, eg.MODEL_ISING, shells, flags=flags, seed=seed, **kw)
    beta = beta_of(kT)
    sw.set_beta(beta)
    if variant is not None:
        sw.set_variant(variant)
    sw.set_streams(stream=[stream], step=[0])
    ncol, col, rank = osys.colouring()
    gcol, grank = sw.colouring()
    assert ncol == sw.info().n_colours
    np.testing.assert_array_equal(col, gcol)
    np.testing.assert_array_equal(rank, grank)
    ion = random_ising(lat, 7)
    sw.set_spins(ion)
    if autotune:
        sw.autotune()
    acc_o = []
    for t in range(sweeps):
        acc_o.append(osys.metropolis_colour(ion, None, 64, beta, seed, stream, t, col, rank, ncol))
    acc_g = sw.metropolis(sweeps)
    g = sw.get_spins(lat.ion)
    return sw, ion, g, sum(acc_o), acc_g[0]


# L = 8 and (24, 6, 4) take the 4-byte vectors (L1/2 = 4, 12), 16 the 8-byte ones, 6 and 5
# the general path
@pytest.mark.parametrize("L,flags", [(8, 0), (16, 0), (8, eg.FLAG_FORCE_GENERAL), (6, 0), (5, 0),
                                     ((16, 8, 12), 0), ((24, 6, 4), 0)])
@pytest.mark.parametrize("kT", [4.511, 2.0, 10.0])
def test_ising_sc_bit_exact(L, flags, kT):
    lat = eg.simple_cubic(L)
    sw, ion, g, ao, ag = ising_replay(lat, FM, kT, 20, flags=flags)
    np.testing.assert_array_equal(g[:, 3], ion[:, 3])
    assert ao == pytest.approx(ag, abs=1e-12)
    if flags == 0 and L in (8, 16, (24, 6, 4)):
        assert sw.info().fast_path == 1


@pytest.mark.parametrize("variant", [161, 162, 164, 81, 82, 84, 41, 42, 44, 2162, 2164, 6162, 1162, 1164,
                                     1082, 1084, 1042, 1044, 3162, 3164])
def test_ising_sc_every_kernel_variant_bit_exact(variant):
    lat = eg.simple_cubic((32, 8, 6))
    sw, ion, g, ao, ag = ising_replay(lat, FM, 4.511, 8, variant=variant)
    np.testing.assert_array_equal(g[:, 3], ion[:, 3])
    assert ao == pytest.approx(ag, abs=1e-12)


# the shared-memory staged kernel: one halo stage (32 x 16 x 32: 2 steps per replica) and two
# halo stages with the ring wrapping many times (128 x 64 x 16: 16 steps per replica)
@pytest.mark.parametrize("variant", [4011, 4014, 4021, 4041])
@pytest.mark.parametrize("L", [(32, 16, 64), (128, 64, 32)])
def test_ising_staged_kernel_bit_exact(variant, L):
    lat = eg.simple_cubic(L)
    sw, ion, g, ao, ag = ising_replay(lat, FM, 4.511, 6, variant=variant)
    np.testing.assert_array_equal(g[:, 3], ion[:, 3])
    assert ao == pytest.approx(ag, abs=1e-12)
    sw.sync()  # no bounded wait ran out


def test_ising_general_lattice_both_kernel_forms_bit_exact():
    """The general-lattice Ising phase has two forms: a group of eight sites per thread when
    the colour classes of all replicas hold enough groups to fill the GPU, one site per thread
    otherwise.  32^3 through the general path with 48 replicas takes the group form; replicas
    0 and 47 are replayed by the oracle."""
    lat = eg.simple_cubic(32)
    sw, osys = make_pair(lat, eg.MODEL_ISING, FM, replicas=48, flags=eg.FLAG_FORCE_GENERAL)
    beta = beta_of(4.511)
    sw.set_beta(beta)
    assert sw.info().fast_path == 0
    ncol, col, rank = osys.colouring()
    ions = [random_ising(lat, 100 + r) for r in range(48)]
    for r in range(48):
        sw.set_spins(ions[r], r)
    sw.metropolis(3)
    for r in (0, 47):
        ion = ions[r].copy()
        for t in range(3):
            osys.metropolis_colour(ion, None, 64, beta, 1992, r, t, col, rank, ncol)
        np.testing.assert_array_equal(sw.get_spins(lat.ion, r)[:, 3], ion[:, 3])


def test_ising_tie_path_bit_exact():
    """1.3M updates: about 20 sites whose high 16 random bits tie with the threshold's and
    are decided by the low halves (the rarely taken branch of both kernels)."""
    for flags in (0, eg.FLAG_FORCE_GENERAL):
        lat = eg.simple_cubic(32)
        sw, ion, g, ao, ag = ising_replay(lat, FM, 4.511, 40, flags=flags)
        np.testing.assert_array_equal(g[:, 3], ion[:, 3])
        assert ao == pytest.approx(ag, abs=1e-12)


def test_autotuner_restores_state_and_stays_bit_exact():
    lat = eg.simple_cubic(32)
    sw, ion, g, ao, ag = ising_replay(lat, FM, 4.511, 12, autotune=True)
    np.testing.assert_array_equal(g[:, 3], ion[:, 3])
    assert ao == pytest.approx(ag, abs=1e-12)


def test_ising_open_bc_and_zeeman_bit_exact():
    lat = eg.simple_cubic((6, 5, 4), bc="coc")
    sw, ion, g, ao, ag = ising_replay(lat, FM, 3.0, 15, zeeman=True, h=(0.0, 0.0, 2.0),
                                      g_factor=2.0)
    np.testing.assert_array_equal(g[:, 3], ion[:, 3])
    assert sw.info().n_types > 1


def test_ising_pyrochlore_two_shells_bit_exact():
    lat = eg.pyrochlore(2, shells=(2.97243, 5.1484))
    lat = eg.Lattice(lat.basis_cart, [1] * 16, lat.abc, (2, 2, 2), [2.97243, 5.1484], tol=1e-3)
    sw, ion, g, ao, ag = ising_replay(lat, AFM_J1_J2, 1.5, 25)
    np.testing.assert_array_equal(g[:, 3], ion[:, 3])
    assert sw.info().n_colours > 2


def xyz_replay(lat, shells, kT, sweeps, flags=0, seed=1992, stream=3, variant=None, autotune=False,
               **kw):
    sw, osys = make_pair(lat, eg.MODEL_XYZ, shells, flags=flags, seed=seed, **kw)
    beta = beta_of(kT)
    sw.set_beta(beta)
    if variant is not None:
        sw.set_variant(variant)
    sw.set_streams(stream=[stream], step=[0])
    ncol, col, rank = osys.colouring()
    ion = random_xyz(lat, 11)
    sw.set_spins(ion)
    if autotune:
        sw.autotune()
    sp4 = osys.spin4(ion)
    ion64 = ion.copy()
    for t in range(sweeps):
        osys.metropolis_colour(ion, sp4, 32, beta, seed, stream, t, col, rank, ncol)
        osys.metropolis_colour(ion64, None, 64, beta, seed, stream, t, col, rank, ncol)
    sw.metropolis(sweeps)
    g = sw.get_spins(lat.ion)
    return sw, osys, sp4, ion64, g


@pytest.mark.parametrize("L,flags", [(4, 0), (8, 0), (8, eg.FLAG_FORCE_GENERAL), (5, 0)])
@pytest.mark.parametrize("angle", [False, True])
def test_xyz_sc_matches_fp32_mirror(L, flags, angle):
    lat = eg.simple_cubic(L)
    sw, osys, sp4, ion64, g = xyz_replay(lat, FM, 1.443, 30, flags=flags, angle=angle,
                                         dphi=np.deg2rad(50.0))
    np.testing.assert_array_equal(g[:, 1].astype(np.float32), sp4[:, 0])
    np.testing.assert_array_equal(g[:, 2].astype(np.float32), sp4[:, 1])
    np.testing.assert_array_equal(g[:, 3].astype(np.float32), sp4[:, 2])
    np.testing.assert_array_equal(g[:, 5].astype(np.float32), sp4[:, 3])


# every simple-cubic XYZ kernel variant (sites per thread, register cap), for both option
# sets (exchange only with Marsaglia proposals, and ANGLE with a Zeeman field); (20, 6, 6)
# has 360 sites per colour, so the two-site variants meet a ragged last tile
@pytest.mark.parametrize("variant", [5011, 5012, 5013, 5014, 5015, 5021, 5022])
@pytest.mark.parametrize("opts", [{}, {"angle": True, "dphi": 0.7, "zeeman": True, "h": (0.0, 0.5, 1.0)}])
def test_xyz_sc_every_kernel_variant_matches_fp32_mirror(variant, opts):
    lat = eg.simple_cubic((20, 6, 6))
    sw, osys, sp4, ion64, g = xyz_replay(lat, FM, 1.443, 12, variant=variant, **opts)
    assert sw.info().fast_path == 1
    for k, col in ((1, 0), (2, 1), (3, 2), (5, 3)):
        np.testing.assert_array_equal(g[:, k].astype(np.float32), sp4[:, col])


def test_xyz_autotuner_restores_state_and_matches_fp32_mirror():
    lat = eg.simple_cubic(16)
    sw, osys, sp4, ion64, g = xyz_replay(lat, FM, 1.443, 10, autotune=True)
    v, _ = sw.autotune()
    assert 5011 <= v <= 5022
    for k, col in ((1, 0), (2, 1), (3, 2), (5, 3)):
        np.testing.assert_array_equal(g[:, k].astype(np.float32), sp4[:, col])


def test_xyz_zeeman_sia_pyrochlore_matches_fp32_mirror():
    lat = eg.Lattice(eg.pyrochlore(2).basis_cart, [1] * 16, np.eye(3) * eg.model.PYROCHLORE_A,
                     (2, 2, 2), [2.97243, 5.1484], tol=1e-3)
    sia = np.array([[0.0, 0.0, -0.2e-3]])
    sw, osys, sp4, ion64, g = xyz_replay(lat, AFM_J1_J2, 2.0, 20, zeeman=True, h=(0.0, 0.0, 1.0),
                                         g_factor=2.0, sia=True, sia_vec=sia)
    np.testing.assert_array_equal(g[:, 1:4].astype(np.float32), sp4[:, 0:3])


def test_xyz_observables_within_1e5_of_fp64_over_100_sweeps():
    """Fixed-stream tolerance check: FP32 GPU vs the FP64 replay of the same draws."""
    lat = eg.simple_cubic(8)
    sw, osys, sp4, ion64, g = xyz_replay(lat, FM, 1.443, 100)
    E_gpu = sw.tot_energy()[0]
    M_gpu = np.linalg.norm(sw.tot_magnetisation()[0])
    E_64 = osys.tot_energy(ion64)
    M_64 = np.linalg.norm(osys.tot_magnetisation(ion64))
    assert abs(E_gpu - E_64) <= 1e-5 * abs(E_64)
    assert abs(M_gpu - M_64) <= 1e-5 * abs(M_64)


def test_energy_magnetisation_match_oracle():
    lat = eg.simple_cubic(6, checkerboard=True)
    for model in (eg.MODEL_ISING, eg.MODEL_XYZ):
        sw, osys = make_pair(lat, model, FM, zeeman=True, h=(0.3, -0.2, 1.0), g_factor=2.0)
        ion = random_ising(lat, 3) if model == eg.MODEL_ISING else random_xyz(lat, 3)
        sw.set_spins(ion)
        E = sw.tot_energy()[0]
        M = sw.tot_magnetisation()[0]
        if model == eg.MODEL_ISING:
            assert E == pytest.approx(osys.tot_energy(ion), rel=1e-12, abs=1e-15)
            np.testing.assert_allclose(M, osys.tot_magnetisation(ion), rtol=1e-12, atol=1e-12)
        else:
            sp4 = osys.spin4(ion)
            assert E == pytest.approx(osys.tot_energy_f32(ion, sp4), rel=1e-12)
            assert E == pytest.approx(osys.tot_energy(ion), rel=1e-5)
            np.testing.assert_allclose(M, osys.tot_magnetisation_f32(ion, sp4), rtol=1e-12, atol=1e-9)


# flags 0: the simple-cubic kernel (closed-form neighbours); FORCE_GENERAL: the ELL kernel
@pytest.mark.parametrize("flags", [0, eg.FLAG_FORCE_GENERAL])
@pytest.mark.parametrize("para", [0.4, 1.0, 1.7])
def test_overrelaxation_matches_oracle_and_conserves_energy(para, flags):
    lat = eg.simple_cubic(8)
    sw, osys = make_pair(lat, eg.MODEL_XYZ, FM, flags=flags)
    assert sw.info().fast_path == (0 if flags else 1)
    sw.set_beta(1.0)
    sw.set_streams(stream=[5], step=[0])
    ion = random_xyz(lat, 5)
    sw.set_spins(ion)
    E0 = sw.tot_energy()[0]
    ncol, col, rank = osys.colouring()
    sp4 = osys.spin4(ion)
    osys.overrelax_colour(ion, sp4, para, 1992, 5, 0, col, rank, ncol)
    sw.overrelaxation(para)
    g = sw.get_spins(lat.ion)
    np.testing.assert_array_equal(g[:, 1:4].astype(np.float32), sp4[:, 0:3])
    E1 = sw.tot_energy()[0]
    assert E1 == pytest.approx(E0, rel=1e-5)


@pytest.mark.parametrize("model,angle", [(eg.MODEL_ISING, False), (eg.MODEL_XYZ, False),
                                         (eg.MODEL_XYZ, True)])
def test_fresh_spins_match_oracle(model, angle):
    lat = eg.simple_cubic(6)
    sw, osys = make_pair(lat, model, FM, angle=angle, dphi=0.5)
    sw.set_streams(stream=[9], step=[0])
    ion = random_ising(lat, 1) if model == eg.MODEL_ISING else random_xyz(lat, 1)
    sw.set_spins(ion)
    sp4 = osys.spin4(ion)
    osys.fresh_spins_colour(ion, sp4, 1992, 9, 0)
    sw.fresh_spins()
    g = sw.get_spins(lat.ion)
    if model == eg.MODEL_ISING:
        np.testing.assert_array_equal(g[:, 3], ion[:, 3])
    else:
        np.testing.assert_array_equal(g[:, 1:4].astype(np.float32), sp4[:, 0:3])


def test_replicas_are_independent_streams():
    lat = eg.simple_cubic(16)
    sw, osys = make_pair(lat, eg.MODEL_ISING, FM, replicas=4)
    sw.set_beta([beta_of(4.511)] * 4)
    sw.set_streams(stream=[0, 1, 0, 2], step=[0, 0, 0, 0])
    ion = random_ising(lat, 2)
    sw.set_spins(ion)
    sw.metropolis(10, accept=False)
    s = [sw.get_spins(lat.ion, r)[:, 3] for r in range(4)]
    np.testing.assert_array_equal(s[0], s[2])
    assert not np.array_equal(s[0], s[1])
    assert not np.array_equal(s[1], s[3])


@pytest.mark.parametrize("model", [eg.MODEL_ISING, eg.MODEL_XYZ])
@pytest.mark.parametrize("L", [(8, 6, 4), (5, 5, 5)])
def test_set_spins_every_replica(model, L):
    """replica = -1: one upload, replicated on the device (sizes with and without 16-byte
    multiples per replica)."""
    lat = eg.simple_cubic(L)
    sw, osys = make_pair(lat, model, FM, replicas=5)
    ion = random_ising(lat, 3) if model == eg.MODEL_ISING else random_xyz(lat, 3)
    sw.set_spins(ion)
    cols = [3] if model == eg.MODEL_ISING else [1, 2, 3, 5]
    for r in range(5):
        g = sw.get_spins(lat.ion, r)
        np.testing.assert_array_equal(g[:, cols], ion[:, cols].astype(np.float32).astype(np.float64))
    other = random_ising(lat, 4) if model == eg.MODEL_ISING else random_xyz(lat, 4)
    sw.set_spins(other, 2)
    np.testing.assert_array_equal(sw.get_spins(lat.ion, 2)[:, cols], other[:, cols].astype(np.float32).astype(np.float64))
    np.testing.assert_array_equal(sw.get_spins(lat.ion, 3)[:, cols], ion[:, cols].astype(np.float32).astype(np.float64))


# The general-lattice kernels are instantiated for common ELL widths: bcc (8 nearest
# neighbours), fcc (12), and the simple-cubic first + second shells (6 + 12 = 18); every form
# must reproduce the oracle bit for bit.
def _lattice(kind):
    if kind == "bcc":
        return eg.Lattice([[0.0, 0.0, 0.0], [0.5, 0.5, 0.5]], [1, 1], np.eye(3), (4, 4, 4), [0.8660254]), FM
    if kind == "fcc":
        return eg.Lattice([[0.0, 0.0, 0.0], [0.0, 0.5, 0.5], [0.5, 0.0, 0.5], [0.5, 0.5, 0.0]], [1, 1, 1, 1],
                          np.eye(3), (3, 3, 3), [0.70710678]), FM
    return eg.Lattice([[0.0, 0.0, 0.0]], [1], np.eye(3), (6, 6, 6), [1.0, 1.41421356]), AFM_J1_J2


@pytest.mark.parametrize("kind,width", [("bcc", 8), ("fcc", 12), ("sc2", 18)])
def test_general_lattice_widths_bit_exact(kind, width):
    lat, shells = _lattice(kind)
    sw, ion, g, ao, ag = ising_replay(lat, shells, 4.0, 12)
    assert sw.info().fast_path == 0
    np.testing.assert_array_equal(g[:, 3], ion[:, 3])
    assert ao == pytest.approx(ag, abs=1e-12)
    sw, osys, sp4, ion64, g = xyz_replay(lat, shells, 1.5, 12)
    for k, col in ((1, 0), (2, 1), (3, 2), (5, 3)):
        np.testing.assert_array_equal(g[:, k].astype(np.float32), sp4[:, col])


@pytest.mark.parametrize("model", [eg.MODEL_ISING, eg.MODEL_XYZ])
def test_single_sweep_with_acceptance_graph_equals_direct_launches(model):
    """ether_metropolis(ctx, 1, accept) replays a captured graph (one per kernel variant);
    with ETHER_FLAG_NO_GRAPHS it launches directly: same spins and acceptance ratios, also
    across a change of kernel variant."""
    lat = eg.simple_cubic((32, 8, 6))
    runs = []
    for flags in (0, eg.FLAG_NO_GRAPHS):
        j = eg.couplings(1, FM, [1.0])
        sw = eg.Sweep.from_lattice(lat, j, np.array([1.0]), model, replicas=3, seed=17, flags=flags)
        sw.set_beta([beta_of(k) for k in (3.0, 4.5, 6.0)] if model == eg.MODEL_ISING else
                    [beta_of(k) for k in (1.0, 1.4, 2.0)])
        sw.set_spins(random_ising(lat, 3) if model == eg.MODEL_ISING else random_xyz(lat, 3))
        accs = [sw.metropolis(1) for _ in range(4)]
        sw.set_variant(81 if model == eg.MODEL_ISING else 5021)
        accs += [sw.metropolis(1) for _ in range(4)]
        runs.append((np.array(accs), sw.get_spins(lat.ion, 2)[:, [1, 2, 3]].copy()))
        sw.close()
    np.testing.assert_array_equal(runs[0][0], runs[1][0])
    np.testing.assert_array_equal(runs[0][1], runs[1][1])


@pytest.mark.parametrize("staged", [False, True])
@pytest.mark.parametrize("model,L,R", [(eg.MODEL_ISING, (64, 32, 32), 70), (eg.MODEL_XYZ, (32, 16, 20), 60)])
def test_spins_batch_equals_per_replica_calls(model, L, R, staged):
    """ether_set_spins_batch / ether_get_spins_batch move ion(0:8, N, n) of many replicas at
    once: the same device state and the same ion records as one ether_set_spins /
    ether_get_spins per replica, both where a kernel reads and writes the records in place
    (a device that addresses pageable host memory) and with the conversion in chunks of whole
    replicas on several host threads (ETHER_FLAG_STAGED_SPINS).  The sizes give two (Ising)
    and three (XYZ) staging chunks, the last one partial."""
    lat = eg.simple_cubic(L)
    sw, _ = make_pair(lat, model, FM, replicas=R, flags=eg.FLAG_STAGED_SPINS if staged else 0)
    direct = sw.info().ion_direct
    print("ion records moved %s" % ("in place by a kernel" if direct else "through host staging"))
    if staged:
        assert direct == 0
    sw.set_beta(beta_of(4.511 if model == eg.MODEL_ISING else 1.443))
    mk = random_ising if model == eg.MODEL_ISING else random_xyz
    ions = np.stack([mk(lat, 500 + r) for r in range(R)])
    sw.set_spins_batch(ions)
    cols = [3] if model == eg.MODEL_ISING else [1, 2, 3, 5]
    for r in (0, 1, R // 2, R - 1):
        np.testing.assert_array_equal(sw.get_spins(lat.ion, r)[:, cols],
                                      ions[r][:, cols].astype(np.float32).astype(np.float64))
    sw.metropolis(2, accept=False)
    got = np.stack([lat.ion] * R).copy()
    got[:, :, 0] = -7.0  # columns the call must not touch
    sw.get_spins_batch(got)
    assert np.all(got[:, :, 0] == -7.0)
    for r in range(R):
        np.testing.assert_array_equal(got[r][:, cols], sw.get_spins(lat.ion, r)[:, cols])
    # a sub-range: replicas 5 .. 5+k-1
    k = R - 9
    sub = ions[:k].copy()
    sub[:, :, 3] *= -1.0 if model == eg.MODEL_ISING else 1.0
    sw.set_spins_batch(sub, r0=5)
    back = np.stack([lat.ion] * k).copy()
    sw.get_spins_batch(back, r0=5)
    np.testing.assert_array_equal(back[:, :, cols], sub[:, :, cols].astype(np.float32).astype(np.float64))
    np.testing.assert_array_equal(sw.get_spins(lat.ion, 4)[:, cols], got[4][:, cols])
    sw.close()


def test_spins_batch_shares_the_work_and_keeps_the_records():
    """Where the records can move in place: an upload shares its replicas between the kernel
    (chunks from the front) and the host's cores (chunks from the back) as it runs, and so does
    a read-back.  Every call leaves the same device state and records, also right after a
    sweep that is still running."""
    lat = eg.simple_cubic((32, 16, 16))
    R = 40
    sw, _ = make_pair(lat, eg.MODEL_ISING, FM, replicas=R)
    if not sw.info().ion_direct:
        sw.close()
        pytest.skip("the records are staged through the host on this system")
    sw.set_beta(beta_of(4.5))
    ions = np.stack([random_ising(lat, 40 + r) for r in range(R)])
    gets, sets = [], []
    for k in range(5):
        sw.metropolis(1, accept=False)   # left running: the upload must wait for it
        sw.set_spins_batch(ions)
        sets.append(sw.spins_batch_split()[1])
        back = np.stack([lat.ion] * R).copy()
        back[:, :, 0] = 5.0
        sw.get_spins_batch(back)
        gets.append(sw.spins_batch_split()[0])
        np.testing.assert_array_equal(back[:, :, 3], ions[:, :, 3])
        assert np.all(back[:, :, 0] == 5.0)
    print("kernel share of the uploads", sets, "of the read-backs", gets, "of", R)
    assert all(0 <= k <= R for k in sets + gets)
    sw.close()


def test_spins_batch_refuses_device_memory_before_any_launch():
    """Where a kernel moves the records in place, a pointer to device memory is refused before
    anything is launched (ETHER_ERR_ARG), in both directions, and the context keeps working."""
    torch = pytest.importorskip("torch")
    lat = eg.simple_cubic(8)
    sw, _ = make_pair(lat, eg.MODEL_ISING, FM, replicas=2)
    if not sw.info().ion_direct:
        sw.close()
        pytest.skip("the records are staged through the host on this system")
    sw.set_beta(beta_of(4.5))
    dev = torch.zeros(2 * lat.N * 9, dtype=torch.float64, device="cuda")
    launches = sw.info().kernel_launches
    for fn in (sw.lib.ether_set_spins_batch, sw.lib.ether_get_spins_batch):
        rc = fn(sw.h, 0, 2, C.cast(C.c_void_p(dev.data_ptr()), C.POINTER(C.c_double)))
        assert rc == -1  # ETHER_ERR_ARG
        assert b"not host memory" in sw.lib.ether_last_error()
    assert sw.info().kernel_launches == launches
    ions = np.stack([random_ising(lat, 3)] * 2)
    sw.set_spins_batch(ions)
    back = np.stack([lat.ion] * 2).copy()
    sw.get_spins_batch(back)
    np.testing.assert_array_equal(back[:, :, 3], ions[:, :, 3])
    sw.close()


def _sia_local(axes, D):
    return np.ascontiguousarray(np.concatenate([axes, np.broadcast_to(np.asarray(D, float), (len(axes),))[:, None]],
                                               axis=1))


def test_xyz_local_axis_sia_pyrochlore_matches_fp32_mirror():
    """Single-ion anisotropy D (a_i . S)^2 about each site's local <111> axis (D = -0.2 meV,
    easy axis), beside the reference's diagonal term and a Zeeman field, on the pyrochlore
    lattice with two shells: the GPU state equals the oracle's FP32 mirror bit for bit; E
    equals the mirror's to rounding and the FP64 replay's to 1e-5."""
    lat = eg.Lattice(eg.pyrochlore(2).basis_cart, [1] * 16, np.eye(3) * eg.model.PYROCHLORE_A,
                     (2, 2, 2), [2.97243, 5.1484], tol=1e-3)
    sia_local = _sia_local(eg.local_111_axes(lat), -0.2e-3)
    sw, osys, sp4, ion64, g = xyz_replay(lat, AFM_J1_J2, 2.0, 20, zeeman=True, h=(0.0, 0.0, 1.0),
                                         g_factor=2.0, sia=True, sia_vec=np.array([[0.0, 0.05e-3, 0.0]]),
                                         sia_local=sia_local)
    assert sw.info().fast_path == 0
    np.testing.assert_array_equal(g[:, 1:4].astype(np.float32), sp4[:, 0:3])
    E = sw.tot_energy()[0]
    ion = lat.ion.copy()
    assert E == pytest.approx(osys.tot_energy_f32(ion, sp4), rel=1e-12)
    assert E == pytest.approx(osys.tot_energy(ion64), rel=1e-5)


def test_xyz_local_axis_sia_simple_cubic_fast_path():
    """Two anisotropy classes (axis and D per checkerboard sublattice) on the simple-cubic fast
    kernel: bit-exact against the FP32 mirror; energy as the oracle's."""
    lat = eg.simple_cubic(8)
    rng = np.random.default_rng(4)
    two = rng.normal(size=(2, 3))
    two /= np.linalg.norm(two, axis=1, keepdims=True)
    par = (np.arange(lat.N) % 8 + (np.arange(lat.N) // 8) % 8 + np.arange(lat.N) // 64) % 2
    sia_local = _sia_local(two[par], np.where(par == 0, -0.3e-3, 0.2e-3))
    sw, osys, sp4, ion64, g = xyz_replay(lat, FM, 1.443, 15, sia_local=sia_local)
    assert sw.info().fast_path == 1
    for k, col in ((1, 0), (2, 1), (3, 2)):
        np.testing.assert_array_equal(g[:, k].astype(np.float32), sp4[:, col])
    assert sw.tot_energy()[0] == pytest.approx(osys.tot_energy_f32(lat.ion.copy(), sp4), rel=1e-12)


def test_local_axis_sia_turns_overrelaxation_off_in_mcs():
    """As the reference's SIA does (src/ether.f90:163-168): ether_mcs with ovrr on leaves a
    context with local-axis anisotropy exactly as without ovrr."""
    lat = eg.simple_cubic(8)
    axes = np.tile([[0.0, 0.6, 0.8]], (lat.N, 1))
    runs = []
    for ovrr in (False, True):
        sw, _ = make_pair(lat, eg.MODEL_XYZ, FM, replicas=2, sia_local=_sia_local(axes, -0.1e-3))
        sw.set_beta([beta_of(1.2), beta_of(2.0)])
        sw.set_spins(random_xyz(lat, 8))
        sw.mcs(0, 30, 10, 5, ovrr=ovrr, ovrr_para=1.0, ovrr_mcs=3)
        runs.append(np.stack([sw.get_spins(lat.ion, r)[:, 1:4] for r in range(2)]))
        sw.close()
    np.testing.assert_array_equal(runs[0], runs[1])
