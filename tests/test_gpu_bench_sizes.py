"""Parity at the sizes the benchmark times.

The small-lattice parity tests fix the arithmetic; these run the same kernels with the
benchmark's own shapes, variants and replica counts, where the index arithmetic (replica
offsets near 2^28 bytes, grid.y = 1024, many tiles per colour class) differs:

* 64^3 Ising x 1024 replicas at T_c with the headline variant (16-byte vectors, four per
  thread, register cap) and with the autotuner's choice: replicas 0, 511 and 1023 replayed
  bit for bit by the oracle (src/Metropolis.f90:39-62 in Checkerboard order);
* 32^3 Heisenberg (the 32^3 + overrelaxation deck's lattice), 100 sweeps: FP32 state equal
  to the oracle's FP32 mirror, E and |M| within 1e-5 relative of the FP64 replay of the
  same draws; and 64^3 x 64 replicas (the Heisenberg benchmark) with the autotuned variant;
* the pyrochlore 16-site cell x 12^3 (27648 sites) with J1/J2, Zeeman and single-ion
  anisotropy along each site's local <111> axis, 64 replicas on the geometric 1-50 K ladder:
  bit-exact against the FP32 mirror;
* S(q) at N = 27648 on 512 sampled points of the 64^3 q-grid against the FP64 direct sum
  (utility/Structure_Factor/structure_factor.f90:131-183), with the error printed.
"""
import numpy as np
import pytest

import ether_gb300 as eg
from tests.helpers import KB, beta_of, make_pair, random_ising, random_xyz
from tests.test_gpu_sq import _gpu_sq, _oracle_sq

pytestmark = pytest.mark.gpu

FM = [[(1, 1, (-1.0, -1.0, -1.0))]]
PYRO_HEIS = [[(1, 1, (1.0, 1.0, 1.0))], [(1, 1, (-0.1, -0.1, -0.1))]]
PYRO_ISING = [[(1, 1, (-1.0, -1.0, -1.0))], [(1, 1, (-0.1, -0.1, -0.1))]]


@pytest.mark.parametrize("variant", [2164, "autotune"])
def test_ising_64cubed_1024_replicas_bit_exact(variant):
    L, R, sweeps = 64, 1024, 3
    lat = eg.simple_cubic(L)
    sw, osys = make_pair(lat, eg.MODEL_ISING, FM, replicas=R)
    beta = beta_of(4.511)
    sw.set_beta(beta)
    ion = random_ising(lat, 1992)
    sw.set_spins(ion)  # one upload, replicated; every replica has its own stream
    last = random_ising(lat, 7)
    sw.set_spins(last, R - 1)
    if variant == "autotune":
        v, _ = sw.autotune()
    else:
        sw.set_variant(variant)
        v = variant
    assert sw.info().fast_path == 1
    sw.metropolis(sweeps, accept=False)
    ncol, col, rank = osys.colouring()
    for r, start in ((0, ion), (511, ion), (R - 1, last)):
        want = start.copy()
        for t in range(sweeps):
            osys.metropolis_colour(want, None, 64, beta, 1992, r, t, col, rank, ncol)
        np.testing.assert_array_equal(sw.get_spins(lat.ion, r)[:, 3], want[:, 3],
                                      err_msg="replica %d, variant %s" % (r, v))
    sw.close()


def test_xyz_32cubed_100_sweeps_fp32_mirror_and_1e5_of_fp64():
    L, R, sweeps = 32, 2, 100
    lat = eg.simple_cubic(L)
    sw, osys = make_pair(lat, eg.MODEL_XYZ, FM, replicas=R)
    beta = beta_of(1.443)
    sw.set_beta(beta)
    sw.set_streams(stream=[0, 17], step=[0, 0])
    ion = random_xyz(lat, 11)
    sw.set_spins(ion)
    sw.metropolis(sweeps, accept=False)
    E_gpu = sw.tot_energy()
    M_gpu = np.linalg.norm(sw.tot_magnetisation(), axis=1)
    ncol, col, rank = osys.colouring()
    sp4 = osys.spin4(ion)
    ion64 = ion.copy()
    ion32 = ion.copy()
    for t in range(sweeps):
        osys.metropolis_colour(ion32, sp4, 32, beta, 1992, 17, t, col, rank, ncol)
        osys.metropolis_colour(ion64, None, 64, beta, 1992, 17, t, col, rank, ncol)
    g = sw.get_spins(lat.ion, 1)
    np.testing.assert_array_equal(g[:, 1:4].astype(np.float32), sp4[:, 0:3])
    E_64 = osys.tot_energy(ion64)
    M_64 = np.linalg.norm(osys.tot_magnetisation(ion64))
    print("ERROR Heisenberg 32^3, 100 sweeps, GPU FP32 against the FP64 replay: E %.3e, |M| %.3e "
          "relative" % (abs(E_gpu[1] - E_64) / abs(E_64), abs(M_gpu[1] - M_64) / abs(M_64)))
    assert abs(E_gpu[1] - E_64) <= 1e-5 * abs(E_64), (E_gpu[1], E_64)
    assert abs(M_gpu[1] - M_64) <= 1e-5 * abs(M_64), (M_gpu[1], M_64)
    sw.close()


def test_xyz_64cubed_64_replicas_autotuned_bit_exact():
    L, R, sweeps = 64, 64, 2
    lat = eg.simple_cubic(L)
    sw, osys = make_pair(lat, eg.MODEL_XYZ, FM, replicas=R)
    beta = beta_of(1.443)
    sw.set_beta(beta)
    ion = random_xyz(lat, 3)
    sw.set_spins(ion)
    v, _ = sw.autotune()
    assert 5011 <= v <= 5022
    sw.metropolis(sweeps, accept=False)
    ncol, col, rank = osys.colouring()
    for r in (0, R - 1):
        work = ion.copy()
        sp4 = osys.spin4(work)
        for t in range(sweeps):
            osys.metropolis_colour(work, sp4, 32, beta, 1992, r, t, col, rank, ncol)
        g = sw.get_spins(lat.ion, r)
        np.testing.assert_array_equal(g[:, 1:4].astype(np.float32), sp4[:, 0:3],
                                      err_msg="replica %d, variant %d" % (r, v))
    sw.close()


def _pyrochlore_12():
    return eg.pyrochlore(12, shells=(2.97243, 5.1484), tol=1e-3)


@pytest.mark.parametrize("model", [eg.MODEL_XYZ, eg.MODEL_ISING])
def test_pyrochlore_12_cells_ladder_bit_exact(model):
    """The benchmark's frustrated configuration: 27648 sites, two shells (6 + 12 neighbours),
    Zeeman H = (0, 0, 1) T with g = 2, for Heisenberg also D = -0.2 meV along each site's
    local <111> axis; 64 replicas on the geometric 1-50 K ladder; replicas 0, 31 and 63
    replayed."""
    lat = _pyrochlore_12()
    assert lat.N == 27648
    R, sweeps = 64, 3
    kw = dict(zeeman=True, h=(0.0, 0.0, 1.0), g_factor=2.0)
    if model == eg.MODEL_XYZ:
        axes = eg.local_111_axes(lat)
        kw.update(sia_local=np.concatenate([axes, np.full((lat.N, 1), -0.2e-3)], axis=1))
        shells = PYRO_HEIS
    else:
        shells = PYRO_ISING
    sw, osys = make_pair(lat, model, shells, replicas=R, **kw)
    temps = np.geomspace(1.0, 50.0, R)
    betas = 1.0 / (KB * temps)
    sw.set_beta(betas)
    assert sw.info().fast_path == 0 and sw.info().n_colours > 2
    ion = random_ising(lat, 5) if model == eg.MODEL_ISING else random_xyz(lat, 5)
    sw.set_spins(ion)
    sw.metropolis(sweeps, accept=False)
    ncol, col, rank = osys.colouring()
    for r in (0, 31, R - 1):
        work = ion.copy()
        sp4 = osys.spin4(work) if model == eg.MODEL_XYZ else None
        for t in range(sweeps):
            osys.metropolis_colour(work, sp4, 32 if sp4 is not None else 64, betas[r], 1992, r, t,
                                   col, rank, ncol)
        g = sw.get_spins(lat.ion, r)
        if model == eg.MODEL_XYZ:
            np.testing.assert_array_equal(g[:, 1:4].astype(np.float32), sp4[:, 0:3],
                                          err_msg="replica %d" % r)
        else:
            np.testing.assert_array_equal(g[:, 3], work[:, 3], err_msg="replica %d" % r)
    sw.close()


@pytest.mark.parametrize("model", [eg.MODEL_XYZ, eg.MODEL_ISING])
def test_structure_factor_at_27648_sites_error_against_fp64(model):
    """S(q) of the pyrochlore 16 x 12^3 lattice on the benchmark's 64^3 q-grid (q0 = -1,
    dq = 2/64 in reciprocal-lattice units), two replicas, 512 sampled q-points against the
    FP64 direct sum.  The measured errors are printed (ERROR line); the bounds are the small
    lattices' bounds."""
    lat = eg.pyrochlore(12)
    R = 2
    sw, _ = make_pair(lat, model, [[(1, 1, (1.0, 1.0, 1.0))]], replicas=R)
    spins = []
    for r in range(R):
        ion = random_ising(lat, 30 + r) if model == eg.MODEL_ISING else random_xyz(lat, 30 + r)
        sw.set_spins(ion, replica=r)
        g = sw.get_spins(lat.ion, r)
        spins.append(g[:, 1:4] if model == eg.MODEL_XYZ else
                     np.stack([0 * g[:, 3], 0 * g[:, 3], g[:, 3]], 1))
    M = 64
    abc = np.eye(3) * eg.model.PYROCHLORE_A
    nq, q0, dq = (M, M, M), (-1.0, -1.0, -1.0), (2.0 / M,) * 3
    sq, comp = _gpu_sq(sw, abc, nq, q0, dq)
    qidx = np.random.default_rng(0).choice(M ** 3, 512, replace=False)
    # the q-points with the largest values too: the sampled ones are mostly near 1/N
    qidx = np.unique(np.concatenate([qidx, np.argsort(sq[0])[-16:]]))
    ref_sq, ref_comp = _oracle_sq(lat, spins, abc, nq, q0, dq, qidx)
    dc = comp[:, qidx, :] - ref_comp
    ds = sq[:, qidx] - ref_sq
    print("ERROR S(q) %s N=%d R=%d q-points=%d: |S_a|/N max %.3e rms %.3e; |S|^2/N^2 max %.3e "
          "rms %.3e (largest value %.3e)" %
          ("Ising" if model == eg.MODEL_ISING else "Heisenberg", lat.N, R, len(qidx),
           np.abs(dc).max(), np.sqrt((dc ** 2).mean()), np.abs(ds).max(),
           np.sqrt((ds ** 2).mean()), ref_sq.max()))
    assert np.all(np.isfinite(sq)) and np.all(np.isfinite(comp))
    np.testing.assert_allclose(comp[:, qidx, :], ref_comp, atol=3e-4, rtol=0)
    np.testing.assert_allclose(sq[:, qidx], ref_sq, atol=1e-3 * max(ref_sq.max(), 1e-6), rtol=0)
    sw.close()
