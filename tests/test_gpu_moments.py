"""Per-species moment vectors and the spiral-state observable on the GPU against the oracle's
restatements of src/get_moment_vectors.f90 and src/get_spiral_state.f90."""
import numpy as np
import pytest

import ether_gb300 as eg
from oracle import pyoracle as po
from tests.helpers import random_ising, random_xyz

pytestmark = pytest.mark.gpu


def two_species_sc(n, checkerboard=True):
    """Rock-salt-like cell: species 1 at the origin, species 2 at the body centre of a cubic
    cell of edge 2 (nearest-neighbour distance sqrt(3))."""
    abc = np.eye(3) * 2.0
    cart = np.array([[0.0, 0.0, 0.0], [1.0, 1.0, 1.0]])
    return eg.model.Lattice(cart, [1, 2], abc, (n, n, n), [np.sqrt(3.0)], checkerboard=checkerboard)


def contexts(lat, model, s, R, seed):
    nsp = lat.n_species
    j = eg.couplings(nsp, [[(si, sj, (-1.0, -1.0, -1.0)) for si in range(1, nsp + 1)
                            for sj in range(1, nsp + 1)]], list(s))
    sw = eg.Sweep.from_lattice(lat, j, np.asarray(s, float), model, replicas=R, seed=seed)
    osys = po.System.from_lattice(lat, j, np.asarray(s, float), model)
    ions = []
    for r in range(R):
        ion = random_ising(lat, seed + r) if model == eg.MODEL_ISING else random_xyz(lat, seed + r)
        sw.set_spins(ion, r)
        ions.append(ion)
    return sw, osys, ions


@pytest.mark.parametrize("model", [eg.MODEL_ISING, eg.MODEL_XYZ])
@pytest.mark.parametrize("which", ["two_species", "pyrochlore", "sc"])
def test_moment_vectors_match_oracle(model, which):
    if which == "two_species":
        lat, s = two_species_sc(4), (1.0, 2.5)
    elif which == "pyrochlore":
        lat, s = eg.pyrochlore(2), (1.5,)
    else:
        lat, s = eg.simple_cubic(6, checkerboard=True), (1.0,)
    sw, osys, ions = contexts(lat, model, s, 3, 11)
    mm = sw.moment_vectors()
    assert mm.shape == (3, lat.n_species, 3)
    for r in range(3):
        g = sw.get_spins(lat.ion, r)
        ref = osys.moment_vectors(g)
        np.testing.assert_allclose(mm[r], ref, rtol=1e-12, atol=1e-9)
    # their sum is the total magnetisation
    np.testing.assert_allclose(mm.sum(axis=1), sw.tot_magnetisation(), rtol=1e-12, atol=1e-9)


@pytest.mark.parametrize("direc,lat_deg,dis", [((0, 0, 1), 60.0, 3.0), ((1, 1, 0), 50.0, 3.0),
                                               ((0, 0, 1), 2.0, 8.5)])
def test_spiral_state_matches_oracle(direc, lat_deg, dis):
    lat = eg.pyrochlore(2)
    sw, osys, ions = contexts(lat, eg.MODEL_XYZ, (1.0,), 4, 21)
    ifs, n = po.spiral_pairs(lat.ion, dis, direc, lat_deg, 12)
    assert n > 0
    count = sw.spiral_setup(dis, direc, lat_deg, 12)
    assert count == n
    ss = sw.spiral_state()
    for r in range(4):
        g = sw.get_spins(lat.ion, r)
        assert ss[r] == pytest.approx(po.spiral_state(g, ifs, n), rel=1e-9, abs=1e-12)


def test_spiral_after_sweeps_and_errors():
    lat = eg.simple_cubic(8)
    sw, osys, ions = contexts(lat, eg.MODEL_XYZ, (1.0,), 2, 5)
    sw.set_beta([1.0 / (1.0 * 1e-3)] * 2)
    sw.metropolis(5)
    ifs, n = po.spiral_pairs(lat.ion, 1.01, (0, 0, 1), 2.0, 5)
    assert sw.spiral_setup(1.01, (0, 0, 1), 2.0, 5) == n == lat.N * 7 // 8  # top plane: no partner
    ss = sw.spiral_state()
    for r in range(2):
        assert ss[r] == pytest.approx(po.spiral_state(sw.get_spins(lat.ion, r), ifs, n), rel=1e-9)
    with pytest.raises(eg.EtherError):
        sw.spiral_setup(3.5, (0, 0, 1), 90.0, 2)   # more partners than the capacity
    lat2 = eg.simple_cubic(4)
    sw2, _, _ = contexts(lat2, eg.MODEL_ISING, (1.0,), 1, 3)
    with pytest.raises(eg.EtherError):
        sw2.spiral_setup(1.01)
