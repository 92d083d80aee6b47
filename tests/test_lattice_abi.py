"""CPU checks of the product's host side: the O(N) lattice builder against the oracle's
brute-force restatement of getting_nbd, and the C-ABI's exported surface."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import ether_gb300 as eg
from ether_gb300 import abi
from oracle import pyoracle as po

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _check(basis, species, abc, sc, bc, shells, tol, cap=20, checkerboard=False):
    lat = eg.Lattice(basis, species, abc, sc, shells, bc=bc, tol=tol, cap=cap,
                     checkerboard=checkerboard)
    ion, stgg = po.supercell(basis, species, abc, sc, checkerboard=checkerboard)
    rc, nn = po.neighbours_bruteforce(ion, abc, sc, bc, shells, tol, cap)
    assert rc == 0
    np.testing.assert_array_equal(lat.ion, ion)
    np.testing.assert_array_equal(lat.stgg, stgg)
    np.testing.assert_array_equal(lat.nn, nn)
    return lat


@pytest.mark.parametrize("sc,bc", [((2, 2, 2), "ccc"), ((3, 3, 3), "ccc"), ((4, 4, 4), "ccc"),
                                   ((5, 4, 3), "coc"), ((3, 2, 5), "ooo"), ((1, 4, 4), "ccc")])
def test_simple_cubic_neighbours_match_bruteforce(sc, bc):
    _check([[0, 0, 0]], [1], np.eye(3), sc, bc, [1.0], 1e-5, checkerboard=True)


def test_simple_cubic_two_shells():
    _check([[0, 0, 0]], [1], np.eye(3), (4, 4, 4), "ccc", [1.0, np.sqrt(2.0)], 1e-5)


def test_pyrochlore_two_shells_match_bruteforce():
    abc = np.eye(3) * eg.model.PYROCHLORE_A
    cart = [[abc[0, d] * f[0] + abc[1, d] * f[1] + abc[2, d] * f[2] for d in range(3)]
            for f in eg.model.PYROCHLORE_FRAC]
    lat = _check(cart, [1] * 16, abc, (2, 2, 2), "ccc", [2.97243, 5.1484], 1e-3)
    assert (lat.nn[0, 0, :, 0] == 6).all() and (lat.nn[0, 0, :, 1] == 12).all()


def test_triangular_two_species_match_bruteforce():
    abc = np.array([[1.0, 0, 0], [0.5, np.sqrt(3) / 2, 0], [0, 0, 1.2]])
    _check([[0, 0, 0], [0.5, np.sqrt(3) / 6, 0.6]], [1, 2], abc, (3, 3, 3), "ccc",
           [1.0, 1.2], 1e-5)


def test_neighbour_capacity_overflow_is_an_error():
    with pytest.raises(eg.EtherError) as e:
        eg.Lattice([[0, 0, 0]], [1], np.eye(3), (4, 4, 4), [1.0], cap=4)
    assert e.value.code == -5


def test_large_lattice_build_is_linear():
    lat = eg.simple_cubic(32)
    assert (lat.nn[0, 0, :, 0] == 6).all()


def test_library_exports_every_declared_symbol():
    hdr = open(os.path.join(ROOT, "include", "ether_gpu.h")).read()
    declared = set(re.findall(r"\b(ether_[a-z_0-9]+)\s*\(", hdr))
    lib = abi.load()
    for name in declared:
        assert hasattr(lib, name), name
    assert declared == set(abi.SIGNATURES), declared ^ set(abi.SIGNATURES)
    assert lib.ether_abi_version() == 2


def test_create_without_gpu_or_bad_input_fails_cleanly():
    lib = abi.load()
    h = C.c_void_p()
    d = abi.Desc()
    d.n_sites = 0
    rc = lib.ether_create(C.byref(d), C.byref(h))
    assert rc == -1 and not h.value
    assert b"non-positive" in lib.ether_last_error()
