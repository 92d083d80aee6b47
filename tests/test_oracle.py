"""Pins of the oracle (CPU, no GPU): known-answer vectors, exact enumeration, analytic
two-spin results, and its own internal consistency."""
import ctypes as C
import math
import os
import subprocess

import numpy as np
import pytest

import ether_gb300 as eg
from oracle import pyoracle as po
from tests.helpers import beta_of, random_xyz

# Random123 kat_vectors, philox4x32 with 10 rounds: (counter, key, result)
PHILOX_KAT = [
    ([0, 0, 0, 0], [0, 0], [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]),
    ([0xffffffff] * 4, [0xffffffff] * 2, [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]),
    ([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], [0xa4093822, 0x299f31d0],
     [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]),
]


@pytest.mark.parametrize("ctr,key,out", PHILOX_KAT)
def test_philox_known_answers(ctr, key, out):
    assert po.philox(ctr, key).tolist() == out


def test_philox_agrees_with_pytorch_header(tmp_path):
    """Second, independent implementation: ATen's PhiloxRNGEngine (header source)."""
    torch = pytest.importorskip("torch")
    inc = os.path.join(os.path.dirname(torch.__file__), "include")
    hdr = os.path.join(inc, "ATen", "core", "PhiloxRNGEngine.h")
    if not os.path.exists(hdr):
        pytest.skip("PhiloxRNGEngine.h not shipped")
    src = tmp_path / "p.cpp"
    src.write_text(
        '#include <ATen/core/PhiloxRNGEngine.h>\n#include <cstdio>\n'
        'int main(){ for (unsigned long long s : {0ULL, 1992ULL, 0xDEADBEEF12345678ULL}) {\n'
        ' at::Philox4_32 e(s, 7, 3); unsigned a = e(), b = e(), c = e(), d = e();\n'
        ' printf("%u %u %u %u\\n", a, b, c, d);}}\n')
    exe = tmp_path / "p"
    r = subprocess.run(["g++", "-std=c++17", "-I", inc, "-I", os.path.join(inc, "torch", "csrc", "api", "include"),
                        str(src), "-o", str(exe)], capture_output=True, text=True)
    if r.returncode != 0:
        pytest.skip("could not compile against the torch header: " + r.stderr[-200:])
    lines = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    for s, line in zip([0, 1992, 0xDEADBEEF12345678], lines):
        # at::Philox4_32(seed, subsequence, offset): key = seed (lo, hi), counter =
        # (offset lo, offset hi, subsequence lo, subsequence hi)
        want = [int(x) for x in line.split()]
        key = [s & 0xFFFFFFFF, s >> 32]
        ctr = [3, 0, 7, 0]
        assert po.philox(ctr, key).tolist() == want


def test_own_exp_and_sincos_accuracy():
    L = po.lib()
    xs = np.concatenate([np.linspace(-87.0, 0.0, 20001), -np.logspace(-8, 1.9, 2000)]).astype(np.float32)
    worst = 0.0
    for x in xs:
        y = L.orc_expf_neg(float(x))
        ref = math.exp(float(x))
        worst = max(worst, abs(y - ref) / ref)
    assert worst < 2.5e-7  # ~2 ulp
    s = C.c_float()
    c = C.c_float()
    for x in np.linspace(-np.pi, np.pi, 5001).astype(np.float32):
        L.orc_sincosf(float(x), C.byref(s), C.byref(c))
        assert abs(s.value - math.sin(float(x))) < 3e-7
        assert abs(c.value - math.cos(float(x))) < 3e-7


def _sc_system(L, model, J=-1.0, **kw):
    lat = eg.simple_cubic(L)
    j = eg.couplings(1, [[(1, 1, (J, J, J))]], [1.0])
    return lat, po.System.from_lattice(lat, j, np.array([1.0]), model, **kw)


def test_exact_enumeration_ising_2x2x2():
    """2x2x2 periodic SC: each site has one neighbour per axis in the reference's search
    (src/search_nbd.f90 captures a site once).  Exact <e>, C_v, <|m|> by enumerating all
    256 states vs a long typewriter Metropolis run of the oracle."""
    lat, osys = _sc_system(2, eg.MODEL_ISING)
    N = lat.N
    beta = beta_of(3.0)
    Es, Ms = [], []
    for state in range(1 << N):
        ion = lat.ion.copy()
        ion[:, 3] = [1.0 if (state >> i) & 1 else -1.0 for i in range(N)]
        Es.append(osys.tot_energy(ion))
        Ms.append(abs(ion[:, 3].sum()))
    Es, Ms = np.array(Es), np.array(Ms)
    w = np.exp(-beta * (Es / 2.0 - (Es / 2.0).min()))  # E_raw double counts bonds
    w /= w.sum()
    e = Es / (2 * N)
    m = Ms / N
    e_ex = (w * e).sum()
    cv_ex = beta ** 2 * ((w * e * e).sum() - e_ex ** 2) * N
    m_ex = (w * m).sum()
    st = po.stream(1992, 1)
    ion = lat.ion.copy()
    acc = po.Acc()
    for sweep in range(60000):
        osys.metropolis_typewriter(ion, beta, st)
        if sweep >= 2000:
            po.lib().orc_acc_sample(C.byref(acc), osys.tot_energy(ion),
                                    osys.tot_magnetisation(ion).ctypes.data_as(po.PD), N)
    out = np.zeros(6)
    po.lib().orc_acc_average(C.byref(acc), beta, N, out.ctypes.data_as(po.PD))
    assert out[0] == pytest.approx(e_ex, abs=3e-3 * abs(e_ex) + 2e-6)
    assert out[3] == pytest.approx(m_ex, rel=1e-2)
    assert out[2] == pytest.approx(cv_ex, rel=5e-2)


def test_heisenberg_dimer_langevin():
    """Two XYZ spins coupled by J: <cos theta> = L(-beta J), the Langevin function."""
    lat = eg.Lattice([[0, 0, 0], [1.0, 0, 0]], [1, 1], np.eye(3) * 10.0, (1, 1, 1), [1.0],
                     bc="ooo")
    j = eg.couplings(1, [[(1, 1, (-1.0, -1.0, -1.0))]], [1.0])
    osys = po.System.from_lattice(lat, j, np.array([1.0]), eg.MODEL_XYZ)
    beta = beta_of(0.7)
    x = beta * 1e-3
    langevin = 1.0 / math.tanh(x) - 1.0 / x
    st = po.stream(5, 5)
    ion = lat.ion.copy()
    ion[:, 1:4] = [[0, 0, 1], [0, 0, 1]]
    cs = []
    for sweep in range(200000):
        osys.metropolis_typewriter(ion, beta, st)
        if sweep > 1000:
            cs.append(float(np.dot(ion[0, 1:4], ion[1, 1:4])))
    assert np.mean(cs) == pytest.approx(langevin, abs=5e-3)


def test_colour_mode_fp32_mirror_tracks_fp64():
    lat, osys = _sc_system(8, eg.MODEL_XYZ)
    ncol, col, rank = osys.colouring()
    assert ncol == 2
    ion = random_xyz(lat, 4)
    sp4 = osys.spin4(ion)
    ion64 = ion.copy()
    beta = beta_of(1.443)
    for t in range(40):
        a32 = osys.metropolis_colour(ion, sp4, 32, beta, 1, 2, t, col, rank, ncol)
        a64 = osys.metropolis_colour(ion64, None, 64, beta, 1, 2, t, col, rank, ncol)
        assert a32 == a64
    assert abs(osys.tot_energy_f32(ion, sp4) - osys.tot_energy(ion64)) < 1e-6 * abs(osys.tot_energy(ion64))


def test_greedy_colouring_is_proper_and_parity_on_even_sc():
    for L in (4, 5, 6):
        lat, osys = _sc_system(L, eg.MODEL_ISING)
        n, col, rank = osys.colouring()
        nn = lat.nn
        for i in range(lat.N):
            for k in range(1, nn[0, 0, i, 0] + 1):
                assert col[i] != col[nn[1, k, i, 0] - 1]
        if L % 2 == 0:
            x = np.arange(lat.N) % L
            y = (np.arange(lat.N) // L) % L
            z = np.arange(lat.N) // (L * L)
            np.testing.assert_array_equal(col, (x + y + z) % 2)


def test_parallel_tempering_rule():
    beta = np.array([1.0, 2.0, 3.0, 4.0])
    E = np.array([-1.0, -5.0, -2.0, -10.0])
    ros = np.arange(4, dtype=np.int32)
    n = po.lib().orc_parallel_tempering(4, beta.ctypes.data_as(po.PD), E.ctypes.data_as(po.PD),
                                        ros.ctypes.data_as(po.PI), 2, 7, 0, 0, None)
    # pairs (0,1): delta = -(2-1)*(-1+5) = -4; (2,3): delta = -(4-3)*(-2+10) = -8
    u = []
    for s in (0, 2):
        o = po.philox([s, 2, 0x50540000, 3], [7, 0x45544852])
        u.append(o[0] * 2.0 ** -32)
    want = [u[0] < math.exp(-4.0), u[1] < math.exp(-8.0)]
    assert n == sum(want)


def test_per_repeat_matches_formula():
    vals = np.random.default_rng(0).normal(size=(5, 6))
    mean = np.zeros(6)
    err = np.zeros(6)
    po.lib().orc_per_repeat(5, np.ascontiguousarray(vals).ctypes.data_as(po.PD),
                            mean.ctypes.data_as(po.PD), err.ctypes.data_as(po.PD))
    np.testing.assert_allclose(mean, vals.mean(0))
    np.testing.assert_allclose(err, vals.std(0, ddof=1) / math.sqrt(5))


@pytest.mark.parametrize("L", [3, 4, (5, 3, 4), (3, 6, 5)])
def test_closed_form_simple_cubic_equals_bruteforce_getting_nbd(L):
    """The oracle's own simple-cubic builder (used by the CPU baseline, which must not load the
    product library) gives the same ion and nn arrays as the brute-force restatement of
    getting_nbd / search_nbd."""
    lat = po.ScLattice(L)
    sc = np.array([L] * 3 if np.isscalar(L) else L, dtype=np.int32)
    N = int(np.prod(sc))
    ion = np.zeros((N, 9))
    po.lib().orc_supercell(1, po._d(np.zeros(3)), po._i(np.ones(1, dtype=np.int32)),
                           po._d(np.eye(3)), po._i(sc), 0, po._d(ion), None)
    nn = np.zeros((2, 21, N, 1), dtype=np.int32)
    rc = po.lib().orc_neighbours_bruteforce(N, po._d(ion), po._d(np.eye(3)), po._i(sc), b"ccc", 1,
                                            po._d(np.array([1.0])), 1e-5, 20, po._i(nn))
    assert rc == 0
    np.testing.assert_array_equal(lat.ion, ion)
    np.testing.assert_array_equal(lat.nn, nn)


def test_timed_build_computes_the_same_energies():
    """The CPU baseline's build (the reference's optimisation flags) and the checker build
    agree on get_tot_energy to rounding."""
    lat = po.ScLattice(6)
    j = po.sc_couplings((-1.0, -1.0, -1.0))
    for model in (0, 1):
        osys = po.System.from_lattice(lat, j, np.array([1.0]), model)
        rng = np.random.default_rng(model)
        ion = lat.ion.copy()
        v = rng.normal(size=(lat.N, 3))
        ion[:, 1:4] = v / np.linalg.norm(v, axis=1, keepdims=True) if model else 0.0
        if not model:
            ion[:, 3] = rng.choice([-1.0, 1.0], size=lat.N)
        a = po.lib().orc_tot_energy(osys.p(), po._d(ion))
        b = po.timed_lib().orc_tot_energy(osys.p(), po._d(ion))
        assert b == pytest.approx(a, rel=1e-12)


def test_oracle_local_axis_anisotropy_energy():
    """The oracle's local-axis anisotropy: with the exchange switched off, get_tot_energy of
    spins along their own axes is N D, and a trial move's Hamiltonian(.TRUE.) equals the
    difference of the two site energies."""
    lat = po.ScLattice(4)
    rng = np.random.default_rng(3)
    ax = rng.normal(size=(lat.N, 3))
    ax /= np.linalg.norm(ax, axis=1, keepdims=True)
    D = -0.2e-3
    sl = np.concatenate([ax, np.full((lat.N, 1), D)], axis=1)
    osys = po.System.from_lattice(lat, po.sc_couplings((0.0, 0.0, 0.0)), np.array([1.0]), 1, sia_local=sl)
    ion = lat.ion.copy()
    ion[:, 1:4] = ax
    assert osys.tot_energy(ion) == pytest.approx(lat.N * D, rel=1e-12)
    i = 5
    new = rng.normal(size=3)
    new /= np.linalg.norm(new)
    old = ion[i, 1:4].copy()
    dE = po.lib().orc_hamiltonian(osys.p(), po._d(ion), i, po._d(new), po._d(old), 1)
    assert dE == pytest.approx(D * ((ax[i] @ new) ** 2 - (ax[i] @ old) ** 2), rel=1e-12)
