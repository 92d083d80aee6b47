"""The Monte Carlo path against exact solutions.

Ising: the nearest-neighbour ferromagnet on a finite square torus, whose partition function
is Kaufman's closed form (tests/exact2d.py).

CPU: the closed form equals the enumeration of all 2^(mn) states of small tori.
GPU: a 16 x 16 torus (one site per cell, the third axis 8 lattice constants long, so each site
has its four in-plane neighbours and nothing else; the general-lattice kernels) sampled by
ether_mcs at kT = 2.0, 2.269 (near the infinite lattice's T_c) and 3.0 J, 64 independent
chains per temperature, 20 000 measurements each after 2 000 equilibration steps.  The energy
per site (src/get_eng.f90:36-40, E / 2N) and the heat capacity per site from its fluctuations
agree with the exact values: each of the 6 differences, over the spread of the 64 chains'
estimates, passes a two-sided z-test at 0.01 / 6 (Bonferroni, a family-wise 1%).  The same
holds on a ladder of kT = 2.0, 2.1, 2.269 and 2.5 J with parallel tempering when the swap
exponent uses the Hamiltonian energy; the reference's raw-sum exponent (every bond counted
twice) measurably biases the coldest slot.

Heisenberg (XYZ): the classical ferromagnetic ring of 64 unit spins (the other two axes 8
lattice constants long: two neighbours per site).  Its transfer matrix gives the energy per
site -J L(K) and the heat capacity per site 1 - K^2 / sinh^2 K (L the Langevin function,
K = J / kT; M. E. Fisher, Am. J. Phys. 32, 343 (1964)), up to terms of relative order
L(K)^64 (below 1e-17 here).  ether_mcs with Marsaglia proposals and an overrelaxation pass
every step (src/ether.f90:163-172) at kT = 0.5, 1 and 2 J, the same rule as above.

Ising in a field: the ring of 64 spins in a Zeeman field, against its transfer matrix (the
reported energy per site and its variance).

Independent Heisenberg spins in a single-ion anisotropy and a Zeeman field (no exchange): the
averages are integrals over cos theta; the simple-cubic fast kernels with Marsaglia proposals,
the general-lattice kernels with ANGLE proposals, and anisotropy about per-site local axes.
"""
import numpy as np
import pytest

import ether_gb300 as eg
from tests.helpers import beta_of, make_pair, random_ising, random_xyz

FM = [[(1, 1, (-1.0, -1.0, -1.0))]]   # ETHER's sign: J < 0 is ferromagnetic, |J| = 1 meV

# kT / J -> (energy per site / J, heat capacity per site / k_B) of the 16 x 16 torus, from the
# closed form (test_exact_values_are_the_closed_forms checks them; the GPU test needs no mpmath)
EXACT_16 = {2.0: (-1.7455306689909191, 0.7255087677365641),
            2.1: (-1.662024277054132, 0.9601262642539019),
            2.269: (-1.4533425476693835, 1.4983111034990866),
            2.5: (-1.131317984410729, 1.0649768828534356),
            3.0: (-0.8176893678695545, 0.4043325741653013)}


def _exact2d():
    pytest.importorskip("mpmath")
    from tests import exact2d
    return exact2d


@pytest.mark.parametrize("m,n", [(4, 4), (2, 4), (3, 4), (4, 5)])
def test_closed_form_equals_enumeration(m, n):
    exact2d = _exact2d()
    for K in (0.2, 0.4406867935, 0.6, 1.0):
        assert abs(float(exact2d.ln_z(K, m, n) - exact2d.brute_force_ln_z(K, m, n))) < 1e-40


def test_closed_form_approaches_onsager_at_tc():
    """At K_c = ln(1 + sqrt 2) / 2: the energy per site of the L x L torus approaches the
    infinite lattice's -sqrt(2) J as 1/L, and the heat capacity per site grows by Onsager's
    (8 / pi) K_c^2 ln 2 each time L doubles (its logarithmic divergence)."""
    exact2d = _exact2d()
    Kc = float(np.log(1 + np.sqrt(2)) / 2)
    res = {L: exact2d.energy_cv(Kc, L, L) for L in (16, 32, 64, 128)}
    slope = [(res[L][0] + np.sqrt(2)) * L for L in (16, 32, 64, 128)]
    assert max(slope) - min(slope) < 0.01 * abs(slope[-1])
    step = 8 / np.pi * Kc * Kc * np.log(2)
    for L in (16, 32, 64):
        assert abs(res[2 * L][1] - res[L][1] - step) < 0.02 * step


def test_exact_values_are_the_closed_forms():
    exact2d = _exact2d()
    for t, (e, cv) in EXACT_16.items():
        assert np.allclose(exact2d.energy_cv(1.0 / t, 16, 16), (e, cv), rtol=1e-14, atol=0)


def _square_torus(L):
    return eg.Lattice([[0.0, 0.0, 0.0]], [1], np.diag([1.0, 1.0, 8.0]), (L, L, 1), [1.0])


def _torus_run(pt, flags=0):
    """Per (chain, temperature) energy and heat capacity per site, and the exact values."""
    L, G = 16, 64
    temps = (2.0, 2.1, 2.269, 2.5) if pt else (2.0, 2.269, 3.0)
    lat = _square_torus(L)
    sw, _ = make_pair(lat, eg.MODEL_ISING, FM, replicas=G * len(temps), flags=flags)
    info = sw.info()
    assert info.fast_path == 0 and info.n_colours == 2
    sw.set_ladder([beta_of(t) for t in temps])
    # every site has its four in-plane neighbours: the all-up state has E / 2N = -2 J
    up = lat.ion.copy()
    up[:, 3] = 1.0
    sw.set_spins(up)
    assert np.allclose(np.asarray(sw.tot_energy()) / (2 * lat.N), -2e-3)
    sw.set_streams(stream=list(range(sw.R)), step=[0] * sw.R)
    sw.set_spins(random_ising(lat, 11))
    sw.zero_avg()
    # PT runs on steps that are multiples of 5 but not measurement steps (src/ether.f90:190-191):
    # with PT a measurement every second step, so the swaps come every 10
    eq, meas, coa = 2000, 20000, 2 if pt else 1
    swaps = sw.mcs(0, eq + meas, eq, coa, pt=pt, exchange_interval=5)
    if pt:
        assert swaps > 0
        if not flags & eg.FLAG_PT_REFERENCE_COPY:  # a true swap exchanges slots
            assert not np.array_equal(sw.slots(), np.arange(sw.R) % len(temps))
    sums = sw.sums().reshape(G, len(temps), 7)
    sw.close()
    out = []
    for k, t in enumerate(temps):
        K = 1.0 / t
        cnt = sums[:, k, 0]
        assert np.all(cnt == meas // coa)
        e = sums[:, k, 1] / cnt / 1e-3            # per chain, units of J
        e2 = sums[:, k, 2] / cnt / 1e-6
        cv = lat.N * K * K * (e2 - e * e)         # per chain
        e_ex, cv_ex = EXACT_16[t]
        for name, x, ref in (("E/N", e, e_ex), ("C/N", cv, cv_ex)):
            z = (x.mean() - ref) / (x.std(ddof=1) / np.sqrt(G))
            print("kT=%.3f %s: GPU %.5f +- %.5f, exact %.5f, z = %.2f" %
                  (t, name, x.mean(), x.std(ddof=1) / np.sqrt(G), ref, z))
            out.append((t, name, x.mean(), ref, z))
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("pt", ["off", "swap", "copy"])
def test_mcs_energy_and_heat_capacity_equal_the_exact_torus(pt):
    """pt: each chain is a ladder of kT = 2.0, 2.1, 2.269 and 2.5 J with parallel-tempering
    steps every 10 steps (src/parallel_tempering.f90:39-108) whose exponent uses the
    Hamiltonian energy (ETHER_FLAG_PT_TRUE_ENERGY), which leaves every temperature's ensemble
    exact; the statistics are per (chain, temperature slot).  "copy": on acceptance only the
    colder slot takes the hotter one's configuration (the reference's effective copy,
    ETHER_FLAG_PT_REFERENCE_COPY) -- for the colder slot a Metropolis-Hastings move with the
    hotter slot's configuration as the proposal, so each slot's ensemble is still exact."""
    from scipy.special import erfcinv
    flags = {"off": 0, "swap": eg.FLAG_PT_TRUE_ENERGY,
             "copy": eg.FLAG_PT_TRUE_ENERGY | eg.FLAG_PT_REFERENCE_COPY}[pt]
    res = _torus_run(pt != "off", flags=flags)
    zmax = float(np.sqrt(2) * erfcinv(0.01 / len(res)))   # two-sided 0.01 / 6 (or / 8): |z| < 3.14 (3.23)
    for t, name, got, ref, z in res:
        assert abs(z) < zmax, (t, name, got, ref, z)


@pytest.mark.gpu
def test_reference_pt_exponent_biases_the_cold_end():
    """The reference's PT exponent takes get_tot_energy's raw sum, which counts every bond
    twice (src/ether.f90:177, src/get_tot_energy.f90:33-47): the swap acceptance is
    exp(2 dbeta dH) instead of exp(dbeta dH), which breaks detailed balance.  The default mode
    reproduces it, and on the same ladder the coldest slot's energy is measurably below the
    exact value (the chains are seeded, so the figure is reproducible).  It is this exponent,
    not the reference's copy in place of a swap, that biases its ladders: the copy with the
    Hamiltonian exponent is exact (above)."""
    res = _torus_run(True)
    t, name, got, ref, z = res[0]
    assert (t, name) == (2.0, "E/N")
    assert z < -5.0, res[0]


@pytest.mark.gpu
def test_mcs_heisenberg_ring_equals_the_exact_chain():
    N, G = 64, 64
    temps = (0.5, 1.0, 2.0)
    lat = eg.Lattice([[0.0, 0.0, 0.0]], [1], np.diag([1.0, 8.0, 8.0]), (N, 1, 1), [1.0])
    sw, _ = make_pair(lat, eg.MODEL_XYZ, FM, replicas=G * len(temps))
    info = sw.info()
    assert info.fast_path == 0 and info.n_colours == 2
    sw.set_ladder([beta_of(t) for t in temps])
    # two neighbours per site: the aligned state has E / 2N = -J
    al = lat.ion.copy()
    al[:, 1:4] = (0.0, 0.0, 1.0)
    sw.set_spins(al)
    assert np.allclose(np.asarray(sw.tot_energy()) / (2 * N), -1e-3)
    sw.set_streams(stream=list(range(sw.R)), step=[0] * sw.R)
    sw.set_spins(random_xyz(lat, 12))
    sw.zero_avg()
    eq, meas = 2000, 40000
    sw.mcs(0, eq + meas, eq, 1, ovrr=True, ovrr_para=1.0, ovrr_mcs=1)
    sums = sw.sums().reshape(G, len(temps), 7)
    from scipy.special import erfcinv
    zmax = float(np.sqrt(2) * erfcinv(0.01 / (2 * len(temps))))
    for k, t in enumerate(temps):
        K = 1.0 / t
        cnt = sums[:, k, 0]
        assert np.all(cnt == meas)
        e = sums[:, k, 1] / cnt / 1e-3
        e2 = sums[:, k, 2] / cnt / 1e-6
        cv = N * K * K * (e2 - e * e)
        e_ex = -(1.0 / np.tanh(K) - 1.0 / K)
        cv_ex = 1.0 - (K / np.sinh(K)) ** 2
        for name, x, ref in (("E/N", e, e_ex), ("C/N", cv, cv_ex)):
            z = (x.mean() - ref) / (x.std(ddof=1) / np.sqrt(G))
            print("Heisenberg ring kT=%.2f %s: GPU %.5f +- %.5f, exact %.5f, z = %.2f" %
                  (t, name, x.mean(), x.std(ddof=1) / np.sqrt(G), ref, z))
            assert abs(z) < zmax, (t, name, x.mean(), ref, z)
    sw.close()


def _chain_f(K, h):
    """ln of the larger transfer-matrix eigenvalue of the Ising chain, weights
    exp(K s s' + h s): the free energy per site of a long ring, in units of -kT."""
    return np.log(np.exp(K) * np.cosh(h) + np.sqrt(np.exp(2 * K) * np.sinh(h) ** 2 + np.exp(-2 * K)))


def _chain_derivs(K, h, d=1e-4):
    """f_K, f_h, f_KK, f_hh, f_Kh by central differences (step 1e-4: errors ~1e-8)."""
    f = _chain_f
    fK = (f(K + d, h) - f(K - d, h)) / (2 * d)
    fh = (f(K, h + d) - f(K, h - d)) / (2 * d)
    fKK = (f(K + d, h) - 2 * f(K, h) + f(K - d, h)) / d ** 2
    fhh = (f(K, h + d) - 2 * f(K, h) + f(K, h - d)) / d ** 2
    fKh = (f(K + d, h + d) - f(K + d, h - d) - f(K - d, h + d) + f(K - d, h - d)) / (4 * d * d)
    return fK, fh, fKK, fhh, fKh


def test_chain_transfer_matrix_equals_enumeration():
    """The eigenvalue formula against the enumeration of a 14-site ring (K = 0.7, h = 0.3):
    <s s'> and <s> per site agree to the ring's (lambda_- / lambda_+)^14 correction."""
    n, K, h = 14, 0.7, 0.3
    s = 1 - 2 * ((np.arange(1 << n)[:, None] >> np.arange(n)) & 1)
    ss = (s * np.roll(s, 1, axis=1)).sum(axis=1)
    m = s.sum(axis=1)
    w = np.exp(K * ss + h * m)
    w /= w.sum()
    fK, fh, *_ = _chain_derivs(K, h)
    assert abs((w * ss).sum() / n - fK) < 1e-3
    assert abs((w * m).sum() / n - fh) < 1e-3


@pytest.mark.gpu
def test_mcs_ising_ring_in_a_field_equals_the_transfer_matrix():
    """A ring of 64 Ising spins (the general-lattice kernels) with exchange |J| = 1 meV and a
    Zeeman field H = 2 T along z (g = 2, s = 1: h = g mu_B H per spin).  The reported energy
    per site is E_raw / 2N = -|J| <s s'> - (h / 2) <s> (the half Zeeman term of
    src/get_eng.f90:36), and N Var(e) = |J|^2 f_KK + (h / 2)^2 f_hh + |J| h f_Kh, both from
    the transfer matrix's eigenvalue (ring corrections below 1e-12).  kT = 0.5, 1 and 2 meV;
    64 chains each; the same family-wise rule."""
    N, G, Hz = 64, 64, 2.0
    temps = (0.5, 1.0, 2.0)
    lat = eg.Lattice([[0.0, 0.0, 0.0]], [1], np.diag([1.0, 8.0, 8.0]), (N, 1, 1), [1.0])
    sw, _ = make_pair(lat, eg.MODEL_ISING, FM, replicas=G * len(temps), zeeman=True,
                      h=(0.0, 0.0, Hz), g_factor=2.0)
    assert sw.info().fast_path == 0 and sw.info().n_colours == 2
    sw.set_ladder([beta_of(t) for t in temps])
    h_mev = 2.0 * eg.MB_EV * Hz * 1e3
    up = lat.ion.copy()
    up[:, 3] = 1.0
    sw.set_spins(up)
    e_up = np.asarray(sw.tot_energy())[0] / (2 * N) / 1e-3
    up[:, 3] = -1.0
    sw.set_spins(up)
    e_dn = np.asarray(sw.tot_energy())[0] / (2 * N) / 1e-3
    # the field lowers an up spin's energy by h; the reported energy carries half of it
    assert np.isclose(e_up, -1.0 - h_mev / 2) and np.isclose(e_dn, -1.0 + h_mev / 2)
    sw.set_streams(stream=list(range(sw.R)), step=[0] * sw.R)
    sw.set_spins(random_ising(lat, 13))
    sw.zero_avg()
    eq, meas = 2000, 40000
    sw.mcs(0, eq + meas, eq, 1)
    sums = sw.sums().reshape(G, len(temps), 7)
    from scipy.special import erfcinv
    zmax = float(np.sqrt(2) * erfcinv(0.01 / (2 * len(temps))))
    for k, t in enumerate(temps):
        K, hb = 1.0 / t, h_mev / t
        fK, fh, fKK, fhh, fKh = _chain_derivs(K, hb)
        e_ex = -fK - (h_mev / 2) * fh
        var_ex = fKK + (h_mev / 2) ** 2 * fhh + h_mev * fKh     # N Var(e), meV^2
        cnt = sums[:, k, 0]
        assert np.all(cnt == meas)
        e = sums[:, k, 1] / cnt / 1e-3
        var = N * (sums[:, k, 2] / cnt / 1e-6 - e * e)
        for name, x, ref in (("E/N", e, e_ex), ("N Var(E/N)", var, var_ex)):
            z = (x.mean() - ref) / (x.std(ddof=1) / np.sqrt(G))
            print("Ising ring in H=%.0f T, kT=%.2f %s: GPU %.5f +- %.5f, exact %.5f, z = %.2f" %
                  (Hz, t, name, x.mean(), x.std(ddof=1) / np.sqrt(G), ref, z))
            assert abs(z) < zmax, (t, name, x.mean(), ref, z)
    sw.close()


def _single_spin_moments(A, B, kT):
    """<u>, <u^2>, <u^3>, <u^4> of u = cos(theta) over the sphere with weight
    exp(-(A u^2 + B u) / kT) (Simpson's rule on 200 001 points)."""
    u = np.linspace(-1.0, 1.0, 200001)
    w = np.exp(-(A * u * u + B * u - min(A + B, A - B, 0.0)) / kT)
    h = u[1] - u[0]
    c = np.ones_like(u)
    c[1:-1:2], c[2:-1:2] = 4.0, 2.0
    z = (c * w).sum()
    return [float((c * w * u ** k).sum() / z) for k in (1, 2, 3, 4)]


@pytest.mark.gpu
@pytest.mark.parametrize("form", ["sc_marsaglia", "general_angle", "local_axes"])
def test_mcs_independent_spins_with_anisotropy_and_field_equal_the_integral(form):
    """No exchange: each Heisenberg spin is alone in its single-ion anisotropy D and Zeeman
    field, E(u) = A u^2 + B u with u the spin's component along the axis (cos theta), and the
    thermal averages are one-dimensional integrals over the sphere.  The reported energy per
    site is half of it (src/get_eng.f90:36: SIA and Zeeman enter E_raw once), and
    N Var(e) = Var(E(u)) / 4.  A and B are read off the library itself (the energies of the
    all-up and all-down states) and checked against D and g mu_B H.
    sc_marsaglia: 8^3 simple cubic (the fast kernels), easy axis D = -0.3 meV along z, H = 1 T
    along z, Marsaglia proposals.  general_angle: the same on the general-lattice kernels with
    ANGLE proposals (dphi = 0.6).  local_axes: easy plane D = +0.4 meV about a random unit axis
    (16 axes over the sites, ether_desc.sia_local), no field: the same integral for every
    site."""
    L, G = 8, 32
    temps = (0.1, 0.4)   # kT in meV
    lat = eg.simple_cubic(L)
    zero = [[(1, 1, (0.0, 0.0, 0.0))]]
    kw = {}
    if form == "local_axes":
        rng = np.random.default_rng(5)
        ax = rng.normal(size=(16, 3))    # 16 axes (at most 256 distinct classes per context)
        ax /= np.linalg.norm(ax, axis=1, keepdims=True)
        ax = ax[rng.integers(0, 16, size=lat.N)]
        kw = dict(sia_local=np.concatenate([ax, np.full((lat.N, 1), 0.4e-3)], axis=1))
        D, Hz = 0.4, 0.0
    else:
        D, Hz = -0.3, 1.0
        kw = dict(sia=True, sia_vec=np.array([[0.0, 0.0, D * 1e-3]]), zeeman=True, h=(0.0, 0.0, Hz),
                  g_factor=2.0)
        if form == "general_angle":
            kw.update(angle=True, dphi=0.6)
    flags = eg.FLAG_FORCE_GENERAL if form == "general_angle" else 0
    seed = {"sc_marsaglia": 1992, "general_angle": 2024, "local_axes": 77}[form]  # independent draws
    sw, _ = make_pair(lat, eg.MODEL_XYZ, zero, replicas=G * len(temps), flags=flags, seed=seed, **kw)
    assert sw.info().fast_path == (0 if form == "general_angle" else 1)
    sw.set_ladder([1.0 / (t * 1e-3) for t in temps])
    # E(u) = A u^2 + B u: the all-up and all-down states (along z, or along each site's axis)
    st = lat.ion.copy()
    st[:, 1:4] = kw["sia_local"][:, :3] if form == "local_axes" else (0.0, 0.0, 1.0)
    sw.set_spins(st)
    e_up = float(np.asarray(sw.tot_energy())[0]) / (2 * lat.N) / 1e-3
    st[:, 1:4] *= -1.0
    sw.set_spins(st)
    e_dn = float(np.asarray(sw.tot_energy())[0]) / (2 * lat.N) / 1e-3
    A, B = e_up + e_dn, e_up - e_dn     # twice the reported halves
    assert np.isclose(A, D, rtol=1e-6)
    assert np.isclose(B, -2.0 * eg.MB_EV * Hz * 1e3, rtol=1e-6, atol=1e-9)
    sw.set_streams(stream=list(range(sw.R)), step=[0] * sw.R)
    sw.set_spins(random_xyz(lat, 17))
    sw.zero_avg()
    # ANGLE moves cross the 3 kT barrier between the field-split wells slowly: a long start
    eq, meas = 5000, 10000
    sw.mcs(0, eq + meas, eq, 1)
    sums = sw.sums().reshape(G, len(temps), 7)
    from scipy.special import erfcinv
    zmax = float(np.sqrt(2) * erfcinv(0.01 / (2 * len(temps))))
    for k, t in enumerate(temps):
        m1, m2, m3, m4 = _single_spin_moments(A, B, t)
        mean_E = A * m2 + B * m1
        var_E = A * A * m4 + 2 * A * B * m3 + B * B * m2 - mean_E ** 2
        e_ex, var_ex = mean_E / 2, var_E / 4
        cnt = sums[:, k, 0]
        assert np.all(cnt == meas)
        e = sums[:, k, 1] / cnt / 1e-3
        var = lat.N * (sums[:, k, 2] / cnt / 1e-6 - e * e)
        for name, x, ref in (("E/N", e, e_ex), ("N Var(E/N)", var, var_ex)):
            z = (x.mean() - ref) / (x.std(ddof=1) / np.sqrt(G))
            print("%s kT=%.2f meV %s: GPU %.6f +- %.6f, exact %.6f, z = %.2f" %
                  (form, t, name, x.mean(), x.std(ddof=1) / np.sqrt(G), ref, z))
            assert abs(z) < zmax, (form, t, name, x.mean(), ref, z)
    sw.close()


@pytest.mark.gpu
def test_mcs_independent_ising_spins_in_a_field_equal_tanh():
    """No exchange: each Ising spin of a 32^3 simple-cubic lattice (the fast kernels with
    16-byte vectors, as the benchmark runs them) is alone in a Zeeman field, E(s) = B s with
    B = -g mu_B H, so <s> = -tanh(B / kT) and the reported energy per site (half the Zeeman
    term) is B <s> / 2 with N Var(e) = (B / 2)^2 (1 - <s>^2).  H = 2 T, kT = 0.1 and 0.3 meV,
    16 chains each; the same family-wise rule."""
    L, G, Hz = 32, 16, 2.0
    temps = (0.1, 0.3)
    lat = eg.simple_cubic(L)
    sw, _ = make_pair(lat, eg.MODEL_ISING, [[(1, 1, (0.0, 0.0, 0.0))]], replicas=G * len(temps),
                      zeeman=True, h=(0.0, 0.0, Hz), g_factor=2.0, seed=31)
    assert sw.info().fast_path == 1
    sw.set_ladder([1.0 / (t * 1e-3) for t in temps])
    B = -2.0 * eg.MB_EV * Hz * 1e3
    st = lat.ion.copy()
    st[:, 3] = 1.0
    sw.set_spins(st)
    assert np.isclose(float(np.asarray(sw.tot_energy())[0]) / (2 * lat.N) / 1e-3, B / 2, rtol=1e-9)
    sw.set_streams(stream=list(range(sw.R)), step=[0] * sw.R)
    sw.set_spins(random_ising(lat, 19))
    sw.zero_avg()
    eq, meas = 200, 2000
    sw.mcs(0, eq + meas, eq, 1)
    sums = sw.sums().reshape(G, len(temps), 7)
    from scipy.special import erfcinv
    zmax = float(np.sqrt(2) * erfcinv(0.01 / (2 * len(temps))))
    for k, t in enumerate(temps):
        s_mean = -np.tanh(B / t)
        e_ex, var_ex = B * s_mean / 2, (B / 2) ** 2 * (1 - s_mean ** 2)
        cnt = sums[:, k, 0]
        assert np.all(cnt == meas)
        e = sums[:, k, 1] / cnt / 1e-3
        var = lat.N * (sums[:, k, 2] / cnt / 1e-6 - e * e)
        for name, x, ref in (("E/N", e, e_ex), ("N Var(E/N)", var, var_ex)):
            z = (x.mean() - ref) / (x.std(ddof=1) / np.sqrt(G))
            print("Ising spins in H=%.0f T, kT=%.2f meV %s: GPU %.7f +- %.7f, exact %.7f, z = %.2f" %
                  (Hz, t, name, x.mean(), x.std(ddof=1) / np.sqrt(G), ref, z))
            assert abs(z) < zmax, (t, name, x.mean(), ref, z)
    sw.close()
