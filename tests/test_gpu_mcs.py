"""The per-MCS loop of src/ether.f90:159-203 on the GPU: graph replay vs direct launches,
parallel tempering against the oracle's restatement of src/parallel_tempering.f90, the
observable accumulators against get_eng / get_mag / observables_per_repeat, and statistical
parity of E, |M|, C_v, chi and the Binder cumulants with the oracle's reference-order run."""
import ctypes as C

import numpy as np
import pytest

import ether_gb300 as eg
from oracle import pyoracle as po
from tests.helpers import KB, assert_same_ensemble, beta_of, make_pair, random_ising, random_xyz

pytestmark = pytest.mark.gpu

FM = [[(1, 1, (-1.0, -1.0, -1.0))]]


def _state(sw, lat):
    return np.stack([sw.get_spins(lat.ion, r)[:, 1:4] for r in range(sw.R)])


@pytest.mark.parametrize("model", [eg.MODEL_ISING, eg.MODEL_XYZ])
def test_graph_replay_equals_direct_launches(model):
    lat = eg.simple_cubic(16)
    ktc = 4.511 if model == eg.MODEL_ISING else 1.443
    ladder = [beta_of(ktc * f) for f in (0.9, 1.0, 1.1, 1.3)]
    runs = []
    for flags in (0, eg.FLAG_NO_GRAPHS):
        sw, _ = make_pair(lat, model, FM, replicas=8, flags=flags)
        sw.set_ladder(ladder)
        sw.set_streams(stream=list(range(8)), step=[0] * 8)
        ion = random_ising(lat, 3) if model == eg.MODEL_ISING else random_xyz(lat, 3)
        sw.set_spins(ion)
        sc = sw.mcs(0, 47, tmcs_eq=20, coa=5, ovrr=True, ovrr_para=0.5, ovrr_mcs=3, pt=True,
                    exchange_interval=4)
        sc = sw.mcs(47, 40, tmcs_eq=20, coa=5, ovrr=True, ovrr_para=0.5, ovrr_mcs=3, pt=True,
                    exchange_interval=4, swap_count=sc)
        runs.append((_state(sw, lat), sw.sums(), sw.slots(), sc, sw.accept_counts()))
    a, b = runs
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])
    np.testing.assert_array_equal(a[2], b[2])
    assert a[3] == b[3] == 87 // 4 - 87 // 20
    np.testing.assert_array_equal(a[4], b[4])


def test_graph_replay_after_a_ladder_change():
    """ether_mcs, a new ladder with another slot count (4 slots x 2 groups -> 2 slots x 4
    groups), and ether_mcs again over steps with the same gate pattern: the graphs captured
    for the first ladder are not replayed with its launch arguments; the run equals direct
    launches."""
    lat = eg.simple_cubic(12)
    sch = dict(tmcs_eq=0, coa=5, ovrr=True, ovrr_para=0.5, ovrr_mcs=3, pt=True, exchange_interval=4)
    runs = []
    for flags in (0, eg.FLAG_NO_GRAPHS):
        sw, _ = make_pair(lat, eg.MODEL_XYZ, FM, replicas=8, flags=flags)
        sw.set_ladder([beta_of(1.443 * f) for f in (0.9, 1.0, 1.1, 1.3)])
        sw.set_spins(random_xyz(lat, 4))
        sc = sw.mcs(0, 60, **sch)
        sw.set_ladder([beta_of(1.443 * f) for f in (0.8, 1.2)])
        sc = sw.mcs(60, 60, swap_count=sc, **sch)
        runs.append((_state(sw, lat), sw.sums(), sw.slots(), sc))
    a, b = runs
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)


def test_mcs_equals_the_reference_call_sequence():
    """ether_mcs == the host loop of src/ether.f90:159-203 through the single-call entries."""
    lat = eg.simple_cubic(16)
    ladder = [beta_of(1.443 * f) for f in (0.8, 1.0, 1.2, 1.5)]
    s1, _ = make_pair(lat, eg.MODEL_XYZ, FM, replicas=4)
    s2, _ = make_pair(lat, eg.MODEL_XYZ, FM, replicas=4)
    ion = random_xyz(lat, 8)
    for s in (s1, s2):
        s.set_ladder(ladder)
        s.set_streams(stream=[0, 1, 2, 3], step=[0] * 4)
        s.set_spins(ion)
    tmcs_eq, coa, ovrr_mcs, para, ex = 10, 5, 3, 0.4, 4
    s1.mcs(0, 30, tmcs_eq, coa, ovrr=True, ovrr_para=para, ovrr_mcs=ovrr_mcs, pt=True,
           exchange_interval=ex)
    swap = 0
    for step in range(1, 31):
        if step % ovrr_mcs == 0 and step % coa != 0:
            s2.overrelaxation(para)
        s2.metropolis(1, accept=False)
        if step % ex == 0 and step % coa != 0:
            swap += 1
            s2.parallel_tempering(swap)
        s2.observable(step, tmcs_eq, coa)
    np.testing.assert_array_equal(_state(s1, lat), _state(s2, lat))
    np.testing.assert_array_equal(s1.sums(), s2.sums())
    np.testing.assert_array_equal(s1.slots(), s2.slots())


@pytest.mark.parametrize("model,R", [(eg.MODEL_XYZ, 18), (eg.MODEL_ISING, 18), (eg.MODEL_XYZ, 36),
                                     (eg.MODEL_ISING, 36)])
def test_mcs_in_replica_parts_equals_the_reference_call_sequence(model, R):
    """A general lattice with 16 or more replicas: ether_mcs runs the sweeps between PT and
    measurement steps as two (R >= 16) or four (R >= 32) replica parts on as many streams.  The
    result equals the single-call sequence (one launch per colour phase over all replicas):
    spins, sums, slots, swaps and acceptance counters."""
    lat = eg.pyrochlore(2, shells=(2.97243, 5.1484), tol=1e-3)
    shells = [[(1, 1, (1.0, 1.0, 1.0))], [(1, 1, (-0.1, -0.1, -0.1))]]
    ladder = [beta_of(0.5 * 1.25 ** k) for k in range(6)]
    kw = dict(zeeman=True, h=(0.0, 0.0, 1.0), g_factor=2.0)
    s1, _ = make_pair(lat, model, shells, replicas=R, **kw)
    s2, _ = make_pair(lat, model, shells, replicas=R, **kw)
    assert s1.info().fast_path == 0
    ion = random_xyz(lat, 8) if model == eg.MODEL_XYZ else random_ising(lat, 8)
    for s in (s1, s2):
        s.set_ladder(ladder)
        s.set_streams(stream=list(range(R)), step=[0] * R)
        s.set_spins(ion)
        s.zero_avg()
    tmcs_eq, coa, ex = 6, 5, 3
    sc = s1.mcs(0, 40, tmcs_eq, coa, pt=True, exchange_interval=ex)
    swap = 0
    for step in range(1, 41):
        s2.metropolis(1, accept=False)
        if step % ex == 0 and step % coa != 0:
            swap += 1
            s2.parallel_tempering(swap)
        s2.observable(step, tmcs_eq, coa)
    assert sc == swap
    np.testing.assert_array_equal(_state(s1, lat), _state(s2, lat))
    np.testing.assert_array_equal(s1.sums(), s2.sums())
    np.testing.assert_array_equal(s1.slots(), s2.slots())
    np.testing.assert_array_equal(s1.accept_counts(), s2.accept_counts())


@pytest.mark.parametrize("model", [eg.MODEL_XYZ, eg.MODEL_ISING])
def test_metropolis_in_replica_parts_equals_single_sweeps(model):
    """ether_metropolis(n > 1) on a general lattice with 36 replicas runs the n sweeps as four
    replica parts on parallel streams: the same spins and acceptance counters as n calls of one
    sweep."""
    lat = eg.pyrochlore(2, shells=(2.97243, 5.1484), tol=1e-3)
    shells = [[(1, 1, (1.0, 1.0, 1.0))], [(1, 1, (-0.1, -0.1, -0.1))]]
    R = 36
    s1, _ = make_pair(lat, model, shells, replicas=R)
    s2, _ = make_pair(lat, model, shells, replicas=R)
    ion = random_xyz(lat, 4) if model == eg.MODEL_XYZ else random_ising(lat, 4)
    for s in (s1, s2):
        s.set_beta([beta_of(0.4 + 0.1 * r) for r in range(R)])
        s.set_streams(stream=list(range(R)), step=[0] * R)
        s.set_spins(ion)
    s1.metropolis(12, accept=False)
    for _ in range(12):
        s2.metropolis(1, accept=False)
    np.testing.assert_array_equal(_state(s1, lat), _state(s2, lat))
    np.testing.assert_array_equal(s1.accept_counts(), s2.accept_counts())


@pytest.mark.parametrize("model", [eg.MODEL_XYZ, eg.MODEL_ISING])
def test_mcs_equals_the_oracles_replay_of_the_loop(model):
    """ether_mcs (overrelaxation every 3 steps for XYZ, PT every 2, a measurement every 4 after
    4 equilibration steps; 4 slots x 2 groups) against the oracle's replay of the same loop:
    Checkerboard sweeps of every replica at its current slot's temperature, overrelaxation
    passes, the total energies, PT swaps of each group (src/parallel_tempering.f90:39-108 with
    the same draws) and the observable accumulators (src/observable.f90:30-43).  Spins, slots
    and the swap count agree exactly; the accumulators to 1e-12 (energies are summed in another
    order)."""
    lat = eg.simple_cubic(8)
    ns, R, steps = 4, 8, 24
    ladder = np.array([beta_of(f * (1.443 if model == eg.MODEL_XYZ else 4.511)) for f in (0.8, 1.0, 1.2, 1.5)])
    sw, osys = make_pair(lat, model, FM, replicas=R)
    sw.set_ladder(ladder)
    streams = [3 * r + 1 for r in range(R)]
    sw.set_streams(stream=streams, step=[0] * R)
    xyz = model == eg.MODEL_XYZ
    ions = [(random_xyz if xyz else random_ising)(lat, 60 + r) for r in range(R)]
    for r in range(R):
        sw.set_spins(ions[r], replica=r)
    sw.zero_avg()
    tmcs_eq, coa, ovrr_mcs, para, ex = 4, 4, 3, 0.5, 2
    sc = sw.mcs(0, steps, tmcs_eq, coa, ovrr=xyz, ovrr_para=para, ovrr_mcs=ovrr_mcs, pt=True,
                exchange_interval=ex)

    ncol, col, rank = osys.colouring()
    sp4 = [osys.spin4(ion) if xyz else None for ion in ions]
    sor = np.arange(R) % ns                      # slot of each replica
    ros = np.arange(R, dtype=np.int32)           # per group: replica of each slot
    sums = np.zeros((R, 7))
    swap = 0
    N = lat.N

    def energy(r):
        return osys.tot_energy_f32(ions[r], sp4[r]) if xyz else osys.tot_energy(ions[r])

    def mag(r):
        return osys.tot_magnetisation_f32(ions[r], sp4[r]) if xyz else osys.tot_magnetisation(ions[r])

    t_ovrr = 0  # the overrelaxation counter advances once per overrelaxation step
    for step in range(1, steps + 1):
        if xyz and step % ovrr_mcs == 0 and step % coa != 0:
            for r in range(R):
                osys.overrelax_colour(ions[r], sp4[r], para, 1992, streams[r], t_ovrr, col, rank, ncol)
            t_ovrr += 1
        for r in range(R):
            osys.metropolis_colour(ions[r], sp4[r], 32 if xyz else 64, float(ladder[sor[r]]), 1992, streams[r],
                                   step - 1, col, rank, ncol)
        if step % ex == 0 and step % coa != 0:
            E = np.array([energy(r) for r in range(R)])
            swap += 1
            copy_from = np.zeros(ns, dtype=np.int32)
            for g in range(R // ns):
                sub = np.ascontiguousarray(ros[g * ns:(g + 1) * ns])
                po.lib().orc_parallel_tempering(ns, ladder.ctypes.data_as(po.PD), E.ctypes.data_as(po.PD),
                                                sub.ctypes.data_as(po.PI), swap, 1992, g, 0,
                                                copy_from.ctypes.data_as(po.PI))
                ros[g * ns:(g + 1) * ns] = sub
            for g in range(R // ns):
                for s_ in range(ns):
                    sor[ros[g * ns + s_]] = s_
        if step > tmcs_eq and step % coa == 0:
            for r in range(R):
                e = energy(r) / (2.0 * N)
                m = np.linalg.norm(mag(r)) / N
                a = sums[(r // ns) * ns + sor[r]]
                a += [1.0, e, e * e, (e * e) * (e * e), m, m * m, (m * m) * (m * m)]
    assert sc == swap
    np.testing.assert_array_equal(sw.slots(), sor)
    for r in range(R):
        g = sw.get_spins(lat.ion, r)
        if xyz:
            np.testing.assert_array_equal(g[:, [1, 2, 3, 5]].astype(np.float32), sp4[r], err_msg="replica %d" % r)
        else:
            np.testing.assert_array_equal(g[:, 3], ions[r][:, 3], err_msg="replica %d" % r)
    np.testing.assert_allclose(sw.sums(), sums, rtol=1e-12, atol=1e-15)


@pytest.mark.parametrize("copy_mode", [False, True])
def test_parallel_tempering_matches_oracle(copy_mode):
    lat = eg.simple_cubic(8)
    R = 6
    flags = eg.FLAG_PT_REFERENCE_COPY if copy_mode else 0
    sw, _ = make_pair(lat, eg.MODEL_ISING, FM, replicas=R, flags=flags)
    beta = np.array([beta_of(k) for k in (6.0, 5.0, 4.6, 4.4, 4.2, 3.0)])
    sw.set_ladder(beta)
    ions = [random_ising(lat, 40 + r) for r in range(R)]
    for r in range(R):
        sw.set_spins(ions[r], replica=r)
    for swap_count in (1, 2, 3):
        E = sw.tot_energy()
        before = np.stack([sw.get_spins(lat.ion, r)[:, 3] for r in range(R)])
        ros = np.argsort(sw.slots()).astype(np.int32)
        want = ros.copy()
        copy_from = np.full(R, -1, dtype=np.int32)
        n = po.lib().orc_parallel_tempering(R, beta.ctypes.data_as(po.PD), E.ctypes.data_as(po.PD),
                                            want.ctypes.data_as(po.PI), swap_count, 1992, 0,
                                            1 if copy_mode else 0, copy_from.ctypes.data_as(po.PI))
        got = sw.parallel_tempering(swap_count)
        assert got == n
        if copy_mode:
            after = np.stack([sw.get_spins(lat.ion, r)[:, 3] for r in range(R)])
            for s in range(R):
                src = copy_from[s]
                np.testing.assert_array_equal(after[ros[s]], before[ros[src]] if src >= 0 else before[ros[s]])
        else:
            np.testing.assert_array_equal(np.argsort(sw.slots()), want)


def test_observables_match_get_eng_get_mag():
    lat = eg.simple_cubic(8)
    R = 4
    sw, osys = make_pair(lat, eg.MODEL_XYZ, FM, replicas=R)
    beta = np.array([beta_of(k) for k in (1.0, 1.3, 1.6, 2.0)])
    sw.set_beta(beta)
    sw.set_streams(stream=[5, 6, 7, 8], step=[0] * 4)
    sw.set_spins(random_xyz(lat, 2))
    sw.zero_avg()
    acc = [po.Acc() for _ in range(R)]
    for step in range(1, 41):
        sw.metropolis(1, accept=False)
        sw.observable(step, 10, 2)
        if step > 10 and step % 2 == 0:
            E = sw.tot_energy()
            M = sw.tot_magnetisation()
            for r in range(R):
                m = np.ascontiguousarray(M[r])
                po.lib().orc_acc_sample(C.byref(acc[r]), E[r], m.ctypes.data_as(po.PD), lat.N)
    got = sw.avg()
    for r in range(R):
        want = np.zeros(6)
        po.lib().orc_acc_average(C.byref(acc[r]), beta[r], lat.N, want.ctypes.data_as(po.PD))
        np.testing.assert_allclose(got[r], want, rtol=1e-9)


def test_statistical_parity_with_reference_order_run():
    """E, |M|, C_v, chi, U_E, U_M per temperature from REPEAT = 16 independent repeats on the
    GPU (Checkerboard order, replicas) vs the oracle's reference-order (typewriter) run of
    src/ether.f90's per-temperature loop, compared in units of the combined REPEAT error bars
    (per temperature, jointly over the six observables: assert_same_ensemble)."""
    L, REP, TMCS, EQ, COA = 12, 16, 1200, 400, 5
    temps = [3.6, 4.4, 4.6, 6.0]
    lat = eg.simple_cubic(L)
    j = eg.couplings(1, FM, [1.0])
    osys = po.System.from_lattice(lat, j, np.array([1.0]), eg.MODEL_ISING)
    betas = np.array([beta_of(k) for k in temps])
    cfg = po.RunCfg(tmcs=TMCS, tmcs_eq=EQ, coa=COA, repeat=REP, ovrr=0, ovrr_para=0.0, ovrr_mcs=0,
                    seed=1992, itemp=1, rank=0)
    vals = np.zeros(6 * REP * len(temps))
    accr = np.zeros(len(temps))
    po.lib().orc_run_temperatures(osys.p(), osys.ion0.ctypes.data_as(po.PD), len(temps),
                                  betas.ctypes.data_as(po.PD), C.byref(cfg), 0,
                                  vals.ctypes.data_as(po.PD), accr.ctypes.data_as(po.PD))
    vals = vals.reshape(len(temps), REP, 6)
    mine = _gpu_run(lat, j, eg.MODEL_ISING, betas, REP, TMCS, EQ, COA)
    assert_same_ensemble(mine, vals)


def _reference_order(osys, lat, betas, cfg, ex=0):
    """The oracle's reference-order run: per temperature the loop of src/ether.f90:150-214
    (typewriter Metropolis, random-site overrelaxation, get_tot_energy every MCS); with ex > 0
    the temperatures run in lockstep as MPI ranks with parallel_tempering every ex MCS.
    Returns the per-REPEAT values (temperatures, REPEATs, 6)."""
    nT, REP = len(betas), cfg.repeat
    vals = np.zeros(6 * REP * nT)
    accr = np.zeros(nT)
    b = np.ascontiguousarray(betas, dtype=np.float64)
    if ex:
        n = C.c_long(0)
        po.lib().orc_run_ladder(osys.p(), osys.ion0.ctypes.data_as(po.PD), nT, b.ctypes.data_as(po.PD),
                                C.byref(cfg), ex, 0, vals.ctypes.data_as(po.PD),
                                accr.ctypes.data_as(po.PD), C.byref(n))
        assert n.value > 100  # the ladder does exchange configurations
    else:
        po.lib().orc_run_temperatures(osys.p(), osys.ion0.ctypes.data_as(po.PD), nT,
                                      b.ctypes.data_as(po.PD), C.byref(cfg), 0,
                                      vals.ctypes.data_as(po.PD), accr.ctypes.data_as(po.PD))
    return vals.reshape(nT, REP, 6)


def _gpu_run(lat, j, model, betas, REP, TMCS, EQ, COA, seed=77, **mcs_kw):
    kw = {k: mcs_kw.pop(k) for k in ("zeeman", "h", "g_factor", "sia", "sia_vec") if k in mcs_kw}
    sw = eg.Sweep.from_lattice(lat, j, np.array([1.0]), model, replicas=REP * len(betas), seed=seed,
                               **kw)
    sw.set_ladder(betas)
    sw.set_spins(lat.ion)
    sw.fresh_spins()
    sw.zero_avg()
    sw.mcs(0, TMCS, EQ, COA, **mcs_kw)
    mean, err = sw.per_repeat()
    # per-REPEAT values: replica g * nT + t is REPEAT g at temperature slot t
    vals = sw.avg().reshape(REP, len(betas), 6).transpose(1, 0, 2)
    np.testing.assert_allclose(vals.mean(1), mean, rtol=1e-9, atol=1e-12)
    sw.close()
    return vals


def test_heisenberg_overrelaxation_schedule_same_ensemble_as_reference_order():
    """The 32^3 + overrelaxation deck's schedule scaled down: 10^3 Heisenberg, OVRR (one pass,
    ovrr_para = 1) every 5 MCS gated as src/ether.f90:163-168 (so at steps = 5 mod 10 with
    COA 10), 4 temperatures around T_c = 1.443 J, REPEAT 16.  The GPU's colour-ordered
    reflection passes against the reference's nint(N ovrr_para) reflections at random sites
    (src/overrelaxation.f90:30-61) with typewriter Metropolis: the same ensemble."""
    L, REP, TMCS, EQ, COA = 10, 16, 2000, 600, 10
    lat = eg.simple_cubic(L)
    j = eg.couplings(1, FM, [1.0])
    osys = po.System.from_lattice(lat, j, np.array([1.0]), eg.MODEL_XYZ)
    betas = np.array([beta_of(k) for k in (1.0, 1.4, 1.5, 2.5)])
    cfg = po.RunCfg(tmcs=TMCS, tmcs_eq=EQ, coa=COA, repeat=REP, ovrr=1, ovrr_para=1.0, ovrr_mcs=5,
                    seed=1992, itemp=1, rank=0)
    ref = _reference_order(osys, lat, betas, cfg)
    mine = _gpu_run(lat, j, eg.MODEL_XYZ, betas, REP, TMCS, EQ, COA, ovrr=True, ovrr_para=1.0,
                    ovrr_mcs=5)
    assert_same_ensemble(mine, ref)


def test_heisenberg_pt_ladder_zeeman_sia_same_ensemble_as_reference_order():
    """Heisenberg 8^3 with a Zeeman field (0, 0, 0.5) T (g = 2) and single-ion anisotropy
    D = -0.2 meV along z, a 6-temperature geometric ladder 1.2 .. 1.8 J, parallel tempering
    every 7 MCS except at measurement steps, REPEAT 16: the GPU's slot-index swaps against the
    oracle's ranks in lockstep exchanging configurations (src/parallel_tempering.f90:39-108,
    raw get_tot_energy in the exponent)."""
    L, REP, TMCS, EQ, COA, EX = 8, 16, 1600, 500, 10, 7
    lat = eg.simple_cubic(L)
    j = eg.couplings(1, FM, [1.0])
    opts = dict(zeeman=True, h=(0.0, 0.0, 0.5), g_factor=2.0, sia=True,
                sia_vec=np.array([[0.0, 0.0, -0.2e-3]]))
    osys = po.System.from_lattice(lat, j, np.array([1.0]), eg.MODEL_XYZ, **opts)
    betas = np.array([beta_of(k) for k in np.geomspace(1.2, 1.8, 6)])
    cfg = po.RunCfg(tmcs=TMCS, tmcs_eq=EQ, coa=COA, repeat=REP, ovrr=0, ovrr_para=0.0, ovrr_mcs=0,
                    seed=1992, itemp=1, rank=0)
    ref = _reference_order(osys, lat, betas, cfg, ex=EX)
    mine = _gpu_run(lat, j, eg.MODEL_XYZ, betas, REP, TMCS, EQ, COA, pt=True, exchange_interval=EX,
                    **opts)
    assert_same_ensemble(mine, ref)


def test_ising_pt_ladder_same_ensemble_as_reference_order():
    """Ising 10^3, 6 temperatures 4.2 .. 4.9 J around T_c = 4.511 J, PT every 5 MCS except at
    measurement steps (COA 4), REPEAT 16."""
    L, REP, TMCS, EQ, COA, EX = 10, 16, 1600, 500, 4, 5
    lat = eg.simple_cubic(L)
    j = eg.couplings(1, FM, [1.0])
    osys = po.System.from_lattice(lat, j, np.array([1.0]), eg.MODEL_ISING)
    betas = np.array([beta_of(k) for k in np.geomspace(4.2, 4.9, 6)])
    cfg = po.RunCfg(tmcs=TMCS, tmcs_eq=EQ, coa=COA, repeat=REP, ovrr=0, ovrr_para=0.0, ovrr_mcs=0,
                    seed=1992, itemp=1, rank=0)
    ref = _reference_order(osys, lat, betas, cfg, ex=EX)
    mine = _gpu_run(lat, j, eg.MODEL_ISING, betas, REP, TMCS, EQ, COA, pt=True, exchange_interval=EX)
    assert_same_ensemble(mine, ref)


@pytest.mark.parametrize("L", [16, (16, 8, 16)])
@pytest.mark.parametrize("model", [eg.MODEL_ISING, eg.MODEL_XYZ])
def test_record_series_equals_step_by_step(model, L):
    """ether_record_series against the same sweeps with ether_tot_energy /
    ether_tot_magnetisation after each stride.  (16, 8, 16): 2048 sites, one reduction block
    per replica, where the Ising magnetisation is counted 16 bytes at a time."""
    lat = eg.simple_cubic(L)
    runs = []
    for way in ("series", "steps"):
        sw, _ = make_pair(lat, model, FM, replicas=3)
        sw.set_beta([beta_of(k) for k in (4.0, 4.5, 5.0)] if model == eg.MODEL_ISING else
                    [beta_of(k) for k in (1.2, 1.4, 1.6)])
        sw.set_streams(stream=[1, 2, 3], step=[0, 0, 0])
        sw.set_spins(random_ising(lat, 6) if model == eg.MODEL_ISING else random_xyz(lat, 6))
        if way == "series":
            m, e = sw.record_series(24, stride=4, energy=True)
            m2 = sw.record_series(8, stride=2)  # magnetisation-only path
        else:
            m = np.zeros((3, 6)); e = np.zeros((3, 6)); m2 = np.zeros((3, 4))
            for t in range(6):
                sw.metropolis(4, accept=False)
                e[:, t] = sw.tot_energy()
                m[:, t] = np.linalg.norm(sw.tot_magnetisation(), axis=1)
            for t in range(4):
                sw.metropolis(2, accept=False)
                m2[:, t] = np.linalg.norm(sw.tot_magnetisation(), axis=1)
        runs.append((m, e, m2))
    (a, b, c), (x, y, z) = runs
    np.testing.assert_allclose(a, x, rtol=1e-12)
    np.testing.assert_allclose(b, y, rtol=1e-12)
    np.testing.assert_allclose(c, z, rtol=1e-12)


@pytest.mark.parametrize("L", [16, 8, 24])
def test_resident_sweeps_equal_phase_launches(L):
    """A small simple-cubic Ising lattice with enough replicas runs the sweeps between PT and
    measurement steps in the shared-memory resident kernel: same draws, so the configurations,
    observable sums, PT slots and acceptance counts equal those of the phase-by-phase launches
    (ETHER_FLAG_NO_RESIDENT), with far fewer launches.  L = 16: 8-byte vectors; 8 and 24:
    4-byte vectors."""
    lat = eg.simple_cubic(L)
    j = eg.couplings(1, FM, [1.0])
    temps = np.linspace(3.5, 6.0, 48)
    runs = []
    for flags in (0, eg.FLAG_NO_RESIDENT):
        sw = eg.Sweep.from_lattice(lat, j, np.array([1.0]), eg.MODEL_ISING, replicas=96, seed=5,
                                   flags=flags)
        sw.set_ladder([beta_of(k) for k in temps])
        sw.set_spins(lat.ion)
        sw.fresh_spins()
        sw.zero_avg()
        n0 = sw.info().kernel_launches
        swaps = sw.mcs(0, 150, 40, 10, pt=True, exchange_interval=11)
        swaps = sw.mcs(150, 63, 40, 10, pt=True, exchange_interval=11, swap_count=swaps)
        runs.append(dict(launches=sw.info().kernel_launches - n0, sums=sw.sums(), slots=sw.slots(),
                         acc=sw.accept_counts(), swaps=swaps,
                         spins=np.stack([sw.get_spins(lat.ion, r)[:, 3] for r in (0, 37, 95)])))
        sw.close()
    a, b = runs
    np.testing.assert_array_equal(a["spins"], b["spins"])
    np.testing.assert_array_equal(a["sums"], b["sums"])
    np.testing.assert_array_equal(a["slots"], b["slots"])
    np.testing.assert_array_equal(a["acc"], b["acc"])
    assert a["swaps"] == b["swaps"] and (a["slots"] != np.arange(96) % 48).any()
    assert a["launches"] * 2 < b["launches"]
