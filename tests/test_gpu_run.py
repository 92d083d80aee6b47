"""ether_run end to end on the GPU: the output files of src/ether.f90 (ETHER.obs, ETHER.spn and
the .dat / .xsf files written from them) against the oracle's restatement of the writers on
the same records; the run's thermodynamics against the oracle's reference-order run of the
same deck; PT rounds, STATUS, resume from ETHER.spn; and the per-temperature acceptance and
spiral-state accumulators that the driver reads."""
import ctypes as C
import os

import numpy as np
import pytest

import ether_gb300 as eg
from oracle import deck_oracle as do
from oracle import pyoracle as po
from tests.helpers import assert_means_agree
from tests.test_deck import SC_STRUCT, write_deck

pytestmark = pytest.mark.gpu

ISING_DECK = ("model = ising\nmcs = 1500 500\ntemp = 70 40 7.5\nspin = 1\nspecies = A\n"
              "sc = 10 10 10\nrepeat = 8\ncoa = 5\nseed = 1992\n")
J_FM = "1\n1.0 1\nA A -1.0 -1.0 -1.0\n"


def _oracle_lattice(deck):
    b, sp = do.basis(deck)
    ion, stgg = po.supercell(b, sp, np.asarray(deck["abc"]), deck["sc"], checkerboard=deck["cb"])
    rc, nn = po.neighbours_bruteforce(ion, np.asarray(deck["abc"]), deck["sc"], "".join(deck["bc"]),
                                      deck["nbd_dis"], deck["nbdfc"], deck["nbd_capacity"])
    assert rc == 0
    return ion, stgg, nn


def test_run_outputs_match_the_reference_writers(tmp_path):
    indir = write_deck(str(tmp_path / "in"), ISING_DECK.replace("sc = 10 10 10", "sc = 6 6 6")
                       .replace("mcs = 1500 500", "mcs = 300 100").replace("repeat = 8", "repeat = 3"),
                       SC_STRUCT, J_FM)
    out = str(tmp_path / "out")
    os.makedirs(out)
    open(os.path.join(out, "STATUS"), "w").close()
    info = eg.run(indir, out)
    deck = do.read_deck(indir)
    n, nt = 216, deck["nscan"]
    assert nt == 5 and info["n_rounds"] == 1 and info["site_updates"] == n * nt * 3 * 300
    assert not os.path.exists(os.path.join(out, "STATUS"))  # answered and removed
    obs = do.read_obs(os.path.join(out, "ETHER.obs"), 1)
    spn = do.read_spn(os.path.join(out, "ETHER.spn"), n)
    assert obs.shape == (nt, 23) and spn.shape == (nt, n, 9)
    ion0, _, _ = _oracle_lattice(deck)
    np.testing.assert_array_equal(obs[:, 0], [70.0, 62.5, 55.0, 47.5, 40.0])
    for t in range(nt):
        np.testing.assert_array_equal(spn[t][:, [0, 4, 5, 6, 7, 8]], ion0[:, [0, 4, 5, 6, 7, 8]])
        assert set(np.unique(spn[t][:, 3])) <= {-1.0, 1.0} and not spn[t][:, 1:3].any()
        # ETHER.obs keeps get_moment_vectors of the configuration ETHER.spn keeps
        assert obs[t, 22] == spn[t][:, 3].sum()
    assert np.all(np.isfinite(obs[:, 1:14])) and not obs[:, 14:20].any()
    acc = obs[:, 13]
    assert np.all((acc > 0) & (acc < 100)) and np.all(np.diff(acc) < 0), acc
    assert np.all(np.diff(obs[:, 1]) > 0), obs[:, 1]  # |M| grows on cooling
    want = do.output_files(deck, obs, spn, ion0)
    for name, text in want.items():
        got = open(os.path.join(out, "data", name), encoding="utf-8").read()
        assert got == text, name
    for t in range(nt):
        path = os.path.join(out, "spins", do.spk_name(obs[t, 0]))
        rows = open(path).read().splitlines()
        assert rows[0] == " CRYSTAL" and rows[10] == "         216  1"
        assert "\n".join(rows[11:]) + "\n" == do.spk_rows(deck, spn[t])
    assert os.path.exists(os.path.join(out, "data", "graph.sh"))


def test_run_thermodynamics_match_oracle_run(tmp_path):
    """ETHER.obs of a 10^3 Ising deck vs the oracle's reference-order run of the same deck
    (typewriter Metropolis, REPEATs one after another): |M|, chi, U_M, E, C_v, U_E per
    temperature in units of the combined REPEAT error bars (the family-wise rule of
    assert_means_agree), and the acceptance rate."""
    indir = write_deck(str(tmp_path / "in"), ISING_DECK, SC_STRUCT, J_FM)
    out = str(tmp_path / "out")
    eg.run(indir, out)
    deck = do.read_deck(indir)
    obs = do.read_obs(os.path.join(out, "ETHER.obs"), 1)
    ion0, stgg, nn = _oracle_lattice(deck)
    osys = po.System(ion0, nn, np.asarray(deck["j_exc"]), np.asarray(deck["s"]), model=eg.MODEL_ISING,
                     n_species=1, n_shells=deck["nsh"], cap=deck["nbd_capacity"], stgg=stgg)
    nt, rep = deck["nscan"], deck["repeat"]
    betas = np.array([1.0 / (deck["kb"] * (deck["ht"] - deck["tint"] * t)) for t in range(nt)])
    cfg = po.RunCfg(tmcs=deck["tmcs"], tmcs_eq=deck["tmcs_eq"], coa=int(deck["coa"]), repeat=rep, ovrr=0,
                    ovrr_para=0.0, ovrr_mcs=0, seed=1992, itemp=1, rank=0)
    vals = np.zeros(6 * rep * nt)
    accr = np.zeros(nt)
    po.lib().orc_run_temperatures(osys.p(), osys.ion0.ctypes.data_as(po.PD), nt, betas.ctypes.data_as(po.PD),
                                  C.byref(cfg), 0, vals.ctypes.data_as(po.PD), accr.ctypes.data_as(po.PD))
    vals = vals.reshape(nt, rep, 6)  # (e, U_E, C_v, |m|, U_M, chi) per repeat
    ref = np.zeros((nt, 6))
    ref_err = np.zeros((nt, 6))
    for t in range(nt):
        ref[t], ref_err[t] = do.per_repeat(vals[t])
    # ETHER.obs order: 1 |M|, 2 chi, 3 d|M|, 4 dchi, 5 U_M, 6 dU_M, 7 E, 8 C_v, 9 dE, 10 dC_v, 11 U_E, 12 dU_E
    mine = obs[:, [7, 11, 8, 1, 5, 2]]
    mine_err = obs[:, [9, 12, 10, 3, 6, 4]]
    assert_means_agree(mine, mine_err, ref, ref_err, rep, rep)
    np.testing.assert_allclose(obs[:, 13], 100.0 * accr, rtol=0.05, atol=0.5)


def test_run_pt_rounds_and_resume(tmp_path):
    deck_text = ("model = xyz\nmcs = 400 100\ntemp = 20 2 3\nspin = 1\nspecies = A\nsc = 8 8 8\n"
                 "repeat = 2\ncoa = 4\npt = .T. 3\n")
    indir = write_deck(str(tmp_path / "in"), deck_text, SC_STRUCT, J_FM)
    out = str(tmp_path / "out")
    a = eg.run(indir, out, ranks=4)  # 7 temperatures: rounds of 4 and 3
    assert a["n_rounds"] == 2 and a["n_temperatures"] == 7
    obs = do.read_obs(os.path.join(out, "ETHER.obs"), 1)
    assert np.all(np.isfinite(obs[:, 1:14])) and np.all(np.diff(obs[:, 13]) < 0)
    b = eg.run(indir, str(tmp_path / "out1"))  # one ladder of seven
    assert b["n_rounds"] == 1
    # resume: every temperature starts from its ETHER.spn record instead of a fresh state
    short = deck_text.replace("mcs = 400 100", "mcs = 8 4").replace("coa = 4", "coa = 1")
    indir2 = write_deck(str(tmp_path / "in2"), short, SC_STRUCT, J_FM)
    spn = do.read_spn(os.path.join(out, "ETHER.spn"), 512)
    eg.run(indir2, out, resume=True)
    resumed = do.read_obs(os.path.join(out, "ETHER.obs"), 1)
    fresh_dir = str(tmp_path / "fresh")
    eg.run(indir2, fresh_dir)
    fresh = do.read_obs(os.path.join(fresh_dir, "ETHER.obs"), 1)
    m_spn = np.array([np.linalg.norm(s[:, 1:4].sum(0)) / 512 for s in spn])
    assert resumed[-1, 1] > 0.85 and resumed[-1, 1] > fresh[-1, 1] + 0.2, (resumed[:, 1], fresh[:, 1])
    assert abs(resumed[-1, 1] - m_spn[-1]) < 0.1
    # a record of another lattice is refused
    with open(os.path.join(fresh_dir, "ETHER.spn"), "r+b") as f:
        f.truncate(100)
    with pytest.raises(eg.EtherError, match="ETHER.spn"):
        eg.run(indir2, fresh_dir, resume=True)


def _ladder_sweep(model, L, temps, groups, seed=5):
    lat = eg.simple_cubic(L)
    j = eg.couplings(1, [[(1, 1, (-1.0, -1.0, -1.0))]], [1.0])
    sw = eg.Sweep.from_lattice(lat, j, np.array([1.0]), model, replicas=len(temps) * groups, seed=seed)
    sw.set_ladder([1.0 / (eg.KB_EV * t) for t in temps])
    sw.set_spins(lat.ion)
    sw.fresh_spins()
    sw.zero_avg()
    return lat, sw


def test_slot_accept_counts_follow_the_slots():
    """Per-(group, slot) acceptance equals each replica's accepts credited, step by step, to
    the slot it held during that step; without PT it equals the per-replica count."""
    lat, sw = _ladder_sweep(eg.MODEL_ISING, 8, [46.0, 50.0, 54.0, 58.0], 2)
    sw.metropolis(5, accept=False)
    np.testing.assert_array_equal(sw.slot_accept_counts(), sw.accept_counts())
    sw.reset_accept_counts()
    want = np.zeros(sw.R, dtype=np.uint64)
    prev = sw.accept_counts()
    ns = 4
    swaps = 0
    for step in range(1, 61):
        slots = sw.slots()
        swaps = sw.mcs(step - 1, 1, 1000, 7, pt=True, exchange_interval=2, swap_count=swaps)
        now = sw.accept_counts()
        for r in range(sw.R):
            want[(r // ns) * ns + slots[r]] += now[r] - prev[r]
        prev = now
    assert (sw.slots() != np.arange(sw.R) % ns).any()  # PT moved replicas
    np.testing.assert_array_equal(sw.slot_accept_counts(), want)
    per_slot = sw.slot_accept_counts().reshape(2, ns).sum(0)
    assert np.all(np.diff(per_slot.astype(np.int64)) > 0)  # slot 0 is the coldest


def test_spiral_avg_equals_host_accumulation():
    lat, sw = _ladder_sweep(eg.MODEL_XYZ, 6, [0.5, 5.0, 30.0], 2, seed=9)
    count = sw.spiral_setup(1.01, (0.0, 0.0, 1.0), 5.0, 4)
    sw.zero_avg()
    acc = np.zeros((sw.R, 4))
    coa, eq = 3, 6
    swaps = 0
    for step in range(1, 31):
        swaps = sw.mcs(step - 1, 1, eq, coa, pt=True, exchange_interval=5, swap_count=swaps)
        if step > eq and step % coa == 0:
            x = sw.spiral_state()
            slots = sw.slots()
            for r in range(sw.R):
                pos = (r // 3) * 3 + slots[r]
                acc[pos] += [1.0, x[r], x[r] ** 2, x[r] ** 4]
    got = sw.spiral_avg()
    betas = np.array([1.0 / (eg.KB_EV * t) for t in [0.5, 5.0, 30.0]] * 2)
    m, m2, m4 = acc[:, 1] / acc[:, 0], acc[:, 2] / acc[:, 0], acc[:, 3] / acc[:, 0]
    want = np.stack([m, 1.5 - 0.5 * m4 / m2 ** 2, betas * (m2 - m ** 2) * count], axis=1)
    np.testing.assert_allclose(got, want, rtol=1e-10, atol=1e-14)
    assert acc[0, 0] == 8
    sw.zero_avg()
    sw.mcs(30, 6, 0, 3)
    assert np.all(np.isfinite(sw.spiral_avg()))


def test_per_repeat_with_one_group_gives_nan_errors():
    lat, sw = _ladder_sweep(eg.MODEL_ISING, 6, [40.0, 60.0], 1)
    sw.mcs(0, 20, 5, 5)
    mean, err = sw.per_repeat()
    assert np.all(np.isfinite(mean)) and np.all(np.isnan(err))


AFM_STRUCT = ("two species\n1.0\n 2.0 0 0\n 0 2.0 0\n 0 0 2.0\n A B\n 4 4\nDirect\n"
              " 0 0 0\n 0 0.5 0.5\n 0.5 0 0.5\n 0.5 0.5 0\n 0 0 0.5\n 0 0.5 0\n 0.5 0 0\n 0.5 0.5 0.5\n")


def test_run_two_species_staggered_spiral_deck(tmp_path):
    """An XYZ deck with two species on the rock-salt split of a simple-cubic lattice,
    antiferromagnetic A-B bonds, staggered signs from the 'staggered' file, overrelaxation and
    the spiral-state observable: the general-lattice kernels, OVRR, the spiral accumulators
    and every writer, through ether_run."""
    deck_text = ("model = xyz\nmcs = 600 200\ntemp = 20 5 5\nspin = 1 1\nspecies = A B\nsc = 3 3 3\n"
                 "repeat = 3\ncoa = 5\nstg = .T.\novrr = .T. 0.5 4\nssp = .T.\nss_dis = 1.01\n"
                 "ss_lat = 5\nss_direc = 0 0 1\nspiral_capacity = 4\n")
    indir = write_deck(str(tmp_path / "in"), deck_text, AFM_STRUCT, "1\n1.0 1\nA B 3.0 3.0 3.0\n",
                       staggered="-1 B\n")
    out = str(tmp_path / "out")
    info = eg.run(indir, out)
    deck = do.read_deck(indir)
    n = 8 * 27
    assert info["n_sites"] == n and info["n_temperatures"] == 4
    obs = do.read_obs(os.path.join(out, "ETHER.obs"), 2)
    spn = do.read_spn(os.path.join(out, "ETHER.spn"), n)
    ion0, _, _ = _oracle_lattice(deck)
    for name, text in do.output_files(deck, obs, spn, ion0).items():
        assert open(os.path.join(out, "data", name), encoding="utf-8").read() == text, name
    assert np.all(np.isfinite(obs[:, 1:20]))
    assert np.all(obs[:, 14] > 0.0)                     # spiral state <|psi|>
    # staggered |M| orders on cooling (A-B antiferromagnet, B counted with sign -1)
    assert obs[-1, 1] > 0.6 and obs[-1, 1] > obs[0, 1]
    # get_moment_vectors includes the staggered sign: B's moment, counted with -1, points
    # along A's at the lowest temperature
    mA, mB = obs[-1, 20:23], obs[-1, 23:26]
    assert np.dot(mA, mB) > 0.0
    for t in range(4):
        nrm = np.linalg.norm(spn[t][:, 1:4], axis=1)
        np.testing.assert_allclose(nrm, 1.0, atol=1e-6)
