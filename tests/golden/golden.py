"""Golden fixtures: small seeded cases of the Monte Carlo path with the oracle's results.

Test infrastructure, used by tests/test_golden.py and tests/golden/make_golden.py only.  A
fixture (tests/golden/<name>.npz) holds the inputs exactly as ether_create takes them (the
reference's ion(0:8, N), nn, j_exc, s, stgg, sia_vec arrays and the local-axis anisotropy),
each replica's initial configuration, the inverse temperatures, random streams and a
schedule of Metropolis sweeps and overrelaxation passes, and the oracle's results: every
replica's final spins (Ising +-1; XYZ the FP32 state S_x, S_y, S_z, phi), its total energy
(src/get_tot_energy.f90:33-47) and magnetisation (src/get_tot_magnetisation.f90:32-40).
Structure-factor fixtures hold the FP64 direct sums of
utility/Structure_Factor/structure_factor.f90:131-183 on a small q-grid.

The reference itself cannot be built here (no Fortran compiler) and ships no golden vectors,
so these fixtures pin the oracle against drift and give the GPU a fixed target; they do not
pin the oracle to the reference.
"""
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

SWEEP_CASES = ["sc3_ising_zeeman", "sc8x4x4_ising_staggered", "sc3_xyz_zeeman_sia",
               "sc8x6x4_xyz_ovrr", "pyro3_xyz_angle_local_sia", "pyro3_ising_j1j2"]
SQ_CASES = ["pyro2_sq_xyz", "pyro2_sq_ising"]
MODEL_ISING, MODEL_XYZ = 0, 1


def path(name):
    return os.path.join(HERE, name + ".npz")


def load(name):
    z = np.load(path(name), allow_pickle=False)
    fix = {k: z[k] for k in z.files}
    fix["meta"] = json.loads(str(fix["meta"]))
    return fix


def save(name, fix):
    out = {k: v for k, v in fix.items() if k != "meta"}
    out["meta"] = np.array(json.dumps(fix["meta"], sort_keys=True))
    np.savez_compressed(path(name), **out)


def options(fix):
    """Keyword arguments shared by the oracle's System and the library's Sweep."""
    m = fix["meta"]
    kw = dict(model=m["model"], n_species=m["n_species"], n_shells=m["n_shells"], cap=m["cap"],
              angle=m["angle"], dphi=m["dphi"], zeeman=m["zeeman"], h=tuple(m["h"]),
              g_factor=m["g_factor"], sia=m["sia"])
    for k in ("stgg", "sia_vec", "sia_local"):
        kw[k] = fix[k] if k in fix else None
    return kw


# ------------------------------------------------------------------ oracle replay -------
def oracle_sweeps(fix):
    """The oracle's Checkerboard replay of the schedule for every replica (FP32 mirror for
    XYZ): final spins, E and M per replica."""
    from oracle import pyoracle as po
    m = fix["meta"]
    osys = po.System(fix["ion"], fix["nn"], fix["j_exc"], fix["s"], **options(fix))
    ncol, col, rank = osys.colouring()
    xyz = m["model"] == MODEL_XYZ
    spins, E, M = [], [], []
    for r in range(m["replicas"]):
        ion = fix["spins0"][r].copy()
        sp4 = osys.spin4(ion) if xyz else None
        t = to = 0
        for op, arg in m["schedule"]:
            if op == "metro":
                for _ in range(int(arg)):
                    osys.metropolis_colour(ion, sp4, 32 if xyz else 64, float(fix["betas"][r]), m["seed"],
                                           int(fix["streams"][r]), t, col, rank, ncol)
                    t += 1
            else:
                osys.overrelax_colour(ion, sp4, float(arg), m["seed"], int(fix["streams"][r]), to, col,
                                      rank, ncol)
                to += 1
        if xyz:
            spins.append(sp4.copy())
            E.append(osys.tot_energy_f32(ion, sp4))
            M.append(osys.tot_magnetisation_f32(ion, sp4))
        else:
            spins.append(np.where(ion[:, 3] > 0, 1, -1).astype(np.int8))
            E.append(osys.tot_energy(ion))
            M.append(osys.tot_magnetisation(ion))
    return {"spins": np.array(spins), "E": np.array(E), "M": np.array(M)}


def reciprocal(abc):
    abc = np.asarray(abc, float)
    vol = np.dot(abc[0], np.cross(abc[1], abc[2]))
    return 2 * np.pi * np.array([np.cross(abc[1], abc[2]), np.cross(abc[2], abc[0]),
                                 np.cross(abc[0], abc[1])]) / vol


def oracle_sq(fix):
    """FP64 direct sums on every q-point of the grid (flat index h1 + n0 (h2 + n1 h3))."""
    from oracle import pyoracle as po
    m = fix["meta"]
    nq, q0, dq = m["nq"], m["q0"], m["dq"]
    Q = int(np.prod(nq))
    qidx = np.arange(Q)
    h1, h2, h3 = qidx % nq[0], (qidx // nq[0]) % nq[1], qidx // (nq[0] * nq[1])
    coef = np.stack([q0[0] + h1 * dq[0], q0[1] + h2 * dq[1], q0[2] + h3 * dq[2]], axis=1)
    qv = np.ascontiguousarray(coef @ reciprocal(fix["abc"]))
    pos = np.ascontiguousarray(fix["ion"][:, 6:9])
    N = pos.shape[0]
    sq, comp = [], []
    for S in fix["S"]:
        out = np.zeros(6 * Q)
        po.lib().orc_structure_factor(N, pos.ctypes.data_as(po.PD),
                                      np.ascontiguousarray(S, dtype=np.float64).ctypes.data_as(po.PD), Q,
                                      qv.ctypes.data_as(po.PD), out.ctypes.data_as(po.PD))
        out = out.reshape(-1, 3, 2)
        m2 = (out ** 2).sum(axis=2)
        sq.append(m2.sum(axis=1) / N ** 2)
        comp.append(np.sqrt(m2) / N)
    return {"sq": np.array(sq), "comp": np.array(comp)}


# ------------------------------------------------------------------ GPU replay ----------
def _sweep(fix):
    import ether_gb300 as eg
    m = fix["meta"]
    return eg.Sweep(fix["ion"], fix["nn"], fix["j_exc"], fix["s"], replicas=m["replicas"], seed=m["seed"],
                    sc=tuple(m["sc"]), basis=m["basis"], **options(fix))


def gpu_sweeps(fix):
    """The same schedule through the C-ABI: ether_set_beta, ether_set_streams,
    ether_set_spins, ether_metropolis / ether_overrelaxation, ether_get_spins, ether_tot_energy,
    ether_tot_magnetisation."""
    m = fix["meta"]
    R = m["replicas"]
    sw = _sweep(fix)
    try:
        sw.set_beta(fix["betas"])
        sw.set_streams(stream=[int(x) for x in fix["streams"]], step=[0] * R)
        for r in range(R):
            sw.set_spins(fix["spins0"][r], r)
        for op, arg in m["schedule"]:
            if op == "metro":
                sw.metropolis(int(arg), accept=False)
            else:
                sw.overrelaxation(float(arg))
        spins = []
        for r in range(R):
            g = sw.get_spins(fix["ion"], r)
            if m["model"] == MODEL_XYZ:
                spins.append(g[:, [1, 2, 3, 5]].astype(np.float32))
            else:
                spins.append(np.where(g[:, 3] > 0, 1, -1).astype(np.int8))
        return {"spins": np.array(spins), "E": np.asarray(sw.tot_energy()),
                "M": np.asarray(sw.tot_magnetisation())}, sw.info().fast_path
    finally:
        sw.close()


def gpu_sq(fix):
    """ether_structure_factor of the fixture's configurations."""
    import ctypes as C
    from ether_gb300 import abi
    m = fix["meta"]
    sw = _sweep(fix)
    try:
        ion = fix["ion"].copy()
        for r in range(m["replicas"]):
            S = fix["S"][r]
            if m["model"] == MODEL_XYZ:
                ion[:, 1:4] = S
            else:
                ion[:, 3] = S[:, 2]
            sw.set_spins(ion, r)
        Q = int(np.prod(m["nq"]))
        sq = np.zeros(m["replicas"] * Q, dtype=np.float32)
        comp = np.zeros(m["replicas"] * Q * 3, dtype=np.float32)
        a = np.ascontiguousarray(fix["abc"], dtype=np.float64).ravel()
        abi.check(sw.lib.ether_structure_factor(
            sw.h, abi.dptr(a), abi.iptr(np.asarray(m["nq"], dtype=np.int32)),
            abi.dptr(np.asarray(m["q0"], float)), abi.dptr(np.asarray(m["dq"], float)),
            sq.ctypes.data_as(C.POINTER(C.c_float)), comp.ctypes.data_as(C.POINTER(C.c_float))))
        return {"sq": sq.reshape(m["replicas"], Q), "comp": comp.reshape(m["replicas"], Q, 3)}
    finally:
        sw.close()
