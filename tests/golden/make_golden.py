#!/usr/bin/env python
"""Writes the golden fixtures of tests/golden (see golden.py): builds each case's inputs with
the package's lattice builders, seeded random configurations, and runs the oracle on them.

    python tests/golden/make_golden.py            (after building: __graft_entry__.build())

Test infrastructure: rerun only when a case is added or the oracle is deliberately changed.
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import ether_gb300 as eg  # noqa: E402
from tests.golden import golden  # noqa: E402

FM = [[(1, 1, (-1.0, -1.0, -1.0))]]      # ETHER's sign: J < 0 is ferromagnetic
AFM = [[(1, 1, (1.0, 1.0, 1.0))]]
J1J2 = [[(1, 1, (1.0, 1.0, 1.0))], [(1, 1, (-0.1, -0.1, -0.1))]]
SEED = 1992


def beta(kT_mev):
    return 1.0 / (kT_mev * 1e-3)


def ising_spins(lat, R, seed):
    rng = np.random.default_rng(seed)
    out = np.repeat(lat.ion[None].copy(), R, axis=0)
    out[:, :, 1:3] = 0.0
    out[:, :, 3] = rng.choice([-1.0, 1.0], size=(R, lat.N))
    return out


def xyz_spins(lat, R, seed):
    rng = np.random.default_rng(seed)
    out = np.repeat(lat.ion[None].copy(), R, axis=0)
    v = rng.normal(size=(R, lat.N, 3))
    v /= np.linalg.norm(v, axis=2, keepdims=True)
    out[:, :, 1:4] = v.astype(np.float32).astype(np.float64)  # the FP32 state the GPU holds
    out[:, :, 5] = rng.uniform(-np.pi, np.pi, size=(R, lat.N)).astype(np.float32)
    return out


def base(lat, model, shells, kTs, streams, schedule, seed_spins, s=(1.0,), **opts):
    R = len(kTs)
    j = eg.couplings(lat.n_species, shells, list(s))
    fix = {"ion": lat.ion, "nn": lat.nn, "j_exc": j, "s": np.asarray(s, float),
           "betas": np.array([beta(k) for k in kTs]), "streams": np.asarray(streams, dtype=np.int64),
           "spins0": (ising_spins if model == golden.MODEL_ISING else xyz_spins)(lat, R, seed_spins)}
    if lat.stgg is not None:
        fix["stgg"] = np.asarray(lat.stgg, float)
    for k in ("sia_vec", "sia_local"):
        if opts.get(k) is not None:
            fix[k] = np.asarray(opts.pop(k), float)
        else:
            opts.pop(k, None)
    fix["meta"] = {"model": model, "n_species": int(j.shape[1]), "n_shells": int(lat.nsh),
                   "cap": int(lat.cap), "replicas": R, "seed": SEED, "schedule": schedule,
                   "sc": [int(x) for x in lat.sc], "basis": int(lat.nbasis),
                   "angle": bool(opts.get("angle", False)), "dphi": float(opts.get("dphi", 0.0)),
                   "zeeman": bool(opts.get("zeeman", False)), "h": list(opts.get("h", (0.0, 0.0, 0.0))),
                   "g_factor": float(opts.get("g_factor", 2.0)), "sia": bool(opts.get("sia", False))}
    return fix


def sweep_cases():
    pyro = eg.pyrochlore(3, shells=(2.97243, 5.1484), tol=1e-3)
    axes = eg.local_111_axes(pyro)
    sia_local = np.concatenate([axes, np.full((pyro.N, 1), -0.2e-3)], axis=1)
    return {
        # odd sides: no Checkerboard two-colouring, the general (ELL) Ising kernel
        "sc3_ising_zeeman": base(eg.simple_cubic(3), golden.MODEL_ISING, FM, [3.5, 4.5, 6.0], [0, 5, 11],
                                 [["metro", 6]], 1, zeeman=True, h=(0.0, 0.0, 0.5), g_factor=2.0),
        # the simple-cubic fast kernel (4-byte vectors), staggered magnetisation
        "sc8x4x4_ising_staggered": base(eg.simple_cubic((8, 4, 4), checkerboard=True), golden.MODEL_ISING,
                                        AFM, [2.0, 4.5], [3, 4], [["metro", 5]], 2),
        "sc3_xyz_zeeman_sia": base(eg.simple_cubic(3), golden.MODEL_XYZ, FM, [1.0, 2.0], [1, 2],
                                   [["metro", 8]], 3, zeeman=True, h=(0.2, 0.0, 1.0), g_factor=2.0,
                                   sia=True, sia_vec=np.array([[0.0, 0.0, -0.3e-3]])),
        # the simple-cubic fast kernel and overrelaxation (full and partial passes)
        "sc8x6x4_xyz_ovrr": base(eg.simple_cubic((8, 6, 4)), golden.MODEL_XYZ, FM, [1.2, 1.6], [7, 8],
                                 [["metro", 3], ["ovrr", 0.6], ["metro", 2], ["ovrr", 1.0], ["metro", 1]], 4),
        # two shells, ANGLE proposals, Zeeman, anisotropy about each site's local <111> axis
        "pyro3_xyz_angle_local_sia": base(pyro, golden.MODEL_XYZ, J1J2, [0.2, 2.0], [0, 1], [["metro", 4]], 5,
                                          angle=True, dphi=0.6, zeeman=True, h=(0.0, 0.0, 1.0),
                                          g_factor=2.0, sia_local=sia_local),
        "pyro3_ising_j1j2": base(pyro, golden.MODEL_ISING, [[(1, 1, (-1.0, -1.0, -1.0))], [(1, 1, (-0.1,) * 3)]],
                                 [0.5, 5.0], [2, 9], [["metro", 4]], 6, zeeman=True, h=(0.0, 0.0, 1.0),
                                 g_factor=2.0),
    }


def sq_cases():
    lat = eg.pyrochlore(2)
    out = {}
    for name, model in (("pyro2_sq_xyz", golden.MODEL_XYZ), ("pyro2_sq_ising", golden.MODEL_ISING)):
        fix = base(lat, model, FM, [1.0, 1.0], [0, 1], [], 7 + model)
        sp = fix.pop("spins0")
        fix["S"] = sp[:, :, 1:4] if model == golden.MODEL_XYZ else np.stack(
            [0 * sp[:, :, 3], 0 * sp[:, :, 3], sp[:, :, 3]], axis=2)
        fix["abc"] = np.eye(3) * eg.model.PYROCHLORE_A
        fix["meta"].update(nq=[64, 2, 2], q0=[-1.0, -1.0, -1.0], dq=[2.0 / 64, 1.0, 1.0])
        out[name] = fix
    return out


def main():
    for name, fix in sweep_cases().items():
        fix.update(golden.oracle_sweeps(fix))
        golden.save(name, fix)
        print("wrote", golden.path(name))
    for name, fix in sq_cases().items():
        fix.update(golden.oracle_sq(fix))
        golden.save(name, fix)
        print("wrote", golden.path(name))


if __name__ == "__main__":
    main()
