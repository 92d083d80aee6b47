#!/usr/bin/env python
"""Benchmark of ETHER's Monte Carlo sweep on one GB300.

Headline (metric "spin updates/ns"): plain Checkerboard Metropolis sweeps of the 64^3
simple-cubic Ising model at k_B T_c = 4.511 J (J = 1 meV, ferromagnetic, periodic), a batch of
R = 1024 independent replicas (each its own Philox stream) so the int8 state (268 MB) is
larger than the 129 MB L2.  A step is one full sweep (both colour phases) of every replica.

  value        spin updates / ns over the timed steps (state resident in HBM, CUDA events)
  e2e          the same sweeps through the C-ABI with host buffers: every replica's
               configuration in the reference's ion(0:8, N) layout uploaded before the sweeps
               (ether_set_spins_batch), the acceptance ratios of all replicas returned to the
               host every step (the reference's Metropolis(beta, accept) boundary), every
               replica read back after the last sweep (ether_get_spins_batch)
  roofline     the dominant kernel (one colour phase) at 3 algorithmic bytes per update
  cpu_baseline the oracle's typewriter restatement of src/Metropolis.f90 + get_tot_energy per
               MCS (what src/ether.f90:172-177 does), one replica per host core, built with
               the reference's optimisation flags

components (same JSON line): the 64^3 Heisenberg sweep (48 B per update), the structure
factor on the tensor cores at the pyrochlore size (16-site cell x 12^3 = 27648 sites, 64
replicas, 64^3 q-grid), and tau_int(|M|) at T_c with the independent samples per second it
implies.

--impl reference times the oracle's CPU restatement on all host cores (the Fortran reference
cannot be built: no gfortran / MPI on this image or the GPU machine); that arm never loads the
product library.
--model sq times only the structure factor (for profiling); --model batch-mcs only the
batched MCS loop of the 256-chain mix (ether_batch_mcs; --batch-config fixes the tiles).
--model program times the whole program (ether_run) on a deck (--deck): the 16^3 Ising deck
(19 temperatures x 10 REPEATs x 5000 MCS) or the 32^3 Heisenberg + overrelaxation deck (29
temperatures x 10 REPEATs x 20000 MCS): deck read, lattice, MCS loop with measurements, and
every output file written.
"""
import argparse
import ctypes as C
import ctypes.util
import json
import os
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

J_MEV = 1.0
KTC_ISING = 4.511      # k_B T_c / J, 3D simple-cubic Ising
KTC_HEIS = 1.443       # k_B T_c / J, 3D simple-cubic classical Heisenberg
BYTES_ISING = 3.0      # algorithmic bytes per int8 site update (read own, write own, read neighbours)
BYTES_HEIS = 48.0      # float4: 16 read own + 16 write own + 16 neighbours
MODEL_ISING, MODEL_XYZ = 0, 1   # ETHER_MODEL_ISING / ETHER_MODEL_XYZ


def _cudart():
    for name in ("libcudart.so.13", "libcudart.so", ctypes.util.find_library("cudart")):
        if not name:
            continue
        try:
            return C.CDLL(name)
        except OSError:
            pass
    raise RuntimeError("libcudart not found")


class Events:
    def __init__(self, stream):
        self.rt = _cudart()
        self.stream = C.c_void_p(stream)

    def record(self):
        ev = C.c_void_p()
        assert self.rt.cudaEventCreate(C.byref(ev)) == 0
        assert self.rt.cudaEventRecord(ev, self.stream) == 0
        return ev

    def ms(self, a, b):
        self.rt.cudaEventSynchronize(b)
        t = C.c_float()
        assert self.rt.cudaEventElapsedTime(C.byref(t), a, b) == 0
        return t.value

    def free(self, evs):
        for e in evs:
            self.rt.cudaEventDestroy(e)


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during a timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu=0):
        self.gpu = gpu
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except ValueError:
                continue
            for nm, v in zip(names, r[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(mx)) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def make_workload(model, L, replicas, seed=1992, flags=0):
    import ether_gb300 as eg
    lat = eg.simple_cubic(L)
    j = eg.couplings(1, [[(1, 1, (-J_MEV, -J_MEV, -J_MEV))]], [1.0])
    sw = eg.Sweep.from_lattice(lat, j, np.array([1.0]), model, replicas=replicas, seed=seed, flags=flags)
    ktc = KTC_ISING if model == eg.MODEL_ISING else KTC_HEIS
    beta = 1.0 / (ktc * J_MEV * 1e-3)
    sw.set_beta(beta)
    rng = np.random.default_rng(seed)
    ion = lat.ion.copy()
    if model == eg.MODEL_ISING:
        ion[:, 3] = rng.choice([-1.0, 1.0], size=lat.N)  # uniform random initial
    else:
        v = rng.normal(size=(lat.N, 3))
        ion[:, 1:4] = v / np.linalg.norm(v, axis=1, keepdims=True)
    return lat, j, sw, ion, beta


def run_sweeps(model, L, replicas, steps, warmup, rank, world, force_variant=0, clocks=True,
               e2e=True, flags=0):
    import ether_gb300 as eg
    lat, j, sw, ion, beta = make_workload(model, L, replicas, seed=1992 + 7919 * rank, flags=flags)
    sw.set_spins(ion)
    if force_variant:
        sw.set_variant(force_variant)
        variant = force_variant
    else:
        variant, _ = sw.autotune()
    N, R = lat.N, replicas
    ev = Events(sw.stream())
    for _ in range(warmup):
        sw.metropolis(1, accept=False)
    sw.sync()
    _barrier(world)
    launches0 = sw.info().kernel_launches
    sampler = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")) if world > 1 else 0)
    if clocks:
        sampler.start()
        time.sleep(0.3)
    marks = []
    t0 = ev.record()
    for _ in range(steps):
        a = ev.record()
        sw.phase(0)
        b = ev.record()
        sw.phase(1)
        c = ev.record()
        sw.end_sweep()
        marks.append((a, b, c))
    t1 = ev.record()
    sw.sync()
    total_ms = ev.ms(t0, t1)
    phase_ms = [ev.ms(a, b) for a, b, c in marks] + [ev.ms(b, c) for a, b, c in marks]
    clk = sampler.stop() if clocks else None
    launches = sw.info().kernel_launches - launches0
    ev.free([t0, t1] + [e for m in marks for e in m])
    _barrier(world)
    total_ms = _max_over_ranks(total_ms, world)
    updates = float(N) * R * steps
    value = updates / (total_ms * 1e6) * world
    bpu = BYTES_ISING if model == eg.MODEL_ISING else BYTES_HEIS
    phase_avg_ms = float(np.mean(phase_ms))
    achieved_gbs = bpu * (R * N / 2.0) / (phase_avg_ms * 1e-3) / 1e9
    res = {"value": value, "ms_per_step": total_ms / steps, "phase_ms": phase_avg_ms,
           "achieved_gbs": achieved_gbs, "bytes_per_update": bpu, "launches": int(launches),
           "clocks": clk, "variant": variant}
    if e2e:
        # every replica's configuration as the reference holds it, ion(0:8, N) per replica
        # (72 B per site), uploaded before the sweeps and read back after them through the
        # C-ABI; the acceptance ratios of all replicas come back to the host every sweep
        ions = np.empty((R, N, 9))
        ions[:] = ion
        # untimed rounds: the first allocates the pinned staging area and the copy stream (where
        # the records can also move in place, each call shares its replicas between the kernel
        # and the host's cores as it runs)
        for _ in range(3):
            sw.set_spins_batch(ions)
            sw.get_spins_batch(ions)
        sw.sync()
        acc = None
        t_start = time.perf_counter()
        sw.set_spins_batch(ions)
        t_set = time.perf_counter()
        for _ in range(steps):
            acc = sw.metropolis(1, accept=True)   # D2H of R doubles every step
        t_run = time.perf_counter()
        sw.get_spins_batch(ions)
        t_end = time.perf_counter()
        t_e2e = t_end - t_start
        # bytes that cross the link per site: the spin fields of the records for the replicas a
        # kernel moved in place (ion(3) as FP64; ion(1:3), ion(5)), the device layout for those
        # the host's cores staged (the timed calls' split, from the library)
        direct = sw.info().ion_direct
        dsize = 1 if model == eg.MODEL_ISING else 16
        fsize = 8 if model == eg.MODEL_ISING else 32
        k_get, k_set = sw.spins_batch_split() if direct else (0, 0)
        up = k_set * N * fsize + (R - k_set) * N * dsize
        down = k_get * N * fsize + (R - k_get) * N * dsize
        res.update({"e2e": updates / (t_e2e * 1e9) * world,
                    "h2d": up / steps,   # every replica, once per timed run
                    "d2h": 8.0 * R + down / steps,
                    "e2e_detail": {"steps": steps, "records": ("replicas moved in place by a kernel (the rest staged "
                                   "on the host's cores): upload %d, read-back %d of %d" % (k_set, k_get, R))
                                   if direct else "converted on the host's cores through pinned staging",
                                   "set_spins_batch_s": t_set - t_start,
                                   "sweeps_s": t_run - t_set, "get_spins_batch_s": t_end - t_run,
                                   "host_ion_bytes": R * N * 72},
                    "accept_mean": float(np.mean(acc))})
        del ions
    sw.close()
    return res


def run_sq(cells=12, replicas=64, M=64, calls=3, warmup=1, model=MODEL_XYZ):
    """Structure factor of `replicas` pyrochlore configurations (16-site cell x cells^3) on an
    M^3 q-grid; the fastest kernel time and the tensor throughput.  Useful FLOPs: 2 (cos, sin)
    x 2 x Q x N per spin component (three for Heisenberg, one for Ising); tensor FLOPs: the
    BF16 products issued (three per useful product for Heisenberg, two for Ising, whose
    B_lo is zero)."""
    import ether_gb300 as eg
    from ether_gb300 import abi
    lat = eg.pyrochlore(cells)
    j = eg.couplings(1, [[(1, 1, (1.0, 1.0, 1.0))]], [1.0])
    sw = eg.Sweep.from_lattice(lat, j, np.array([1.0]), model, replicas=replicas)
    rng = np.random.default_rng(0)
    ion = lat.ion.copy()
    if model == MODEL_XYZ:
        v = rng.normal(size=(lat.N, 3))
        ion[:, 1:4] = v / np.linalg.norm(v, axis=1, keepdims=True)
    else:
        ion[:, 3] = rng.choice([-1.0, 1.0], size=lat.N)
    sw.set_spins(ion)
    nq = np.array([M, M, M], dtype=np.int32)
    Q = M ** 3
    sq = np.zeros(replicas * Q, np.float32)
    comp = np.zeros(replicas * Q * 3, np.float32)
    abc = (np.eye(3) * eg.model.PYROCHLORE_A).ravel()
    q0 = np.array([-1.0, -1.0, -1.0])
    dq = np.array([2.0 / M] * 3)
    times = []
    for it in range(warmup + calls):
        abi.check(sw.lib.ether_structure_factor(
            sw.h, abi.dptr(abc), abi.iptr(nq), abi.dptr(q0), abi.dptr(dq),
            sq.ctypes.data_as(C.POINTER(C.c_float)), comp.ctypes.data_as(C.POINTER(C.c_float))))
        if it >= warmup:
            times.append(sw.info().sq_kernel_ms)
    ms = min(times)
    comps, products = (3, 3) if model == MODEL_XYZ else (1, 2)
    useful = 2.0 * (2 * Q) * (comps * replicas) * lat.N
    sw.close()
    return {"model": "Heisenberg" if model == MODEL_XYZ else "Ising", "sites": lat.N,
            "replicas": replicas, "q_points": Q, "kernel_ms": ms,
            "tensor_tflops": products * useful / ms / 1e9, "useful_tflops": useful / ms / 1e9}


def run_tau(L=64, replicas=1024, equil=20000, sweeps=100000, stride=10):
    """tau_int(|M|) of the plain Checkerboard sweep at T_c, and the independent samples/s, on
    the headline's 1024 replicas (|M| of every replica recorded every `stride` sweeps)."""
    import ether_gb300 as eg
    from ether_gb300.analysis import tau_int
    lat, j, sw, ion, beta = make_workload(eg.MODEL_ISING, L, replicas, seed=4242)
    sw.set_spins(ion)
    sw.autotune()
    sw.metropolis(equil, accept=False)
    sw.sync()
    t = time.perf_counter()
    m = sw.record_series(sweeps, stride=stride)
    dt = time.perf_counter() - t
    tau, err, W = tau_int(m)
    tau_sweeps = tau * stride
    sweeps_per_s = sweeps / dt
    sw.close()
    return {"L": L, "replicas": replicas, "equilibration_sweeps": equil, "measured_sweeps": sweeps,
            "stride": stride, "tau_int_absM_sweeps": tau_sweeps, "tau_err_sweeps": err * stride,
            "window": W, "sweeps_per_s_per_replica": sweeps_per_s,
            "independent_samples_per_s": replicas * sweeps_per_s / (2.0 * tau_sweeps)}


BATCH_SIZES = (8, 12, 16, 24, 32, 48)


def make_batch_members(chains=256, ladder=32, seed=1992, grouped=True, mix="mixed", sizes=None):
    """Mixed batch: `chains` chains with L drawn uniformly from BATCH_SIZES, half Ising and
    half Heisenberg (mix "mixed"; "ising" or "heisenberg": all of one model), J = +-1 meV per
    chain, a `ladder`-temperature geometric ladder each (0.6 .. 1.6 T_c); `sizes` replaces
    BATCH_SIZES.  grouped: chains with the same (model, L, J) share one context, one ladder
    group per chain; else one context per chain."""
    import ether_gb300 as eg
    rng = np.random.default_rng(seed)
    groups = {}
    keys = []
    for c in range(chains):
        ising = c < chains // 2 if mix == "mixed" else mix == "ising"
        model = eg.MODEL_ISING if ising else eg.MODEL_XYZ
        key = (model, int(rng.choice(sizes or BATCH_SIZES)), int(rng.choice([-1, 1])))
        groups[key] = groups.get(key, 0) + 1
        keys.append(key)
    items = sorted(groups.items()) if grouped else [(k, 1) for k in keys]
    members = []
    for k, ((model, L, sign), n) in enumerate(items):
        lat = eg.simple_cubic(L)
        j = eg.couplings(1, [[(1, 1, (sign * J_MEV,) * 3)]], [1.0])
        sw = eg.Sweep.from_lattice(lat, j, np.array([1.0]), model, replicas=ladder * n,
                                   seed=seed + 101 * k)
        ktc = KTC_ISING if model == eg.MODEL_ISING else KTC_HEIS
        kT = ktc * np.geomspace(0.6, 1.6, ladder)
        sw.set_ladder(1.0 / (kT * J_MEV * 1e-3))
        ion = lat.ion.copy()
        if model == eg.MODEL_ISING:
            ion[:, 3] = rng.choice([-1.0, 1.0], size=lat.N)
        else:
            v = rng.normal(size=(lat.N, 3))
            ion[:, 1:4] = v / np.linalg.norm(v, axis=1, keepdims=True)
        sw.set_spins(ion)
        members.append(sw)
    return members, groups


def _time_batch(members, steps, warmup, config=None):
    import ether_gb300 as eg
    b = eg.Batch(members)
    if config:
        b.set_config(*config)
        cfg = tuple(config)
    else:
        cfg, _ = b.autotune()
    b.metropolis(warmup)
    ev = Events(b.stream())
    t0 = ev.record()
    b.metropolis(steps)
    t1 = ev.record()
    ms = ev.ms(t0, t1)
    info = b.info()
    ev.free([t0, t1])
    b.close()
    return ms, info, cfg


# the MCS-loop comparison's schedule: overrelaxation (exchange-only Heisenberg members) and PT
# every 5 steps, a measurement every 10
MCS_SCHEDULE = dict(tmcs_eq=0, coa=10, ovrr=True, ovrr_para=1.0, ovrr_mcs=5, pt=True,
                    exchange_interval=5)


def _time_batch_mcs(members, steps, config):
    """Wall time per MCS step of the whole loop body (OVRR, sweep, PT, measurement) for every
    member: one ether_batch_mcs call, against each member's own ether_mcs in turn.  The
    warm-up is one period of the schedule's gates and the timed steps whole periods, so the
    timed calls replay graphs captured in the warm-up."""
    import ether_gb300 as eg
    warmup = MCS_SCHEDULE["coa"]
    steps = max(1, steps // warmup) * warmup
    b = eg.Batch(members)
    b.set_config(*config)
    sc = b.mcs(0, warmup, **MCS_SCHEDULE)
    t = time.perf_counter()
    b.mcs(warmup, steps, swap_counts=sc, **MCS_SCHEDULE)   # synchronous: swap counters read back
    batch_s = time.perf_counter() - t
    event_ms = b.info().last_sweep_ms
    b.close()
    n0 = warmup + steps
    sc = [m.mcs(n0, warmup, **MCS_SCHEDULE) for m in members]
    t = time.perf_counter()
    for m, s0 in zip(members, sc):
        m.mcs(n0 + warmup, steps, swap_count=int(s0), **MCS_SCHEDULE)
    own_s = time.perf_counter() - t
    return {"schedule": MCS_SCHEDULE, "steps": steps,
            "batch_ms_per_step": batch_s * 1e3 / steps, "batch_event_ms_per_step": event_ms,
            "own_ms_per_step": own_s * 1e3 / steps, "speedup": own_s / batch_s}


def _time_plain(members, steps, warmup):
    for m in members:
        m.metropolis(warmup, accept=False)
    for m in members:
        m.sync()
    t = time.perf_counter()
    for _ in range(steps):
        for m in members:
            m.metropolis(1, accept=False)
    for m in members:
        m.sync()
    return time.perf_counter() - t


def run_batch(steps=200, warmup=5, chains=256, ladder=32, config=None, forms=(False, True),
              plain=True, mix="mixed", sizes=None):
    """The mixed batch advanced by ether_batch (one kernel per member group, colour phase and
    member class, one graph per sweep, autotuned tiles) and by each member's own sweeps (per-context kernels
    on the members' streams), with one context per chain and with chains grouped by
    (model, L, J)."""
    import ether_gb300 as eg
    out = {}
    for grouped in forms:
        t = time.perf_counter()
        members, groups = make_batch_members(chains, ladder, grouped=grouped, mix=mix, sizes=sizes)
        setup_s = time.perf_counter() - t
        ms, info, cfg = _time_batch(members, steps, warmup, config)
        updates = float(info.site_updates_per_sweep) * steps
        n_ising = sum(m.N * m.R for m in members if m.model == eg.MODEL_ISING)
        n_heis = sum(m.N * m.R for m in members if m.model == eg.MODEL_XYZ)
        bytes_per_sweep = BYTES_ISING * n_ising + BYTES_HEIS * n_heis
        plain_steps = max(5, steps // 4)
        plain_s = _time_plain(members, plain_steps, warmup) if plain else float("nan")
        res = {"contexts": len(members), "setup_s": setup_s,
               "value": updates / (ms * 1e6), "ms_per_sweep": ms / steps,
               "tile_config": list(cfg), "kernels_per_sweep": info.kernels_per_sweep,
               "segments": info.n_segments, "grid": info.grid,
               "achieved_gbs": bytes_per_sweep / (ms / steps * 1e-3) / 1e9,
               "plain_value": float(info.site_updates_per_sweep) * plain_steps / (plain_s * 1e9),
               "plain_kernels_per_sweep": 3 * len(members)}
        res["speedup_vs_plain"] = res["value"] / res["plain_value"]
        if plain and not grouped:
            res["mcs"] = _time_batch_mcs(members, max(20, steps // 4), cfg)
        out["grouped" if grouped else "per_chain"] = res
        for m in members:
            m.close()
    pc = out["per_chain"] if "per_chain" in out else out["grouped"]
    n_ising = {"mixed": chains // 2, "ising": chains, "heisenberg": 0}[mix]
    return {"workload": "%d chains, L ~ U%s, %d Ising + %d Heisenberg, J = +-1 meV, %d-T "
                        "geometric ladder (0.6-1.6 T_c) each: %d replicas, %.3g spins"
                        % (chains, list(sizes or BATCH_SIZES), n_ising, chains - n_ising, ladder,
                           info.n_replicas, info.site_updates_per_sweep),
            "value": pc["value"], "unit": "spin updates/ns", "achieved_gbs": pc["achieved_gbs"],
            "plain_note": "plain = each context's own ether_metropolis per sweep on its own "
                          "stream (wall clock, host-synchronised)",
            **out}


def run_learned(L=64, R=256, train_steps=3000, n_plain=40000, n_learn=20000, heisenberg=False, stride=10):
    """Learned 4^3-patch proposal at T_c of the L^3 Ising (or Heisenberg) model: trained on
    plain-sweep configurations of an 8-temperature ladder (0.9 .. 1.1 T_c), then tau_int(|M|)
    and the independent samples per second of (a) plain sweeps, (b) plain + learned sweep per
    step, (c) learned sweeps alone, all with R replicas at T_c.  |M| is recorded every
    `stride` steps in all three chains (as a production run measures every COA steps), so the
    recording adds the same small cost per step to each and tau is converted to steps."""
    import ether_gb300 as eg
    from ether_gb300.analysis import tau_int
    lat = eg.simple_cubic(L)
    j = eg.couplings(1, [[(1, 1, (-J_MEV, -J_MEV, -J_MEV))]], [1.0])
    model = eg.MODEL_XYZ if heisenberg else eg.MODEL_ISING
    sw = eg.Sweep.from_lattice(lat, j, np.array([1.0]), model, replicas=R, seed=31)
    ktc = (KTC_HEIS if heisenberg else KTC_ISING) * J_MEV * 1e-3
    sw.set_beta(1.0 / (np.repeat(ktc * np.linspace(0.9, 1.1, 8), R // 8)))
    rng = np.random.default_rng(7)
    ion = lat.ion.copy()
    if heisenberg:
        v = rng.normal(size=(lat.N, 3))
        ion[:, 1:4] = v / np.linalg.norm(v, axis=1, keepdims=True)
    else:
        ion[:, 3] = rng.choice([-1.0, 1.0], size=lat.N)
    sw.set_spins(ion)
    sw.metropolis(2000, accept=False)
    lr = eg.Learned(sw, seed=5, capacity=1 << 21)
    for _ in range(40):
        sw.metropolis(20, accept=False)
        lr.collect((L // 4) ** 3 // 4)
    loss = lr.train(train_steps, batch=1024, lr=1e-3)
    train_ms = lr.info().last_train_ms
    sw.set_beta([1.0 / ktc] * R)
    sw.metropolis(5000, accept=False)
    sw.autotune()  # the plain sweeps below run the fastest kernel variant
    sw.sync()

    def series(n, plain, learned):
        t = time.perf_counter()
        out = lr.record_series(n, 1 if plain else 0, 1 if learned else 0, stride=stride)
        return out, time.perf_counter() - t

    t = time.perf_counter()
    m_plain = sw.record_series(n_plain, stride=stride)
    s_plain = time.perf_counter() - t
    a0, p0 = lr.accepts().sum(), lr.info().proposed
    m_both, s_both = series(n_learn, True, True)
    m_learn, s_learn = series(n_learn, False, True)
    acc = (lr.accepts().sum() - a0) / max(1, lr.info().proposed - p0)
    lr.sweep_(20)
    sweep_ms = lr.info().last_sweep_ms
    res = {"workload": "learned 4^3-patch proposal, %d^3 %s at T_c, %d replicas"
                       % (L, "Heisenberg" if heisenberg else "Ising", R),
           "train_steps": train_steps, "final_loss": loss, "train_ms": train_ms,
           "acceptance_at_tc": acc, "learned_sweep_ms": sweep_ms, "record_stride_steps": stride}
    for name, m, n, secs in (("plain", m_plain, n_plain, s_plain), ("plain_plus_learned", m_both, n_learn, s_both),
                             ("learned_only", m_learn, n_learn, s_learn)):
        tau, err, W = tau_int(m)
        tau, err = tau * stride, err * stride
        res[name] = {"tau_int_absM_steps": tau, "tau_err": err, "steps": n,
                     "steps_per_s": n / secs,
                     "independent_samples_per_s": R * n / secs / (2.0 * tau)}
    base = res["plain"]["independent_samples_per_s"]
    for name in ("plain_plus_learned", "learned_only"):
        res[name]["gain_vs_plain"] = res[name]["independent_samples_per_s"] / base
    lr.close()
    sw.close()
    return res


def run_learned_sweep(L=64, R=256, sweeps=3, heisenberg=False):
    """Time of the learned sweep alone (untrained network, T_c): the profiling case."""
    import ether_gb300 as eg
    lat = eg.simple_cubic(L)
    j = eg.couplings(1, [[(1, 1, (-J_MEV, -J_MEV, -J_MEV))]], [1.0])
    model = eg.MODEL_XYZ if heisenberg else eg.MODEL_ISING
    sw = eg.Sweep.from_lattice(lat, j, np.array([1.0]), model, replicas=R, seed=31)
    sw.set_beta(1.0 / ((KTC_HEIS if heisenberg else KTC_ISING) * J_MEV * 1e-3))
    rng = np.random.default_rng(7)
    ion = lat.ion.copy()
    if heisenberg:
        v = rng.normal(size=(lat.N, 3))
        ion[:, 1:4] = v / np.linalg.norm(v, axis=1, keepdims=True)
    else:
        ion[:, 3] = rng.choice([-1.0, 1.0], size=lat.N)
    sw.set_spins(ion)
    lr = eg.Learned(sw, seed=5, capacity=4096)
    sw.metropolis(10, accept=False)
    lr.sweep_(1)  # warm-up: first launches and library loading stay out of the timed sweeps
    sw.sync()
    lr.sweep_(sweeps)
    sw.sync()
    res = {"L": L, "replicas": R, "learned_sweep_ms": lr.info().last_sweep_ms,
           "acceptance": float(lr.accepts().sum() / lr.info().proposed)}
    lr.close()
    sw.close()
    return res


PROGRAM_STRUCT = ("simple cubic\n1.0\n 1.0 0.0 0.0\n 0.0 1.0 0.0\n 0.0 0.0 1.0\n A\n 1\n"
                  "Direct\n 0.0 0.0 0.0\n")
PROGRAM_J = "1\n1.0 1\nA A -1.0 -1.0 -1.0\n"
# the simple-cubic decks of the benchmark's configurations (J = 1 meV ferromagnetic)
PROGRAM_DECKS = {
    "c1_ising_16": ("simple-cubic 16^3 Ising, 19 T (100..10 K) x 10 REPEAT x 5000 MCS (3000 "
                    "equilibration), coa 10, Checkerboard staggered signs",
                    "model = ising\nmcs = 5000 3000\ntemp = 100 10 5\nspin = 1\nspecies = A\n"
                    "sc = 16 16 16\nbc = c c c\nrepeat = 10\ncoa = 10\nseed = 1992\ncb = .T.\n"),
    "c2_heisenberg_32": ("simple-cubic 32^3 Heisenberg + overrelaxation every 5 MCS (one pass), "
                         "29 T (150..10 K) x 10 REPEAT x 20000 MCS (10000 equilibration), coa 10",
                         "model = xyz\nmcs = 20000 10000\ntemp = 150 10 5\nspin = 1\nspecies = A\n"
                         "sc = 32 32 32\nbc = c c c\nrepeat = 10\ncoa = 10\nseed = 1992\n"
                         "ovrr = .T. 1.0 5\n"),
}


def run_program(deck="c1_ising_16", repeats=2):
    """ether_run end to end on one of PROGRAM_DECKS: wall time from the deck on disk to the
    last output file, and the MCS loop alone (best of `repeats` runs; the first also pays
    the library's one-time set-up)."""
    import ether_gb300 as eg
    what, text = PROGRAM_DECKS[deck]
    work = tempfile.mkdtemp(prefix="ether_run_")
    indir = os.path.join(work, "deck")
    os.makedirs(indir)
    for name, body in (("in.ether", text), ("structure.vasp", PROGRAM_STRUCT),
                       ("j_exchange", PROGRAM_J)):
        with open(os.path.join(indir, name), "w") as f:
            f.write(body)
    best = None
    for k in range(repeats):
        t0 = time.perf_counter()
        info = eg.run(indir, os.path.join(work, "out%d" % k))
        wall = time.perf_counter() - t0
        if best is None or wall < best[0]:
            best = (wall, info)
    wall, info = best
    ups = info["site_updates"]
    return {"workload": "ether_run: " + what + ", every output file", "site_updates": ups,
            "wall_s": wall, "mcs_loop_s": info["seconds"],
            "updates_per_ns_wall": ups / wall / 1e9, "updates_per_ns_loop": ups / info["seconds"] / 1e9}


def run_pyrochlore_pt(cells=12, replicas=64, mcs=2000, warmup=50, ising=False):
    """The frustrated Heisenberg configuration: pyrochlore 16-site cell x 12^3 (27648 sites),
    J1 = +1 meV (antiferromagnetic in ETHER's sign) and J2 = -0.1 meV, easy-axis single-ion
    anisotropy D = -0.2 meV along each site's local <111> axis (sia_local; the reference's
    anisotropy is diagonal per species and cannot express it), Zeeman H = (0, 0, 1) T with
    g = 2, 64 replicas on a geometric 1-50 K ladder, PT every 11 MCS,
    measured every 10 MCS: ether_mcs timed with CUDA events.  ising: the same lattice, ladder
    and schedule for the Ising model (J1 = -1 meV, ferromagnetic as the reference's pyrochlore
    example, and J2; Zeeman field, no anisotropy)."""
    import ether_gb300 as eg
    lat = eg.pyrochlore(cells, shells=(2.97243, 5.1484), tol=1e-3)
    if ising:
        j = eg.couplings(1, [[(1, 1, (-1.0, -1.0, -1.0))], [(1, 1, (-0.1, -0.1, -0.1))]], [1.0])
        sw = eg.Sweep.from_lattice(lat, j, np.array([1.0]), eg.MODEL_ISING, replicas=replicas,
                                   seed=1992, zeeman=True, h=(0.0, 0.0, 1.0), g_factor=2.0)
    else:
        j = eg.couplings(1, [[(1, 1, (1.0, 1.0, 1.0))], [(1, 1, (-0.1, -0.1, -0.1))]], [1.0])
        sia_local = np.concatenate([eg.local_111_axes(lat), np.full((lat.N, 1), -0.2e-3)], axis=1)
        sw = eg.Sweep.from_lattice(lat, j, np.array([1.0]), eg.MODEL_XYZ, replicas=replicas, seed=1992,
                                   zeeman=True, h=(0.0, 0.0, 1.0), g_factor=2.0, sia_local=sia_local)
    temps = np.geomspace(1.0, 50.0, replicas)
    sw.set_ladder(1.0 / (eg.KB_EV * temps))
    sw.set_spins(lat.ion)
    sw.fresh_spins()
    sw.zero_avg()
    swaps = sw.mcs(0, warmup, 10 ** 9, 10, pt=True, exchange_interval=11)
    sw.sync()
    ev = Events(sw.stream())
    t0 = ev.record()
    sw.mcs(warmup, mcs, warmup, 10, pt=True, exchange_interval=11, swap_count=swaps)
    t1 = ev.record()
    sw.sync()
    ms = ev.ms(t0, t1)
    ev.free([t0, t1])
    ups = float(lat.N) * replicas * mcs
    info = sw.info()
    sw.close()
    return {"workload": "pyrochlore 16 x %d^3 = %d sites, %s, 64-replica geometric ladder 1-50 K, "
                        "PT every 11 MCS, ether_mcs" % (cells, lat.N, "Ising, J1/J2, Zeeman" if ising
                                                         else "Heisenberg, J1/J2, local <111> SIA, Zeeman"),
            "mcs": mcs, "ms": ms, "value": ups / (ms * 1e6), "unit": "spin updates/ns",
            "n_colours": info.n_colours}


def cpu_reference(model, L, mcs, threads, seed=1992, steps=1, warmup=0):
    """The oracle's typewriter restatement of the reference's per-MCS work (Metropolis
    + get_tot_energy), one replica (temperature) per thread, built with the reference's
    optimisation flags.  Lattice and couplings come from the oracle's own builders: this arm
    does not load the product library.  Each step is one bounded sample (`threads` replicas x
    `mcs` MCS from the initial state); `warmup` untimed steps, then `steps` timed ones."""
    from oracle import pyoracle as po
    lat = po.ScLattice(L)
    j = po.sc_couplings((-J_MEV, -J_MEV, -J_MEV))
    osys = po.System.from_lattice(lat, j, np.array([1.0]), model)
    ktc = KTC_ISING if model == MODEL_ISING else KTC_HEIS
    beta = 1.0 / (ktc * J_MEV * 1e-3)
    cfg = po.RunCfg(tmcs=mcs, tmcs_eq=mcs, coa=1 << 30, repeat=1, ovrr=0, ovrr_para=0.0,
                    ovrr_mcs=0, seed=seed, itemp=1, rank=0)
    nT = threads
    vals = np.zeros(6 * nT)
    acc = np.zeros(nT)
    b = np.full(nT, beta)
    times = []
    for k in range(warmup + steps):
        t = time.perf_counter()
        po.timed_lib().orc_run_temperatures(osys.p(), osys.ion0.ctypes.data_as(po.PD), nT,
                                            b.ctypes.data_as(po.PD), C.byref(cfg), threads,
                                            vals.ctypes.data_as(po.PD), acc.ctypes.data_as(po.PD))
        if k >= warmup:
            times.append(time.perf_counter() - t)
    dt = float(np.sum(times))
    updates = float(lat.N) * mcs * nT * steps
    return {"value": updates / (dt * 1e9), "unit": "spin updates/ns", "cores": threads,
            "kind": "port", "ms_per_step": 1e3 * dt / steps,
            "sample": "%d step(s) of %d replicas x %d MCS of %d^3 %s, typewriter order, FP64, per-MCS "
                      "get_tot_energy as src/ether.f90:177, built -O3 -fopenmp -funroll-loops "
                      "-finline-functions -fno-math-errno -fno-trapping-math (%.1f s timed)" %
                      (steps, nT, mcs, L, "Ising" if model == 0 else "Heisenberg", dt),
            "seconds": dt}


def _barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def _max_over_ranks(x, world):
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        return {}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--model", default="ising",
                    choices=["ising", "heisenberg", "sq", "sq-ising", "batch", "batch-mcs", "learned",
                             "learned-heisenberg", "learned-sweep",
                             "learned-sweep-heisenberg",
                             "program", "pyrochlore", "pyrochlore-ising"])
    ap.add_argument("--L", type=int, default=64)
    ap.add_argument("--replicas", type=int, default=0)
    ap.add_argument("--cpu-mcs", type=int, default=0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-components", action="store_true")
    ap.add_argument("--variant", type=int, default=0)
    ap.add_argument("--staged-spins", action="store_true",
                    help="e2e: the records converted on the host's cores through pinned staging "
                         "(ETHER_FLAG_STAGED_SPINS) instead of moved in place by kernels")
    ap.add_argument("--learn-steps", type=int, default=0,
                    help="--model learned / learned-heisenberg: Adam steps (default 3000 / 4000)")
    ap.add_argument("--sq-cells", type=int, default=12)
    ap.add_argument("--chains", type=int, default=256)
    ap.add_argument("--mcs-parts", action="store_true",
                    help="batch-mcs: also time the loop with parts of the schedule switched off")
    ap.add_argument("--deck", default="c1_ising_16", choices=sorted(PROGRAM_DECKS))
    ap.add_argument("--batch-mix", default="mixed", choices=["mixed", "ising", "heisenberg"],
                    help="--model batch: half Ising and half Heisenberg chains, or one model only")
    ap.add_argument("--batch-L", default="",
                    help="--model batch: comma-separated lattice sizes to draw L from (default 8..48)")
    ap.add_argument("--batch-config", default="",
                    help="threads,units_per_thread,blocks_per_sm,walk (default: autotune)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        os.environ.setdefault("CUDA_VISIBLE_DEVICES", os.environ.get("LOCAL_RANK", "0"))
        import torch.distributed as dist
        dist.init_process_group("gloo")

    peaks = _peaks()
    hbm_peak = peaks.get("hbm_gbs") or 6800.0
    peak_src = "measured" if peaks.get("hbm_gbs") else "fallback"
    bf16_peak = peaks.get("bf16_tflops") or 1900.0
    cores = os.cpu_count() or 1

    model = MODEL_ISING if args.model == "ising" else MODEL_XYZ
    replicas = args.replicas or (1024 if model == MODEL_ISING else 64)
    workload = ("plain checkerboard Metropolis, simple-cubic %d^3 %s at kT_c=%.3f J "
                "(J=1 meV FM, periodic), %d independent replicas per GPU" %
                (args.L, "Ising int8" if model == 0 else "Heisenberg float4",
                 KTC_ISING if model == 0 else KTC_HEIS, replicas))
    state_mb = args.L ** 3 * replicas * (1 if model == 0 else 16) / 1e6
    config = {"workload": workload, "L": args.L, "replicas": replicas,
              "sites_per_replica": args.L ** 3, "state_MB": round(state_mb, 1),
              "l2_policy": "inputs larger than L2 (%.0f MB > 129 MB)" % state_mb,
              "parallelism": "replicas only (independent chains per GPU)"}

    if args.impl == "reference":
        # the reference's path on the host cores: the product library is never loaded here
        if rank != 0:
            return 0
        # each step a bounded sample: cores replicas x m MCS, m sized so that the whole
        # warm-up + timed run stays within a few minutes of host time
        m = args.cpu_mcs or max(2, min(40, 4000 // (args.steps + args.warmup)))
        ref = cpu_reference(model, args.L, m, cores, steps=args.steps, warmup=args.warmup)
        line = {"metric": "spin updates/ns", "value": ref["value"], "unit": "spin updates/ns",
                "impl": "reference", "n_gpus": args.gpus, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ref["ms_per_step"], "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": config,
                "cpu_baseline": {k: ref[k] for k in ("value", "unit", "cores", "kind", "sample")},
                "e2e": {"value": ref["value"], "unit": "spin updates/ns",
                        "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                "note": "Fortran reference not buildable (no gfortran/MPI): its path restated "
                        "in C (oracle/) and timed on all host cores; a step is one bounded "
                        "sample of the workload (see cpu_baseline.sample)"}
        print(json.dumps(line))
        return 0

    import ether_gb300 as eg

    if args.model in ("sq", "sq-ising"):
        if rank != 0:
            return 0
        r = run_sq(cells=args.sq_cells, replicas=args.replicas or 64, calls=1, warmup=args.warmup,
                   model=MODEL_ISING if args.model == "sq-ising" else MODEL_XYZ)
        print(json.dumps({"metric": "structure factor kernel ms", "value": r["kernel_ms"],
                          "unit": "ms", "higher_is_better": False, "detail": r,
                          "roofline": {"bound": "tensor", "achieved": r["useful_tflops"],
                                       "peak": bf16_peak, "unit": "TFLOP/s",
                                       "frac": r["useful_tflops"] / bf16_peak,
                                       "note": "useful FLOPs (tensor_tflops counts every "
                                               "BF16 split product)"}}))
        return 0

    if args.model == "program":
        if rank != 0:
            return 0
        r = run_program(args.deck)
        print(json.dumps({"metric": "program wall s", "value": r["wall_s"], "unit": "s",
                          "higher_is_better": False, "detail": r}))
        return 0

    if args.model in ("pyrochlore", "pyrochlore-ising"):
        if rank != 0:
            return 0
        r = run_pyrochlore_pt(ising=args.model == "pyrochlore-ising")
        print(json.dumps({"metric": "spin updates/ns", "value": r["value"], "unit": "spin updates/ns",
                          "higher_is_better": True, "detail": r}))
        return 0

    if args.model == "learned-heisenberg":
        if rank != 0:
            return 0
        r = run_learned(args.L, R=64, train_steps=args.learn_steps or 4000, n_plain=60000, n_learn=20000,
                        heisenberg=True)
        print(json.dumps({"metric": "independent samples/s gain", "value": r["learned_only"]["gain_vs_plain"],
                          "unit": "x plain", "higher_is_better": True, "detail": r}))
        return 0

    if args.model in ("learned-sweep", "learned-sweep-heisenberg"):
        if rank != 0:
            return 0
        r = run_learned_sweep(args.L, args.replicas or 256, heisenberg=args.model == "learned-sweep-heisenberg")
        print(json.dumps({"metric": "learned sweep ms", "value": r["learned_sweep_ms"], "unit": "ms",
                          "higher_is_better": False, "detail": r}))
        return 0

    if args.model == "learned":
        if rank != 0:
            return 0
        r = run_learned(args.L, train_steps=args.learn_steps or 3000)
        print(json.dumps({"metric": "independent samples/s gain", "value": r["learned_only"]["gain_vs_plain"],
                          "unit": "x plain", "higher_is_better": True, "detail": r}))
        return 0

    if args.model == "batch-mcs":
        # the whole MCS loop of the mixed batch (one context per chain) through
        # ether_batch_mcs alone: --steps timed steps after --warmup, tiles autotuned or given
        if rank != 0:
            return 0
        import ether_gb300 as eg
        members, _ = make_batch_members(args.chains, 32, grouped=False, mix=args.batch_mix)
        b = eg.Batch(members)
        if args.batch_config:
            b.set_config(*[int(x) for x in args.batch_config.split(",")])
        else:
            b.autotune()
        period = MCS_SCHEDULE["coa"]
        warm = max(1, args.warmup // period) * period
        steps = max(1, args.steps // period) * period
        parts = {}
        if args.mcs_parts:
            # the same loop with parts of the schedule switched off (time per step by parts)
            off = dict(MCS_SCHEDULE, tmcs_eq=10 ** 9, ovrr=False, pt=False)
            step0 = 0
            for name, sch in (("sweeps", off), ("sweeps + measurement every 10", dict(off, tmcs_eq=0)),
                              ("sweeps + PT every 5", dict(off, pt=True)),
                              ("sweeps + overrelaxation every 5", dict(off, ovrr=True))):
                sc0 = b.mcs(step0, warm, **sch)
                t = time.perf_counter()
                b.mcs(step0 + warm, steps, swap_counts=sc0, **sch)
                parts[name] = (time.perf_counter() - t) * 1e3 / steps
                step0 += warm + steps
        sc = b.mcs(0, warm, **MCS_SCHEDULE)
        t = time.perf_counter()
        b.mcs(warm, steps, swap_counts=sc, **MCS_SCHEDULE)
        wall = time.perf_counter() - t
        info = b.info()
        print(json.dumps({"metric": "batch MCS step", "value": wall * 1e3 / steps, "unit": "ms",
                          "higher_is_better": False, "detail": {
                              "contexts": len(members), "replicas": info.n_replicas,
                              "site_updates_per_sweep": info.site_updates_per_sweep,
                              "schedule": MCS_SCHEDULE, "steps": steps, "warmup": warm,
                              "event_ms_per_step": info.last_sweep_ms, "parts_ms_per_step": parts,
                              "tile_config": [info.threads, info.units_per_thread, info.blocks_per_sm, info.walk]}}))
        b.close()
        for m in members:
            m.close()
        return 0

    if args.model == "batch":
        if rank != 0:
            return 0
        cfg = [int(x) for x in args.batch_config.split(",")] if args.batch_config else None
        r = run_batch(steps=min(args.steps, 500), warmup=args.warmup, chains=args.chains,
                      config=cfg, forms=(False,) if cfg else (False, True), plain=not cfg,
                      mix=args.batch_mix,
                      sizes=[int(x) for x in args.batch_L.split(",")] if args.batch_L else None)
        print(json.dumps({"metric": "spin updates/ns", "value": r["value"],
                          "unit": "spin updates/ns", "higher_is_better": True, "detail": r}))
        return 0

    from ether_gb300.abi import FLAG_STAGED_SPINS
    res = run_sweeps(model, args.L, replicas, args.steps, args.warmup, rank, world, args.variant,
                     flags=FLAG_STAGED_SPINS if args.staged_spins else 0)
    if rank != 0:
        return 0
    traffic = None
    try:
        traffic = (json.load(open(os.path.join(ROOT, "profiles", "traffic.json")))
                   .get(args.model) or {}).get("bytes_per_launch")
    except (OSError, ValueError):
        pass
    line = {
        "metric": "spin updates/ns", "value": res["value"], "unit": "spin updates/ns",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": res["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u8" if model == 0 else "f32", "data": "synthetic",
        "config": config,
        "roofline": {"bound": "hbm", "achieved": res["achieved_gbs"], "peak": hbm_peak,
                     "unit": "GB/s", "frac": res["achieved_gbs"] / hbm_peak,
                     "peak_source": peak_src, "traffic": traffic,
                     "kernel": ("ising_sc_kernel (one colour phase)" if model == 0
                                else "xyz_sc_kernel (one colour phase)"),
                     "bytes_per_update": res["bytes_per_update"], "phase_ms": res["phase_ms"],
                     "autotuned_variant": res["variant"]},
        "e2e": {"value": res["e2e"], "unit": "spin updates/ns",
                "h2d_bytes_per_step": res["h2d"], "d2h_bytes_per_step": res["d2h"],
                "detail": res["e2e_detail"]},
        "gpu_launches": res["launches"],
        "clocks": res["clocks"],
        "accept_ratio": res["accept_mean"],
    }
    if not args.no_components and model == eg.MODEL_ISING:
        comp = {}
        h = run_sweeps(eg.MODEL_XYZ, args.L, 64, 300, 5, rank, 1, clocks=False, e2e=False)
        comp["heisenberg_sweep"] = {
            "workload": "simple-cubic %d^3 Heisenberg float4 at kT_c=1.443 J, 64 replicas" % args.L,
            "value": h["value"], "unit": "spin updates/ns",
            "roofline": {"bound": "hbm", "achieved": h["achieved_gbs"], "peak": hbm_peak,
                         "unit": "GB/s", "frac": h["achieved_gbs"] / hbm_peak,
                         "bytes_per_update": BYTES_HEIS}}
        s = run_sq(cells=args.sq_cells)
        comp["structure_factor"] = dict(s, roofline={
            "bound": "tensor", "achieved": s["useful_tflops"], "peak": bf16_peak,
            "unit": "TFLOP/s", "frac": s["useful_tflops"] / bf16_peak,
            "note": "useful FLOPs; the BF16 hi/lo split issues 3 tensor products per useful "
                    "product (tensor_tflops)"})
        si = run_sq(cells=args.sq_cells, model=MODEL_ISING)
        comp["structure_factor_ising"] = dict(si, roofline={
            "bound": "tensor", "achieved": si["useful_tflops"], "peak": bf16_peak,
            "unit": "TFLOP/s", "frac": si["useful_tflops"] / bf16_peak,
            "note": "useful FLOPs; 2 tensor products per useful product (B_lo = 0 for +-1 spins)"})
        bt = run_batch()
        bt["roofline"] = {"bound": "hbm", "achieved": bt.pop("achieved_gbs"), "peak": hbm_peak,
                          "unit": "GB/s", "note": "3 B per Ising and 48 B per Heisenberg update"}
        bt["roofline"]["frac"] = bt["roofline"]["achieved"] / hbm_peak
        comp["batch"] = bt
        comp["tau"] = run_tau(args.L)
        comp["learned"] = run_learned(args.L)
        comp["learned_heisenberg"] = run_learned(args.L, R=64, train_steps=4000, n_plain=60000, n_learn=20000,
                                                 heisenberg=True)
        comp["program_c1"] = run_program("c1_ising_16")
        comp["program_c2"] = run_program("c2_heisenberg_32", repeats=1)
        comp["pyrochlore_pt"] = run_pyrochlore_pt()
        comp["pyrochlore_pt_ising"] = run_pyrochlore_pt(ising=True)
        line["components"] = comp
    if not args.no_cpu:
        line["cpu_baseline"] = {k: v for k, v in
                                cpu_reference(model, args.L, args.cpu_mcs or 600, cores).items()
                                if k in ("value", "unit", "cores", "kind", "sample")}
    print(json.dumps(line))
    return 0


if __name__ == "__main__":
    sys.exit(main())
