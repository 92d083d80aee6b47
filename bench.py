#!/usr/bin/env python
"""Benchmark of the plain Checkerboard Metropolis sweep on one GB300.

Workload (the L = 64 simple-cubic target): plain colour-ordered Metropolis sweeps of the
64^3 simple-cubic Ising model at k_B T_c = 4.511 J (J = 1 meV, ferromagnetic), a batch of
R = 1024 independent replicas (each its own Philox stream) so the int8 state (268 MB) is
larger than the 129 MB L2.  A step is one full sweep (both colour phases) of every replica.

  value  = spin updates / ns over the timed steps (device-resident state, CUDA events)
  e2e    = same metric through the C-ABI with host buffers: the configuration is uploaded
           from host memory at the start, each step returns the acceptance ratios to the
           host (the reference's Metropolis(beta, accept) boundary), the final
           configuration of replica 0 is read back at the end
  roofline = dominant kernel (one colour phase) at 3 algorithmic bytes per site update
  cpu_baseline = the oracle's typewriter restatement of src/Metropolis.f90 +
           src/get_tot_energy.f90 (what ether.f90 does per MCS), one replica per host core

--impl reference times that CPU restatement on all host cores as the reference arm (the
Fortran reference itself cannot be built: no gfortran / MPI on this image or the box).
"""
import argparse
import ctypes as C
import ctypes.util
import json
import os
import subprocess
import sys
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


def _cudart():
    for name in ("libcudart.so.13", "libcudart.so", ctypes.util.find_library("cudart")):
        if not name:
            continue
        try:
            return C.CDLL(name)
        except OSError:
            pass
    for d in ("/usr/local/cuda/lib64", "/usr/local/cuda/targets/sbsa-linux/lib",
              "/usr/local/cuda/targets/x86_64-linux/lib"):
        p = os.path.join(d, "libcudart.so")
        if os.path.exists(p):
            return C.CDLL(p)
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
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

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


def make_workload(model, L, replicas, seed=1992):
    import ether_gb300 as eg
    lat = eg.simple_cubic(L)
    j = eg.couplings(1, [[(1, 1, (-J_MEV, -J_MEV, -J_MEV))]], [1.0])
    sw = eg.Sweep.from_lattice(lat, j, np.array([1.0]), model, replicas=replicas, seed=seed)
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


def run_gpu(model, L, replicas, steps, warmup, rank, world, force_variant=0):
    import ether_gb300 as eg
    lat, j, sw, ion, beta = make_workload(model, L, replicas, seed=1992 + 7919 * rank)
    sw.set_spins(ion)
    if force_variant:
        sw.set_variant(force_variant)
        variant = force_variant
    else:
        variant, tuned_ms = sw.autotune()
    N, R = lat.N, replicas
    ev = Events(sw.stream())
    for _ in range(warmup):
        sw.metropolis(1, accept=False)
    sw.sync()
    _barrier(world)
    launches0 = sw.info().kernel_launches
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")) if world > 1 else 0)
    clocks.start()
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
    clk = clocks.stop()
    launches = sw.info().kernel_launches - launches0
    ev.free([t0, t1] + [e for m in marks for e in m])
    _barrier(world)
    total_ms = _max_over_ranks(total_ms, world)
    updates = float(N) * R * steps
    value = updates / (total_ms * 1e6) * world
    # dominant kernel: one colour phase = R*N/2 updates
    bpu = BYTES_ISING if model == eg.MODEL_ISING else BYTES_HEIS
    phase_avg_ms = float(np.mean(phase_ms))
    achieved_gbs = bpu * (R * N / 2.0) / (phase_avg_ms * 1e-3) / 1e9

    # end to end through the C-ABI with host buffers
    acc = None
    t_start = time.perf_counter()
    sw.set_spins(ion)
    ev2 = Events(sw.stream())
    e0 = ev2.record()
    for _ in range(steps):
        acc = sw.metropolis(1, accept=True)   # D2H of R doubles every step
    out = sw.get_spins(lat.ion, 0)
    e1 = ev2.record()
    sw.sync()
    t_e2e = time.perf_counter() - t_start
    ev2.free([e0, e1])
    e2e = updates / (t_e2e * 1e9) * world
    h2d = (N * (1 if model == eg.MODEL_ISING else 16) * R) / steps
    d2h = 8.0 * R + (N * (1 if model == eg.MODEL_ISING else 16)) / steps
    sw.close()
    return {
        "value": value, "ms_per_step": total_ms / steps, "phase_ms": phase_avg_ms,
        "achieved_gbs": achieved_gbs, "bytes_per_update": bpu, "launches": int(launches),
        "clocks": clk, "e2e": e2e, "h2d": h2d, "d2h": d2h,
        "accept_mean": float(np.mean(acc)) if acc is not None else None,
        "check_spin_sum": float(out[:, 3].sum()),
        "variant": variant,
    }


def cpu_reference(model, L, mcs, threads, seed=1992):
    """The oracle's typewriter restatement of the reference's per-MCS work (Metropolis
    + get_tot_energy), one replica (temperature) per thread."""
    import ether_gb300 as eg
    from oracle import pyoracle as po
    lat = eg.simple_cubic(L)
    j = eg.couplings(1, [[(1, 1, (-J_MEV, -J_MEV, -J_MEV))]], [1.0])
    osys = po.System.from_lattice(lat, j, np.array([1.0]), model)
    ktc = KTC_ISING if model == eg.MODEL_ISING else KTC_HEIS
    beta = 1.0 / (ktc * J_MEV * 1e-3)
    cfg = po.RunCfg(tmcs=mcs, tmcs_eq=mcs, coa=1 << 30, repeat=1, ovrr=0, ovrr_para=0.0,
                    ovrr_mcs=0, seed=seed, itemp=1, rank=0)
    nT = threads
    vals = np.zeros(6 * nT)
    acc = np.zeros(nT)
    b = np.full(nT, beta)
    t = time.perf_counter()
    po.lib().orc_run_temperatures(osys.p(), osys.ion0.ctypes.data_as(po.PD), nT,
                                  b.ctypes.data_as(po.PD), C.byref(cfg), threads,
                                  vals.ctypes.data_as(po.PD), acc.ctypes.data_as(po.PD))
    dt = time.perf_counter() - t
    updates = float(lat.N) * mcs * nT
    return {"value": updates / (dt * 1e9), "unit": "spin updates/ns", "cores": threads,
            "kind": "port",
            "sample": "%d replicas x %d MCS of %d^3 %s, typewriter order, FP64, per-MCS "
                      "get_tot_energy as src/ether.f90:177 (%.1f s wall)" %
                      (nT, mcs, L, "Ising" if model == 0 else "Heisenberg", dt),
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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--model", default="ising", choices=["ising", "heisenberg"])
    ap.add_argument("--L", type=int, default=64)
    ap.add_argument("--replicas", type=int, default=0)
    ap.add_argument("--cpu-mcs", type=int, default=0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--variant", type=int, default=0)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        os.environ.setdefault("CUDA_VISIBLE_DEVICES", os.environ.get("LOCAL_RANK", "0"))
        import torch.distributed as dist
        dist.init_process_group("gloo")

    import ether_gb300 as eg
    model = eg.MODEL_ISING if args.model == "ising" else eg.MODEL_XYZ
    replicas = args.replicas or (1024 if model == eg.MODEL_ISING else 64)
    cores = os.cpu_count() or 1
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
        if rank != 0:
            return 0
        mcs = args.cpu_mcs or 300
        ref = cpu_reference(model, args.L, mcs, cores)
        line = {"metric": "spin updates/ns", "value": ref["value"], "unit": "spin updates/ns",
                "impl": "reference", "n_gpus": args.gpus, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": config,
                "cpu_baseline": {k: ref[k] for k in ("value", "unit", "cores", "kind", "sample")},
                "e2e": {"value": ref["value"], "unit": "spin updates/ns",
                        "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                "note": "Fortran reference not buildable (no gfortran/MPI): its path restated "
                        "in C (oracle/) and timed on all host cores"}
        print(json.dumps(line))
        return 0

    res = run_gpu(model, args.L, replicas, args.steps, args.warmup, rank, world, args.variant)
    if rank != 0:
        return 0
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    peak = peaks.get("hbm_gbs")
    peak_src = "measured" if peak else "fallback"
    peak = peak or 6800.0
    traffic = None
    try:
        prof = json.load(open(os.path.join(ROOT, "profiles", "traffic.json")))
        traffic = prof.get(args.model)
    except (OSError, ValueError):
        pass
    line = {
        "metric": "spin updates/ns", "value": res["value"], "unit": "spin updates/ns",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": res["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u8" if model == 0 else "f32", "data": "synthetic",
        "config": config,
        "roofline": {"bound": "hbm", "achieved": res["achieved_gbs"], "peak": peak,
                     "unit": "GB/s", "frac": res["achieved_gbs"] / peak,
                     "peak_source": peak_src, "traffic": traffic,
                     "kernel": "ising_sc_kernel<16> (one colour phase)" if model == 0
                     else "xyz_sc_kernel (one colour phase)",
                     "bytes_per_update": res["bytes_per_update"],
                     "phase_ms": res["phase_ms"], "autotuned_variant": res["variant"]},
        "e2e": {"value": res["e2e"], "unit": "spin updates/ns",
                "h2d_bytes_per_step": res["h2d"], "d2h_bytes_per_step": res["d2h"]},
        "gpu_launches": res["launches"],
        "clocks": res["clocks"],
        "accept_ratio": res["accept_mean"],
    }
    if not args.no_cpu:
        mcs = args.cpu_mcs or 300
        line["cpu_baseline"] = {k: v for k, v in cpu_reference(model, args.L, mcs, cores).items()
                                if k in ("value", "unit", "cores", "kind", "sample")}
    print(json.dumps(line))
    return 0


if __name__ == "__main__":
    sys.exit(main())
