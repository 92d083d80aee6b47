"""ctypes binding of the C-ABI declared in include/ether_gpu.h.

The shared library is built in-tree (ether_gb300/libether_gpu.so) by ether_gb300.build.
There is no CPU fallback: if the library is missing, load() raises.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libether_gpu.so")

ETHER_OK = 0
ERRORS = {
    -1: "ETHER_ERR_ARG", -2: "ETHER_ERR_CUDA", -3: "ETHER_ERR_NOMEM",
    -4: "ETHER_ERR_UNSUPPORTED", -5: "ETHER_ERR_CAPACITY", -6: "ETHER_ERR_TIMEOUT",
    -7: "ETHER_ERR_STATE", -8: "ETHER_ERR_NODEV", -9: "ETHER_ERR_PARSE",
}
MODEL_ISING, MODEL_XYZ = 0, 1
FLAG_FORCE_GENERAL = 1 << 0
FLAG_PT_TRUE_ENERGY = 1 << 1
FLAG_PT_REFERENCE_COPY = 1 << 2
FLAG_NO_GRAPHS = 1 << 3
FLAG_NO_RESIDENT = 1 << 4
FLAG_STAGED_SPINS = 1 << 5
RUN_PARSE_ONLY = 1 << 0
RUN_QUIET = 1 << 1
RUN_RESUME = 1 << 2


class EtherError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (ERRORS.get(code, "?"), code, msg))
        self.code = code


class Desc(C.Structure):
    _fields_ = [
        ("n_sites", C.c_int32), ("n_species", C.c_int32), ("n_shells", C.c_int32),
        ("nbd_capacity", C.c_int32), ("model", C.c_int32), ("angle", C.c_int32),
        ("dphi", C.c_double), ("zeeman", C.c_int32), ("h", C.c_double * 3),
        ("g_factor", C.c_double), ("mb", C.c_double), ("sia", C.c_int32),
        ("ion", C.POINTER(C.c_double)), ("nn", C.POINTER(C.c_int32)),
        ("j_exc", C.POINTER(C.c_double)), ("sia_vec", C.POINTER(C.c_double)),
        ("s", C.POINTER(C.c_double)), ("stgg", C.POINTER(C.c_double)),
        ("n_replicas", C.c_int32), ("seed", C.c_uint32), ("sc", C.c_int32 * 3),
        ("basis", C.c_int32), ("flags", C.c_int32), ("sia_local", C.POINTER(C.c_double)),
    ]


class Schedule(C.Structure):
    _fields_ = [
        ("tmcs_eq", C.c_int32), ("coa", C.c_int32), ("ovrr", C.c_int32),
        ("ovrr_para", C.c_double), ("ovrr_mcs", C.c_int32), ("pt", C.c_int32),
        ("exchange_interval", C.c_int32),
    ]


class Info(C.Structure):
    _fields_ = [
        ("n_colours", C.c_int32), ("fast_path", C.c_int32), ("n_types", C.c_int32),
        ("table_entries", C.c_int32), ("n_slots", C.c_int32), ("n_groups", C.c_int32),
        ("device_bytes", C.c_size_t), ("kernel_launches", C.c_uint64),
        ("sq_kernel_ms", C.c_float), ("ion_direct", C.c_int32),
    ]


class BatchInfo(C.Structure):
    _fields_ = [
        ("n_members", C.c_int32), ("n_replicas", C.c_int32), ("threads", C.c_int32),
        ("units_per_thread", C.c_int32), ("blocks_per_sm", C.c_int32), ("grid", C.c_int32),
        ("walk", C.c_int32),
        ("n_segments", C.c_int32), ("kernels_per_sweep", C.c_int32),
        ("site_updates_per_sweep", C.c_int64), ("kernel_launches", C.c_uint64),
        ("last_sweep_ms", C.c_float),
    ]


class LearnDesc(C.Structure):
    _fields_ = [("patch", C.c_int32), ("hidden", C.c_int32), ("seed", C.c_uint32),
                ("capacity", C.c_int64)]


class LearnInfo(C.Structure):
    _fields_ = [
        ("n_params", C.c_int32), ("train_steps", C.c_int32), ("patches_per_class", C.c_int64),
        ("n_samples", C.c_int64), ("capacity", C.c_int64), ("proposed", C.c_uint64),
        ("kernel_launches", C.c_uint64), ("last_sweep_ms", C.c_float),
        ("last_train_ms", C.c_float),
    ]


class RunInfo(C.Structure):
    _fields_ = [
        ("ranks", C.c_int32), ("model", C.c_int32), ("n_sites", C.c_int32),
        ("n_species", C.c_int32), ("n_shells", C.c_int32), ("n_temperatures", C.c_int32),
        ("repeat", C.c_int32), ("n_rounds", C.c_int32), ("site_updates", C.c_uint64),
        ("seconds", C.c_double),
    ]


P = C.c_void_p
PD = C.POINTER(C.c_double)
PI32 = C.POINTER(C.c_int32)
PU32 = C.POINTER(C.c_uint32)
PU64 = C.POINTER(C.c_uint64)

# name -> (restype, argtypes); the complete exported surface of include/ether_gpu.h
SIGNATURES = {
    "ether_abi_version": (C.c_int, []),
    "ether_last_error": (C.c_char_p, []),
    "ether_create": (C.c_int, [C.POINTER(Desc), C.POINTER(P)]),
    "ether_destroy": (C.c_int, [P]),
    "ether_set_beta": (C.c_int, [P, PD]),
    "ether_set_ladder": (C.c_int, [P, C.c_int32, PD]),
    "ether_set_streams": (C.c_int, [P, PU32, PU32]),
    "ether_set_spins": (C.c_int, [P, C.c_int32, PD]),
    "ether_get_spins": (C.c_int, [P, C.c_int32, PD]),
    "ether_set_spins_batch": (C.c_int, [P, C.c_int32, C.c_int32, PD]),
    "ether_get_spins_batch": (C.c_int, [P, C.c_int32, C.c_int32, PD]),
    "ether_spins_batch_split": (C.c_int, [P, PI32, PI32]),
    "ether_fresh_spins": (C.c_int, [P]),
    "ether_metropolis": (C.c_int, [P, C.c_int32, PD]),
    "ether_overrelaxation": (C.c_int, [P, C.c_double]),
    "ether_tot_energy": (C.c_int, [P, PD]),
    "ether_tot_magnetisation": (C.c_int, [P, PD]),
    "ether_observable": (C.c_int, [P, C.c_int32, C.c_int32, C.c_int32]),
    "ether_zero_avg": (C.c_int, [P]),
    "ether_get_sums": (C.c_int, [P, PD]),
    "ether_avg": (C.c_int, [P, PD]),
    "ether_per_repeat": (C.c_int, [P, PD, PD]),
    "ether_parallel_tempering": (C.c_int, [P, C.c_int32, PI32]),
    "ether_get_slots": (C.c_int, [P, PI32]),
    "ether_mcs": (C.c_int, [P, C.POINTER(Schedule), C.c_int32, C.c_int32, PI32]),
    "ether_record_series": (C.c_int, [P, C.c_int32, C.c_int32, PD, PD]),
    "ether_get_accept_counts": (C.c_int, [P, PU64]),
    "ether_reset_accept_counts": (C.c_int, [P]),
    "ether_get_slot_accept_counts": (C.c_int, [P, PU64]),
    "ether_get_info": (C.c_int, [P, C.POINTER(Info)]),
    "ether_get_colouring": (C.c_int, [P, PI32, PI32]),
    "ether_sync": (C.c_int, [P]),
    "ether_get_stream": (C.c_int, [P, C.POINTER(P)]),
    "ether_metropolis_phase": (C.c_int, [P, C.c_int32]),
    "ether_end_sweep": (C.c_int, [P]),
    "ether_autotune": (C.c_int, [P, PI32, C.POINTER(C.c_float)]),
    "ether_set_variant": (C.c_int, [P, C.c_int32]),
    "ether_structure_factor": (C.c_int, [P, PD, PI32, PD, PD, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "ether_moment_vectors": (C.c_int, [P, PD]),
    "ether_spiral_setup": (C.c_int, [P, C.c_double, PD, C.c_double, C.c_int32, C.POINTER(C.c_int64)]),
    "ether_spiral_state": (C.c_int, [P, PD]),
    "ether_spiral_avg": (C.c_int, [P, PD]),
    "ether_batch_create": (C.c_int, [C.POINTER(P), C.c_int32, C.POINTER(P)]),
    "ether_batch_destroy": (C.c_int, [P]),
    "ether_batch_metropolis": (C.c_int, [P, C.c_int32]),
    "ether_batch_mcs": (C.c_int, [P, C.POINTER(Schedule), C.c_int32, C.c_int32, PI32]),
    "ether_batch_set_config": (C.c_int, [P, C.c_int32, C.c_int32, C.c_int32, C.c_int32]),
    "ether_batch_autotune": (C.c_int, [P, PI32, C.POINTER(C.c_float)]),
    "ether_batch_get_info": (C.c_int, [P, C.POINTER(BatchInfo)]),
    "ether_batch_get_stream": (C.c_int, [P, C.POINTER(P)]),
    "ether_learn_create": (C.c_int, [P, C.POINTER(LearnDesc), C.POINTER(P)]),
    "ether_learn_destroy": (C.c_int, [P]),
    "ether_learn_collect": (C.c_int, [P, C.c_int32]),
    "ether_learn_train": (C.c_int, [P, C.c_int32, C.c_int32, C.c_float, PD]),
    "ether_learn_batch_sweep": (C.c_int, [C.POINTER(C.c_void_p), C.c_int32, C.c_int32, C.c_int32]),
    "ether_learn_sweep": (C.c_int, [P, C.c_int32]),
    "ether_learn_record_series": (C.c_int, [P, C.c_int32, C.c_int32, C.c_int32, C.c_int32, PD]),
    "ether_learn_get_accepts": (C.c_int, [P, PU64]),
    "ether_learn_get_params": (C.c_int, [P, C.POINTER(C.c_float)]),
    "ether_learn_set_params": (C.c_int, [P, C.POINTER(C.c_float)]),
    "ether_learn_loss_grad": (C.c_int, [P, C.POINTER(C.c_float), PU32, C.c_int32, PD,
                                        C.POINTER(C.c_float)]),
    "ether_learn_forward": (C.c_int, [P, C.POINTER(C.c_float), C.c_int32, C.POINTER(C.c_float)]),
    "ether_learn_loss_grad_f": (C.c_int, [P, C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_int32, PD,
                                          C.POINTER(C.c_float)]),
    "ether_learn_get_shape": (C.c_int, [P, PI32, PI32, PI32]),
    "ether_learn_set_dump": (C.c_int, [P, C.c_int32]),
    "ether_learn_get_dump": (C.c_int, [P, C.POINTER(C.c_float)]),
    "ether_learn_get_info": (C.c_int, [P, C.POINTER(LearnInfo)]),
    "ether_sc_energy_noalloc": (C.c_int, [C.c_int32, P, PI32, C.c_int32, PD, PD, PD, PD, P]),
    "ether_build_lattice": (C.c_int, [C.c_int32, PD, PI32, PD, PI32, C.c_char_p, C.c_int32,
                                      C.c_int32, PD, C.c_double, C.c_int32, PD, PD, PI32]),
    "ether_run": (C.c_int, [C.c_char_p, C.c_char_p, C.c_int32, C.POINTER(RunInfo)]),
}

_lib = None


def load(path=None):
    """Loads libether_gpu.so (raises if it has not been built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError("libether_gpu.so not built: run `python -m ether_gb300.build` "
                           "(there is no CPU fallback)")
    lib = C.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def check(rc):
    if rc != ETHER_OK:
        msg = load().ether_last_error()
        raise EtherError(rc, msg.decode() if msg else "")
    return rc


def dptr(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(PD)


def iptr(a):
    if a is None:
        return None
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(PI32)


def uptr(a):
    if a is None:
        return None
    assert a.dtype == np.uint32 and a.flags.c_contiguous
    return a.ctypes.data_as(PU32)
