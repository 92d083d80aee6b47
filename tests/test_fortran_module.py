"""The Fortran module (fortran/ether_gpu_mod.f90) against the C header (include/ether_gpu.h).

No Fortran compiler exists here, so the module is checked as text: every bind(C) interface
names a function the header declares, with as many dummy arguments as the C parameters, and
every entry point that stands for a call site of src/ether.f90 has an interface.
"""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# the header's entry points for src/ether.f90's call sites (ether_run: the whole program)
CALL_SITES = [
    "ether_create", "ether_destroy", "ether_set_beta", "ether_set_ladder", "ether_set_streams",
    "ether_set_spins", "ether_get_spins", "ether_set_spins_batch", "ether_get_spins_batch",
    "ether_fresh_spins", "ether_metropolis", "ether_overrelaxation", "ether_tot_energy",
    "ether_tot_magnetisation", "ether_parallel_tempering", "ether_observable", "ether_zero_avg",
    "ether_avg", "ether_per_repeat", "ether_mcs", "ether_moment_vectors", "ether_spiral_setup",
    "ether_spiral_state", "ether_spiral_avg", "ether_run",
]


def _c_decls():
    text = open(os.path.join(ROOT, "include", "ether_gpu.h")).read()
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    out = {}
    for m in re.finditer(r"\b(?:int|const char\s*\*)\s*(ether_\w+)\s*\(([^)]*)\)\s*;", text):
        params = m.group(2).strip()
        out[m.group(1)] = 0 if params in ("", "void") else len(params.split(","))
    return out


def _f_interfaces():
    text = open(os.path.join(ROOT, "fortran", "ether_gpu_mod.f90")).read()
    text = re.sub(r"&\s*\n\s*", " ", text)  # join continuation lines
    out = {}
    for m in re.finditer(r"function\s+(\w+)\s*\(([^)]*)\)\s*bind\(C,\s*name=\"(ether_\w+)\"\)", text):
        args = [a for a in m.group(2).split(",") if a.strip()]
        out[m.group(3)] = len(args)
    return out


def test_interfaces_match_the_header():
    c, f = _c_decls(), _f_interfaces()
    assert len(f) >= 40
    for name, nargs in f.items():
        assert name in c, name
        assert nargs == c[name], (name, nargs, c[name])


def test_every_call_site_has_an_interface():
    c, f = _c_decls(), _f_interfaces()
    for name in CALL_SITES:
        assert name in c, name
        assert name in f, name
