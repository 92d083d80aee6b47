"""ctypes binding of oracle/_build/libether_oracle.so (TEST INFRASTRUCTURE ONLY).

Used by tests/, __graft_entry__.smoke() and bench.py's CPU baseline as the checker; the
product never imports it.  Arrays use the reference's Fortran layouts (see
oracle/ether_oracle.h).
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SO = os.path.join(HERE, "_build", "libether_oracle.so")
SO_TIMED = os.path.join(HERE, "_build", "libether_oracle_timed.so")

PD = C.POINTER(C.c_double)
PF = C.POINTER(C.c_float)
PI = C.POINTER(C.c_int32)
PU = C.POINTER(C.c_uint32)


class Sys(C.Structure):
    _fields_ = [("n_sites", C.c_int), ("n_species", C.c_int), ("n_shells", C.c_int),
                ("cap", C.c_int), ("model", C.c_int), ("angle", C.c_int), ("dphi", C.c_double),
                ("zeeman", C.c_int), ("h", C.c_double * 3), ("g_factor", C.c_double),
                ("mb", C.c_double), ("sia", C.c_int), ("nn", PI), ("j_exc", PD),
                ("sia_vec", PD), ("s", PD), ("stgg", PD), ("sia_local", PD)]


class Stream(C.Structure):
    _fields_ = [("key", C.c_uint32 * 2), ("n", C.c_uint64)]


class Acc(C.Structure):
    _fields_ = [(k, C.c_double) for k in ("n", "e", "e2", "e4", "m", "m2", "m4")]


class RunCfg(C.Structure):
    _fields_ = [("tmcs", C.c_int), ("tmcs_eq", C.c_int), ("coa", C.c_int), ("repeat", C.c_int),
                ("ovrr", C.c_int), ("ovrr_para", C.c_double), ("ovrr_mcs", C.c_int),
                ("seed", C.c_uint32), ("itemp", C.c_int), ("rank", C.c_int)]


_lib = None
_timed = None


def build():
    subprocess.run(["sh", os.path.join(HERE, "build.sh")], check=True)


def lib():
    """The checker build (every FP32 operation rounded separately)."""
    global _lib
    if _lib is None:
        if not os.path.exists(SO):
            build()
        _lib = _bind(C.CDLL(SO), learn=True)
    return _lib


def timed_lib():
    """The same restatement built with the reference's optimisation flags: the CPU baseline
    that bench.py times (its arithmetic may contract a*b+c; it is never the checker)."""
    global _timed
    if _timed is None:
        if not os.path.exists(SO_TIMED):
            build()
        _timed = _bind(C.CDLL(SO_TIMED), learn=False)
    return _timed


def _bind(L, learn):
    """Declares the argument and result types of the oracle's entry points on L."""
    L.orc_philox4x32_10.argtypes = [PU, PU, PU]
    L.orc_supercell.restype = C.c_int
    L.orc_supercell.argtypes = [C.c_int, PD, PI, PD, PI, C.c_int, PD, PD]
    L.orc_neighbours_bruteforce.restype = C.c_int
    L.orc_neighbours_bruteforce.argtypes = [C.c_int, PD, PD, PI, C.c_char_p, C.c_int, PD,
                                            C.c_double, C.c_int, PI]
    L.orc_greedy_colouring.restype = C.c_int
    L.orc_greedy_colouring.argtypes = [C.c_int, C.c_int, C.c_int, PI, PI, PI]
    L.orc_hamiltonian.restype = C.c_double
    L.orc_tot_energy.restype = C.c_double
    L.orc_tot_energy.argtypes = [C.POINTER(Sys), PD]
    L.orc_tot_magnetisation.argtypes = [C.POINTER(Sys), PD, PD]
    L.orc_tot_energy_f32.restype = C.c_double
    L.orc_tot_energy_f32.argtypes = [C.POINTER(Sys), PD, PF]
    L.orc_tot_magnetisation_f32.argtypes = [C.POINTER(Sys), PD, PF, PD]
    L.orc_stream_init.argtypes = [C.POINTER(Stream), C.c_uint32, C.c_uint32]
    L.orc_stream_uniform.restype = C.c_double
    L.orc_stream_uniform.argtypes = [C.POINTER(Stream)]
    L.orc_metropolis_typewriter.restype = C.c_double
    L.orc_metropolis_typewriter.argtypes = [C.POINTER(Sys), PD, C.c_double, C.POINTER(Stream)]
    L.orc_fresh_spins_typewriter.argtypes = [C.POINTER(Sys), PD, C.POINTER(Stream)]
    L.orc_overrelaxation_typewriter.argtypes = [C.POINTER(Sys), PD, C.c_int, C.POINTER(Stream)]
    L.orc_metropolis_colour.restype = C.c_double
    L.orc_metropolis_colour.argtypes = [C.POINTER(Sys), PD, PF, C.c_int, C.c_double,
                                        C.c_uint32, C.c_uint32, C.c_uint32, PI, PI, C.c_int]
    L.orc_overrelax_colour.argtypes = [C.POINTER(Sys), PD, PF, C.c_double, C.c_uint32,
                                       C.c_uint32, C.c_uint32, PI, PI, C.c_int]
    L.orc_fresh_spins_colour.argtypes = [C.POINTER(Sys), PD, PF, C.c_uint32, C.c_uint32,
                                         C.c_uint32]
    L.orc_parallel_tempering.restype = C.c_int
    L.orc_parallel_tempering.argtypes = [C.c_int, PD, PD, PI, C.c_int, C.c_uint32,
                                         C.c_uint32, C.c_int, PI]
    L.orc_acc_sample.argtypes = [C.POINTER(Acc), C.c_double, PD, C.c_int]
    L.orc_acc_average.argtypes = [C.POINTER(Acc), C.c_double, C.c_int, PD]
    L.orc_per_repeat.argtypes = [C.c_int, PD, PD, PD]
    L.orc_structure_factor.argtypes = [C.c_int, PD, PD, C.c_int, PD, PD]
    L.orc_run_temperature.restype = C.c_double
    L.orc_run_temperature.argtypes = [C.POINTER(Sys), PD, C.c_double, C.POINTER(RunCfg), PD]
    L.orc_run_temperatures.argtypes = [C.POINTER(Sys), PD, C.c_int, PD, C.POINTER(RunCfg),
                                       C.c_int, PD, PD]
    L.orc_run_ladder.argtypes = [C.POINTER(Sys), PD, C.c_int, PD, C.POINTER(RunCfg), C.c_int,
                                 C.c_int, PD, PD, C.POINTER(C.c_long)]
    L.orc_expf_neg.restype = C.c_float
    L.orc_expf_neg.argtypes = [C.c_float]
    L.orc_sincosf.argtypes = [C.c_float, PF, PF]
    L.orc_moment_vectors.argtypes = [C.POINTER(Sys), PD, PD]
    L.orc_spiral_pairs.restype = C.c_long
    L.orc_spiral_pairs.argtypes = [C.c_int, PD, C.c_double, PD, C.c_double, C.c_int, PI]
    L.orc_spiral_state.restype = C.c_double
    L.orc_spiral_state.argtypes = [C.c_int, PD, C.c_int, PI, C.c_long]
    if not learn:
        return L
    PU8 = C.POINTER(C.c_uint8)
    L.orc_bf16_round.restype = C.c_float
    L.orc_bf16_round.argtypes = [C.c_float]
    L.orc_logf_own.restype = C.c_float
    L.orc_logf_own.argtypes = [C.c_float]
    L.orc_mlp_n_params.restype = C.c_int
    L.orc_mlp_forward.argtypes = [PF, PF, C.c_int, C.c_int, PF]
    L.orc_mlp_loss_grad.restype = C.c_double
    L.orc_mlp_loss_grad.argtypes = [PF, PF, PU, C.c_int, C.c_int, PD]
    L.orc_patch_tables.argtypes = [PI, PI, PI, PI]
    L.orc_patch_gather.argtypes = [PU8, PI, PI, C.c_int, C.c_int, C.c_int, C.c_float, PF, PU,
                                   PU, PU]
    L.orc_patch_btables.argtypes = [C.c_double, PU, PF, PF]
    L.orc_patch_offsets.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32, PI]
    L.orc_patch_sweep.restype = C.c_long
    L.orc_patch_sweep.argtypes = [PU8, PI, C.c_double, PF, C.c_uint32, C.c_uint32, C.c_uint32]
    L.orc_patch_chain.argtypes = [PI, C.c_double, C.c_long, C.c_long, C.c_int, C.c_float,
                                  C.c_float, C.c_uint32, PD]
    L.orc_xmlp_n_params.restype = C.c_int
    L.orc_xmlp_forward.argtypes = [PF, PF, C.c_int, C.c_int, PF]
    L.orc_xmlp_loss_grad.restype = C.c_double
    L.orc_xmlp_loss_grad.argtypes = [PF, PF, PF, C.c_int, C.c_int, PD]
    L.orc_vmf_logpdf.restype = C.c_float
    L.orc_vmf_logpdf.argtypes = [C.c_float] * 6
    L.orc_vmf_sample.argtypes = [C.c_float] * 5 + [PF]
    L.orc_xpatch_sweep.restype = C.c_long
    L.orc_xpatch_sweep.argtypes = [PF, PI, C.c_float, PF, PF, C.c_uint32, C.c_uint32, C.c_uint32]
    return L


class ScLattice:
    """The periodic L1 x L2 x L3 simple-cubic lattice (lattice constant 1, one species, one
    neighbour shell at distance 1) in the reference's layouts, built without the product
    library: sites by orc_supercell (generate_supercell, src/generate_supercell.f90:104-132)
    and the neighbour table nn(1, N, 0:cap, 0:1) in closed form.  getting_nbd
    (src/getting_nbd.f90:34-78) lists a site's neighbours by increasing site number, each
    once; with every extent >= 3 the six are distinct (at 2 the search finds one site for two
    periodic images).  Attributes as the product's Lattice: ion (N, 9), nn (2, cap+1, N, 1),
    stgg, N, nsh, cap."""

    def __init__(self, L, cap=20):
        L1, L2, L3 = (L, L, L) if np.isscalar(L) else tuple(L)
        if min(L1, L2, L3) < 3:
            raise ValueError("every extent must be >= 3")
        self.N = N = L1 * L2 * L3
        self.nsh, self.cap = 1, int(cap)
        self.ion = np.zeros((N, 9))
        self.stgg = np.zeros(N)
        sc = np.array([L1, L2, L3], dtype=np.int32)
        lib().orc_supercell(1, _d(np.zeros(3)), _i(np.ones(1, dtype=np.int32)), _d(np.eye(3)),
                            _i(sc), 0, _d(self.ion), _d(self.stgg))
        i = np.arange(N)
        x, y, z = i % L1, (i // L1) % L2, i // (L1 * L2)
        nb = np.stack([(x + 1) % L1 + L1 * (y + L2 * z), (x - 1) % L1 + L1 * (y + L2 * z),
                       x + L1 * ((y + 1) % L2 + L2 * z), x + L1 * ((y - 1) % L2 + L2 * z),
                       x + L1 * (y + L2 * ((z + 1) % L3)), x + L1 * (y + L2 * ((z - 1) % L3))], axis=1)
        nb.sort(axis=1)
        self.nn = np.zeros((2, self.cap + 1, N, 1), dtype=np.int32)
        self.nn[0, 0, :, 0] = 6
        self.nn[0, 1:7, :, 0] = (nb + 1).T
        self.nn[1, 1:7, :, 0] = (nb + 1).T


def sc_couplings(J_mev):
    """j_exc(1, 1, 1, 3) of one species with spin length 1 and a diagonal J (meV) on the one
    shell, after parameters.f90 (meV -> eV): layout (3, nsp, nsp, nsh)."""
    j = np.zeros((3, 1, 1, 1))
    j[:, 0, 0, 0] = np.asarray(J_mev, dtype=np.float64) / 1000.0
    return j


def _d(a):
    return None if a is None else a.ctypes.data_as(PD)


def _i(a):
    return None if a is None else a.ctypes.data_as(PI)


def _f(a):
    return None if a is None else a.ctypes.data_as(PF)


def philox(ctr, key):
    c = np.ascontiguousarray(ctr, dtype=np.uint32)
    k = np.ascontiguousarray(key, dtype=np.uint32)
    o = np.zeros(4, dtype=np.uint32)
    lib().orc_philox4x32_10(c.ctypes.data_as(PU), k.ctypes.data_as(PU), o.ctypes.data_as(PU))
    return o


class System:
    """Holds the arrays of one lattice + couplings and an orc_sys pointing at them."""

    def __init__(self, ion, nn, j_exc, s, *, model, n_species, n_shells, cap, angle=False,
                 dphi=0.0, zeeman=False, h=(0, 0, 0), g_factor=2.0, mb=5.7883818060e-5,
                 sia=False, sia_vec=None, stgg=None, sia_local=None):
        self.ion0 = np.ascontiguousarray(ion, dtype=np.float64)
        self.nn = np.ascontiguousarray(nn, dtype=np.int32)
        self.j_exc = np.ascontiguousarray(j_exc, dtype=np.float64)
        self.s = np.ascontiguousarray(s, dtype=np.float64)
        self.sia_vec = None if sia_vec is None else np.ascontiguousarray(sia_vec, dtype=np.float64)
        self.sia_local = None if sia_local is None else np.ascontiguousarray(sia_local, dtype=np.float64)
        self.stgg = None if stgg is None else np.ascontiguousarray(stgg, dtype=np.float64)
        self.N = self.ion0.shape[0]
        y = Sys()
        y.n_sites, y.n_species, y.n_shells, y.cap = self.N, n_species, n_shells, cap
        y.model, y.angle, y.dphi = model, int(bool(angle)), float(dphi)
        y.zeeman = int(bool(zeeman))
        for k in range(3):
            y.h[k] = float(h[k])
        y.g_factor, y.mb, y.sia = float(g_factor), float(mb), int(bool(sia))
        y.nn, y.j_exc, y.sia_vec = _i(self.nn), _d(self.j_exc), _d(self.sia_vec)
        y.s, y.stgg = _d(self.s), _d(self.stgg)
        y.sia_local = _d(self.sia_local)
        self.sys = y
        self.model = model

    @classmethod
    def from_lattice(cls, lat, j_exc, s, model, **kw):
        kw.setdefault("stgg", lat.stgg)
        return cls(lat.ion, lat.nn, j_exc, s, model=model, n_species=j_exc.shape[1],
                   n_shells=lat.nsh, cap=lat.cap, **kw)

    def p(self):
        return C.byref(self.sys)

    def colouring(self):
        col = np.zeros(self.N, dtype=np.int32)
        rank = np.zeros(self.N, dtype=np.int32)
        n = lib().orc_greedy_colouring(self.N, self.sys.n_shells, self.sys.cap, _i(self.nn),
                                       _i(col), _i(rank))
        return n, col, rank

    def spin4(self, ion):
        s = np.zeros((self.N, 4), dtype=np.float32)
        s[:, 0:3] = ion[:, 1:4]
        s[:, 3] = ion[:, 5]
        return s

    def tot_energy(self, ion):
        return lib().orc_tot_energy(self.p(), _d(ion))

    def tot_magnetisation(self, ion):
        m = np.zeros(3)
        lib().orc_tot_magnetisation(self.p(), _d(ion), _d(m))
        return m

    def tot_energy_f32(self, ion, sp4):
        return lib().orc_tot_energy_f32(self.p(), _d(ion), _f(sp4))

    def tot_magnetisation_f32(self, ion, sp4):
        m = np.zeros(3)
        lib().orc_tot_magnetisation_f32(self.p(), _d(ion), _f(sp4), _d(m))
        return m

    def metropolis_colour(self, ion, sp4, prec, beta, seed, stream, t, col, rank, ncol):
        return lib().orc_metropolis_colour(self.p(), _d(ion), _f(sp4), prec, beta, seed, stream,
                                           t, _i(col), _i(rank), ncol)

    def overrelax_colour(self, ion, sp4, frac, seed, stream, t, col, rank, ncol):
        lib().orc_overrelax_colour(self.p(), _d(ion), _f(sp4), frac, seed, stream, t, _i(col),
                                   _i(rank), ncol)

    def fresh_spins_colour(self, ion, sp4, seed, stream, call):
        lib().orc_fresh_spins_colour(self.p(), _d(ion), _f(sp4), seed, stream, call)

    def metropolis_typewriter(self, ion, beta, st):
        return lib().orc_metropolis_typewriter(self.p(), _d(ion), beta, C.byref(st))

    def moment_vectors(self, ion):
        mm = np.zeros((self.sys.n_species, 3))
        lib().orc_moment_vectors(self.p(), _d(np.ascontiguousarray(ion, dtype=np.float64)), _d(mm))
        return mm


def spiral_pairs(ion, ss_dis, ss_direc, ss_latency, cap):
    """(ifs(N, cap) 1-based, count) of get_spiral_state's 'ions_for_spiral' (count -1: a site
    has more than cap)."""
    ion = np.ascontiguousarray(ion, dtype=np.float64)
    N = ion.shape[0]
    ifs = np.zeros((N, cap), dtype=np.int32)
    d = np.ascontiguousarray(ss_direc, dtype=np.float64)
    n = lib().orc_spiral_pairs(N, _d(ion), ss_dis, _d(d), ss_latency, cap, _i(ifs))
    return ifs, n


def spiral_state(ion, ifs, count):
    ion = np.ascontiguousarray(ion, dtype=np.float64)
    return lib().orc_spiral_state(ion.shape[0], _d(ion), ifs.shape[1], _i(np.ascontiguousarray(ifs)), count)


def stream(seed, sid):
    st = Stream()
    lib().orc_stream_init(C.byref(st), seed, sid)
    return st


def supercell(basis_cart, basis_species, abc, sc, checkerboard=False):
    bc = np.ascontiguousarray(basis_cart, dtype=np.float64).reshape(-1, 3)
    bs = np.ascontiguousarray(basis_species, dtype=np.int32)
    a = np.ascontiguousarray(abc, dtype=np.float64).reshape(3, 3)
    s = np.ascontiguousarray(sc, dtype=np.int32)
    N = int(np.prod(s)) * bc.shape[0]
    ion = np.zeros((N, 9))
    stgg = np.zeros(N)
    lib().orc_supercell(bc.shape[0], _d(bc), _i(bs), _d(a), _i(s), int(checkerboard), _d(ion),
                        _d(stgg))
    return ion, stgg


def neighbours_bruteforce(ion, abc, sc, bc, shells, tol, cap):
    N = ion.shape[0]
    sh = np.ascontiguousarray(shells, dtype=np.float64)
    nn = np.zeros((2, cap + 1, N, len(sh)), dtype=np.int32)
    a = np.ascontiguousarray(abc, dtype=np.float64).reshape(3, 3)
    s = np.ascontiguousarray(sc, dtype=np.int32)
    rc = lib().orc_neighbours_bruteforce(N, _d(np.ascontiguousarray(ion)), _d(a), _i(s),
                                         bc.encode(), len(sh), _d(sh), tol, cap, _i(nn))
    return rc, nn


# ----------------------------------------------------------- learned patch proposal ----
PU8 = C.POINTER(C.c_uint8)


def mlp_n_params():
    return lib().orc_mlp_n_params()


def mlp_forward(params, x, quant=True):
    p = np.ascontiguousarray(params, dtype=np.float32)
    xx = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, 128)
    z = np.zeros((xx.shape[0], 32), dtype=np.float32)
    lib().orc_mlp_forward(_f(p), _f(xx), xx.shape[0], int(quant), _f(z))
    return z


def mlp_loss_grad(params, x, y, quant=True):
    p = np.ascontiguousarray(params, dtype=np.float32)
    xx = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, 128)
    yy = np.ascontiguousarray(y, dtype=np.uint32)
    g = np.zeros(p.size, dtype=np.float64)
    loss = lib().orc_mlp_loss_grad(_f(p), _f(xx), yy.ctypes.data_as(PU), xx.shape[0], int(quant),
                                   _d(g))
    return loss, g


def patch_tables():
    A = np.zeros((32, 3), np.int32)
    B = np.zeros((32, 3), np.int32)
    Bn = np.zeros((32, 6), np.int32)
    Ab = np.zeros((32, 3), np.int32)
    lib().orc_patch_tables(_i(A), _i(B), _i(Bn), _i(Ab))
    return A, B, Bn, Ab


def patch_offsets(seed, stream, t):
    o = np.zeros(3, np.int32)
    lib().orc_patch_offsets(seed, stream, t, _i(o))
    return o


def patch_gather(sp, L, off, i, j, k, k4):
    """(x[128], boundary bits[3], A bits, B bits) of patch (i, j, k) of one replica's
    colour-split uint8 spins."""
    spa = np.ascontiguousarray(sp, dtype=np.uint8)
    LL = np.ascontiguousarray(L, dtype=np.int32)
    oo = np.ascontiguousarray(off, dtype=np.int32)
    x = np.zeros(128, np.float32)
    bnd = np.zeros(3, np.uint32)
    a = np.zeros(1, np.uint32)
    b = np.zeros(1, np.uint32)
    lib().orc_patch_gather(spa.ctypes.data_as(PU8), _i(LL), _i(oo), i, j, k, k4, _f(x),
                           bnd.ctypes.data_as(PU), a.ctypes.data_as(PU), b.ctypes.data_as(PU))
    return x, bnd, int(a[0]), int(b[0])


def patch_sweep(sp, L, betaJ, logits, seed, stream, t):
    """One learned sweep (both classes) of one replica in place; returns accepted patches."""
    assert sp.dtype == np.uint8 and sp.flags.c_contiguous
    LL = np.ascontiguousarray(L, dtype=np.int32)
    z = np.ascontiguousarray(logits, dtype=np.float32)
    return lib().orc_patch_sweep(sp.ctypes.data_as(PU8), _i(LL), betaJ, _f(z), seed, stream, t)


def patch_chain(L, betaJ, nsteps, nequil, use_patch, zscale=0.0, zbias=0.0, seed=1):
    LL = np.ascontiguousarray(L, dtype=np.int32)
    out = np.zeros(5)
    lib().orc_patch_chain(_i(LL), betaJ, nsteps, nequil, int(use_patch), zscale, zbias, seed,
                          _d(out))
    return {"e": out[0], "e_err": out[1], "m": out[2], "m_err": out[3], "accept": out[4]}


# ----------------------------------------------------- the XYZ learned proposal ----
def xmlp_n_params():
    return lib().orc_xmlp_n_params()


def xmlp_forward(params, x, quant=True):
    """vMF parameters m (B, 96) of the XYZ network on inputs x (B, 304), output bias included.
    quant: False FP64; True BF16 weights and hidden activations; 2 also BF16 hidden biases
    (the GPU inference path)."""
    p = np.ascontiguousarray(params, dtype=np.float32)
    xx = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, 304)
    z = np.zeros((xx.shape[0], 96), dtype=np.float32)
    lib().orc_xmlp_forward(_f(p), _f(xx), xx.shape[0], int(quant), _f(z))
    return z


def xmlp_loss_grad(params, x, y, quant=True):
    """Mean vMF negative log density of the targets y (B, 96) and its FP64 gradient."""
    p = np.ascontiguousarray(params, dtype=np.float32)
    xx = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, 304)
    yy = np.ascontiguousarray(y, dtype=np.float32).reshape(-1, 96)
    g = np.zeros(p.size, dtype=np.float64)
    loss = lib().orc_xmlp_loss_grad(_f(p), _f(xx), _f(yy), xx.shape[0], int(quant), _d(g))
    return loss, g


def vmf_logpdf(m, x):
    return lib().orc_vmf_logpdf(*[float(v) for v in m], *[float(v) for v in x])


def vmf_sample(m, u, v):
    out = np.zeros(3, np.float32)
    lib().orc_vmf_sample(*[float(c) for c in m], float(u), float(v), _f(out))
    return out


def xpatch_sweep(sp4, L, beta, J, mdump, seed, stream, t):
    """One XYZ learned sweep (both classes) of one replica in place: sp4 (N, 4) float32 spins
    in storage order; mdump (2, Pc, 96) the vMF parameters the GPU used.  Returns the
    accepted patches."""
    assert sp4.dtype == np.float32 and sp4.flags.c_contiguous
    LL = np.ascontiguousarray(L, dtype=np.int32)
    JJ = np.ascontiguousarray(J, dtype=np.float32)
    m = np.ascontiguousarray(mdump, dtype=np.float32)
    return lib().orc_xpatch_sweep(_f(sp4), _i(LL), float(beta), _f(JJ), _f(m), seed, stream, t)
