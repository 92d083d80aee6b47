"""Host-side mirror of the reference's set-up for the sweep, on top of the C-ABI.

`Lattice` replaces generate_supercell + getting_nbd (src/generate_supercell.f90,
src/getting_nbd.f90) through ether_build_lattice; `couplings` replaces j_values.f90 +
parameters.f90; `Sweep` owns one ether_ctx and exposes the reference's per-MCS routines
under their reference names.  Arrays keep the reference's Fortran layouts:
    ion      (N, 9)                 ion(0:8, N)
    nn       (2, cap+1, N, nsh)     nn(nsh, N, 0:cap, 0:1)
    j_exc    (3, nsp, nsp, nsh)     j_exc(nsh, nsp, nsp, 3)
    sia_vec  (nsp, 3)               sia_vec(3, nsp)
"""
import ctypes as C
import math
import os

import numpy as np

from . import abi

KB_EV = 8.617333262e-5      # src/init.f90:47
MB_EV = 5.7883818060e-5     # src/parameters.f90:41


class Lattice:
    """Supercell + neighbour shells built by ether_build_lattice (O(N))."""

    def __init__(self, basis_cart, basis_species, abc, sc, shells, bc="ccc", checkerboard=False,
                 tol=1e-5, cap=20):
        lib = abi.load()
        self.basis_cart = np.ascontiguousarray(basis_cart, dtype=np.float64).reshape(-1, 3)
        self.nbasis = self.basis_cart.shape[0]
        self.basis_species = np.ascontiguousarray(basis_species, dtype=np.int32)
        self.abc = np.ascontiguousarray(abc, dtype=np.float64).reshape(3, 3)
        self.sc = np.ascontiguousarray(sc, dtype=np.int32)
        self.shells = np.ascontiguousarray(shells, dtype=np.float64)
        self.nsh = len(self.shells)
        self.cap = int(cap)
        self.bc = bc
        self.tol = float(tol)
        self.checkerboard = bool(checkerboard)
        self.N = int(np.prod(self.sc)) * self.nbasis
        self.ion = np.zeros((self.N, 9), dtype=np.float64)
        self.stgg = np.zeros(self.N, dtype=np.float64)
        self.nn = np.zeros((2, self.cap + 1, self.N, max(self.nsh, 1)), dtype=np.int32)
        abi.check(lib.ether_build_lattice(
            self.nbasis, abi.dptr(self.basis_cart), abi.iptr(self.basis_species),
            abi.dptr(self.abc), abi.iptr(self.sc), bc.encode(), int(self.checkerboard), self.nsh,
            abi.dptr(self.shells), self.tol, self.cap, abi.dptr(self.ion), abi.dptr(self.stgg),
            abi.iptr(self.nn)))

    @property
    def n_species(self):
        return int(self.basis_species.max())


def simple_cubic(L, bc="ccc", checkerboard=False, cap=20):
    L = (L, L, L) if np.isscalar(L) else tuple(L)
    return Lattice([[0.0, 0.0, 0.0]], [1], np.eye(3), L, [1.0], bc=bc,
                   checkerboard=checkerboard, cap=cap)


PYROCHLORE_FRAC = [
    (0.0, 0.0, 0.0), (0.750000028, 0.25, 0.5), (0.25, 0.750000028, 0.5),
    (0.25, 0.5, 0.750000028), (0.750000028, 0.5, 0.25), (0.5, 0.750000028, 0.25),
    (0.5, 0.25, 0.750000028), (0.0, 0.5, 0.5), (0.750000028, 0.750000028, 0.0),
    (0.25, 0.25, 0.0), (0.25, 0.0, 0.25), (0.750000028, 0.0, 0.750000028),
    (0.5, 0.0, 0.5), (0.0, 0.750000028, 0.750000028), (0.0, 0.25, 0.25), (0.5, 0.5, 0.0),
]
PYROCHLORE_A = 8.4072999954


def pyrochlore(n, shells=(2.97243,), cap=20, tol=1e-5):
    """The 16-site cubic pyrochlore cell of the reference's examples/Pyrochlore deck,
    replicated n x n x n (fractional -> cartesian as src/frac_to_cart.f90)."""
    n = (n, n, n) if np.isscalar(n) else tuple(n)
    abc = np.eye(3) * PYROCHLORE_A
    cart = np.array([[abc[0, d] * f[0] + abc[1, d] * f[1] + abc[2, d] * f[2] for d in range(3)]
                     for f in PYROCHLORE_FRAC])
    return Lattice(cart, [1] * 16, abc, n, list(shells), cap=cap, tol=tol)


def local_111_axes(lat, shell=0):
    """Per-site local easy axes of a lattice of corner-sharing tetrahedra (pyrochlore): the
    unit vector from a site to the centroid of one of its nearest-neighbour triangles (the
    three other corners of a tetrahedron it belongs to), which is the site's local <111>
    direction.  Bond vectors use the minimum image of the periodic supercell.  Returns (N, 3),
    each axis with its first non-zero component positive ((a . S)^2 does not depend on the
    sign)."""
    pos = lat.ion[:, 6:9]
    SC = lat.abc * lat.sc[:, None]          # supercell vectors as rows
    SCinv = np.linalg.inv(SC)
    cnt = lat.nn[0, 0, :, shell]
    nbrs = [set((lat.nn[0, 1:cnt[i] + 1, i, shell] - 1).tolist()) for i in range(lat.N)]
    axes = np.zeros((lat.N, 3))
    for i in range(lat.N):
        nb = sorted(nbrs[i])
        a = nb[0]
        tri = [a] + [j for j in nb[1:] if j in nbrs[a]]
        if len(tri) != 3:
            raise ValueError("site %d: its nearest neighbours do not form triangles" % (i + 1))
        d = pos[tri] - pos[i]
        d -= np.round(d @ SCinv) @ SC
        v = d.sum(axis=0)
        v /= np.linalg.norm(v)
        k = int(np.argmax(np.abs(v) > 1e-9))  # the first non-zero component made positive
        v = v if v[k] > 0 else -v
        # rounded to 1e-9 and renormalised: sites whose axes differ only by the rounding of
        # their bond sums get the same axis (and so share one anisotropy class)
        v = np.round(v, 9)
        axes[i] = v / np.linalg.norm(v)
    return axes


def couplings(n_species, shells, s, para=None):
    """j_values.f90:61-86 + parameters.f90:26-38.

    shells: one entry per bond shell: list of (si, sj, (Jxx, Jyy, Jzz)) in meV, species
    1-based.  j_exc(b,si,sj,:) = J*s(si)*s(sj), symmetric; then divided by J_para when
    `para` is given, else by 1000 (meV -> eV)."""
    nsh = len(shells)
    j = np.zeros((3, n_species, n_species, nsh), dtype=np.float64)
    s = np.asarray(s, dtype=np.float64)
    for b, entries in enumerate(shells):
        for si, sj, J in entries:
            v = np.asarray(J, dtype=np.float64) * s[si - 1] * s[sj - 1]
            j[:, si - 1, sj - 1, b] = v
            j[:, sj - 1, si - 1, b] = v
    j = j / (abs(para) if para else 1000.0)
    return np.ascontiguousarray(j)


def units(para=None):
    """(kB, mB, g override) as parameters.f90 sets them."""
    if para:
        return 1.0, 1.0, 1.0
    return KB_EV, MB_EV, None


class Sweep:
    """One ether_ctx: R replicas of a lattice, advanced by the GPU kernels."""

    def __init__(self, ion, nn, j_exc, s, *, model, n_species, n_shells, cap, replicas=1,
                 seed=1992, angle=False, dphi=0.0, zeeman=False, h=(0.0, 0.0, 0.0),
                 g_factor=2.0, mb=MB_EV, sia=False, sia_vec=None, stgg=None, sc=(0, 0, 0),
                 basis=0, flags=0, sia_local=None):
        self.lib = abi.load()
        self._keep = []

        def keep(a, dt):
            if a is None:
                return None
            a = np.ascontiguousarray(a, dtype=dt)
            self._keep.append(a)
            return a

        ion = keep(ion, np.float64)
        d = abi.Desc()
        d.n_sites = ion.shape[0] if ion.ndim == 2 else ion.size // 9
        d.n_species = n_species
        d.n_shells = n_shells
        d.nbd_capacity = cap
        d.model = model
        d.angle = int(bool(angle))
        d.dphi = float(dphi)
        d.zeeman = int(bool(zeeman))
        for k in range(3):
            d.h[k] = float(h[k])
        d.g_factor = float(g_factor)
        d.mb = float(mb)
        d.sia = int(bool(sia))
        d.ion = abi.dptr(ion)
        d.nn = abi.iptr(keep(nn, np.int32))
        d.j_exc = abi.dptr(keep(j_exc, np.float64))
        d.sia_vec = abi.dptr(keep(sia_vec, np.float64))
        d.s = abi.dptr(keep(s, np.float64))
        d.stgg = abi.dptr(keep(stgg, np.float64))
        d.n_replicas = replicas
        d.seed = seed & 0xFFFFFFFF
        for k in range(3):
            d.sc[k] = int(sc[k])
        d.basis = basis
        d.flags = flags
        d.sia_local = abi.dptr(keep(sia_local, np.float64))  # (N, 4): axis, D per site
        self.N = d.n_sites
        self.R = replicas
        self._nsp = n_species
        self.model = model
        h_ = C.c_void_p()
        abi.check(self.lib.ether_create(C.byref(d), C.byref(h_)))
        self.h = h_
        self._keep = []

    @classmethod
    def from_lattice(cls, lat, j_exc, s, model, **kw):
        kw.setdefault("stgg", lat.stgg)
        return cls(lat.ion, lat.nn, j_exc, s, model=model, n_species=j_exc.shape[1],
                   n_shells=lat.nsh, cap=lat.cap, sc=tuple(int(x) for x in lat.sc),
                   basis=lat.nbasis, **kw)

    def close(self):
        if getattr(self, "h", None):
            self.lib.ether_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- state
    def set_beta(self, beta):
        b = np.ascontiguousarray(np.broadcast_to(np.asarray(beta, np.float64), (self.R,)))
        abi.check(self.lib.ether_set_beta(self.h, abi.dptr(b)))

    def set_ladder(self, beta_slots):
        b = np.ascontiguousarray(beta_slots, dtype=np.float64)
        abi.check(self.lib.ether_set_ladder(self.h, len(b), abi.dptr(b)))

    def set_streams(self, stream=None, step=None):
        st = None if stream is None else np.ascontiguousarray(stream, dtype=np.uint32)
        sp = None if step is None else np.ascontiguousarray(step, dtype=np.uint32)
        abi.check(self.lib.ether_set_streams(self.h, abi.uptr(st), abi.uptr(sp)))

    def set_spins(self, ion, replica=-1):
        ion = np.ascontiguousarray(ion, dtype=np.float64)
        abi.check(self.lib.ether_set_spins(self.h, replica, abi.dptr(ion)))

    def get_spins(self, ion, replica=0):
        out = np.array(ion, dtype=np.float64, copy=True, order="C")
        abi.check(self.lib.ether_get_spins(self.h, replica, abi.dptr(out)))
        return out

    def set_spins_batch(self, ions, r0=0):
        """ions: (n, N, 9) -- ion(0:8, N) of replicas r0 .. r0+n-1 back to back."""
        ions = np.ascontiguousarray(ions, dtype=np.float64)
        abi.check(self.lib.ether_set_spins_batch(self.h, r0, ions.shape[0], abi.dptr(ions)))

    def get_spins_batch(self, ions, r0=0):
        """Fills ions (n, N, 9), C-contiguous float64, in place: ion(1:3, :) and ion(5, :) of
        replicas r0 .. r0+n-1; the other columns keep their values."""
        assert ions.dtype == np.float64 and ions.flags.c_contiguous
        abi.check(self.lib.ether_get_spins_batch(self.h, r0, ions.shape[0], abi.dptr(ions)))
        return ions

    # -- reference routines
    def spins_batch_split(self):
        """Replicas the last get_spins_batch / set_spins_batch moved in place by a kernel."""
        g, st = C.c_int32(0), C.c_int32(0)
        abi.check(self.lib.ether_spins_batch_split(self.h, C.byref(g), C.byref(st)))
        return g.value, st.value

    def fresh_spins(self):
        abi.check(self.lib.ether_fresh_spins(self.h))

    def metropolis(self, nsweeps=1, accept=True):
        out = np.zeros(self.R, dtype=np.float64) if accept else None
        abi.check(self.lib.ether_metropolis(self.h, nsweeps, abi.dptr(out)))
        return out

    def overrelaxation(self, ovrr_para):
        abi.check(self.lib.ether_overrelaxation(self.h, float(ovrr_para)))

    def tot_energy(self):
        out = np.zeros(self.R, dtype=np.float64)
        abi.check(self.lib.ether_tot_energy(self.h, abi.dptr(out)))
        return out

    def tot_magnetisation(self):
        out = np.zeros((self.R, 3), dtype=np.float64)
        abi.check(self.lib.ether_tot_magnetisation(self.h, abi.dptr(out)))
        return out

    def observable(self, step, tmcs_eq, coa):
        abi.check(self.lib.ether_observable(self.h, step, tmcs_eq, coa))

    def zero_avg(self):
        abi.check(self.lib.ether_zero_avg(self.h))

    def sums(self):
        out = np.zeros((self.R, 7), dtype=np.float64)
        abi.check(self.lib.ether_get_sums(self.h, abi.dptr(out)))
        return out

    def avg(self):
        out = np.zeros((self.R, 6), dtype=np.float64)
        abi.check(self.lib.ether_avg(self.h, abi.dptr(out)))
        return out

    def per_repeat(self):
        info = self.info()
        mean = np.zeros((info.n_slots, 6), dtype=np.float64)
        err = np.zeros((info.n_slots, 6), dtype=np.float64)
        abi.check(self.lib.ether_per_repeat(self.h, abi.dptr(mean), abi.dptr(err)))
        return mean, err

    def parallel_tempering(self, swap_count):
        acc = C.c_int32(0)
        abi.check(self.lib.ether_parallel_tempering(self.h, swap_count, C.byref(acc)))
        return acc.value

    def slots(self):
        out = np.zeros(self.R, dtype=np.int32)
        abi.check(self.lib.ether_get_slots(self.h, abi.iptr(out)))
        return out

    def mcs(self, step0, nsteps, tmcs_eq, coa, ovrr=False, ovrr_para=0.0, ovrr_mcs=0, pt=False,
            exchange_interval=11, swap_count=0):
        s = abi.Schedule(tmcs_eq, coa, int(ovrr), float(ovrr_para), ovrr_mcs, int(pt),
                         exchange_interval)
        sc = C.c_int32(swap_count)
        abi.check(self.lib.ether_mcs(self.h, C.byref(s), step0, nsteps, C.byref(sc)))
        return sc.value

    def record_series(self, nsweeps, stride=1, energy=False):
        """nsweeps sweeps; |M| (and E) of every replica after each stride-th sweep.
        Returns arrays of shape (R, nsweeps // stride)."""
        n = nsweeps // stride
        m = np.zeros((n, self.R), dtype=np.float64)
        e = np.zeros((n, self.R), dtype=np.float64) if energy else None
        abi.check(self.lib.ether_record_series(self.h, nsweeps, stride, abi.dptr(m), abi.dptr(e)))
        return (m.T.copy(), e.T.copy()) if energy else m.T.copy()

    def accept_counts(self):
        out = np.zeros(self.R, dtype=np.uint64)
        abi.check(self.lib.ether_get_accept_counts(self.h, out.ctypes.data_as(abi.PU64)))
        return out

    def slot_accept_counts(self):
        """Accepted moves per (group, slot) position, index group * n_slots + slot."""
        out = np.zeros(self.R, dtype=np.uint64)
        abi.check(self.lib.ether_get_slot_accept_counts(self.h, out.ctypes.data_as(abi.PU64)))
        return out

    def reset_accept_counts(self):
        abi.check(self.lib.ether_reset_accept_counts(self.h))

    def info(self):
        i = abi.Info()
        abi.check(self.lib.ether_get_info(self.h, C.byref(i)))
        return i

    def colouring(self):
        col = np.zeros(self.N, dtype=np.int32)
        rank = np.zeros(self.N, dtype=np.int32)
        abi.check(self.lib.ether_get_colouring(self.h, abi.iptr(col), abi.iptr(rank)))
        return col, rank

    def sync(self):
        abi.check(self.lib.ether_sync(self.h))

    def stream(self):
        s = C.c_void_p()
        abi.check(self.lib.ether_get_stream(self.h, C.byref(s)))
        return s.value or 0

    def phase(self, colour):
        abi.check(self.lib.ether_metropolis_phase(self.h, colour))

    def end_sweep(self):
        abi.check(self.lib.ether_end_sweep(self.h))

    def moment_vectors(self):
        """get_moment_vectors: (R, n_species, 3)."""
        out = np.zeros((self.R, self._nsp, 3), dtype=np.float64)
        abi.check(self.lib.ether_moment_vectors(self.h, abi.dptr(out)))
        return out

    def spiral_setup(self, ss_dis, ss_direc=(0.0, 0.0, 1.0), ss_latency=2.0, capacity=5):
        d = np.ascontiguousarray(ss_direc, dtype=np.float64)
        n = C.c_int64(0)
        abi.check(self.lib.ether_spiral_setup(self.h, float(ss_dis), abi.dptr(d), float(ss_latency),
                                              int(capacity), C.byref(n)))
        return n.value

    def spiral_state(self):
        out = np.zeros(self.R, dtype=np.float64)
        abi.check(self.lib.ether_spiral_state(self.h, abi.dptr(out)))
        return out

    def spiral_avg(self):
        """get_spiral_state 'avg_spiral_state' per (group, slot): (R, 3) = <x>, U, chi."""
        out = np.zeros((self.R, 3), dtype=np.float64)
        abi.check(self.lib.ether_spiral_avg(self.h, abi.dptr(out)))
        return out

    def autotune(self):
        v = C.c_int32(0)
        ms = C.c_float(0.0)
        abi.check(self.lib.ether_autotune(self.h, C.byref(v), C.byref(ms)))
        return v.value, ms.value

    def set_variant(self, variant):
        abi.check(self.lib.ether_set_variant(self.h, variant))


class Batch:
    """ether_batch: kernels per member group, colour phase and member class, captured in one
    graph per sweep, advance the Metropolis sweeps of every member Sweep (mixed sizes and
    models), leaving each member exactly as its own metropolis() would.  The members must
    outlive the batch."""

    def __init__(self, members):
        self.lib = abi.load()
        self.members = list(members)
        arr = (C.c_void_p * len(self.members))(*[m.h.value for m in self.members])
        h_ = C.c_void_p()
        abi.check(self.lib.ether_batch_create(arr, len(self.members), C.byref(h_)))
        self.h = h_

    def close(self):
        if getattr(self, "h", None):
            self.lib.ether_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def metropolis(self, nsweeps=1):
        abi.check(self.lib.ether_batch_metropolis(self.h, nsweeps))

    def mcs(self, step0, nsteps, tmcs_eq, coa, ovrr=False, ovrr_para=0.0, ovrr_mcs=0, pt=False,
            exchange_interval=11, swap_counts=None):
        """The MCS loop of every member under one schedule (Sweep.mcs's arguments); returns
        the members' PT swap counters (started from swap_counts, default all 0)."""
        s = abi.Schedule(tmcs_eq, coa, int(ovrr), float(ovrr_para), ovrr_mcs, int(pt),
                         exchange_interval)
        sc = np.zeros(len(self.members), dtype=np.int32)
        if swap_counts is not None:
            sc[:] = swap_counts
        abi.check(self.lib.ether_batch_mcs(self.h, C.byref(s), step0, nsteps, abi.iptr(sc)))
        return sc

    def set_config(self, threads=256, units_per_thread=2, blocks_per_sm=0, walk=0):
        abi.check(self.lib.ether_batch_set_config(self.h, threads, units_per_thread,
                                                  blocks_per_sm, walk))

    def autotune(self):
        cfg = np.zeros(4, dtype=np.int32)
        ms = C.c_float(0.0)
        abi.check(self.lib.ether_batch_autotune(self.h, abi.iptr(cfg), C.byref(ms)))
        return tuple(int(x) for x in cfg), ms.value

    def info(self):
        i = abi.BatchInfo()
        abi.check(self.lib.ether_batch_get_info(self.h, C.byref(i)))
        return i

    def stream(self):
        s = C.c_void_p()
        abi.check(self.lib.ether_batch_get_stream(self.h, C.byref(s)))
        return s.value or 0


N_LEARN_PARAMS = 128 * 128 + 128 + 128 * 128 + 128 + 32 * 128 + 32


class Learned:
    """ether_learn: the learned 4^3-patch proposal of a simple-cubic Ising or Heisenberg (XYZ)
    Sweep, accepted by exact Metropolis-Hastings (the plain sweep stays the fallback;
    interleave the two).  n_in, n_out, n_params: the network's widths (Ising 128, 32, 37152;
    XYZ 304, 96 von Mises-Fisher parameters, 67936)."""

    def __init__(self, sweep, seed=7, capacity=1 << 20):
        self.lib = abi.load()
        self.sweep = sweep
        d = abi.LearnDesc()
        d.patch = 4
        d.hidden = 128
        d.seed = seed & 0xFFFFFFFF
        d.capacity = int(capacity)
        h_ = C.c_void_p()
        abi.check(self.lib.ether_learn_create(sweep.h, C.byref(d), C.byref(h_)))
        self.h = h_
        ni, no, npar = C.c_int32(0), C.c_int32(0), C.c_int32(0)
        abi.check(self.lib.ether_learn_get_shape(self.h, C.byref(ni), C.byref(no), C.byref(npar)))
        self.n_in, self.n_out, self.n_params = ni.value, no.value, npar.value

    def close(self):
        if getattr(self, "h", None):
            self.lib.ether_learn_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def collect(self, per_replica):
        abi.check(self.lib.ether_learn_collect(self.h, per_replica))

    def train(self, steps, batch=1024, lr=1e-3):
        loss = C.c_double(0.0)
        abi.check(self.lib.ether_learn_train(self.h, steps, batch, lr, C.byref(loss)))
        return loss.value

    def sweep_(self, nsweeps=1):
        abi.check(self.lib.ether_learn_sweep(self.h, nsweeps))

    def record_series(self, nsteps, plain_per_step=1, learned_per_step=1, stride=1):
        """|M| of every replica after every stride-th step, shape (R, nsteps // stride)."""
        out = np.zeros((nsteps // stride, self.sweep.R), dtype=np.float64)
        abi.check(self.lib.ether_learn_record_series(self.h, nsteps, plain_per_step,
                                                     learned_per_step, stride, abi.dptr(out)))
        return out.T.copy()

    def accepts(self):
        out = np.zeros(self.sweep.R, dtype=np.uint64)
        abi.check(self.lib.ether_learn_get_accepts(self.h, out.ctypes.data_as(abi.PU64)))
        return out

    def params(self):
        p = np.zeros(self.n_params, dtype=np.float32)
        abi.check(self.lib.ether_learn_get_params(self.h, p.ctypes.data_as(C.POINTER(C.c_float))))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        abi.check(self.lib.ether_learn_set_params(self.h, p.ctypes.data_as(C.POINTER(C.c_float))))

    def loss_grad(self, x, y):
        """Mean training loss and its gradient on inputs x (B, n_in); y: Ising colour-0 bits
        (B,) as unsigned integers, or float targets (B, n_out) (XYZ: spin components)."""
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, self.n_in)
        g = np.zeros(self.n_params, dtype=np.float32)
        loss = C.c_double(0.0)
        y = np.asarray(y)
        if np.issubdtype(y.dtype, np.floating):
            y = np.ascontiguousarray(y, dtype=np.float32).reshape(-1, self.n_out)
            abi.check(self.lib.ether_learn_loss_grad_f(
                self.h, x.ctypes.data_as(C.POINTER(C.c_float)), y.ctypes.data_as(C.POINTER(C.c_float)),
                x.shape[0], C.byref(loss), g.ctypes.data_as(C.POINTER(C.c_float))))
        else:
            y = np.ascontiguousarray(y, dtype=np.uint32)
            abi.check(self.lib.ether_learn_loss_grad(
                self.h, x.ctypes.data_as(C.POINTER(C.c_float)), y.ctypes.data_as(abi.PU32), x.shape[0],
                C.byref(loss), g.ctypes.data_as(C.POINTER(C.c_float))))
        return loss.value, g

    def forward(self, x):
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, self.n_in)
        z = np.zeros((x.shape[0], self.n_out), dtype=np.float32)
        abi.check(self.lib.ether_learn_forward(self.h, x.ctypes.data_as(C.POINTER(C.c_float)),
                                               x.shape[0], z.ctypes.data_as(C.POINTER(C.c_float))))
        return z

    def set_dump(self, on=True):
        abi.check(self.lib.ether_learn_set_dump(self.h, int(bool(on))))

    def dump(self):
        i = self.info()
        z = np.zeros((2, self.sweep.R, i.patches_per_class, self.n_out), dtype=np.float32)
        abi.check(self.lib.ether_learn_get_dump(self.h, z.ctypes.data_as(C.POINTER(C.c_float))))
        return z

    def info(self):
        i = abi.LearnInfo()
        abi.check(self.lib.ether_learn_get_info(self.h, C.byref(i)))
        return i


def learn_batch_sweep(learners, nsweeps=1, plain_per_sweep=1):
    """ether_learn_batch_sweep: the learners' contexts advance together, nsweeps steps of
    plain_per_sweep Metropolis sweeps then one learned sweep each (asynchronous)."""
    lib = abi.load()
    hs = (C.c_void_p * len(learners))(*[l.h.value for l in learners])
    abi.check(lib.ether_learn_batch_sweep(hs, len(learners), nsweeps, plain_per_sweep))


def run(indir, outdir, parse_only=False, ranks=0, resume=False, quiet=True):
    """src/ether.f90 for one input directory (ether_run): reads the deck in indir, runs the
    temperature scan on the GPU and writes the reference's output files into outdir.
    parse_only reads the deck and builds the lattice only (no GPU).  Returns the run info
    as a dict."""
    lib = abi.load()
    info = abi.RunInfo()
    info.ranks = int(ranks)
    flags = ((abi.RUN_PARSE_ONLY if parse_only else 0) | (abi.RUN_QUIET if quiet else 0) |
             (abi.RUN_RESUME if resume else 0))
    abi.check(lib.ether_run(os.fsencode(indir), os.fsencode(outdir), flags, C.byref(info)))
    return {k: getattr(info, k) for k, _ in abi.RunInfo._fields_}
