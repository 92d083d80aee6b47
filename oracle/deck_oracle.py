"""Pure-Python restatement of the reference's input readers and output writers.

TEST INFRASTRUCTURE ONLY: tests/ use it as the checker of ether_run (the product never
imports anything under oracle/).  Each function follows the Fortran routine it names;
nothing here is shared with the C++ reader (ether_gb300/csrc/deck.cpp), so the two are
independent restatements of the same files.

Parity is unpinned against the reference itself: the reference is Fortran and no Fortran
compiler exists here, so the readers are pinned only by the reference's own example decks
(parsed by both restatements) and by the behaviour read from the sources.
"""
import math
import os
import struct

import numpy as np

KB = 8.617333262e-5         # src/init.f90:47
MB = 5.7883818060e-5        # src/parameters.f90:39
PI = 4.0 * math.atan(1.0)   # src/init.f90:44


# --------------------------------------------------------------------- text utilities ----
def lu(text, case):
    """src/lu.f90: ASCII letters to upper ('U') or lower ('L') case."""
    return text.upper() if case == "U" else text.lower()


def process_file(lines):
    """src/process_file.f90:44-68: each line is character(len=200); scanning stops at '!'
    or '#' (the line keeps what came before), tabs become blanks; blank lines are dropped."""
    out = []
    for line in lines:
        tag = line[:200]
        kept = ""
        for ch in tag:
            if ch == "\t":
                ch = " "
            if ch in "!#":
                break
            kept += ch
        if kept.strip() != "":
            out.append(kept)
    return out


def count_species(line):
    """src/count_species.f90: the number of blank-separated words of a line."""
    return len(line.split())


def split_values(record):
    """The values of one list-directed record (separators: blanks, commas; quotes; r*c)."""
    vals = []
    i, n = 0, len(record)
    while i < n:
        c = record[i]
        if c in " ,\t":
            i += 1
            continue
        if c == "/":
            break
        if c in "'\"":
            j = i + 1
            tok = ""
            while j < n:
                if record[j] == c:
                    if j + 1 < n and record[j + 1] == c:
                        tok += c
                        j += 2
                        continue
                    j += 1
                    break
                tok += record[j]
                j += 1
            vals.append(tok)
            i = j
            continue
        j = i
        while j < n and record[j] not in " ,\t/":
            j += 1
        tok = record[i:j]
        i = j
        head, star, tail = tok.partition("*")
        if star and head.isdigit():
            vals.extend([tail] * int(head))
        else:
            vals.append(tok)
    return vals


class Records:
    """A sequential formatted file read with list-directed READ statements."""

    def __init__(self, path, name):
        with open(path, "rb") as f:
            self.lines = [l.decode("latin-1").rstrip("\r") for l in f.read().split(b"\n")]
        if self.lines and self.lines[-1] == "":
            self.lines.pop()
        self.at = 0
        self.name = name

    def read(self, n, what):
        vals = []
        while len(vals) < n:
            if self.at >= len(self.lines):
                raise DeckError("%s: end of file while reading %s" % (self.name, what))
            vals += split_values(self.lines[self.at])
            self.at += 1
        return vals[:n]

    def skip_blank(self):
        while self.at < len(self.lines) and not split_values(self.lines[self.at]):
            self.at += 1
        return self.at >= len(self.lines)


class DeckError(Exception):
    pass


def real(tok):
    t = tok
    for a in "dDqQ":
        t = t.replace(a, "e")
    try:
        return float(t)
    except ValueError:
        raise DeckError("cannot read a real from %r" % tok)


def integer(tok):
    try:
        return int(tok)
    except ValueError:
        raise DeckError("cannot read an integer from %r" % tok)


def logical(tok):
    t = tok[1:] if tok.startswith(".") else tok
    if t[:1] in ("t", "T"):
        return True
    if t[:1] in ("f", "F"):
        return False
    raise DeckError("cannot read a logical from %r" % tok)


def char_var(tok, length):
    """A value stored in character(len=length), first letter upper and second lower (lu)."""
    s = (tok[:length]).ljust(length)
    s = lu(s[0], "U") + (lu(s[1], "L") if length > 1 else "") + s[2:]
    return s.rstrip(" ")


# --------------------------------------------------------------------------- readers ----
def defaults():
    """src/defaults.f90 (plus the module defaults of src/init.f90)."""
    return dict(model="ising", ising=True, xyz=False, model_fallback=False, tmcs=5000,
                tmcs_eq=3000, ht=100.0, lt=10.0, tint=5.0, s=[], species_to_include=[],
                sc=[2, 2, 2], bc=["c", "c", "c"], repeat=10, angle=False, dphi=0.0, coa=10.0,
                zeeman=False, h=[0.0, 0.0, 0.0], g_factor=2.0, stg=False, sia=False,
                para=False, j_para=1.0, ovrr=False, ovrr_para=0.0, ovrr_mcs=0, seed=1992,
                nbdfc=0.00001, pt=False, exchange_interval=11, cb=False, ss_dis=4.0,
                ss_lat=2.0, ss_direc=[0.0, 0.0, 1.0], ssp=False, spiral_capacity=5,
                nbd_capacity=20, kb=KB, mb=MB)


def get_tot_species(path):
    """src/get_tot_species.f90: line 7 of structure.vasp."""
    with open(path, "rb") as f:
        lines = f.read().decode("latin-1").split("\n")
    if len(lines) < 7:
        raise DeckError("structure.vasp: fewer than 7 lines")
    n = count_species(lines[6].rstrip("\r"))
    if n < 1:
        raise DeckError("structure.vasp: no ion counts on line 7")
    return n


def read_structure(d, path, nsp):
    """src/read_structure.f90:43-95 with src/frac_to_cart.f90:39-45."""
    f = Records(path, "structure.vasp")
    f.read(1, "title")
    f.read(1, "scale")
    abc = np.zeros((3, 3))
    for i in range(3):
        abc[i] = [real(t) for t in f.read(3, "lattice vector")]
    species = [char_var(t, 2) for t in f.read(nsp, "species")]
    ions = [integer(t) for t in f.read(nsp, "ions")]
    if any(n < 0 for n in ions):
        raise DeckError("negative ion count")
    label = lu(f.read(1, "label")[0], "L")
    cart = []
    for _ in range(sum(ions)):
        p = [real(t) for t in f.read(3, "coordinates")]
        if label == "direct":
            cart.append([abc[0, k] * p[0] + abc[1, k] * p[1] + abc[2, k] * p[2] for k in range(3)])
        elif label == "cartesian":
            cart.append(p)
        else:
            raise DeckError("Incorrect structure file")
    if label not in ("direct", "cartesian"):
        raise DeckError("Incorrect structure file")
    d.update(abc=abc, species=species, ions=ions, cart=np.array(cart).reshape(-1, 3),
             atom_species=[k + 1 for k in range(nsp) for _ in range(ions[k])])


def read_input(d, path, nsp):
    """src/read_input.f90:42-148."""
    if not os.path.exists(path):
        raise DeckError("Required file 'in.ether' is not present")
    with open(path, "rb") as f:
        raw = [l.rstrip("\r") for l in f.read().decode("latin-1").split("\n")]
    if raw and raw[-1] == "":
        raw.pop()
    d["s"] = [0.0] * nsp
    for line in process_file(raw):
        text = lu(line, "L")
        j = text.find("=")
        if j < 0:
            raise DeckError("Missing '=' in the given line")
        key, value = text[:j].strip(" "), text[j + 1:]
        v = split_values(value)

        def need(n):
            if len(v) < n:
                raise DeckError("too few values for " + key)

        if key == "model":
            need(1)
            d["model"] = v[0][:5]
            d["ising"], d["xyz"] = d["model"] == "ising", d["model"] == "xyz"
        elif key == "mcs":
            need(2)
            d["tmcs"], d["tmcs_eq"] = integer(v[0]), integer(v[1])
            if d["tmcs"] <= d["tmcs_eq"]:
                raise DeckError("TOTAL MCS  < EQUILIBRATIONS MCS steps")
        elif key == "temp":
            need(3)
            d["ht"], d["lt"], d["tint"] = real(v[0]), real(v[1]), real(v[2])
        elif key == "spin":
            need(nsp)
            d["s"] = [real(t) for t in v[:nsp]]
        elif key == "species":
            n = count_species(value)
            need(n)
            d["species_to_include"] = [char_var(t, 2) for t in v[:n]]
        elif key == "sc":
            need(3)
            d["sc"] = [integer(t) for t in v[:3]]
        elif key == "stg":
            need(1)
            d["stg"] = logical(v[0])
        elif key == "bc":
            need(3)
            d["bc"] = [t[:1] if t else " " for t in v[:3]]
        elif key == "repeat":
            need(1)
            d["repeat"] = integer(v[0])
        elif key == "angle":
            need(2)
            d["angle"] = logical(v[0])
            d["dphi"] = (PI / 180.0) * real(v[1])
        elif key == "coa":
            need(1)
            d["coa"] = real(v[0])
        elif key == "zeeman":
            need(4)
            d["zeeman"] = logical(v[0])
            d["h"] = [real(t) for t in v[1:4]]
        elif key == "g_factor":
            need(1)
            d["g_factor"] = real(v[0])
        elif key == "sia":
            need(1)
            d["sia"] = logical(v[0])
        elif key == "para":
            need(2)
            d["para"] = logical(v[0])
            d["j_para"] = abs(real(v[1]))
            if d["j_para"] == 0 and d["para"]:
                raise DeckError("parameter value is set ON and value cannot be zero")
        elif key == "ovrr":
            need(3)
            d["ovrr"], d["ovrr_para"], d["ovrr_mcs"] = logical(v[0]), abs(real(v[1])), integer(v[2])
        elif key == "seed":
            need(1)
            d["seed"] = integer(v[0])
        elif key == "nbdfc":
            need(1)
            d["nbdfc"] = real(v[0])
        elif key == "pt":
            need(2)
            d["pt"], d["exchange_interval"] = logical(v[0]), integer(v[1])
        elif key == "cb":
            need(1)
            d["cb"] = logical(v[0])
        elif key == "ss_dis":
            need(1)
            d["ss_dis"] = real(v[0])
        elif key == "ss_lat":
            need(1)
            d["ss_lat"] = real(v[0])
        elif key == "ss_direc":
            need(3)
            d["ss_direc"] = [real(t) for t in v[:3]]
        elif key == "ssp":
            need(1)
            d["ssp"] = logical(v[0])
        elif key == "spiral_capacity":
            need(1)
            d["spiral_capacity"] = integer(v[0])
        elif key == "nbd_capacity":
            need(1)
            d["nbd_capacity"] = integer(v[0])
        else:
            raise DeckError("Found unknown/missing information: " + text.strip())
    if not d["ising"] and not d["xyz"]:   # src/startup.f90:36-43
        d.update(model="xyz", xyz=True, model_fallback=True)


def include_species(d):
    """src/generate_supercell.f90:66-99: the included species and the basis atoms."""
    nsp = len(d["species"])
    start = np.concatenate([[0], np.cumsum(d["ions"])]).astype(int)
    included, basis = [], []
    for name in d["species_to_include"]:
        found = 0
        for j in range(nsp):
            if name == d["species"][j]:
                found = j + 1
                basis += list(range(start[j] + 1, start[j + 1] + 1))
        included.append(found)
    if not basis:
        raise DeckError("Selected ions from 'in.ether' are not present in 'structure.vasp' file")
    d.update(included_id=included, basis_atom=basis)


def _species_id(d, name3, stale):
    """Comparison of a character(len=3) symbol with the len=2 species names (blank padded)."""
    if len(name3) > 2:
        return stale
    hit = stale
    for k, sp in enumerate(d["species"]):
        if sp == name3:
            hit = k + 1
    return hit


def j_values(d, path):
    """src/j_values.f90:46-86."""
    if not os.path.exists(path):
        raise DeckError("Required file 'j_exchange' is not present")
    f = Records(path, "j_exchange")
    nsp = len(d["species"])
    nsh = integer(f.read(1, "bonds")[0])
    if nsh < 0:
        raise DeckError("negative bond count")
    dis = np.zeros(nsh)
    jx = np.zeros((3, nsp, nsp, nsh))  # Fortran j_exc(nsh, nsp, nsp, 3) in C order
    jid = [0, 0]
    for i in range(nsh):
        t = f.read(2, "bond")
        dis[i], similar = real(t[0]), integer(t[1])
        for _ in range(similar):
            t = f.read(5, "bond line")
            for a in range(2):
                jid[a] = _species_id(d, char_var(t[a], 3), jid[a])
            if 0 in jid:
                raise DeckError("unknown species in j_exchange")
            an = [real(x) for x in t[2:5]]
            for c in range(3):
                val = an[c] * d["s"][jid[0] - 1] * d["s"][jid[1] - 1]
                jx[c, jid[1] - 1, jid[0] - 1, i] = val
                jx[c, jid[0] - 1, jid[1] - 1, i] = val
    d.update(nsh=nsh, nbd_dis=dis, j_exc=jx)


def get_sia_values(d, path):
    """src/get_sia_values.f90:32-62."""
    nsp = len(d["species"])
    sia = np.zeros((nsp, 3))
    if d["sia"] and d["xyz"]:
        if not os.path.exists(path):
            raise DeckError("SIA is .TRUE. but file 'single_ion_anisotropy' is not found")
        f = Records(path, "single_ion_anisotropy")
        sid = 0
        while not f.skip_blank():
            t = f.read(4, "SIA")
            sid = _species_id(d, char_var(t[0], 2), sid)
            if sid == 0:
                raise DeckError("unknown species in single_ion_anisotropy")
            sia[sid - 1] = [real(x) * d["s"][sid - 1] ** 2 for x in t[1:4]]
    d["sia_vec"] = sia


def get_staggered_info(d, path):
    """src/get_staggered_info.f90:35-57 (the per-species values)."""
    stg = [1.0] * len(d["species"])
    if not d["cb"] and d["stg"] and os.path.exists(path):
        f = Records(path, "staggered")
        for _ in range(len(f.lines)):
            if f.skip_blank():
                break
            t = f.read(2, "staggered")
            val, k = real(t[0]), _species_id(d, char_var(t[1], 3), 0)
            if k:
                stg[k - 1] = val
    d["stg_id"] = stg


def parameters(d):
    """src/parameters.f90:26-55."""
    if d["para"]:
        d["j_exc"] = d["j_exc"] / d["j_para"]
        if d["sia"] and d["xyz"]:
            d["sia_vec"] = d["sia_vec"] / d["j_para"]
        d["kb"], d["mb"], d["g_factor"] = 1.0, 1.0, 1.0
        if d["zeeman"]:
            d["h"] = [x / d["j_para"] for x in d["h"]]
    else:
        d["j_exc"] = d["j_exc"] / 1000.0
        if d["sia"] and d["xyz"]:
            d["sia_vec"] = d["sia_vec"] / 1000.0
        d["mb"] = MB


def read_deck(directory):
    """The input half of src/ether.f90:54-76, in its order."""
    d = defaults()
    spath = os.path.join(directory, "structure.vasp")
    if not os.path.exists(spath):
        raise DeckError("Required file 'structure.vasp' is not present")
    nsp = get_tot_species(spath)
    read_structure(d, spath, nsp)
    read_input(d, os.path.join(directory, "in.ether"), nsp)
    include_species(d)
    j_values(d, os.path.join(directory, "j_exchange"))
    get_sia_values(d, os.path.join(directory, "single_ion_anisotropy"))
    get_staggered_info(d, os.path.join(directory, "staggered"))
    parameters(d)
    d["nscan"] = int(math.floor((d["ht"] - d["lt"]) / d["tint"] + 0.5)) if \
        (d["ht"] - d["lt"]) / d["tint"] >= 0 else -int(math.floor(-(d["ht"] - d["lt"]) / d["tint"] + 0.5))
    d["nscan"] += 1
    return d


def g17(x):
    return "%.17g" % x


def listing(d):
    """The normalised listing ether_run writes as deck.txt."""
    def L(k, vals):
        return k + " =" + "".join(" " + v for v in vals) + "\n"

    def D(k, vals):
        return L(k, [g17(float(v)) for v in vals])

    def I(k, vals):
        return L(k, [str(int(v)) for v in vals])

    def B(k, b):
        return L(k, ["1" if b else "0"])

    jx = np.asarray(d["j_exc"])          # (3, nsp, nsp, nsh) C order == Fortran order flat
    sia = np.asarray(d["sia_vec"])       # (nsp, 3) C order == Fortran sia_vec(3, nsp)
    out = [L("model", [d["model"]]), B("model_fallback", d["model_fallback"]),
           I("mcs", [d["tmcs"], d["tmcs_eq"]]), D("temp", [d["ht"], d["lt"], d["tint"]]),
           I("n_temperatures", [d["nscan"]]), D("spin", d["s"]),
           L("species_to_include", d["species_to_include"]), I("sc", d["sc"]), L("bc", d["bc"]),
           I("repeat", [d["repeat"]]), B("angle", d["angle"]), D("dphi", [d["dphi"]]),
           D("coa", [d["coa"]]), B("zeeman", d["zeeman"]), D("h", d["h"]),
           D("g_factor", [d["g_factor"]]), B("stg", d["stg"]), B("sia", d["sia"]),
           B("para", d["para"]), D("j_para", [d["j_para"]]), B("ovrr", d["ovrr"]),
           D("ovrr_para", [d["ovrr_para"]]), I("ovrr_mcs", [d["ovrr_mcs"]]), I("seed", [d["seed"]]),
           D("nbdfc", [d["nbdfc"]]), B("pt", d["pt"]), I("exchange_interval", [d["exchange_interval"]]),
           B("cb", d["cb"]), D("ss_dis", [d["ss_dis"]]), D("ss_lat", [d["ss_lat"]]),
           D("ss_direc", d["ss_direc"]), B("ssp", d["ssp"]), I("spiral_capacity", [d["spiral_capacity"]]),
           I("nbd_capacity", [d["nbd_capacity"]]), D("abc", np.asarray(d["abc"]).ravel()),
           L("species", d["species"]), I("ions", d["ions"]), D("cart", np.asarray(d["cart"]).ravel()),
           I("included_id", d["included_id"]), I("basis_atom", d["basis_atom"]),
           I("n_basis", [len(d["basis_atom"])]), D("nbd_dis", d["nbd_dis"]), D("j_exc", jx.ravel()),
           D("sia_vec", sia.ravel()), D("stg_id", d["stg_id"]), D("kb", [d["kb"]]), D("mb", [d["mb"]])]
    return "".join(out)


def basis(d):
    """Basis positions and species of the included atoms, in basis order."""
    idx = np.asarray(d["basis_atom"]) - 1
    return np.asarray(d["cart"])[idx], np.asarray(d["atom_species"])[idx]


# ------------------------------------------------------------------- edit descriptors ----
def _special(x, w):
    s = "NaN" if math.isnan(x) else ("-Infinity" if x < 0 else "Infinity")
    if len(s) > w:
        s = "NaN" if math.isnan(x) else ("-Inf" if x < 0 else "Inf")
    return "*" * w if len(s) > w else s.rjust(w)


def F(x, w, d):
    """Fw.d"""
    x = float(x)
    if not math.isfinite(x):
        return _special(x, w)
    s = "%.*f" % (d, x)
    return "*" * w if len(s) > w else s.rjust(w)


def ES(x, w, d):
    """ESw.d"""
    x = float(x)
    if not math.isfinite(x):
        return _special(x, w)
    m, e = ("%.*E" % (d, x)).split("E")
    e = int(e)
    s = m + ("E%+03d" % e if abs(e) <= 99 else "%+04d" % e)
    return "*" * w if len(s) > w else s.rjust(w)


def I(v, w):
    """Iw"""
    s = "%d" % v
    return "*" * w if len(s) > w else s.rjust(w)


def A(s, length, w):
    """Aw of a character(len=length) variable."""
    t = s.encode("utf-8").ljust(length, b" ")[:length]
    out = t[:w] if w <= length else b" " * (w - length) + t
    return out.decode("utf-8", errors="surrogateescape")


# --------------------------------------------------------------------------- writers ----
def nbd_dat(d, nn, n_sites):
    """src/write_nbd.f90:29-61; nn in the reference layout nn(nsh, N, 0:cap, 0:1) as a C
    array of shape (2, cap + 1, N, nsh)."""
    pad = " " * 24
    head = [" # This file can be used to confirm the neighbourhood " + pad + "details of any selected",
            " # central ion with ion number (<ION no.>).",
            " # [NOTE: The content of nbd.dat is independent of the " + pad +
            "species labels present in 'structure.vasp'.",
            " # The contents of nbd.dat depend only on the bond " + pad +
            "lengths provided in the 'j_exchange' file.]",
            " # To visualize the structure, use the 'VESTA' software " + pad +
            "(https://jp-minerals.org/vesta/en/download.html)",
            " # and open the generated 'fetched_lattice_network.xsf' file.",
            " # Check the neighbourhood details (given in this file) " + pad +
            "using the <Atom Label> for the selected central <ION no.> IDs.", " "]
    out = [l + "\n" for l in head]
    for i in range(n_sites):
        out.append(" ION no. " + I(i + 1, 5) + "\n")
        out.append(" ~~~~~~~~~~~~~~\n")
        for m in range(d["nsh"]):
            cnt = nn[0, 0, i, m]
            ids = "".join(I(nn[0, k, i, m], 7) for k in range(1, cnt + 1))
            out.append(" For bond length: " + F(d["nbd_dis"][m], 12, 8) + ", nbds are ==> " + ids + "\n")
        out.append(" \n")
    return "".join(out)


def read_obs(path, n_species):
    """ETHER.obs (src/process_observables.f90:34-77): one record of 20 + 3 nsp doubles per
    temperature, no record markers."""
    raw = open(path, "rb").read()
    n = 20 + 3 * n_species
    vals = np.frombuffer(raw, dtype="<f8")
    assert vals.size % n == 0
    return vals.reshape(-1, n)


def read_spn(path, n_sites):
    """ETHER.spn (src/rw_file.f90): one record ion(0:8, N) per temperature."""
    vals = np.frombuffer(open(path, "rb").read(), dtype="<f8")
    assert vals.size % (9 * n_sites) == 0
    return vals.reshape(-1, n_sites, 9)


def output_files(d, obs, spn, ion0):
    """magnetization.dat, energy.dat, moment_vectors.dat, spiral_state_parameters.dat and
    gss.dat from the ETHER.obs / ETHER.spn records (src/write_output_files.f90,
    src/write_gss.f90)."""
    nsp = len(d["species"])
    n_sites = ion0.shape[0]
    tions = [int((ion0[:, 4] == k + 1).sum()) for k in range(nsp)]
    ssp = d["ssp"] and d["xyz"]
    m_head = ["# 1 Temp.", "2 |M|", "3 χ", "4 Δ|M|", "5 Δχ", "6 U(|M|)", "7 ΔU(|M|)"]
    ss_head = ["# 1 Temp.", "2 |ψ|", "3 ψ", "4 Δ|ψ|", "5 Δψ", "6 U(|ψ|)",
               "7 ΔU(|ψ|)"]
    e_head = ["# 1 Temp.", "2 E", "3 Cv" if d["para"] else "3 Cv/kB", "4 ΔE",
              "5 ΔCv" if d["para"] else "5 Δ(Cv/kB)", "6 U(E)", "7 ΔU(E)", "8 Accpt. (%)"]

    def fmt103(h):
        a = [A(x, 20, 13) for x in h]
        return a[0] + a[1] + a[2] + " " + a[3] + " " + a[4] + "  " + a[5] + a[6] + "\n"

    mag = fmt103(m_head)
    ea = [A(x, 20, 13) for x in e_head]
    eng = ea[0] + ea[1] + ea[2] + ea[3] + " " + ea[4] + " " + ea[5] + ea[6] + ea[7] + "\n"
    sss = fmt103(ss_head) if ssp else ""
    mom = " # Showing moment vectors (Mx, My, Mz) for species(sp):\n"
    names = [d["species"][i - 1] if i > 0 else "" for i in d["included_id"]]
    for k in range(0, max(len(names), 1), 5):
        mom += " #\t" + "".join(A(nm, 2, 3) for nm in names[k:k + 5]) + "\n"
    mom += " # Temp, sp1(Mx,My,Mz), sp1(Mx,My,Mz),..spN(Mx,My,Mz), sp1|M|, sp2|M|,..spN|M|\n"
    sc = d["sc"]
    gss = " ".join(I(v, 5) for v in [d["nscan"]] + list(sc)) + "\n"
    gss += " ".join(I(v, 5) for v in [1, 1, 1] + list(sc)) + "\n"
    gss += I(len(d["basis_atom"]), 5) + " " + I(nsp, 5) + F(d["ht"], 11, 5) + " " + F(d["lt"], 11, 5) + " " + \
        F(d["tint"], 11, 5) + "\n"
    gss += A(" KbT/J" if d["para"] else " K", 30, 20) + "\n"
    for k in range(0, nsp, 5):
        gss += " ".join(I(v, 8) for v in tions[k:k + 5]) + "\n"
    for i in range(3):
        gss += " ".join(F(v, 10, 5) for v in np.asarray(d["abc"])[i]) + "\n"
    gss += " # lattice points\n"
    for i in range(n_sites):
        gss += " ".join(F(v, 11, 6) for v in ion0[i, 6:9]) + " " + I(int(ion0[i, 0]), 8) + "\n"
    for t in range(obs.shape[0]):
        o = obs[t]
        mag += F(o[0], 11, 5) + "".join(" " + ES(o[k], 12, 5) for k in range(1, 7)) + "\n"
        eng += F(o[0], 11, 5) + "".join(" " + ES(o[k], 12, 5) for k in range(7, 13)) + " " + F(o[13], 7, 2) + "\n"
        if ssp:
            sss += F(o[0], 11, 5) + "".join(" " + ES(o[k], 12, 5) for k in range(14, 20)) + "\n"
        row = F(o[0], 11, 5) + "  "
        inc = [i for i in d["included_id"] if i > 0]
        for i in inc:
            row += "".join(F(o[20 + 3 * (i - 1) + a] / tions[i - 1], 9, 3) for a in range(3))
        for i in inc:
            m = o[20 + 3 * (i - 1):23 + 3 * (i - 1)]
            row += F(math.sqrt(float(np.dot(m, m))) / tions[i - 1], 9, 3)
        mom += row + "\n"
        gss += F(o[0], 11, 5) + "\n"
        for i in range(n_sites):
            gss += " ".join(F(v, 11, 6) for v in spn[t, i, 1:4]) + " " + I(int(spn[t, i, 4]), 8) + "\n"
    return {"magnetization.dat": mag, "energy.dat": eng, "moment_vectors.dat": mom,
            "spiral_state_parameters.dat": sss, "gss.dat": gss}


def spk_name(temp):
    """src/write_spins_at_K.f90:34: format(f9.4, 'spK.xsf') then adjustl."""
    return (F(temp, 9, 4) + "spK.xsf").strip()


def spk_rows(d, cfg):
    """src/write_spins_at_K.f90:52-60: (A5, 1x, f13.7 x6 with 1x) per site."""
    return "".join(A(d["species"][int(r[4]) - 1], 2, 5) + "".join(" " + F(r[k], 13, 7) for k in (6, 7, 8, 1, 2, 3))
                   + "\n" for r in cfg)


def per_repeat(vals):
    """src/observables_per_repeat.f90: vals (repeat, q) -> mean (q,), err (q,)."""
    vals = np.asarray(vals, dtype=np.float64)
    rep = vals.shape[0]
    mean = vals.sum(0) / rep
    with np.errstate(divide="ignore", invalid="ignore"):
        r1 = np.float64(1.0) / (rep * (rep - 1.0))
        err = np.sqrt(r1 * ((vals - mean) ** 2).sum(0))
    return mean, err


def pack_record(values):
    return struct.pack("<%dd" % len(values), *values)
