"""ether_run's input side on the CPU (ETHER_RUN_PARSE_ONLY: no GPU work): the C++ deck
reader against the oracle's Python restatement of src/read_input.f90, src/read_structure.f90,
src/get_tot_species.f90, src/j_values.f90, src/get_sia_values.f90, src/get_staggered_info.f90,
src/parameters.f90 and the species filter of src/generate_supercell.f90, on decks that
exercise the readers' rules; nbd.dat against src/write_nbd.f90 restated over the oracle's
brute-force neighbour search; and the reader's error cases."""
import os

import numpy as np
import pytest

import ether_gb300 as eg
from oracle import deck_oracle as do
from oracle import pyoracle as po

# the reference checkout's examples/ folder, given by the environment; the test that reads it
# is skipped when the variable is unset or the folder is absent
REF_EXAMPLES = os.environ.get("ETHER_REFERENCE_EXAMPLES", "")

SC_STRUCT = """simple cubic
1.0
  1.0 0.0 0.0
  0.0 1.0 0.0
  0.0 0.0 1.0
  A
  1
Direct
  0.0 0.0 0.0
"""


def write_deck(d, in_ether, structure, j_exchange, sia=None, staggered=None):
    os.makedirs(d, exist_ok=True)
    for name, text in (("in.ether", in_ether), ("structure.vasp", structure),
                       ("j_exchange", j_exchange), ("single_ion_anisotropy", sia),
                       ("staggered", staggered)):
        if text is not None:
            with open(os.path.join(d, name), "w", encoding="latin-1") as f:
                f.write(text)
    return d


DECKS = {
    # comments after '!' and '#', tabs, upper-case keys and values, defaults elsewhere
    "sc_ising": (
        "MODEL = Ising\t! the model\nmcs = 400 200\n# a comment line\n\ntemp = 6 4 0.5\n"
        "spin = 1\nspecies = a\nsc = 4 4 4\nPT = .T. 11\t\t# exchange\ncb = .t.\n",
        SC_STRUCT, "1 ! shells\n1.0 1\nA A -1.0 -1.0 -1.0\n", None, None),
    # two species, staggered file, OVRR, ANGLE
    "afm_xyz": (
        "model = xyz\nmcs = 300 100\ntemp = 80 2 2\nspin = 1 1\nspecies = A B\nsc = 2 2 2\n"
        "bc = c c c\nrepeat = 4\nangle = .T. 50\ncoa = 10\nstg = .T.\novrr = .T. 0.60 12\n",
        "two species\n1.0\n 2.0 0 0\n 0 2.0 0\n 0 0 2.0\n A B\n 4 4\nDirect\n"
        " 0 0 0\n 0 0.5 0.5\n 0.5 0 0.5\n 0.5 0.5 0\n 0 0 0.5\n 0 0.5 0\n 0.5 0 0\n 0.5 0.5 0.5\n",
        "1\n1.0 1\nA B 3.0 3.0 3.0\n", None, "-1 B\n\n"),
    # species filter reorders and drops, cartesian coordinates, a three-letter symbol that
    # matches nothing (the previous species id is kept), a bond line split over two records
    "filter_cartesian": (
        "model = ising\nmcs = 50 10\ntemp = 3 1 1\nspin = 1.5 2 2.5\nspecies = CO fe\n"
        "sc = 3 2 2\nbc = c o c\nrepeat = 2\n",
        "three species\n1.0\n 3.0 0 0\n 0 3.0 0\n 0 0 3.0\n Fe O Co\n 1 2 1\nCartesian\n"
        " 0 0 0\n 1.5 0 0\n 0 1.5 0\n 1.5 1.5 1.5\n",
        "2\n1.5 2\nfe o -1 -1 -1\nFe3 co -2 -2\n -2\n2.598076 1\nCo Co 0.5 0.5 0.5\n", None, None),
    # para units, Zeeman, SIA (XYZ), r*c repeat counts, quoted value, ovrr off
    "para_sia": (
        "model = 'xyz'\nmcs = 60 20\ntemp = 2.0 1.0 0.25\nspin = 2\nspecies = A\nsc = 3*3\n"
        "para = .T. 2.5\nzeeman = .T. 0 0 5\nsia = .T.\ng_factor = 2\nseed = 7\nnbdfc = 1d-4\n",
        SC_STRUCT, "2\n1.0 1\nA A -1 -1 -2\n1.41421356 1\nA A 0.1 0.1 0.1\n",
        "\nA 0 0 -0.5\n", None),
    # a model name that is neither ising nor xyz runs as xyz; spiral keys; nbd_capacity
    "fallback_model": (
        "model = heisenberg\nmcs = 30 10\ntemp = 1 1 1\nspin = 1\nspecies = A\nsc = 5 5 5\n"
        "ssp = .T.\nss_dis = 1.01\nss_lat = 5\nss_direc = 0 0 1\nspiral_capacity = 2\n"
        "nbd_capacity = 8\n",
        SC_STRUCT, "1\n1.0 1\nA A -1 -1 -1\n", None, None),
}


def _nbd_oracle(deck):
    b, sp = do.basis(deck)
    ion, stgg = po.supercell(b, sp, np.asarray(deck["abc"]), deck["sc"], checkerboard=deck["cb"])
    rc, nn = po.neighbours_bruteforce(ion, np.asarray(deck["abc"]), deck["sc"], "".join(deck["bc"]),
                                      deck["nbd_dis"], deck["nbdfc"], deck["nbd_capacity"])
    assert rc == 0
    return ion, nn


def _compare(indir, outdir, check_nbd=True):
    info = eg.run(indir, outdir, parse_only=True)
    deck = do.read_deck(indir)
    got = open(os.path.join(outdir, "deck.txt")).read()
    want = do.listing(deck)
    assert got == want, "\n".join(a + "  |  " + b for a, b in zip(got.splitlines(), want.splitlines()) if a != b)
    assert info["n_temperatures"] == deck["nscan"]
    assert info["n_sites"] == len(deck["basis_atom"]) * int(np.prod(deck["sc"]))
    if check_nbd:
        ion, nn = _nbd_oracle(deck)
        got = open(os.path.join(outdir, "data", "nbd.dat")).read()
        assert got == do.nbd_dat(deck, nn, ion.shape[0])
        rows = open(os.path.join(outdir, "data", "fetched_lattice_network.xsf")).read().splitlines()[11:]
        assert len(rows) == ion.shape[0]
        for r, line in zip(ion, rows):
            assert line == do.A(deck["species"][int(r[4]) - 1], 2, 5) + "".join(do.F(x, 13, 7) for x in r[6:9])
    return deck, info


@pytest.mark.parametrize("name", sorted(DECKS))
def test_deck_matches_oracle(tmp_path, name):
    indir = write_deck(str(tmp_path / "in"), *DECKS[name])
    deck, info = _compare(indir, str(tmp_path / "out"))
    if name == "filter_cartesian":
        # Co (structure species 3) first, then Fe; O dropped
        assert deck["included_id"] == [3, 1] and deck["basis_atom"] == [4, 1]
        # the 'Fe3' line kept the previous first id (Fe) and matched Co second: Fe-Co -2 s s
        jx = deck["j_exc"]
        assert jx[2, 2, 0, 0] == pytest.approx(-2 * 1.5 * 2.5 / 1000.0)
    if name == "para_sia":
        assert deck["kb"] == 1.0 and deck["mb"] == 1.0 and deck["g_factor"] == 1.0
        assert deck["h"] == [0.0, 0.0, 2.0] and deck["sc"] == [3, 3, 3]
        assert deck["sia_vec"][0, 2] == pytest.approx(-0.5 * 4 / 2.5)
    if name == "fallback_model":
        assert deck["model"] == "xyz" and deck["model_fallback"] and info["model"] == eg.MODEL_XYZ
    if name == "afm_xyz":
        assert deck["stg_id"] == [1.0, -1.0]


BAD = {
    "no_equals": ("model ising\n", "Missing '='"),
    "unknown_key": ("model = ising\ndope = .F.\n", "unknown/missing"),
    "mcs_order": ("mcs = 100 200\n", "EQUILIBRATIONS"),
    "no_species": ("model = ising\n", "Selected ions"),
    "absent_species": ("species = B\n", "Selected ions"),
    "bad_logical": ("species = A\ncb = maybe\n", "logical"),
    "para_zero": ("species = A\npara = .T. 0\n", "cannot be zero"),
    "sia_file": ("species = A\nmodel = xyz\nsia = .T.\n", "single_ion_anisotropy"),
}


@pytest.mark.parametrize("name", sorted(BAD))
def test_deck_errors(tmp_path, name):
    text, msg = BAD[name]
    indir = write_deck(str(tmp_path / "in"), text, SC_STRUCT, "1\n1.0 1\nA A -1 -1 -1\n")
    with pytest.raises(eg.EtherError) as e:
        eg.run(indir, str(tmp_path / "out"), parse_only=True)
    assert e.value.code == -9 and msg in str(e.value)
    with pytest.raises(do.DeckError):
        do.read_deck(indir)


def test_missing_files(tmp_path):
    indir = write_deck(str(tmp_path / "in"), "species = A\n", SC_STRUCT, None)
    with pytest.raises(eg.EtherError, match="j_exchange"):
        eg.run(indir, str(tmp_path / "out"), parse_only=True)
    os.remove(os.path.join(indir, "structure.vasp"))
    with pytest.raises(eg.EtherError, match="structure.vasp"):
        eg.run(indir, str(tmp_path / "out"), parse_only=True)
    bad = write_deck(str(tmp_path / "bad"), "species = A\n", SC_STRUCT.replace("Direct", "Selective"),
                     "1\n1.0 1\nA A -1 -1 -1\n")
    with pytest.raises(eg.EtherError, match="Incorrect structure file"):
        eg.run(bad, str(tmp_path / "out"), parse_only=True)


def test_edit_descriptors():
    """The oracle's Fortran edit descriptors on the values the output files hold."""
    assert do.F(4.5, 11, 5) == "    4.50000"
    assert do.F(-0.0000001, 11, 6) == "  -0.000000"
    assert do.F(12345.678, 7, 2) == "*******"
    assert do.ES(-123.456, 12, 5) == "-1.23456E+02"
    assert do.ES(0.0, 12, 5) == " 0.00000E+00"
    assert do.ES(1e-120, 12, 5) == " 1.00000-120"
    assert do.ES(float("nan"), 12, 5) == "         NaN"
    assert do.I(7, 5) == "    7" and do.I(123456, 5) == "*****"
    assert do.A("Fe", 2, 5) == "   Fe" and do.A("# 1 Temp.", 20, 13) == "# 1 Temp.    "
    assert do.spk_name(4.5) == "4.5000spK.xsf" and do.spk_name(80) == "80.0000spK.xsf"


@pytest.mark.skipif(not (REF_EXAMPLES and os.path.isdir(REF_EXAMPLES)),
                    reason="ETHER_REFERENCE_EXAMPLES does not name the reference's examples folder")
def test_reference_example_decks(tmp_path):
    """Every example deck shipped with the reference, read by both restatements."""
    dirs = []
    for root, _, files in os.walk(REF_EXAMPLES):
        if "in.ether" in files and "structure.vasp" in files and "j_exchange" in files:
            dirs.append(root)
    assert len(dirs) >= 7
    for k, d in enumerate(sorted(dirs)):
        deck = do.read_deck(d)
        n = len(deck["basis_atom"]) * int(np.prod(deck["sc"]))
        _compare(d, str(tmp_path / ("o%d" % k)), check_nbd=n <= 4000)
