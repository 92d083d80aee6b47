// deck.cpp -- ether_run: the program src/ether.f90 for one input directory, on the GPU.
//
// Input (read exactly as the reference reads it):
//   in.ether               src/read_input.f90, src/defaults.f90, src/process_file.f90,
//                          src/lu.f90, src/count_species.f90
//   structure.vasp         src/get_tot_species.f90, src/read_structure.f90, src/frac_to_cart.f90
//   j_exchange             src/j_values.f90
//   single_ion_anisotropy  src/get_sia_values.f90
//   staggered              src/get_staggered_info.f90
// then src/parameters.f90, the species filter and supercell of src/generate_supercell.f90
// (through ether_build_lattice), and the temperature scan of src/ether.f90:79-240.
//
// Execution: every temperature of the scan is a slot of one PT ladder and every REPEAT a
// group of replicas, all advanced together by ether_mcs.  This is the reference run with one
// MPI rank per temperature; run_info.ranks = P < n_temperatures instead runs the reference's
// rounds of P consecutive temperatures (src/ether.f90:94-122) one after another, each slot
// carrying its configuration into the next round as a rank does.  REPEATs run side by side
// rather than one after another, so REPEAT k does not start from the state REPEAT k-1 left.
//
// Output (in outdir, laid out as the reference leaves its working directory):
//   ETHER.obs, ETHER.spn             src/process_observables.f90, src/rw_file.f90
//   data/magnetization.dat, data/energy.dat, data/moment_vectors.dat,
//   data/spiral_state_parameters.dat src/write_output_files.f90
//   data/gss.dat                     src/write_gss.f90
//   data/nbd.dat                     src/write_nbd.f90
//   data/fetched_lattice_network.xsf src/write_fetched_lattice_network.f90
//   data/graph.sh                    src/graph.f90
//   spins/<T>spK.xsf                 src/write_spins_at_K.f90
//   deck.txt                         everything read, after the unit conversion (no
//                                    counterpart: the reference prints parts of it)
// Files written with explicit edit descriptors match the reference byte for byte; files
// written list-directed follow gfortran's list-directed layout.
#include <sys/stat.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <exception>
#include <fstream>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "../../include/ether_gpu.h"

namespace ether {
void set_error(const std::string &msg);
}

namespace {

struct DeckError {
    int code;
    std::string msg;
};

[[noreturn]] void perr(const std::string &m) { throw DeckError{ETHER_ERR_PARSE, m}; }

struct RunError {
    int code;
};

#define RTRY(expr)                                \
    do {                                          \
        const int _rc = (expr);                   \
        if (_rc != ETHER_OK) throw RunError{_rc}; \
    } while (0)

// ------------------------------------------------------------------ Fortran text input ----
bool read_lines(const std::string &path, std::vector<std::string> &out) {
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    std::string line;
    while (std::getline(f, line)) {
        if (!line.empty() && line.back() == '\r') line.pop_back();
        out.push_back(line);
    }
    return true;
}

char up(char c) { return (c >= 'a' && c <= 'z') ? (char)(c - 'a' + 'A') : c; }
char low(char c) { return (c >= 'A' && c <= 'Z') ? (char)(c - 'A' + 'a') : c; }
std::string lower(std::string s) {
    for (char &c : s) c = low(c);
    return s;
}
std::string rtrim(std::string s) {
    while (!s.empty() && s.back() == ' ') s.pop_back();
    return s;
}
std::string trim(const std::string &s) {
    const size_t a = s.find_first_not_of(' ');
    if (a == std::string::npos) return std::string();
    return rtrim(s.substr(a));
}

// The values of one list-directed record: separated by blanks or commas, quotes stripped,
// r*c repeat counts expanded, a slash ends the record.
std::vector<std::string> list_values(const std::string &rec) {
    std::vector<std::string> v;
    size_t i = 0;
    const size_t n = rec.size();
    while (i < n) {
        const char c = rec[i];
        if (c == ' ' || c == ',' || c == '\t') {
            ++i;
            continue;
        }
        if (c == '/') break;
        std::string tok;
        if (c == '\'' || c == '"') {
            const char q = c;
            ++i;
            while (i < n) {
                if (rec[i] == q) {
                    if (i + 1 < n && rec[i + 1] == q) {
                        tok += q;
                        i += 2;
                        continue;
                    }
                    ++i;
                    break;
                }
                tok += rec[i++];
            }
            v.push_back(tok);
            continue;
        }
        while (i < n && rec[i] != ' ' && rec[i] != ',' && rec[i] != '\t' && rec[i] != '/') tok += rec[i++];
        const size_t star = tok.find('*');
        if (star != std::string::npos && star > 0 && tok.find_first_not_of("0123456789") == star) {  // r*c
            const long r = std::strtol(tok.substr(0, star).c_str(), nullptr, 10);
            const std::string val = tok.substr(star + 1);
            for (long k = 0; k < r && k < 100000; ++k) v.push_back(val);
        } else {
            v.push_back(tok);
        }
    }
    return v;
}

// A list-directed READ statement on a sequential file: starts at the next record, takes
// records until it has n values, and leaves the rest of the last record unread.
struct ListFile {
    std::vector<std::string> rec;
    size_t at = 0;
    std::string name;
    bool eof() const { return at >= rec.size(); }
    std::vector<std::string> read(size_t n, const std::string &what) {
        std::vector<std::string> v;
        while (v.size() < n) {
            if (at >= rec.size()) perr(name + ": end of file while reading " + what);
            const auto more = list_values(rec[at++]);
            v.insert(v.end(), more.begin(), more.end());
        }
        v.resize(n);
        return v;
    }
};

double to_real(const std::string &t, const std::string &what) {
    std::string u = t;
    for (char &c : u)
        if (c == 'd' || c == 'D' || c == 'q' || c == 'Q') c = 'e';
    char *end = nullptr;
    const double v = std::strtod(u.c_str(), &end);
    if (u.empty() || end == u.c_str() || *end != '\0') perr("cannot read a real from '" + t + "' (" + what + ")");
    return v;
}
long to_int(const std::string &t, const std::string &what) {
    char *end = nullptr;
    const long v = std::strtol(t.c_str(), &end, 10);
    if (t.empty() || end == t.c_str() || *end != '\0') perr("cannot read an integer from '" + t + "' (" + what + ")");
    return v;
}
// list-directed logical: optional '.', then T or F, then anything
bool to_logical(const std::string &t, const std::string &what) {
    size_t i = (!t.empty() && t[0] == '.') ? 1 : 0;
    if (i < t.size() && (t[i] == 't' || t[i] == 'T')) return true;
    if (i < t.size() && (t[i] == 'f' || t[i] == 'F')) return false;
    perr("cannot read a logical from '" + t + "' (" + what + ")");
}

// A value read into character(len=w): the first w characters, blank padded; then lu makes
// the first one upper and the second one lower case (src/read_structure.f90:56-61,
// src/read_input.f90:81-86, src/j_values.f90:69-79).  Returned without trailing blanks.
std::string symbol(const std::string &tok, size_t w) {
    std::string s = tok.substr(0, std::min(w, tok.size()));
    s.resize(w, ' ');
    s[0] = up(s[0]);
    if (w > 1) s[1] = low(s[1]);
    return rtrim(s);
}

// ---------------------------------------------------------------------------- the deck ----
struct Deck {
    // in.ether, with the values of src/defaults.f90
    std::string model = "ising";
    bool ising = true, xyz = false, model_fallback = false;
    long tmcs = 5000, tmcs_eq = 3000;
    double ht = 100, lt = 10, tint = 5;
    std::vector<double> s;
    std::vector<std::string> species_to_include;
    long sc[3] = {2, 2, 2};
    char bc[3] = {'c', 'c', 'c'};
    long repeat = 10;
    bool angle = false;
    double dphi = 0.0;  // radians
    double coa = 10;    // to_cal is real(dp)
    bool zeeman = false;
    double h[3] = {0, 0, 0};
    double g_factor = 2;
    bool staggered = false, sia = false, para = false;
    double j_para = 1.0;
    bool ovrr = false;
    double ovrr_para = 0.0;
    long ovrr_mcs = 0;
    long seed = 1992;
    double nbdfc = 0.00001;
    bool pt = false;
    long exchange_interval = 11;
    bool cb = false;
    double ss_dis = 4.0, ss_lat = 2;
    double ss_direc[3] = {0, 0, 1};
    bool ssp = false;
    long spiral_capacity = 5, nbd_capacity = 20;
    // structure.vasp
    double abc[9] = {0};
    std::vector<std::string> species;  // per structure species, 1-based in the files
    std::vector<long> ions;
    std::vector<double> cart;          // 3 per structure atom
    std::vector<int> atom_species;     // 1-based
    // species filter: the included atoms (structure atom index, 1-based) in basis order
    std::vector<int> basis_atom;
    std::vector<int> included_id;      // included_species_ID, 0 where nothing matched
    // j_exchange: nbd_dis(nsh), j_exc(nsh, nsp, nsp, 3) = J s_i s_j (after parameters.f90)
    int nsh = 0;
    std::vector<double> nbd_dis, j_exc;
    // single_ion_anisotropy: sia_vec(3, nsp) = D s^2 (after parameters.f90)
    std::vector<double> sia_vec;
    // staggered values per species (src/get_staggered_info.f90:41-57)
    std::vector<double> stg_id;
    double kb = 8.617333262e-5, mb = 5.7883818060e-5;
};

int nspecies(const Deck &d) { return (int)d.species.size(); }

int find_species(const Deck &d, const std::string &name, int stale) {
    int id = stale;
    for (int k = 0; k < nspecies(d); ++k)
        if (d.species[k] == name) id = k + 1;  // the last match, as the loops do
    return id;
}

void read_structure(const std::string &dir, Deck &d) {
    ListFile f;
    f.name = "structure.vasp";
    if (!read_lines(dir + "/structure.vasp", f.rec)) perr("Required file 'structure.vasp' is not present");
    // get_tot_species: line 7 gives the species count (blank-separated words) and the ions
    if (f.rec.size() < 7) perr("structure.vasp: fewer than 7 lines");
    int nsp = 0;
    {
        std::istringstream is(f.rec[6]);
        std::string w;
        while (is >> w) ++nsp;
    }
    if (nsp < 1) perr("structure.vasp: no ion counts on line 7");
    f.read(1, "the title");
    f.read(1, "the scale");  // read and not used (src/read_structure.f90:44)
    for (int i = 0; i < 3; ++i) {
        const auto v = f.read(3, "a lattice vector");
        for (int j = 0; j < 3; ++j) d.abc[3 * i + j] = to_real(v[j], "lattice vector");
    }
    for (const auto &t : f.read(nsp, "the species names")) d.species.push_back(symbol(t, 2));
    long tions = 0;
    for (const auto &t : f.read(nsp, "the ions per species")) {
        d.ions.push_back(to_int(t, "ions per species"));
        if (d.ions.back() < 0) perr("structure.vasp: negative ion count");
        tions += d.ions.back();
    }
    const std::string label = lower(f.read(1, "the coordinate label")[0]);
    if (label != "direct" && label != "cartesian") perr("Incorrect structure file");
    for (long i = 0; i < tions; ++i) {
        const auto v = f.read(3, "coordinates");
        double p[3];
        for (int a = 0; a < 3; ++a) p[a] = to_real(v[a], "coordinate");
        if (label == "direct") {  // frac_to_cart: r(i) = abc(1,i) f1 + abc(2,i) f2 + abc(3,i) f3
            for (int a = 0; a < 3; ++a) d.cart.push_back(d.abc[a] * p[0] + d.abc[3 + a] * p[1] + d.abc[6 + a] * p[2]);
        } else {
            for (int a = 0; a < 3; ++a) d.cart.push_back(p[a]);
        }
    }
    for (int k = 0; k < nsp; ++k)
        for (long i = 0; i < d.ions[k]; ++i) d.atom_species.push_back(k + 1);
}

// process_file: a line stops at the first '!' or '#', tabs become blanks, lines are
// character(len=200), blank lines are dropped
std::vector<std::string> processed(const std::vector<std::string> &raw) {
    std::vector<std::string> out;
    for (std::string t : raw) {
        if (t.size() > 200) t.resize(200);
        std::string u;
        for (char c : t) {
            if (c == '!' || c == '#') break;
            u += (c == '\t') ? ' ' : c;
        }
        if (!trim(u).empty()) out.push_back(u);
    }
    return out;
}

void read_in_ether(const std::string &dir, Deck &d) {
    std::vector<std::string> raw;
    if (!read_lines(dir + "/in.ether", raw)) perr("Required file 'in.ether' is not present");
    const int nsp = nspecies(d);
    d.s.assign(nsp, 0.0);
    for (const std::string &line : processed(raw)) {
        const std::string text = lower(line);
        const size_t eq = text.find('=');
        if (eq == std::string::npos) perr("Missing '=' in the given line: " + trim(text));
        const std::string key = trim(text.substr(0, eq));
        const std::string value = text.substr(eq + 1);
        const auto v = list_values(value);
        auto need = [&](size_t n) {
            if (v.size() < n) perr("too few values for '" + key + "': " + trim(text));
        };
        if (key == "model") {
            need(1);
            d.model = v[0].substr(0, 5);  // character(len=5)
            d.ising = d.model == "ising";
            d.xyz = d.model == "xyz";
        } else if (key == "mcs") {
            need(2);
            d.tmcs = to_int(v[0], key);
            d.tmcs_eq = to_int(v[1], key);
            if (d.tmcs <= d.tmcs_eq) perr("TOTAL MCS  < EQUILIBRATIONS MCS steps");
        } else if (key == "temp") {
            need(3);
            d.ht = to_real(v[0], key);
            d.lt = to_real(v[1], key);
            d.tint = to_real(v[2], key);
        } else if (key == "spin") {
            need(nsp);
            for (int k = 0; k < nsp; ++k) d.s[k] = to_real(v[k], key);
        } else if (key == "species") {
            // count_species counts blank-separated words; that many values are read
            size_t n = 0;
            {
                std::istringstream is(value);
                std::string w;
                while (is >> w) ++n;
            }
            need(n);
            d.species_to_include.clear();
            for (size_t k = 0; k < n; ++k) d.species_to_include.push_back(symbol(v[k], 2));
        } else if (key == "sc") {
            need(3);
            for (int k = 0; k < 3; ++k) d.sc[k] = to_int(v[k], key);
        } else if (key == "stg") {
            need(1);
            d.staggered = to_logical(v[0], key);
        } else if (key == "bc") {
            need(3);
            for (int k = 0; k < 3; ++k) d.bc[k] = v[k].empty() ? ' ' : v[k][0];
        } else if (key == "repeat") {
            need(1);
            d.repeat = to_int(v[0], key);
        } else if (key == "angle") {
            need(2);
            d.angle = to_logical(v[0], key);
            d.dphi = (4.0 * std::atan(1.0) / 180.0) * to_real(v[1], key);
        } else if (key == "coa") {
            need(1);
            d.coa = to_real(v[0], key);
        } else if (key == "zeeman") {
            need(4);
            d.zeeman = to_logical(v[0], key);
            for (int k = 0; k < 3; ++k) d.h[k] = to_real(v[1 + k], key);
        } else if (key == "g_factor") {
            need(1);
            d.g_factor = to_real(v[0], key);
        } else if (key == "sia") {
            need(1);
            d.sia = to_logical(v[0], key);
        } else if (key == "para") {
            need(2);
            d.para = to_logical(v[0], key);
            d.j_para = std::fabs(to_real(v[1], key));
            if (d.j_para == 0.0 && d.para) perr("parameter value is set ON and value cannot be zero");
        } else if (key == "ovrr") {
            need(3);
            d.ovrr = to_logical(v[0], key);
            d.ovrr_para = std::fabs(to_real(v[1], key));
            d.ovrr_mcs = to_int(v[2], key);
        } else if (key == "seed") {
            need(1);
            d.seed = to_int(v[0], key);
        } else if (key == "nbdfc") {
            need(1);
            d.nbdfc = to_real(v[0], key);
        } else if (key == "pt") {
            need(2);
            d.pt = to_logical(v[0], key);
            d.exchange_interval = to_int(v[1], key);
        } else if (key == "cb") {
            need(1);
            d.cb = to_logical(v[0], key);
        } else if (key == "ss_dis") {
            need(1);
            d.ss_dis = to_real(v[0], key);
        } else if (key == "ss_lat") {
            need(1);
            d.ss_lat = to_real(v[0], key);
        } else if (key == "ss_direc") {
            need(3);
            for (int k = 0; k < 3; ++k) d.ss_direc[k] = to_real(v[k], key);
        } else if (key == "ssp") {
            need(1);
            d.ssp = to_logical(v[0], key);
        } else if (key == "spiral_capacity") {
            need(1);
            d.spiral_capacity = to_int(v[0], key);
        } else if (key == "nbd_capacity") {
            need(1);
            d.nbd_capacity = to_int(v[0], key);
        } else {
            perr("Found unknown/missing information: " + trim(text));
        }
    }
    // src/startup.f90:36-43: a model that is neither ising nor xyz runs as xyz
    if (!d.ising && !d.xyz) {
        d.model_fallback = true;
        d.model = "xyz";
        d.xyz = true;
    }
}

// generate_supercell.f90:66-99: included_species_ID and the basis, in the order of the
// 'species' list (each entry takes the atoms of every structure species of that name)
void filter_species(Deck &d) {
    d.included_id.assign(d.species_to_include.size(), 0);
    std::vector<long> start(nspecies(d) + 1, 0);
    for (int j = 0; j < nspecies(d); ++j) start[j + 1] = start[j] + d.ions[j];
    for (size_t i = 0; i < d.species_to_include.size(); ++i)
        for (int j = 0; j < nspecies(d); ++j)
            if (d.species_to_include[i] == d.species[j]) {
                d.included_id[i] = j + 1;
                for (long k = start[j]; k < start[j + 1]; ++k) d.basis_atom.push_back((int)k + 1);
            }
    if (d.basis_atom.empty()) perr("Selected ions from 'in.ether' are not present in 'structure.vasp' file");
}

// character(len=3) symbols of j_exchange and staggered against the len=2 species names
int match3(const Deck &d, const std::string &tok, int stale) {
    const std::string t = symbol(tok, 3);
    if (t.size() > 2) return stale;  // a third character: equal to no species name
    return find_species(d, t, stale);
}

void read_couplings(const std::string &dir, Deck &d) {
    ListFile f;
    f.name = "j_exchange";
    if (!read_lines(dir + "/j_exchange", f.rec)) perr("Required file 'j_exchange' is not present");
    const int nsp = nspecies(d);
    d.nsh = (int)to_int(f.read(1, "the number of bonds")[0], "no_of_nbd");
    if (d.nsh < 0) perr("j_exchange: negative number of bonds");
    d.nbd_dis.assign(d.nsh, 0.0);
    d.j_exc.assign((size_t)d.nsh * nsp * nsp * 3, 0.0);
    int id[2] = {0, 0};  // j_ID keeps its value when a name matches nothing
    for (int b = 0; b < d.nsh; ++b) {
        auto v = f.read(2, "a bond length");
        d.nbd_dis[b] = to_real(v[0], "bond length");
        const long similar = to_int(v[1], "similar bonds");
        for (long k = 0; k < similar; ++k) {
            v = f.read(5, "a bond line");
            for (int a = 0; a < 2; ++a) id[a] = match3(d, v[a], id[a]);
            if (id[0] == 0 || id[1] == 0) perr("j_exchange: species '" + v[0] + "' / '" + v[1] + "' not in structure.vasp");
            for (int c = 0; c < 3; ++c) {
                const double J = to_real(v[2 + c], "J") * d.s[id[0] - 1] * d.s[id[1] - 1];
                d.j_exc[b + (size_t)d.nsh * ((id[0] - 1) + (size_t)nsp * ((id[1] - 1) + (size_t)nsp * c))] = J;
                d.j_exc[b + (size_t)d.nsh * ((id[1] - 1) + (size_t)nsp * ((id[0] - 1) + (size_t)nsp * c))] = J;
            }
        }
    }
}

void read_sia(const std::string &dir, Deck &d) {
    const int nsp = nspecies(d);
    d.sia_vec.assign((size_t)3 * nsp, 0.0);
    if (!(d.sia && d.xyz)) return;
    ListFile f;
    f.name = "single_ion_anisotropy";
    if (!read_lines(dir + "/single_ion_anisotropy", f.rec))
        perr("SIA is .TRUE. but file 'single_ion_anisotropy' is not found");
    int id = 0;  // SIA_ID keeps its value when a name matches nothing
    while (true) {
        // the read ends the loop at the end of the file (end=10); blank records are skipped
        while (!f.eof() && list_values(f.rec[f.at]).empty()) ++f.at;
        if (f.eof()) break;
        const auto v = f.read(4, "an SIA line");
        id = find_species(d, symbol(v[0], 2), id);
        if (id == 0) perr("single_ion_anisotropy: species '" + v[0] + "' not in structure.vasp");
        const double s2 = d.s[id - 1] * d.s[id - 1];
        for (int a = 0; a < 3; ++a) d.sia_vec[3 * (id - 1) + a] = to_real(v[1 + a], "SIA") * s2;
    }
}

void read_staggered(const std::string &dir, Deck &d) {
    d.stg_id.assign(nspecies(d), 1.0);
    if (d.cb || !d.staggered) return;
    ListFile f;
    f.name = "staggered";
    if (!read_lines(dir + "/staggered", f.rec)) return;
    const size_t total = f.rec.size();
    for (size_t i = 0; i < total; ++i) {
        while (!f.eof() && list_values(f.rec[f.at]).empty()) ++f.at;
        if (f.eof()) break;
        const auto v = f.read(2, "a staggered line");
        const double val = to_real(v[0], "staggered value");
        const int k = match3(d, v[1], 0);
        if (k) d.stg_id[k - 1] = val;
    }
}

// src/parameters.f90
void apply_parameters(Deck &d) {
    if (d.para) {
        for (double &j : d.j_exc) j = j / d.j_para;
        if (d.sia && d.xyz)
            for (double &v : d.sia_vec) v = v / d.j_para;
        d.kb = 1.0;
        d.mb = 1.0;
        d.g_factor = 1.0;
        if (d.zeeman)
            for (double &x : d.h) x = x / d.j_para;
    } else {
        for (double &j : d.j_exc) j = j / 1000.0;
        if (d.sia && d.xyz)
            for (double &v : d.sia_vec) v = v / 1000.0;
        d.mb = 5.7883818060e-5;
    }
}

// ----------------------------------------------------------------- Fortran text output ----
std::string g17(double x) {
    char b[40];
    std::snprintf(b, sizeof b, "%.17g", x);
    return b;
}

std::string special(double x, int w) {
    std::string s = std::isnan(x) ? "NaN" : (x < 0 ? "-Infinity" : "Infinity");
    if ((int)s.size() > w) s = std::isnan(x) ? "NaN" : (x < 0 ? "-Inf" : "Inf");
    if ((int)s.size() > w) return std::string(w, '*');
    return std::string(w - s.size(), ' ') + s;
}
// Fw.d
std::string fF(double x, int w, int d) {
    if (!std::isfinite(x)) return special(x, w);
    char b[400];
    std::snprintf(b, sizeof b, "%*.*f", w, d, x);
    std::string s = b;
    return (int)s.size() > w ? std::string(w, '*') : s;
}
// ESw.d (two exponent digits, the letter dropped for three)
std::string fES(double x, int w, int d) {
    if (!std::isfinite(x)) return special(x, w);
    char b[64];
    std::snprintf(b, sizeof b, "%.*E", d, x);
    std::string s = b;
    const size_t e = s.find('E');
    const std::string mant = s.substr(0, e);
    const int ex = std::atoi(s.c_str() + e + 1);
    char eb[16];
    if (std::abs(ex) <= 99) std::snprintf(eb, sizeof eb, "E%c%02d", ex < 0 ? '-' : '+', std::abs(ex));
    else std::snprintf(eb, sizeof eb, "%c%03d", ex < 0 ? '-' : '+', std::abs(ex));
    s = mant + eb;
    if ((int)s.size() > w) return std::string(w, '*');
    return std::string(w - s.size(), ' ') + s;
}
// Iw
std::string fI(long v, int w) {
    char b[40];
    std::snprintf(b, sizeof b, "%*ld", w, v);
    std::string s = b;
    return (int)s.size() > w ? std::string(w, '*') : s;
}
// Aw of a character(len) variable holding s
std::string fA(const std::string &s, int len, int w) {
    std::string t = s;
    t.resize(len, ' ');
    if (w <= len) return t.substr(0, w);
    return std::string(w - len, ' ') + t;
}

// gfortran list-directed items: a record starts with a blank, items are separated by one
// blank; REAL(8) is G25.17 (F form between 0.1 and 1e17, followed by five blanks), INTEGER(4)
// is I11, characters as they are.
struct ListRecord {
    std::string s;
    ListRecord &real(double x) {
        s += ' ';
        const double a = std::fabs(x);
        char b[64];
        if (x == 0.0 || (a >= 0.1 && a < 1e17)) {
            const int k = (x == 0.0) ? 1 : (int)std::floor(std::log10(a)) + 1;
            std::snprintf(b, sizeof b, "%.*f", std::max(0, 17 - k), x);
            const std::string t = b;
            s += std::string(t.size() < 20 ? 20 - t.size() : 0, ' ') + t + "     ";
        } else {
            std::snprintf(b, sizeof b, "%.16E", x);
            std::string t = b;
            const size_t e = t.find('E');
            const int ex = std::atoi(t.c_str() + e + 1);
            char eb[16];
            std::snprintf(eb, sizeof eb, "E%c%03d", ex < 0 ? '-' : '+', std::abs(ex));
            t = t.substr(0, e) + eb;
            s += std::string(t.size() < 25 ? 25 - t.size() : 0, ' ') + t;
        }
        return *this;
    }
    ListRecord &integer(long v) {
        s += ' ' + fI(v, 11);
        return *this;
    }
    ListRecord &chars(const std::string &c) {
        s += ' ' + c;
        return *this;
    }
    std::string line() const { return s + "\n"; }
};

void write_file(const std::string &path, const std::string &s) {
    std::ofstream f(path, std::ios::binary | std::ios::trunc);
    if (!f) throw DeckError{ETHER_ERR_ARG, "cannot write " + path};
    f << s;
    if (!f) throw DeckError{ETHER_ERR_ARG, "cannot write " + path};
}

void make_dir(const std::string &path) {
    struct stat st;
    if (stat(path.c_str(), &st) == 0 && S_ISDIR(st.st_mode)) return;
    if (mkdir(path.c_str(), 0755) != 0) throw DeckError{ETHER_ERR_ARG, "cannot create directory " + path};
}

// An open output file, closed on every exit path.
struct OutFile {
    std::FILE *f = nullptr;
    std::string path;
    OutFile(const std::string &p, const char *mode) : path(p) {
        f = std::fopen(p.c_str(), mode);
        if (!f) throw DeckError{ETHER_ERR_ARG, "cannot open " + p};
    }
    ~OutFile() {
        if (f) std::fclose(f);
    }
    OutFile(const OutFile &) = delete;
    OutFile &operator=(const OutFile &) = delete;
    void put(const std::string &s) {
        if (std::fwrite(s.data(), 1, s.size(), f) != s.size()) throw DeckError{ETHER_ERR_ARG, "cannot write " + path};
    }
    // record `rec` of `bytes` bytes (direct access, no record markers)
    void put_record(long rec, const void *data, size_t bytes) {
        if (std::fseek(f, (long)((size_t)rec * bytes), SEEK_SET) != 0 || std::fwrite(data, 1, bytes, f) != bytes)
            throw DeckError{ETHER_ERR_ARG, "cannot write " + path};
    }
    void get_record(long rec, void *data, size_t bytes) {
        if (std::fseek(f, (long)((size_t)rec * bytes), SEEK_SET) != 0 || std::fread(data, 1, bytes, f) != bytes)
            throw DeckError{ETHER_ERR_PARSE, "resume: ETHER.spn does not hold one record of this lattice per temperature"};
    }
};

bool file_exists(const std::string &p) {
    struct stat st;
    return stat(p.c_str(), &st) == 0;
}

std::string listing(const Deck &d, long nscan, int nbasis) {
    std::ostringstream o;
    auto L = [&](const std::string &k, const std::vector<std::string> &v) {
        o << k << " =";
        for (const auto &x : v) o << ' ' << x;
        o << '\n';
    };
    auto D = [&](const std::string &k, const double *p, size_t n) {
        std::vector<std::string> v;
        for (size_t i = 0; i < n; ++i) v.push_back(g17(p[i]));
        L(k, v);
    };
    auto I = [&](const std::string &k, const std::vector<long> &p) {
        std::vector<std::string> v;
        for (long x : p) v.push_back(std::to_string(x));
        L(k, v);
    };
    auto B = [&](const std::string &k, bool b) { L(k, {b ? "1" : "0"}); };
    L("model", {d.model});
    B("model_fallback", d.model_fallback);
    I("mcs", {d.tmcs, d.tmcs_eq});
    D("temp", std::vector<double>{d.ht, d.lt, d.tint}.data(), 3);
    I("n_temperatures", {nscan});
    D("spin", d.s.data(), d.s.size());
    L("species_to_include", d.species_to_include);
    I("sc", {d.sc[0], d.sc[1], d.sc[2]});
    L("bc", {std::string(1, d.bc[0]), std::string(1, d.bc[1]), std::string(1, d.bc[2])});
    I("repeat", {d.repeat});
    B("angle", d.angle);
    D("dphi", &d.dphi, 1);
    D("coa", &d.coa, 1);
    B("zeeman", d.zeeman);
    D("h", d.h, 3);
    D("g_factor", &d.g_factor, 1);
    B("stg", d.staggered);
    B("sia", d.sia);
    B("para", d.para);
    D("j_para", &d.j_para, 1);
    B("ovrr", d.ovrr);
    D("ovrr_para", &d.ovrr_para, 1);
    I("ovrr_mcs", {d.ovrr_mcs});
    I("seed", {d.seed});
    D("nbdfc", &d.nbdfc, 1);
    B("pt", d.pt);
    I("exchange_interval", {d.exchange_interval});
    B("cb", d.cb);
    D("ss_dis", &d.ss_dis, 1);
    D("ss_lat", &d.ss_lat, 1);
    D("ss_direc", d.ss_direc, 3);
    B("ssp", d.ssp);
    I("spiral_capacity", {d.spiral_capacity});
    I("nbd_capacity", {d.nbd_capacity});
    D("abc", d.abc, 9);
    L("species", d.species);
    I("ions", d.ions);
    D("cart", d.cart.data(), d.cart.size());
    I("included_id", std::vector<long>(d.included_id.begin(), d.included_id.end()));
    I("basis_atom", std::vector<long>(d.basis_atom.begin(), d.basis_atom.end()));
    I("n_basis", {nbasis});
    D("nbd_dis", d.nbd_dis.data(), d.nbd_dis.size());
    D("j_exc", d.j_exc.data(), d.j_exc.size());
    D("sia_vec", d.sia_vec.data(), d.sia_vec.size());
    D("stg_id", d.stg_id.data(), d.stg_id.size());
    D("kb", &d.kb, 1);
    D("mb", &d.mb, 1);
    return o.str();
}

// src/write_nbd.f90 (the continued literals keep their next line's 24 leading blanks)
std::string nbd_text(const Deck &d, long N, int cap, const std::vector<int32_t> &nn) {
    const std::string pad(24, ' ');
    std::string o;
    o += " # This file can be used to confirm the neighbourhood " + pad + "details of any selected\n";
    o += " # central ion with ion number (<ION no.>).\n";
    o += " # [NOTE: The content of nbd.dat is independent of the " + pad + "species labels present in 'structure.vasp'.\n";
    o += " # The contents of nbd.dat depend only on the bond " + pad + "lengths provided in the 'j_exchange' file.]\n";
    o += " # To visualize the structure, use the 'VESTA' software " + pad + "(https://jp-minerals.org/vesta/en/download.html)\n";
    o += " # and open the generated 'fetched_lattice_network.xsf' file.\n";
    o += " # Check the neighbourhood details (given in this file) " + pad + "using the <Atom Label> for the selected central <ION no.> IDs.\n";
    o += " \n";
    const size_t nsh = d.nsh;
    for (long i = 0; i < N; ++i) {
        o += " ION no. " + fI(i + 1, 5) + "\n";  // format 10
        o += " ~~~~~~~~~~~~~~\n";
        for (size_t m = 0; m < nsh; ++m) {  // format 11
            o += " For bond length: " + fF(d.nbd_dis[m], 12, 8) + ", nbds are ==> ";
            const int cnt = nn[m + nsh * (size_t)i];
            for (int k = 1; k <= cnt && k <= cap; ++k) o += fI(nn[m + nsh * ((size_t)i + (size_t)N * (size_t)k)], 7);
            o += "\n";
        }
        o += " \n";
    }
    return o;
}

// src/write_fetched_lattice_network.f90 and the header of src/write_spins_at_K.f90
std::string xsf_header(const Deck &d, long N) {
    std::string o;
    o += ListRecord().chars("CRYSTAL").line();
    o += ListRecord().chars("PRIMVEC").line();
    for (int pass = 0; pass < 2; ++pass) {
        for (int i = 0; i < 3; ++i) {
            ListRecord r;
            for (int j = 0; j < 3; ++j) r.real(d.abc[3 * i + j] * (double)d.sc[i]);
            o += r.line();
        }
        if (pass == 0) o += ListRecord().chars("CONVEC").line();
    }
    o += ListRecord().chars("PRIMCOORD").line();
    o += ListRecord().integer(N).chars(" 1").line();
    return o;
}

// src/graph.f90
std::string graph_text(const Deck &d) {
    const std::string pad(24, ' ');
    std::string o;
    auto w = [&](const std::string &s) { o += " " + s + "\n"; };
    auto xlabel = [&]() {  // formats 301 / 302
        o += d.para ? " set xlabel \"Temperature (k_{B}T/J)\"\n" : " set xlabel \"Temperature (K)\"\n";
    };
    w("# set labels, lables, and xtics/ytics accordingly");
    w("unset key");
    w("set terminal png size 1100, 900 font \"Times-New-Roman,18\"");
    w("set output 'results_Ether.png'");
    w("set multiplot");
    w("set size squar 0.5,0.5");
    w("set nokey");
    w("set format y \"%g\"");
    o += " set xtics " + fF(d.lt, 11, 5) + "," + fF(std::fabs(d.ht - d.lt) / 5.0, 11, 5) + "," + fF(d.ht, 11, 5) + "\n";
    w("set mxtics 10");
    w("set origin 0.0,0.0");
    w("set grid");
    xlabel();
    w(d.staggered ? "set ylabel \"Staggered Magnetization (M)\"" : "set ylabel \"Magnetization (M)\"");
    w("plot 'magnetization.dat' u 1:2:4 with yerrorbars " + pad + "lt 6 notitle");
    w("set origin 0.5, 0.0");
    xlabel();
    w(d.staggered ? "set ylabel \"Staggered Susceptibility (\xcf\x87)\"" : "set ylabel \"Susceptibility (\xcf\x87)\"");
    w("plot 'magnetization.dat' u 1:3:5 with yerrorbars " + pad + "lt 6 notitle");
    w("set origin 0.0,0.5");
    xlabel();
    if (d.para) {
        w("set ylabel \"Energy\"");
        w("plot 'energy.dat' u 1:2:4 with yerrorbars " + pad + "lt 6 notitle");
    } else {
        w("set ylabel \"Energy (meV)\"");
        w("plot 'energy.dat' u 1:($2*1000):4 with yerrorbars " + pad + "lt 6 notitle");
    }
    w("set origin 0.5,0.5");
    xlabel();
    if (d.para) w("set ylabel \"Specific Heat (C_{V})\"");
    else w("set ylabel \"Specific Heat \t\t\t(C_{V}k_{B}^{-1})\"");
    w("plot 'energy.dat' u 1:3:5 with yerrorbars " + pad + "lt 6 notitle");
    w("unset multiplot");
    return o;
}

// observables_per_repeat (src/observables_per_repeat.f90:29-94): mean over the groups and
// sqrt(sum (x - mean)^2 / (m (m - 1))) of q quantities per slot, vals(q, slot, group);
// one group gives NaN errors, as the reference's 1/0 * 0 does
void per_repeat(const std::vector<double> &vals, int q, int nslots, int ngroups, std::vector<double> &mean,
                std::vector<double> &err) {
    mean.assign((size_t)q * nslots, 0.0);
    err.assign((size_t)q * nslots, 0.0);
    const double rep = ngroups;
    const double r1 = 1.0 / (rep * (rep - 1.0));
    for (int s = 0; s < nslots; ++s)
        for (int k = 0; k < q; ++k) {
            double sum = 0.0;
            for (int g = 0; g < ngroups; ++g) sum += vals[(size_t)q * ((size_t)g * nslots + s) + k];
            const double mu = sum / rep;
            double e = 0.0;
            for (int g = 0; g < ngroups; ++g) {
                const double dv = vals[(size_t)q * ((size_t)g * nslots + s) + k] - mu;
                e += dv * dv;
            }
            mean[(size_t)q * s + k] = mu;
            err[(size_t)q * s + k] = std::sqrt(r1 * e);
        }
}

}  // namespace

extern "C" int ether_run(const char *indir, const char *outdir, int32_t flags, ether_run_info *info) {
    if (!indir || !outdir) {
        ether::set_error("ether_run: null directory");
        return ETHER_ERR_ARG;
    }
    const bool quiet = (flags & ETHER_RUN_QUIET) != 0;
    ether_ctx *ctx = nullptr;
    try {
        const std::string dir(indir), out(outdir);
        const int32_t ranks_in = info ? info->ranks : 0;
        // ------------------------------------------------ input (src/ether.f90:54-76) ----
        Deck d;
        read_structure(dir, d);
        read_in_ether(dir, d);
        filter_species(d);
        read_couplings(dir, d);
        read_sia(dir, d);
        read_staggered(dir, d);
        apply_parameters(d);
        if (d.sc[0] < 1 || d.sc[1] < 1 || d.sc[2] < 1) perr("sc: the supercell must be at least 1 x 1 x 1");
        if (d.nbd_capacity < 1 || d.nbd_capacity > 4096) perr("nbd_capacity must be in [1, 4096]");
        if (!(d.tint != 0.0) || !std::isfinite((d.ht - d.lt) / d.tint)) perr("temp: the interval must be non-zero");
        const long nscan = std::lround((d.ht - d.lt) / d.tint) + 1;  // src/ether.f90:79
        const int nsp = nspecies(d);
        const int nbasis = (int)d.basis_atom.size();
        const long ncell = d.sc[0] * d.sc[1] * d.sc[2];
        if (ncell * nbasis > 0x7FFFFFFFL / 16) perr("the supercell is too large");
        const long N = ncell * nbasis;
        const int cap = (int)d.nbd_capacity;
        // lattice (generate_supercell + getting_nbd)
        std::vector<double> basis((size_t)3 * nbasis);
        std::vector<int32_t> bsp(nbasis);
        for (int l = 0; l < nbasis; ++l) {
            const int a = d.basis_atom[l];
            for (int k = 0; k < 3; ++k) basis[3 * l + k] = d.cart[3 * (size_t)(a - 1) + k];
            bsp[l] = d.atom_species[a - 1];
        }
        std::vector<double> ion((size_t)9 * N), stgg(N);
        std::vector<int32_t> nn((size_t)std::max(d.nsh, 1) * N * (cap + 1) * 2, 0);
        const int32_t sc[3] = {(int32_t)d.sc[0], (int32_t)d.sc[1], (int32_t)d.sc[2]};
        RTRY(ether_build_lattice(nbasis, basis.data(), bsp.data(), d.abc, sc, d.bc, d.cb ? 1 : 0, d.nsh,
                                 d.nbd_dis.data(), d.nbdfc, cap, ion.data(), stgg.data(), nn.data()));
        for (long i = 0; i < N; ++i) {
            const int a = d.basis_atom[i % nbasis];  // atom(i, 3) = (-1)**i over the structure's atoms
            ion[9 * i + 3] = d.ising ? ((a % 2 == 0) ? 1.0 : -1.0) : 1.0;
            if (!d.cb) stgg[i] = d.stg_id[(int)ion[9 * i + 4] - 1];
        }
        std::vector<long> tions(nsp, 0);
        for (long i = 0; i < N; ++i) tions[(int)ion[9 * i + 4] - 1]++;
        if (info) {
            std::memset(info, 0, sizeof(*info));
            info->ranks = ranks_in;
            info->model = d.ising ? ETHER_MODEL_ISING : ETHER_MODEL_XYZ;
            info->n_sites = (int32_t)N;
            info->n_species = nsp;
            info->n_shells = d.nsh;
            info->n_temperatures = (int32_t)nscan;
            info->repeat = (int32_t)d.repeat;
        }
        make_dir(out);
        make_dir(out + "/data");
        make_dir(out + "/spins");
        write_file(out + "/deck.txt", listing(d, nscan, nbasis));
        {
            std::string o = xsf_header(d, N);
            for (long i = 0; i < N; ++i) {  // format 101: (A5, 7f13.7), positions only
                o += fA(d.species[(int)ion[9 * i + 4] - 1], 2, 5);
                for (int k = 6; k <= 8; ++k) o += fF(ion[9 * i + k], 13, 7);
                o += "\n";
            }
            write_file(out + "/data/fetched_lattice_network.xsf", o);
        }
        write_file(out + "/data/nbd.dat", nbd_text(d, N, cap, nn));
        if (flags & ETHER_RUN_PARSE_ONLY) return ETHER_OK;
        // ------------------------------------------ the temperature scan (src/ether.f90) ----
        if (nscan < 1 || d.repeat < 1) perr("nothing to run: no temperatures or REPEAT < 1");
        if (d.coa < 1.0 || d.coa != std::floor(d.coa) || d.coa > 2147483647.0)
            perr("coa must be a positive whole number of steps");
        if (d.tmcs < 1 || d.tmcs > 2147483647L || d.tmcs_eq < 0) perr("mcs out of range");
        std::vector<double> temperature(nscan);
        for (long t = 0; t < nscan; ++t) temperature[t] = d.ht - d.tint * (double)t;
        const long P = (ranks_in > 0 && ranks_in < nscan) ? ranks_in : nscan;
        const long rounds = (nscan + P - 1) / P;
        const int rep = (int)d.repeat;
        const int nobs = 20 + 3 * nsp;
        std::vector<double> obs((size_t)nobs * nscan, 0.0);
        const bool ssp = d.ssp && d.xyz;
        const bool resume = (flags & ETHER_RUN_RESUME) != 0;
        const size_t rec_bytes = (size_t)9 * N * sizeof(double);  // one ETHER.spn record: ion(0:8, N)
        if (resume) {
            struct stat st;
            if (stat((out + "/ETHER.spn").c_str(), &st) != 0) perr("resume: ETHER.spn not found in the output directory");
            if ((size_t)st.st_size != rec_bytes * (size_t)nscan)
                perr("resume: ETHER.spn does not hold one record of this lattice per temperature");
        }
        // Written as the rounds finish, temperature by temperature: ETHER.spn (src/rw_file.f90),
        // the gss.dat blocks (src/write_gss.f90) and the spK files; the rest from ETHER.obs at the end.
        OutFile spn_f(out + "/ETHER.spn", resume ? "r+b" : "wb");
        OutFile gss_f(out + "/data/gss.dat", "wb");
        {  // gss.dat header (src/write_gss.f90:41-63)
            std::string g = fI(nscan, 5) + " " + fI(d.sc[0], 5) + " " + fI(d.sc[1], 5) + " " + fI(d.sc[2], 5) + "\n";
            g += fI(1, 5) + " " + fI(1, 5) + " " + fI(1, 5) + " " + fI(d.sc[0], 5) + " " + fI(d.sc[1], 5) + " " +
                 fI(d.sc[2], 5) + "\n";
            g += fI(nbasis, 5) + " " + fI(nsp, 5) + fF(d.ht, 11, 5) + " " + fF(d.lt, 11, 5) + " " + fF(d.tint, 11, 5) + "\n";
            g += fA(d.para ? " KbT/J" : " K", 30, 20) + "\n";
            for (int k = 0; k < nsp; k += 5) {  // (I8,1x,I8,1x,I8,1x,I8,1x,I8), reverting after five
                for (int j = k; j < std::min(nsp, k + 5); ++j) g += (j > k ? " " : "") + fI(tions[j], 8);
                g += "\n";
            }
            for (int i = 0; i < 3; ++i)
                g += fF(d.abc[3 * i], 10, 5) + " " + fF(d.abc[3 * i + 1], 10, 5) + " " + fF(d.abc[3 * i + 2], 10, 5) + "\n";
            g += " # lattice points\n";
            for (long i = 0; i < N; ++i)
                g += fF(ion[9 * i + 6], 11, 6) + " " + fF(ion[9 * i + 7], 11, 6) + " " + fF(ion[9 * i + 8], 11, 6) + " " +
                     fI((long)ion[9 * i], 8) + "\n";
            gss_f.put(g);
        }
        ether_schedule sch;
        std::memset(&sch, 0, sizeof(sch));
        sch.tmcs_eq = (int32_t)d.tmcs_eq;
        sch.coa = (int32_t)d.coa;
        sch.ovrr = d.ovrr ? 1 : 0;  // ether_mcs applies the rest of the gate (src/ether.f90:163-167)
        sch.ovrr_para = d.ovrr_para;
        sch.ovrr_mcs = (int32_t)d.ovrr_mcs;
        sch.pt = d.pt ? 1 : 0;
        sch.exchange_interval = (int32_t)d.exchange_interval;
        std::vector<double> carry;  // per slot of the last round: 9N each
        double secs = 0.0;
        uint64_t updates = 0;
        for (long e = 0; e < rounds; ++e) {
            const long t0 = e * P;
            const int np = (int)std::min(P, nscan - t0);
            const int R = np * rep;
            ether_desc desc;
            std::memset(&desc, 0, sizeof(desc));
            desc.n_sites = (int32_t)N;
            desc.n_species = nsp;
            desc.n_shells = d.nsh;
            desc.nbd_capacity = cap;
            desc.model = d.ising ? ETHER_MODEL_ISING : ETHER_MODEL_XYZ;
            desc.angle = d.angle ? 1 : 0;
            desc.dphi = d.dphi;
            desc.zeeman = d.zeeman ? 1 : 0;
            for (int a = 0; a < 3; ++a) desc.h[a] = d.h[a];
            desc.g_factor = d.g_factor;
            desc.mb = d.mb;
            desc.sia = (d.sia && d.xyz) ? 1 : 0;
            desc.ion = ion.data();
            desc.nn = nn.data();
            desc.j_exc = d.j_exc.data();
            desc.sia_vec = desc.sia ? d.sia_vec.data() : nullptr;
            desc.s = d.s.data();
            desc.stgg = stgg.data();
            desc.n_replicas = R;
            desc.seed = (uint32_t)d.seed;
            for (int a = 0; a < 3; ++a) desc.sc[a] = sc[a];
            desc.basis = nbasis;
            if (ctx) {
                ether_destroy(ctx);
                ctx = nullptr;
            }
            RTRY(ether_create(&desc, &ctx));
            std::vector<double> beta(np);
            for (int s = 0; s < np; ++s) beta[s] = 1.0 / (d.kb * temperature[t0 + s]);
            RTRY(ether_set_ladder(ctx, np, beta.data()));
            // streams: one per (temperature, REPEAT), distinct across rounds
            std::vector<uint32_t> sid(R), st(R, 0);
            for (int g = 0; g < rep; ++g)
                for (int s = 0; s < np; ++s) sid[(size_t)g * np + s] = (uint32_t)((size_t)g * nscan + t0 + s);
            RTRY(ether_set_streams(ctx, sid.data(), st.data()));
            // start states: the lattice's, a slot's state carried from the last round, or
            // the temperature's record of ETHER.spn
            if (resume || !carry.empty()) {
                std::vector<double> rec((size_t)9 * N);
                for (int s = 0; s < np; ++s) {
                    const double *src = rec.data();
                    if (resume) spn_f.get_record(t0 + s, rec.data(), rec_bytes);
                    else src = carry.data() + (size_t)9 * N * s;
                    for (int g = 0; g < rep; ++g) RTRY(ether_set_spins(ctx, g * np + s, src));
                }
            }
            if (!resume) RTRY(ether_fresh_spins(ctx));  // src/ether.f90:155
            RTRY(ether_zero_avg(ctx));
            RTRY(ether_reset_accept_counts(ctx));
            if (ssp) {
                const double dir3[3] = {d.ss_direc[0], d.ss_direc[1], d.ss_direc[2]};
                int64_t spiral_count = 0;
                RTRY(ether_spiral_setup(ctx, d.ss_dis, dir3, d.ss_lat, (int32_t)d.spiral_capacity, &spiral_count));
            }
            // the MCS loop, in pieces so that a STATUS file can be answered (src/get_status.f90)
            int32_t swaps = 0;
            const auto c0 = std::chrono::steady_clock::now();
            const int32_t piece = 2000;
            for (int32_t step0 = 0; step0 < (int32_t)d.tmcs; step0 += piece) {
                const int32_t n = (int32_t)std::min<long>(piece, d.tmcs - step0);
                RTRY(ether_mcs(ctx, &sch, step0, n, &swaps));
                if (file_exists(out + "/STATUS")) {
                    RTRY(ether_sync(ctx));
                    if (!quiet)
                        std::printf("STATUS >> temperatures %ld-%ld of %ld, MCS %d/%ld, REPEATs 1-%d side by side\n",
                                    t0 + 1, t0 + np, nscan, step0 + n, d.tmcs, rep);
                    std::remove((out + "/STATUS").c_str());
                }
            }
            RTRY(ether_sync(ctx));
            secs += std::chrono::duration<double>(std::chrono::steady_clock::now() - c0).count();
            updates += (uint64_t)N * (uint64_t)R * (uint64_t)d.tmcs;
            // observables per repeat (src/ether.f90:205-214)
            std::vector<double> avg((size_t)6 * R), mean, err;
            RTRY(ether_avg(ctx, avg.data()));
            per_repeat(avg, 6, np, rep, mean, err);
            std::vector<double> smean, serr;
            if (ssp) {
                std::vector<double> savg((size_t)3 * R);
                RTRY(ether_spiral_avg(ctx, savg.data()));
                per_repeat(savg, 3, np, rep, smean, serr);
            } else {  // the accumulators stay zero: zero means, zero errors (NaN for one REPEAT)
                per_repeat(std::vector<double>((size_t)3 * R, 0.0), 3, np, rep, smean, serr);
            }
            std::vector<uint64_t> accepts(R);
            RTRY(ether_get_slot_accept_counts(ctx, accepts.data()));
            std::vector<int32_t> slots(R);
            RTRY(ether_get_slots(ctx, slots.data()));
            std::vector<double> mm((size_t)R * nsp * 3);
            RTRY(ether_moment_vectors(ctx, mm.data()));
            carry.assign((size_t)9 * N * np, 0.0);
            // the configuration the last REPEAT left at each temperature
            std::vector<int> last(np, -1);
            for (int s = 0; s < np; ++s) {
                for (int r = (rep - 1) * np; r < R; ++r)
                    if (slots[r] == s) last[s] = r;
                if (last[s] < 0) throw RunError{ETHER_ERR_STATE};
                std::copy(ion.begin(), ion.end(), carry.begin() + (size_t)9 * N * s);
                RTRY(ether_get_spins(ctx, last[s], carry.data() + (size_t)9 * N * s));
            }
            // gss.dat blocks (src/write_gss.f90:65-77) and <T>spK.xsf files
            // (src/write_spins_at_K.f90): the text of every temperature is formatted on the
            // host's cores side by side, then written in temperature order
            std::vector<std::string> gss_txt(np), xsf_txt(np);
            {
                const int T = (int)std::max(1u, std::min<unsigned>(std::thread::hardware_concurrency(), (unsigned)np));
                std::vector<std::thread> pool;
                std::vector<std::exception_ptr> failed(T);  // rethrown after the join
                for (int w = 0; w < T; ++w)
                    pool.emplace_back([&, w]() {
                      try {
                        for (int s = w; s < np; s += T) {
                            const double *cfg = carry.data() + (size_t)9 * N * s;
                            std::string g = fF(temperature[t0 + s], 11, 5) + "\n";
                            for (long i = 0; i < N; ++i)
                                g += fF(cfg[9 * i + 1], 11, 6) + " " + fF(cfg[9 * i + 2], 11, 6) + " " +
                                     fF(cfg[9 * i + 3], 11, 6) + " " + fI((long)cfg[9 * i + 4], 8) + "\n";
                            std::string xs = xsf_header(d, N);
                            for (long i = 0; i < N; ++i) {  // format 101: (A5, 1x, six f13.7 separated by 1x)
                                xs += fA(d.species[(int)cfg[9 * i + 4] - 1], 2, 5);
                                for (int k : {6, 7, 8, 1, 2, 3}) xs += " " + fF(cfg[9 * i + k], 13, 7);
                                xs += "\n";
                            }
                            gss_txt[s].swap(g);
                            xsf_txt[s].swap(xs);
                        }
                      } catch (...) {
                        failed[w] = std::current_exception();
                      }
                    });
                for (auto &th : pool) th.join();
                for (const std::exception_ptr &e : failed)
                    if (e) std::rethrow_exception(e);
            }
            for (int s = 0; s < np; ++s) {
                const long t = t0 + s;
                const int r_last = last[s];
                spn_f.put_record(t, carry.data() + (size_t)9 * N * s, rec_bytes);
                gss_f.put(gss_txt[s]);
                // name: format(f9.4, 'spK.xsf'), adjustl
                write_file(out + "/spins/" + trim(fF(temperature[t], 9, 4) + "spK.xsf"), xsf_txt[s]);
                std::string().swap(gss_txt[s]);
                std::string().swap(xsf_txt[s]);
                double acc = 0.0;  // acceptance_counting / (repeat tmcs), src/ether.f90:212
                for (int g = 0; g < rep; ++g) acc += (double)accepts[(size_t)g * np + s] / (double)N;
                acc /= (double)rep * (double)d.tmcs;
                const double *mu = mean.data() + 6 * s, *er = err.data() + 6 * s;  // (e, U_E, Cv, m, U_M, chi)
                const double *smu = smean.data() + 3 * s, *ser = serr.data() + 3 * s;
                double *o = obs.data() + (size_t)nobs * t;  // src/process_observables.f90:42-73
                o[0] = temperature[t];
                o[1] = mu[3]; o[2] = mu[5]; o[3] = er[3]; o[4] = er[5]; o[5] = mu[4]; o[6] = er[4];
                o[7] = mu[0]; o[8] = mu[2]; o[9] = er[0]; o[10] = er[2]; o[11] = mu[1]; o[12] = er[1];
                o[13] = acc * 100.0;
                o[14] = smu[0]; o[15] = smu[2]; o[16] = ser[0]; o[17] = ser[2]; o[18] = smu[1]; o[19] = ser[1];
                for (int k = 0; k < nsp; ++k)
                    for (int a = 0; a < 3; ++a) o[20 + 3 * k + a] = mm[((size_t)r_last * nsp + k) * 3 + a];
                if (!quiet) std::printf(" Task for temperature %11.4g is completed.\n", temperature[t]);
            }
            if (!quiet) std::fflush(stdout);
        }
        ether_destroy(ctx);
        ctx = nullptr;
        // ------------------------------------------------------------------ output files ----
        write_file(out + "/ETHER.obs", std::string(reinterpret_cast<const char *>(obs.data()), obs.size() * sizeof(double)));
        static const char *m_head[7] = {"# 1 Temp.", "2 |M|", "3 \xcf\x87", "4 \xce\x94|M|", "5 \xce\x94\xcf\x87",
                                        "6 U(|M|)", "7 \xce\x94U(|M|)"};
        static const char *ss_head[7] = {"# 1 Temp.", "2 |\xcf\x88|", "3 \xcf\x88", "4 \xce\x94|\xcf\x88|",
                                         "5 \xce\x94\xcf\x88", "6 U(|\xcf\x88|)", "7 \xce\x94U(|\xcf\x88|)"};
        const char *e_head[8] = {"# 1 Temp.", "2 E", d.para ? "3 Cv" : "3 Cv/kB", "4 \xce\x94" "E",
                                 d.para ? "5 \xce\x94" "Cv" : "5 \xce\x94(Cv/kB)", "6 U(E)", "7 \xce\x94U(E)",
                                 "8 Accpt. (%)"};
        auto head103 = [](const char *const *h) {  // (A13,A13,A13,1x,A13,1x,A13,2x,A13,A13)
            return fA(h[0], 20, 13) + fA(h[1], 20, 13) + fA(h[2], 20, 13) + " " + fA(h[3], 20, 13) + " " +
                   fA(h[4], 20, 13) + "  " + fA(h[5], 20, 13) + fA(h[6], 20, 13) + "\n";
        };
        std::string mag = head103(m_head), sss = ssp ? head103(ss_head) : std::string();
        // (A13,A13,A13,A13,1x,A13,1x,A13,A13,A13)
        std::string eng = fA(e_head[0], 20, 13) + fA(e_head[1], 20, 13) + fA(e_head[2], 20, 13) +
                          fA(e_head[3], 20, 13) + " " + fA(e_head[4], 20, 13) + " " + fA(e_head[5], 20, 13) +
                          fA(e_head[6], 20, 13) + fA(e_head[7], 20, 13) + "\n";
        std::string mom = " # Showing moment vectors (Mx, My, Mz) for species(sp):\n";
        {  // format 105: (' #<tab>', 5A3), reverting to a new record after five names
            const size_t n = d.included_id.size();
            size_t i = 0;
            do {
                mom += " #\t";
                for (size_t k = 0; k < 5 && i < n; ++k, ++i) {
                    const int id = d.included_id[i];
                    mom += fA(id > 0 ? d.species[id - 1] : std::string("  "), 2, 3);
                }
                mom += "\n";
            } while (i < n);
        }
        mom += " # Temp, sp1(Mx,My,Mz), sp1(Mx,My,Mz),..spN(Mx,My,Mz), sp1|M|, sp2|M|,..spN|M|\n";
        for (long t = 0; t < nscan; ++t) {
            const double *o = obs.data() + (size_t)nobs * t;
            // format 102: (f11.5, 1x, es12.5 x6, 1x, f7.2)
            mag += fF(o[0], 11, 5);
            for (int k = 1; k <= 6; ++k) mag += " " + fES(o[k], 12, 5);
            mag += "\n";
            eng += fF(o[0], 11, 5);
            for (int k = 7; k <= 12; ++k) eng += " " + fES(o[k], 12, 5);
            eng += " " + fF(o[13], 7, 2) + "\n";
            if (ssp) {
                sss += fF(o[0], 11, 5);
                for (int k = 14; k <= 19; ++k) sss += " " + fES(o[k], 12, 5);
                sss += "\n";
            }
            // format 101: (f11.5, 2X, 500f9.3): the included species' M / tions, then |M| / tions
            mom += fF(o[0], 11, 5) + "  ";
            for (int id : d.included_id)
                if (id > 0)
                    for (int a = 0; a < 3; ++a) mom += fF(o[20 + 3 * (id - 1) + a] / (double)tions[id - 1], 9, 3);
            for (int id : d.included_id)
                if (id > 0) {
                    const double *m = o + 20 + 3 * (id - 1);
                    mom += fF(std::sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]) / (double)tions[id - 1], 9, 3);
                }
            mom += "\n";
        }
        write_file(out + "/data/magnetization.dat", mag);
        write_file(out + "/data/energy.dat", eng);
        write_file(out + "/data/moment_vectors.dat", mom);
        write_file(out + "/data/spiral_state_parameters.dat", sss);
        write_file(out + "/data/graph.sh", graph_text(d));
        if (info) {
            info->n_rounds = (int32_t)rounds;
            info->seconds = secs;
            info->site_updates = updates;
        }
        return ETHER_OK;
    } catch (const DeckError &e) {
        if (ctx) ether_destroy(ctx);
        ether::set_error("ether_run: " + e.msg);
        return e.code;
    } catch (const RunError &e) {
        if (ctx) ether_destroy(ctx);
        return e.code;
    } catch (const std::exception &e) {
        if (ctx) ether_destroy(ctx);
        ether::set_error(std::string("ether_run: ") + e.what());
        return ETHER_ERR_NOMEM;
    }
}
