// lattice.cpp -- generate_supercell (src/generate_supercell.f90:38-132) and the neighbour
// search of getting_nbd / search_nbd (src/getting_nbd.f90:34-82, src/search_nbd.f90:20-64)
// in O(N).
//
// The reference compares every pair of sites (O(N^2)) under the 27 periodic images
// {0,+1,-1}^3 of the supercell (only the 0 image along an open axis), and captures j for
// shell b when |d_b - |r_i - r_j'|| <= nbdfc for any image j'.  Here the candidates come
// from cell offsets: for basis atoms l, l' the displacement o.abc + b_l' - b_l depends only
// on the cell offset o, so the offsets whose length can fall inside a shell are found once
// per basis pair; each site then visits only those cells.  Every candidate is confirmed with
// the reference's own test (same image order and the same floating-point expression), and
// the captured sites are emitted in increasing site number, which is the reference's order.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/ether_gpu.h"

extern "C" const char *ether_last_error(void);
namespace ether {
void set_error(const std::string &msg);
}

namespace {

struct V3 {
    double x, y, z;
};

inline double reference_distance(const double *p0, const double *p1, const double SC[3][3], int a,
                                 int b, int c) {
    double r[3];
    for (int d = 0; d < 3; ++d) {
        double q = SC[0][d] * a + SC[1][d] * b + SC[2][d] * c + p1[d];
        r[d] = p0[d] - q;
    }
    return std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
}

}  // namespace

extern "C" int ether_build_lattice(int32_t nbasis, const double *basis_cart,
                                   const int32_t *basis_species, const double *abc,
                                   const int32_t sc[3], const char bc[3], int32_t checkerboard,
                                   int32_t nsh, const double *nbd_dis, double tol, int32_t cap,
                                   double *ion, double *stgg, int32_t *nn) {
    if (nbasis <= 0 || !basis_cart || !basis_species || !abc || !sc || !bc || !ion ||
        (nsh > 0 && (!nbd_dis || !nn)) || nsh < 0 || cap < 0 || sc[0] <= 0 || sc[1] <= 0 ||
        sc[2] <= 0) {
        ether::set_error("ether_build_lattice: invalid argument");
        return ETHER_ERR_ARG;
    }
    const long Nl = (long)sc[0] * sc[1] * sc[2] * nbasis;
    if (Nl > 0x7FFFFFFFL / 16) {
        ether::set_error("ether_build_lattice: lattice too large");
        return ETHER_ERR_ARG;
    }
    const int N = (int)Nl;
    // ---- supercell, generate_supercell.f90:109-132 (x fastest, then y, z; basis innermost)
    int n = 0;
    for (int k = 1; k <= sc[2]; ++k)
        for (int j = 1; j <= sc[1]; ++j)
            for (int i = 1; i <= sc[0]; ++i)
                for (int l = 1; l <= nbasis; ++l) {
                    double *r = ion + 9 * (size_t)n;
                    r[0] = n + 1;
                    r[1] = 0.0;
                    r[2] = 0.0;
                    r[3] = (l % 2 == 0) ? 1.0 : -1.0;
                    r[4] = basis_species[l - 1];
                    r[5] = 0.0;
                    for (int d = 0; d < 3; ++d)
                        r[6 + d] = abc[0 * 3 + d] * (i - 1) + abc[1 * 3 + d] * (j - 1) +
                                   abc[2 * 3 + d] * (k - 1) + basis_cart[3 * (l - 1) + d];
                    if (stgg) stgg[n] = checkerboard ? (((i + j + k + l) % 2 == 0) ? 1.0 : -1.0) : 1.0;
                    ++n;
                }
    if (nsh == 0) return ETHER_OK;

    double SC[3][3];
    for (int a = 0; a < 3; ++a)
        for (int d = 0; d < 3; ++d) SC[a][d] = sc[a] * abc[3 * a + d];
    bool closed[3];
    for (int a = 0; a < 3; ++a) closed[a] = !(bc[a] == 'o' || bc[a] == 'O');

    // ---- candidate cell offsets per (l, l'): |o.abc + b_l' - b_l| within the largest shell
    double dmax = 0.0;
    for (int b = 0; b < nsh; ++b) dmax = std::max(dmax, nbd_dis[b]);
    dmax += tol + 1e-6 * (1.0 + dmax);
    // bound on |o_a|: distance to the plane spanned by the other two vectors
    int omax[3];
    {
        V3 a[3];
        for (int q = 0; q < 3; ++q) a[q] = V3{abc[3 * q], abc[3 * q + 1], abc[3 * q + 2]};
        auto cross = [](V3 u, V3 v) { return V3{u.y * v.z - u.z * v.y, u.z * v.x - u.x * v.z, u.x * v.y - u.y * v.x}; };
        auto dot = [](V3 u, V3 v) { return u.x * v.x + u.y * v.y + u.z * v.z; };
        double vol = std::fabs(dot(a[0], cross(a[1], a[2])));
        if (!(vol > 0.0)) {
            ether::set_error("ether_build_lattice: lattice vectors are degenerate");
            return ETHER_ERR_ARG;
        }
        double bspan = 0.0;
        for (int l = 0; l < nbasis; ++l)
            for (int m = 0; m < nbasis; ++m) {
                double dx = basis_cart[3 * m] - basis_cart[3 * l], dy = basis_cart[3 * m + 1] - basis_cart[3 * l + 1],
                       dz = basis_cart[3 * m + 2] - basis_cart[3 * l + 2];
                bspan = std::max(bspan, std::sqrt(dx * dx + dy * dy + dz * dz));
            }
        for (int q = 0; q < 3; ++q) {
            V3 cr = cross(a[(q + 1) % 3], a[(q + 2) % 3]);
            double h = vol / std::sqrt(dot(cr, cr));
            omax[q] = (int)std::ceil((dmax + bspan) / h) + 1;
            // the reference reaches offsets up to 2*sc-1 (image shifts of +-1 supercell)
            omax[q] = std::min(omax[q], closed[q] ? 2 * sc[q] - 1 : sc[q] - 1);
        }
    }
    struct Off {
        int o[3];
        int lp;
    };
    std::vector<std::vector<Off>> offs(nbasis);
    for (int l = 0; l < nbasis; ++l)
        for (int lp = 0; lp < nbasis; ++lp)
            for (int o0 = -omax[0]; o0 <= omax[0]; ++o0)
                for (int o1 = -omax[1]; o1 <= omax[1]; ++o1)
                    for (int o2 = -omax[2]; o2 <= omax[2]; ++o2) {
                        double v[3];
                        for (int d = 0; d < 3; ++d)
                            v[d] = abc[d] * o0 + abc[3 + d] * o1 + abc[6 + d] * o2 +
                                   basis_cart[3 * lp + d] - basis_cart[3 * l + d];
                        double len = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
                        if (len <= dmax) offs[l].push_back(Off{{o0, o1, o2}, lp});
                    }

    const size_t cap1 = (size_t)cap + 1;
    std::memset(nn, 0, sizeof(int32_t) * (size_t)nsh * N * cap1 * 2);
    const int to[3] = {closed[0] ? 3 : 1, closed[1] ? 3 : 1, closed[2] ? 3 : 1};
    const int shift[3] = {0, 1, -1};
    std::vector<int> cand;
    std::vector<int> got;
    for (int i = 0; i < N; ++i) {
        const int l = i % nbasis;
        const int cell = i / nbasis;
        const int ci[3] = {cell % sc[0], (cell / sc[0]) % sc[1], cell / (sc[0] * sc[1])};
        cand.clear();
        for (const Off &f : offs[l]) {
            int cj[3];
            bool ok = true;
            for (int a = 0; a < 3 && ok; ++a) {
                int t = ci[a] + f.o[a];
                int m = ((t % sc[a]) + sc[a]) % sc[a];
                int s = (t - m) / sc[a];
                if (closed[a] ? (s < -1 || s > 1) : (s != 0)) ok = false;
                cj[a] = m;
            }
            if (!ok) continue;
            int j = f.lp + nbasis * (cj[0] + sc[0] * (cj[1] + sc[1] * cj[2]));
            if (j != i) cand.push_back(j);
        }
        std::sort(cand.begin(), cand.end());
        cand.erase(std::unique(cand.begin(), cand.end()), cand.end());
        const double *p0 = ion + 9 * (size_t)i + 6;
        for (int b = 0; b < nsh; ++b) {
            got.clear();
            for (int j : cand) {
                const double *p1 = ion + 9 * (size_t)j + 6;
                bool captured = false;
                for (int a = 0; a < to[0] && !captured; ++a)
                    for (int bb = 0; bb < to[1] && !captured; ++bb)
                        for (int c = 0; c < to[2] && !captured; ++c)
                            if (std::fabs(nbd_dis[b] - reference_distance(p0, p1, SC, shift[a], shift[bb], shift[c])) <= tol)
                                captured = true;
                if (captured) got.push_back(j);
            }
            if ((int)got.size() > cap) {
                ether::set_error("ether_build_lattice: shell " + std::to_string(b + 1) + " of site " +
                                 std::to_string(i + 1) + " has " + std::to_string(got.size()) +
                                 " neighbours, more than nbd_capacity");
                return ETHER_ERR_CAPACITY;
            }
            nn[b + (size_t)nsh * i] = (int32_t)got.size();
            for (size_t k = 0; k < got.size(); ++k) {
                nn[b + (size_t)nsh * ((size_t)i + (size_t)N * ((k + 1) + cap1 * 0))] = got[k] + 1;
                nn[b + (size_t)nsh * ((size_t)i + (size_t)N * ((k + 1) + cap1 * 1))] = got[k] + 1;
            }
        }
    }
    return ETHER_OK;
}
