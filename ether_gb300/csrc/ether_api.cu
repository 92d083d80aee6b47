// ether_api.cu -- the C-ABI (include/ether_gpu.h): context set-up and the per-MCS calls.
//
// Set-up does on the host, once, what the kernels must not redo per sweep: it reads the
// reference arrays (ion, nn, j_exc, ...), colours the neighbour graph greedily in site
// order, lays the sites out colour-major, converts the nn table to CSR in that order,
// recognises the even periodic simple-cubic lattice (arithmetic neighbours), and builds
// the FP64 Ising acceptance-threshold tables per temperature slot.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <atomic>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include <sys/mman.h>
#include <unistd.h>

#include "internal.h"

using namespace ether;

static thread_local std::string g_err;

static int fail(int code, const std::string &msg) {
    g_err = msg;
    return code;
}

void ether::set_error(const std::string &msg) { g_err = msg; }

// A failed call is reported here and its error read off the runtime (cudaGetLastError), so
// that a later launch check does not report it again; a sticky error stays with the context.
#define CUDA_TRY(expr)                                                                     \
    do {                                                                                   \
        cudaError_t _e = (expr);                                                           \
        if (_e != cudaSuccess) {                                                           \
            cudaGetLastError();                                                            \
            return fail(_e == cudaErrorMemoryAllocation ? ETHER_ERR_NOMEM : ETHER_ERR_CUDA, \
                        std::string(#expr) + ": " + cudaGetErrorString(_e));               \
        }                                                                                  \
    } while (0)

extern "C" int ether_abi_version(void) { return ETHER_ABI_VERSION; }
extern "C" const char *ether_last_error(void) { return g_err.c_str(); }

namespace {

template <class T>
int dev_alloc(Ctx &c, T **p, size_t n) {
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc((void **)p, n * sizeof(T));
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(ETHER_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    }
    c.device_bytes += n * sizeof(T);
    return ETHER_OK;
}

template <class T>
int dev_upload(Ctx &c, T **p, const std::vector<T> &v) {
    int rc = dev_alloc(c, p, v.size());
    if (rc) return rc;
    if (!v.empty()) CUDA_TRY(cudaMemcpy(*p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    return ETHER_OK;
}

struct Nbr {
    int j;   // 0-based site
    int b;   // shell
    int sj;  // 1-based species
};

// ---------------------------------------------------------------- Ising tables --------
// Site type = (species, neighbours per (shell, neighbour-species) group).  Index inside a
// type's half-table = sum over groups of stride_g * (up neighbours in g).
int build_ising_types(Ctx &c, const std::vector<int> &sp, const std::vector<std::vector<Nbr>> &adj,
                      std::vector<uint16_t> &itype_site, std::vector<int32_t> &wstride_site) {
    const int G = c.nsh * c.nsp;
    std::map<std::vector<int>, int> types;
    std::vector<std::vector<int>> keys;
    itype_site.assign(c.N, 0);
    for (int i = 0; i < c.N; ++i) {
        std::vector<int> key(G + 1, 0);
        key[0] = sp[i];
        for (const Nbr &n : adj[i]) key[1 + n.b * c.nsp + (n.sj - 1)]++;
        auto it = types.find(key);
        int id;
        if (it == types.end()) {
            id = (int)keys.size();
            types.emplace(key, id);
            keys.push_back(key);
        } else {
            id = it->second;
        }
        itype_site[i] = (uint16_t)id;
    }
    if (keys.size() > 65535) return fail(ETHER_ERR_CAPACITY, "too many Ising site types");
    c.n_types = (int)keys.size();
    c.h_type_base.assign(c.n_types, 0);
    c.h_type_half.assign(c.n_types, 0);
    c.type_groupcount.assign(c.n_types, std::vector<int>(G, 0));
    c.type_species.assign(c.n_types, 0);
    std::vector<std::vector<int>> strides(c.n_types, std::vector<int>(G, 0));
    long total = 0;
    for (int ty = 0; ty < c.n_types; ++ty) {
        long half = 1;
        for (int g = 0; g < G; ++g) {
            c.type_groupcount[ty][g] = keys[ty][1 + g];
            strides[ty][g] = (int)half;
            half *= (keys[ty][1 + g] + 1);
            if (half > (1L << 22)) return fail(ETHER_ERR_CAPACITY, "Ising threshold table too large");
        }
        c.type_species[ty] = keys[ty][0];
        c.h_type_half[ty] = (int)half;
        c.h_type_base[ty] = (int)total;
        total += 2 * half;
        if (total > (1L << 24)) return fail(ETHER_ERR_CAPACITY, "Ising threshold table too large");
    }
    c.table_entries = (int)total;
    // strides per (type, group); emitted per CSR slot by the caller
    wstride_site.resize((size_t)c.n_types * G);
    for (int ty = 0; ty < c.n_types; ++ty)
        for (int g = 0; g < G; ++g) wstride_site[(size_t)ty * G + g] = strides[ty][g];
    return ETHER_OK;
}

// Thresholds for one temperature: the same FP64 expression as the oracle's colour mode.
// A site flips iff its uniform u32 u <= T, T = max(ceil(2^32 p), 1) - 1 with
// p = exp(-beta dE): the reference's -beta dE > log(eta) for eta = u 2^-32, where eta = 0
// (log = -inf) always accepts.
void ising_thresholds(const Ctx &c, double beta, uint32_t *thr) {
    const int G = c.nsh * c.nsp;
    std::vector<int> nup(G);
    for (int ty = 0; ty < c.n_types; ++ty) {
        const int si = c.type_species[ty];
        const std::vector<int> &cnt = c.type_groupcount[ty];
        const int half = c.h_type_half[ty];
        const double gms = c.g * c.mb * c.s_len[si - 1];
        for (int own = 0; own < 2; ++own) {
            const double sig = own ? 1.0 : -1.0;
            for (int idx = 0; idx < half; ++idx) {
                int rem = idx;
                for (int g = 0; g < G; ++g) {
                    nup[g] = rem % (cnt[g] + 1);
                    rem /= (cnt[g] + 1);
                }
                double field = 0.0;
                for (int b = 0; b < c.nsh; ++b)
                    for (int q = 0; q < c.nsp; ++q) {
                        const int g = b * c.nsp + q;
                        const int m = 2 * nup[g] - cnt[g];
                        const size_t jx = (size_t)b * c.nsp * c.nsp + (size_t)(si - 1) * c.nsp + q;
                        field += c.h_Jd[3 * jx + 2] * (double)m;
                    }
                double dE = (-2.0 * sig) * field;
                if (c.zeeman) dE += -(gms * ((-2.0 * sig) * c.h[2]));
                const double q = std::exp(-beta * dE) * 4294967296.0;
                const size_t e = (size_t)c.h_type_base[ty] + (size_t)own * half + idx;
                if (q >= 4294967296.0) {
                    thr[e] = 0xFFFFFFFFu;
                } else {
                    const double u = std::ceil(q);
                    thr[e] = u < 1.0 ? 0u : (uint32_t)(u - 1.0);
                }
            }
        }
    }
}

int upload_ladder(Ctx &c) {
    std::vector<float> bf(c.n_slots);
    for (int s = 0; s < c.n_slots; ++s) bf[s] = (float)c.beta_slots[s];
    CUDA_TRY(cudaMemcpyAsync(c.beta_slot, c.beta_slots.data(), sizeof(double) * c.n_slots,
                             cudaMemcpyHostToDevice, c.stream));
    CUDA_TRY(cudaMemcpyAsync(c.beta_slot_f, bf.data(), sizeof(float) * c.n_slots,
                             cudaMemcpyHostToDevice, c.stream));
    std::vector<int32_t> sor(c.R), ros(c.R);
    for (int r = 0; r < c.R; ++r) {
        sor[r] = r % c.n_slots;
        ros[r] = r;
    }
    CUDA_TRY(cudaMemcpyAsync(c.slot_of_rep, sor.data(), sizeof(int32_t) * c.R, cudaMemcpyHostToDevice, c.stream));
    CUDA_TRY(cudaMemcpyAsync(c.rep_of_slot, ros.data(), sizeof(int32_t) * c.R, cudaMemcpyHostToDevice, c.stream));
    if (c.model == 0) {
        std::vector<uint32_t> thr((size_t)c.n_slots * c.table_entries);
        for (int s = 0; s < c.n_slots; ++s)
            ising_thresholds(c, c.beta_slots[s], thr.data() + (size_t)s * c.table_entries);
        CUDA_TRY(cudaMemcpyAsync(c.thr, thr.data(), thr.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, c.stream));
        CUDA_TRY(cudaStreamSynchronize(c.stream));
    }
    CUDA_TRY(cudaStreamSynchronize(c.stream));
    c.beta_set = true;
    return ETHER_OK;
}

void free_ctx(Ctx &c) {
    void *ptrs[] = {c.t.row_ptr, c.t.nbr, c.t.jidx, c.t.wstride, c.t.species, c.t.itype,
                    c.t.ell_nbr, c.t.ell_j, c.t.ell_deg, c.t.J4, c.t.ell_ws, c.t.ell_desc,
                    c.t.type_base, c.t.type_half, c.t.J, c.t.Jd, c.t.zee, c.t.zeed, c.t.D,
                    c.t.mweight, c.t.site_of_storage, c.spins, c.spins4, c.beta_slot,
                    c.beta_slot_f, c.slot_of_rep, c.rep_of_slot, c.thr, c.stream_id,
                    c.step, c.ovrr_step, c.fresh_call, c.acc_count, c.E, c.M, c.sums,
                    c.partials, c.pt_accepts, c.swap_dev, c.copy_from, c.err, c.spiral_ptr,
                    c.spiral_nbr, c.acc_before, c.acc_ratio, c.spiral_part, c.spiral_sums,
                    c.acc_slot, c.acc_mark, c.t.sia_cls, c.t.sia_ax, c.t.mweight_f, c.t.storage};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    if (c.acc_host) cudaFreeHost(c.acc_host);
    if (c.stage) cudaFreeHost(c.stage);
    for (cudaEvent_t e : c.ion_ev)
        if (e) cudaEventDestroy(e);
    if (c.ion_copy) cudaStreamDestroy(c.ion_copy);
    for (auto &kv : c.graphs) cudaGraphExecDestroy(kv.second);
    if (c.ev_fork) cudaEventDestroy(c.ev_fork);
    for (int k = 0; k < Ctx::kMaxParts - 1; ++k) {
        if (c.ev_join[k]) cudaEventDestroy(c.ev_join[k]);
        if (c.aux[k]) cudaStreamDestroy(c.aux[k]);
    }
    if (c.stream) cudaStreamDestroy(c.stream);
    c = Ctx();
}

}  // namespace

extern "C" int ether_create(const ether_desc *d, ether_ctx **out) {
    if (!d || !out) return fail(ETHER_ERR_ARG, "null descriptor or output pointer");
    *out = nullptr;
    if (d->n_sites <= 0 || d->n_species <= 0 || d->n_shells < 0 || d->nbd_capacity < 0 ||
        d->n_replicas <= 0)
        return fail(ETHER_ERR_ARG, "non-positive size in descriptor");
    if (d->model != ETHER_MODEL_ISING && d->model != ETHER_MODEL_XYZ)
        return fail(ETHER_ERR_ARG, "model must be ETHER_MODEL_ISING or ETHER_MODEL_XYZ");
    if (!d->ion || !d->s || (d->n_shells > 0 && (!d->nn || !d->j_exc)))
        return fail(ETHER_ERR_ARG, "missing ion, nn, j_exc or s array");
    if (d->sia && d->model == ETHER_MODEL_XYZ && !d->sia_vec)
        return fail(ETHER_ERR_ARG, "sia set but sia_vec is NULL");
    if (d->n_species > 255) return fail(ETHER_ERR_UNSUPPORTED, "more than 255 species");
    if ((long)d->n_shells * d->n_species * d->n_species > 65535)
        return fail(ETHER_ERR_UNSUPPORTED, "too many coupling entries");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return fail(ETHER_ERR_NODEV, "no CUDA device");

    ether_ctx *h = new (std::nothrow) ether_ctx();
    if (!h) return fail(ETHER_ERR_NOMEM, "host allocation failed");
    Ctx &c = h->c;
    c.N = d->n_sites;
    c.nsp = d->n_species;
    c.nsh = d->n_shells;
    c.cap = d->nbd_capacity;
    c.model = d->model;
    c.angle = d->angle ? 1 : 0;
    c.dphi = d->dphi;
    c.zeeman = d->zeeman ? 1 : 0;
    c.sia = (d->sia && d->model == ETHER_MODEL_XYZ) ? 1 : 0;
    c.sia_local = (d->sia_local && d->model == ETHER_MODEL_XYZ) ? 1 : 0;
    for (int k = 0; k < 3; ++k) c.h[k] = d->h[k];
    c.g = d->g_factor;
    c.mb = d->mb;
    c.R = d->n_replicas;
    c.seed = d->seed;
    c.flags = d->flags;
    c.s_len.assign(d->s, d->s + c.nsp);
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&c.sm_count, cudaDevAttrMultiProcessorCount, dev);

    auto bail = [&](int rc) {
        free_ctx(c);
        delete h;
        return rc;
    };

    // ----- species and neighbour lists in the reference's nn order
    const int N = c.N;
    std::vector<int> sp(N);
    for (int i = 0; i < N; ++i) {
        double v = d->ion[4 + 9 * (size_t)i];
        int q = (int)v;
        if (q < 1 || q > c.nsp) return bail(fail(ETHER_ERR_ARG, "ion(4,i) species out of range at site " + std::to_string(i + 1)));
        sp[i] = q;
    }
    std::vector<std::vector<Nbr>> adj(N);
    const size_t cap1 = (size_t)c.cap + 1;
    for (int i = 0; i < N; ++i)
        for (int b = 0; b < c.nsh; ++b) {
            int cnt = d->nn[b + (size_t)c.nsh * i];
            if (cnt < 0 || cnt > c.cap) return bail(fail(ETHER_ERR_ARG, "nn count out of range at site " + std::to_string(i + 1)));
            for (int k = 1; k <= cnt; ++k) {
                int j = d->nn[b + (size_t)c.nsh * ((size_t)i + (size_t)N * ((size_t)k + cap1))];
                if (j < 1 || j > N) return bail(fail(ETHER_ERR_ARG, "nn neighbour index out of range at site " + std::to_string(i + 1)));
                adj[i].push_back(Nbr{j - 1, b, sp[j - 1]});
            }
        }

    // ----- greedy colouring over the symmetric closure
    {
        std::vector<std::vector<int>> und(N);
        for (int i = 0; i < N; ++i)
            for (const Nbr &n : adj[i]) {
                und[i].push_back(n.j);
                und[n.j].push_back(i);
            }
        c.colour.assign(N, -1);
        c.ncol = 0;
        std::vector<int> mark(kMaxColours + 1, -1);
        for (int i = 0; i < N; ++i) {
            for (int j : und[i])
                if (j < i && c.colour[j] >= 0) mark[c.colour[j]] = i;
            int col = 0;
            while (col <= kMaxColours && mark[col] == i) ++col;
            if (col >= kMaxColours) return bail(fail(ETHER_ERR_CAPACITY, "neighbour graph needs more than 64 colours"));
            c.colour[i] = col;
            c.ncol = std::max(c.ncol, col + 1);
        }
        std::vector<int> cnt(c.ncol, 0);
        c.rank.assign(N, 0);
        for (int i = 0; i < N; ++i) c.rank[i] = cnt[c.colour[i]]++;
        c.col_off[0] = 0;
        for (int k = 0; k < c.ncol; ++k) c.col_off[k + 1] = c.col_off[k] + cnt[k];
        c.storage.assign(N, 0);
        c.site_of_storage.assign(N, 0);
        for (int i = 0; i < N; ++i) {
            c.storage[i] = c.col_off[c.colour[i]] + c.rank[i];
            c.site_of_storage[c.storage[i]] = i;
        }
    }

    // ----- simple-cubic fast path: one site per cell, one species, one shell of the six
    //       periodic nearest neighbours, even extents >= 4
    c.fast = false;
    if (!(c.flags & ETHER_FLAG_FORCE_GENERAL) && c.nsp == 1 && c.nsh == 1 && d->basis == 1) {
        const int L1 = d->sc[0], L2 = d->sc[1], L3 = d->sc[2];
        bool ok = L1 >= 4 && L2 >= 4 && L3 >= 4 && L1 % 2 == 0 && L2 % 2 == 0 && L3 % 2 == 0 &&
                  (long)L1 * L2 * L3 == N;
        for (int i = 0; ok && i < N; ++i) {
            int x = i % L1, y = (i / L1) % L2, z = i / (L1 * L2);
            if ((int)adj[i].size() != 6 || c.colour[i] != ((x + y + z) & 1)) { ok = false; break; }
            int want[6] = {((x + 1) % L1) + L1 * (y + L2 * z), ((x + L1 - 1) % L1) + L1 * (y + L2 * z),
                           x + L1 * (((y + 1) % L2) + L2 * z), x + L1 * (((y + L2 - 1) % L2) + L2 * z),
                           x + L1 * (y + L2 * ((z + 1) % L3)), x + L1 * (y + L2 * ((z + L3 - 1) % L3))};
            std::sort(want, want + 6);
            int have[6];
            for (int k = 0; k < 6; ++k) have[k] = adj[i][k].j;
            for (int k = 0; k < 6; ++k)
                if (have[k] != want[k]) { ok = false; break; }
        }
        if (ok) {
            c.L[0] = L1; c.L[1] = L2; c.L[2] = L3;
            const int H = L1 / 2;
            c.vec_bytes = (H % 16 == 0) ? 16 : (H % 8 == 0) ? 8 : (H % 4 == 0) ? 4 : 0;
            c.fast = (c.model == ETHER_MODEL_XYZ) || c.vec_bytes > 0;
        }
    }

    // ----- couplings
    const size_t nJ = (size_t)std::max(1, c.nsh) * c.nsp * c.nsp;
    c.h_Jf.assign(3 * nJ, 0.f);
    c.h_Jd.assign(3 * nJ, 0.0);
    for (int b = 0; b < c.nsh; ++b)
        for (int si = 0; si < c.nsp; ++si)
            for (int sj = 0; sj < c.nsp; ++sj)
                for (int k = 0; k < 3; ++k) {
                    double v = d->j_exc[b + (size_t)c.nsh * (si + (size_t)c.nsp * (sj + (size_t)c.nsp * k))];
                    size_t jx = (size_t)b * c.nsp * c.nsp + (size_t)si * c.nsp + sj;
                    c.h_Jd[3 * jx + k] = v;
                    c.h_Jf[3 * jx + k] = (float)v;
                }
    std::vector<float> zee(3 * c.nsp), D(3 * c.nsp, 0.f);
    std::vector<double> zeed(3 * c.nsp);
    for (int q = 0; q < c.nsp; ++q) {
        double gms = c.g * c.mb * c.s_len[q];
        for (int k = 0; k < 3; ++k) {
            zeed[3 * q + k] = -(gms * c.h[k]);
            zee[3 * q + k] = (float)zeed[3 * q + k];
            if (c.sia) D[3 * q + k] = (float)d->sia_vec[k + 3 * (size_t)q];
        }
    }

    // ----- local-axis anisotropy: distinct (a, D) in FP32 as classes, one byte per site
    std::vector<float4> sia_ax;
    std::vector<uint8_t> sia_site;
    if (c.sia_local) {
        std::map<std::vector<float>, int> cls;
        sia_site.assign(N, 0);
        for (int i = 0; i < N; ++i) {
            const double *a = d->sia_local + 4 * (size_t)i;
            for (int k = 0; k < 4; ++k)
                if (!std::isfinite(a[k])) return bail(fail(ETHER_ERR_ARG, "sia_local is not finite at site " + std::to_string(i + 1)));
            const std::vector<float> key = {(float)a[0], (float)a[1], (float)a[2], (float)a[3]};
            auto it = cls.find(key);
            if (it == cls.end()) {
                if (cls.size() == 256)
                    return bail(fail(ETHER_ERR_CAPACITY, "sia_local: more than 256 distinct (axis, D) pairs"));
                it = cls.emplace(key, (int)cls.size()).first;
                sia_ax.push_back(make_float4(key[0], key[1], key[2], key[3]));
            }
            sia_site[i] = (uint8_t)it->second;
        }
    }

    // ----- CSR in storage order
    std::vector<int32_t> row_ptr(N + 1, 0), nbr, wstr;
    std::vector<uint16_t> jidx;
    std::vector<uint8_t> spc(N);
    std::vector<uint16_t> ity(N, 0);
    std::vector<double> mw(N);
    std::vector<uint16_t> itype_site;
    std::vector<int32_t> type_strides;
    if (c.model == ETHER_MODEL_ISING) {
        int rc = build_ising_types(c, sp, adj, itype_site, type_strides);
        if (rc) return bail(rc);
    }
    const int G = c.nsh * c.nsp;
    for (int s = 0; s < N; ++s) {
        const int i = c.site_of_storage[s];
        for (const Nbr &n : adj[i]) {
            nbr.push_back(c.storage[n.j]);
            jidx.push_back((uint16_t)((size_t)n.b * c.nsp * c.nsp + (size_t)(sp[i] - 1) * c.nsp + (n.sj - 1)));
            if (c.model == ETHER_MODEL_ISING)
                wstr.push_back(type_strides[(size_t)itype_site[i] * G + n.b * c.nsp + (n.sj - 1)]);
        }
        row_ptr[s + 1] = (int32_t)nbr.size();
        spc[s] = (uint8_t)sp[i];
        if (c.model == ETHER_MODEL_ISING) ity[s] = itype_site[i];
        mw[s] = (d->stgg ? d->stgg[i] : 1.0) * c.s_len[sp[i] - 1];
        for (int k = 0; k < 3; ++k) c.pos.push_back(d->ion[6 + k + 9 * (size_t)i]);
    }

    // exact shortcuts of the energy reduction: one z coupling on every bond, one |weight|,
    // weights exact in FP32
    c.juni_set = !jidx.empty();
    if (c.juni_set) {
        c.ising_juni = c.h_Jd[3 * (size_t)jidx[0] + 2];
        for (uint16_t j : jidx)
            if (c.h_Jd[3 * (size_t)j + 2] != c.ising_juni) { c.juni_set = false; break; }
    }
    c.mw_abs = N > 0 ? std::fabs(mw[0]) : 0.0;
    c.mw_pos = N > 0;
    bool mw_f32 = true;
    std::vector<float> mwf(N);
    for (int s = 0; s < N; ++s) {
        if (std::fabs(mw[s]) != c.mw_abs) c.mw_abs = 0.0;
        if (!(mw[s] > 0.0)) c.mw_pos = false;
        mwf[s] = (float)mw[s];
        if ((double)mwf[s] != mw[s]) mw_f32 = false;
    }

    // ----- device
    CUDA_TRY(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking));
    int rc = ETHER_OK;
#define TRY(x) do { rc = (x); if (rc) return bail(rc); } while (0)
    c.nnz = (long)nbr.size();
    TRY(dev_upload(c, &c.t.row_ptr, row_ptr));
    TRY(dev_upload(c, &c.t.nbr, nbr));
    TRY(dev_upload(c, &c.t.jidx, jidx));
    TRY(dev_upload(c, &c.t.wstride, wstr));
    TRY(dev_upload(c, &c.t.species, spc));
    TRY(dev_upload(c, &c.t.itype, ity));
    TRY(dev_upload(c, &c.t.type_base, c.h_type_base));
    TRY(dev_upload(c, &c.t.type_half, c.h_type_half));
    TRY(dev_upload(c, &c.t.J, c.h_Jf));
    TRY(dev_upload(c, &c.t.Jd, c.h_Jd));
    TRY(dev_upload(c, &c.t.zee, zee));
    TRY(dev_upload(c, &c.t.zeed, zeed));
    TRY(dev_upload(c, &c.t.D, D));
    if (c.sia_local) {
        std::vector<uint8_t> scls(N);
        for (int s = 0; s < N; ++s) scls[s] = sia_site[c.site_of_storage[s]];
        TRY(dev_upload(c, &c.t.sia_cls, scls));
        TRY(dev_upload(c, &c.t.sia_ax, sia_ax));
    }
    TRY(dev_upload(c, &c.t.mweight, mw));
    if (mw_f32) TRY(dev_upload(c, &c.t.mweight_f, mwf));
    TRY(dev_upload(c, &c.t.site_of_storage, c.site_of_storage));
    TRY(dev_upload(c, &c.t.storage, c.storage));
    c.ion_direct = !(c.flags & ETHER_FLAG_STAGED_SPINS) && ion_direct_possible(dev);
    {
        // ELL blocks per colour class: coalesced neighbour reads for the general-lattice
        // kernels (XYZ: coupling index per entry; Ising: threshold-table stride per entry)
        std::vector<uint16_t> deg(N);
        c.ell_off.assign(c.ncol + 1, 0);
        c.ell_width.assign(c.ncol, 0);
        for (int col = 0; col < c.ncol; ++col) {
            int w = 0;
            for (int s = c.col_off[col]; s < c.col_off[col + 1]; ++s) {
                const int dg = row_ptr[s + 1] - row_ptr[s];
                if (dg > 65535) return bail(fail(ETHER_ERR_CAPACITY, "more than 65535 neighbours of one site"));
                deg[s] = (uint16_t)dg;
                w = std::max(w, dg);
            }
            c.ell_width[col] = w;
            c.ell_off[col + 1] = c.ell_off[col] + (long)w * (c.col_off[col + 1] - c.col_off[col]);
        }
        if (c.ell_off[c.ncol] >= (1L << 31))  // the kernels index a block with 32-bit ints
            return bail(fail(ETHER_ERR_CAPACITY, "neighbour lists of more than 2^31 entries"));
        const bool xyz = c.model == ETHER_MODEL_XYZ;
        std::vector<int32_t> enb((size_t)c.ell_off[c.ncol], 0);
        std::vector<uint16_t> ej(xyz ? (size_t)c.ell_off[c.ncol] : 0, 0);
        std::vector<int32_t> ews(xyz ? 0 : (size_t)c.ell_off[c.ncol], 0);
        for (int col = 0; col < c.ncol; ++col) {
            const long n_c = c.col_off[col + 1] - c.col_off[col];
            for (long rho = 0; rho < n_c; ++rho) {
                const int s = c.col_off[col] + (int)rho;
                for (int k = 0; k < deg[s]; ++k) {
                    const size_t e = (size_t)c.ell_off[col] + (size_t)k * n_c + rho;
                    enb[e] = nbr[row_ptr[s] + k];
                    if (xyz) ej[e] = jidx[row_ptr[s] + k];
                    else ews[e] = wstr[row_ptr[s] + k];
                }
                for (int k = deg[s]; k < c.ell_width[col]; ++k)  // padding: never read
                    enb[(size_t)c.ell_off[col] + (size_t)k * n_c + rho] = s;
            }
        }
        TRY(dev_upload(c, &c.t.ell_nbr, enb));
        TRY(dev_upload(c, &c.t.ell_deg, deg));
        std::vector<int2> desc(c.ncol);
        for (int col = 0; col < c.ncol; ++col) desc[col] = make_int2((int)c.ell_off[col], c.ell_width[col]);
        TRY(dev_upload(c, &c.t.ell_desc, desc));
        if (xyz) {
            std::vector<float4> j4(c.h_Jf.size() / 3);
            for (size_t q = 0; q < j4.size(); ++q)
                j4[q] = make_float4(c.h_Jf[3 * q], c.h_Jf[3 * q + 1], c.h_Jf[3 * q + 2], 0.f);
            TRY(dev_upload(c, &c.t.ell_j, ej));
            TRY(dev_upload(c, &c.t.J4, j4));
        } else {
            TRY(dev_upload(c, &c.t.ell_ws, ews));
        }
    }
    const size_t RN = (size_t)c.R * N;
    if (c.model == ETHER_MODEL_ISING) TRY(dev_alloc(c, &c.spins, RN));
    else TRY(dev_alloc(c, &c.spins4, RN));
    TRY(dev_alloc(c, &c.beta_slot, c.R));
    TRY(dev_alloc(c, &c.beta_slot_f, c.R));
    TRY(dev_alloc(c, &c.slot_of_rep, c.R));
    TRY(dev_alloc(c, &c.rep_of_slot, c.R));
    if (c.model == ETHER_MODEL_ISING) {
        TRY(dev_alloc(c, &c.thr, (size_t)c.R * c.table_entries));
    }
    TRY(dev_alloc(c, &c.stream_id, c.R));
    TRY(dev_alloc(c, &c.step, c.R));
    TRY(dev_alloc(c, &c.ovrr_step, c.R));
    TRY(dev_alloc(c, &c.fresh_call, c.R));
    TRY(dev_alloc(c, &c.acc_count, c.R));
    TRY(dev_alloc(c, &c.E, 2 * (size_t)c.R));
    TRY(dev_alloc(c, &c.M, 3 * (size_t)c.R));
    TRY(dev_alloc(c, &c.sums, 7 * (size_t)c.R));
    c.partial_blocks = energy_blocks(c);
    {
        // small simple-cubic Ising lattices: ether_mcs keeps each replica in shared memory for
        // the sweeps between two PT or measurement steps, when the replicas alone fill the GPU
        int dev = 0, optin = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        const size_t room = optin > 1024 ? (size_t)optin - 1024 : 0;  // leave the static shared memory
        c.resident = !(c.flags & ETHER_FLAG_NO_RESIDENT) && ising_resident_possible(c, room) &&
                     (long)c.R * c.N <= (16L << 20) && 2 * c.R >= c.sm_count;
        if (c.resident) CUDA_TRY(prepare_ising_resident(c));
    }
    TRY(dev_alloc(c, &c.partials, (size_t)c.R * c.partial_blocks * 5));
    TRY(dev_alloc(c, &c.pt_accepts, 1));
    TRY(dev_alloc(c, &c.swap_dev, 1));
    TRY(dev_alloc(c, &c.err, 1));
    TRY(dev_alloc(c, &c.acc_before, c.R));
    TRY(dev_alloc(c, &c.acc_ratio, c.R));
    TRY(dev_alloc(c, &c.acc_slot, c.R));
    TRY(dev_alloc(c, &c.acc_mark, c.R));
    CUDA_TRY(cudaMallocHost((void **)&c.acc_host, sizeof(double) * c.R));
    CUDA_TRY(cudaMemset(c.err, 0, sizeof(int)));
    TRY(dev_alloc(c, &c.copy_from, c.R));
#undef TRY
    std::vector<uint32_t> sid(c.R);
    std::iota(sid.begin(), sid.end(), 0u);
    CUDA_TRY(cudaMemcpy(c.stream_id, sid.data(), sizeof(uint32_t) * c.R, cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemset(c.step, 0, sizeof(uint32_t) * c.R));
    CUDA_TRY(cudaMemset(c.ovrr_step, 0, sizeof(uint32_t) * c.R));
    CUDA_TRY(cudaMemset(c.fresh_call, 0, sizeof(uint32_t) * c.R));
    CUDA_TRY(cudaMemset(c.acc_count, 0, sizeof(unsigned long long) * c.R));
    CUDA_TRY(cudaMemset(c.acc_slot, 0, sizeof(unsigned long long) * c.R));
    CUDA_TRY(cudaMemset(c.acc_mark, 0, sizeof(unsigned long long) * c.R));
    CUDA_TRY(cudaMemset(c.sums, 0, sizeof(double) * 7 * c.R));
    CUDA_TRY(cudaMemset(c.E, 0, sizeof(double) * 2 * c.R));
    CUDA_TRY(cudaMemset(c.M, 0, sizeof(double) * 3 * c.R));
    c.n_slots = c.R;
    c.n_groups = 1;
    c.beta_slots.assign(c.R, 0.0);
    c.beta_set = false;
    *out = h;
    int src = ether_set_spins(h, -1, d->ion);
    if (src) {
        *out = nullptr;
        return bail(src);
    }
    return ETHER_OK;
}

extern "C" int ether_destroy(ether_ctx *h) {
    if (!h) return ETHER_OK;
    cudaStreamSynchronize(h->c.stream);
    free_ctx(h->c);
    delete h;
    return ETHER_OK;
}

extern "C" int ether_set_beta(ether_ctx *h, const double *beta) {
    if (!h || !beta) return fail(ETHER_ERR_ARG, "null argument");
    Ctx &c = h->c;
    for (int r = 0; r < c.R; ++r)
        if (!std::isfinite(beta[r])) return fail(ETHER_ERR_ARG, "beta is not finite for replica " + std::to_string(r));
    if (c.beta_set) CUDA_TRY(launch_acc_bin(c));
    c.n_slots = c.R;
    c.n_groups = 1;
    c.beta_slots.assign(beta, beta + c.R);
    return upload_ladder(c);
}

extern "C" int ether_set_ladder(ether_ctx *h, int32_t n_slots, const double *beta_slots) {
    if (!h || !beta_slots) return fail(ETHER_ERR_ARG, "null argument");
    Ctx &c = h->c;
    if (n_slots <= 0 || c.R % n_slots != 0) return fail(ETHER_ERR_ARG, "n_slots must divide the replica count");
    for (int s = 0; s < n_slots; ++s)
        if (!std::isfinite(beta_slots[s])) return fail(ETHER_ERR_ARG, "beta is not finite for slot " + std::to_string(s));
    // accepts so far belong to the positions of the old ladder
    if (c.beta_set) CUDA_TRY(launch_acc_bin(c));
    c.n_slots = n_slots;
    c.n_groups = c.R / n_slots;
    c.beta_slots.assign(beta_slots, beta_slots + n_slots);
    return upload_ladder(c);
}

extern "C" int ether_set_streams(ether_ctx *h, const uint32_t *stream, const uint32_t *step) {
    if (!h) return fail(ETHER_ERR_ARG, "null context");
    Ctx &c = h->c;
    if (stream) CUDA_TRY(cudaMemcpyAsync(c.stream_id, stream, sizeof(uint32_t) * c.R, cudaMemcpyHostToDevice, c.stream));
    if (step) CUDA_TRY(cudaMemcpyAsync(c.step, step, sizeof(uint32_t) * c.R, cudaMemcpyHostToDevice, c.stream));
    CUDA_TRY(cudaStreamSynchronize(c.stream));
    return ETHER_OK;
}

extern "C" int ether_set_spins(ether_ctx *h, int32_t replica, const double *ion) {
    if (!h || !ion) return fail(ETHER_ERR_ARG, "null argument");
    Ctx &c = h->c;
    if (replica < -1 || replica >= c.R) return fail(ETHER_ERR_ARG, "replica out of range");
    const int N = c.N;
    if (c.model == ETHER_MODEL_ISING) {
        std::vector<uint8_t> v(N);
        for (int i = 0; i < N; ++i) v[c.storage[i]] = ion[3 + 9 * (size_t)i] > 0.0 ? 1 : 0;
        // one upload; every replica: replicated on the device
        CUDA_TRY(cudaMemcpyAsync(c.spins + (size_t)(replica < 0 ? 0 : replica) * N, v.data(), N,
                                 cudaMemcpyHostToDevice, c.stream));
        if (replica < 0) CUDA_TRY(launch_broadcast(c, c.spins, (size_t)N));
        CUDA_TRY(cudaStreamSynchronize(c.stream));
    } else {
        std::vector<float4> v(N);
        for (int i = 0; i < N; ++i) {
            const double *p = ion + 9 * (size_t)i;
            v[c.storage[i]] = make_float4((float)p[1], (float)p[2], (float)p[3], (float)p[5]);
        }
        CUDA_TRY(cudaMemcpyAsync(c.spins4 + (size_t)(replica < 0 ? 0 : replica) * N, v.data(),
                                 sizeof(float4) * N, cudaMemcpyHostToDevice, c.stream));
        if (replica < 0) CUDA_TRY(launch_broadcast(c, c.spins4, sizeof(float4) * (size_t)N));
        CUDA_TRY(cudaStreamSynchronize(c.stream));
    }
    return ETHER_OK;
}

extern "C" int ether_get_spins(ether_ctx *h, int32_t replica, double *ion) {
    if (!h || !ion) return fail(ETHER_ERR_ARG, "null argument");
    Ctx &c = h->c;
    if (replica < -1 || replica >= c.R) return fail(ETHER_ERR_ARG, "replica out of range");
    if (replica < 0) replica = 0;
    const int N = c.N;
    if (c.model == ETHER_MODEL_ISING) {
        std::vector<uint8_t> v(N);
        CUDA_TRY(cudaMemcpyAsync(v.data(), c.spins + (size_t)replica * N, N, cudaMemcpyDeviceToHost, c.stream));
        CUDA_TRY(cudaStreamSynchronize(c.stream));
        for (int i = 0; i < N; ++i) ion[3 + 9 * (size_t)i] = v[c.storage[i]] ? 1.0 : -1.0;
    } else {
        std::vector<float4> v(N);
        CUDA_TRY(cudaMemcpyAsync(v.data(), c.spins4 + (size_t)replica * N, sizeof(float4) * N, cudaMemcpyDeviceToHost, c.stream));
        CUDA_TRY(cudaStreamSynchronize(c.stream));
        for (int i = 0; i < N; ++i) {
            double *p = ion + 9 * (size_t)i;
            const float4 q = v[c.storage[i]];
            p[1] = q.x; p[2] = q.y; p[3] = q.z; p[5] = q.w;
        }
    }
    return ETHER_OK;
}

// ----------------------------------------------------------------------------------------
// Every replica's ion(0:8, N) at once.  A driver that replaces the reference's MPI ranks by
// the replica batch holds one ion array per replica: n of them back to back, ion(0:8, N, n).
// The conversion to and from the device layout (a strided read or write of ion(3) or
// ion(1:3,5) per 72-byte record, and the colour-major permutation) is the cost of this
// boundary.  Where the device cannot read the records in place (spins_batch below), it runs on
// the host's cores into a pinned staging area, in chunks of whole replicas whose copies start
// as soon as a chunk is converted.
namespace {
constexpr size_t kStageMax = size_t(512) << 20;  // pinned staging, per context
constexpr size_t kChunkBytes = size_t(4) << 20;  // a copy per ~4 MB of spins

int host_threads() {
    const unsigned t = std::thread::hardware_concurrency();
    return (int)std::max(1u, std::min(t, 32u));
}

int ensure_stage(Ctx &c, size_t bytes) {
    if (c.stage_bytes >= bytes) return ETHER_OK;
    if (c.stage) cudaFreeHost(c.stage);
    c.stage = nullptr;
    c.stage_bytes = 0;
    CUDA_TRY(cudaHostAlloc(&c.stage, bytes, cudaHostAllocDefault));
    c.stage_bytes = bytes;
    return ETHER_OK;
}

// Runs f(k) for k in [0, n) on up to host_threads() threads (f must not throw).  The
// workers make the caller's device current first: a new thread starts on device 0, and f
// issues copies on streams of the caller's device.
template <class F>
void parallel_for(int n, F f) {
    const int T = std::min(n, host_threads());
    if (T <= 1) {
        for (int k = 0; k < n; ++k) f(k);
        return;
    }
    int dev = 0;
    cudaGetDevice(&dev);
    std::atomic<int> next{0};
    std::vector<std::thread> pool;
    pool.reserve(T);
    for (int t = 0; t < T; ++t)
        pool.emplace_back([&]() {
            cudaSetDevice(dev);
            for (int k = next.fetch_add(1); k < n; k = next.fetch_add(1)) f(k);
        });
    for (auto &th : pool) th.join();
}

void ion_to_device_layout(const Ctx &c, const double *ion, void *dst) {
    const int N = c.N;
    if (c.model == ETHER_MODEL_ISING) {
        uint8_t *v = static_cast<uint8_t *>(dst);
        for (int i = 0; i < N; ++i) v[c.storage[i]] = ion[3 + 9 * (size_t)i] > 0.0 ? 1 : 0;
    } else {
        float4 *v = static_cast<float4 *>(dst);
        for (int i = 0; i < N; ++i) {
            const double *p = ion + 9 * (size_t)i;
            v[c.storage[i]] = make_float4((float)p[1], (float)p[2], (float)p[3], (float)p[5]);
        }
    }
}

void device_layout_to_ion(const Ctx &c, const void *src, double *ion) {
    const int N = c.N;
    if (c.model == ETHER_MODEL_ISING) {
        const uint8_t *v = static_cast<const uint8_t *>(src);
        for (int i = 0; i < N; ++i) ion[3 + 9 * (size_t)i] = v[c.storage[i]] ? 1.0 : -1.0;
    } else {
        const float4 *v = static_cast<const float4 *>(src);
        for (int i = 0; i < N; ++i) {
            double *p = ion + 9 * (size_t)i;
            const float4 q = v[c.storage[i]];
            p[1] = q.x; p[2] = q.y; p[3] = q.z; p[5] = q.w;
        }
    }
}
}  // namespace

static int spins_staged(Ctx &c, int32_t r0, int32_t n, double *ion, bool to_device, double *host_s = nullptr);

// Whether [p, p + bytes) is host memory mapped in this process, checked before a kernel reads
// or writes it in place (a wrong pointer must not reach the device): device memory is refused
// by the CUDA runtime's attributes, an unmapped page by msync (ENOMEM), which with MS_ASYNC
// only checks the mappings.
static bool host_range_mapped(const void *p, size_t bytes) {
    cudaPointerAttributes pa{};
    if (cudaPointerGetAttributes(&pa, p) != cudaSuccess) {
        cudaGetLastError();  // an unknown pointer is not a lasting error
    } else if (pa.type == cudaMemoryTypeDevice) {
        return false;
    }
    const uintptr_t page = (uintptr_t)sysconf(_SC_PAGESIZE);
    const uintptr_t a = (uintptr_t)p & ~(page - 1), b = (uintptr_t)p + bytes;
    return msync(reinterpret_cast<void *>(a), (size_t)(b - a), MS_ASYNC) == 0;
}

// A transfer of n replicas shared between the in-place kernel and the host's cores as it runs:
// this thread hands chunks of about n/32 replicas from the front to the kernel, keeping two in
// flight on c.stream (so a chunk is claimed only when the device is about to need it), while
// the host's other threads take chunks of an eighth of that from the back through the staging
// area (an upload: convert, then copy on c.ion_copy; a read-back: copy on c.ion_copy, wait for
// it, convert).  The two ends meet where the two rates put them in this call, whatever the
// link does.  kernel_reps: replicas the kernel moved.
static int spins_shared(Ctx &c, int32_t r0, int32_t n, double *ion, bool to_device, int *kernel_reps) {
    const size_t per_rep = c.model == ETHER_MODEL_ISING ? (size_t)c.N : sizeof(float4) * c.N;
    const size_t ion_rep = (size_t)9 * c.N;
    uint8_t *dev = c.model == ETHER_MODEL_ISING ? c.spins : reinterpret_cast<uint8_t *>(c.spins4);
    const char *who = to_device ? "ether_set_spins_batch: " : "ether_get_spins_batch: ";
    // claims in replicas: the kernel takes kc at a time from the front (about 1/32 of the call,
    // a few milliseconds of device work), a host thread hc from the back (about a millisecond
    // of a core's work), so the meeting point follows the two rates closely
    const int kc = std::max(1, (n + 31) / 32);
    const int hc = std::max(1, kc / 8);
    {
        const int rc = ensure_stage(c, per_rep * (size_t)n);
        if (rc) return rc;
    }
    if (!c.ion_copy) CUDA_TRY(cudaStreamCreateWithFlags(&c.ion_copy, cudaStreamNonBlocking));
    for (int k = 0; k < 2; ++k)  // timing events: the rate-based path times its kernel with them
        if (!c.ion_ev[k]) CUDA_TRY(cudaEventCreate(&c.ion_ev[k]));
    // the copies start after the work already on the context's stream (sweeps still reading or
    // writing the spins), as the kernel's chunks do
    CUDA_TRY(cudaEventRecord(c.ion_ev[0], c.stream));
    CUDA_TRY(cudaStreamWaitEvent(c.ion_copy, c.ion_ev[0], 0));
    uint8_t *stage = static_cast<uint8_t *>(c.stage);
    std::mutex mu;
    int front = 0, back = n;  // replicas [0, front) to the kernel, [back, n) to the host
    std::atomic<int> err{0};
    int dev_id = 0;
    cudaGetDevice(&dev_id);
    const int T = std::max(1, std::min((n + hc - 1) / hc, host_threads() - 1));
    std::vector<std::thread> pool;
    pool.reserve(T);
    for (int t = 0; t < T; ++t)
        pool.emplace_back([&]() {
            cudaSetDevice(dev_id);
            cudaEvent_t done = nullptr;  // a read-back waits for its own copy only
            if (!to_device && cudaEventCreateWithFlags(&done, cudaEventDisableTiming) != cudaSuccess) {
                err.store((int)cudaErrorMemoryAllocation);
                return;
            }
            for (;;) {
                int a, m;
                {
                    std::lock_guard<std::mutex> g(mu);
                    if (front >= back || err.load()) break;
                    m = std::min(hc, back - front);
                    back -= m;
                    a = back;
                }
                uint8_t *sd = dev + per_rep * (size_t)(r0 + a);
                uint8_t *ss = stage + per_rep * a;
                if (to_device) {
                    for (int r = a; r < a + m; ++r)
                        ion_to_device_layout(c, ion + ion_rep * (size_t)r, stage + per_rep * r);
                    const cudaError_t e = cudaMemcpyAsync(sd, ss, per_rep * m, cudaMemcpyHostToDevice, c.ion_copy);
                    if (e != cudaSuccess) err.store((int)e);
                } else {
                    cudaError_t e = cudaMemcpyAsync(ss, sd, per_rep * m, cudaMemcpyDeviceToHost, c.ion_copy);
                    if (e == cudaSuccess) e = cudaEventRecord(done, c.ion_copy);
                    if (e == cudaSuccess) e = cudaEventSynchronize(done);
                    if (e != cudaSuccess) {
                        err.store((int)e);
                        break;
                    }
                    for (int r = a; r < a + m; ++r)
                        device_layout_to_ion(c, stage + per_rep * r, ion + ion_rep * (size_t)r);
                }
            }
            if (done) cudaEventDestroy(done);
        });
    cudaError_t e = cudaSuccess;
    int launched = 0;
    for (;;) {
        int a, m;
        {
            std::lock_guard<std::mutex> g(mu);
            if (front >= back || err.load()) break;
            a = front;
            m = std::min(kc, back - front);
            front += m;
        }
        e = launch_ion_copy(c, r0 + a, m, ion + ion_rep * (size_t)a, to_device);
        if (e == cudaSuccess) e = cudaEventRecord(c.ion_ev[launched & 1], c.stream);
        if (e != cudaSuccess) {
            err.store((int)e);
            break;
        }
        ++launched;
        // two chunks in flight: wait for the one before the last
        if (launched >= 2) e = cudaEventSynchronize(c.ion_ev[launched & 1]);
        if (e != cudaSuccess) {
            err.store((int)e);
            break;
        }
        // a link far slower than the cores: its traffic only competes with theirs for the
        // host's memory, so after a few chunks the kernel is given no more once the cores have
        // claimed more than twice what it has finished (at most two chunks still in flight)
        if (launched >= 4) {
            std::lock_guard<std::mutex> g(mu);
            if (n - back > 2 * (front - 2 * kc)) break;
        }
    }
    for (auto &th : pool) th.join();
    // the kernel's chunks and the copies both end before the call returns (the records and the
    // staging area are the caller's and this context's again)
    cudaError_t e2 = cudaStreamSynchronize(c.stream);
    const cudaError_t e3 = cudaStreamSynchronize(c.ion_copy);
    if (e2 == cudaSuccess) e2 = e3;
    if (e2 == cudaSuccess && err.load()) e2 = (cudaError_t)err.load();
    if (e2 != cudaSuccess) {
        cudaGetLastError();
        return fail(ETHER_ERR_CUDA, std::string(who) + cudaGetErrorString(e2));
    }
    *kernel_reps = front;
    return ETHER_OK;
}

// Where the device reads and writes host memory in place (c.ion_direct) a kernel can move the
// records, and the host's cores can convert them through the staging area at the same time;
// which does how much is measured per context and direction, because the in-place path's
// speed depends on the host: on most Grace machines it is the faster (64^3 x 1024 Ising records:
// upload 77 ms by the kernel alone, 83-86 by the cores alone, 53-61 split 5/8; read-back 100
// against 148 ms), on some it was several times slower (0.23 s and 0.72 s in one process).
// Both directions are shared as they run (spins_shared) when the staging area holds the whole
// call; the kernel's rate on one box changed between calls by up to 4x, so only a division made
// during the call itself holds.  (On a good box a shared read-back costs a little against the
// kernel alone, 100 ms: each 8-byte write is a read-modify-write of a line in host memory and
// the two sides compete for it.)  A call too large for the staging area is divided by rates
// measured in earlier calls:
// * Upload: the kernel reads the first share of the replicas while the host's cores convert
//   the rest, the staged copies following the kernel on the stream: 5/8 : 3/8 the first time
//   (8 or more replicas and host threads; 1/2 and 3/4 measured 67 and 59 ms), later in
//   proportion to the two rates measured side by side in the previous upload.
// * Read-back: not split.  The first three calls run the kernel, the host's cores and the
//   kernel again, later calls the way with the better of its measured rates.
// Rates come from CUDA events around the kernel and the wall time of the host's conversion.
static int spins_batch(Ctx &c, int32_t r0, int32_t n, double *ion, bool to_device) {
    if (!c.ion_direct) return spins_staged(c, r0, n, ion, to_device);
    if (!host_range_mapped(ion, sizeof(double) * 9 * (size_t)c.N * n))
        return fail(ETHER_ERR_ARG, std::string(to_device ? "ether_set_spins_batch" : "ether_get_spins_batch") +
                                       ": ion is not host memory mapped for n replicas' records");
    const size_t per_rep = c.model == ETHER_MODEL_ISING ? (size_t)c.N : sizeof(float4) * c.N;
    if (n >= 2 && host_threads() >= 2 && per_rep * (size_t)n <= kStageMax) {
        int nk = 0;
        const int rc = spins_shared(c, r0, n, ion, to_device, &nk);
        if (rc == ETHER_OK) c.ion_last_kernel[to_device ? 1 : 0] = nk;
        return rc;
    }
    const int d = to_device ? 1 : 0;
    const double rk = c.ion_rate_k[d], rh = c.ion_rate_h[d];
    int nk;
    if (to_device) {
        if (rk > 0.0 && rh > 0.0)
            nk = (int)std::lround((double)n * rk / (rk + rh));
        else
            nk = n >= 8 && host_threads() >= 8 ? n - n * 3 / 8 : n;
    } else {
        const int k = c.ion_gets++;
        nk = k == 0 || k == 2 ? n : k == 1 ? 0 : (rk >= rh ? n : 0);
    }
    nk = std::max(0, std::min(n, nk));
    const char *who = to_device ? "ether_set_spins_batch: " : "ether_get_spins_batch: ";
    cudaError_t e = cudaSuccess;
    if (nk > 0) {
        for (int k = 0; k < 2 && e == cudaSuccess; ++k)
            if (!c.ion_ev[k]) e = cudaEventCreate(&c.ion_ev[k]);
        if (e == cudaSuccess) e = cudaEventRecord(c.ion_ev[0], c.stream);
        if (e == cudaSuccess) e = launch_ion_copy(c, r0, nk, ion, to_device);
        if (e == cudaSuccess) e = cudaEventRecord(c.ion_ev[1], c.stream);
        if (e == cudaSuccess && nk == n) e = cudaStreamSynchronize(c.stream);
        if (e != cudaSuccess) {
            cudaGetLastError();
            cudaStreamSynchronize(c.stream);  // launches before a failed one may still be reading ion
            return fail(ETHER_ERR_CUDA, std::string(who) + cudaGetErrorString(e));
        }
    }
    double host_s = 0.0;
    if (nk < n) {
        // the staged part synchronises the stream (kernel included) before it returns; on an
        // early failure the kernel may still be reading the caller's records, so wait for it
        const int rc = spins_staged(c, r0 + nk, n - nk, ion + (size_t)9 * c.N * nk, to_device, &host_s);
        if (rc != ETHER_OK) {
            cudaStreamSynchronize(c.stream);
            return rc;
        }
        if (host_s > 0.0) {
            // an upload's rates are those of the last split; a read-back keeps the best seen
            const double r = (double)(n - nk) / host_s;
            c.ion_rate_h[d] = to_device ? r : std::max(c.ion_rate_h[d], r);
        }
    }
    if (nk > 0) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, c.ion_ev[0], c.ion_ev[1]) == cudaSuccess && ms > 0.f) {
            const double r = (double)nk / (1e-3 * ms);
            c.ion_rate_k[d] = to_device ? r : std::max(c.ion_rate_k[d], r);
        } else {
            cudaGetLastError();
        }
    }
    c.ion_last_kernel[d] = nk;
    return ETHER_OK;
}

// host_s (may be null) accumulates the wall time of the host's conversion loops.
static int spins_staged(Ctx &c, int32_t r0, int32_t n, double *ion, bool to_device, double *host_s) {
    const size_t per_rep = c.model == ETHER_MODEL_ISING ? (size_t)c.N : sizeof(float4) * c.N;
    const size_t ion_rep = (size_t)9 * c.N;
    uint8_t *dev = c.model == ETHER_MODEL_ISING ? c.spins : reinterpret_cast<uint8_t *>(c.spins4);
    const int per_chunk = (int)std::max<size_t>(1, kChunkBytes / per_rep);
    const int per_pass = (int)std::max<size_t>((size_t)per_chunk, kStageMax / per_rep / per_chunk * per_chunk);
    {
        const int rc = ensure_stage(c, per_rep * (size_t)std::min(n, per_pass));
        if (rc) return rc;
    }
    uint8_t *stage = static_cast<uint8_t *>(c.stage);
    for (int p0 = 0; p0 < n; p0 += per_pass) {
        const int np = std::min(per_pass, n - p0);
        const int nchunk = (np + per_chunk - 1) / per_chunk;
        std::vector<cudaEvent_t> ev(nchunk, nullptr);
        std::atomic<int> cuda_err{0};
        if (!to_device) {
            // device -> staging, one event per chunk; the host converts each as it lands
            for (int k = 0; k < nchunk; ++k) {
                const int a = k * per_chunk, b = std::min(np, a + per_chunk);
                cudaError_t e = cudaMemcpyAsync(stage + per_rep * a, dev + per_rep * (size_t)(r0 + p0 + a),
                                                per_rep * (b - a), cudaMemcpyDeviceToHost, c.stream);
                if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev[k], cudaEventDisableTiming);
                if (e == cudaSuccess) e = cudaEventRecord(ev[k], c.stream);
                if (e != cudaSuccess) {
                    for (cudaEvent_t x : ev)
                        if (x) cudaEventDestroy(x);
                    return fail(ETHER_ERR_CUDA, std::string("ether_get_spins_batch: ") + cudaGetErrorString(e));
                }
            }
        }
        const auto t0 = std::chrono::steady_clock::now();
        parallel_for(nchunk, [&](int k) {
            const int a = k * per_chunk, b = std::min(np, a + per_chunk);
            if (to_device) {
                for (int r = a; r < b; ++r)
                    ion_to_device_layout(c, ion + ion_rep * (size_t)(p0 + r), stage + per_rep * r);
                const cudaError_t e = cudaMemcpyAsync(dev + per_rep * (size_t)(r0 + p0 + a), stage + per_rep * a,
                                                      per_rep * (b - a), cudaMemcpyHostToDevice, c.stream);
                if (e != cudaSuccess) cuda_err.store((int)e);
            } else {
                const cudaError_t e = cudaEventSynchronize(ev[k]);
                if (e != cudaSuccess) {
                    cuda_err.store((int)e);
                    return;
                }
                for (int r = a; r < b; ++r)
                    device_layout_to_ion(c, stage + per_rep * r, ion + ion_rep * (size_t)(p0 + r));
            }
        });
        if (host_s) host_s[0] += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        for (cudaEvent_t x : ev)
            if (x) cudaEventDestroy(x);
        // the staging area is reused by the next pass (and the next call)
        cudaError_t e = cudaStreamSynchronize(c.stream);
        if (e == cudaSuccess && cuda_err.load()) e = (cudaError_t)cuda_err.load();
        if (e != cudaSuccess)
            return fail(ETHER_ERR_CUDA, std::string(to_device ? "ether_set_spins_batch: " : "ether_get_spins_batch: ") +
                                            cudaGetErrorString(e));
    }
    return ETHER_OK;
}

extern "C" int ether_spins_batch_split(ether_ctx *h, int32_t *get_kernel, int32_t *set_kernel) {
    if (!h || !get_kernel || !set_kernel) return fail(ETHER_ERR_ARG, "null argument");
    Ctx &c = h->c;
    *get_kernel = c.ion_last_kernel[0];
    *set_kernel = c.ion_last_kernel[1];
    return ETHER_OK;
}

extern "C" int ether_set_spins_batch(ether_ctx *h, int32_t r0, int32_t n, const double *ion) {
    if (!h || !ion) return fail(ETHER_ERR_ARG, "null argument");
    Ctx &c = h->c;
    if (r0 < 0 || n <= 0 || (long)r0 + n > c.R) return fail(ETHER_ERR_ARG, "replica range out of bounds");
    return spins_batch(c, r0, n, const_cast<double *>(ion), true);
}

extern "C" int ether_get_spins_batch(ether_ctx *h, int32_t r0, int32_t n, double *ion) {
    if (!h || !ion) return fail(ETHER_ERR_ARG, "null argument");
    Ctx &c = h->c;
    if (r0 < 0 || n <= 0 || (long)r0 + n > c.R) return fail(ETHER_ERR_ARG, "replica range out of bounds");
    return spins_batch(c, r0, n, ion, false);
}

extern "C" int ether_fresh_spins(ether_ctx *h) {
    if (!h) return fail(ETHER_ERR_ARG, "null context");
    Ctx &c = h->c;
    CUDA_TRY(launch_fresh(c));
    CUDA_TRY(launch_advance(c, c.fresh_call));
    return ETHER_OK;
}

static int sweep_once(Ctx &c) {
    for (int col = 0; col < c.ncol; ++col) {
        if (c.model == ETHER_MODEL_ISING) CUDA_TRY(launch_ising_sweep(c, col));
        else CUDA_TRY(launch_xyz_sweep(c, col));
    }
    CUDA_TRY(launch_advance(c, c.step));
    return ETHER_OK;
}

int ether::plain_sweep(Ctx &c) { return sweep_once(c); }

// How many replica parts ether_mcs splits this context's sweeps into (general lattices:
// their colour phases are small, dependent, latency-bound launches): 1 (no split), 2 or 4.
static int sweep_parts(const Ctx &c) {
    if (c.fast || c.resident) return 1;
    return c.R >= 32 ? 4 : c.R >= 16 ? 2 : 1;
}

// m sweeps of every replica as replica parts side by side, on c.stream and the aux streams
// (each part its own chain of colour phases, joined at the end): replicas are independent,
// so this is the same work and the same results.
static int sweeps_in_parts(Ctx &c, int m) {
    const int P = c.n_parts;
    CUDA_TRY(cudaEventRecord(c.ev_fork, c.stream));
    for (int p = 1; p < P; ++p) CUDA_TRY(cudaStreamWaitEvent(c.aux[p - 1], c.ev_fork, 0));
    const cudaStream_t own = c.stream;
    int rc = ETHER_OK;
    for (int p = 0; p < P && !rc; ++p) {
        c.stream = p ? c.aux[p - 1] : own;
        c.rw0 = (int)((long)c.R * p / P);
        c.rwn = (int)((long)c.R * (p + 1) / P) - c.rw0;
        for (int k = 0; k < m && !rc; ++k) rc = sweep_once(c);
    }
    c.stream = own;
    c.rw0 = c.rwn = 0;
    if (rc) return rc;
    for (int p = 1; p < P; ++p) {
        CUDA_TRY(cudaEventRecord(c.ev_join[p - 1], c.aux[p - 1]));
        CUDA_TRY(cudaStreamWaitEvent(c.stream, c.ev_join[p - 1], 0));
    }
    return ETHER_OK;
}

// The streams of the replica parts, made once per context (outside any capture).
static int ensure_parts(Ctx &c) {
    if (c.n_parts) return ETHER_OK;
    const int P = sweep_parts(c);
    if (P > 1) CUDA_TRY(cudaEventCreateWithFlags(&c.ev_fork, cudaEventDisableTiming));
    for (int p = 1; p < P; ++p) {
        CUDA_TRY(cudaStreamCreateWithFlags(&c.aux[p - 1], cudaStreamNonBlocking));
        CUDA_TRY(cudaEventCreateWithFlags(&c.ev_join[p - 1], cudaEventDisableTiming));
    }
    c.n_parts = P;
    return ETHER_OK;
}


static int variant_of(const Ctx &c);

extern "C" int ether_metropolis(ether_ctx *h, int32_t nsweeps, double *accept) {
    if (!h) return fail(ETHER_ERR_ARG, "null context");
    Ctx &c = h->c;
    if (nsweeps < 0) return fail(ETHER_ERR_ARG, "negative sweep count");
    if (!c.beta_set) return fail(ETHER_ERR_STATE, "beta not set (ether_set_beta / ether_set_ladder)");
    if (accept && nsweeps == 1 && !(c.flags & ETHER_FLAG_NO_GRAPHS)) {
        // the reference's per-MCS call (Metropolis, then its acceptance): snapshot, sweep,
        // ratios and the copy to pinned memory captured once per kernel variant and replayed
        const std::string key = "metropolis1/" + std::to_string(variant_of(c));
        auto it = c.graphs.find(key);
        if (it == c.graphs.end()) {
            cudaGraph_t g = nullptr;
            CUDA_TRY(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal));
            cudaError_t ce = cudaMemcpyAsync(c.acc_before, c.acc_count, sizeof(unsigned long long) * c.R,
                                             cudaMemcpyDeviceToDevice, c.stream);
            int rc = ce == cudaSuccess ? sweep_once(c) : ETHER_ERR_CUDA;
            if (rc == ETHER_OK) ce = launch_accept_ratio(c, c.acc_ratio);
            if (rc == ETHER_OK && ce == cudaSuccess)
                ce = cudaMemcpyAsync(c.acc_host, c.acc_ratio, sizeof(double) * c.R, cudaMemcpyDeviceToHost, c.stream);
            const cudaError_t ee = cudaStreamEndCapture(c.stream, &g);
            if (rc != ETHER_OK || ce != cudaSuccess || ee != cudaSuccess) {
                if (g) cudaGraphDestroy(g);
                if (rc != ETHER_OK) return rc;
                CUDA_TRY(ce != cudaSuccess ? ce : ee);
            }
            cudaGraphExec_t ex = nullptr;
            ce = cudaGraphInstantiate(&ex, g, 0);
            cudaGraphDestroy(g);
            CUDA_TRY(ce);
            it = c.graphs.emplace(key, ex).first;
        }
        CUDA_TRY(cudaGraphLaunch(it->second, c.stream));
        CUDA_TRY(cudaStreamSynchronize(c.stream));
        std::memcpy(accept, c.acc_host, sizeof(double) * c.R);
        return ETHER_OK;
    }
    // acceptance: a device snapshot of the counters, one kernel for the ratios and one copy
    // into pinned memory, so a call that returns them costs a single small D2H and one sync
    if (accept)
        CUDA_TRY(cudaMemcpyAsync(c.acc_before, c.acc_count, sizeof(unsigned long long) * c.R,
                                 cudaMemcpyDeviceToDevice, c.stream));
    if (nsweeps > 1) {
        const int rc = ensure_parts(c);
        if (rc) return rc;
    }
    if (nsweeps > 1 && c.n_parts > 1) {  // general lattices: replica parts side by side, same bits
        const int rc = sweeps_in_parts(c, nsweeps);
        if (rc) return rc;
    } else {
        for (int k = 0; k < nsweeps; ++k) {
            int rc = sweep_once(c);
            if (rc) return rc;
        }
    }
    if (accept) {
        CUDA_TRY(launch_accept_ratio(c, c.acc_ratio));
        CUDA_TRY(cudaMemcpyAsync(c.acc_host, c.acc_ratio, sizeof(double) * c.R, cudaMemcpyDeviceToHost, c.stream));
        CUDA_TRY(cudaStreamSynchronize(c.stream));
        std::memcpy(accept, c.acc_host, sizeof(double) * c.R);
    }
    return ETHER_OK;
}

static int overrelax_once(Ctx &c, double para) {
    const int full = (int)std::floor(para);
    const float part = (float)(para - full);
    const int npass = full + (part > 0.0f ? 1 : 0);
    for (int p = 0; p < npass; ++p)
        for (int col = 0; col < c.ncol; ++col) CUDA_TRY(launch_overrelax(c, col, p, p < full ? 1.0f : part));
    CUDA_TRY(launch_advance(c, c.ovrr_step));
    return ETHER_OK;
}

extern "C" int ether_overrelaxation(ether_ctx *h, double ovrr_para) {
    if (!h) return fail(ETHER_ERR_ARG, "null context");
    Ctx &c = h->c;
    if (c.model != ETHER_MODEL_XYZ) return fail(ETHER_ERR_ARG, "overrelaxation needs the XYZ model");
    if (!(ovrr_para >= 0.0) || ovrr_para > 1000.0) return fail(ETHER_ERR_ARG, "ovrr_para out of range");
    return overrelax_once(c, ovrr_para);
}

extern "C" int ether_tot_energy(ether_ctx *h, double *E) {
    if (!h) return fail(ETHER_ERR_ARG, "null context");
    Ctx &c = h->c;
    CUDA_TRY(launch_energy_mag(c, true));
    if (E) {
        CUDA_TRY(cudaMemcpyAsync(E, c.E, sizeof(double) * c.R, cudaMemcpyDeviceToHost, c.stream));
        CUDA_TRY(cudaStreamSynchronize(c.stream));
    }
    return ETHER_OK;
}

extern "C" int ether_tot_magnetisation(ether_ctx *h, double *M) {
    if (!h) return fail(ETHER_ERR_ARG, "null context");
    Ctx &c = h->c;
    CUDA_TRY(launch_energy_mag(c, false));
    if (M) {
        CUDA_TRY(cudaMemcpyAsync(M, c.M, sizeof(double) * 3 * c.R, cudaMemcpyDeviceToHost, c.stream));
        CUDA_TRY(cudaStreamSynchronize(c.stream));
    }
    return ETHER_OK;
}

extern "C" int ether_observable(ether_ctx *h, int32_t step, int32_t tmcs_eq, int32_t coa) {
    if (!h) return fail(ETHER_ERR_ARG, "null context");
    if (coa <= 0) return fail(ETHER_ERR_ARG, "coa must be positive");
    Ctx &c = h->c;
    if (step > tmcs_eq && step % coa == 0) {
        CUDA_TRY(launch_energy_mag(c, true));
        CUDA_TRY(launch_measure(c));
    }
    return ETHER_OK;
}

extern "C" int ether_zero_avg(ether_ctx *h) {
    if (!h) return fail(ETHER_ERR_ARG, "null context");
    Ctx &c = h->c;
    CUDA_TRY(cudaMemsetAsync(c.sums, 0, sizeof(double) * 7 * c.R, c.stream));
    if (c.spiral_sums) CUDA_TRY(cudaMemsetAsync(c.spiral_sums, 0, sizeof(double) * 4 * c.R, c.stream));
    return ETHER_OK;
}

extern "C" int ether_get_sums(ether_ctx *h, double *sums) {
    if (!h || !sums) return fail(ETHER_ERR_ARG, "null argument");
    Ctx &c = h->c;
    CUDA_TRY(cudaMemcpyAsync(sums, c.sums, sizeof(double) * 7 * c.R, cudaMemcpyDeviceToHost, c.stream));
    CUDA_TRY(cudaStreamSynchronize(c.stream));
    return ETHER_OK;
}

// get_eng('avg_eng') (src/get_eng.f90:42-60) and get_mag('avg_mag') (src/get_mag.f90:43-59).
extern "C" int ether_avg(ether_ctx *h, double *out) {
    if (!h || !out) return fail(ETHER_ERR_ARG, "null argument");
    Ctx &c = h->c;
    std::vector<double> s(7 * (size_t)c.R);
    int rc = ether_get_sums(h, s.data());
    if (rc) return rc;
    for (int g = 0; g < c.n_groups; ++g)
        for (int sl = 0; sl < c.n_slots; ++sl) {
            const size_t idx = (size_t)g * c.n_slots + sl;
            const double *a = s.data() + 7 * idx;
            const double beta = c.beta_slots[sl];
            const double n = a[0];
            const double e = a[1] / n, e2 = a[2] / n, e4 = a[3] / n;
            const double m = a[4] / n, m2 = a[5] / n, m4 = a[6] / n;
            double *o = out + 6 * idx;
            o[0] = e;
            o[1] = 1.0 - (1.0 / 3.0) * (e4 / (e2 * e2));
            o[2] = (beta * beta) * (e2 - e * e) * c.N;
            o[3] = m;
            o[4] = 1.0 - (1.0 / 3.0) * (m4 / (m2 * m2));
            o[5] = beta * (m2 - m * m) * c.N;
        }
    return ETHER_OK;
}

// observables_per_repeat (src/observables_per_repeat.f90:29-69) across the REPEAT groups.
extern "C" int ether_per_repeat(ether_ctx *h, double *mean, double *err) {
    if (!h || !mean || !err) return fail(ETHER_ERR_ARG, "null argument");
    Ctx &c = h->c;
    std::vector<double> v(6 * (size_t)c.R);
    int rc = ether_avg(h, v.data());
    if (rc) return rc;
    const double rep = c.n_groups;
    const double r1 = 1.0 / (rep * (rep - 1.0));  // +inf for one group: errors NaN, as the reference
    for (int sl = 0; sl < c.n_slots; ++sl)
        for (int q = 0; q < 6; ++q) {
            double sum = 0.0;
            for (int g = 0; g < c.n_groups; ++g) sum += v[6 * ((size_t)g * c.n_slots + sl) + q];
            const double mu = sum / rep;
            double e = 0.0;
            for (int g = 0; g < c.n_groups; ++g) {
                const double d = v[6 * ((size_t)g * c.n_slots + sl) + q] - mu;
                e += d * d;
            }
            mean[6 * sl + q] = mu;
            err[6 * sl + q] = std::sqrt(r1 * e);
        }
    return ETHER_OK;
}

extern "C" int ether_parallel_tempering(ether_ctx *h, int32_t swap_count, int32_t *accepted) {
    if (!h) return fail(ETHER_ERR_ARG, "null context");
    Ctx &c = h->c;
    if (!c.beta_set) return fail(ETHER_ERR_STATE, "beta not set");
    if (swap_count < 0) return fail(ETHER_ERR_ARG, "negative swap_count");
    CUDA_TRY(launch_energy_mag(c, true));
    CUDA_TRY(launch_pt(c, swap_count));
    if (accepted) {
        CUDA_TRY(cudaMemcpyAsync(accepted, c.pt_accepts, sizeof(int32_t), cudaMemcpyDeviceToHost, c.stream));
        CUDA_TRY(cudaStreamSynchronize(c.stream));
    }
    return ETHER_OK;
}

extern "C" int ether_get_slots(ether_ctx *h, int32_t *slot_of_replica) {
    if (!h || !slot_of_replica) return fail(ETHER_ERR_ARG, "null argument");
    Ctx &c = h->c;
    CUDA_TRY(cudaMemcpyAsync(slot_of_replica, c.slot_of_rep, sizeof(int32_t) * c.R, cudaMemcpyDeviceToHost, c.stream));
    CUDA_TRY(cudaStreamSynchronize(c.stream));
    return ETHER_OK;
}

namespace ether {

// Whether src/ether.f90:163-169 overrelaxes this context at all: XYZ spins with neither a
// field nor anisotropy (overrelaxation conserves the exchange energy only).
bool mcs_ovrr_on(const Ctx &c, const ether_schedule *sch) {
    return sch->ovrr && c.model == ETHER_MODEL_XYZ && !c.zeeman && !c.sia && !c.sia_local && sch->ovrr_mcs > 0;
}

int mcs_check(const Ctx &c, const ether_schedule *sch) {
    if (!c.beta_set) return fail(ETHER_ERR_STATE, "beta not set");
    const bool pt_on = sch->pt && sch->exchange_interval > 0;
    if (pt_on && !(c.flags & ETHER_FLAG_PT_REFERENCE_COPY) && c.n_slots < 2)
        return fail(ETHER_ERR_STATE, "PT needs a ladder of at least two slots");
    return ETHER_OK;
}

// The gates of MCS step `step`: bit 0 overrelaxation (:163-169), bit 1 total energy + PT
// (:177, :189-198), bit 2 observable (:201).
int mcs_gates(const Ctx &c, const ether_schedule *sch, int step) {
    const bool ov = mcs_ovrr_on(c, sch) && step % sch->ovrr_mcs == 0 && step % sch->coa != 0;
    const bool pt = sch->pt && sch->exchange_interval > 0 && step % sch->exchange_interval == 0 &&
                    step % sch->coa != 0;
    const bool me = step > sch->tmcs_eq && step % sch->coa == 0;
    return (ov ? 1 : 0) | (pt ? 2 : 0) | (me ? 4 : 0);
}

// The parts of one MCS before and after the Metropolis sweep, on the context's stream.
int mcs_before_sweep(Ctx &c, const ether_schedule *sch, int gates) {
    if (gates & 1) return overrelax_once(c, sch->ovrr_para);
    return ETHER_OK;
}

int mcs_after_sweep(Ctx &c, int gates) {
    if (gates & 2) {
        CUDA_TRY(launch_energy_mag(c, true));
        CUDA_TRY(launch_pt(c, -1));  // the swap counter lives on the device
    }
    if (gates & 4) {
        CUDA_TRY(launch_energy_mag(c, true));
        CUDA_TRY(launch_measure(c));
        if (c.spiral_ptr) CUDA_TRY(launch_spiral_measure(c));  // src/observable.f90:41
    }
    return ETHER_OK;
}

// The period of the gates in steps.
long mcs_period(const ether_schedule *sch, bool ovrr_on, bool pt_on) {
    auto lcm = [](long x, long y) { long g = x, b = y; while (b) { long t = g % b; g = b; b = t; } return x / g * y; };
    long period = sch->coa;
    if (ovrr_on) period = lcm(period, sch->ovrr_mcs);
    if (pt_on) period = lcm(period, sch->exchange_interval);
    return period;
}

// Steps per captured chunk: the period of the gates, kept between 1 and 256 steps (at least 8
// where doubling allows).
int mcs_chunk(long period) {
    int chunk = (int)(period <= 256 ? period : 64);
    while (chunk < 8 && chunk * 2 <= 256) chunk *= 2;
    return chunk;
}

}  // namespace ether

// One MCS of src/ether.f90:163-201 given its gates: OVRR (:163-169), Metropolis (:172),
// total energy + PT when PT runs (:177, :189-198), observable on measurement steps (:201).
static int issue_step(Ctx &c, const ether_schedule *sch, int gates) {
    int rc = mcs_before_sweep(c, sch, gates);
    if (rc) return rc;
    rc = sweep_once(c);
    if (rc) return rc;
    return mcs_after_sweep(c, gates);
}

static int variant_of(const Ctx &c);

// Steps sig[0 .. n): with a resident context the sweeps that no OVRR, PT or measurement
// separates run as one ising_sc_resident launch; otherwise step by step.
static int issue_steps(Ctx &c, const ether_schedule *sch, const int8_t *sig, int n) {
    if (c.n_parts > 1) {
        // runs of sweeps that no OVRR, PT or measurement separates, in replica parts
        for (int k = 0; k < n;) {
            int rc = mcs_before_sweep(c, sch, sig[k]);
            if (rc) return rc;
            int j = k + 1;
            while (j < n && !(sig[j - 1] & 6) && !(sig[j] & 1)) ++j;
            rc = sweeps_in_parts(c, j - k);
            if (rc) return rc;
            rc = mcs_after_sweep(c, sig[j - 1]);
            if (rc) return rc;
            k = j;
        }
        return ETHER_OK;
    }
    if (!c.resident) {
        for (int k = 0; k < n; ++k) {
            int rc = issue_step(c, sch, sig[k]);
            if (rc) return rc;
        }
        return ETHER_OK;
    }
    int pending = 0;
    for (int k = 0; k < n; ++k) {
        if (sig[k] & 1) {  // not reached for Ising (no OVRR), kept for the order of operations
            if (pending) CUDA_TRY(launch_ising_resident(c, pending));
            pending = 0;
            int rc = overrelax_once(c, sch->ovrr_para);
            if (rc) return rc;
        }
        ++pending;
        if (sig[k] & 6) {
            CUDA_TRY(launch_ising_resident(c, pending));
            pending = 0;
            if (sig[k] & 2) {
                CUDA_TRY(launch_energy_mag(c, true));
                CUDA_TRY(launch_pt(c, -1));
            }
            if (sig[k] & 4) {
                CUDA_TRY(launch_energy_mag(c, true));
                CUDA_TRY(launch_measure(c));
            }
        }
    }
    if (pending) CUDA_TRY(launch_ising_resident(c, pending));
    return ETHER_OK;
}

// The loop body for steps step0+1 .. step0+nsteps.  Steps are issued in chunks; a chunk's
// launches depend only on its gate pattern (everything that changes from step to step --
// sweep counters, PT swap count, slot permutation -- is read from device memory), so each
// distinct pattern is captured once as a CUDA graph and replayed.  With periodic gates the
// chunk length is the gates' period, and one or two graphs cover a whole run.
extern "C" int ether_mcs(ether_ctx *h, const ether_schedule *sch, int32_t step0, int32_t nsteps,
                         int32_t *swap_count) {
    if (!h || !sch) return fail(ETHER_ERR_ARG, "null argument");
    Ctx &c = h->c;
    if (sch->coa <= 0 || nsteps < 0 || step0 < 0)
        return fail(ETHER_ERR_ARG, "coa must be positive, step0 and nsteps >= 0");
    {
        const int rc = mcs_check(c, sch);
        if (rc) return rc;
    }
    const bool ovrr_on = mcs_ovrr_on(c, sch);
    const bool pt_on = sch->pt && sch->exchange_interval > 0;
    const int32_t sc0 = swap_count ? *swap_count : 0;
    CUDA_TRY(cudaMemcpyAsync(c.swap_dev, &sc0, sizeof(int32_t), cudaMemcpyHostToDevice, c.stream));
    {
        const int rc = ensure_parts(c);
        if (rc) return rc;
    }
    const long period = mcs_period(sch, ovrr_on, pt_on);
    int chunk = mcs_chunk(period);
    // resident contexts: the longest multiple of the period up to 256 steps, so that the
    // eventless stretches (equilibration) run as few long resident launches
    if (c.resident && period <= 256) chunk = (int)(256 / period * period);
    const bool use_graphs = !(c.flags & ETHER_FLAG_NO_GRAPHS);
    int step = step0 + 1;
    const int last = step0 + nsteps;
    while (step <= last) {
        const int n = std::min(chunk, last - step + 1);
        std::vector<int8_t> sig;
        sig.reserve(n + 1);
        for (int k = 0; k < n; ++k) sig.push_back((int8_t)mcs_gates(c, sch, step + k));
        if (!use_graphs || n < 4) {
            int rc = issue_steps(c, sch, sig.data(), n);
            if (rc) return rc;
        } else {
            // the kernel variant and the ladder's shape are part of the key: a graph keeps the
            // kernels and launch arguments it was captured with
            std::string key(sig.begin(), sig.end());
            key += std::to_string(variant_of(c)) + "/" + std::to_string(sch->ovrr_para) + "/" +
                   std::to_string(c.n_slots) + (c.spiral_ptr ? "/s" : "");
            auto it = c.graphs.find(key);
            if (it == c.graphs.end()) {
                if (c.graphs.size() >= 64) {
                    for (auto &kv : c.graphs) cudaGraphExecDestroy(kv.second);
                    c.graphs.clear();
                }
                cudaGraph_t g = nullptr;
                CUDA_TRY(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal));
                int rc = ETHER_OK;
                rc = issue_steps(c, sch, sig.data(), n);
                cudaError_t ce = cudaStreamEndCapture(c.stream, &g);
                if (rc) {
                    if (g) cudaGraphDestroy(g);
                    return rc;
                }
                CUDA_TRY(ce);
                cudaGraphExec_t ex = nullptr;
                ce = cudaGraphInstantiate(&ex, g, 0);
                cudaGraphDestroy(g);
                CUDA_TRY(ce);
                it = c.graphs.emplace(key, ex).first;
            }
            CUDA_TRY(cudaGraphLaunch(it->second, c.stream));
        }
        step += n;
    }
    if (swap_count) {
        CUDA_TRY(cudaMemcpyAsync(swap_count, c.swap_dev, sizeof(int32_t), cudaMemcpyDeviceToHost, c.stream));
        CUDA_TRY(cudaStreamSynchronize(c.stream));
    }
    return ETHER_OK;
}

extern "C" int ether_get_accept_counts(ether_ctx *h, uint64_t *counts) {
    if (!h || !counts) return fail(ETHER_ERR_ARG, "null argument");
    Ctx &c = h->c;
    CUDA_TRY(cudaMemcpyAsync(counts, c.acc_count, sizeof(uint64_t) * c.R, cudaMemcpyDeviceToHost, c.stream));
    CUDA_TRY(cudaStreamSynchronize(c.stream));
    return ETHER_OK;
}

extern "C" int ether_reset_accept_counts(ether_ctx *h) {
    if (!h) return fail(ETHER_ERR_ARG, "null context");
    Ctx &c = h->c;
    CUDA_TRY(cudaMemsetAsync(c.acc_count, 0, sizeof(unsigned long long) * c.R, c.stream));
    CUDA_TRY(cudaMemsetAsync(c.acc_slot, 0, sizeof(unsigned long long) * c.R, c.stream));
    CUDA_TRY(cudaMemsetAsync(c.acc_mark, 0, sizeof(unsigned long long) * c.R, c.stream));
    return ETHER_OK;
}

// Accepted Metropolis moves per temperature: the count src/ether.f90:173 accumulates on the
// rank that owns a temperature, here per (group, slot) however PT moved the replicas.
extern "C" int ether_get_slot_accept_counts(ether_ctx *h, uint64_t *counts) {
    if (!h || !counts) return fail(ETHER_ERR_ARG, "null argument");
    Ctx &c = h->c;
    if (!c.beta_set) return fail(ETHER_ERR_STATE, "beta not set");
    CUDA_TRY(launch_acc_bin(c));
    CUDA_TRY(cudaMemcpyAsync(counts, c.acc_slot, sizeof(uint64_t) * c.R, cudaMemcpyDeviceToHost, c.stream));
    CUDA_TRY(cudaStreamSynchronize(c.stream));
    return ETHER_OK;
}

extern "C" int ether_get_info(ether_ctx *h, ether_info *info) {
    if (!h || !info) return fail(ETHER_ERR_ARG, "null argument");
    Ctx &c = h->c;
    info->n_colours = c.ncol;
    info->fast_path = c.fast ? 1 : 0;
    info->n_types = c.n_types;
    info->table_entries = c.table_entries;
    info->n_slots = c.n_slots;
    info->n_groups = c.n_groups;
    info->device_bytes = c.device_bytes;
    info->kernel_launches = c.launches;
    info->sq_kernel_ms = c.sq_ms;
    info->ion_direct = c.ion_direct ? 1 : 0;
    return ETHER_OK;
}

extern "C" int ether_get_colouring(ether_ctx *h, int32_t *colour, int32_t *rank_in_colour) {
    if (!h) return fail(ETHER_ERR_ARG, "null context");
    Ctx &c = h->c;
    if (colour) std::copy(c.colour.begin(), c.colour.end(), colour);
    if (rank_in_colour) std::copy(c.rank.begin(), c.rank.end(), rank_in_colour);
    return ETHER_OK;
}

extern "C" int ether_sync(ether_ctx *h) {
    if (!h) return fail(ETHER_ERR_ARG, "null context");
    CUDA_TRY(cudaStreamSynchronize(h->c.stream));
    int e = 0;
    CUDA_TRY(cudaMemcpy(&e, h->c.err, sizeof(int), cudaMemcpyDeviceToHost));
    if (e) {
        CUDA_TRY(cudaMemset(h->c.err, 0, sizeof(int)));
        return fail(ETHER_ERR_TIMEOUT, "a staged sweep kernel's bounded wait ran out (code " + std::to_string(e) + ")");
    }
    return ETHER_OK;
}

extern "C" int ether_get_stream(ether_ctx *h, void **stream) {
    if (!h || !stream) return fail(ETHER_ERR_ARG, "null argument");
    *stream = (void *)h->c.stream;
    return ETHER_OK;
}

extern "C" int ether_metropolis_phase(ether_ctx *h, int32_t colour) {
    if (!h) return fail(ETHER_ERR_ARG, "null context");
    Ctx &c = h->c;
    if (!c.beta_set) return fail(ETHER_ERR_STATE, "beta not set");
    if (colour < 0 || colour >= c.ncol) return fail(ETHER_ERR_ARG, "colour out of range");
    if (c.model == ETHER_MODEL_ISING) CUDA_TRY(launch_ising_sweep(c, colour));
    else CUDA_TRY(launch_xyz_sweep(c, colour));
    return ETHER_OK;
}

extern "C" int ether_end_sweep(ether_ctx *h) {
    if (!h) return fail(ETHER_ERR_ARG, "null context");
    CUDA_TRY(launch_advance(h->c, h->c.step));
    return ETHER_OK;
}

// ---------------------------------------------------------------- autotuner ----------
// Times every kernel variant of this context's fast path on its own data -- one colour
// phase of each, with the spins and acceptance counters restored afterwards -- and keeps
// the fastest.  Choices are cached per size class (model, extents, replicas) for the life
// of the process, so later contexts of the same shape skip the timing.
#include <mutex>
namespace {
std::mutex g_tune_mu;
std::map<std::vector<long>, int> g_tune_cache;  // variant per (model, L, R)
}  // namespace

static int variant_of(const Ctx &c) {
    if (c.model == ETHER_MODEL_XYZ) return 5000 + c.xyz_variant;
    if (c.ising_stream) return 4000 + 10 * c.ising_vpt + (c.ising_cap ? 4 : 1);
    if (c.ising_cap5) return 6000 + c.vec_bytes * 10 + c.ising_vpt;
    return (c.ising_persist ? 1000 : 0) + (c.ising_cap ? 2000 : 0) + c.vec_bytes * 10 + c.ising_vpt;
}

namespace ether {
int ctx_variant(const Ctx &c) { return variant_of(c); }
}  // namespace ether

// variant = 1000 (persistent kernel) + 2000 (register cap: four 256-thread blocks per SM)
//           + 10 * bytes per vector + vectors per thread
//           or 6162: the phase kernel capped at five blocks per SM (two 16-byte vectors
//           per thread in 48 registers)
//           or 4000 + 10 * vectors per thread and step + 1 / 4 (register cap): the
//           shared-memory staged kernel (4011, 4014, 4021, 4041)
//           or 5000 + 10 * sites per thread + register cap (blocks per SM) for the
//           simple-cubic XYZ kernel (5011 .. 5015, 5021 .. 5024, 5041, 5042; with two or
//           more sites per thread a warp draws the second Philox block of its sites together)
static bool apply_variant(Ctx &c, int variant) {
    if (c.model == ETHER_MODEL_XYZ) {
        if (!xyz_variant_valid(variant - 5000)) return false;
        c.xyz_variant = variant - 5000;
        return true;
    }
    if (variant == 4011 || variant == 4014 || variant == 4021 || variant == 4041) {
        const int vs = (variant / 10) % 10;
        if (!ising_stream_supported(c, vs)) return false;
        c.ising_stream = true;
        c.ising_cap5 = false;
        c.ising_cap = variant % 10 == 4;
        c.vec_bytes = 16;
        c.ising_vpt = vs;
        return true;
    }
    if (variant == 6162) {
        if ((c.L[0] / 2) % 16) return false;
        c.ising_stream = false;
        c.ising_persist = false;
        c.ising_cap = false;
        c.ising_cap5 = true;
        c.vec_bytes = 16;
        c.ising_vpt = 2;
        return true;
    }
    if (variant < 0 || variant >= 4000) return false;
    c.ising_stream = false;
    c.ising_cap5 = false;
    const bool p = (variant / 1000) & 1, cap = (variant / 1000) >= 2;
    const int rest = variant % 1000, w = rest / 10, v = rest % 10;
    if ((w != 4 && w != 8 && w != 16) || (c.L[0] / 2) % w) return false;
    if (p ? (v != 2 && v != 4) : (v != 1 && v != 2 && v != 4)) return false;
    if (cap && (w != 16 || v == 1)) return false;
    c.ising_persist = p;
    c.ising_cap = cap;
    c.vec_bytes = w;
    c.ising_vpt = v;
    return true;
}

// The simple-cubic XYZ kernel's variants timed on both colour phases (three sweeps each);
// the configuration and acceptance counters are restored afterwards.
static int autotune_xyz(Ctx &c, int32_t *variant, float *best_ms) {
    const std::vector<long> key = {c.model, c.L[0], c.L[1], c.L[2], c.R, (long)c.zeeman, (long)(c.sia || c.sia_local),
                                   (long)c.angle};
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) {
            apply_variant(c, it->second);
            if (variant) *variant = variant_of(c);
            return ETHER_OK;
        }
    }
    const size_t bytes = (size_t)c.R * c.N * sizeof(float4);
    void *backup = nullptr;
    unsigned long long *acc_backup = nullptr;
    CUDA_TRY(cudaMalloc(&backup, bytes));
    CUDA_TRY(cudaMalloc(&acc_backup, sizeof(unsigned long long) * c.R));
    CUDA_TRY(cudaMemcpyAsync(backup, c.spins4, bytes, cudaMemcpyDeviceToDevice, c.stream));
    CUDA_TRY(cudaMemcpyAsync(acc_backup, c.acc_count, sizeof(unsigned long long) * c.R, cudaMemcpyDeviceToDevice, c.stream));
    int best_var = variant_of(c);
    float best = 1e30f;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    for (int cand : {5011, 5012, 5013, 5014, 5015, 5021, 5022, 5023, 5024, 5041, 5042}) {
        if (!apply_variant(c, cand)) continue;
        CUDA_TRY(launch_xyz_sweep(c, 0));  // warm-up
        CUDA_TRY(cudaEventRecord(e0, c.stream));
        for (int k = 0; k < 3; ++k) {
            CUDA_TRY(launch_xyz_sweep(c, 0));
            CUDA_TRY(launch_xyz_sweep(c, 1));
        }
        CUDA_TRY(cudaEventRecord(e1, c.stream));
        CUDA_TRY(cudaEventSynchronize(e1));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        ms /= 6.0f;
        if (ms < best) {
            best = ms;
            best_var = cand;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    apply_variant(c, best_var);
    CUDA_TRY(cudaMemcpyAsync(c.spins4, backup, bytes, cudaMemcpyDeviceToDevice, c.stream));
    CUDA_TRY(cudaMemcpyAsync(c.acc_count, acc_backup, sizeof(unsigned long long) * c.R, cudaMemcpyDeviceToDevice, c.stream));
    CUDA_TRY(cudaStreamSynchronize(c.stream));
    cudaFree(backup);
    cudaFree(acc_backup);
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune_cache[key] = best_var;
    }
    if (variant) *variant = best_var;
    if (best_ms) *best_ms = best;
    return ETHER_OK;
}

extern "C" int ether_autotune(ether_ctx *h, int32_t *variant, float *best_ms) {
    if (!h) return fail(ETHER_ERR_ARG, "null context");
    Ctx &c = h->c;
    if (variant) *variant = variant_of(c);
    if (best_ms) *best_ms = 0.f;
    if (!c.fast) return ETHER_OK;
    if (!c.beta_set) return fail(ETHER_ERR_STATE, "beta not set");
    if (c.model == ETHER_MODEL_XYZ) return autotune_xyz(c, variant, best_ms);
    const std::vector<long> key = {c.model, c.L[0], c.L[1], c.L[2], c.R};
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) {
            apply_variant(c, it->second);
            if (variant) *variant = variant_of(c);
            return ETHER_OK;
        }
    }
    const size_t bytes = (size_t)c.R * c.N;
    uint8_t *backup = nullptr;
    unsigned long long *acc_backup = nullptr;
    CUDA_TRY(cudaMalloc(&backup, bytes));
    CUDA_TRY(cudaMalloc(&acc_backup, sizeof(unsigned long long) * c.R));
    CUDA_TRY(cudaMemcpyAsync(backup, c.spins, bytes, cudaMemcpyDeviceToDevice, c.stream));
    CUDA_TRY(cudaMemcpyAsync(acc_backup, c.acc_count, sizeof(unsigned long long) * c.R,
                             cudaMemcpyDeviceToDevice, c.stream));
    int best_var = variant_of(c);
    float best = 1e30f;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    for (int cand : {161, 162, 164, 81, 82, 84, 41, 42, 44, 2162, 2164, 6162, 1162, 1164, 1082, 1084, 1042,
                     1044, 3162, 3164, 4011, 4014, 4021, 4041}) {
        if (!apply_variant(c, cand)) continue;
        CUDA_TRY(launch_ising_sweep(c, 0));  // warm-up
        CUDA_TRY(cudaEventRecord(e0, c.stream));
        for (int k = 0; k < 3; ++k) {
            CUDA_TRY(launch_ising_sweep(c, 0));
            CUDA_TRY(launch_ising_sweep(c, 1));
        }
        CUDA_TRY(cudaEventRecord(e1, c.stream));
        CUDA_TRY(cudaEventSynchronize(e1));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        ms /= 6.0f;
        if (ms < best) {
            best = ms;
            best_var = cand;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    apply_variant(c, best_var);
    CUDA_TRY(cudaMemcpyAsync(c.spins, backup, bytes, cudaMemcpyDeviceToDevice, c.stream));
    CUDA_TRY(cudaMemcpyAsync(c.acc_count, acc_backup, sizeof(unsigned long long) * c.R,
                             cudaMemcpyDeviceToDevice, c.stream));
    CUDA_TRY(cudaStreamSynchronize(c.stream));
    cudaFree(backup);
    cudaFree(acc_backup);
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune_cache[key] = best_var;
    }
    if (variant) *variant = best_var;
    if (best_ms) *best_ms = best;
    return ETHER_OK;
}

extern "C" int ether_set_variant(ether_ctx *h, int32_t variant) {
    if (!h) return fail(ETHER_ERR_ARG, "null context");
    Ctx &c = h->c;
    if (!c.fast) return ETHER_OK;
    if (!apply_variant(c, variant)) return fail(ETHER_ERR_ARG, "variant not available for this lattice");
    return ETHER_OK;
}

// Time series for autocorrelation analysis: nsweeps Metropolis sweeps, and after every
// stride-th sweep |M| (get_tot_magnetisation) and optionally E (get_tot_energy) of every
// replica.  absM, E: (nsweeps / stride) x R host arrays (E may be NULL).
extern "C" int ether_record_series(ether_ctx *h, int32_t nsweeps, int32_t stride, double *absM,
                                   double *E) {
    if (!h || !absM) return fail(ETHER_ERR_ARG, "null argument");
    Ctx &c = h->c;
    if (nsweeps <= 0 || stride <= 0 || nsweeps / stride <= 0)
        return fail(ETHER_ERR_ARG, "need nsweeps >= stride >= 1");
    if (!c.beta_set) return fail(ETHER_ERR_STATE, "beta not set");
    const int nrec = nsweeps / stride;
    double *mser = nullptr, *eser = nullptr;
    const size_t bytes = sizeof(double) * (size_t)nrec * c.R;
    CUDA_TRY(cudaMalloc(&mser, bytes));
    if (E && cudaMalloc(&eser, bytes) != cudaSuccess) {
        cudaGetLastError();  // reported here; not left for the next launch check to find
        cudaFree(mser);
        return fail(ETHER_ERR_NOMEM, "cudaMalloc of the energy series failed");
    }
    int rc = ETHER_OK;
    int t = 0;
    int32_t *t_dev = nullptr;
    cudaGraphExec_t ex = nullptr;
    bool use_graph = nrec >= 4 && !(c.flags & ETHER_FLAG_NO_GRAPHS);
    if (use_graph && cudaMalloc(&t_dev, sizeof(int32_t)) != cudaSuccess) {
        cudaGetLastError();  // direct launches instead; the failed allocation is not a lasting error
        t_dev = nullptr;
        use_graph = false;
    }
    if (use_graph) {
        // one stride -- stride sweeps and the record of row *t_dev -- captured once, replayed
        // for every row
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaMemsetAsync(t_dev, 0, sizeof(int32_t), c.stream);
        if (e == cudaSuccess) e = cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            for (int k = 0; k < stride && rc == ETHER_OK; ++k) rc = sweep_once(c);
            if (rc == ETHER_OK) e = launch_record(c, 0, E != nullptr, mser, eser, t_dev);
            const cudaError_t ee = cudaStreamEndCapture(c.stream, &g);
            if (e == cudaSuccess) e = ee;
        }
        if (rc == ETHER_OK && e == cudaSuccess) e = cudaGraphInstantiate(&ex, g, 0);
        if (g) cudaGraphDestroy(g);
        for (int i = 0; i < nrec && rc == ETHER_OK && e == cudaSuccess; ++i) e = cudaGraphLaunch(ex, c.stream);
        if (rc == ETHER_OK && e != cudaSuccess) rc = fail(ETHER_ERR_CUDA, std::string("series graph: ") + cudaGetErrorString(e));
        // the sweeps after the last recorded row
        for (int k = nrec * stride + 1; k <= nsweeps && rc == ETHER_OK; ++k) rc = sweep_once(c);
    } else {
        for (int k = 1; k <= nsweeps && rc == ETHER_OK; ++k) {
            rc = sweep_once(c);
            if (rc == ETHER_OK && k % stride == 0 && t < nrec) {
                cudaError_t e = launch_record(c, t++, E != nullptr, mser, eser);
                if (e != cudaSuccess) rc = fail(ETHER_ERR_CUDA, std::string("record: ") + cudaGetErrorString(e));
            }
        }
    }
    if (rc == ETHER_OK) {
        cudaError_t e = cudaMemcpyAsync(absM, mser, bytes, cudaMemcpyDeviceToHost, c.stream);
        if (e == cudaSuccess && E) e = cudaMemcpyAsync(E, eser, bytes, cudaMemcpyDeviceToHost, c.stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
        if (e != cudaSuccess) rc = fail(ETHER_ERR_CUDA, std::string("series copy: ") + cudaGetErrorString(e));
    }
    if (ex) cudaGraphExecDestroy(ex);
    if (t_dev) cudaFree(t_dev);
    cudaFree(mser);
    if (eser) cudaFree(eser);
    return rc;
}

// structure_factor (utility/Structure_Factor/structure_factor.f90:99-183) on the tensor cores;
// see k_sq.cu.  Positions become fractional coordinates of the cell abc (rows = a1, a2, a3).
extern "C" int ether_structure_factor(ether_ctx *h, const double *abc, const int32_t nq[3],
                                      const double q0[3], const double dq[3], float *sq,
                                      float *comp) {
    if (!h || !abc || !nq || !q0 || !dq || !sq || !comp) return fail(ETHER_ERR_ARG, "null argument");
    Ctx &c = h->c;
    // inverse of the matrix whose rows are the lattice vectors: r = sum_a f_a a_a
    const double *A = abc;
    const double det = A[0] * (A[4] * A[8] - A[5] * A[7]) - A[1] * (A[3] * A[8] - A[5] * A[6]) +
                       A[2] * (A[3] * A[7] - A[4] * A[6]);
    if (!(std::fabs(det) > 1e-300)) return fail(ETHER_ERR_ARG, "cell vectors are degenerate");
    // columns of inv(A^T): f = inv(A^T) r
    double inv[9];  // inv of A (row-major), f_a = sum_d r_d inv[d*3 + a]
    inv[0] = (A[4] * A[8] - A[5] * A[7]) / det;
    inv[1] = -(A[1] * A[8] - A[2] * A[7]) / det;
    inv[2] = (A[1] * A[5] - A[2] * A[4]) / det;
    inv[3] = -(A[3] * A[8] - A[5] * A[6]) / det;
    inv[4] = (A[0] * A[8] - A[2] * A[6]) / det;
    inv[5] = -(A[0] * A[5] - A[2] * A[3]) / det;
    inv[6] = (A[3] * A[7] - A[4] * A[6]) / det;
    inv[7] = -(A[0] * A[7] - A[1] * A[6]) / det;
    inv[8] = (A[0] * A[4] - A[1] * A[3]) / det;
    std::vector<double> frac(3 * (size_t)c.N);
    for (int s = 0; s < c.N; ++s)
        for (int a = 0; a < 3; ++a)
            frac[3 * (size_t)s + a] = c.pos[3 * (size_t)s] * inv[0 * 3 + a] + c.pos[3 * (size_t)s + 1] * inv[1 * 3 + a] +
                                      c.pos[3 * (size_t)s + 2] * inv[2 * 3 + a];
    std::string msg;
    const int nqi[3] = {nq[0], nq[1], nq[2]};
    const int rc = structure_factor_launch(c, frac.data(), nqi, q0, dq, sq, comp, msg);
    if (rc) return fail(rc, "ether_structure_factor: " + msg);
    return ETHER_OK;
}
