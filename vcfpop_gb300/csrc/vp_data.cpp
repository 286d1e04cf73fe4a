// Host-side dataset preparation: the part of CalcBayesian that runs before the
// MCMC (src/structure.cpp:2337-2395) plus the loader/filter facts it depends
// on -- which loci survive the default monomorphic-locus filter and how wide
// each locus' genotype ids are, since that width orders the loci and the locus
// index keys the reference's random streams.
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <thread>

#include <cuda_runtime.h>

#include "vp_internal.h"

template <typename T>
void HostBuf<T>::release() {
    if (!p) return;
    if (pinned) cudaFreeHost(p);
    else free(p);
    p = nullptr;
    n = 0;
}
template <typename T>
void HostBuf<T>::resize(size_t m) {
    release();
    if (m == 0) return;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) == cudaSuccess && ndev > 0 && cudaMallocHost((void**)&p, m * sizeof(T)) == cudaSuccess)
        pinned = true;
    else {
        cudaGetLastError();
        p = (T*)malloc(m * sizeof(T));
        pinned = false;
    }
    n = m;
}
template struct HostBuf<uint32_t>;

namespace {

thread_local char g_err[1024];

// CeilLog2 of the number of genotype ids at a locus (src/math2.h:503-512)
int ceil_log2(int64_t v) {
    if (v <= 1) return 1;
    int b = 0;
    uint64_t x = (uint64_t)(v - 1);
    while (x) { b++; x >>= 1; }
    return b;
}

template <typename F>
void parallel_for(int64_t n, F f) {
    int nt = (int)std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
    if (n < 4096) nt = 1;
    std::vector<std::thread> th;
    for (int t = 0; t < nt; ++t)
        th.emplace_back([=, &f] {
            for (int64_t i = n * t / nt; i < n * (t + 1) / nt; ++i) f(i);
        });
    for (auto& x : th) x.join();
}

bool is_coprime(int64_t x, int64_t y) {
    int64_t z = 1;
    while (x % y != 0) { z = x % y; x = y; y = z; }
    return z == 1;
}

inline int code_at(const uint32_t* row, int i) { return (row[i >> 4] >> ((i & 15) * 2)) & 3; }

// Per input locus, from its calls: whether the locus is polymorphic (a
// typed genotype with two alleles, or two different typed genotypes:
// ApplyFilter, src/filter.cpp:102-133; fewer than 2 alleles never) and how
// many genotype ids the loader gives it (one per distinct typed genotype
// plus one missing id per ploidy level of the individuals,
// src/load.cpp:2180-2230)
void table_facts(const vp_input* in, bool p2, int vmax, uint8_t* pass, int32_t* ngeno) {
    const int32_t N = in->n_ind;
    const int Nw = (N + 15) / 16;
    parallel_for(in->n_loc, [&](int64_t l) {
        pass[l] = 0;
        ngeno[l] = 1;
        if (in->n_alleles[l] < 2) return;
        if (p2) {
            const uint32_t* row = in->packed2 + (size_t)l * Nw;
            int seen = 0;  // bit c set when code c observed
            for (int i = 0; i < N; ++i) seen |= 1 << code_at(row, i);
            int typed = seen & 7;
            pass[l] = (typed & 2) || ((typed & 5) == 5);
            ngeno[l] = 1 + ((typed & 1) != 0) + ((typed & 2) != 0) + ((typed & 4) != 0);
            return;
        }
        const int8_t* G = in->alleles + (size_t)l * N * vmax;
        int first = -1, ok = 0;
        std::vector<uint64_t> keys;
        keys.reserve(N);
        uint32_t used = 0;
        for (int i = 0; i < N; ++i) {
            const int8_t* g = G + (size_t)i * vmax;
            int v = in->ploidy[i];
            used |= 1u << v;
            if (g[0] < 0) continue;
            uint64_t h = (uint64_t)v;
            for (int c = 0; c < v; ++c) {
                h = h * 64 + (uint64_t)(g[c] + 1);
                if (g[c] != g[0]) ok = 1;
            }
            if (first < 0) first = g[0];
            else if (g[0] != first) ok = 1;
            keys.push_back(h);
        }
        std::sort(keys.begin(), keys.end());
        int64_t ng = __builtin_popcount(used);
        for (size_t j = 0; j < keys.size(); ++j)
            if (j == 0 || keys[j] != keys[j - 1]) ng++;
        pass[l] = (uint8_t)ok;
        ngeno[l] = (int32_t)ng;
    });
}

}  // namespace

void vp_set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
}

extern "C" const char* vp_last_error(void) { return g_err; }

extern "C" int vp_genotype_table(const vp_input* in, uint8_t* poly, int32_t* ngeno) {
    if (!in || !poly || !ngeno || in->n_ind <= 0 || in->n_loc <= 0 || !in->ploidy || !in->n_alleles ||
        (!in->alleles && !in->packed2) || (!in->packed2 && (in->vmax <= 0 || in->vmax > 10))) {
        vp_set_error("vp_genotype_table: missing or empty input");
        return VP_E_ARG;
    }
    const bool p2 = in->packed2 != nullptr;
    table_facts(in, p2, p2 ? 2 : in->vmax, poly, ngeno);
    return VP_OK;
}

extern "C" int vp_dataset_prepare(const vp_input* in, vp_dataset** out) {
    if (!in || !out || in->n_ind <= 0 || in->n_loc <= 0 || !in->ploidy || !in->n_alleles || !in->popid ||
        in->n_pop <= 0 || (!in->alleles && !in->packed2)) {
        vp_set_error("vp_dataset_prepare: missing or empty input");
        return VP_E_ARG;
    }
    const int32_t N = in->n_ind;
    const int64_t L0 = in->n_loc;
    const int Nw = (N + 15) / 16;
    bool p2 = in->packed2 != nullptr;
    if (p2) {
        for (int i = 0; i < N; ++i)
            if (in->ploidy[i] != 2) { vp_set_error("packed2 input needs ploidy 2 for every individual"); return VP_E_ARG; }
        for (int64_t l = 0; l < L0; ++l)
            if (in->n_alleles[l] != 2) { vp_set_error("packed2 input needs 2 alleles at every locus"); return VP_E_ARG; }
    } else if (in->vmax <= 0 || in->vmax > 10) {
        vp_set_error("vmax must be in 1..10");
        return VP_E_ARG;
    }
    for (int i = 0; i < N; ++i)
        if (in->popid[i] < 0 || in->popid[i] >= in->n_pop || (i && in->popid[i] < in->popid[i - 1])) {
            vp_set_error("popid must be in [0, n_pop) and non-decreasing (individuals grouped by population)");
            return VP_E_ARG;
        }
    const int vmax = p2 ? 2 : in->vmax;
    auto* d = new vp_dataset();
    d->N = N; d->S = in->n_pop; d->vmax = vmax; d->Nw = Nw; d->packed2 = p2;

    // 1. per input locus: pass flag (polymorphic in the loader's genotype
    //    table) and genotype-id width, from the table facts when given
    std::vector<uint8_t> pass(L0, 0), width(L0, 0);
    if (in->table_poly && in->table_ngeno) {
        for (int64_t l = 0; l < L0; ++l) {
            pass[l] = in->n_alleles[l] >= 2 && in->table_poly[l];
            width[l] = (uint8_t)ceil_log2(std::max<int32_t>(1, in->table_ngeno[l]));
        }
    } else {
        std::vector<int32_t> ng(L0, 1);
        table_facts(in, p2, vmax, pass.data(), ng.data());
        for (int64_t l = 0; l < L0; ++l) width[l] = (uint8_t)ceil_log2(ng[l]);
    }
    std::vector<int64_t> keep;
    for (int64_t l = 0; l < L0; ++l)
        if (pass[l]) keep.push_back(l);
    const int64_t L = (int64_t)keep.size();
    if (L == 0) {
        delete d;
        vp_set_error("all %lld loci are monomorphic", (long long)L0);
        return VP_E_ARG;
    }
    // 2. stable order by (width, input index)
    std::vector<int64_t> pos(L);
    for (int64_t j = 0; j < L; ++j) pos[j] = j;
    std::stable_sort(pos.begin(), pos.end(), [&](int64_t a, int64_t b) { return width[keep[a]] < width[keep[b]]; });
    d->L = L;
    d->order.resize(L);
    d->k.resize(L);
    d->off.resize(L);
    int64_t KT = 0;
    for (int64_t l = 0; l < L; ++l) {
        d->order[l] = keep[pos[l]];
        d->k[l] = in->n_alleles[d->order[l]];
        d->off[l] = KT;
        KT += d->k[l];
        d->maxK = std::max(d->maxK, d->k[l]);
    }
    d->KT = KT;
    d->kdis.assign(d->maxK + 1, 0);
    for (int64_t l = 0; l < L; ++l) d->kdis[d->k[l]]++;
    // 3. genotypes in sorted order, typed copies per individual
    d->vt.assign(N, 0);
    if (p2) {
        d->g2.resize((size_t)L * Nw);
        parallel_for(L, [&](int64_t l) {
            memcpy(&d->g2[(size_t)l * Nw], in->packed2 + (size_t)d->order[l] * Nw, Nw * sizeof(uint32_t));
        });
        std::vector<int64_t> typed(N, 0);
        for (int64_t l = 0; l < L; ++l) {
            const uint32_t* row = &d->g2[(size_t)l * Nw];
            for (int i = 0; i < N; ++i) typed[i] += code_at(row, i) != 3;
        }
        for (int i = 0; i < N; ++i) d->vt[i] = 2 * typed[i];
        d->maxploidy = 0;
        for (int i = 0; i < N; ++i) if (typed[i]) d->maxploidy = 2;
    } else {
        d->gb.assign((size_t)L * N * vmax, 0xFF);
        parallel_for(L, [&](int64_t l) {
            const int8_t* G = in->alleles + (size_t)d->order[l] * N * vmax;
            uint8_t* o = &d->gb[(size_t)l * N * vmax];
            for (int i = 0; i < N; ++i) {
                const int8_t* g = G + (size_t)i * vmax;
                if (g[0] < 0) continue;
                for (int c = 0; c < in->ploidy[i]; ++c) o[(size_t)i * vmax + c] = (uint8_t)g[c];
            }
        });
        for (int64_t l = 0; l < L; ++l) {
            const uint8_t* o = &d->gb[(size_t)l * N * vmax];
            for (int i = 0; i < N; ++i)
                if (o[(size_t)i * vmax] != 0xFF) {
                    d->vt[i] += in->ploidy[i];
                    d->maxploidy = std::max(d->maxploidy, in->ploidy[i]);
                }
        }
        // with mixed ploidy the per-copy kernels take individuals in ascending
        // ploidy, so that a warp's lanes loop over the same number of copies
        bool mixed = false;
        for (int i = 1; i < N; ++i) mixed |= in->ploidy[i] != in->ploidy[0];
        if (mixed) {
            d->perm.resize(N);
            for (int i = 0; i < N; ++i) d->perm[i] = i;
            std::stable_sort(d->perm.begin(), d->perm.end(),
                             [&](int32_t a, int32_t b) { return in->ploidy[a] < in->ploidy[b]; });
        }
    }
    // 4. total-population frequencies and typed copies in the FILTERED INPUT
    //    order: CalcFreq runs before the sort (src/function.cpp:4690-4694,
    //    3974-4017) and InitFmodel later reads them with sorted offsets.
    d->totfreq.assign(KT, 0.f);
    d->nhaplo.assign(L, 0);
    {
        std::vector<int64_t> off_in(L);
        int64_t o = 0;
        for (int64_t j = 0; j < L; ++j) { off_in[j] = o; o += in->n_alleles[keep[j]]; }
        parallel_for(L, [&](int64_t j) {
            int64_t l = keep[j];
            int k2 = in->n_alleles[l];
            float* p = &d->totfreq[off_in[j]];
            int nh = 0;
            if (p2) {
                const uint32_t* row = in->packed2 + (size_t)l * Nw;
                int64_t c1 = 0, t = 0;
                for (int i = 0; i < N; ++i) { int c = code_at(row, i); if (c != 3) { t++; c1 += c; } }
                p[0] = (float)(2 * t - c1);
                p[1] = (float)c1;
                nh = (int)(2 * t);
            } else {
                const int8_t* G = in->alleles + (size_t)l * N * vmax;
                for (int i = 0; i < N; ++i) {
                    const int8_t* g = G + (size_t)i * vmax;
                    if (g[0] < 0) continue;
                    nh += in->ploidy[i];
                    for (int c = 0; c < in->ploidy[i]; ++c) p[g[c]] += 1.0f;
                }
            }
            d->nhaplo[j] = nh;
            double s = 0;  // Unify(float*) (src/math2.cpp:2288-2305)
            for (int a = 0; a < k2; ++a) s += p[a];
            double inv = 1.0 / (s + k2 * 1e-10);
            for (int a = 0; a < k2; ++a) p[a] = (float)(((double)p[a] + 1e-10) * inv);
        });
    }
    d->popid.assign(in->popid, in->popid + N);
    d->pop_ind0.assign(d->S, 0);
    d->pop_nind.assign(d->S, 0);
    for (int i = 0; i < N; ++i)
        if (d->pop_nind[d->popid[i]]++ == 0) d->pop_ind0[d->popid[i]] = i;
    // 5. locus visiting stride of the reference's threads (src/structure.cpp:2384-2386)
    int64_t cp = L <= 67 ? 1 : 67;
    while (!is_coprime(L, cp)) cp++;
    if (cp >= L) cp = 1;
    d->coprime = cp;
    *out = d;
    return VP_OK;
}

extern "C" int vp_dataset_info_get(const vp_dataset* d, vp_dataset_info* info) {
    if (!d || !info) { vp_set_error("null argument"); return VP_E_ARG; }
    info->n_ind = d->N; info->n_pop = d->S; info->maxploidy = d->maxploidy; info->max_alleles = d->maxK;
    info->packed2 = d->packed2; info->n_loc = d->L; info->n_alleles_total = d->KT; info->coprime = d->coprime;
    return VP_OK;
}

extern "C" int vp_dataset_order(const vp_dataset* d, int64_t* order) {
    if (!d || !order) { vp_set_error("null argument"); return VP_E_ARG; }
    memcpy(order, d->order.data(), d->L * sizeof(int64_t));
    return VP_OK;
}

extern "C" void vp_dataset_free(vp_dataset* d) {
    if (d && d->refs.fetch_sub(1, std::memory_order_acq_rel) == 1) delete d;
}

void vp_dataset_retain(const vp_dataset* d) { const_cast<vp_dataset*>(d)->refs.fetch_add(1, std::memory_order_relaxed); }

extern "C" void vp_params_default(vp_params* p) {
    memset(p, 0, sizeof *p);
    // src/parameters.cpp:584-627 (yes = 1, no = 0)
    p->K = 2;
    p->nburnin = 1000; p->nreps = 10000; p->nthinning = 10; p->nadmburnin = 500;
    p->lambda = 1; p->stdlambda = 0.3; p->maxlambda = 10;
    p->inferlambda = 0;  // the reference never infers lambda (src/structure.cpp:430)
    p->alpha = 1; p->stdalpha = 0.025; p->maxalpha = 10; p->alphapriora = 0.05; p->alphapriorb = 0.001;
    p->metrofreq = 10; p->inferalpha = 1; p->diffalpha = 0; p->uniformalpha = 1;
    p->r = 1; p->maxr = 20; p->epsr = 0.1; p->epseta = 0.025; p->epsgamma = 0.025;
    p->pmeanf = 0.01; p->pstdf = 0.05; p->stdf = 0.05; p->fsame = 0;
    p->rng = VP_RNG_COUNTER;
    p->form = VP_FORM_PLAIN;
}

static uint32_t crc32c_u64(uint32_t crc, uint64_t v) {
    for (int b = 0; b < 8; ++b) {
        crc ^= (uint32_t)(v & 0xFF);
        v >>= 8;
        for (int j = 0; j < 8; ++j) crc = (crc >> 1) ^ (0x82F63B78u & (0u - (crc & 1u)));
    }
    return crc;
}

extern "C" uint64_t vp_run_seed(int64_t g_seed, int32_t run_id) {
    return (uint64_t)crc32c_u64(0xB385FDA9u, (uint64_t)(g_seed + run_id));
}
