/*
 * ORACLE (test infrastructure only): CPU restatement of vcfpop's Bayesian
 * STRUCTURE MCMC, REAL = float, -g_fastsingle=yes, one thread, scalar math
 * (-g_simd=none). Every step cites the reference (vcfpop v1.08b, src/).
 *
 * Parity is pinned against the reference program compiled from its own
 * sources (oracle/Makefile) through the golden fixtures under tests/golden/.
 * Nothing in the product links this file.
 */
#include "structure_oracle.h"
#include "orc_core.h"
#include <stdlib.h>
#include <string.h>
#include <stdio.h>
#include <pthread.h>

#define NEW(T, n) ((T*)calloc((size_t)((n) > 0 ? (n) : 1), sizeof(T)))

/* ================= dataset construction ================= */

struct orc_owned_data {
    orc_data v;
    int32_t *k, *popid, *pop_ind0, *pop_nind, *nhaplo;
    int64_t *off, *vt, *order;
    uint8_t *gcopies, *galleles;
    float* totfreq;
};

/* CeilLog2 (math2.h:503-512): the bit width of a locus' genotype ids */
static int ceil_log2(int64_t v) {
    if (v <= 1) return 1;
    int b = 0;
    uint64_t x = (uint64_t)(v - 1);
    while (x) { b++; x >>= 1; }
    return b;
}

/* IsCoprime (structure.cpp:2184-2197) */
static int is_coprime(int64_t x, int64_t y) {
    int64_t z = 1;
    while (x % y != 0) { z = x % y; x = y; y = z; }
    return z == 1;
}

static int cmp_u64(const void* a, const void* b) {
    uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
    return x < y ? -1 : x > y;
}

orc_owned_data* orc_data_build(int32_t N, int64_t L, int32_t vmax, const int8_t* G,
                               const int32_t* ploidy, const int32_t* k,
                               const int32_t* popid, int32_t S) {
    return orc_data_build_ex(N, L, vmax, G, ploidy, k, popid, S, NULL);
}

orc_owned_data* orc_data_build_ex(int32_t N, int64_t L, int32_t vmax, const int8_t* G,
                                  const int32_t* ploidy, const int32_t* k,
                                  const int32_t* popid, int32_t S, const int8_t* Gtable) {
    orc_owned_data* d = NEW(orc_owned_data, 1);
    /* the loader's genotype table holds the calls before the genotype filter
     * (load.cpp:2145-2230): the polymorphism test and the id widths read it */
    const int8_t* T = Gtable ? Gtable : G;
    /* 0. keep loci that are polymorphic in the genotype table: a heterozygote
     *    or two different homozygotes (filter.cpp:102-131); k < 2 never passes */
    int64_t* keep = NEW(int64_t, L);
    int64_t L0 = L;
    L = 0;
    for (int64_t l = 0; l < L0; ++l) {
        int pass = 0, first = -1;
        if (k[l] >= 2)
            for (int32_t i = 0; i < N && !pass; ++i) {
                const int8_t* g = T + ((size_t)l * N + i) * vmax;
                if (g[0] < 0) continue;
                for (int c = 1; c < ploidy[i]; ++c) if (g[c] != g[0]) pass = 1;
                if (first < 0) first = g[0];
                else if (g[0] != first) pass = 1;
            }
        if (pass) keep[L++] = l;
    }
    /* 1. bit width per locus: one id per distinct typed genotype plus one
     *    "missing" id per ploidy level seen at the locus (load.cpp:1656-1702) */
    uint64_t* key = NEW(uint64_t, L);
    uint64_t* gk = NEW(uint64_t, N);
    for (int64_t l = 0; l < L; ++l) {
        int used[16] = {0};
        int ng = 0, n = 0;
        for (int32_t i = 0; i < N; ++i) {
            const int8_t* g = T + ((size_t)keep[l] * N + i) * vmax;
            int v = ploidy[i];
            if (!used[v]) { used[v] = 1; ng++; }
            if (g[0] < 0) continue;
            uint64_t h = (uint64_t)v;
            for (int c = 0; c < v; ++c) h = h * 64 + (uint64_t)(g[c] + 1);
            gk[n++] = h;
        }
        qsort(gk, (size_t)n, sizeof(uint64_t), cmp_u64);
        for (int j = 0; j < n; ++j) if (j == 0 || gk[j] != gk[j - 1]) ng++;
        key[l] = ((uint64_t)ceil_log2(ng) << 40) | (uint64_t)l;
    }
    free(gk);
    /* 2. stable sort by (bit width, input index): QSLocus2, structure.cpp:2202-2273 */
    qsort(key, (size_t)L, sizeof(uint64_t), cmp_u64);
    d->order = NEW(int64_t, L);
    for (int64_t l = 0; l < L; ++l) d->order[l] = (int64_t)(key[l] & 0xFFFFFFFFFFull);
    free(key);
    /* order[] indexes the filtered loci; sorted position -> filtered index */

    /* 3. offsets in sorted order (structure.cpp:2374-2381) */
    d->k = NEW(int32_t, L);
    d->off = NEW(int64_t, L);
    int64_t KT = 0;
    int maxK = 0;
    for (int64_t l = 0; l < L; ++l) {
        d->k[l] = k[keep[d->order[l]]];
        d->off[l] = KT;
        KT += d->k[l];
        if (d->k[l] > maxK) maxK = d->k[l];
    }
    /* 4. genotypes in sorted locus order, typed copies per call */
    d->gcopies = NEW(uint8_t, (size_t)L * N);
    d->galleles = NEW(uint8_t, (size_t)L * N * vmax);
    d->vt = NEW(int64_t, N);
    int maxploidy = 0;
    for (int64_t l = 0; l < L; ++l) {
        int64_t lo = keep[d->order[l]];
        for (int32_t i = 0; i < N; ++i) {
            const int8_t* g = G + ((size_t)lo * N + i) * vmax;
            uint8_t* o = d->galleles + ((size_t)l * N + i) * vmax;
            if (g[0] < 0) { d->gcopies[(size_t)l * N + i] = 0; continue; }
            int v = ploidy[i];
            d->gcopies[(size_t)l * N + i] = (uint8_t)v;
            for (int c = 0; c < v; ++c) o[c] = (uint8_t)g[c];
            d->vt[i] += v;                         /* AssignPloidyThread, function.cpp:4873-4880 */
            if (v > maxploidy) maxploidy = v;
        }
    }
    /* 5. total-population allele frequencies and typed copies per locus, in
     *    INPUT locus order (CalcFreq runs before the sort: function.cpp:4690-4694,
     *    POP::CalcFreqGcount function.cpp:3974-4017). */
    int64_t* off_in = NEW(int64_t, L);
    int64_t kt2 = 0;
    for (int64_t l = 0; l < L; ++l) { off_in[l] = kt2; kt2 += k[keep[l]]; }
    d->totfreq = NEW(float, KT);
    d->nhaplo = NEW(int32_t, L);
    for (int64_t l = 0; l < L; ++l) {
        float* p = d->totfreq + off_in[l];
        int nh = 0;
        for (int32_t i = 0; i < N; ++i) {
            const int8_t* g = G + ((size_t)keep[l] * N + i) * vmax;
            if (g[0] < 0) continue;
            int v = ploidy[i];
            nh += v;
            for (int c = 0; c < v; ++c) p[g[c]] += 1.0f;
        }
        d->nhaplo[l] = nh;
        orc_unify_f(p, k[keep[l]]);
    }
    free(off_in);
    for (int64_t l = 0; l < L; ++l) d->order[l] = keep[d->order[l]];
    d->popid = NEW(int32_t, N);
    d->pop_ind0 = NEW(int32_t, S);
    d->pop_nind = NEW(int32_t, S);
    for (int32_t i = 0; i < N; ++i) {
        d->popid[i] = popid[i];
        if (d->pop_nind[popid[i]]++ == 0) d->pop_ind0[popid[i]] = i;
    }
    /* 6. locus visiting order stride (structure.cpp:2384-2386) */
    int64_t cp = L <= 67 ? 1 : 67;
    while (!is_coprime(L, cp)) cp++;
    if (cp >= L) cp = 1;

    orc_data* v = &d->v;
    v->N = N; v->L = L; v->S = S; v->vmax = vmax; v->maxploidy = maxploidy; v->maxK = maxK; v->KT = KT;
    v->k = d->k; v->off = d->off; v->gcopies = d->gcopies; v->galleles = d->galleles; v->vt = d->vt;
    v->popid = d->popid; v->pop_ind0 = d->pop_ind0; v->pop_nind = d->pop_nind;
    v->totfreq = d->totfreq; v->nhaplo = d->nhaplo; v->coprime = cp;
    free(keep);
    return d;
}

const orc_data* orc_data_view(const orc_owned_data* d) { return &d->v; }
const int64_t* orc_data_order(const orc_owned_data* d) { return d->order; }
void orc_data_free(orc_owned_data* d) {
    if (!d) return;
    free(d->k); free(d->popid); free(d->pop_ind0); free(d->pop_nind); free(d->nhaplo);
    free(d->off); free(d->vt); free(d->order); free(d->gcopies); free(d->galleles); free(d->totfreq);
    free(d);
}
uint32_t orc_hash_ulong_c(uint64_t v) { return orc_hash_ulong(v); }

/* ================= chain ================= */

#define FREQ(c, k, l) ((c)->Freq + (int64_t)(k) * (c)->KT + (c)->D->off[l])
#define GC(c, l, i) ((c)->D->gcopies[(size_t)(l) * (c)->N + (i)])
#define GA(c, l, i) ((c)->D->galleles + ((size_t)(l) * (c)->N + (i)) * (c)->D->vmax)

orc_chain* orc_chain_new(const orc_data* D, const orc_params* P) {
    orc_chain* c = NEW(orc_chain, 1);
    c->P = *P; c->D = D;
    /* ReadPar, structure.cpp:405-464 */
    c->K = P->K; c->N = D->N; c->L = D->L; c->S = D->S; c->KT = D->KT;
    c->nburnin = P->nburnin; c->nreps = P->nreps; c->nthinning = P->nthinning;
    c->kdis = NEW(int64_t, D->maxK + 1);
    for (int64_t l = 0; l < D->L; ++l) c->kdis[D->k[l]]++;
    c->nadmburnin = (!P->locpriori && !P->admix) ? P->nadmburnin : 0;
    c->nburnin += c->nadmburnin;
    return c;
}

void orc_chain_free(orc_chain* c) {
    if (!c) return;
    free(c->Freq); free(c->FreqM); free(c->FreqA); free(c->Lambda); free(c->MiSum); free(c->Z);
    free(c->Mi); free(c->Q); free(c->Ni); free(c->Alpha); free(c->f); free(c->F); free(c->Eta);
    free(c->Gamma); free(c->Di); free(c->AlphaLocal); free(c->SumAlpha); free(c->fbuf1); free(c->fbuf2);
    free(c->bufNK1); free(c->bufNK2); free(c->bufN1); free(c->bufN2); free(c->bufK); free(c->lnL);
    free(c->rout); free(c->kdis); free(c);
}

/* InitFix: structure.cpp:466-553 */
static void init_fix(orc_chain* c) {
    int K = c->K, N = c->N; int64_t KT = c->KT;
    c->nr = 0; c->r = 1;
    c->Freq = NEW(float, K * KT);
    c->FreqM = NEW(float, K * KT);
    c->FreqA = NEW(float, 3 * KT);
    c->bufNK1 = NEW(double, (N > 64 ? N : 64) * K);
    c->bufNK2 = NEW(double, (N > 64 ? N : 64) * K);
    c->bufN1 = NEW(double, N);
    c->bufN2 = NEW(double, N);
    c->bufK = NEW(float, K);
    c->MiSum = NEW(int64_t, N * K);
    for (int64_t j = 0; j < K * KT; ++j) c->Freq[j] = 0.5f;
    c->Ni = NEW(int32_t, K * KT);
    c->Mi = NEW(int64_t, N * K);
    c->Q = NEW(float, N * K);
    for (int64_t j = 0; j < (int64_t)N * K; ++j) c->Q[j] = (float)(1.0 / K);
    c->Alpha = NEW(double, K);
    for (int k = 0; k < K; ++k) c->Alpha[k] = c->P.alpha;
    c->Lambda = NEW(double, K);
    for (int k = 0; k < K; ++k) c->Lambda[k] = c->P.lambda;
    int nf = c->P.fmodel ? (c->P.fsame ? 1 : K) : 0;
    int na = c->P.admix ? (c->P.diffalpha ? K : 1) : 0;
    int nl = c->P.difflambda ? K : 1;
    c->rlen = c->P.locpriori ? 4 + nl + 1 + K + K * c->S + nf : 4 + nl + na + nf;
    c->rout = NEW(double, c->rlen);
    /* Record writes at m % nthinning == 0 in burn-in and every nthinning-th
     * sweep after it: ceil(nburnin / t) + ceil(nreps / t) values */
    if (c->P.writelnl) {
        const int t = c->nthinning;
        c->lnL = NEW(double, (c->nburnin + t - 1) / t + (c->nreps + t - 1) / t + 1);
        c->nlnL = 0;
    }
    for (int64_t l = 0; l < c->L; ++l) {
        int k2 = c->D->k[l];
        if (k2 == 2) continue;
        for (int k = 0; k < K; ++k) {
            float* p = FREQ(c, k, l);
            for (int a = 0; a < k2; ++a) p[a] = (float)(1.0 / k2);
        }
    }
}

/* InitAdmix: structure.cpp:555-649 */
static void init_admix(orc_chain* c) {
    int K = c->K, N = c->N; int64_t KT = c->KT;
    c->Z = NEW(uint16_t, N + 32);
    c->singlez = c->nadmburnin == 0 && !c->P.admix;
    if (c->singlez) {
        orc_rng64 rng; orc_rng64_init(&rng, c->P.seed - 1, SALT_INITADM);
        for (int i = 0; i < N; ++i) {
            c->Z[i] = (uint16_t)orc_rng64_nextn(&rng, K);
            c->Mi[i * K + c->Z[i]] = c->D->vt[i];
        }
        for (int64_t l = 0; l < c->L; ++l)
            for (int i = 0; i < N; ++i) {
                int v = GC(c, l, i);
                if (!v) continue;
                int32_t* ni = c->Ni + (int64_t)c->Z[i] * KT + c->D->off[l];
                const uint8_t* als = GA(c, l, i);
                for (int a = 0; a < v; ++a) ni[als[a]]++;
            }
    } else {
        for (int64_t ll = 0; ll < c->L; ++ll) {
            int64_t l = ll * c->D->coprime % c->L;
            int64_t o = c->D->off[l];
            orc_rng64 rng; orc_rng64_init(&rng, c->P.seed + l, SALT_INITADM);
            int64_t* mi = c->Mi;
            for (int i = 0; i < N; ++i, mi += K) {
                int v = GC(c, l, i);
                if (!v) continue;
                const uint8_t* als = GA(c, l, i);
                for (int a = 0; a < v; ++a) {
                    uint16_t k2 = (uint16_t)orc_rng64_nextn(&rng, K);
                    mi[k2]++;
                    c->Ni[o + k2 * KT + als[a]]++;
                }
            }
        }
    }
}

/* InitLocPriori: structure.cpp:651-675 */
static void init_locpriori(orc_chain* c) {
    if (!c->P.locpriori) return;
    int K = c->K, S = c->S;
    c->SumAlpha = NEW(double, S);
    c->AlphaLocal = NEW(double, S * K);
    for (int j = 0; j < S * K; ++j) c->AlphaLocal[j] = c->P.alpha;
    if (!c->P.admix) {
        c->Eta = NEW(double, K);
        for (int k = 0; k < K; ++k) c->Eta[k] = (double)(1.0 / K);
        c->Gamma = NEW(double, S * K);
        for (int j = 0; j < S * K; ++j) c->Gamma[j] = (double)(1.0 / K);
        c->Di = NEW(float, S * K);
    }
}

/* InitFmodel: structure.cpp:677-708. The total-population frequencies were
 * computed in input locus order but are read here with the sorted order's
 * offsets and locus indices, exactly as the reference does. */
static void init_fmodel(orc_chain* c) {
    if (!c->P.fmodel) return;
    int K = c->K; int64_t KT = c->KT;
    c->f = NEW(double, K);
    c->F = NEW(double, K);
    c->fbuf1 = NEW(float, (c->D->maxK + 16) * 32);
    c->fbuf2 = NEW(float, (c->D->maxK + 16) * 32);
    for (int k = 0; k < K; ++k) { c->F[k] = c->P.pmeanf; c->f[k] = (1 - c->F[k]) / c->F[k]; }
    for (int k = 0; k < K; ++k)
        for (int64_t j = 0; j < KT; ++j) c->Freq[k * KT + j] = (float)c->Lambda[k];
    float* p = c->FreqA;
    double lambda = c->P.lambda;
    for (int64_t j = 0; j < KT; ++j) p[j] = (float)lambda;
    for (int64_t l = 0; l < c->L; ++l) {
        int k2 = c->D->k[l];
        const float* p2 = c->D->totfreq + c->D->off[l];
        int nhaplo = c->D->nhaplo[l];
        for (int a = 0; a < k2; ++a) p[a] = (float)((lambda + p2[a] * nhaplo) / (k2 * lambda + nhaplo));
        p += k2;
    }
}

void orc_init(orc_chain* c) {
    init_fix(c);
    init_admix(c);
    init_locpriori(c);
    init_fmodel(c);
}

/* Dirichlet(res, a, b, n): statistics.cpp:266-279, res float */
static void dirichlet_f_fi(orc_rng64* rng, float* res, const float* a, const int32_t* b, int n) {
    double s = 0;
    for (int i = 0; i < n; ++i) {
        double v = orc_rng64_gamma(rng, (double)a[i] + (double)b[i], 1);
        res[i] = (float)v;
        s += v;
    }
    float inv = (float)(1.0 / s);
    for (int i = 0; i < n; ++i) res[i] *= inv;
}
static void dirichlet_f_dl(orc_rng64* rng, float* res, const double* a, const int64_t* b, int n) {
    double s = 0;
    for (int i = 0; i < n; ++i) {
        double v = orc_rng64_gamma(rng, (double)a[i] + (double)b[i], 1);
        res[i] = (float)v;
        s += v;
    }
    float inv = (float)(1.0 / s);
    for (int i = 0; i < n; ++i) res[i] *= inv;
}
/* Dirichlet(res, a, n, f=1): statistics.cpp:253-264 */
static void dirichlet_f_d(orc_rng64* rng, float* res, const double* a, int n) {
    double s = 0;
    for (int i = 0; i < n; ++i) {
        double v = orc_rng64_gamma(rng, a[i] * 1.0, 1);
        res[i] = (float)v;
        s += v;
    }
    float inv = (float)(1.0 / s);
    for (int i = 0; i < n; ++i) res[i] *= inv;
}
static void dirichlet_f_f(orc_rng64* rng, float* res, const float* a, int n) {
    double s = 0;
    for (int i = 0; i < n; ++i) {
        double v = orc_rng64_gamma(rng, a[i] * 1.0, 1);
        res[i] = (float)v;
        s += v;
    }
    float inv = (float)(1.0 / s);
    for (int i = 0; i < n; ++i) res[i] *= inv;
}

/* UpdateP: structure.cpp:810-862 */
void orc_update_p(orc_chain* c) {
    int K = c->K; int64_t KT = c->KT, L = c->L;
    if (c->P.fmodel) {
        if (c->P.fsame) {
            float f0 = (float)c->f[0];
            for (int64_t j = 0; j < KT; ++j) c->Freq[j] = c->FreqA[j] * f0;
            for (int k = 1; k < K; ++k) memcpy(c->Freq + k * KT, c->Freq, KT * sizeof(float));
        } else
            for (int k = 0; k < K; ++k) {
                float fk = (float)c->f[k];
                for (int64_t j = 0; j < KT; ++j) c->Freq[k * KT + j] = c->FreqA[j] * fk;
            }
    } else
        for (int k = 0; k < K; ++k)
            for (int64_t j = 0; j < KT; ++j) c->Freq[k * KT + j] = (float)c->Lambda[k];
    for (int blockid = 0; blockid < 128; ++blockid) {
        int64_t kl_start = (int64_t)(blockid * K) * L / 128;
        int64_t kl_end = (int64_t)((blockid + 1) * K) * L / 128;
        orc_rng64 rng; orc_rng64_init(&rng, c->P.seed + (uint64_t)(c->m * 128 + blockid), SALT_UPDATEP);
        for (int64_t kl = kl_start; kl < kl_end; ++kl) {
            int64_t k = kl / L, l = kl % L;
            int32_t* ni = c->Ni + k * KT + c->D->off[l];
            float* p = FREQ(c, k, l);
            dirichlet_f_fi(&rng, p, p, ni, c->D->k[l]);
        }
    }
}

/* The locus loop of UpdateQNoAdmixCPU (structure.cpp:902-932) on bufNK1/2 */
static void qnoadmix_loglik(orc_chain* c) {
    int K = c->K, N = c->N; int64_t KT = c->KT;
    int64_t* sl = (int64_t*)c->bufNK1;
    double* pr = c->bufNK2;
    for (int64_t j = 0; j < (int64_t)N * K; ++j) { sl[j] = 0; pr[j] = 1; }
    if (c->P.locpriori)
        for (int i = 0; i < N; ++i) {
            if (c->D->vt[i] == 0) continue;
            const double* g = c->Gamma + c->D->popid[i] * K;
            for (int k = 0; k < K; ++k) orc_chargelog_d(&sl[i * K + k], &pr[i * K + k], g[k]);
        }
    for (int64_t ll = 0; ll < c->L; ++ll) {
        int64_t l = ll * c->D->coprime % c->L;
        const float* p = c->Freq + c->D->off[l];
        for (int i = 0; i < N; ++i) {
            int v = GC(c, l, i);
            if (!v) continue;
            const uint8_t* als = GA(c, l, i);
            for (int a = 0; a < v; ++a)
                for (int k = 0; k < K; ++k)
                    orc_chargelog_f(&sl[i * K + k], &pr[i * K + k], p[k * KT + als[a]]);
        }
    }
    for (int64_t j = 0; j < (int64_t)N * K; ++j) c->bufNK1[j] = orc_closelog(sl[j], pr[j]);
}

void orc_loglik_noadmix(orc_chain* c, double* out) {
    qnoadmix_loglik(c);
    memcpy(out, c->bufNK1, sizeof(double) * c->N * c->K);
}

/* UpdateQNoAdmixCPU: structure.cpp:864-933 */
void orc_update_q_noadmix(orc_chain* c) {
    int K = c->K, N = c->N;
    c->binaryq = 1;
    memset(c->Q, 0, sizeof(float) * N * K);
    qnoadmix_loglik(c);
    double* buf1 = c->bufNK1;
    float* q = c->Q;
    orc_rng64 rng; orc_rng64_init(&rng, c->P.seed + (uint64_t)c->m, SALT_UPDATEQ);
    for (int i = 0; i < N; ++i, buf1 += K, q += K) {
        if (c->D->vt[i] == 0) continue;
        uint16_t k2 = (uint16_t)orc_rng64_polylog(&rng, buf1, K);
        q[k2] = 1;
        c->Z[i] = k2;
    }
}

/* UpdateQAdmix: structure.cpp:984-1004 */
void orc_update_q_admix(orc_chain* c) {
    int K = c->K, N = c->N;
    c->binaryq = 0;
    orc_rng64 rng; orc_rng64_init(&rng, c->P.seed + (uint64_t)c->m, SALT_UPDATEQ);
    for (int i = 0; i < N; ++i) {
        if (!c->D->vt[i]) continue;
        const double* a = c->P.locpriori ? c->AlphaLocal + c->D->popid[i] * K : c->Alpha;
        dirichlet_f_dl(&rng, c->Q + i * K, a, c->Mi + i * K, K);
    }
}

/* UpdateQMetroCPU<fast_fp32 = true>: structure.cpp:1006-1086 */
void orc_update_q_metro(orc_chain* c) {
    int K = c->K, N = c->N; int64_t KT = c->KT;
    c->binaryq = 0;
    orc_rng64 rng; orc_rng64_init(&rng, c->P.seed + (uint64_t)c->m, SALT_UPDATEQ);
    float* prop = (float*)c->bufNK1;
    for (int i = 0; i < N; ++i) {
        if (c->D->vt[i] == 0) continue;
        const double* a = c->P.locpriori ? c->AlphaLocal + c->D->popid[i] * K : c->Alpha;
        dirichlet_f_d(&rng, prop + i * K, a, K);
    }
    int64_t* sl = (int64_t*)c->bufN1;
    double* pr = c->bufN2;
    for (int i = 0; i < N; ++i) { sl[i] = 0; pr[i] = 1; }
    for (int64_t ll = 0; ll < c->L; ++ll) {
        int64_t l = ll * c->D->coprime % c->L;
        const float* p = c->Freq + c->D->off[l];
        for (int i = 0; i < N; ++i) {
            int v = GC(c, l, i);
            if (!v) continue;
            const uint8_t* als = GA(c, l, i);
            const float *bi = prop + i * K, *q = c->Q + i * K;
            for (int a = 0; a < v; ++a) {
                /* SumProdDivx: math2.cpp:1632-1655 */
                float re1 = 0, re2 = 0;
                for (int k = 0; k < K; ++k) {
                    volatile float v1 = bi[k] * p[k * KT + als[a]];
                    volatile float v2 = q[k] * p[k * KT + als[a]];
                    re1 += v1; re2 += v2;
                }
                orc_chargelog_f(&sl[i], &pr[i], re1 / re2);
            }
        }
    }
    for (int i = 0; i < N; ++i) c->bufN1[i] = orc_closelog(sl[i], pr[i]);
    for (int i = 0; i < N; ++i) {
        if (c->D->vt[i] == 0) continue;
        if (c->bufN1[i] >= ORC_NZERO || orc_rng64_uniform(&rng, 0, 1) < exp(c->bufN1[i]))
            memcpy(c->Q + i * K, prop + i * K, K * sizeof(float));
    }
}

/* UpdateQ: structure.cpp:1138-1166 */
void orc_update_q(orc_chain* c) {
    int K = c->K;
    if (!c->P.admix) {
        if (c->m >= c->nadmburnin) orc_update_q_noadmix(c);
        else orc_update_q_admix(c);
        if (c->P.locpriori) {
            memset(c->Di, 0, sizeof(float) * c->S * K);
            for (int i = 0; i < c->N; ++i)
                if (c->D->vt[i]) {
                    float* di = c->Di + c->D->popid[i] * K;
                    for (int k = 0; k < K; ++k) di[k] += c->Q[i * K + k];
                }
        }
    } else {
        if (c->P.metrofreq > 0 && c->m % c->P.metrofreq == 0) orc_update_q_metro(c);
        else orc_update_q_admix(c);
    }
}

/* UpdateLocPriori: structure.cpp:1168-1255 */
void orc_update_locpriori(orc_chain* c) {
    if (!c->P.locpriori) return;
    int K = c->K, S = c->S;
    double r = c->r, epsr = c->P.epsr;
    orc_rng64 rng; orc_rng64_init(&rng, c->P.seed + (uint64_t)c->m, SALT_UPDATELOC);
    if (c->P.admix) {
        double rm = orc_rng64_uniform(&rng, r - epsr, r + epsr);
        if (rm > 0 && rm < c->P.maxr) {
            double dlnL = 0, d = rm - r, dt1 = rm * orc_mylog(rm) - r * orc_mylog(r);
            for (int k = 0; k < K; ++k) {
                dlnL += S * (c->Alpha[k] * dt1 - lgamma(rm * c->Alpha[k]) + lgamma(r * c->Alpha[k]));
                dlnL += c->Alpha[k] * d * orc_logprod_d(c->AlphaLocal + k, S, K) - orc_sum_d(c->AlphaLocal + k, S, K) * d;
            }
            if (dlnL >= ORC_NZERO || orc_rng64_uniform(&rng, 0, 1) < exp(dlnL)) c->r = rm;
        }
    } else {
        double rm = orc_rng64_uniform(&rng, r - epsr, r + epsr);
        if (rm > 0 && rm < c->P.maxr) {
            double dlnL = lgamma(rm) - lgamma(r);
            for (int k = 0; k < K; ++k) dlnL += lgamma(r * c->Eta[k]) - lgamma(rm * c->Eta[k]);
            dlnL *= S;
            for (int k = 0; k < K; ++k) dlnL += (rm - r) * c->Eta[k] * orc_logprod_d(c->Gamma + k, S, K);
            if (dlnL >= ORC_NZERO || orc_rng64_uniform(&rng, 0, 1) < exp(dlnL)) c->r = rm;
        }
        r = c->r;
        if (K >= 2) {
            int64_t i1 = (int64_t)orc_rng64_nextn(&rng, K), j1 = (int64_t)orc_rng64_nextavoid(&rng, K, i1);
            double delta = orc_rng64_uniform(&rng, 0, c->P.epseta);
            double e1 = c->Eta[i1] + delta, e2 = c->Eta[j1] - delta;
            if (e1 < 1 && e2 > 0) {
                double dlnL = S * (lgamma(r * c->Eta[i1]) + lgamma(r * c->Eta[j1]) - lgamma(r * e1) - lgamma(r * e2));
                dlnL += r * delta * orc_logproddiv_d(c->Gamma + i1, c->Gamma + j1, S, K);
                if (dlnL >= ORC_NZERO || orc_rng64_uniform(&rng, 0, 1) < exp(dlnL)) {
                    c->Eta[i1] += delta;
                    c->Eta[j1] -= delta;
                }
            }
        }
        if (K >= 2) {
            for (int s = 0; s < S; ++s) {
                int64_t i1 = (int64_t)orc_rng64_nextn(&rng, K), j1 = (int64_t)orc_rng64_nextavoid(&rng, K, i1);
                double delta = orc_rng64_uniform(&rng, 0, c->P.epsgamma);
                double* G = c->Gamma + s * K;
                if (G[i1] + delta < 1 && G[j1] - delta > 0) {
                    double dlnL = (r * c->Eta[i1] - 1.0 + c->Di[s * K + i1]) * orc_mylog(1 + delta / G[i1]) +
                                  (r * c->Eta[j1] - 1.0 + c->Di[s * K + j1]) * orc_mylog(1 - delta / G[j1]);
                    if (dlnL >= ORC_NZERO || orc_rng64_uniform(&rng, 0, 1) < exp(dlnL)) {
                        G[i1] += delta;
                        G[j1] -= delta;
                    }
                }
            }
        }
        if (c->m % 10 == 0) {
            orc_unify_d(c->Eta, K);
            for (int s = 0; s < S; ++s) orc_unify_d(c->Gamma + s * K, K);
        }
    }
}

/* UpdateZNoAdmixCPU: structure.cpp:1257-1301 */
void orc_update_z_noadmix(orc_chain* c) {
    int K = c->K, N = c->N; int64_t KT = c->KT;
    memset(c->Mi, 0, sizeof(int64_t) * N * K);
    memset(c->Ni, 0, sizeof(int32_t) * K * KT);
    for (int i = 0; i < N; ++i) c->Mi[i * K + c->Z[i]] = c->D->vt[i];
    for (int64_t l = 0; l < c->L; ++l) {
        int64_t o = c->D->off[l];
        for (int i = 0; i < N; ++i) {
            int v = GC(c, l, i);
            if (!v) continue;
            const uint8_t* als = GA(c, l, i);
            int32_t* ni = c->Ni + (int64_t)c->Z[i] * KT + o;
            for (int a = 0; a < v; ++a) ni[als[a]]++;
        }
    }
}

/* UpdateZAdmixCPU<fast_fp32 = true>: structure.cpp:1350-1438 */
void orc_update_z_admix(orc_chain* c) {
    int K = c->K, N = c->N; int64_t KT = c->KT, L = c->L;
    int maxploidy = c->D->maxploidy;
    memset(c->Mi, 0, sizeof(int64_t) * N * K);
    memset(c->Ni, 0, sizeof(int32_t) * K * KT);
    float* bufk = c->bufK;
    for (int64_t ll = 0; ll < L; ++ll) {
        int64_t l = ll * c->D->coprime % L;
        int64_t o = c->D->off[l];
        orc_rng32 rng; orc_rng32_init(&rng, c->P.seed + (uint64_t)((int64_t)c->m * L + l), SALT_UPDATEZ);
        int64_t* mi = c->Mi;
        const float* q = c->Q;
        for (int i = 0; i < N; ++i, mi += K, q += K) {
            int ploidy = GC(c, l, i);
            const uint8_t* als = GA(c, l, i);
            for (int a = 0; a < maxploidy; ++a) {
                if (a >= ploidy) { orc_rng32_next(&rng); continue; }
                if (a == 0 || als[a] != als[a - 1])
                    for (int k = 0; k < K; ++k) bufk[k] = q[k] * c->Freq[k * KT + o + als[a]];
                uint16_t k2 = (uint16_t)orc_rng32_poly(&rng, bufk, K);
                mi[k2]++;
                c->Ni[k2 * KT + o + als[a]]++;
            }
        }
    }
}

void orc_update_z(orc_chain* c) {
    if (c->binaryq) orc_update_z_noadmix(c);
    else orc_update_z_admix(c);
}

/* UpdateAlpha: structure.cpp:1499-1594 */
void orc_update_alpha(orc_chain* c) {
    int K = c->K, N = c->N, S = c->S;
    orc_rng64 rng; orc_rng64_init(&rng, c->P.seed + (uint64_t)c->m, SALT_UPDATEALPHA);
    const orc_params* P = &c->P;
    if (P->locpriori && P->admix) {
        double r = c->r;
        for (int k = 0; k < K; ++k) {
            double am = orc_rng64_normal(&rng, c->Alpha[k], P->stdalpha);
            if (am > 0 && am < P->maxalpha) {
                double d = am - c->Alpha[k];
                double dlnL = S * (d * r * orc_mylog(r) + lgamma(r * c->Alpha[k]) - lgamma(r * am));
                dlnL += r * d * orc_logprod_d(c->AlphaLocal + k, S, K);
                if (dlnL >= ORC_NZERO || orc_rng64_uniform(&rng, 0, 1) < exp(dlnL)) c->Alpha[k] = am;
            }
        }
        if (c->m % 10 == 0)
            for (int s = 0; s < S; ++s) c->SumAlpha[s] = orc_sum_d(c->AlphaLocal + s * K, K, 1);
        for (int s = 0; s < S; ++s) {
            int snind = c->D->pop_nind[s];
            const float* sq = c->Q + (int64_t)c->D->pop_ind0[s] * K;
            for (int k = 0; k < K; ++k) {
                double ao = c->AlphaLocal[s * K + k], am = orc_rng64_normal(&rng, ao, P->stdalpha);
                if (am > 0 && am < P->maxalpha) {
                    double d = am - ao;
                    double dlnL = (r * c->Alpha[k] - 1) * orc_mylog(am / ao) - d * r +
                        snind * (lgamma(c->SumAlpha[s] + d) - lgamma(am) - lgamma(c->SumAlpha[s]) + lgamma(ao));
                    dlnL += d * orc_logprod_f(sq + k, snind, K);
                    if (dlnL >= ORC_NZERO || orc_rng64_uniform(&rng, 0, 1) < exp(dlnL)) {
                        c->AlphaLocal[s * K + k] = am;
                        c->SumAlpha[s] += d;
                    }
                }
            }
        }
    } else if (P->inferalpha) {
        if (!P->admix && c->m >= c->nadmburnin) return;
        if (P->diffalpha) {
            double sumalpha = 0;
            for (int k = 0; k < K; ++k) sumalpha += c->Alpha[k];
            for (int k = 0; k < K; ++k) {
                double am = orc_rng64_normal(&rng, c->Alpha[k], P->stdalpha);
                if (am <= 0 || (am >= P->maxalpha && P->uniformalpha)) continue;
                double ao = c->Alpha[k], d = am - ao;
                double dlnL = P->uniformalpha ? 0 : ((P->alphapriora - 1) * orc_mylog(am / ao) + (ao - am) / P->alphapriorb);
                dlnL += (am - ao) * orc_logprod_f(c->Q + k, N, K) +
                        (lgamma(sumalpha + d) - lgamma(sumalpha) - lgamma(am) + lgamma(ao)) * N;
                if (dlnL >= ORC_NZERO || orc_rng64_uniform(&rng, 0, 1) < exp(dlnL)) c->Alpha[k] = am;
            }
        } else {
            double am = orc_rng64_normal(&rng, c->Alpha[0], P->stdalpha);
            if (am <= 0 || (am >= P->maxalpha && P->uniformalpha)) return;
            double ao = c->Alpha[0];
            double dlnL = P->uniformalpha ? 0 : ((P->alphapriora - 1) * orc_mylog(am / ao) + (ao - am) / P->alphapriorb);
            dlnL += (am - ao) * orc_logprod_f(c->Q, (int64_t)N * K, 1) +
                    (lgamma(K * am) - lgamma(K * ao) - K * lgamma(am) + K * lgamma(ao)) * N;
            if (dlnL >= ORC_NZERO || orc_rng64_uniform(&rng, 0, 1) < exp(dlnL))
                for (int k = 0; k < K; ++k) c->Alpha[k] = am;
        }
    }
}

/* UpdateA1: structure.cpp:1646-1695 */
static void update_a1(orc_chain* c) {
    int K = c->K; int64_t L = c->L, KT = c->KT;
    int maxK = c->D->maxK;
    double lam = c->Lambda[0];
    for (int blockid = 0; blockid < 32; ++blockid) {
        int64_t l_start = blockid * L / 32, l_end = (blockid + 1) * L / 32;
        orc_rng64 rng; orc_rng64_init(&rng, c->P.seed + (uint64_t)(c->m * 32 + blockid), SALT_UPDATEA);
        for (int64_t l = l_start; l < l_end; ++l) {
            int k2 = c->D->k[l];
            float* pa = c->FreqA + c->D->off[l];
            float* pb = c->fbuf1 + (maxK + 16) * blockid;
            float* pc = c->fbuf2 + (maxK + 16) * blockid;
            for (int a = 0; a < k2; ++a) pb[a] = (float)lam;
            for (int k = 0; k < K; ++k) {
                const float* pk = FREQ(c, k, l);
                float fk = (float)c->f[k];
                for (int a = 0; a < k2; ++a) pb[a] += pk[a] * fk;
            }
            dirichlet_f_f(&rng, pc, pb, k2);
            double dlnL = 0;
            for (int a = 0; a < k2; ++a) dlnL += (pb[a] - lam) * (orc_mylog(pa[a] / pc[a]));
            for (int k = 0; k < K; ++k) {
                const float* pk = FREQ(c, k, l);
                double fr = c->f[k];
                for (int a = 0; a < k2; ++a)
                    dlnL += lgamma(fr * pa[a]) - lgamma(fr * pc[a]) + fr * (pc[a] - pa[a]) * orc_mylog(pk[a]);
            }
            if (dlnL >= ORC_NZERO || orc_rng64_uniform(&rng, 0, 1) < exp(dlnL))
                memcpy(pa, pc, k2 * sizeof(float));
        }
    }
    (void)KT;
}

/* UpdateA2: structure.cpp:1745-1804 */
static void update_a2(orc_chain* c) {
    int K = c->K; int64_t L = c->L, KT = c->KT;
    double lam = c->Lambda[0];
    for (int blockid = 0; blockid < 32; ++blockid) {
        int64_t l_start = blockid * L / 32, l_end = (blockid + 1) * L / 32;
        orc_rng64 rng; orc_rng64_init(&rng, c->P.seed + (uint64_t)(c->m * 32 + blockid), SALT_UPDATEA);
        if (l_start >= l_end) continue;
        int64_t lo = c->D->off[l_start];
        float* pa = c->FreqA + lo;
        const float* p = c->Freq + lo;
        for (int64_t l = l_start; l < l_end; ++l) {
            int k2 = c->D->k[l];
            int m1 = (int)orc_rng64_nextn(&rng, k2), n1 = (int)orc_rng64_nextavoid(&rng, k2, m1);
            double delta = orc_rng64_uniform(&rng, 0, pow(c->N, -0.5));
            double pm0 = pa[m1], pm1 = pm0 + delta, pn0 = pa[n1], pn1 = pn0 - delta;
            /* the reference advances pa but not p on this path (structure.cpp:1770-1774) */
            if (pm1 >= 1 || pn1 <= 0) { pa += k2; continue; }
            double dlnL = (lam - 1) * orc_mylog(pm1 * pn1 / pm0 / pn0);
            for (int k = 0; k < K; ++k) {
                double fr = c->f[k];
                dlnL += lgamma(fr * pm0) + lgamma(fr * pn0) - lgamma(fr * pm1) - lgamma(fr * pn1) +
                        (fr * delta) * orc_mylog(p[k * KT + m1] / p[k * KT + n1]);
            }
            if (dlnL >= ORC_NZERO || orc_rng64_uniform(&rng, 0, 1) < exp(dlnL)) {
                pa[m1] = (float)pm1;
                pa[n1] = (float)pn1;
            }
            p += k2; pa += k2;
        }
    }
}

/* UpdateA: structure.cpp:1637-1644 */
void orc_update_a(orc_chain* c) {
    if (!c->P.fmodel) return;
    if (orc_hash_ulong(c->P.seed + (uint64_t)c->m) & 1) update_a1(c);
    else update_a2(c);
}

/* UpdateF: structure.cpp:1806-1858 */
void orc_update_f(orc_chain* c) {
    if (!c->P.fmodel) return;
    int K = c->K; int64_t KT = c->KT;
    const orc_params* P = &c->P;
    orc_rng64 rng; orc_rng64_init(&rng, c->P.seed + (uint64_t)c->m, SALT_UPDATEF);
    for (int k = 0; k < K; ++k) {
        double Fo = c->F[k];
        double Fm = orc_rng64_normal(&rng, Fo, P->stdf);
        if (Fm < 0 || Fm > 1) { if (P->fsame) break; else continue; }
        double fo = c->f[k], fm = (1 - Fm) / Fm;
        double dlnL = P->pmeanf * (Fo - Fm) / (P->pstdf * P->pstdf) +
                      (P->pmeanf * P->pmeanf / (P->pstdf * P->pstdf) - 1) * orc_mylog(Fm / Fo) +
                      (P->fsame ? K : 1) * c->L * (lgamma(fm) - lgamma(fo));
        for (int k2 = k; k2 < K; ++k2) {
            const float* p = c->Freq + k2 * KT;
            const float* pa = c->FreqA;
            for (int64_t a = 0; a < KT; ++a) {
                float pa2 = *pa++;
                dlnL += pa2 * (fm - fo) * orc_mylog(*p++) + lgamma(fo * pa2) - lgamma(fm * pa2);
            }
            if (!P->fsame) break;
        }
        if (dlnL >= ORC_NZERO || orc_rng64_uniform(&rng, 0, 1) < exp(dlnL)) {
            if (P->fsame) { for (int j = 0; j < K; ++j) { c->F[j] = Fm; c->f[j] = fm; } }
            else { c->F[k] = Fm; c->f[k] = fm; }
        }
        if (P->fsame) break;
    }
}

/* RecordCPU likelihood (structure.cpp:1902-1938), fast_fp32 */
double orc_record_lnl(orc_chain* c) {
    int K = c->K, N = c->N; int64_t KT = c->KT;
    int64_t slog = 0; double prod = 1;
    for (int64_t ll = 0; ll < c->L; ++ll) {
        int64_t l = ll * c->D->coprime % c->L;
        const float* p = c->Freq + c->D->off[l];
        const float* q = c->Q;
        for (int i = 0; i < N; ++i, q += K) {
            int v = GC(c, l, i);
            if (!v) continue;
            const uint8_t* als = GA(c, l, i);
            const float* pp = p + KT * c->Z[i];
            for (int a = 0; a < v; ++a) {
                if (!c->binaryq) {
                    float re = 0;       /* SumProdx: math2.cpp:1700-1720 */
                    for (int k = 0; k < K; ++k) { volatile float v1 = q[k] * p[k * KT + als[a]]; re += v1; }
                    orc_chargelog_f(&slog, &prod, re);
                } else
                    orc_chargelog_f(&slog, &prod, pp[als[a]]);
            }
        }
    }
    return 0.0 + orc_closelog(slog, prod);
}

/* Record: structure.cpp:1941-2045 */
void orc_record(orc_chain* c) {
    int m = c->m, K = c->K;
    if ((c->P.writelnl && m < c->nburnin && m % c->nthinning == 0) ||
        (m >= c->nburnin && (m - c->nburnin) % c->nthinning == 0)) {
        for (int64_t j = 0; j < (int64_t)c->N * K; ++j) c->MiSum[j] += c->Mi[j];
        double like = orc_record_lnl(c);
        if (c->P.writelnl) c->lnL[c->nlnL++] = like;
        if (m >= c->nburnin) {
            c->nr++;
            c->rout[0] += like;
            c->rout[1] += like * like;
            int nf = c->P.fmodel ? (c->P.fsame ? 1 : K) : 0;
            int na = c->P.admix ? (c->P.diffalpha ? K : 1) : 0;
            int nl = c->P.difflambda ? K : 1;
            for (int j = 0; j < nl; ++j) c->rout[4 + j] += c->Lambda[j];
            if (c->P.locpriori) {
                c->rout[4 + nl] += c->r;
                const double* g = c->P.admix ? c->Alpha : c->Eta;
                for (int j = 0; j < K; ++j) c->rout[4 + nl + 1 + j] += g[j];
                const double* gl = c->P.admix ? c->AlphaLocal : c->Gamma;
                for (int j = 0; j < K * c->S; ++j) c->rout[4 + nl + 1 + K + j] += gl[j];
            } else if (c->P.admix)
                for (int j = 0; j < na; ++j) c->rout[4 + nl + j] += c->Alpha[j];
            for (int j = 0; j < nf; ++j) c->rout[c->rlen - nf + j] += c->F[j];
            for (int64_t j = 0; j < K * c->KT; ++j) c->FreqM[j] += c->Freq[j];
        }
    }
}

void orc_sweep(orc_chain* c) {
    orc_update_p(c);
    orc_update_q(c);
    orc_update_locpriori(c);
    orc_update_z(c);
    orc_update_alpha(c);
    orc_update_a(c);
    orc_update_f(c);
    orc_record(c);
    c->m++;
}

/* Arrange: structure.cpp:1860-1869 */
void orc_arrange(orc_chain* c) {
    int K = c->K, N = c->N;
    double* ms = (double*)c->MiSum;
    for (int64_t j = 0; j < (int64_t)N * K; ++j) ms[j] = (double)c->MiSum[j];
    for (int i = 0; i < N; ++i) orc_unify_d(ms + i * K, K);
    double inv = 1.0 / c->nr;
    for (int j = 0; j < c->rlen; ++j) c->rout[j] *= inv;
    c->rout[2] = c->rout[1] - c->rout[0] * c->rout[0];
    c->rout[3] = c->rout[0] - c->rout[2] / 2;
    float finv = (float)(1.0 / c->nr);
    for (int64_t j = 0; j < K * c->KT; ++j) c->FreqM[j] *= finv;
}

void orc_run(orc_chain* c) {
    orc_init(c);
    for (c->m = 0; c->m < c->nburnin + c->nreps;) orc_sweep(c);
    orc_arrange(c);
}

/* ================= output (structure.cpp:86-377) ================= */

static char g_fmt[16];
static void wr(FILE* f, double v) {
    if (isnan(v) || isinf(v)) fprintf(f, "nan");
    else fprintf(f, g_fmt, v);
}

int orc_write_structure(orc_chain* c, const char* prefix, int rep, int id,
                        const char* const* ind_names, const char* const* pop_names,
                        const char* const* loc_names, int decimal, int diversity) {
    const char* LB = "\r\n";
    char D = '\t';
    char fn[8192];
    int K = c->K, N = c->N, S = c->S; int64_t L = c->L;
    snprintf(g_fmt, sizeof g_fmt, "%%0.%df", decimal);
    if (c->P.writelnl) {
        snprintf(fn, sizeof fn, "%s.structure.k=%d_rep=%d_id=%d.lnl.txt", prefix, K, rep, id);
        FILE* f = fopen(fn, "wb");
        if (!f) return -1;
        fprintf(f, "%d%s", c->nburnin, LB);
        fprintf(f, "Iteration%clnL%s", D, LB);
        double* lnl = c->lnL;
        for (int i = 0; i < c->nburnin; i += c->nthinning) { fprintf(f, "%d%c", i, D); wr(f, *lnl++); fprintf(f, "%s", LB); }
        for (int i = 0; i < c->nreps; i += c->nthinning) { fprintf(f, "%d%c", i + c->nburnin, D); wr(f, *lnl++); fprintf(f, "%s", LB); }
        fclose(f);
    }
    snprintf(fn, sizeof fn, "%s.structure.k=%d_rep=%d_id=%d.txt", prefix, K, rep, id);
    FILE* f = fopen(fn, "wb");
    if (!f) return -1;
    fprintf(f, "%s%sParameters:%s", LB, LB, LB);
    fprintf(f, "Seed=%lld%s", (long long)c->P.seed, LB);
    fprintf(f, "Model=%s,%s,%s%s", c->P.admix ? "ADM" : "NOADM", c->P.locpriori ? "LOC" : "NOLOC", c->P.fmodel ? "F" : "NOF", LB);
    fprintf(f, "Number of cluster=%d%s", K, LB);
    fprintf(f, "Replicate=%d%s", rep, LB);
    fprintf(f, "Run id=%d%s", id, LB);
    fprintf(f, "Mean value of ln likelihood="); wr(f, c->rout[0]); fprintf(f, "%s", LB);
    fprintf(f, "Variance of ln likelihood="); wr(f, c->rout[2]); fprintf(f, "%s", LB);
    fprintf(f, "Estimated Ln Prob of Data="); wr(f, c->rout[3]); fprintf(f, "%s%s", LB, LB);
    int nf = c->P.fmodel ? (c->P.fsame ? 1 : K) : 0;
    int nl = c->P.difflambda ? K : 1;
    if (c->P.locpriori) {
        fprintf(f, "%sMean value of r=", LB); wr(f, c->rout[4 + nl]);
        fprintf(f, "%sMean value of global %s", LB, c->P.admix ? "alpha" : "eta");
        fprintf(f, "%s%cCluster%s", LB, D, LB);
        for (int j = 0; j < K; ++j) fprintf(f, "%c%d", D, j + 1);
        fprintf(f, "%s", LB);
        for (int j = 0; j < K; ++j) { fprintf(f, "%c", D); wr(f, c->rout[4 + nl + 1 + j]); }
        fprintf(f, "%sMean value of local %s for each location", LB, c->P.admix ? "alpha" : "gamma");
        fprintf(f, "%s%cCluster%sPop", LB, D, LB);
        for (int j = 0; j < K; ++j) fprintf(f, "%c%d", D, j + 1);
        for (int i = 0; i < S; ++i) {
            fprintf(f, "%s%s", LB, pop_names[i]);
            for (int j = 0; j < K; ++j) { fprintf(f, "%c", D); wr(f, c->rout[4 + nl + 1 + K + i * K + j]); }
        }
    } else if (c->P.admix && c->P.inferalpha) {
        if (!c->P.diffalpha) { fprintf(f, "%sMean value of alpha=", LB); wr(f, c->rout[4 + nl]); }
        else for (int j = 0; j < K; ++j) { fprintf(f, "%sMean value of alpha_%d=", LB, j + 1); wr(f, c->rout[4 + nl + j]); }
    }
    if (c->P.fmodel) {
        if (c->P.fsame) { fprintf(f, "%sMean value of Fst=", LB); wr(f, c->rout[c->rlen - 1]); }
        else {
            fprintf(f, "%sMean value of Fst", LB);
            fprintf(f, "%s%cCluster%s", LB, D, LB);
            for (int j = 0; j < K; ++j) fprintf(f, "%c%d", D, j + 1);
            fprintf(f, "%s", LB);
            for (int i = 0; i < nf; ++i) { fprintf(f, "%c", D); wr(f, c->rout[c->rlen - nf + i]); }
        }
    }
    float* O = NEW(float, S * K);
    fprintf(f, "%s%sProportion of membership of each pre-defined population in each of the %d clusters", LB, LB, K);
    fprintf(f, "%s%cCluster%sPop", LB, D, LB);
    for (int i = 0; i < N; ++i)
        for (int k = 0; k < K; ++k) O[c->D->popid[i] * K + k] += c->Q[i * K + k];
    for (int s = 0; s < S; ++s) orc_unify_f(O + s * K, K);
    for (int k = 0; k < K; ++k) fprintf(f, "%c%d", D, k + 1);
    for (int s = 0; s < S; ++s) {
        fprintf(f, "%s%s", LB, pop_names[s]);
        for (int k = 0; k < K; ++k) { fprintf(f, "%c", D); wr(f, O[s * K + k]); }
    }
    fprintf(f, "%s%sInferred ancestry of individuals", LB, LB);
    fprintf(f, "%s%c%cCluster", LB, D, D);
    fprintf(f, "%sInd%cPop%cRegL1", LB, D, D);
    for (int j = 0; j < K; ++j) fprintf(f, "%c%d", D, j + 1);
    const double* ms = (const double*)c->MiSum;
    for (int i = 0; i < N; ++i) {
        fprintf(f, "%s%s%c%s%c%s", LB, ind_names[i], D, pop_names[c->D->popid[i]], D, "Total");
        for (int k = 0; k < K; ++k) { fprintf(f, "%c", D); wr(f, ms[i * K + k]); }
    }
    free(O);
    double* H = NEW(double, K);
    double* Dm = NEW(double, K * K);
    double* H2 = NEW(double, K * L);
    for (int k = 0; k < K; ++k) {
        const float* p = c->FreqM + k * c->KT;
        for (int64_t l = 0; l < L; ++l) {
            int k2 = c->D->k[l];
            double ss = 0;
            for (int a = 0; a < k2; ++a) ss += (double)p[a] * (double)p[a];
            double h = 1 - ss;
            H2[k * L + l] = h;
            H[k] += h;
            p += k2;
        }
        H[k] /= L;
        for (int j = 0; j <= k; ++j) {
            const float *p1 = c->FreqM + k * c->KT, *p2 = c->FreqM + j * c->KT;
            double dt = 0;
            for (int64_t l = 0; l < L; ++l) {
                int k2 = c->D->k[l];
                double sp = 0;
                for (int a = 0; a < k2; ++a) sp += (double)p1[a] * (double)p2[a];
                dt += 1 - sp;
                p1 += k2; p2 += k2;
            }
            Dm[j * K + k] = Dm[k * K + j] = dt / L - (H[k] + H[j]) / 2;
        }
    }
    fprintf(f, "%s%sAllele-frequency divergence among pops (Net nucleotide distance)", LB, LB);
    fprintf(f, "%s%cCluster%sCluster", LB, D, LB);
    for (int j = 0; j < K; ++j) fprintf(f, "%c%d", D, j + 1);
    for (int i = 0; i < K; ++i) {
        fprintf(f, "%s%d", LB, i + 1);
        for (int j = 0; j < K; ++j) { fprintf(f, "%c", D); wr(f, Dm[i * K + j]); }
    }
    if (diversity) {
        fprintf(f, "%s%sEstimated genetic diversity in each cluster", LB, LB);
        fprintf(f, "%sLocus%cCluster%cHeterozygosity", LB, D, D);
        for (int a = 0; a < c->D->maxK; ++a) fprintf(f, "%cAllele%d", D, a);
        for (int k = 0; k < K; ++k) {
            fprintf(f, "%s%s%c%d", LB, k ? "" : "Average", D, k + 1);
            wr(f, H[k]);
        }
        for (int64_t l = 0; l < L; ++l)
            for (int k = 0; k < K; ++k) {
                fprintf(f, "%s%s%c%d%c", LB, k ? "" : loc_names[l], D, k + 1, D);
                wr(f, H2[k * L + l]);
                const float* p = c->FreqM + k * c->KT + c->D->off[l];
                for (int a = 0; a < c->D->k[l]; ++a) { fprintf(f, "%c", D); wr(f, p[a]); }
            }
    }
    free(H); free(Dm); free(H2);
    fclose(f);
    return 0;
}

/* ================= test access ================= */
void* orc_field(orc_chain* c, int f, int64_t* n) {
    int64_t K = c->K, N = c->N, KT = c->KT, S = c->S;
    switch (f) {
        case 1: *n = K * KT; return c->Freq;
        case 2: *n = N * K; return c->Q;
        case 3: *n = N; return c->Z;
        case 4: *n = K * KT; return c->Ni;
        case 5: *n = N * K; return c->Mi;
        case 6: *n = N * K; return c->bufNK1;
        case 7: *n = K; return c->Alpha;
        case 10: *n = KT; return c->FreqA;
        case 11: *n = c->f ? K : 0; return c->f;
        case 12: *n = c->F ? K : 0; return c->F;
        case 13: *n = c->Di ? S * K : 0; return c->Di;
        case 14: *n = N; return c->bufN1;
        case 15: *n = c->Eta ? K : 0; return c->Eta;
        case 16: *n = c->Gamma ? S * K : 0; return c->Gamma;
        case 17: *n = c->AlphaLocal ? S * K : 0; return c->AlphaLocal;
        case 18: *n = c->SumAlpha ? S : 0; return c->SumAlpha;
        case 19: *n = c->rlen; return c->rout;
        case 20: *n = c->nlnL; return c->lnL;
        case 21: *n = N * K; return c->MiSum;
        case 22: *n = K * KT; return c->FreqM;
    }
    *n = 0;
    return NULL;
}
int32_t* orc_m(orc_chain* c) { return &c->m; }
int32_t* orc_nlnl(orc_chain* c) { return &c->nlnL; }
double* orc_r(orc_chain* c) { return &c->r; }
int32_t* orc_binaryq(orc_chain* c) { return &c->binaryq; }
const void* orc_data_field(const orc_data* d, int f, int64_t* n) {
    switch (f) {
        case 1: *n = d->L; return d->k;
        case 2: *n = d->L; return d->off;
        case 3: *n = d->N; return d->vt;
        case 4: *n = d->L * d->N; return d->gcopies;
        case 5: *n = d->L * d->N * d->vmax; return d->galleles;
    }
    *n = 0;
    return 0;
}

/* ================= multi-chain runner (baseline timing) ================= */
typedef struct { orc_chain** cs; int n, nsweeps, init; int next; pthread_mutex_t mu; } orc_pool;
static void* orc_worker(void* arg) {
    orc_pool* p = (orc_pool*)arg;
    for (;;) {
        pthread_mutex_lock(&p->mu);
        int j = p->next++;
        pthread_mutex_unlock(&p->mu);
        if (j >= p->n) break;
        if (p->init) orc_init(p->cs[j]);
        for (int s = 0; s < p->nsweeps; ++s) orc_sweep(p->cs[j]);
    }
    return NULL;
}
void orc_sweep_many(orc_chain** cs, int n, int nsweeps, int nthreads, int init) {
    orc_pool p;
    p.cs = cs; p.n = n; p.nsweeps = nsweeps; p.init = init; p.next = 0;
    pthread_mutex_init(&p.mu, NULL);
    if (nthreads < 1) nthreads = 1;
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * nthreads);
    for (int t = 0; t < nthreads; ++t) pthread_create(&th[t], NULL, orc_worker, &p);
    for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
    free(th);
    pthread_mutex_destroy(&p.mu);
}

/* structure.cpp:293-324: per-locus 1 - SumSquare, and 1 - SumProd summed over
 * loci for every pair, both in double from float frequencies */
void orc_divergence(const float* freqm, const int32_t* k, int64_t L, int64_t KT, int K, double* H, double* D,
                    double* Hl) {
    for (int a = 0; a < K; ++a) {
        const float* p = freqm + a * KT;
        H[a] = 0;
        for (int64_t l = 0; l < L; ++l) {
            double ss = 0;
            for (int b = 0; b < k[l]; ++b) ss += (double)p[b] * (double)p[b];
            if (Hl) Hl[a * L + l] = 1 - ss;
            H[a] += 1 - ss;
            p += k[l];
        }
        H[a] /= L;
        for (int j = 0; j <= a; ++j) {
            const float *p1 = freqm + a * KT, *p2 = freqm + j * KT;
            double dt = 0;
            for (int64_t l = 0; l < L; ++l) {
                double sp = 0;
                for (int b = 0; b < k[l]; ++b) sp += (double)p1[b] * (double)p2[b];
                dt += 1 - sp;
                p1 += k[l];
                p2 += k[l];
            }
            D[j * K + a] = D[a * K + j] = dt / L - (H[a] + H[j]) / 2;
        }
    }
}

/* load.cpp AddVCFGenotype for biallelic diploid calls: one line at a time,
 * fields split at tabs, the GT part of each sample field split at '/' or '|' */
/* ReadIntegerKeep (string2.cpp:711-727): characters up to the first digit
 * or '-' are skipped, then digits are read (int arithmetic, wrapping). The
 * reference's scan has no end; this one stops at `end` with what it read. */
static int read_integer_keep(const char* p, const char* end) {
    int c, sign = 0;
    unsigned x = 0;
    for (c = p < end ? *p : 0, ++p; c < '0' || c > '9'; c = p < end ? *p : 0, ++p) {
        if (p > end) return 0;
        if (c == '-') {
            sign = 1;
            c = p < end ? *p : 0;
            ++p;
            break;
        }
    }
    for (; c >= '0' && c <= '9'; c = p < end ? *p : 0, ++p) x = (x << 1) + (x << 3) + (unsigned)(c - '0');
    return sign ? -(int)x : (int)x;
}

int orc_call_filtered(char* call, size_t room, int dpid, int gqid, int v, const orc_call_filter* cf) {
    char* end = call + room;
    /* AddVCFGenotype: count this call's keys, splitting them into '\0' */
    int fmtc = 0;
    for (char* q = call;;) {
        fmtc++;
        while (q < end && *q != ':' && *q != '\t' && *q != '\n' && *q != 0) q++;
        if (q < end && *q == ':') *q++ = 0;
        else {
            if (q < end) *q = 0;
            break;
        }
    }
    /* GetTagValue (load.cpp:3596-3602): past `id` terminators */
#define TAG(id, out)                                        \
    do {                                                    \
        char* r_ = call;                                    \
        for (int i_ = 0; i_ < (id); ++i_) while (*r_++) {}  \
        (out) = r_;                                         \
    } while (0)
    if (cf->dp_b && dpid >= 0 && dpid < fmtc) {
        char* t;
        TAG(dpid, t);
        const unsigned dp = (unsigned)read_integer_keep(t, end);
        if (dp != (unsigned)-1 && (dp < (unsigned)cf->dp_min || dp > (unsigned)cf->dp_max)) return 1;
    }
    if (cf->gq_b && gqid >= 0 && gqid < fmtc) {
        char* t;
        TAG(gqid, t);
        const int gq = read_integer_keep(t, end);
        if (gq != -1 && (gq < cf->gq_min || gq > cf->gq_max)) return 1;
    }
#undef TAG
    if (cf->ploidy_b && (v < cf->ploidy_min || v > cf->ploidy_max)) return 1;
    return 0;
}

size_t orc_rewrite_calls(const char* fmt, const char* fmt_end, const char* calls, const char* end, int n,
                         char* out, size_t* call_at, int* dpid, int* gqid) {
    /* FORMAT keys: kept when two bytes GT, DP or GQ then ':' or the tab */
    int kept[1024], nk = 0, nkept = 0;
    *dpid = *gqid = -1;
    for (const char* k = fmt; k <= fmt_end && nk < 1024;) {
        const char* ke = k;
        while (ke < fmt_end && *ke != ':') ++ke;
        const int two = ke - k == 2;
        const int gt = two && k[0] == 'G' && k[1] == 'T', dp = two && k[0] == 'D' && k[1] == 'P',
                  gq = two && k[0] == 'G' && k[1] == 'Q';
        kept[nk++] = gt || dp || gq;
        /* LOCUS::GetFormatId on the rewritten keys: the first DP, the first GQ */
        if (dp && *dpid < 0) *dpid = nkept;
        if (gq && *gqid < 0) *gqid = nkept;
        nkept += gt || dp || gq;
        if (ke >= fmt_end) break;
        k = ke + 1;
    }
    /* each call: the values of the kept keys, joined by ':'; calls by tabs */
    size_t o = 0;
    const char* c = calls;
    for (int i = 0; i < n && c <= end; ++i) {
        call_at[i] = o;
        int writed = 0;
        for (int j = 0; j < nk; ++j) {
            const char* v = c;
            while (c < end && *c != ':' && *c != '\t') ++c;
            if (kept[j]) {
                if (writed) out[o++] = ':';
                memcpy(out + o, v, (size_t)(c - v));
                o += (size_t)(c - v);
            }
            if (c >= end || *c == '\t') break;
            ++c;
            if (kept[j]) writed = 1;
        }
        while (c < end && *c != '\t') ++c;      /* keys beyond FORMAT */
        ++c;
        if (i + 1 < n) out[o++] = '\t';
    }
    out[o] = 0;
    return o;
}

int64_t orc_vcf_pack2(const char* text, size_t bytes, int n_ind, uint32_t* packed, int64_t max_loci) {
    return orc_vcf_pack2_ex(text, bytes, n_ind, packed, max_loci, NULL);
}

int64_t orc_vcf_pack2_ex(const char* text, size_t bytes, int n_ind, uint32_t* packed, int64_t max_loci,
                         const orc_call_filter* cf) {
    const int filter = cf && (cf->dp_b || cf->gq_b || cf->ploidy_b);
    char* copy = NULL;
    size_t copy_cap = 0;
    const int Nw = (n_ind + 15) / 16;
    const char* p = text;
    const char* end = text + bytes;
    int64_t l = 0;
    while (p < end) {
        const char* e = memchr(p, '\n', (size_t)(end - p));
        const char* le = e ? e : end;
        if (le > p && le[-1] == '\r') --le;
        if (l >= max_loci) { free(copy); return -(l + 1); }
        uint32_t* row = packed + l * Nw;
        memset(row, 0, (size_t)Nw * 4);
        int field = 0, nalt = 0, dpid = -1, gqid = -1;
        size_t* call_at = NULL;
        size_t rw_len = 0;
        if (filter) {   /* the loader's rewritten calls, for the in-place key split and the value scans */
            const char* fmt = p;
            for (int c = 0; c < 8 && fmt < le; ++c) { fmt = memchr(fmt, '\t', (size_t)(le - fmt)); if (!fmt) break; ++fmt; }
            const char* fe = fmt ? memchr(fmt, '\t', (size_t)(le - fmt)) : NULL;
            if (!fmt || !fe) { free(copy); return -(l + 1); }
            const size_t n = (size_t)(le - p);
            if (n + 1 > copy_cap) { copy_cap = 2 * (n + 1); copy = realloc(copy, copy_cap); }
            call_at = malloc(sizeof(size_t) * (size_t)n_ind);
            rw_len = orc_rewrite_calls(fmt, fe, fe + 1, le, n_ind, copy, call_at, &dpid, &gqid);
        }
        const char* f = p;
        while (f <= le) {
            const char* t = memchr(f, '\t', (size_t)(le - f));
            const char* fe = t ? t : le;
            if (field == 4) {           /* alleles: REF + the comma-separated ALT list */
                nalt = 2;
                for (const char* c = f; c < fe; ++c) nalt += *c == ',';
            } else if (field == 8) {
                if (!(fe - f >= 2 && f[0] == 'G' && f[1] == 'T' && (fe - f == 2 || f[2] == ':'))) { free(copy); return -(l + 1); }
            } else if (field >= 9) {
                const int i = field - 9;
                if (i >= n_ind) { free(copy); return -(l + 1); }
                const char* g = f;
                const char* ge = memchr(f, ':', (size_t)(fe - f));
                if (!ge) ge = fe;
                if (ge - g != 3 || (g[1] != '/' && g[1] != '|')) { free(copy); return -(l + 1); }
                int miss = 0, sum = 0;
                for (int c = 0; c < 3; c += 2) {
                    if (g[c] == '.') miss = 1;
                    else if (g[c] == '0' || g[c] == '1') sum += g[c] - '0';
                    else { free(copy); return -(l + 1); }
                }
                if (!miss && filter && orc_call_filtered(copy + call_at[i], rw_len - call_at[i], dpid, gqid, 2, cf)) miss = 1;
                row[i >> 4] |= (uint32_t)(miss ? 3 : sum) << (2 * (i & 15));
            }
            ++field;
            if (!t) break;
            f = t + 1;
        }
        free(call_at);
        if (field != 9 + n_ind || nalt != 2) { free(copy); return -(l + 1); }
        for (int i = n_ind; i < Nw * 16; ++i) row[i >> 4] |= 3u << (2 * (i & 15));
        ++l;
        if (!e) break;
        p = e + 1;
    }
    free(copy);
    return l;
}

/* diversity.cpp:144-311 for one biallelic diploid locus, with REAL the
 * reference's float type: genotype counts, allele counts in REAL, Unify
 * (math2.cpp: ((double)A + MIN_FREQ) / (sum + n MIN_FREQ), stored in REAL),
 * CountK (misc.h: alleles above MIN_FREQ), the statistics in REAL; then the
 * MarkerDiversity conditions (filter.cpp:494-507) against double windows */
#define ORC_LOCUS_STATS(REAL, LOG)                                                                       \
    do {                                                                                                 \
        REAL fre[2] = {0, 0}, ho = 0, how = 0;                                                           \
        int n = 0, nhaplo = 0;                                                                           \
        for (int g = 0; g < 3; ++g) {                                                                    \
            const unsigned c = gcount[g];                                                                \
            if (!c) continue;                                                                            \
            nhaplo += 2 * c;                                                                             \
            ho += (g == 1 ? 1.0 : 0.0) * c * 2 * 1; /* HIndex * c * v * (v - 1) */                       \
            how += c * 2 * 1;                                                                            \
            n += c;                                                                                      \
            fre[0] += (REAL)(c * (2 - g));                                                               \
            fre[1] += (REAL)(c * g);                                                                     \
        }                                                                                                \
        ptype = n / (REAL)n_ind;                                                                         \
        nn = n;                                                                                          \
        if (n) {                                                                                         \
            const double invsum = 1.0 / ((double)fre[0] + (double)fre[1] + 2 * MINF);                    \
            fre[0] = (REAL)(((double)fre[0] + MINF) * invsum);                                           \
            fre[1] = (REAL)(((double)fre[1] + MINF) * invsum);                                           \
            k = (fre[0] > MINF) + (fre[1] > MINF);                                                       \
        }                                                                                                \
        if (k >= 2) {                                                                                    \
            REAL Iv = 0, b = 1, a2 = 0, picv = 0;                                                        \
            hoo = ho / how;                                                                              \
            const int nh = (int)(nhaplo + 0.5);                                                          \
            for (int a = 0; a < 2; ++a) {                                                                \
                const REAL af = fre[a];                                                                  \
                if (af * nh < 1e-5) continue;                                                            \
                if (af > 1e-5) Iv += -af * LOG(af);                                                      \
                if (b > af) b = af;                                                                      \
                a2 += af * af;                                                                           \
                for (int c = a + 1; c < 2; ++c)                                                          \
                    if (fre[c] > 0) picv += 2 * af * fre[c] * (1 - af * fre[c]);                         \
            }                                                                                            \
            if (b > 0.5) b = 1 - b;                                                                      \
            bmaf = b; he = 1 - a2; ae = 1 / a2; I = Iv; pic = picv;                                      \
            /* HWE G-test (diversity.cpp:337-492): expected count of each observed genotype */          \
            /* GFZ * n (HWECoef x product of frequencies, in double, stored in REAL); any   */          \
            /* expectation below 5 collapses two alleles into one, which leaves no test     */          \
            REAL G = 0;                                                                                  \
            int ok = 1;                                                                                  \
            for (int g = 0; g < 3 && ok; ++g) {                                                          \
                if (!gcount[g]) continue;                                                                \
                const double gf = g == 1 ? 2.0 * (double)fre[1] * (double)fre[0]                         \
                                         : (double)fre[g >> 1] * (double)fre[g >> 1];                     \
                const REAL obs = (REAL)gcount[g], ex = (REAL)(gf * n);                                   \
                if (ex < 5) ok = 0;                                                                      \
                else G += 2 * obs * LOG(obs / ex);                                                       \
            }                                                                                            \
            /* df = C(ploidy + k - 1, ploidy) - k = 1; 1 - the chi-square CDF */                        \
            if (ok) pval = (REAL)(1.0 - erf(sqrt(0.5 * (double)G)));                                     \
        }                                                                                                \
    } while (0)

void orc_locus_filter_pack2(const uint32_t* packed, int64_t L, int n_ind, const orc_locus_filter* f, uint8_t* keep,
                            double* stats) {
    const int Nw = (n_ind + 15) / 16;
    const double MINF = 1e-10, NANV = 0.0 / 0.0;
    for (int64_t l = 0; l < L; ++l) {
        unsigned gcount[4] = {0, 0, 0, 0};
        for (int i = 0; i < n_ind; ++i) gcount[(packed[l * Nw + (i >> 4)] >> (2 * (i & 15))) & 3]++;
        int k = 0, nn = 0;
        double ptype, bmaf = NANV, he = NANV, hoo = NANV, pic = NANV, ae = NANV, I = NANV, pval = NANV;
        if (f->single) ORC_LOCUS_STATS(float, logf);
        else ORC_LOCUS_STATS(double, log);
#define OUT(v, lo, hi) ((v) < (lo) || (v) > (hi))
        const int fail = k == 0 || (f->bmaf_b && k == 2 && OUT(bmaf, f->bmaf_min, f->bmaf_max)) ||
                         (f->k_b && (k < f->k_min || k > f->k_max)) || (f->n_b && (nn < f->n_min || nn > f->n_max)) ||
                         (f->ptype_b && OUT(ptype, f->ptype_min, f->ptype_max)) ||
                         (f->he_b && OUT(he, f->he_min, f->he_max)) || (f->ho_b && OUT(hoo, f->ho_min, f->ho_max)) ||
                         (f->pic_b && OUT(pic, f->pic_min, f->pic_max)) || (f->ae_b && OUT(ae, f->ae_min, f->ae_max)) ||
                         (f->I_b && OUT(I, f->I_min, f->I_max)) ||
                         (f->pval_b && pval != -1 && OUT(pval, f->pval_min, f->pval_max));
#undef OUT
        keep[l] = fail ? 0 : 1;
        if (stats) {
            double* o = stats + l * 10;
            o[0] = nn; o[1] = k; o[2] = ptype; o[3] = bmaf; o[4] = he; o[5] = hoo; o[6] = pic; o[7] = ae; o[8] = I;
            o[9] = pval;
        }
    }
}

/* ---- locus statistics of any ploidy and allele count ---------------------
 * DIVERSITY::CalcDiversity (diversity.cpp:144-492) for the general genotype
 * layout, and MarkerDiversity's windows (filter.cpp:494-507). The locus'
 * genotype table lists its typed genotypes in order of first appearance
 * (the loader's table, load.cpp:2180-2230): the sums over genotypes run in
 * that order, in the reference's REAL. */

/* one genotype: ploidy, sorted alleles, its count, and its dosage pattern:
 * distinct alleles by descending copy count, ties by the larger allele first
 * (GENOTYPE::GENOTYPE, function.cpp:259-337) */
typedef struct {
    int v, na;
    int al[16], key[16], cnt[16];
    unsigned count;
} orc_gtype;

static void orc_gtype_pattern(orc_gtype* g) {
    g->na = 0;
    for (int i = 0; i < g->v; ++i) {
        int isnew = 1;
        for (int j = i - 1; j >= 0; --j) if (g->al[i] == g->al[j]) { isnew = 0; break; }
        if (!isnew) continue;
        int ac = 1;
        for (int j = i + 1; j < g->v; ++j) ac += g->al[j] == g->al[i];
        g->key[g->na] = g->al[i];
        g->cnt[g->na++] = ac;
    }
    for (int i = 0; i < g->na; ++i)
        for (int j = i + 1; j < g->na; ++j)
            if (g->cnt[i] < g->cnt[j] || (g->cnt[i] == g->cnt[j] && g->key[i] < g->key[j])) {
                int t = g->cnt[i]; g->cnt[i] = g->cnt[j]; g->cnt[j] = t;
                t = g->key[i]; g->key[i] = g->key[j]; g->key[j] = t;
            }
}

/* GENOTYPE::HIndex: the share of ordered pairs of copies that differ, as
 * the reference's table holds it, a literal of 15 decimals: the double
 * nearest to round(p / q x 10^15) / 10^15 (0 for one copy) */
static double orc_hindex(const orc_gtype* g) {
    const long long q = (long long)g->v * (g->v - 1);
    if (q == 0) return 0;
    long long same = 0;
    for (int i = 0; i < g->na; ++i) same += (long long)g->cnt[i] * (g->cnt[i] - 1);
    const long long p = q - same;
    const long long n15 = (2 * p * 1000000000000000LL + q) / (2 * q);
    return (double)n15 / 1e15;
}

/* GENOTYPE::HWECoef: the multinomial coefficient v! / prod cnt! */
static double orc_hwecoef(const orc_gtype* g) {
    double f = 1;
    for (int i = 2; i <= g->v; ++i) f *= i;
    for (int a = 0; a < g->na; ++a)
        for (int i = 2; i <= g->cnt[a]; ++i) f /= i;
    return f;
}

/* IntegerPower (math2.h:307-350) in double */
static double orc_ipow(double x, int n) {
    switch (n) {
        case 0: return 1;
        case 1: return x;
        case 2: return x * x;
        case 3: return x * x * x;
        case 4: { double x2 = x * x; return x2 * x2; }
        case 5: { double x2 = x * x; return x2 * x2 * x; }
        case 6: { double x3 = x * x * x; return x3 * x3; }
        case 7: { double x3 = x * x * x; return x3 * x3 * x; }
        case 8: { double x2 = x * x, x4 = x2 * x2; return x4 * x4; }
        case 9: { double x3 = x * x * x; return x3 * x3 * x3; }
        case 10: { double x2 = x * x, x4 = x2 * x2; return x4 * x4 * x2; }
        default: return pow(x, (double)n);
    }
}

/* the upper tail of the chi-square distribution with df degrees of freedom:
 * erfc for df = 1 (as the biallelic kernel), else 1 - P(df/2, x/2), the
 * regularized lower incomplete gamma function by its series (x < a + 1) or
 * its continued fraction (Numerical Recipes, 6.2) */
static double orc_chi2_upper(double x, int df) {
    if (df == 1) return 1.0 - erf(sqrt(0.5 * x));
    const double a = 0.5 * df, z = 0.5 * x;
    if (z <= 0) return 1;
    const double lg = lgamma(a);
    if (z < a + 1) {
        double ap = a, sum = 1.0 / a, del = sum;
        for (int n = 0; n < 1000; ++n) { ap += 1; del *= z / ap; sum += del; if (fabs(del) < fabs(sum) * 1e-16) break; }
        return 1.0 - sum * exp(-z + a * log(z) - lg);
    }
    double b = z + 1 - a, c = 1.0 / 1e-300, d = 1.0 / b, h = d;
    for (int i = 1; i < 1000; ++i) {
        const double an = -i * (i - a);
        b += 2;
        d = an * d + b; if (fabs(d) < 1e-300) d = 1e-300;
        c = b + an / c; if (fabs(c) < 1e-300) c = 1e-300;
        d = 1.0 / d;
        const double del = d * c;
        h *= del;
        if (fabs(del - 1) < 1e-16) break;
    }
    return exp(-z + a * log(z) - lg) * h;
}

#define ORC_GENERAL_STATS(NAME, REAL, LOG)                                                                      \
static void NAME(orc_gtype* tab, int ng, int k2, int ni, double* out) {                                        \
    const double MINF = 1e-10, NANV = 0.0 / 0.0;                                                               \
    REAL fre[64], ho = 0, how = 0;                                                                             \
    for (int a = 0; a < k2; ++a) fre[a] = 0;                                                                   \
    int n = 0, nhaplo = 0, minp = 100, maxp = 0, varploidy = 0;                                                \
    for (int gi = 0; gi < ng; ++gi) {                                                                          \
        const orc_gtype* g = tab + gi;                                                                         \
        if (!g->count) continue;                                                                               \
        const unsigned c = g->count;                                                                           \
        const int v = g->v;                                                                                    \
        nhaplo += v * c;                                                                                       \
        if (v > maxp) maxp = v;                                                                                \
        if (v < minp) minp = v;                                                                                \
        if (maxp != minp) varploidy = 1;                                                                       \
        ho += orc_hindex(g) * c * v * (v - 1);                                                                 \
        how += c * v * (v - 1);                                                                                \
        n += c;                                                                                                \
        for (int i = 0; i < v; ++i) fre[g->al[i]] += c;                                                        \
    }                                                                                                          \
    const REAL ptype = n / (REAL)ni;                                                                           \
    {   /* Unify (math2.cpp:2268-2304) */                                                                      \
        double s = 0;                                                                                          \
        for (int a = 0; a < k2; ++a) s += fre[a];                                                              \
        const double invsum = 1.0 / (s + k2 * MINF);                                                           \
        for (int a = 0; a < k2; ++a) fre[a] = (REAL)(((double)fre[a] + MINF) * invsum);                       \
    }                                                                                                          \
    int k = 0;                                                                                                 \
    if (n) for (int a = 0; a < k2; ++a) k += fre[a] > MINF;                                                    \
    double bmaf = NANV, he = NANV, hoo = NANV, pic = NANV, ae = NANV, I = NANV, pval = NANV;                   \
    if (k >= 2) {                                                                                              \
        hoo = ho / how;                                                                                        \
        REAL b = 1, a2 = 0, picv = 0, Iv = 0;                                                                  \
        const int nh = (int)(nhaplo + 0.5);                                                                    \
        for (int a = 0; a < k2; ++a) {                                                                         \
            const REAL af = fre[a];                                                                            \
            if (af * nh < 1e-5) continue;                                                                      \
            if (af > 1e-5) Iv += -af * LOG(af);                                                                \
            if (b > af) b = af;                                                                                \
            a2 += af * af;                                                                                     \
            for (int c = a + 1; c < k2; ++c)                                                                   \
                if (fre[c] > 0) picv += 2 * af * fre[c] * (1 - af * fre[c]);                                  \
        }                                                                                                      \
        if (b > 0.5) b = 1 - b;                                                                                \
        bmaf = b; he = (REAL)(1 - a2); ae = (REAL)(1 / a2); I = Iv; pic = picv;                               \
        if (!varploidy) {                                                                                      \
            /* HWE G-test with allele collapsing (diversity.cpp:337-492), genotype model 0 */                  \
            const int ploidy = maxp;                                                                           \
            orc_gtype* t1 = malloc(sizeof(orc_gtype) * (size_t)(ng + 1));                                      \
            orc_gtype* t2 = malloc(sizeof(orc_gtype) * (size_t)(ng + 1));                                      \
            int n1 = 0;                                                                                        \
            for (int gi = 0; gi < ng; ++gi) t1[n1++] = tab[gi];                                                \
            REAL f1[64], f2[64];                                                                               \
            int amap[64];                                                                                      \
            for (int a = 0; a < k2; ++a) f1[a] = fre[a];                                                       \
            REAL G = 0;                                                                                        \
            int flag = 0;                                                                                      \
            for (int kk = k2; kk >= 1 && !flag; kk = (kk <= k ? kk - 1 : k)) {                                 \
                if (kk == 1) break;                                                                            \
                for (int a = 0; a < kk; ++a) f2[a] = 0;                                                        \
                if (kk <= k) {                                                                                 \
                    flag = 1;                                                                                  \
                    G = 0;                                                                                     \
                    for (int gi = 0; gi < n1; ++gi) {                                                          \
                        const orc_gtype* g = t1 + gi;                                                          \
                        if (!g->count) continue;                                                               \
                        double gfz = orc_hwecoef(g);                                                           \
                        for (int ai = g->na - 1; ai >= 0; --ai) gfz *= orc_ipow((double)f1[g->key[ai]], g->cnt[ai]); \
                        const REAL obs = (REAL)g->count, ex = (REAL)(gfz * n);                                  \
                        if (ex < 5) { flag = 0; break; }                                                       \
                        G += 2 * obs * LOG(obs / ex);                                                          \
                    }                                                                                          \
                }                                                                                              \
                if (flag) {                                                                                    \
                    /* df = C(ploidy + kk - 1, ploidy) - kk (Binomial via factorials) */                       \
                    double bin = 1;                                                                            \
                    for (int i = 2; i <= ploidy + kk - 1; ++i) bin *= i;                                       \
                    for (int i = 2; i <= ploidy; ++i) bin /= i;                                                \
                    for (int i = 2; i <= kk - 1; ++i) bin /= i;                                                \
                    const int df = (int)(bin - kk + 0.5);                                                      \
                    pval = (REAL)orc_chi2_upper((double)G, df);                                                \
                    break;                                                                                     \
                }                                                                                              \
                if (kk <= k) {                                                                                 \
                    /* merge the two rarest alleles (GetMinID: the first minimum) */                           \
                    int m1 = 0;                                                                                \
                    for (int a = 1; a < kk; ++a) if (f1[m1] > f1[a]) m1 = a;                                   \
                    f1[m1]++;                                                                                  \
                    int m2 = 0;                                                                                \
                    for (int a = 1; a < kk; ++a) if (f1[m2] > f1[a]) m2 = a;                                   \
                    f1[m1]--;                                                                                  \
                    if (m1 > m2) { int t = m1; m1 = m2; m2 = t; }                                              \
                    for (int j = 0, p = 0; j < kk; ++j) {                                                      \
                        if (j == m2) { amap[j] = m1; f2[m1] = f1[m1] + f1[m2]; }                               \
                        else { amap[j] = p; f2[p++] = f1[j]; }                                                 \
                    }                                                                                          \
                } else {                                                                                       \
                    /* drop absent alleles onto the most frequent one (GetMaxID: the first maximum) */          \
                    int m1 = 0;                                                                                \
                    for (int a = 1; a < kk; ++a) if (f1[m1] < f1[a]) m1 = a;                                   \
                    for (int j = 0, p = 0; j < kk; ++j) amap[j] = f1[j] < MINF ? -1 : p++;                     \
                    for (int j = 0; j < kk; ++j) amap[j] = amap[j] == -1 ? amap[m1] : amap[j];                 \
                }                                                                                              \
                /* the collapsed genotype table, in order of first mapping */                                  \
                int n2 = 0;                                                                                    \
                for (int gi = 0; gi < n1; ++gi) {                                                              \
                    const orc_gtype* g = t1 + gi;                                                              \
                    if (!g->count) continue;                                                                   \
                    orc_gtype h;                                                                               \
                    h.v = ploidy;                                                                              \
                    for (int ai = 0; ai < ploidy; ++ai) h.al[ai] = amap[g->al[ai]];                            \
                    for (int x = 1; x < ploidy; ++x) {                                                         \
                        const int y0 = h.al[x]; int y = x - 1;                                                 \
                        while (y >= 0 && h.al[y] > y0) { h.al[y + 1] = h.al[y]; --y; }                         \
                        h.al[y + 1] = y0;                                                                      \
                    }                                                                                          \
                    for (int j = 0; j < ploidy; ++j) f2[h.al[j]] += g->count;                                  \
                    int found = -1;                                                                            \
                    for (int x = 0; x < n2 && found < 0; ++x)                                                  \
                        if (!memcmp(t2[x].al, h.al, sizeof(int) * (size_t)ploidy)) found = x;                  \
                    if (found < 0) { h.count = g->count; orc_gtype_pattern(&h); t2[n2++] = h; }                \
                    else t2[found].count += g->count;                                                          \
                }                                                                                              \
                {   double s = 0;                                                                              \
                    for (int a = 0; a < kk; ++a) s += f2[a];                                                   \
                    const double invsum = 1.0 / (s + kk * MINF);                                               \
                    for (int a = 0; a < kk; ++a) f2[a] = (REAL)(((double)f2[a] + MINF) * invsum);             \
                }                                                                                              \
                orc_gtype* tt = t1; t1 = t2; t2 = tt; n1 = n2;                                                 \
                for (int a = 0; a < kk; ++a) f1[a] = f2[a];                                                    \
            }                                                                                                  \
            free(t1); free(t2);                                                                                \
        }                                                                                                      \
    }                                                                                                          \
    out[0] = n; out[1] = k; out[2] = ptype; out[3] = bmaf; out[4] = he; out[5] = hoo; out[6] = pic;           \
    out[7] = ae; out[8] = I; out[9] = pval;                                                                    \
}
ORC_GENERAL_STATS(orc_general_stats_f, float, logf)
ORC_GENERAL_STATS(orc_general_stats_d, double, log)

void orc_locus_filter_general(const int8_t* G, const int8_t* Gtable, int64_t L, int n_ind, int vmax,
                              const int32_t* k, const orc_locus_filter* f, uint8_t* keep, double* stats) {
    orc_gtype* tab = malloc(sizeof(orc_gtype) * (size_t)(n_ind + 1));
    for (int64_t l = 0; l < L; ++l) {
        /* the table's order: first appearance among the calls the loader saw
         * (Gtable, before the genotype filter); its counts: the calls kept */
        int ng = 0;
        for (int pass = 0; pass < 2; ++pass) {
            const int8_t* src = pass == 0 ? (Gtable ? Gtable : G) : G;
            for (int i = 0; i < n_ind; ++i) {
                const int8_t* g = src + ((size_t)l * n_ind + i) * vmax;
                if (g[0] < 0) continue;
                orc_gtype h;
                memset(&h, 0, sizeof h);
                h.v = 0;
                int bad = 0;
                while (h.v < vmax && g[h.v] >= 0) { bad |= g[h.v] >= k[l]; h.al[h.v] = g[h.v]; h.v++; }
                if (bad) continue;   /* an allele outside the locus' alleles: missing */
                int found = -1;
                for (int x = 0; x < ng && found < 0; ++x)
                    if (tab[x].v == h.v && !memcmp(tab[x].al, h.al, sizeof(int) * (size_t)h.v)) found = x;
                if (pass == 0) {
                    if (found < 0) { orc_gtype_pattern(&h); h.count = 0; tab[ng++] = h; }
                } else if (found >= 0) tab[found].count++;
            }
        }
        double o[10];
        if (f->single) orc_general_stats_f(tab, ng, k[l], n_ind, o);
        else orc_general_stats_d(tab, ng, k[l], n_ind, o);
        const int kk = (int)o[1], nn = (int)o[0];
#define OUT(v, lo, hi) ((v) < (lo) || (v) > (hi))
        const int fail = kk == 0 || (f->bmaf_b && kk == 2 && OUT(o[3], f->bmaf_min, f->bmaf_max)) ||
                         (f->k_b && (kk < f->k_min || kk > f->k_max)) || (f->n_b && (nn < f->n_min || nn > f->n_max)) ||
                         (f->ptype_b && OUT(o[2], f->ptype_min, f->ptype_max)) ||
                         (f->he_b && OUT(o[4], f->he_min, f->he_max)) || (f->ho_b && OUT(o[5], f->ho_min, f->ho_max)) ||
                         (f->pic_b && OUT(o[6], f->pic_min, f->pic_max)) || (f->ae_b && OUT(o[7], f->ae_min, f->ae_max)) ||
                         (f->I_b && OUT(o[8], f->I_min, f->I_max)) ||
                         (f->pval_b && o[9] != -1 && OUT(o[9], f->pval_min, f->pval_max));
#undef OUT
        keep[l] = fail ? 0 : 1;
        if (stats) memcpy(stats + l * 10, o, sizeof o);
    }
    free(tab);
}
