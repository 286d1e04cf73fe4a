// The result files of one finished run in the reference's format: WriteStructure
// (src/structure.cpp:86-377). The numbers come from the chain's device state
// (vp_chain_result) and the device output reductions (vp_chain_divergence);
// the text, its order and its number format are the reference's.
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "vp_internal.h"

namespace {

struct Out {
    FILE* f;
    const char* fmt;
    const char* delim;
    const char* lb;
    void real(double v) {
        if (std::isnan(v) || std::isinf(v)) fputs("nan", f);
        else fprintf(f, fmt, v);
    }
    void s(const char* t) { fputs(t, f); }
    void n(long long v) { fprintf(f, "%lld", v); }
    void nl() { fputs(lb, f); }
    void d() { fputs(delim, f); }
};

int open_out(const char* path, FILE** f) {
    *f = fopen(path, "wb");
    if (!*f) { vp_set_error("cannot write %s", path); return VP_E_ARG; }
    return VP_OK;
}

}  // namespace

extern "C" int vp_write_structure(vp_chain* c, const vp_write_opts* o) {
    if (!c || !o || !o->prefix || !o->ind_names || !o->pop_names || !o->loc_names) {
        vp_set_error("vp_write_structure: null argument");
        return VP_E_ARG;
    }
    if (o->decimal < 0 || o->decimal > 30) { vp_set_error("decimal places must be in 0..30"); return VP_E_ARG; }
    const vp_dataset* ds = vp_chain_dataset(c);
    vp_params P;
    vp_chain_params(c, &P);
    vp_result r;
    int rc = vp_chain_sizes(c, &r);
    if (rc) return rc;
    const int K = r.K, N = r.N, S = r.S;
    const int64_t L = ds->L, KT = r.KT;
    std::vector<double> rout(r.rlen), lnl(std::max(r.nlnl, 1)), anc((size_t)N * K);
    std::vector<float> Q((size_t)N * K), fm((size_t)K * KT);
    r.rout = rout.data(); r.lnl = lnl.data(); r.Q = Q.data(); r.ancestry = anc.data(); r.freqm = fm.data();
    if ((rc = vp_chain_result(c, &r))) return rc;
    std::vector<double> H(K), Dm((size_t)K * K), H2(o->diversity ? (size_t)K * L : 0);
    if ((rc = vp_chain_divergence(c, H.data(), Dm.data(), o->diversity ? H2.data() : nullptr))) return rc;

    char fmt[16];
    snprintf(fmt, sizeof fmt, "%%0.%df", o->decimal);
    const char* delim = o->comma ? "," : "\t";
    const char* lb = o->unix_lb ? "\n" : "\r\n";
    std::string fn;
    char buf[64];
    if (P.writelnl) {
        // the lnL trace: every thinned sweep of burn-in and sampling (src/structure.cpp:110-121)
        snprintf(buf, sizeof buf, ".structure.k=%d_rep=%d_id=%d.lnl.txt", K, o->rep, o->id);
        fn = std::string(o->prefix) + buf;
        FILE* f;
        if ((rc = open_out(fn.c_str(), &f))) return rc;
        Out w{f, fmt, delim, lb};
        w.n(r.nburnin); w.nl();
        w.s("Iteration"); w.d(); w.s("lnL"); w.nl();
        int j = 0;
        for (int i = 0; i < r.nburnin; i += r.nthinning) { w.n(i); w.d(); w.real(j < r.nlnl ? lnl[j] : NAN); ++j; w.nl(); }
        for (int i = 0; i < r.nreps; i += r.nthinning) {
            w.n(i + r.nburnin); w.d(); w.real(j < r.nlnl ? lnl[j] : NAN); ++j; w.nl();
        }
        fclose(f);
    }
    snprintf(buf, sizeof buf, ".structure.k=%d_rep=%d_id=%d.txt", K, o->rep, o->id);
    fn = std::string(o->prefix) + buf;
    FILE* f;
    if ((rc = open_out(fn.c_str(), &f))) return rc;
    Out w{f, fmt, delim, lb};
    // parameters and the likelihood summary (src/structure.cpp:122-137)
    w.nl(); w.nl(); w.s("Parameters:"); w.nl();
    fprintf(f, "Seed=%lld", (long long)r.seed); w.nl();
    fprintf(f, "Model=%s,%s,%s", P.admix ? "ADM" : "NOADM", P.locpriori ? "LOC" : "NOLOC", P.fmodel ? "F" : "NOF"); w.nl();
    fprintf(f, "Number of cluster=%d", K); w.nl();
    fprintf(f, "Replicate=%d", o->rep); w.nl();
    fprintf(f, "Run id=%d", o->id); w.nl();
    w.s("Mean value of ln likelihood="); w.real(rout[0]); w.nl();
    w.s("Variance of ln likelihood="); w.real(rout[2]); w.nl();
    w.s("Estimated Ln Prob of Data="); w.real(rout[3]); w.nl(); w.nl();
    // parameter means (src/structure.cpp:139-232)
    const int nf = P.fmodel ? (P.fsame ? 1 : K) : 0, nl = P.difflambda ? K : 1;
    if (P.locpriori) {
        w.nl(); w.s("Mean value of r="); w.real(rout[4 + nl]);
        w.nl(); fprintf(f, "Mean value of global %s", P.admix ? "alpha" : "eta");
        w.nl(); w.d(); w.s("Cluster"); w.nl();
        for (int j = 0; j < K; ++j) { w.d(); w.n(j + 1); }
        w.nl();
        for (int j = 0; j < K; ++j) { w.d(); w.real(rout[4 + nl + 1 + j]); }
        w.nl(); fprintf(f, "Mean value of local %s for each location", P.admix ? "alpha" : "gamma");
        w.nl(); w.d(); w.s("Cluster"); w.nl(); w.s("Pop");
        for (int j = 0; j < K; ++j) { w.d(); w.n(j + 1); }
        for (int i = 0; i < S; ++i) {
            w.nl(); w.s(o->pop_names[i]);
            for (int j = 0; j < K; ++j) { w.d(); w.real(rout[4 + nl + 1 + K + i * K + j]); }
        }
    } else if (P.admix && P.inferalpha) {
        if (!P.diffalpha) { w.nl(); w.s("Mean value of alpha="); w.real(rout[4 + nl]); }
        else
            for (int j = 0; j < K; ++j) { w.nl(); fprintf(f, "Mean value of alpha_%d=", j + 1); w.real(rout[4 + nl + j]); }
    }
    if (P.fmodel) {
        if (P.fsame) { w.nl(); w.s("Mean value of Fst="); w.real(rout[r.rlen - 1]); }
        else {
            w.nl(); w.s("Mean value of Fst"); w.nl(); w.d(); w.s("Cluster"); w.nl();
            for (int j = 0; j < K; ++j) { w.d(); w.n(j + 1); }
            w.nl();
            for (int i = 0; i < nf; ++i) { w.d(); w.real(rout[r.rlen - nf + i]); }
        }
    }
    // membership of each pre-defined population from the final Q, each row
    // normalised as Unify<float> does (src/structure.cpp:234-262)
    const int32_t* popid = ds->popid.data();
    std::vector<float> O((size_t)S * K, 0.f);
    w.nl(); w.nl(); fprintf(f, "Proportion of membership of each pre-defined population in each of the %d clusters", K);
    w.nl(); w.d(); w.s("Cluster"); w.nl(); w.s("Pop");
    for (int i = 0; i < N; ++i)
        for (int k = 0; k < K; ++k) O[(size_t)popid[i] * K + k] += Q[(size_t)i * K + k];
    for (int s = 0; s < S; ++s) {
        double sum = 0;
        for (int k = 0; k < K; ++k) sum += O[(size_t)s * K + k];
        const double inv = 1.0 / (sum + K * 1e-10);
        for (int k = 0; k < K; ++k) O[(size_t)s * K + k] = (float)(((double)O[(size_t)s * K + k] + 1e-10) * inv);
    }
    for (int k = 0; k < K; ++k) { w.d(); w.n(k + 1); }
    for (int s = 0; s < S; ++s) {
        w.nl(); w.s(o->pop_names[s]);
        for (int k = 0; k < K; ++k) { w.d(); w.real(O[(size_t)s * K + k]); }
    }
    // ancestry of each individual: the normalised MiSum (src/structure.cpp:264-291)
    w.nl(); w.nl(); w.s("Inferred ancestry of individuals");
    w.nl(); w.d(); w.d(); w.s("Cluster");
    w.nl(); w.s("Ind"); w.d(); w.s("Pop"); w.d(); w.s("RegL1");
    for (int j = 0; j < K; ++j) { w.d(); w.n(j + 1); }
    for (int i = 0; i < N; ++i) {
        w.nl(); w.s(o->ind_names[i]); w.d(); w.s(o->pop_names[popid[i]]); w.d(); w.s("Total");
        for (int k = 0; k < K; ++k) { w.d(); w.real(anc[(size_t)i * K + k]); }
    }
    // net nucleotide distance between clusters (src/structure.cpp:293-324)
    w.nl(); w.nl(); w.s("Allele-frequency divergence among pops (Net nucleotide distance)");
    w.nl(); w.d(); w.s("Cluster"); w.nl(); w.s("Cluster");
    for (int j = 0; j < K; ++j) { w.d(); w.n(j + 1); }
    for (int i = 0; i < K; ++i) {
        w.nl(); w.n(i + 1);
        for (int j = 0; j < K; ++j) { w.d(); w.real(Dm[(size_t)i * K + j]); }
    }
    // per-cluster diversity and mean allele frequencies (src/structure.cpp:326-369)
    if (o->diversity) {
        w.nl(); w.nl(); w.s("Estimated genetic diversity in each cluster");
        w.nl(); w.s("Locus"); w.d(); w.s("Cluster"); w.d(); w.s("Heterozygosity");
        for (int a = 0; a < ds->maxK; ++a) { w.d(); fprintf(f, "Allele%d", a); }
        for (int k = 0; k < K; ++k) { w.nl(); w.s(k ? "" : "Average"); w.d(); w.n(k + 1); w.real(H[k]); }
        int64_t off = 0;
        for (int64_t l = 0; l < L; ++l) {
            const int kl = ds->k[l];
            for (int k = 0; k < K; ++k) {
                w.nl(); w.s(k ? "" : o->loc_names[ds->order[l]]); w.d(); w.n(k + 1); w.d();
                w.real(H2[(size_t)k * L + l]);
                for (int a = 0; a < kl; ++a) { w.d(); w.real(fm[(size_t)k * KT + off + a]); }
            }
            off += kl;
        }
    }
    fclose(f);
    return VP_OK;
}
