/*
 * ORACLE (test infrastructure only): command-line front end of the C
 * restatement, taking the subset of vcfpop's flags that the STRUCTURE path
 * reads (parameters.cpp:584-627, 1230-1307; -g_seed, -g_indtext, -g_decimal)
 * and writing the same per-run and summary files, so its output can be
 * diffed against the reference program's.
 */
#include "structure_oracle.h"
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <ctype.h>

static char* g_input = NULL;
static char* g_output = (char*)"out";
static char* g_indtext = NULL;
static int g_seed = 0, g_decimal = 5, kmin = 1, kmax = 5, nruns = 1;

static int yesno(const char* v) { return strcmp(v, "yes") == 0 ? 1 : 0; }

typedef struct { char** names; int n; } strlist;

/* Read a plain VCF: sample names, per-locus allele counts and GT calls; a
 * typed call that fails the genotype filter (cf, may be null) is missing. */
static int read_vcf(const char* path, int* N, int64_t* L, int* vmax, int8_t** G, int32_t** ploidy,
                    int32_t** k, strlist* inds, strlist* locs, const orc_call_filter* cf) {
    FILE* f = fopen(path, "r");
    if (!f) return -1;
    size_t cap = 1 << 20;
    char* line = malloc(cap);
    int n = 0; int64_t nl = 0, lcap = 1024;
    int vm = 0;
    int32_t* kk = malloc(lcap * sizeof(int32_t));
    int8_t* g = NULL;
    char** lnames = malloc(lcap * sizeof(char*));
    int32_t* pl = NULL;
    ssize_t len;
    while ((len = getline(&line, &cap, f)) > 0) {
        if (line[0] == '#' && line[1] == '#') continue;
        while (len > 0 && (line[len - 1] == '\n' || line[len - 1] == '\r')) line[--len] = 0;
        if (line[0] == '#') {
            char* tok = strtok(line, "\t");
            int col = 0;
            inds->names = malloc(sizeof(char*) * 1000000);
            while (tok) { if (col >= 9) inds->names[n++] = strdup(tok); tok = strtok(NULL, "\t"); col++; }
            inds->n = n;
            pl = calloc(n, sizeof(int32_t));
            continue;
        }
        if (nl == lcap) { lcap *= 2; kk = realloc(kk, lcap * sizeof(int32_t)); lnames = realloc(lnames, lcap * sizeof(char*)); }
        /* the calls of the line, kept whole (with their keys) for the filter */
        const int filter = cf && (cf->dp_b || cf->gq_b || cf->ploidy_b);
        char* calls = NULL;
        char* fields[10]; char* p = line;
        for (int c = 0; c < 9; ++c) { fields[c] = p; p = strchr(p, '\t'); *p++ = 0; }
        /* the loader's rewritten calls (orc_rewrite_calls) for the filter */
        int dpid = -1, gqid = -1;
        size_t* call_at = NULL;
        size_t rw_len = 0;
        if (filter) {
            const size_t plen = strlen(p);
            calls = malloc(plen + 1);
            call_at = malloc(sizeof(size_t) * (size_t)n);
            rw_len = orc_rewrite_calls(fields[8], fields[8] + strlen(fields[8]), p, p + plen, n, calls, call_at,
                                       &dpid, &gqid);
        }
        int nalt = 1;
        for (char* q = fields[4]; *q; ++q) if (*q == ',') nalt++;
        kk[nl] = 1 + nalt;
        char nm[512]; snprintf(nm, sizeof nm, "%s_%s", fields[0], fields[1]);
        lnames[nl] = strdup(nm);
        if (nl == 0) {
            /* ploidy from the first record */
            char* q = p;
            for (int i = 0; i < n; ++i) {
                int v = 1;
                while (*q && *q != '\t') { if (*q == '/' || *q == '|') v++; q++; }
                if (*q) q++;
                pl[i] = v; if (v > vm) vm = v;
            }
            g = malloc((size_t)lcap * n * vm);
        } else if ((size_t)nl >= (size_t)lcap / 2 || 1) {
            g = realloc(g, (size_t)lcap * n * vm);
        }
        int8_t* row = g + (size_t)nl * n * vm;
        char* q = p;
        for (int i = 0; i < n; ++i) {
            int8_t al[16]; int v = 0, miss = 0;
            for (;;) {
                if (*q == '.') { miss = 1; q++; }
                else { al[v] = (int8_t)strtol(q, &q, 10); }
                v++;
                if (*q == '/' || *q == '|') { q++; continue; }
                break;
            }
            while (*q && *q != '\t') q++;
            if (*q) q++;
            for (int c = 0; c < vm; ++c) row[i * vm + c] = -1;
            if (!miss && filter && orc_call_filtered(calls + call_at[i], rw_len - call_at[i], dpid, gqid, v, cf))
                miss = 1;
            if (!miss) {
                for (int a = 0; a < v; ++a)
                    for (int b = a + 1; b < v; ++b)
                        if (al[b] < al[a]) { int8_t t = al[a]; al[a] = al[b]; al[b] = t; }
                for (int c = 0; c < v; ++c) row[i * vm + c] = al[c];
            }
        }
        free(calls);
        free(call_at);
        nl++;
    }
    free(line);
    fclose(f);
    *N = n; *L = nl; *vmax = vm; *G = g; *ploidy = pl; *k = kk;
    locs->names = lnames; locs->n = (int)nl;
    return 0;
}

/* -g_indtext="name:#a-#b,#c name2:#d-#e ..." (1-based ranges) */
static void parse_indtext(const char* s, int N, int32_t* popid, strlist* pops) {
    pops->names = malloc(sizeof(char*) * (N + 1));
    pops->n = 0;
    for (int i = 0; i < N; ++i) popid[i] = -1;
    if (!s) { pops->names[pops->n++] = strdup("pop1"); for (int i = 0; i < N; ++i) popid[i] = 0; return; }
    char* buf = strdup(s);
    char* save = NULL;
    for (char* tok = strtok_r(buf, " ", &save); tok; tok = strtok_r(NULL, " ", &save)) {
        char* colon = strchr(tok, ':');
        if (!colon) continue;
        *colon = 0;
        int pid = pops->n;
        pops->names[pops->n++] = strdup(tok);
        char* save2 = NULL;
        for (char* r = strtok_r(colon + 1, ",", &save2); r; r = strtok_r(NULL, ",", &save2)) {
            int a = 0, b = 0;
            if (sscanf(r, "#%d-#%d", &a, &b) == 2) {}
            else if (sscanf(r, "#%d", &a) == 1) b = a;
            for (int i = a; i <= b && i <= N; ++i) popid[i - 1] = pid;
        }
    }
    free(buf);
}

int main(int argc, char** argv) {
    orc_params P;
    memset(&P, 0, sizeof P);
    /* defaults: parameters.cpp:584-627 */
    P.nburnin = 1000; P.nreps = 10000; P.nthinning = 10; P.nadmburnin = 500;
    P.lambda = 1; P.stdlambda = 0.3; P.maxlambda = 10;
    P.alpha = 1; P.stdalpha = 0.025; P.maxalpha = 10; P.inferalpha = 1; P.diffalpha = 0;
    P.uniformalpha = 1; P.alphapriora = 0.05; P.alphapriorb = 0.001; P.metrofreq = 10;
    P.r = 1; P.maxr = 20; P.epsr = 0.1; P.epseta = 0.025; P.epsgamma = 0.025;
    P.pmeanf = 0.01; P.pstdf = 0.05; P.stdf = 0.05; P.fsame = 0;
    int diversity = 0, ffilter = 0;
    orc_call_filter cf;
    memset(&cf, 0, sizeof cf);
    for (int i = 1; i < argc; ++i) {
        char* a = argv[i];
        char* eq = strchr(a, '=');
        const char* v = eq ? eq + 1 : "";
        size_t nlen = eq ? (size_t)(eq - a) : strlen(a);
#define IS(s) (nlen == strlen(s) && !strncmp(a, s, nlen))
        if (IS("-g_input")) g_input = strdup(v);
        else if (IS("-g_output")) g_output = strdup(v);
        else if (IS("-g_seed")) g_seed = atoi(v);
        else if (IS("-g_decimal")) g_decimal = atoi(v);
        else if (IS("-g_indtext")) { g_indtext = strdup(v); size_t n = strlen(g_indtext); if (n && g_indtext[0] == '"') { memmove(g_indtext, g_indtext + 1, n); g_indtext[n - 2] = 0; } }
        else if (IS("-structure_admix")) P.admix = yesno(v);
        else if (IS("-structure_locpriori")) P.locpriori = yesno(v);
        else if (IS("-structure_f")) P.fmodel = yesno(v);
        else if (IS("-structure_krange")) sscanf(v, "[%d,%d]", &kmin, &kmax);
        else if (IS("-structure_nburnin")) P.nburnin = atoi(v);
        else if (IS("-structure_nreps")) P.nreps = atoi(v);
        else if (IS("-structure_nthinning")) P.nthinning = atoi(v);
        else if (IS("-structure_nruns")) nruns = atoi(v);
        else if (IS("-structure_nadmburnin")) P.nadmburnin = atoi(v);
        else if (IS("-structure_writelnl")) P.writelnl = yesno(v);
        else if (IS("-structure_diversity")) diversity = yesno(v);
        else if (IS("-structure_lambda")) P.lambda = atof(v);
        else if (IS("-structure_alpha")) P.alpha = atof(v);
        else if (IS("-structure_inferalpha")) P.inferalpha = yesno(v);
        else if (IS("-structure_diffalpha")) P.diffalpha = yesno(v);
        else if (IS("-structure_uniformalpha")) P.uniformalpha = yesno(v);
        else if (IS("-structure_stdalpha")) P.stdalpha = atof(v);
        else if (IS("-structure_maxalpha")) P.maxalpha = atof(v);
        else if (IS("-structure_alphapriora")) P.alphapriora = atof(v);
        else if (IS("-structure_alphapriorb")) P.alphapriorb = atof(v);
        else if (IS("-structure_metrofreq")) P.metrofreq = atoi(v);
        else if (IS("-structure_r")) P.r = atof(v);
        else if (IS("-structure_maxr")) P.maxr = atof(v);
        else if (IS("-structure_stdr")) P.epsr = atof(v);
        else if (IS("-structure_epseta")) P.epseta = atof(v);
        else if (IS("-structure_epsgamma")) P.epsgamma = atof(v);
        else if (IS("-structure_pmeanf")) P.pmeanf = atof(v);
        else if (IS("-structure_pstdf")) P.pstdf = atof(v);
        else if (IS("-structure_stdf")) P.stdf = atof(v);
        else if (IS("-structure_singlef")) P.fsame = yesno(v);
        else if (IS("-f")) ffilter = 1;
        else if (IS("-f_dp")) cf.dp_b = sscanf(v, "[%d,%d]", &cf.dp_min, &cf.dp_max) == 2;
        else if (IS("-f_gq")) cf.gq_b = sscanf(v, "[%d,%d]", &cf.gq_min, &cf.gq_max) == 2;
        else if (IS("-f_ploidy")) cf.ploidy_b = sscanf(v, "[%d,%d]", &cf.ploidy_min, &cf.ploidy_max) == 2;
#undef IS
    }
    if (!g_input) { fprintf(stderr, "missing -g_input\n"); return 2; }
    int N, vmax; int64_t L; int8_t* G; int32_t *ploidy, *k;
    strlist inds, locs, pops;
    /* the genotype filter applies only under -f (parameters.cpp:1338-1339) */
    if (read_vcf(g_input, &N, &L, &vmax, &G, &ploidy, &k, &inds, &locs, ffilter ? &cf : NULL)) { fprintf(stderr, "cannot read %s\n", g_input); return 2; }
    /* with the genotype filter, the calls before it (the loader's genotype
     * table, load.cpp:2145-2230) decide the polymorphic loci and their order */
    int8_t* Gt = NULL;
    if (ffilter && (cf.dp_b || cf.gq_b || cf.ploidy_b)) {
        int N2, vmax2; int64_t L2; int32_t *ploidy2, *k2;
        strlist inds2, locs2;
        if (read_vcf(g_input, &N2, &L2, &vmax2, &Gt, &ploidy2, &k2, &inds2, &locs2, NULL) || N2 != N || L2 != L ||
            vmax2 != vmax) { fprintf(stderr, "cannot read %s\n", g_input); return 2; }
    }
    int32_t* popid = malloc(sizeof(int32_t) * N);
    parse_indtext(g_indtext, N, popid, &pops);
    orc_owned_data* od = orc_data_build_ex(N, L, vmax, G, ploidy, k, popid, pops.n, Gt);
    const orc_data* D = orc_data_view(od);
    const int64_t* order = orc_data_order(od);
    /* order[] has one entry per locus kept by the monomorphic filter:
     * sorted position -> input locus */
    char** lsorted = malloc(sizeof(char*) * (size_t)(D->L > 0 ? D->L : 1));
    for (int64_t l = 0; l < D->L; ++l) lsorted[l] = locs.names[order[l]];
    int total = (kmax - kmin + 1) * nruns, id = 0;
    double* res = calloc(total * 3, sizeof(double));
    int* rk = calloc(total, sizeof(int)); int* rr = calloc(total, sizeof(int));
    for (int K = kmin; K <= kmax; ++K)
        for (int rep = 1; rep <= nruns; ++rep) {
            id++;
            P.K = K;
            P.seed = orc_hash_ulong_c((uint64_t)(int64_t)(g_seed + id));
            orc_chain* c = orc_chain_new(D, &P);
            orc_run(c);
            orc_write_structure(c, g_output, rep, id, (const char* const*)inds.names,
                                (const char* const*)pops.names, (const char* const*)lsorted, g_decimal, diversity);
            res[(id - 1) * 3 + 0] = c->rout[0]; res[(id - 1) * 3 + 1] = c->rout[2]; res[(id - 1) * 3 + 2] = c->rout[3];
            rk[id - 1] = K; rr[id - 1] = rep;
            orc_chain_free(c);
        }
    /* numeric table of <out>.structure.txt (structure.cpp:379-401) */
    char fn[8192]; snprintf(fn, sizeof fn, "%s.oracle.structure.txt", g_output);
    FILE* f = fopen(fn, "wb");
    char fmt[16]; snprintf(fmt, sizeof fmt, "%%0.%df", g_decimal);
    fprintf(f, "ID\tk\trep\tMean lnL\tVar lnL\tlnP(D)");
    for (int i = 0; i < total; ++i) {
        fprintf(f, "\r\n%d\t%d\t%d\t", i + 1, rk[i], rr[i]);
        fprintf(f, fmt, res[i * 3]); fprintf(f, "\t"); fprintf(f, fmt, res[i * 3 + 1]); fprintf(f, "\t"); fprintf(f, fmt, res[i * 3 + 2]);
    }
    fclose(f);
    orc_data_free(od);
    return 0;
}
