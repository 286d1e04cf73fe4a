/*
 * ORACLE (test infrastructure only): CPU restatement of vcfpop's Bayesian
 * STRUCTURE MCMC (src/structure.cpp:405-2166) for REAL = float with
 * -g_fastsingle=yes, one thread and the scalar math path (-g_simd=none).
 * Parity pinned against the reference program built from its own sources
 * (oracle/Makefile -> oracle/_ref/vcfpop) through tests/golden/.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
 * this library; the product never links it.
 */
#ifndef STRUCTURE_ORACLE_H
#define STRUCTURE_ORACLE_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* A dataset after the reference's locus sort (structure.cpp:2349-2381) and
 * grouping of individuals by population (filter.cpp:300-345). */
typedef struct {
    int32_t N;            /* individuals */
    int64_t L;            /* loci */
    int32_t S;            /* populations (sampling locations) */
    int32_t vmax;         /* max copies stored per call (>= maxploidy) */
    int32_t maxploidy;    /* max ploidy of a typed call (function.cpp:4906-4912) */
    int32_t maxK;         /* max alleles at a locus */
    int64_t KT;           /* total alleles */
    const int32_t* k;     /* [L] alleles per locus */
    const int64_t* off;   /* [L] allele_freq_offset */
    const uint8_t* gcopies; /* [L*N] typed copies of each call, 0 = missing */
    const uint8_t* galleles;/* [L*N*vmax] allele index per copy, ascending */
    const int64_t* vt;    /* [N] typed allele copies per individual */
    const int32_t* popid; /* [N] population of each individual */
    const int32_t* pop_ind0; /* [S] first individual of each population */
    const int32_t* pop_nind; /* [S] individuals per population */
    const float* totfreq; /* [KT] total-population allele frequency (F-model init) */
    const int32_t* nhaplo;/* [L] typed copies per locus (F-model init) */
    int64_t coprime;      /* structure_loc_coprime (structure.cpp:2384-2386) */
} orc_data;

/* Mirrors BAYESIAN<REAL>::ReadPar (structure.cpp:405-464). */
typedef struct {
    int32_t K;
    int32_t admix, locpriori, fmodel;
    int32_t nburnin, nreps, nthinning, nadmburnin;   /* nadmburnin: flag value */
    int32_t writelnl;
    double lambda, stdlambda, maxlambda;
    int32_t inferlambda, difflambda;
    double alpha, stdalpha, maxalpha, alphapriora, alphapriorb;
    int32_t metrofreq, inferalpha, diffalpha, uniformalpha;
    double r, maxr, epsr, epseta, epsgamma;
    double pmeanf, pstdf, stdf;
    int32_t fsame;
    uint64_t seed;        /* HashULong(g_seed + run id) */
} orc_params;

typedef struct orc_chain orc_chain;

/* Chain state, field by field as BAYESIAN<float> (structure.h:50-170). */
struct orc_chain {
    orc_params P;
    const orc_data* D;
    int32_t K, N, S, nburnin, nreps, nadmburnin, nthinning;
    int64_t L, KT;
    float *Freq, *FreqM, *FreqA;
    double* Lambda;
    int64_t* MiSum;     /* becomes double after arrange (UnifyInt64ToDouble) */
    uint16_t* Z;
    int64_t* Mi;
    float* Q;
    int32_t* Ni;
    double* Alpha;
    double *f, *F;
    double *Eta, *Gamma;
    float* Di;
    double *AlphaLocal, *SumAlpha;
    float *fbuf1, *fbuf2;
    double *bufNK1, *bufNK2, *bufN1, *bufN2;
    float* bufK;
    double r;
    int32_t m, nr, nlnL, rlen;
    double* lnL;
    double* rout;
    int64_t* kdis;
    int32_t binaryq, singlez;
};

/* ---- datasets ---- */
typedef struct orc_owned_data orc_owned_data;
/* Build from per-copy allele arrays in INPUT locus order:
 *   G[l*N*vmax + i*vmax + c] allele index, or -1 when missing / absent copy
 *   ploidy[i] copies in each individual's calls (missing calls keep it)
 *   k[l] alleles per locus. Individuals must already be grouped by pop.
 * Applies the reference's genotype-id counting, locus sort and offsets. */
orc_owned_data* orc_data_build(int32_t N, int64_t L, int32_t vmax, const int8_t* G,
                               const int32_t* ploidy, const int32_t* k,
                               const int32_t* popid, int32_t S);
/* orc_data_build with the calls before the genotype filter (Gtable, same
 * layout; NULL: G): the loader's genotype table holds those, so they decide
 * which loci are polymorphic and the loci's id widths. */
orc_owned_data* orc_data_build_ex(int32_t N, int64_t L, int32_t vmax, const int8_t* G,
                                  const int32_t* ploidy, const int32_t* k,
                                  const int32_t* popid, int32_t S, const int8_t* Gtable);
const orc_data* orc_data_view(const orc_owned_data* d);
const int64_t* orc_data_order(const orc_owned_data* d); /* sorted -> input locus */
void orc_data_free(orc_owned_data* d);

/* ---- chains ---- */
orc_chain* orc_chain_new(const orc_data* D, const orc_params* P);
void orc_chain_free(orc_chain* c);
void orc_init(orc_chain* c);            /* InitFix, InitAdmix, InitLocPriori, InitFmodel */
void orc_sweep(orc_chain* c);           /* one iteration m (structure.cpp:2124-2153), m++ */
void orc_arrange(orc_chain* c);         /* structure.cpp:1860-1869 */
void orc_run(orc_chain* c);             /* init + all sweeps + arrange */

/* individual steps at the chain's current m */
void orc_update_p(orc_chain* c);
void orc_update_q(orc_chain* c);
void orc_update_q_noadmix(orc_chain* c);
void orc_update_q_admix(orc_chain* c);
void orc_update_q_metro(orc_chain* c);
void orc_update_locpriori(orc_chain* c);
void orc_update_z(orc_chain* c);
void orc_update_z_noadmix(orc_chain* c);
void orc_update_z_admix(orc_chain* c);
void orc_update_alpha(orc_chain* c);
void orc_update_a(orc_chain* c);
void orc_update_f(orc_chain* c);
void orc_record(orc_chain* c);
double orc_record_lnl(orc_chain* c);    /* RecordCPU likelihood only, no side effects */
/* LL[i*K+k] = sum log p of UpdateQNoAdmix before PolyLog (no side effects
 * on the chain except scratch). out must hold N*K doubles. */
void orc_loglik_noadmix(orc_chain* c, double* out);

/* Run nsweeps sweeps (after orc_init when init != 0) on each of n chains
 * with nthreads host threads, one chain at a time per thread: the run-level
 * parallelism of the reference's -structure_nstream (structure.cpp:2467-2499). */
void orc_sweep_many(orc_chain** cs, int n, int nsweeps, int nthreads, int init);

/* Genotypes of the data lines of a biallelic diploid VCF (the text after the
 * #CHROM line) as 2-bit codes per call, packed 16 to a word: the copies of
 * allele 1, 3 for a missing or half-missing call and for the padding. The
 * GT key is the first FORMAT key; alleles are separated by '/' or '|'
 * (the reference's VCF genotype reader, load.cpp AddVCFGenotype, for this
 * case). Returns the number of lines, or -(line number) of the first line
 * that is not biallelic diploid 0/1 data. */
int64_t orc_vcf_pack2(const char* text, size_t bytes, int n_ind, uint32_t* packed, int64_t max_loci);

/* The genotype filter of -f_dp, -f_gq, -f_ploidy (AddVCFGenotype,
 * load.cpp:3495-3566; windows parameters.cpp:743-748): a window is used when
 * its flag is non-zero. */
typedef struct {
    int32_t dp_b, dp_min, dp_max, gq_b, gq_min, gq_max, ploidy_b, ploidy_min, ploidy_max;
} orc_call_filter;
/* One typed call of v copies under the genotype filter. `call` is the call's
 * first byte in the line's rewritten calls (orc_rewrite_calls: this call's
 * kept keys up to its tab, the later calls, end at call + room), with dpid
 * and gqid among the kept keys; the call's keys are split at ':' into '\0'
 * as the reference splits them (AddVCFGenotype). Returns 1 when the call
 * becomes missing. */
int orc_call_filtered(char* call, size_t room, int dpid, int gqid, int v, const orc_call_filter* cf);
/* The loader's rewrite of a line's calls (load.cpp:2130-2257): of the FORMAT
 * keys [fmt, fmt_end) it keeps GT, DP and GQ (two bytes, then ':' or the
 * tab), each of the n calls [calls, end) keeps the values of those keys
 * joined by ':', calls joined by tabs. out (room for end - calls + 1 bytes)
 * gets the text, call_at[i] the offset of call i; dpid and gqid the indices
 * of DP and GQ among the kept keys (-1: absent). Returns the length. */
size_t orc_rewrite_calls(const char* fmt, const char* fmt_end, const char* calls, const char* end, int n,
                         char* out, size_t* call_at, int* dpid, int* gqid);
/* orc_vcf_pack2 with the genotype filter applied to each typed call
 * (cf may be null). */
int64_t orc_vcf_pack2_ex(const char* text, size_t bytes, int n_ind, uint32_t* packed, int64_t max_loci,
                         const orc_call_filter* cf);

/* The locus filter (filter.cpp MarkerDiversity over diversity.cpp
 * CalcDiversity) for a packed biallelic diploid matrix; f holds the flags
 * and windows in the layout of vp_locus_filter. keep[L], stats[L][10] (n, k,
 * ptype, bmaf, he, ho, pic, ae, I, pval). */
typedef struct {
    int32_t bmaf_b, k_b, n_b, ptype_b, he_b, ho_b, pic_b, ae_b, I_b;
    int32_t k_min, k_max, n_min, n_max;
    int32_t single;   /* statistics in float (the reference's REAL under -g_float=single), else double */
    double bmaf_min, bmaf_max, ptype_min, ptype_max, he_min, he_max, ho_min, ho_max;
    double pic_min, pic_max, ae_min, ae_max, I_min, I_max;
    int32_t pval_b;
    double pval_min, pval_max;
} orc_locus_filter;
void orc_locus_filter_pack2(const uint32_t* packed, int64_t L, int n_ind, const orc_locus_filter* f, uint8_t* keep,
                            double* stats);
/* The same windows for the general genotype layout G[L][n_ind][vmax] (any
 * ploidy, k[l] alleles per locus, up to 64): the statistics of
 * CalcDiversity over the locus' genotype table in order of first appearance
 * among the calls of Gtable (the calls before the genotype filter; NULL: G),
 * counted over G, and the HWE test with allele collapsing for genotype model
 * 0 (diversity.cpp:337-492; no test with mixed ploidy at the locus). */
void orc_locus_filter_general(const int8_t* G, const int8_t* Gtable, int64_t L, int n_ind, int vmax,
                              const int32_t* k, const orc_locus_filter* f, uint8_t* keep, double* stats);

/* WriteStructure's heterozygosity and net nucleotide distance
 * (structure.cpp:293-324) on mean frequencies freqm[K][KT] of L loci with
 * k[l] alleles each: H[K], D[K*K], Hl[K*L] (Hl may be NULL). */
void orc_divergence(const float* freqm, const int32_t* k, int64_t L, int64_t KT, int K, double* H, double* D,
                    double* Hl);

/* Output files in the reference's format (structure.cpp:86-401). */
int orc_write_structure(orc_chain* c, const char* out_prefix, int rep, int id,
                        const char* const* ind_names, const char* const* pop_names,
                        const char* const* loc_names, int decimal, int diversity);
uint32_t orc_hash_ulong_c(uint64_t v);

/* Raw access to chain state for tests; field ids follow include/vcfpop_structure.h
 * (1 Freq f32, 2 Q f32, 3 Z u16, 4 Ni i32, 5 Mi i64, 6 LL f64 (bufNK1), 7 Alpha f64,
 *  10 FreqA f32, 11 f f64, 12 F f64, 13 Di f32, 14 Metropolis ratio f64 (bufN1),
 *  15 Eta f64, 16 Gamma f64, 17 AlphaLocal f64, 18 SumAlpha f64, 19 rout f64,
 *  20 lnL trace f64, 21 MiSum i64, 22 FreqM f32). *n receives the element count. */
void* orc_field(orc_chain* c, int field, int64_t* n);
int32_t* orc_m(orc_chain* c);
int32_t* orc_nlnl(orc_chain* c);        /* records in the lnL trace (settable, up to its capacity) */
double* orc_r(orc_chain* c);
int32_t* orc_binaryq(orc_chain* c);
/* dataset arrays: 1 k, 2 off(i64), 3 vt(i64), 4 gcopies(u8), 5 galleles(u8) */
const void* orc_data_field(const orc_data* d, int field, int64_t* n);

#ifdef __cplusplus
}
#endif
#endif
