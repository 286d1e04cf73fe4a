/*
 * vcfpop STRUCTURE sweep on one GB300 -- the drop-in C ABI.
 *
 * The reference (vcfpop v1.08b) has no library boundary for this path; it is
 * reached through the -structure flag block and the BAYESIAN<REAL> step
 * methods, with the device crossing inside BAYESIAN<REAL>::*CUDA() and the
 * extern "C" helpers of src/structureCUDA.h:6-52. Each entry point below names
 * the reference interface it replaces.
 *
 * Every call returns 0 on success or a negative VP_E* code; vp_last_error()
 * gives the message of the calling thread's last failure. No call exits the
 * process (the reference's checkErrors exits, src/structureCUDA.cpp:183-196).
 * A context is thread-compatible, not thread-safe: one host thread drives it.
 */
#ifndef VCFPOP_STRUCTURE_H
#define VCFPOP_STRUCTURE_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VP_OK 0
#define VP_E_ARG (-1)      /* invalid argument or size */
#define VP_E_CUDA (-2)     /* CUDA runtime failure (message has the CUDA error) */
#define VP_E_MEM (-3)      /* device or host allocation failed */
#define VP_E_STATE (-4)    /* call not valid in the object's current state */
#define VP_E_NODEV (-5)    /* no CUDA device / extension not usable */

/* random-number streams */
#define VP_RNG_REFERENCE 0 /* the reference's xorshift streams, draw for draw */
#define VP_RNG_COUNTER 1   /* Philox counter streams: every step fully parallel */

/* likelihood form for no-admixture chains */
#define VP_FORM_PLAIN 0    /* FP32 per-individual stream over loci */
#define VP_FORM_TC 1       /* tensor-core contraction, split-BF16 log-frequencies */

/* ---- input genotypes ---------------------------------------------------- */
/* Replaces the loader's genotype store (src/function.h:53-330, GENO_READER
 * src/function.cpp:3499-3568) as the input of CalcBayesian: per call, the
 * allele index of each copy in ascending order (unphased), -1 for missing. */
typedef struct {
    int32_t n_ind;          /* N */
    int64_t n_loc;          /* L, input order (before filtering and sorting) */
    int32_t vmax;           /* copies stored per call */
    const int8_t* alleles;  /* [L][N][vmax] allele per copy, -1 = missing/absent;
                               may be NULL when packed2 is given */
    const uint32_t* packed2;/* optional biallelic-diploid form: [L][ceil(N/16)] words,
                               2 bits per call = count of allele 1, 3 = missing */
    const int32_t* ploidy;  /* [N] copies per call of each individual */
    const int32_t* n_alleles; /* [L] alleles per locus (REF + ALTs) */
    const int32_t* popid;   /* [N] population index, individuals grouped by population */
    int32_t n_pop;          /* S */
    /* optional, per input locus: the facts of the loader's genotype table,
     * which registers every call of a line before the genotype filter
     * (-f_dp, -f_gq, -f_ploidy) turns calls into missing ones
     * (src/load.cpp:2145-2230 and 3545-3566): whether the locus is
     * polymorphic (a genotype with two alleles, or two different ones:
     * ApplyFilter, src/filter.cpp:102-133) and how many genotype ids it has
     * (their bit width orders the loci, src/structure.cpp:2202-2295). From
     * vp_genotype_table on the calls before that filter; NULL: taken from
     * the calls above. */
    const uint8_t* table_poly;
    const int32_t* table_ngeno;
} vp_input;

typedef struct vp_dataset vp_dataset;

/* Filter, sort and index the loci as CalcBayesian does before its runs:
 * monomorphic loci removed (src/filter.cpp:102-131), loci sorted by genotype-id
 * bit width (src/structure.cpp:2202-2295), allele offsets (2374-2381).
 * Host-only; no GPU needed. */
int vp_dataset_prepare(const vp_input* in, vp_dataset** out);
/* The genotype-table facts of each input locus of `in` (its calls, packed2 or
 * alleles): poly[n_loc] and ngeno[n_loc] as vp_input.table_poly and
 * table_ngeno take them. Host-only. */
int vp_genotype_table(const vp_input* in, uint8_t* poly, int32_t* ngeno);

typedef struct {
    int32_t n_ind, n_pop, maxploidy, max_alleles, packed2;
    int64_t n_loc, n_alleles_total;  /* L after filtering, KT */
    int64_t coprime;
} vp_dataset_info;
int vp_dataset_info_get(const vp_dataset* ds, vp_dataset_info* info);
/* sorted position -> input locus index, L entries */
int vp_dataset_order(const vp_dataset* ds, int64_t* order);
/* Drops the caller's reference: a dataset submitted to a server stays alive
 * until its request is released or the server is closed. */
void vp_dataset_free(vp_dataset* ds);

/* ---- device context ------------------------------------------------------ */
typedef struct vp_ctx vp_ctx;
/* Upload the packed genotype matrix once (replaces CopyStructureMemory,
 * src/structureCUDA.cpp:969-1094, and its per-device replicas). The genotype
 * copy runs on the context's stream after the call returns; the context holds
 * a reference to the dataset until vp_close, and a failed copy is reported by
 * the next call that waits for the stream. */
int vp_open(const vp_dataset* ds, int device, vp_ctx** out);
/* Closing a context also destroys its chains that are still open; their
 * handles are invalid afterwards. */
int vp_close(vp_ctx* ctx);
int vp_sync(vp_ctx* ctx);

/* ---- chains ---------------------------------------------------------------- */
/* One (K, replicate) run: the fields of BAYESIAN<REAL>::ReadPar
 * (src/structure.cpp:405-464). Flags use 1 = yes, 0 = no. */
typedef struct {
    int32_t K;
    int32_t admix, locpriori, fmodel;
    int32_t nburnin, nreps, nthinning, nadmburnin;
    int32_t writelnl;
    double lambda, stdlambda, maxlambda;
    int32_t inferlambda, difflambda;
    double alpha, stdalpha, maxalpha, alphapriora, alphapriorb;
    int32_t metrofreq, inferalpha, diffalpha, uniformalpha;
    double r, maxr, epsr, epseta, epsgamma;
    double pmeanf, pstdf, stdf;
    int32_t fsame;
    uint64_t seed;          /* HashULong(g_seed + run id), see vp_run_seed() */
    int32_t rng;            /* VP_RNG_* */
    int32_t form;           /* VP_FORM_* */
} vp_params;

/* Defaults of the -structure_* block (src/parameters.cpp:584-627). */
void vp_params_default(vp_params* p);
/* The reference's per-run seed HashULong(g_seed + id) (src/structure.cpp:463). */
uint64_t vp_run_seed(int64_t g_seed, int32_t run_id);

typedef struct vp_chain vp_chain;
/* Allocate a run's device state and initialise it (InitFix, InitAdmix,
 * InitLocPriori, InitFmodel: src/structure.cpp:466-708). */
int vp_chain_create(vp_ctx* ctx, const vp_params* p, vp_chain** out);
int vp_chain_destroy(vp_chain* c);

/* Advance chains by nsweeps MCMC iterations each (the loop body of
 * BAYESIAN<REAL>::MCMC, src/structure.cpp:2124-2153). Chains that share a
 * context run their sweeps as shared launches. Asynchronous on the context's
 * stream; vp_sync waits. */
int vp_run(vp_chain** chains, int32_t nchains, int32_t nsweeps);

/* Run every remaining sweep of every chain, then Arrange()
 * (src/structure.cpp:1860-1869). */
int vp_finish(vp_chain** chains, int32_t nchains);

typedef struct {
    int32_t K, N, S, nburnin, nreps, nthinning, nr, nlnl, rlen;
    int64_t KT;
    uint64_t seed;
    double* rout;      /* [rlen] mean lnL, E[lnL^2], var, lnP(D), parameter means */
    double* lnl;       /* [nlnl] recorded likelihoods (writelnl) */
    float* Q;          /* [N*K] final admixture proportions */
    double* ancestry;  /* [N*K] normalised MiSum */
    float* freqm;      /* [K*KT] mean allele frequencies */
} vp_result;
/* Copy a finished chain's results into caller-owned buffers (any pointer
 * may be NULL to skip it). Sizes come from vp_chain_sizes. */
int vp_chain_sizes(vp_chain* c, vp_result* sizes);
int vp_chain_result(vp_chain* c, vp_result* out);

/* Output reductions of WriteStructure (src/structure.cpp:293-324) on the
 * device, from a finished chain's mean frequencies: H[K] the mean expected
 * heterozygosity of each cluster, D[K*K] the net nucleotide distance between
 * clusters, and (Hl != NULL) Hl[K*L] the per-locus heterozygosity of the
 * diversity table (-structure_diversity). Host buffers; synchronous. Sums are
 * FP64 of exact float products, in a fixed order (not the reference's
 * sequential order, so the last bits may differ). */
int vp_chain_divergence(vp_chain* c, double* H, double* D, double* Hl);

/* The result files of one finished run (after vp_finish) in the reference's
 * format: WriteStructure, src/structure.cpp:86-377, which writes
 * <prefix>.structure.k=K_rep=R_id=I.txt and, with writelnl, its .lnl.txt.
 * The numbers are the chain's (vp_chain_result) and the device reductions'
 * (vp_chain_divergence). Synchronous; host memory only. */
typedef struct {
    const char* prefix;             /* -g_output */
    int32_t rep, id;                /* replicate and run id of the file names */
    const char* const* ind_names;   /* [N] individuals in the dataset's order */
    const char* const* pop_names;   /* [S] populations (locations) */
    const char* const* loc_names;   /* [n_loc] loci in vp_input's (input) order */
    int32_t decimal;                /* -g_decimal */
    int32_t comma;                  /* -g_delimiter=comma (else tab) */
    int32_t unix_lb;                /* -g_linebreak=unix (else CR LF) */
    int32_t diversity;              /* -structure_diversity */
} vp_write_opts;
int vp_write_structure(vp_chain* c, const vp_write_opts* o);

/* ---- single steps and state access (parity tests, debugging) ------------- */
#define VP_STEP_UPDATEP 1
#define VP_STEP_UPDATEQ 2
#define VP_STEP_LOCPRIORI 3
#define VP_STEP_UPDATEZ 4
#define VP_STEP_ALPHA 5
#define VP_STEP_UPDATEA 6
#define VP_STEP_UPDATEF 7
#define VP_STEP_RECORD 8
#define VP_STEP_NEXT 9      /* m += 1 */
#define VP_STEP_LOGLIK 10   /* no-admix log-likelihood LL[N*K] only (no draws) */

#define VP_F_FREQ 1     /* float [K*KT] */
#define VP_F_Q 2        /* float [N*K] */
#define VP_F_Z 3        /* uint16 [N] */
#define VP_F_NI 4       /* int32 [K*KT] */
#define VP_F_MI 5       /* int32 [N*K] */
#define VP_F_LL 6       /* double [N*K] last log-likelihood */
#define VP_F_ALPHA 7    /* double [K] */
#define VP_F_M 8        /* int32 [1] sweep index */
#define VP_F_LNL 9      /* double [1] last sweep's likelihood */
#define VP_F_FREQA 10   /* float [3*KT] */
#define VP_F_FF 11      /* double [2*K]: f then F */
#define VP_F_LOCP 12    /* double: r, Eta[K], Gamma[S*K], AlphaLocal[S*K], SumAlpha[S] */
#define VP_F_DI 13      /* float [S*K] */
#define VP_F_METRO 14   /* double [N] last Metropolis log ratio */
/* One step at the chain's current sweep index m; VP_E_STATE once m has
 * reached nburnin (+ admixture burn-in) + nreps. vp_chain_set(VP_F_M) takes
 * indices 0..nburnin + nreps only. */
int vp_chain_step(vp_chain* c, int32_t step);
int vp_chain_get(vp_chain* c, int32_t field, void* host, size_t bytes);
int vp_chain_set(vp_chain* c, int32_t field, const void* host, size_t bytes);

/* Error code recorded by the tensor-core kernels of this context (0 = none;
 * non-zero means a pipeline wait timed out and that launch's output is void). */
int vp_tc_status(vp_ctx* ctx);

/* Launch configuration of the batched sweep's two tensor-core contractions
 * (no reference counterpart: the reference has no batched form). The
 * likelihood contraction [N x alleles] . [alleles x cluster rows] runs tiles
 * of `row_tiles` x 128 individuals by `cols` cluster rows (`piece` rows per
 * MMA), `bk` alleles per shared-memory stage, `stages` stages, the alleles
 * split `splits` ways (0: the whole-wave rule), and with `group_major` the
 * column groups of one individual tile launch next to each other. The count
 * contraction has `count_stages` and `count_group_major`. Compiled tiles
 * (bk, row_tiles, cols, piece): (64, 2, 192, 192), (64, 2, 144, 144),
 * (64, 1, 288, 144), (32, 2, 192, 192). */
typedef struct vp_tc_config {
    int32_t bk, row_tiles, cols, piece, stages, splits, group_major;
    int32_t count_stages, count_group_major;
    int32_t candidates;            /* vp_tune: configurations timed */
    float ms_likelihood;           /* vp_tune: device ms per launch, chosen configuration */
    float ms_counts;
    float ms_likelihood_default;   /* vp_tune: device ms per launch, configuration before tuning */
    float ms_counts_default;
} vp_tc_config;

/* Autotuner of the batched sweep (no reference counterpart). Times the
 * contractions of the batch of these tensor-core chains (one context) under
 * candidate configurations on the device, keeps the fastest for the batch and
 * for every later batch of the same shape (individuals, alleles, cluster
 * rows, SMs) in this process, and, when the environment variable
 * VP_TUNE_CACHE names a file, appends it there for later processes. effort
 * 0 times the current configuration only; 1 also every pipeline depth, split
 * count and CTA order of its tile; 2 every compiled tile as well. Chain state
 * is unchanged. `out` (may be null) receives the choice and the timings. */
int vp_tune(vp_chain** chains, int32_t n, int32_t effort, vp_tc_config* out);
/* Sets the configuration of the batch of these chains (timings ignored);
 * VP_E_ARG if it is not compiled in or does not fit. */
int vp_tc_configure(vp_chain** chains, int32_t n, const vp_tc_config* cfg);
/* The configuration the batch of these chains runs with. */
int vp_tc_config_get(vp_chain** chains, int32_t n, vp_tc_config* out);

/* share >= 1: the tensor-core sweep of this context runs by allele ranges,
 * one per split-K slice of the likelihood contraction, UpdateP of a range
 * beside the contraction of the range before it, with at most `share` (1-8)
 * UpdateP blocks on an SM beside one contraction CTA; share = 0 (the
 * default): UpdateP of every locus, then the whole contraction. All give the
 * same values (no reference counterpart: the reference has no batched form).
 * On GB300 the contraction slows by about UpdateP's own time when the two
 * share SMs, so the ranges save nothing there. With profiling mode 1 the
 * profiled span is the contraction's, from its first slice to its last;
 * with mode 2 it is UpdateP's, from its first range to its last. */
int vp_tc_pipeline(vp_ctx* ctx, int share);

/* Diagnostic: D[s][m][n] = sum over this split's k of A[m,k] (B0[n,k] + B1[n,k])
 * through the tensor-core kernel. A [M][K], B0/B1 [N][K] bf16 bit patterns,
 * bk (K elements per pipeline stage) 32 or 64, K % bk == 0, N % BN == 0,
 * BN % piece == 0, piece % 16 == 0, piece <= 256, mt (128-row A tiles per
 * CTA) 1 or 2, BN * mt <= 512; B1 may be NULL. D receives splits*M*N floats.
 * No reference counterpart (a test hook for the contraction kernel). */
int vp_debug_gemm_bf16(const uint16_t* A, const uint16_t* B0, const uint16_t* B1, int32_t M, int32_t N, int32_t K,
                       int32_t BN, int32_t piece, int32_t splits, int32_t stages, int32_t mt, int32_t bk, float* D);

/* Diagnostic: D[m][n] = sum_k A[m,k] B[n,k] with e4m3 operands (raw bytes,
 * A [M][K], B [N][K]) through the kernel's kind::f8f6f4 form, the one the
 * count contraction uses; K % 128 == 0. No reference counterpart. */
int vp_debug_gemm_e4m3(const uint8_t* A, const uint8_t* B, int32_t M, int32_t N, int32_t K, int32_t BN, int32_t piece,
                       int32_t stages, int32_t mt, float* D);

/* Diagnostic: average device time in ms of `iters` launches of the
 * contraction kernel on operands it allocates and fills itself (esz 2 bf16 or
 * 1 e4m3; nb B operands; mode 0 FP32 partials [splits][M][N], mode 1 int32
 * transpose [N][M] with splits == 1; bk * esz = 64 or 128). Used to choose
 * tile and pipeline parameters; no reference counterpart. */
int vp_debug_gemm_time(int32_t M, int32_t N, int32_t K, int32_t BN, int32_t piece, int32_t splits, int32_t stages,
                       int32_t mt, int32_t bk, int32_t esz, int32_t nb, int32_t mode, int32_t iters, double* ms);

/* Diagnostic (no reference counterpart; the reference's checkErrors exits):
 * the tensor-core pipeline's failure path without a device fault. Runs one
 * small contraction whose stage barriers expect 16 bytes more than their
 * copies bring, so every pipeline wait runs out after a short poll limit
 * (*status_timeout: the error code the kernel recorded, non-zero), then the
 * same contraction with the right byte counts on the same device
 * (*status_after: 0) and the largest difference of its result from the exact
 * one (*max_err_after). */
int vp_debug_gemm_wait_timeout(int32_t* status_timeout, int32_t* status_after, double* max_err_after);

/* The likelihood accumulation of UpdateQNoAdmix (src/structure.cpp:902-932;
 * the part BAYESIAN<REAL>::UpdateQNoAdmixCUDA offloads, src/structureCUDA.cpp:
 * 2123-2214) as one call on device buffers, for biallelic diploid data:
 *   geno  [L][ceil(N/16)] 2-bit codes (count of allele 1, 3 = missing)
 *   freq  [K][2L] allele frequencies, cluster-major, 2 alleles per locus
 *   ll    [N][K] output: sum over loci and copies of ln p (a zero frequency
 *         counts as 2^-1023, as in the reference's exponent-split product)
 * Asynchronous on `stream` (NULL = default stream); takes stream-ordered
 * scratch memory for the per-genotype table and per-chunk partial sums. */
int vp_loglik_packed2(const uint32_t* geno, int32_t n_ind, int64_t n_loc, const float* freq, int32_t K,
                      double* ll, void* stream);

/* vp_loglik_packed2 without any device allocation, for callers that may not
 * allocate device memory (a host framework that owns the whole device budget,
 * a plugin whose host forbids allocation on its hot path). No counterpart in
 * the reference: it is an addition of this library.
 * Scratch comes from one fixed array of VP_LOGLIK_NOALLOC_MAX_BYTES (32 MiB)
 * compiled into the library and held on every GPU that loads it until exit;
 * sizes whose table and partial sums need more are rejected with VP_E_ARG.
 * The first call on a device looks the array's device address up (once per
 * device, with that device current); make that first call before any stream
 * capture. The address is kept for the life of the process: after a
 * cudaDeviceReset (or anything else that destroys the device's primary
 * context) this entry point must not be called again in that process.
 * All calls share the array: calls that overlap on the GPU race. */
int vp_loglik_packed2_noalloc(const uint32_t* geno, int32_t n_ind, int64_t n_loc, const float* freq, int32_t K,
                              double* ll, void* stream);

/* Contexts, chains and batches take device memory from a stream-ordered
 * pool per device that keeps freed blocks for the next run (no map/unmap
 * between runs, frees do not wait for the device). This gives the kept
 * blocks back to the device (after a device synchronisation). */
int vp_release_memory(int device);

/* The CUDA stream (cudaStream_t) every launch of this context goes to. */
void* vp_stream(vp_ctx* ctx);
/* on = 1: record CUDA events around each launch of the sweep's dominant
 * kernel (the likelihood stream of the plain no-admixture form, the per-copy
 * label kernel of the admixture form, the likelihood contraction of the
 * tensor-core form), also inside the cached sweep graphs; on = 2: around the
 * tensor-core form's batched UpdateP instead; 0: off. */
int vp_prof_enable(vp_ctx* ctx, int on);
/* Synchronise, then sum the profiled kernel's durations of the last sweep. */
int vp_prof_read(vp_ctx* ctx, double* ms, int32_t* launches);

/* ---- VCF ingest on the device ---------------------------------------------
 * Replaces the genotype part of the reference's VCF loader (LoadVCF /
 * AddVCFGenotype and GENO_WRITER, src/load.cpp) for biallelic diploid data.
 * text[bytes] holds the data lines of a VCF (everything after the #CHROM
 * header line), n_ind samples per line. Writes packed[n_loc][ceil(n_ind/16)]
 * 2-bit codes (copies of allele 1; 3 = missing, also for a half-missing call
 * and the padding), the input of vp_input.packed2, and, if line_start is not
 * NULL, the n_loc + 1 byte offsets of the lines (their ends). With
 * max_loci == 0 it only counts the lines into *n_loc. A line that is not
 * biallelic, has a call that is not a diploid 0/1 genotype, or does not
 * start its FORMAT with GT fails with VP_E_ARG naming the line; such data
 * goes through a general reader. */
int vp_vcf_pack2(const char* text, size_t bytes, int32_t n_ind, int device, uint32_t* packed, int64_t max_loci,
                 int64_t* line_start, int64_t* n_loc);

/* The same ingest for any ploidy and allele count (the general genotype
 * store of vp_input.alleles): alleles[n_loc][n_ind][vmax] gets each call's
 * allele indices in ascending order (unphased, as the reference's
 * AddVCFGenotype), -1 for a missing call (any '.' copy) and for copies past
 * the call's ploidy; copies past vmax are dropped, as the reference's reader
 * keeps the ploidy of each individual's first call. n_alleles[n_loc] = REF +
 * ALTs; ploidy[n_ind] = the copies of each sample's call on the first line.
 * vmax is 1..16; allele indices above 127 and malformed lines fail with
 * VP_E_ARG naming the line. With max_loci == 0 it only counts the lines. */
int vp_vcf_parse(const char* text, size_t bytes, int32_t n_ind, int32_t vmax, int device, int8_t* alleles,
                 int32_t* n_alleles, int32_t* ploidy, int64_t max_loci, int64_t* line_start, int64_t* n_loc);

/* The reference's genotype filter (-f with -f_dp, -f_gq, -f_ploidy;
 * AddVCFGenotype, src/load.cpp:3545-3566, flags src/parameters.cpp:743-748):
 * a typed call becomes missing when its number of copies is outside
 * [ploidy_min, ploidy_max], or when the FORMAT column has a DP (GQ) key, the
 * call has at least that many keys, and its value read as the reference's
 * ReadIntegerKeep reads it (characters up to the first digit or '-' are
 * skipped, so a '.' value takes the next number on the line; here the scan
 * stops at the end of the line, with 0) is outside the window: DP compared as
 * unsigned (-1 never filters), GQ as signed (-1 never filters). FORMAT keys
 * are matched ignoring case. A window is used when its flag is non-zero. */
typedef struct {
    int32_t dp_b, dp_min, dp_max;
    int32_t gq_b, gq_min, gq_max;
    int32_t ploidy_b, ploidy_min, ploidy_max;
} vp_call_filter;
/* vp_vcf_pack2 and vp_vcf_parse with the genotype filter applied to every
 * call as it is decoded (cf may be null: no filter). */
int vp_vcf_pack2_ex(const char* text, size_t bytes, int32_t n_ind, int device, uint32_t* packed, int64_t max_loci,
                    int64_t* line_start, int64_t* n_loc, const vp_call_filter* cf);
int vp_vcf_parse_ex(const char* text, size_t bytes, int32_t n_ind, int32_t vmax, int device, int8_t* alleles,
                    int32_t* n_alleles, int32_t* ploidy, int64_t max_loci, int64_t* line_start, int64_t* n_loc,
                    const vp_call_filter* cf);

/* Locus filter of the reference (-f_bmaf, -f_k, -f_n, -f_ptype, -f_he, -f_ho,
 * -f_pic, -f_ae, -f_I, -f_pval: MarkerDiversity, src/filter.cpp:485-507, on the
 * statistics of DIVERSITY::CalcDiversity, src/diversity.cpp:144-311). Each
 * window is used when its flag is set; a locus fails when no call is typed
 * or any used statistic falls outside its window (a NaN statistic passes,
 * as in the reference). -f_pval uses the HWE G-test's p-value: NaN (the
 * locus passes) when an expected genotype count is below 5. */
typedef struct {
    int32_t bmaf_b, k_b, n_b, ptype_b, he_b, ho_b, pic_b, ae_b, I_b;
    int32_t k_min, k_max, n_min, n_max;
    int32_t single;   /* statistics in float (the reference's REAL under -g_float=single), else double */
    double bmaf_min, bmaf_max, ptype_min, ptype_max, he_min, he_max, ho_min, ho_max;
    double pic_min, pic_max, ae_min, ae_max, I_min, I_max;
    int32_t pval_b;   /* -f_pval: the p-value of the HWE G-test (CalcDiversity, src/diversity.cpp:337-492) */
    double pval_min, pval_max;
} vp_locus_filter;
#define VP_LOCUS_STATS 10  /* n, k, ptype, bmaf, he, ho, pic, ae, I, pval */
/* The statistics and the pass flag of every locus of a packed biallelic
 * diploid matrix (packed[n_loc][ceil(n_ind/16)], as vp_input.packed2) on the
 * device: keep[n_loc] = 1 if the locus passes; stats[n_loc][VP_LOCUS_STATS]
 * (optional) in double, NaN where the reference leaves a statistic
 * undefined (fewer than 2 alleles). Host buffers; synchronous. */
int vp_locus_filter_pack2(const uint32_t* packed, int64_t n_loc, int32_t n_ind, const vp_locus_filter* f, int device,
                          uint8_t* keep, double* stats);
/* The same for the general genotype layout (vp_input.alleles: [n_loc][n_ind]
 * [vmax] allele indices, -1 missing; any ploidy up to 10, n_alleles[l] up to
 * 64). The statistics are CalcDiversity's over the locus' genotype table in
 * order of first appearance (the REAL sums run in that order) among the
 * calls of alleles_table (the calls before the genotype filter, same layout;
 * NULL: alleles), counted over alleles; the HWE p-value comes from the test
 * with allele collapsing (src/diversity.cpp:337-492) for the default
 * genotype model (no -f_model), NaN with mixed ploidy at the locus, and the
 * chi-square upper tail by the regularized incomplete gamma function. The
 * tables live in device scratch sized for n_ind distinct genotypes, so any
 * number of distinct genotypes at a locus is accepted. */
int vp_locus_filter_general(const int8_t* alleles, const int8_t* alleles_table, int64_t n_loc, int32_t n_ind,
                            int32_t vmax, const int32_t* n_alleles, const vp_locus_filter* f, int device,
                            uint8_t* keep, double* stats);

/* ---- serving: many independent runs on one device ------------------------
 * Replaces the reference's run scheduling (BAYESIAN<REAL>::CalcBayesian and
 * BayesianThread, src/structure.cpp:2337-2501, with ManageCUDA's device
 * slotting, src/structure.cpp:710-756), where each run owns one host thread
 * and one device slot for its whole length.
 * A server owns one scheduler thread on one device. Submitted runs queue in
 * arrival order and start when their device bytes (dataset upload plus chain
 * state) fit under mem_budget and fewer than max_active runs are active; each
 * active run has its own context. Small runs are batched: the runs of one
 * size class sweep together in a cohort, one launch per kernel for all of
 * them, joining and leaving it as they start and finish; larger runs keep
 * their own streams. The scheduler keeps up to two chunks of `chunk` sweeps
 * queued per cohort and per run, so runs of every size overlap on the GPU.
 * Results stay on the device until the run is released.
 * The dataset passed to vp_submit must stay alive until the run is done. */
typedef struct vp_server vp_server;
#define VP_REQ_QUEUED 0
#define VP_REQ_RUNNING 1
#define VP_REQ_DONE 2
#define VP_REQ_FAILED 3
typedef struct {
    int32_t state;            /* VP_REQ_* */
    int32_t rc;               /* status of a failed run */
    int64_t sweeps_issued, sweeps_total;
    int64_t device_bytes;     /* bytes the run holds (or will hold) on the device */
    double t_submit, t_start, t_done;   /* seconds since vp_server_open */
    char error[256];
} vp_request_info;
/* mem_budget 0 = 90% of the device's free memory at open; max_active 0 = 64;
 * chunk 0 = 16 sweeps. */
int vp_server_open(int device, int64_t mem_budget, int32_t max_active, int32_t chunk, vp_server** out);
/* Queue one run (a chain of p on ds); *id identifies it. A run that could
 * never fit under the budget is rejected with VP_E_MEM. */
int vp_submit(vp_server* s, const vp_dataset* ds, const vp_params* p, int64_t* id);
/* Non-blocking state of a run. */
int vp_poll(vp_server* s, int64_t id, vp_request_info* info);
/* Wait until the run is done or failed, at most timeout_s seconds (< 0: no
 * limit); returns VP_E_STATE on time-out. */
int vp_wait(vp_server* s, int64_t id, double timeout_s, vp_request_info* info);
/* The finished run's chain, for vp_chain_sizes / vp_chain_result /
 * vp_chain_get; valid until vp_release. */
int vp_request_chain(vp_server* s, int64_t id, vp_chain** chain);
/* Free a finished run's device memory and forget it. */
int vp_release(vp_server* s, int64_t id);
/* Stop the scheduler (active runs are abandoned) and free everything. */
int vp_server_close(vp_server* s);
/* on = 1 (the default): runs whose sweep is small (expected device time of a
 * sweep below about 300 us) are swept in cohorts of their size class, one
 * launch per kernel for all of them (vp_cohort_*); on = 0: every run on its
 * own stream. Set before the first vp_submit. */
int vp_server_set_batching(vp_server* s, int32_t on);
/* Kernel launches the scheduler has queued, and the run-sweeps they carry. */
int vp_server_stats(vp_server* s, int64_t* launches, int64_t* run_sweeps);

/* ---- cohorts: runs of different datasets in shared launches --------------
 * Replaces, with the serving loop below, the reference's scheduling of one run
 * per host thread and device slot (src/structure.cpp:2398-2413, 2467-2501;
 * ManageCUDA 710-756). A cohort sweeps plain-form chains of any contexts on
 * one device -- each with its own individuals, loci, clusters and model -- as
 * one launch per kernel of the sweep (one per compiled variant in use) that
 * covers every member's blocks, captured once into a CUDA graph and replayed.
 * Each member's blocks do exactly the work of that chain's own launch, so its
 * results are the same bit for bit. A member whose sweeps are all done idles
 * (its blocks return at once) until it is removed.
 * While a chain is in a cohort it advances only with the cohort (vp_run on it
 * fails), and neither the chain nor its context can be destroyed: remove it
 * first (vp_cohort_set without it). Operations on a member's own context
 * stream (results, vp_finish's Arrange) are ordered after the cohort's
 * queued sweeps. */
typedef struct vp_cohort vp_cohort;
int vp_cohort_open(int device, vp_cohort** out);
/* The members (n = 0: none); the sweep graph is captured again. */
int vp_cohort_set(vp_cohort* h, vp_chain** chains, int32_t n);
/* Queue nsweeps sweeps of every member (each stops at its own end); asynchronous. */
int vp_cohort_run(vp_cohort* h, int32_t nsweeps);
int vp_cohort_sync(vp_cohort* h);
void* vp_cohort_stream(vp_cohort* h);
/* Kernel launches queued so far; *per_sweep (may be NULL) the launches of one sweep. */
int64_t vp_cohort_launches(vp_cohort* h, int32_t* per_sweep);
int vp_cohort_close(vp_cohort* h);

/* Kernel launches issued by this library since the context was opened. */
int64_t vp_launch_count(vp_ctx* ctx);

const char* vp_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
