// Host side of the device STRUCTURE sweep: contexts, chain state, the launch
// sequence of one sweep, CUDA-graph replay, and the C ABI.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "vp_internal.h"
#include "vp_kernels.cuh"
#include "vp_tc.cuh"

using namespace vp;

struct TcOperands {
    bool ready = false;
    int bk = 64;              // bf16 K elements per pipeline stage of the likelihood contraction
    int bk8 = 128;            // e4m3 K elements per stage of the count contraction
    int64_t Apad = 0, Npad = 0;
    __nv_bfloat16* C = nullptr;   // [Npad][Apad] bf16 counts: the likelihood contraction's A
    uint8_t* CT = nullptr;        // [Apad][Npad] e4m3 counts: the count contraction's A
    float* logpbar = nullptr;
    double* Bc = nullptr;
    int* err = nullptr;
    CUtensorMap mapC, mapCT;
};

// one kernel launch of a chain's sweep: the kernel, its launch shape and its
// scalar arguments (nint ints, or nint == -1: the null accumulator of
// k_record_sweep); the kernel's first argument is the chain's device header
// and its last the cohort block map (null here)
struct SweepRec {
    struct vp_chain* c;
    const void* fn;
    const char* name;
    dim3 grid, block;
    size_t smem;
    int nint, i0, i1;
};

struct vp_ctx {
    int device = 0;
    // set while a cohort records this context's chains' sweeps: launches are
    // appended here instead of issued
    std::vector<SweepRec>* rec = nullptr;
    cudaStream_t stream = nullptr;
    DevData D{};
    std::vector<void*> allocs;
    std::vector<vp_chain*> chains;   // open chains: vp_close destroys those left
    // the dataset whose pinned genotype words the upload reads: held (one
    // reference) until vp_close, so vp_open need not wait for the copy
    const vp_dataset* hold = nullptr;
    int64_t launches = 0;
    int32_t N = 0, S = 0, maxK = 0, maxploidy = 0, packed2 = 0;
    int64_t L = 0, KT = 0;
    int nsm = 132;
    TcOperands tc;
    struct TcBatch* batch = nullptr;
    // cached graph of one sweep of a set of plain-form chains
    std::vector<vp_chain*> pg_chains;
    cudaGraphExec_t pg = nullptr;
    int pg_nodes = 0;
    // CUDA events around the dominant kernel of each sweep (likelihood stream
    // or contraction), captured into the graphs when enabled
    int prof = 0, prof_next = 0, prof_used = 0;
    std::vector<cudaEvent_t> prof_ev;
    // tensor-core sweep by allele ranges: UpdateP of one range beside the
    // likelihood contraction of the range before it, at most this many
    // UpdateP blocks on an SM beside a contraction CTA (0, the default: one
    // pass; vp_tc_pipeline)
    int tc_pipeline = 0;
    // branch streams and events of a captured sweep's fork and join
    std::vector<cudaStream_t> fork;
    std::vector<cudaEvent_t> fork_ev;
    const void* last_gemm = nullptr;    // kernel of the latest contraction launch
};

struct vp_chain {
    vp_ctx* ctx = nullptr;
    vp_params P{};
    DevChain h{};
    DevChain* d = nullptr;
    void* mem = nullptr;
    int total = 0;        // sweeps of the run: nburnin (+ admixture burn-in) + nreps
    int issued = 0;       // sweeps launched so far
    int kc = 16, kgroups = 1;
    bool ll_fma = false;   // likelihood stream in the FMA form (else the table form)
    bool arranged = false;
    double* ancestry = nullptr;
    cudaGraphExec_t graph = nullptr;
    int graph_nodes = 0;
    int32_t* own_ni = nullptr;   // the chain's own Ni (a tensor-core batch may redirect Ni)
    // the initial allele counts (the no-admixture UpdateZ of InitFix) are
    // not computed yet: a tensor-core chain leaves them to its batch, which
    // counts every chain in one count contraction
    bool counts_pending = false;
    // a chain made for a tensor-core batch carves the plain form's likelihood
    // table and chunk partials (lt, LLp) only on its first plain-form use
    bool plain_lazy = false;
    void* plain_mem = nullptr;
    // the cohort whose shared launches sweep this chain (vp_cohort_set)
    struct vp_cohort* cohort = nullptr;
};

// launch configuration of a batch's two contractions: the likelihood
// contraction's tile (K elements per stage, 128-row tiles of individuals and
// cluster rows per CTA, rows per MMA), pipeline depth, split-K count and CTA
// order, and the count contraction's pipeline depth and CTA order
struct TcChoice {
    int bk1 = 64, mt1 = 2, bn1 = 192, piece1 = 192, st1 = 2, splits = 0 /* 0: whole waves */, gm1 = 0;
    int st2 = 4, gm2 = 1;
};

// a set of no-admixture chains sharing one context, swept together with the
// tensor-core contraction
struct TcBatch {
    std::vector<vp_chain*> chains;
    void* mem = nullptr;
    DevChain* dchains = nullptr;
    DevChain** dptrs = nullptr;     // each chain's own device header
    double* lnlrec = nullptr;       // [chain][block] sums of a recorded sweep's lnP(D)
    int32_t *rowchain = nullptr, *rowk = nullptr, *row0 = nullptr;
    // cluster rows padded to whole 192-row column groups of the count
    // contraction (BN cluster rows per CTA, piece per MMA)
    int R = 0, Rpad = 0, G = 0, BN = 192, piece = 192, splits = 1;
    // the count contraction's 128-row A tiles per CTA (compiled in)
    int mt2 = 2;
    TcChoice cfg;
    int G1 = 0;               // column groups of the likelihood contraction (Rpad / cfg.bn1)
    __nv_bfloat16 *Whi = nullptr, *Wlo = nullptr;
    uint8_t* OH = nullptr;
    float* LLpart = nullptr;
    int32_t* NiAll = nullptr;
    CUtensorMap mapC1, mapWhi, mapWlo, mapOH;
    cudaGraphExec_t graph = nullptr;
    int graph_nodes = 0;
    const void* gemm1_fn = nullptr;     // the likelihood contraction's kernel in the captured sweep
    // groups of consecutive chains for the label draw: {first chain, end
    // chain, first row, rows}, and the most rows of a group
    int4* sgrp = nullptr;
    int nsgrp = 0, sgrp_rows = 0;
};

namespace {
void free_batch(vp_ctx* x);
int run_tc(vp_ctx* x, vp_chain** cs, int n, int nsweeps);
int launch_counts_gemm(vp_ctx* x, int32_t* out = nullptr);
tc::BatchDev batch_dev(vp_ctx* x);

#define CK(call)                                                                  \
    do {                                                                          \
        cudaError_t e_ = (call);                                                  \
        if (e_ != cudaSuccess) {                                                  \
            vp_set_error("%s failed: %s", #call, cudaGetErrorString(e_));         \
            return VP_E_CUDA;                                                     \
        }                                                                         \
    } while (0)

int check_launch(vp_ctx* ctx, const char* what) {
    ctx->launches++;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        vp_set_error("launch of %s failed: %s", what, cudaGetErrorString(e));
        return VP_E_CUDA;
    }
    return VP_OK;
}
#define VP_UNPACK(...) __VA_ARGS__
#define LAUNCH(ctx, name, cfg, args)            \
    do {                                        \
        name<<<VP_UNPACK cfg>>> args;           \
        int rc_ = check_launch(ctx, #name);     \
        if (rc_) return rc_;                    \
    } while (0)

// one launch of a sweep kernel for one chain (or, while a cohort records, its
// record): argument list (chain header, the scalar arguments, block map)
int sweep_launch(vp_chain* c, const void* fn, const char* name, dim3 g, dim3 b, size_t sm, int nint, int i0 = 0,
                 int i1 = 0) {
    vp_ctx* x = c->ctx;
    if (x->rec) {
        x->rec->push_back(SweepRec{c, fn, name, g, b, sm, nint, i0, i1});
        return VP_OK;
    }
    const DevChain* d = c->d;
    const int4* map = nullptr;
    double* none = nullptr;
    void* args[4];
    int k = 0;
    args[k++] = (void*)&d;
    if (nint < 0) args[k++] = (void*)&none;
    if (nint >= 1) args[k++] = (void*)&i0;
    if (nint >= 2) args[k++] = (void*)&i1;
    args[k++] = (void*)&map;
    cudaLaunchKernel(fn, g, b, args, sm, x->stream);
    return check_launch(x, name);
}
#define SL(c, fn, g, b, sm, ...)                                                                   \
    do {                                                                                           \
        int rc_ = sweep_launch(c, (const void*)&fn, #fn, dim3 g, dim3 b, (size_t)(sm), __VA_ARGS__); \
        if (rc_) return rc_;                                                                       \
    } while (0)

// The library's device memory: one stream-ordered pool per device that keeps
// freed blocks for the next context, chain or batch, so repeated runs do not
// pay to map and unmap memory (and a free does not wait for the device);
// vp_release_memory gives the kept blocks back.
cudaMemPool_t lib_pool(int device) {
    static std::mutex mu;
    static std::vector<cudaMemPool_t> pools;
    std::lock_guard<std::mutex> lk(mu);
    if ((int)pools.size() <= device) pools.resize(device + 1, nullptr);
    if (!pools[device]) {
        cudaMemPoolProps props{};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = device;
        if (cudaMemPoolCreate(&pools[device], &props) != cudaSuccess) return nullptr;
        uint64_t keep = UINT64_MAX;
        cudaMemPoolSetAttribute(pools[device], cudaMemPoolAttrReleaseThreshold, &keep);
    }
    return pools[device];
}
cudaError_t dev_alloc(void** p, size_t bytes, int device, cudaStream_t s) {
    cudaMemPool_t pool = lib_pool(device);
    if (!pool) return cudaErrorMemoryAllocation;
    return cudaMallocFromPoolAsync(p, bytes, pool, s);
}
void dev_free(void* p, cudaStream_t s) {
    if (p) cudaFreeAsync(p, s);
}

template <typename T>
int upload(vp_ctx* ctx, const T* host, size_t n, const T** dev) {
    if (n == 0) { *dev = nullptr; return VP_OK; }
    void* p = nullptr;
    cudaError_t e = dev_alloc(&p, n * sizeof(T), ctx->device, ctx->stream);
    if (e != cudaSuccess) { vp_set_error("device allocation of %zu bytes failed: %s", n * sizeof(T), cudaGetErrorString(e)); return VP_E_MEM; }
    ctx->allocs.push_back(p);
    CK(cudaMemcpyAsync(p, host, n * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
    *dev = (const T*)p;
    return VP_OK;
}

inline unsigned cdiv(int64_t a, int64_t b) { return (unsigned)((a + b - 1) / b); }

// begin/end markers around one launch of the profiled kernel: the dominant
// kernel (profiling mode 1) or the tensor-core form's UpdateP (mode 2)
enum { PROF_DOMINANT = 1, PROF_UPDATEP_TC = 2 };
void prof_mark(vp_ctx* x, bool begin, int kind = PROF_DOMINANT) {
    if (x->prof != kind || x->rec) return;
    int idx = x->prof_next * 2 + (begin ? 0 : 1);
    while ((int)x->prof_ev.size() <= idx) {
        cudaEvent_t e;
        cudaEventCreate(&e);
        x->prof_ev.push_back(e);
    }
    // external: captured into a graph as an event-record node that fires on
    // every replay (a plain record would only become a capture dependency)
    cudaEventRecordWithFlags(x->prof_ev[idx], x->stream, cudaEventRecordExternal);
    if (!begin) { x->prof_next++; x->prof_used = std::max(x->prof_used, x->prof_next); }
}

// bump allocator over one device allocation
// writes a chain's device header from the launch's own parameter (no host
// copy to stage)
__global__ void k_set_chain(DevChain* dst, const DevChain h) {
    static_assert(sizeof(DevChain) % 4 == 0 && sizeof(DevChain) <= 4000, "DevChain as a kernel parameter");
    const uint32_t* a = reinterpret_cast<const uint32_t*>(&h);
    uint32_t* d = reinterpret_cast<uint32_t*>(dst);
    for (int j = threadIdx.x; j < (int)(sizeof(DevChain) / 4); j += blockDim.x) d[j] = a[j];
}

struct Carve {
    char* base;
    size_t off = 0;
    template <typename T>
    T* take(int64_t n) {
        off = (off + 255) & ~(size_t)255;
        T* p = reinterpret_cast<T*>(base ? base + off : nullptr);
        off += (size_t)std::max<int64_t>(n, 1) * sizeof(T);
        return p;
    }
};

int kc_for(int K) { return K <= 4 ? 4 : K <= 8 ? 8 : K <= 12 ? 12 : 16; }

// likelihood-stream columns and individuals per CTA: the FMA form (2-bit
// data and the cluster counts lf_form picks) or the table form
int ll_kc(bool fma, int K) { return fma ? lf_kc(K) : kc_for(K); }
int ll_individuals(bool fma, int kc) { return fma ? lf_individuals(kc) : LT_BLOCK; }

// resident CTAs per SM of the FMA form's instantiation for kc columns (its
// registers and shared memory), looked up once per process
int lf_resident(int kc) {
    static std::mutex mu;
    static int occ[17] = {0};
    std::lock_guard<std::mutex> lk(mu);
    if (kc < 1 || kc > 16) return 1;
    if (!occ[kc]) {
        const void* fn = nullptr;
        switch (kc) {
            case 1: fn = (const void*)k_loglik_fma<1>; break;
            case 2: fn = (const void*)k_loglik_fma<2>; break;
            case 6: fn = (const void*)k_loglik_fma<6>; break;
            default: fn = (const void*)k_loglik_fma<14>; break;
        }
        int n = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, LL_BLOCK, 0) != cudaSuccess || n < 1) {
            cudaGetLastError();
            n = 1;
        }
        occ[kc] = n;
    }
    return occ[kc];
}

// locus chunks of the likelihood stream. The FMA form fills whole waves of
// its resident CTAs (one wave when the chunks stay long enough: no tail, and
// few chunk partials for the label draw to sum); the table form runs about 12
// of its small CTAs per SM, enough warps to cover the genotype stream's
// latency. Chunks hold at least 64 loci.
int64_t ll_chunks(bool fma, int kc, int kgroups, int32_t N, int64_t L, int nsm) {
    const int64_t nbi = cdiv(N, ll_individuals(fma, kc)) * (int64_t)kgroups;
    const int64_t maxc = std::max<int64_t>(1, L / 64);
    if (!fma) return std::min(std::max<int64_t>(1, (int64_t)nsm * 12 * LL_BLOCK / LT_BLOCK / std::max<int64_t>(nbi, 1)), maxc);
    const int64_t slots = (int64_t)nsm * lf_resident(kc);
    int64_t nch = std::max<int64_t>(1, slots / nbi);
    if (nch > maxc) nch = maxc;
    return nch;
}

int launch_loglik(vp_chain* c, int force) {
    vp_ctx* x = c->ctx;
    prof_mark(x, true);
    struct End { vp_ctx* x; ~End() { prof_mark(x, false); } } end_{x};
    if (c->ll_fma) {
        const dim3 g(cdiv(x->N, lf_individuals(c->kc)), c->h.nchunk, c->kgroups);
        switch (c->kc) {
            case 1: SL(c, k_loglik_fma<1>, (g), (LL_BLOCK), 0, 2, c->kgroups, force); break;
            case 2: SL(c, k_loglik_fma<2>, (g), (LL_BLOCK), 0, 2, c->kgroups, force); break;
            case 6: SL(c, k_loglik_fma<6>, (g), (LL_BLOCK), 0, 2, c->kgroups, force); break;
            default: SL(c, k_loglik_fma<14>, (g), (LL_BLOCK), 0, 2, c->kgroups, force); break;
        }
        return VP_OK;
    }
    dim3 g(cdiv(x->N, LT_BLOCK), c->h.nchunk, c->kgroups);
    switch (c->kc) {
        case 4: SL(c, k_loglik<4>, (g), (LT_BLOCK), 0, 2, c->kgroups, force); break;
        case 8: SL(c, k_loglik<8>, (g), (LT_BLOCK), 0, 2, c->kgroups, force); break;
        case 12: SL(c, k_loglik<12>, (g), (LT_BLOCK), 0, 2, c->kgroups, force); break;
        default: SL(c, k_loglik<16>, (g), (LT_BLOCK), 0, 2, c->kgroups, force); break;
    }
    return VP_OK;
}

size_t count_smem(const vp_chain* c) {
    if (c->ctx->packed2) return (size_t)COUNT_WARPS * 2 * c->P.K * 32 * sizeof(int32_t);
    return (size_t)COUNT_WARPS * c->P.K * c->ctx->maxK * sizeof(int32_t);
}
size_t zadm_smem(const vp_chain* c) {
    const int K = c->P.K, MK = c->ctx->maxK;
    return (size_t)ZA_LC * MK * (K | 1) * 4 + (size_t)ZA_LC * K * MK * 4;
}
// instantiations of the per-copy label kernel: exact cluster counts up to
// 12, then padded sizes
#define VP_ZADM_EXACT(X) X(1) X(2) X(3) X(4) X(5) X(6) X(7) X(8) X(9) X(10) X(11) X(12)
#define VP_ZADM_PADDED(X) X(16) X(32) X(64)

int launch_zadm_ctr(vp_chain* c, int force) {
    vp_ctx* x = c->ctx;
    dim3 g(cdiv(x->N, ZA_WARPS * 32), cdiv(x->L, c->h.zadm_lc), 1);
    size_t sm = zadm_smem(c);
    prof_mark(x, true);
    struct End { vp_ctx* x; ~End() { prof_mark(x, false); } } end_{x};
    const int K = c->P.K;
#define VP_ZE(n) \
    if (K == n) { SL(c, (k_update_z_admix_ctr<n, true>), (g), (ZA_WARPS * 32), sm, 1, force); return VP_OK; }
#define VP_ZP(n) \
    if (K <= n) { SL(c, (k_update_z_admix_ctr<n, false>), (g), (ZA_WARPS * 32), sm, 1, force); return VP_OK; }
    VP_ZADM_EXACT(VP_ZE)
    VP_ZADM_PADDED(VP_ZP)
#undef VP_ZE
#undef VP_ZP
    vp_set_error("K = %d out of range", K);
    return VP_E_ARG;
}

// the Metropolis ratio kernel on the same K instantiations as the label kernel
int launch_metro_ratio(vp_chain* c, int force) {
    vp_ctx* x = c->ctx;
    const dim3 g(cdiv(x->N, 256), cdiv(x->L, c->h.zadm_lc), 1);
    const size_t sm = (size_t)ZA_LC * x->maxK * (c->P.K | 1) * 4;
    const int K = c->P.K;
#define VP_ME(n) \
    if (K == n) { SL(c, (k_metro_ratio<n, true>), (g), (256), sm, 1, force); return VP_OK; }
#define VP_MP(n) \
    if (K <= n) { SL(c, (k_metro_ratio<n, false>), (g), (256), sm, 1, force); return VP_OK; }
    VP_ZADM_EXACT(VP_ME)
    VP_ZADM_PADDED(VP_MP)
#undef VP_ME
#undef VP_MP
    vp_set_error("K = %d out of range", K);
    return VP_E_ARG;
}

// true the first time it is called for a device (kernel attributes belong to
// each device's context); safe from several host threads
bool first_on_device(std::mutex& mu, std::vector<char>& seen, int device) {
    std::lock_guard<std::mutex> lk(mu);
    if ((int)seen.size() <= device) seen.resize(device + 1, 0);
    if (seen[device]) return false;
    seen[device] = 1;
    return true;
}

void set_smem_limits(int device) {
    static std::mutex mu;
    static std::vector<char> seen;
    if (!first_on_device(mu, seen, device)) return;
    const int big = 200 * 1024;
    cudaFuncSetAttribute(k_count_noadmix, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
    cudaFuncSetAttribute(k_count_packed<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
    cudaFuncSetAttribute(k_count_packed<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
    cudaFuncSetAttribute(k_count_packed<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
#define VP_ZE(n) cudaFuncSetAttribute(k_update_z_admix_ctr<n, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
#define VP_ZP(n) cudaFuncSetAttribute(k_update_z_admix_ctr<n, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
    VP_ZADM_EXACT(VP_ZE)
    VP_ZADM_PADDED(VP_ZP)
#undef VP_ZE
#undef VP_ZP
#define VP_ME(n) cudaFuncSetAttribute(k_metro_ratio<n, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
#define VP_MP(n) cudaFuncSetAttribute(k_metro_ratio<n, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
    VP_ZADM_EXACT(VP_ME)
    VP_ZADM_PADDED(VP_MP)
#undef VP_ME
#undef VP_MP
}

// the no-admixture counts: from bit planes on 2-bit packed data with at
// least 32 words per locus (N >= 512) when the masks of a cluster group fit in
// shared memory, else the per-individual pass
int launch_count(vp_chain* c, int force) {
    vp_ctx* x = c->ctx;
    const int K = c->P.K;
    if (x->packed2) {
        const int kc = K <= 4 ? 4 : K <= 8 ? 8 : 16;
        const int kgroups = (K + kc - 1) / kc;
        const size_t sm = (size_t)kc * ((x->D.Nw + 1) / 2) * 4 + kc * 4;   // masks per word pair, sizes
        if (sm <= 200 * 1024 && x->D.Nw >= 32) {
            const dim3 g((unsigned)std::min<int64_t>(cdiv(x->L, 8), (int64_t)x->nsm * 8), 1, (unsigned)kgroups);
            switch (kc) {
                case 4: SL(c, k_count_packed<4>, (g), (256), sm, 2, kgroups, force); break;
                case 8: SL(c, k_count_packed<8>, (g), (256), sm, 2, kgroups, force); break;
                default: SL(c, k_count_packed<16>, (g), (256), sm, 2, kgroups, force); break;
            }
            return VP_OK;
        }
    }
    SL(c, k_count_noadmix, (cdiv(x->L, COUNT_WARPS), 1, 1), (COUNT_WARPS * 32), count_smem(c), 1, force);
    return VP_OK;
}

int launch_step(vp_chain* c, int step, int force) {
    vp_ctx* x = c->ctx;
    const vp_params& P = c->P;
    const int K = P.K;
    const bool ref = P.rng == VP_RNG_REFERENCE;
    switch (step) {
        case VP_STEP_UPDATEP:
            if (ref) SL(c, k_update_p_ref, (1, 1, 1), (128), 0, 0);
            else SL(c, k_update_p_ctr, (cdiv((int64_t)K * x->L, 256), 1, 1), (256), 0, 0);
            return VP_OK;
        case VP_STEP_LOGLIK: {
            int rc = launch_loglik(c, 1);
            if (rc) return rc;
            SL(c, k_sample_noadmix, (c->h.nsampblk, 1, 1), (SAMPLE_BLOCK), 0, 1, 1);
            return VP_OK;
        }
        case VP_STEP_UPDATEQ: {
            const unsigned gi = cdiv(x->N, 256);
            if (!P.admix) {
                int rc = launch_loglik(c, force);
                if (rc) return rc;
                SL(c, k_sample_noadmix, (ref ? 1 : c->h.nsampblk, 1, 1), (SAMPLE_BLOCK), 0, 1, 0);
                if (c->h.nadmburnin > 0) SL(c, k_update_q_admix, (ref ? 1 : gi, 1, 1), (ref ? 32 : 256), 0, 1, 0);
            } else {
                SL(c, k_update_q_admix, (ref ? 1 : gi, 1, 1), (ref ? 32 : 256), 0, 1, 0);
                if (P.metrofreq > 0) {
                    SL(c, k_metro_propose, (ref ? 1 : gi, 1, 1), (ref ? 32 : 256), 0, 1, 0);
                    if (int rc = launch_metro_ratio(c, 0)) return rc;
                    SL(c, k_metro_accept, (ref ? 1 : gi, 1, 1), (ref ? 32 : 256), 0, 1, 0);
                }
            }
            return VP_OK;
        }
        case VP_STEP_LOCPRIORI:
            if (P.locpriori) SL(c, k_update_locpriori, (1, 1, 1), (32), 0, 0);
            return VP_OK;
        case VP_STEP_UPDATEZ:
            if (!P.admix)
                if (int rc = launch_count(c, 0)) return rc;
            if (P.admix || c->h.nadmburnin > 0) {
                SL(c, k_zero_counts, (std::min<unsigned>(1024, cdiv((int64_t)K * x->KT, 256)), 1, 1), (256), 0, 1, 0);
                if (ref) SL(c, k_update_z_admix_ref, (cdiv(x->L, 128), 1, 1), (128), 0, 1, 0);
                else if (int rc = launch_zadm_ctr(c, 0)) return rc;
            }
            return VP_OK;
        case VP_STEP_ALPHA:
            if ((P.inferalpha && (P.admix || c->h.nadmburnin > 0)) || (P.locpriori && P.admix)) {
                SL(c, k_logprod_q, (ref ? std::max(1, (x->S * K + 255) / 256) : LPQ_BLOCKS, 1, 1), (256), 0, 0);
                SL(c, k_update_alpha, (1, 1, 1), (128), 0, 0);
            }
            return VP_OK;
        case VP_STEP_UPDATEA:
            if (P.fmodel) {
                if (ref) SL(c, k_update_a, (1, 1, 1), (32), 0, 0);
                else SL(c, k_update_a, (cdiv(x->L, 128), 1, 1), (128), 0, 0);
            }
            return VP_OK;
        case VP_STEP_UPDATEF:
            if (P.fmodel) SL(c, k_update_f, (1, 1, 1), (256), 0, 0);
            return VP_OK;
        case VP_STEP_RECORD:
            // single steps (parity tests): Record alone, without the advance
            LAUNCH(x, k_record, (dim3(1, 1, 1), 256, 0, x->stream), (c->d));
            LAUNCH(x, k_accumulate, (dim3(std::min<unsigned>(1024, cdiv((int64_t)K * x->KT, 256)), 1, 1), 256, 0, x->stream), (c->d, 0));
            return VP_OK;
        case VP_STEP_NEXT:
            LAUNCH(x, k_advance, (dim3(1, 1, 1), 32, 0, x->stream), (c->d));
            return VP_OK;
    }
    vp_set_error("unknown step %d", step);
    return VP_E_ARG;
}

int launch_sweep(vp_chain* c) {
    static const int seq[] = {VP_STEP_UPDATEP, VP_STEP_UPDATEQ, VP_STEP_LOCPRIORI, VP_STEP_UPDATEZ, VP_STEP_ALPHA,
                              VP_STEP_UPDATEA, VP_STEP_UPDATEF};
    for (int st : seq) {
        int rc = launch_step(c, st, 0);
        if (rc) return rc;
    }
    // Record and m += 1 as one launch; at most 128 blocks: the element-wise
    // part only runs on recorded sweeps, and every block takes part in the
    // last-block count
    vp_ctx* x = c->ctx;
    SL(c, k_record_sweep, (std::min<unsigned>(128, cdiv((int64_t)c->P.K * x->KT, 256)), 1, 1), (256), 0, -1);
    return VP_OK;
}

}  // namespace

// the deferred initial counts of a tensor-core chain, for any use outside
// its batch
int ensure_counts(vp_chain* c) {
    if (!c->counts_pending) return VP_OK;
    int rc = launch_count(c, 1);
    if (!rc) c->counts_pending = false;
    return rc;
}

__global__ void k_set_plain(DevChain* dst, float* lt, double* LLp) {
    dst->lt = lt;
    dst->LLp = LLp;
}

// the plain form's scratch of a chain made for a tensor-core batch, carved on
// its first plain-form use; the likelihood table is filled from the current
// frequencies
int ensure_plain(vp_chain* c) {
    if (!c->plain_lazy || c->plain_mem) return VP_OK;
    vp_ctx* x = c->ctx;
    DevChain& h = c->h;
    const int64_t ltn = x->packed2 ? x->L * 4 * h.kp : (int64_t)c->P.K * x->KT;
    const size_t lt_bytes = ((size_t)ltn * 4 + 255) & ~(size_t)255;
    const size_t bytes = lt_bytes + (size_t)h.nchunk * x->N * c->P.K * 8;
    cudaError_t e = dev_alloc(&c->plain_mem, bytes, x->device, x->stream);
    if (e != cudaSuccess) {
        c->plain_mem = nullptr;
        vp_set_error("device allocation of %zu bytes for the plain form failed: %s", bytes, cudaGetErrorString(e));
        return VP_E_MEM;
    }
    CK(cudaMemsetAsync(c->plain_mem, 0, bytes, x->stream));
    h.lt = (float*)c->plain_mem;
    h.LLp = (double*)((char*)c->plain_mem + lt_bytes);
    LAUNCH(x, k_set_plain, (1, 1, 0, x->stream), (c->d, h.lt, h.LLp));
    LAUNCH(x, k_refresh_lt, (cdiv((int64_t)c->P.K * x->L, 256), 256, 0, x->stream), (c->d));
    return VP_OK;
}

extern "C" int vp_open(const vp_dataset* ds, int device, vp_ctx** out) { return vp_open_ex(ds, device, 0, out); }

int vp_open_ex(const vp_dataset* ds, int device, int priority, vp_ctx** out) {
    if (!ds || !out) { vp_set_error("null argument"); return VP_E_ARG; }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) { vp_set_error("no CUDA device"); return VP_E_NODEV; }
    if (device < 0 || device >= ndev) { vp_set_error("device %d out of range", device); return VP_E_ARG; }
    if (ds->maxK > 64) { vp_set_error("loci with more than 64 alleles are not supported"); return VP_E_ARG; }
    auto* x = new vp_ctx();
    x->device = device;
    cudaSetDevice(device);
    cudaDeviceGetAttribute(&x->nsm, cudaDevAttrMultiProcessorCount, device);
    if (cudaStreamCreateWithPriority(&x->stream, cudaStreamNonBlocking, priority) != cudaSuccess) {
        vp_set_error("cudaStreamCreate failed");
        delete x;
        return VP_E_CUDA;
    }
    x->N = ds->N; x->S = ds->S; x->L = ds->L; x->KT = ds->KT; x->maxK = ds->maxK; x->maxploidy = ds->maxploidy;
    x->packed2 = ds->packed2;
    DevData& D = x->D;
    D.N = ds->N; D.S = ds->S; D.vmax = ds->vmax; D.maxploidy = ds->maxploidy; D.maxK = ds->maxK; D.Nw = ds->Nw;
    D.packed2 = ds->packed2; D.L = ds->L; D.KT = ds->KT; D.coprime = ds->coprime;
    D.popcontig = 1;
    for (int32_t sp = 0; sp < ds->S; ++sp)
        for (int32_t j = 0; j < ds->pop_nind[sp]; ++j)
            if (ds->popid[ds->pop_ind0[sp] + j] != sp) { D.popcontig = 0; break; }
    vp_dataset_retain(ds);
    x->hold = ds;
    // the small (pageable) arrays first: a copy from pageable memory may wait
    // for the stream, which must not wait for the genotype copy
    int rc = 0;
    rc |= upload(x, ds->k.data(), ds->k.size(), &D.k);
    rc |= upload(x, ds->off.data(), ds->off.size(), &D.off);
    rc |= upload(x, ds->vt.data(), ds->vt.size(), &D.vt);
    rc |= upload(x, ds->popid.data(), ds->popid.size(), &D.popid);
    rc |= upload(x, ds->pop_ind0.data(), ds->pop_ind0.size(), &D.pop_ind0);
    rc |= upload(x, ds->pop_nind.data(), ds->pop_nind.size(), &D.pop_nind);
    rc |= upload(x, ds->totfreq.data(), ds->totfreq.size(), &D.totfreq);
    rc |= upload(x, ds->nhaplo.data(), ds->nhaplo.size(), &D.nhaplo);
    D.perm = nullptr;
    if (!ds->perm.empty()) rc |= upload(x, ds->perm.data(), ds->perm.size(), &D.perm);
    // the genotypes last, without a wait: chain set-up on the host overlaps
    // the copy, and every later use of them is ordered after it on the stream
    if (ds->packed2) rc |= upload(x, ds->g2.data(), ds->g2.size(), &D.g2);
    else rc |= upload(x, ds->gb.data(), ds->gb.size(), &D.gb);
    if (rc) { vp_close(x); return rc < 0 ? rc : VP_E_CUDA; }
    *out = x;
    return VP_OK;
}

extern "C" int vp_close(vp_ctx* x) {
    if (!x) return VP_OK;
    for (vp_chain* c : x->chains)
        if (c->cohort) { vp_set_error("a chain of this context belongs to a cohort: remove it (vp_cohort_set) first"); return VP_E_STATE; }
    cudaSetDevice(x->device);
    for (vp_chain* c : std::vector<vp_chain*>(x->chains)) vp_chain_destroy(c);
    if (x->stream) cudaStreamSynchronize(x->stream);
    if (x->batch) { cudaGraphExecDestroy(x->batch->graph); dev_free(x->batch->mem, x->stream); delete x->batch; x->batch = nullptr; }
    if (x->pg) cudaGraphExecDestroy(x->pg);
    for (cudaEvent_t e : x->prof_ev) cudaEventDestroy(e);
    for (cudaEvent_t e : x->fork_ev) cudaEventDestroy(e);
    for (cudaStream_t f : x->fork) cudaStreamDestroy(f);
    for (void* p : x->allocs) dev_free(p, x->stream);
    if (x->stream) {
        cudaStreamSynchronize(x->stream);
        cudaStreamDestroy(x->stream);
    }
    if (x->hold) vp_dataset_free(const_cast<vp_dataset*>(x->hold));
    delete x;
    return VP_OK;
}

extern "C" int vp_sync(vp_ctx* x) {
    if (!x) { vp_set_error("null context"); return VP_E_ARG; }
    CK(cudaStreamSynchronize(x->stream));
    return VP_OK;
}

extern "C" int64_t vp_launch_count(vp_ctx* x) { return x ? x->launches : -1; }

namespace {
// device layout of one chain's state inside its single allocation
// chains that a tensor-core batch runs: no-admixture, no location prior, no
// F model, counter streams, 2-bit data
bool tc_batchable(const vp_ctx* x, const vp_params* P, const DevChain& h) {
    return P->form == VP_FORM_TC && x->packed2 && !P->locpriori && !P->fmodel && P->rng == VP_RNG_COUNTER &&
           h.nadmburnin == 0 && !P->admix;
}

void chain_layout(Carve& cv, vp_chain* c, const vp_ctx* x) {
    DevChain& h = c->h;
    const vp_params* P = &c->P;
    const int K = P->K, N = x->N, S = x->S;
    const int64_t L = x->L, KT = x->KT;
    const int64_t ntrace = h.ntrace;
    const int64_t ltn = x->packed2 ? L * 4 * h.kp : (int64_t)K * KT;
    h.ctl = cv.take<Ctl>(1);
    h.rstate = cv.take<Rng64>(1);
    h.Freq = cv.take<float>(K * KT);
    h.FreqM = cv.take<float>(K * KT);
    h.FreqA = cv.take<float>(P->fmodel ? KT : 1);
    h.lt = c->plain_lazy ? nullptr : cv.take<float>(ltn);
    h.Q = cv.take<float>((int64_t)N * K);
    h.Qprop = cv.take<float>((int64_t)N * K);
    h.Di = cv.take<float>((int64_t)S * K);
    h.fbuf = cv.take<float>(64 * (x->maxK + 16));
    h.Z = cv.take<uint16_t>(N + 32);
    h.Mi = cv.take<int32_t>((int64_t)N * K);
    h.Ni = cv.take<int32_t>(K * KT);
    h.MiSum = cv.take<int64_t>((int64_t)N * K);
    h.LLp = c->plain_lazy ? nullptr : cv.take<double>((int64_t)h.nchunk * N * K);
    h.LL = cv.take<double>((int64_t)N * K);
    h.metro = cv.take<double>(N);
    // Metropolis partials: one per locus range of the per-copy kernels
    h.metrop = cv.take<double>((int64_t)cdiv(L, h.zadm_lc) * N);
    h.Alpha = cv.take<double>(K);
    h.Lambda = cv.take<double>(K);
    h.f = cv.take<double>(K);
    h.F = cv.take<double>(K);
    h.Eta = cv.take<double>(K);
    h.Gamma = cv.take<double>((int64_t)S * K);
    h.AlphaLocal = cv.take<double>((int64_t)S * K);
    h.SumAlpha = cv.take<double>(S);
    h.rout = cv.take<double>(h.rlen);
    h.lnlTrace = cv.take<double>(ntrace);
    h.red = cv.take<double>(((int64_t)S * K + K + 1) * (1 + LPQ_BLOCKS));
    h.lnlp = cv.take<double>(h.nlnlp);
    c->ancestry = cv.take<double>((int64_t)N * K);
    c->d = cv.take<DevChain>(1);
}

// validate the parameters and fill the chain's scalar state and launch
// geometry; *bytes receives the size of its device allocation
int chain_plan(const vp_ctx* x, const vp_params* P, vp_chain* c, size_t* bytes) {
    if (P->K < 1 || P->K > 64) { vp_set_error("K must be in 1..64"); return VP_E_ARG; }
    if (P->nthinning < 1 || P->nburnin < 0 || P->nreps < 0) { vp_set_error("bad MCMC lengths"); return VP_E_ARG; }
    c->P = *P;
    const int K = P->K, N = x->N, S = x->S;
    const int64_t L = x->L;
    DevChain& h = c->h;
    h.D = x->D;
    h.K = K; h.admix = P->admix; h.locpriori = P->locpriori; h.fmodel = P->fmodel;
    // ReadPar (src/structure.cpp:459-463): the no-admixture burn-in only exists
    // without admixture and without the location prior, and lengthens burn-in
    h.nadmburnin = (!P->locpriori && !P->admix) ? P->nadmburnin : 0;
    h.nburnin = P->nburnin + h.nadmburnin;
    h.nreps = P->nreps; h.nthinning = P->nthinning; h.writelnl = P->writelnl;
    h.metrofreq = P->metrofreq; h.inferalpha = P->inferalpha; h.diffalpha = P->diffalpha;
    h.uniformalpha = P->uniformalpha; h.fsame = P->fsame; h.difflambda = P->difflambda; h.rng = P->rng;
    h.lambda = P->lambda; h.alpha = P->alpha; h.stdalpha = P->stdalpha; h.maxalpha = P->maxalpha;
    h.alphapriora = P->alphapriora; h.alphapriorb = P->alphapriorb; h.maxr = P->maxr; h.epsr = P->epsr;
    h.epseta = P->epseta; h.epsgamma = P->epsgamma; h.pmeanf = P->pmeanf; h.pstdf = P->pstdf; h.stdf = P->stdf;
    h.seed = P->seed;
    int nf = P->fmodel ? (P->fsame ? 1 : K) : 0;
    int na = P->admix ? (P->diffalpha ? K : 1) : 0;
    int nl = P->difflambda ? K : 1;
    h.rlen = P->locpriori ? 4 + nl + 1 + K + K * S + nf : 4 + nl + na + nf;
    // lnL trace records: ceil(nburnin / t) + ceil(nreps / t), plus slack;
    // Record never writes more than this many
    h.ntrace = (int32_t)(h.nburnin / h.nthinning + h.nreps / h.nthinning + 2);
    c->ll_fma = x->packed2 && lf_form(K);
    c->kc = ll_kc(c->ll_fma, K);
    c->kgroups = (K + c->kc - 1) / c->kc;
    {
        const int64_t nch = ll_chunks(c->ll_fma, c->kc, c->kgroups, N, L, x->nsm);
        h.lchunk = (int32_t)((L + nch - 1) / nch);
        h.nchunk = (int32_t)((L + h.lchunk - 1) / h.lchunk);
    }
    h.kp = (K + 3) & ~3;
    h.nsampblk = (int32_t)cdiv(N, SAMPLE_BLOCK / 32);   // counter-stream sampling: a warp per individual
    {
        // loci per CTA of the per-copy label kernel: about 64 CTAs' worth per
        // SM (several waves of short CTAs), which evens out CTAs of unequal
        // cost (mixed ploidy) and lets the device take up other streams'
        // blocks between them (measured: 4 -> 16 -> 32 -> 64 per SM took c4
        // from 3.62 to 3.03, 2.85 and 2.77 ms per sweep, c5 p50 from 0.62 to
        // 0.44 s)
        int64_t nx = cdiv(N, ZA_WARPS * 32);
        int64_t ny = std::max<int64_t>(1, (int64_t)x->nsm * 64 / nx);
        int64_t lc = (L + ny - 1) / ny;
        lc = (lc + ZA_LC - 1) / ZA_LC * ZA_LC;
        h.zadm_lc = (int32_t)std::max<int64_t>(lc, ZA_LC);
    }
    if ((size_t)ZA_LC * x->maxK * (K | 1) * 4 + (size_t)ZA_LC * K * x->maxK * 4 > 200 * 1024) {
        vp_set_error("K * max alleles too large for the admixture kernel");
        return VP_E_ARG;
    }
    h.nlnlp = (int32_t)std::max<int64_t>(std::max<int64_t>(cdiv(L, 128), (int64_t)cdiv(N, ZA_WARPS * 32) * cdiv(L, h.zadm_lc)),
                                         std::max<int64_t>(h.nsampblk, cdiv(N, tc::TS_TILE)));
    c->plain_lazy = tc_batchable(x, P, h);
    Carve probe{nullptr};
    chain_layout(probe, c, x);
    *bytes = probe.off;
    return VP_OK;
}
}  // namespace

int64_t vp_request_bytes(const vp_dataset* ds, const vp_params* P, int nsm) {
    vp_ctx g;
    g.N = ds->N; g.S = ds->S; g.L = ds->L; g.KT = ds->KT; g.maxK = ds->maxK; g.maxploidy = ds->maxploidy;
    g.packed2 = ds->packed2; g.nsm = nsm;
    vp_chain c;
    size_t chain = 0;
    if (chain_plan(&g, P, &c, &chain)) return -1;
    // the context's uploads (each rounded to the allocator's 512-byte grain)
    auto r = [](size_t b) { return (int64_t)((b + 511) & ~(size_t)511); };
    int64_t data = ds->packed2 ? r(ds->g2.size() * 4) : r(ds->gb.size());
    data += r(ds->k.size() * 4) + r(ds->off.size() * 8) + r(ds->vt.size() * 8) + r(ds->popid.size() * 4) +
            r(ds->pop_ind0.size() * 4) + r(ds->pop_nind.size() * 4) + r(ds->totfreq.size() * 4) +
            r(ds->nhaplo.size() * 4) + (ds->perm.empty() ? 0 : r(ds->perm.size() * 4));
    return data + (int64_t)chain;
}

extern "C" int vp_chain_create(vp_ctx* x, const vp_params* P, vp_chain** out) {
    if (!x || !P || !out) { vp_set_error("null argument"); return VP_E_ARG; }
    cudaSetDevice(x->device);
    auto* c = new vp_chain();
    c->ctx = x;
    size_t bytes = 0;
    int prc = chain_plan(x, P, c, &bytes);
    if (prc) { delete c; return prc; }
    set_smem_limits(x->device);
    const int K = P->K, N = x->N;
    const int64_t L = x->L;
    DevChain& h = c->h;
    cudaError_t e = dev_alloc(&c->mem, bytes, x->device, x->stream);
    if (e != cudaSuccess) {
        vp_set_error("device allocation of %zu bytes for chain state failed: %s", bytes, cudaGetErrorString(e));
        delete c;
        return VP_E_MEM;
    }
    Carve cv{(char*)c->mem};
    chain_layout(cv, c, x);
    c->own_ni = h.Ni;
    c->total = h.nburnin + h.nreps;
    // InitFix / InitAdmix / InitLocPriori / InitFmodel
    cudaStream_t s = x->stream;
    int rc = VP_OK;
    do {
        if ((e = cudaMemsetAsync(c->mem, 0, bytes, s)) != cudaSuccess) {
            vp_set_error("cudaMemsetAsync of chain state failed: %s", cudaGetErrorString(e));
            rc = VP_E_CUDA;
            break;
        }
        k_set_chain<<<1, 128, 0, s>>>(c->d, h);
        if ((rc = check_launch(x, "k_set_chain"))) break;
        k_init_state<<<dim3(std::min<unsigned>(1024, cdiv(std::max<int64_t>(L, (int64_t)N * K), 256)), 1, 1), 256, 0, s>>>(c->d);
        if ((rc = check_launch(x, "k_init_state"))) break;
        const bool singlez = h.nadmburnin == 0 && !P->admix;
        if (singlez) {
            k_init_z_single<<<P->rng ? cdiv(N, 256) : 1, P->rng ? 256 : 32, 0, s>>>(c->d);
            if ((rc = check_launch(x, "k_init_z_single"))) break;
            if (c->plain_lazy) {
                c->counts_pending = true;
                break;
            }
            if ((rc = launch_count(c, 1))) break;
        } else {
            k_init_admix<<<cdiv(L, 128), 128, 0, s>>>(c->d);
            if ((rc = check_launch(x, "k_init_admix"))) break;
        }
    } while (0);
    if (rc) { dev_free(c->mem, x->stream); delete c; return rc; }
    x->chains.push_back(c);
    *out = c;
    return VP_OK;
}

extern "C" int vp_chain_destroy(vp_chain* c) {
    if (!c) return VP_OK;
    if (c->cohort) { vp_set_error("the chain belongs to a cohort: remove it (vp_cohort_set) first"); return VP_E_STATE; }
    cudaSetDevice(c->ctx->device);
    bool in_batch = false, in_pg = false;
    if (c->ctx->batch)
        for (vp_chain* o : c->ctx->batch->chains) in_batch |= o == c;
    for (vp_chain* o : c->ctx->pg_chains) in_pg |= o == c;
    // graphs are destroyed only once their launches are done; the chain's
    // memory is freed in stream order and needs no wait
    if (in_batch || in_pg || c->graph) cudaStreamSynchronize(c->ctx->stream);
    if (in_batch) free_batch(c->ctx);
    for (vp_chain* o : c->ctx->pg_chains)
        if (o == c) {
            cudaGraphExecDestroy(c->ctx->pg);
            c->ctx->pg = nullptr;
            c->ctx->pg_chains.clear();
            break;
        }
    if (c->graph) cudaGraphExecDestroy(c->graph);
    dev_free(c->plain_mem, c->ctx->stream);
    dev_free(c->mem, c->ctx->stream);   // after every launch already queued for the chain
    auto& open = c->ctx->chains;
    open.erase(std::remove(open.begin(), open.end(), c), open.end());
    delete c;
    return VP_OK;
}

// Capture one sweep of the given chains into a graph (kernels read m from
// device memory, so the same graph serves every sweep).
static int capture_sweep(vp_chain** cs, int n, cudaGraphExec_t* exec, int* nodes) {
    vp_ctx* x = cs[0]->ctx;
    cudaGraph_t g;
    x->prof_next = 0;
    x->prof_used = 0;
    CK(cudaStreamBeginCapture(x->stream, cudaStreamCaptureModeThreadLocal));
    int64_t before = x->launches;
    int rc = VP_OK;
    for (int i = 0; i < n && !rc; ++i) rc = launch_sweep(cs[i]);
    cudaError_t e = cudaStreamEndCapture(x->stream, &g);
    if (rc) { if (e == cudaSuccess) cudaGraphDestroy(g); return rc; }
    if (e != cudaSuccess) { vp_set_error("graph capture failed: %s", cudaGetErrorString(e)); return VP_E_CUDA; }
    *nodes = (int)(x->launches - before);
    x->launches = before;
    e = cudaGraphInstantiate(exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) { vp_set_error("graph instantiate failed: %s", cudaGetErrorString(e)); return VP_E_CUDA; }
    return VP_OK;
}

// plain-form sweeps of a set of chains of one context: chains with sweeps
// left share one cached graph of a sweep while their set does not change
static int run_plain(vp_ctx* x, vp_chain** cs, int n, int nsweeps) {
    for (int i = 0; i < n; ++i) {
        if (int rc0 = ensure_counts(cs[i])) return rc0;
        if (int rc0 = ensure_plain(cs[i])) return rc0;
    }
    int left = nsweeps;
    while (left > 0) {
        std::vector<vp_chain*> act;
        int step = left;
        for (int i = 0; i < n; ++i) {
            int rem = cs[i]->total - cs[i]->issued;
            if (rem > 0) { act.push_back(cs[i]); step = std::min(step, rem); }
        }
        if (act.empty()) break;
        if (x->pg && x->pg_chains != act) {
            cudaGraphExecDestroy(x->pg);
            x->pg = nullptr;
        }
        if (!x->pg) {
            int rc = capture_sweep(act.data(), (int)act.size(), &x->pg, &x->pg_nodes);
            if (rc) return rc;
            x->pg_chains = act;
        }
        for (int s = 0; s < step; ++s) {
            CK(cudaGraphLaunch(x->pg, x->stream));
            x->launches += x->pg_nodes;
        }
        for (vp_chain* c : act) c->issued += step;
        left -= step;
    }
    return VP_OK;
}

extern "C" int vp_run(vp_chain** cs, int32_t n, int32_t nsweeps) {
    if (!cs || n <= 0 || nsweeps < 0) { vp_set_error("bad arguments"); return VP_E_ARG; }
    vp_ctx* x = cs[0]->ctx;
    for (int i = 0; i < n; ++i)
        if (!cs[i] || cs[i]->ctx != x) { vp_set_error("all chains of one vp_run must share a context"); return VP_E_ARG; }
    cudaSetDevice(x->device);
    for (int i = 0; i < n; ++i)
        if (cs[i]->cohort && nsweeps > 0 && cs[i]->issued < cs[i]->total) {
            vp_set_error("a chain of a cohort advances with its cohort (vp_cohort_run)");
            return VP_E_STATE;
        }
    bool all_tc = true;
    for (int i = 0; i < n; ++i) all_tc &= cs[i]->P.form == VP_FORM_TC;
    if (!all_tc) return run_plain(x, cs, n, nsweeps);
    // Tensor-core chains: the sweeps of the no-admixture burn-in (m <
    // nadmburnin, src/structure.cpp:460-462, where Q and Z are drawn per
    // allele copy as with admixture) run in the plain form; from the first
    // single-label sweep on a chain runs in the batch. Each round advances
    // every chain with sweeps left by the same number of sweeps, up to the
    // next phase change or end of a chain.
    int left = nsweeps;
    while (left > 0) {
        std::vector<vp_chain*> burn, batch;
        int step = left;
        for (int i = 0; i < n; ++i) {
            vp_chain* c = cs[i];
            if (c->issued >= c->total) continue;
            const int phase_end = c->issued < c->h.nadmburnin ? c->h.nadmburnin : c->total;
            (c->issued < c->h.nadmburnin ? burn : batch).push_back(c);
            step = std::min(step, phase_end - c->issued);
        }
        if (burn.empty() && batch.empty()) break;
        if (!burn.empty()) {
            // run_plain advances these chains' issued counts itself
            if (int rc = run_plain(x, burn.data(), (int)burn.size(), step)) return rc;
        }
        if (!batch.empty()) {
            if (int rc = run_tc(x, batch.data(), (int)batch.size(), step)) return rc;
            for (vp_chain* c : batch) c->issued += step;
        }
        left -= step;
    }
    return VP_OK;
}

// the rest of every chain's sweeps and the final Arrange, queued on the
// context's stream without waiting
int vp_finish_issue(vp_chain** cs, int32_t n) {
    if (!cs || n <= 0) { vp_set_error("bad arguments"); return VP_E_ARG; }
    int mx = 0;
    for (int i = 0; i < n; ++i) mx = std::max(mx, cs[i]->total - cs[i]->issued);
    int rc = vp_run(cs, n, mx);
    if (rc) return rc;
    vp_ctx* x = cs[0]->ctx;
    for (int i = 0; i < n; ++i) {
        vp_chain* c = cs[i];
        if (c->arranged) continue;
        k_arrange<<<std::min<unsigned>(1024, cdiv((int64_t)c->P.K * x->KT, 256)), 256, 0, x->stream>>>(c->d, c->ancestry);
        rc = check_launch(x, "k_arrange");
        if (rc) return rc;
        c->arranged = true;
    }
    return VP_OK;
}

extern "C" int vp_finish(vp_chain** cs, int32_t n) {
    int rc = vp_finish_issue(cs, n);
    return rc ? rc : vp_sync(cs[0]->ctx);
}

const vp_dataset* vp_chain_dataset(const vp_chain* c) { return c->ctx->hold; }
void vp_chain_params(const vp_chain* c, vp_params* p) { *p = c->P; }

void vp_chain_progress(const vp_chain* c, int64_t* issued, int64_t* total) {
    *issued = c->issued;
    *total = c->total;
}

extern "C" int vp_chain_divergence(vp_chain* c, double* H, double* D, double* Hl) {
    if (!c || !H || !D) { vp_set_error("null argument"); return VP_E_ARG; }
    if (!c->arranged) { vp_set_error("the chain is not finished (vp_finish arranges the mean frequencies)"); return VP_E_STATE; }
    vp_ctx* x = c->ctx;
    cudaSetDevice(x->device);
    const int K = c->P.K;
    const int npairs = K * (K + 1) / 2;
    const int nch = (int)std::min<int64_t>(DIV_CHUNKS, std::max<int64_t>(1, x->L / 256));
    const size_t pb = (size_t)npairs * nch * 8, hb = (size_t)K * 8, db = (size_t)K * K * 8;
    const size_t lb = Hl ? (size_t)K * x->L * 8 : 0;
    char* buf = nullptr;
    CK(cudaMallocAsync((void**)&buf, pb + hb + db + lb + 64, x->stream));
    double* part = (double*)buf;
    double* dH = (double*)(buf + pb);
    double* dD = (double*)(buf + pb + hb);
    double* dHl = (double*)(buf + pb + hb + db);
    int rc = VP_OK;
    do {
        k_divergence_pairs<<<dim3(npairs, nch, 1), 256, 0, x->stream>>>(c->d, part);
        if ((rc = check_launch(x, "k_divergence_pairs"))) break;
        k_divergence_finish<<<1, 32, 0, x->stream>>>(c->d, part, nch, dH, dD);
        if ((rc = check_launch(x, "k_divergence_finish"))) break;
        if (Hl) {
            k_heterozygosity<<<std::min<unsigned>(4096, cdiv((int64_t)K * x->L, 256)), 256, 0, x->stream>>>(c->d, dHl);
            if ((rc = check_launch(x, "k_heterozygosity"))) break;
        }
        cudaError_t e;
        if ((e = cudaMemcpyAsync(H, dH, hb, cudaMemcpyDeviceToHost, x->stream)) != cudaSuccess ||
            (e = cudaMemcpyAsync(D, dD, db, cudaMemcpyDeviceToHost, x->stream)) != cudaSuccess ||
            (Hl && (e = cudaMemcpyAsync(Hl, dHl, lb, cudaMemcpyDeviceToHost, x->stream)) != cudaSuccess)) {
            vp_set_error("divergence copy-out failed: %s", cudaGetErrorString(e));
            rc = VP_E_CUDA;
        }
    } while (0);
    cudaFreeAsync(buf, x->stream);
    cudaError_t e = cudaStreamSynchronize(x->stream);
    if (!rc && e != cudaSuccess) { vp_set_error("divergence failed: %s", cudaGetErrorString(e)); rc = VP_E_CUDA; }
    return rc;
}

extern "C" int vp_chain_sizes(vp_chain* c, vp_result* r) {
    if (!c || !r) { vp_set_error("null argument"); return VP_E_ARG; }
    memset(r, 0, sizeof *r);
    r->K = c->P.K; r->N = c->ctx->N; r->S = c->ctx->S; r->KT = c->ctx->KT;
    r->nburnin = c->h.nburnin; r->nreps = c->h.nreps; r->nthinning = c->h.nthinning; r->rlen = c->h.rlen;
    r->seed = c->P.seed;
    // after the sweeps queued on the chain's (non-blocking) stream
    cudaSetDevice(c->ctx->device);
    CK(cudaStreamSynchronize(c->ctx->stream));
    Ctl ctl;
    CK(cudaMemcpy(&ctl, c->h.ctl, sizeof ctl, cudaMemcpyDeviceToHost));
    r->nr = ctl.nr; r->nlnl = ctl.nlnl;
    return VP_OK;
}

extern "C" int vp_chain_result(vp_chain* c, vp_result* out) {
    if (!c || !out) { vp_set_error("null argument"); return VP_E_ARG; }
    vp_result sz;
    int rc = vp_chain_sizes(c, &sz);
    if (rc) return rc;
    const int64_t NK = (int64_t)sz.N * sz.K;
    CK(cudaStreamSynchronize(c->ctx->stream));
    if (out->rout) CK(cudaMemcpy(out->rout, c->h.rout, sz.rlen * sizeof(double), cudaMemcpyDeviceToHost));
    if (out->lnl) CK(cudaMemcpy(out->lnl, c->h.lnlTrace, sz.nlnl * sizeof(double), cudaMemcpyDeviceToHost));
    if (out->Q) CK(cudaMemcpy(out->Q, c->h.Q, NK * sizeof(float), cudaMemcpyDeviceToHost));
    if (out->ancestry) {
        if (!c->arranged) { vp_set_error("ancestry is available after vp_finish"); return VP_E_STATE; }
        CK(cudaMemcpy(out->ancestry, c->ancestry, NK * sizeof(double), cudaMemcpyDeviceToHost));
    }
    if (out->freqm) CK(cudaMemcpy(out->freqm, c->h.FreqM, sz.K * sz.KT * sizeof(float), cudaMemcpyDeviceToHost));
    double *ro = out->rout, *ln = out->lnl;
    float *q = out->Q, *fm = out->freqm;
    double* an = out->ancestry;
    *out = sz;
    out->rout = ro; out->lnl = ln; out->Q = q; out->freqm = fm; out->ancestry = an;
    return VP_OK;
}

static int field_ptr(vp_chain* c, int f, void** p, size_t* bytes) {
    const DevChain& h = c->h;
    const size_t K = c->P.K, N = c->ctx->N, KT = c->ctx->KT, S = c->ctx->S;
    switch (f) {
        case VP_F_FREQ: *p = h.Freq; *bytes = K * KT * 4; return VP_OK;
        case VP_F_Q: *p = h.Q; *bytes = N * K * 4; return VP_OK;
        case VP_F_Z: *p = h.Z; *bytes = N * 2; return VP_OK;
        case VP_F_NI: *p = h.Ni; *bytes = K * KT * 4; return VP_OK;
        case VP_F_MI: *p = h.Mi; *bytes = N * K * 4; return VP_OK;
        case VP_F_LL: *p = h.LL; *bytes = N * K * 8; return VP_OK;
        case VP_F_ALPHA: *p = h.Alpha; *bytes = K * 8; return VP_OK;
        case VP_F_M: *p = &h.ctl->m; *bytes = 4; return VP_OK;
        case VP_F_LNL: *p = &h.ctl->lnl; *bytes = 8; return VP_OK;
        case VP_F_FREQA: *p = h.FreqA; *bytes = c->P.fmodel ? KT * 4 : 0; return VP_OK;
        // f[K] then F[K]: two separate allocations, copied one by one in
        // vp_chain_get / vp_chain_set
        case VP_F_FF: *p = h.f; *bytes = 2 * K * 8; return VP_OK;
        case VP_F_DI: *p = h.Di; *bytes = S * K * 4; return VP_OK;
        case VP_F_METRO: *p = h.metro; *bytes = N * 8; return VP_OK;
    }
    vp_set_error("unknown field %d", f);
    return VP_E_ARG;
}

// the location-prior state, five arrays in one host buffer: r, Eta[K],
// Gamma[S*K], AlphaLocal[S*K], SumAlpha[S] (all double)
static int locp_copy(vp_chain* c, void* host, size_t bytes, bool to_device) {
    const size_t K = c->P.K, S = c->ctx->S;
    const size_t want = 8 * (1 + K + 2 * S * K + S);
    if (bytes != want) { vp_set_error("field %d holds %zu bytes, not %zu", VP_F_LOCP, want, bytes); return VP_E_ARG; }
    struct Part { void* dev; size_t n; } parts[] = {{&c->h.ctl->r, 1}, {c->h.Eta, K}, {c->h.Gamma, S * K},
                                                     {c->h.AlphaLocal, S * K}, {c->h.SumAlpha, S}};
    char* h = (char*)host;
    for (const Part& p : parts) {
        if (to_device) CK(cudaMemcpy(p.dev, h, p.n * 8, cudaMemcpyHostToDevice));
        else CK(cudaMemcpy(h, p.dev, p.n * 8, cudaMemcpyDeviceToHost));
        h += p.n * 8;
    }
    return VP_OK;
}

extern "C" int vp_chain_get(vp_chain* c, int32_t field, void* host, size_t bytes) {
    if (!c || !host) { vp_set_error("null argument"); return VP_E_ARG; }
    cudaSetDevice(c->ctx->device);
    if (int rc0 = ensure_counts(c)) return rc0;
    CK(cudaStreamSynchronize(c->ctx->stream));
    if (field == VP_F_FF) {
        size_t K = c->P.K;
        if (bytes != 2 * K * 8) { vp_set_error("field %d holds %zu bytes", field, 2 * K * 8); return VP_E_ARG; }
        CK(cudaMemcpy(host, c->h.f, K * 8, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy((char*)host + K * 8, c->h.F, K * 8, cudaMemcpyDeviceToHost));
        return VP_OK;
    }
    if (field == VP_F_LOCP) return locp_copy(c, host, bytes, false);
    void* p; size_t n;
    int rc = field_ptr(c, field, &p, &n);
    if (rc) return rc;
    if (bytes != n) { vp_set_error("field %d holds %zu bytes, not %zu", field, n, bytes); return VP_E_ARG; }
    CK(cudaMemcpyAsync(host, p, n, cudaMemcpyDeviceToHost, c->ctx->stream));
    CK(cudaStreamSynchronize(c->ctx->stream));
    return VP_OK;
}

extern "C" int vp_chain_set(vp_chain* c, int32_t field, const void* host, size_t bytes) {
    if (!c || !host) { vp_set_error("null argument"); return VP_E_ARG; }
    cudaSetDevice(c->ctx->device);
    if (field == VP_F_NI) c->counts_pending = false;   // the caller's counts replace them
    else if (int rc0 = ensure_counts(c)) return rc0;
    CK(cudaStreamSynchronize(c->ctx->stream));
    if (field == VP_F_FF) {
        size_t K = c->P.K;
        if (bytes != 2 * K * 8) { vp_set_error("field %d holds %zu bytes", field, 2 * K * 8); return VP_E_ARG; }
        CK(cudaMemcpy(c->h.f, host, K * 8, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(c->h.F, (const char*)host + K * 8, K * 8, cudaMemcpyHostToDevice));
        return VP_OK;
    }
    if (field == VP_F_LOCP) return locp_copy(c, const_cast<void*>(host), bytes, true);
    void* p; size_t n;
    int rc = field_ptr(c, field, &p, &n);
    if (rc) return rc;
    if (bytes != n) { vp_set_error("field %d holds %zu bytes, not %zu", field, n, bytes); return VP_E_ARG; }
    if (field == VP_F_M) {
        const int32_t m = *(const int32_t*)host;
        if (m < 0 || m > c->total) {
            vp_set_error("sweep index %d outside the run's 0..%d", m, c->total);
            return VP_E_ARG;
        }
    }
    CK(cudaMemcpy(p, host, n, cudaMemcpyHostToDevice));
    if (field == VP_F_FREQ && c->h.lt) {
        // keep the likelihood lookup table in step with the frequencies
        vp_ctx* x = c->ctx;
        k_refresh_lt<<<cdiv((int64_t)c->P.K * x->L, 256), 256, 0, x->stream>>>(c->d);
        rc = check_launch(x, "k_refresh_lt");
        if (rc) return rc;
        CK(cudaStreamSynchronize(x->stream));
    }
    return VP_OK;
}

extern "C" int vp_chain_step(vp_chain* c, int32_t step) {
    if (!c) { vp_set_error("null chain"); return VP_E_ARG; }
    cudaSetDevice(c->ctx->device);
    int rc = ensure_counts(c);
    if (!rc) rc = ensure_plain(c);
    if (rc) return rc;
    // no step past the end of the run: Record and the sweep index would
    // run beyond the state sized for nburnin + nreps sweeps
    int32_t m = 0;
    CK(cudaMemcpyAsync(&m, &c->h.ctl->m, sizeof m, cudaMemcpyDeviceToHost, c->ctx->stream));
    CK(cudaStreamSynchronize(c->ctx->stream));
    if (m >= c->total) {
        vp_set_error("sweep index %d: the run has %d sweeps (nburnin + nreps) and is over", m, c->total);
        return VP_E_STATE;
    }
    rc = launch_step(c, step, 0);
    if (rc) return rc;
    return vp_sync(c->ctx);
}

// ===================== cohorts: runs of different datasets in shared launches =====================
// A cohort sweeps plain-form chains of any contexts on one device with one
// launch per kernel of the sweep (one per compiled variant in use). Each
// member's sweep is recorded (the launches launch_sweep would issue for it
// alone); the recordings are merged in order -- the next launch of every
// member that has the same kernel, block shape and scalar arguments go
// together -- and every merged launch gets a block map listing, for each
// member, every block of that member's own grid. The merged sequence is
// captured once into a CUDA graph and replayed each sweep.
struct vp_cohort {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev = nullptr;                 // after the last queued sweeps
    std::vector<vp_chain*> chains;
    void* mem = nullptr;                      // DevChain copies and block maps of the current graph
    cudaGraphExec_t graph = nullptr;
    int nodes = 0;
    int64_t launches = 0;
    // replaced graphs and their buffers, freed once an event after their last
    // launch has completed
    struct Old { cudaGraphExec_t g; cudaEvent_t e; };
    std::vector<Old> old;
};

namespace {

void cohort_reap(vp_cohort* h, bool wait) {
    for (size_t i = 0; i < h->old.size();) {
        if (wait) cudaEventSynchronize(h->old[i].e);
        if (cudaEventQuery(h->old[i].e) == cudaSuccess) {
            cudaGraphExecDestroy(h->old[i].g);
            cudaEventDestroy(h->old[i].e);
            h->old.erase(h->old.begin() + i);
        } else {
            ++i;
        }
    }
}

// the cohort stream waits for the work already queued on each member's own
// stream (its upload, initialisation, earlier sweeps)
int cohort_wait_members(vp_cohort* h, const std::vector<vp_chain*>& cs) {
    for (vp_chain* c : cs) {
        cudaEvent_t e;
        CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        cudaEventRecord(e, c->ctx->stream);
        cudaStreamWaitEvent(h->stream, e, 0);
        cudaEventDestroy(e);
    }
    return VP_OK;
}

struct MergedLaunch {
    const void* fn;
    const char* name;
    dim3 block;
    size_t smem = 0;
    int nint, i0, i1;
    int64_t map0 = 0, nmap = 0;   // entries in the map buffer
};

int cohort_build(vp_cohort* h) {
    const int n = (int)h->chains.size();
    if (h->graph) {
        // keep the old graph until its queued replays are done
        cudaEvent_t e;
        CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        cudaEventRecord(e, h->stream);
        h->old.push_back({h->graph, e});
        h->graph = nullptr;
    }
    if (h->mem) { dev_free(h->mem, h->stream); h->mem = nullptr; }
    h->nodes = 0;
    if (n == 0) return VP_OK;
    // 1. each member's sweep, recorded
    std::vector<std::vector<SweepRec>> rec(n);
    for (int i = 0; i < n; ++i) {
        vp_chain* c = h->chains[i];
        c->ctx->rec = &rec[i];
        int rc = launch_sweep(c);
        c->ctx->rec = nullptr;
        if (rc) return rc;
    }
    // 2. merge: repeatedly take the next launch of the first member with
    // launches left, and the next launch of every other member that matches it
    std::vector<size_t> pos(n, 0);
    std::vector<MergedLaunch> ml;
    std::vector<int4> maps;
    auto same = [](const SweepRec& a, const SweepRec& b) {
        return a.fn == b.fn && a.block.x == b.block.x && a.block.y == b.block.y && a.block.z == b.block.z &&
               a.nint == b.nint && a.i0 == b.i0 && a.i1 == b.i1;
    };
    for (;;) {
        int lead = -1;
        for (int i = 0; i < n && lead < 0; ++i)
            if (pos[i] < rec[i].size()) lead = i;
        if (lead < 0) break;
        const SweepRec head = rec[lead][pos[lead]];
        MergedLaunch m{head.fn, head.name, head.block, 0, head.nint, head.i0, head.i1, (int64_t)maps.size(), 0};
        for (int i = 0; i < n; ++i) {
            if (pos[i] >= rec[i].size() || !same(rec[i][pos[i]], head)) continue;
            const SweepRec& r = rec[i][pos[i]++];
            m.smem = std::max(m.smem, r.smem);
            for (unsigned z = 0; z < r.grid.z; ++z)
                for (unsigned y = 0; y < r.grid.y; ++y)
                    for (unsigned x = 0; x < r.grid.x; ++x)
                        maps.push_back(make_int4((int)(i * r.grid.z + z), (int)x, (int)y, (int)r.grid.x));
        }
        m.nmap = (int64_t)maps.size() - m.map0;
        ml.push_back(m);
    }
    // 3. the members' headers and the maps in one device buffer
    const size_t hb = ((size_t)n * sizeof(DevChain) + 255) & ~(size_t)255;
    const size_t bytes = hb + maps.size() * sizeof(int4);
    cudaError_t e = dev_alloc(&h->mem, bytes, h->device, h->stream);
    if (e != cudaSuccess) { h->mem = nullptr; vp_set_error("cohort buffer of %zu bytes: %s", bytes, cudaGetErrorString(e)); return VP_E_MEM; }
    std::vector<DevChain> hc(n);
    for (int i = 0; i < n; ++i) hc[i] = h->chains[i]->h;
    DevChain* dchains = (DevChain*)h->mem;
    int4* dmaps = (int4*)((char*)h->mem + hb);
    // (from pageable memory: the copies are staged before the calls return)
    CK(cudaMemcpyAsync(dchains, hc.data(), (size_t)n * sizeof(DevChain), cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(dmaps, maps.data(), maps.size() * sizeof(int4), cudaMemcpyHostToDevice, h->stream));
    // 4. capture one sweep
    cudaGraph_t g;
    CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t le = cudaSuccess;
    const char* bad = nullptr;
    for (const MergedLaunch& m : ml) {
        const DevChain* d = dchains;
        const int4* map = dmaps + m.map0;
        double* none = nullptr;
        int i0 = m.i0, i1 = m.i1;
        void* args[4];
        int k = 0;
        args[k++] = (void*)&d;
        if (m.nint < 0) args[k++] = (void*)&none;
        if (m.nint >= 1) args[k++] = (void*)&i0;
        if (m.nint >= 2) args[k++] = (void*)&i1;
        args[k++] = (void*)&map;
        le = cudaLaunchKernel(m.fn, dim3((unsigned)m.nmap, 1, 1), m.block, args, m.smem, h->stream);
        if (le != cudaSuccess) { bad = m.name; break; }
    }
    cudaError_t ce = cudaStreamEndCapture(h->stream, &g);
    if (le != cudaSuccess) {
        if (ce == cudaSuccess) cudaGraphDestroy(g);
        vp_set_error("cohort launch of %s: %s", bad, cudaGetErrorString(le));
        return VP_E_CUDA;
    }
    if (ce != cudaSuccess) { vp_set_error("cohort capture: %s", cudaGetErrorString(ce)); return VP_E_CUDA; }
    e = cudaGraphInstantiate(&h->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) { h->graph = nullptr; vp_set_error("cohort graph: %s", cudaGetErrorString(e)); return VP_E_CUDA; }
    h->nodes = (int)ml.size();
    return VP_OK;
}

}  // namespace

int vp_cohort_open_ex(int device, int priority, vp_cohort** out) {
    if (!out) { vp_set_error("null argument"); return VP_E_ARG; }
    if (cudaSetDevice(device) != cudaSuccess) { vp_set_error("cudaSetDevice(%d) failed", device); return VP_E_NODEV; }
    auto* h = new vp_cohort();
    h->device = device;
    if (cudaStreamCreateWithPriority(&h->stream, cudaStreamNonBlocking, priority) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->ev, cudaEventDisableTiming) != cudaSuccess) {
        if (h->stream) cudaStreamDestroy(h->stream);
        delete h;
        vp_set_error("cohort stream: %s", cudaGetErrorString(cudaGetLastError()));
        return VP_E_CUDA;
    }
    *out = h;
    return VP_OK;
}

extern "C" int vp_cohort_open(int device, vp_cohort** out) { return vp_cohort_open_ex(device, 0, out); }

// a hash of the kernels, launch shapes and scalar arguments of one sweep of
// the chain: chains with equal signatures merge every launch of a cohort
uint64_t vp_chain_sweep_signature(vp_chain* c) {
    std::vector<SweepRec> rec;
    c->ctx->rec = &rec;
    launch_sweep(c);
    c->ctx->rec = nullptr;
    uint64_t h = 1469598103934665603ull;
    auto mix = [&](uint64_t v) { h = (h ^ v) * 1099511628211ull; };
    for (const SweepRec& r : rec) {
        mix((uint64_t)(uintptr_t)r.fn);
        mix(((uint64_t)r.block.x << 32) | ((uint64_t)r.block.y << 16) | r.block.z);
        mix(((uint64_t)(uint32_t)r.nint << 32) | (uint32_t)r.i0);
        mix((uint64_t)(uint32_t)r.i1);
    }
    return h;
}

extern "C" int vp_cohort_set(vp_cohort* h, vp_chain** cs, int32_t n) {
    if (!h || n < 0 || (n > 0 && !cs)) { vp_set_error("bad arguments"); return VP_E_ARG; }
    cudaSetDevice(h->device);
    std::vector<vp_chain*> next(cs, cs + n);
    for (int i = 0; i < n; ++i) {
        vp_chain* c = cs[i];
        if (!c) { vp_set_error("null chain"); return VP_E_ARG; }
        if (c->ctx->device != h->device) { vp_set_error("chain on device %d, cohort on %d", c->ctx->device, h->device); return VP_E_ARG; }
        if (c->cohort && c->cohort != h) { vp_set_error("the chain belongs to another cohort"); return VP_E_STATE; }
        if (c->P.form == VP_FORM_TC) { vp_set_error("a cohort runs plain-form chains (the tensor-core form has its own batch)"); return VP_E_ARG; }
        for (int j = 0; j < i; ++j)
            if (cs[j] == c) { vp_set_error("chain listed twice"); return VP_E_ARG; }
        if (int rc = ensure_counts(c)) return rc;
        if (int rc = ensure_plain(c)) return rc;
    }
    if (int rc = cohort_wait_members(h, next)) return rc;
    for (vp_chain* c : h->chains) c->cohort = nullptr;
    h->chains = next;
    for (vp_chain* c : h->chains) c->cohort = h;
    cohort_reap(h, false);
    int rc = cohort_build(h);
    if (rc) {
        for (vp_chain* c : h->chains) c->cohort = nullptr;
        h->chains.clear();
    }
    return rc;
}

extern "C" int vp_cohort_run(vp_cohort* h, int32_t nsweeps) {
    if (!h || nsweeps < 0) { vp_set_error("bad arguments"); return VP_E_ARG; }
    if (h->chains.empty() || nsweeps == 0) return VP_OK;
    cudaSetDevice(h->device);
    for (int s = 0; s < nsweeps; ++s) CK(cudaGraphLaunch(h->graph, h->stream));
    h->launches += (int64_t)h->nodes * nsweeps;
    // members' own streams (results, Arrange, later single steps) follow
    CK(cudaEventRecord(h->ev, h->stream));
    for (vp_chain* c : h->chains) {
        CK(cudaStreamWaitEvent(c->ctx->stream, h->ev, 0));
        c->issued = (int)std::min<int64_t>(c->total, (int64_t)c->issued + nsweeps);
    }
    cohort_reap(h, false);
    return VP_OK;
}

extern "C" int vp_cohort_sync(vp_cohort* h) {
    if (!h) { vp_set_error("null argument"); return VP_E_ARG; }
    cudaSetDevice(h->device);
    CK(cudaStreamSynchronize(h->stream));
    cohort_reap(h, true);
    return VP_OK;
}

extern "C" void* vp_cohort_stream(vp_cohort* h) { return h ? (void*)h->stream : nullptr; }

extern "C" int64_t vp_cohort_launches(vp_cohort* h, int32_t* per_sweep) {
    if (!h) return -1;
    if (per_sweep) *per_sweep = h->nodes;
    return h->launches;
}

extern "C" int vp_cohort_close(vp_cohort* h) {
    if (!h) return VP_OK;
    cudaSetDevice(h->device);
    cudaStreamSynchronize(h->stream);
    for (vp_chain* c : h->chains) c->cohort = nullptr;
    h->chains.clear();
    if (h->graph) cudaGraphExecDestroy(h->graph);
    cohort_reap(h, true);
    dev_free(h->mem, h->stream);
    cudaStreamSynchronize(h->stream);
    cudaEventDestroy(h->ev);
    cudaStreamDestroy(h->stream);
    delete h;
    return VP_OK;
}

// ===================== tensor-core K-sweep =====================
namespace {

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
    static const EncodeTiledFn fn = [] {
        cudaDriverEntryPointQueryResult q;
        void* p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            return (EncodeTiledFn)p;
        return (EncodeTiledFn) nullptr;
    }();
    return fn;
}

// 2-D row-major [rows][ld] map of bf16 (esz 2) or bytes (esz 1) with
// box_cols x box_rows boxes; 128-byte box rows use the 128-byte swizzle,
// 64-byte rows the 64-byte one
int make_map(CUtensorMap* m, const void* base, uint64_t rows, uint64_t cols, uint64_t ld, uint32_t box_rows,
             uint32_t box_cols, int esz = 2) {
    const uint32_t rowb = box_cols * esz;
    if ((rowb != 64 && rowb != 128) || (esz != 1 && esz != 2)) { vp_set_error("box rows must be 64 or 128 bytes"); return VP_E_ARG; }
    EncodeTiledFn f = encode_fn();
    if (!f) { vp_set_error("cuTensorMapEncodeTiled unavailable"); return VP_E_CUDA; }
    cuuint64_t dims[2] = {cols, rows};
    cuuint64_t strides[1] = {ld * esz};
    cuuint32_t box[2] = {box_cols, box_rows};
    cuuint32_t es[2] = {1, 1};
    CUresult r = f(m, esz == 2 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_UINT8, 2,
                   const_cast<void*>(base), dims, strides, box, es,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, rowb == 128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B,
                   CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) { vp_set_error("cuTensorMapEncodeTiled failed (%d)", (int)r); return VP_E_CUDA; }
    return VP_OK;
}

template <int BKT, int ESZ, int MT, int NB, int BNT, int PIECE>
int launch_gemm_t(vp_ctx* x, const CUtensorMap& A, const CUtensorMap& B0, const CUtensorMap& B1, const tc::GemmArgs& g,
                  dim3 grid, size_t sm) {
    auto kern = tc::k_gemm_bf16<BKT, ESZ, MT, NB, BNT, PIECE>;
    static std::mutex mu;
    static std::vector<char> seen;
    if (first_on_device(mu, seen, x->device))
        CK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024));
    kern<<<grid, tc::NTHREADS, sm, x->stream>>>(A, B0, B1, g);
    x->last_gemm = (const void*)kern;
    return check_launch(x, "k_gemm_bf16");
}

// the tile shapes compiled into the library (K elements per stage, element
// bytes, 128-row A tiles per CTA, B operands, columns per CTA, columns per MMA)
#define VP_GEMM_TILES(X)             \
    X(64, 2, 2, 2, 192, 192)         \
    X(64, 2, 2, 2, 144, 144)         \
    X(64, 2, 2, 1, 192, 192)         \
    X(128, 1, 2, 1, 192, 192)        \
    X(64, 2, 1, 2, 288, 144)         \
    X(64, 2, 1, 1, 256, 256)         \
    X(32, 2, 2, 2, 192, 192)

int launch_gemm(vp_ctx* x, const CUtensorMap& A, const CUtensorMap& B0, const CUtensorMap& B1, tc::GemmArgs g,
                dim3 grid) {
    if (g.esz != 1 && g.esz != 2) { vp_set_error("gemm element size must be 1 or 2 bytes"); return VP_E_ARG; }
    if (g.bk * g.esz != 64 && g.bk * g.esz != 128) { vp_set_error("gemm stage rows must be 64 or 128 bytes"); return VP_E_ARG; }
    size_t sm = tc::gemm_smem_bytes(g.BN, g.nb, g.stages, g.mt, g.bk, g.esz);
    if (sm > 227 * 1024) { vp_set_error("gemm tile needs %zu bytes of shared memory", sm); return VP_E_ARG; }
    // a CTA whose accumulators take more than half of the SM's 512 TMEM
    // columns allocates all of them: reserve more than half of the SM's
    // shared memory too, so that no second CTA lands on its SM to wait
    if (g.mt * g.BN > 256) sm = std::max<size_t>(sm, 115 * 1024);
#define VP_GEMM_CASE(bk_, es_, mt_, nb_, bn_, pc_)                                                        \
    if (g.bk == bk_ && g.esz == es_ && g.mt == mt_ && g.nb == nb_ && g.BN == bn_ && g.piece == pc_)      \
        return launch_gemm_t<bk_, es_, mt_, nb_, bn_, pc_>(x, A, B0, B1, g, grid, sm);
    VP_GEMM_TILES(VP_GEMM_CASE)
#undef VP_GEMM_CASE
    vp_set_error("gemm tile (bk %d, esz %d, mt %d, nb %d, BN %d, piece %d) is not compiled in", g.bk, g.esz, g.mt, g.nb,
                 g.BN, g.piece);
    return VP_E_ARG;
}

int tc_operands(vp_ctx* x) {
    TcOperands& t = x->tc;
    if (t.ready) return VP_OK;
    if (!x->packed2) { vp_set_error("the tensor-core form needs biallelic diploid (packed) data"); return VP_E_ARG; }
    const int64_t A = 2 * x->L;
    t.Apad = (A + 63) / 64 * 64;
    t.Npad = (x->N + 127) / 128 * 128;
    const size_t cbytes = (size_t)t.Npad * t.Apad * 2, ctbytes = ((size_t)t.Npad * t.Apad + 255) / 256 * 256;
    // locus groups of the operand build (BUILD_TILES tiles of 64 loci each)
    const unsigned groups = cdiv(cdiv(x->L, 64), tc::BUILD_TILES);
    const size_t tail = t.Apad * 4 + t.Npad * 8 + 256 + (size_t)groups * t.Npad * 4;
    void* p = nullptr;
    cudaError_t e = dev_alloc(&p, cbytes + ctbytes + tail, x->device, x->stream);
    if (e != cudaSuccess) {
        vp_set_error("device allocation of %zu bytes for tensor-core operands: %s", cbytes + ctbytes + tail,
                     cudaGetErrorString(e));
        return VP_E_MEM;
    }
    x->allocs.push_back(p);
    char* q = (char*)p;
    t.C = (__nv_bfloat16*)q; q += cbytes;
    t.CT = (uint8_t*)q; q += ctbytes;
    CK(cudaMemsetAsync(q, 0, tail, x->stream));     // C and CT are written whole by k_build_counts
    t.logpbar = (float*)q; q += t.Apad * 4;
    t.Bc = (double*)q; q += t.Npad * 8;
    t.err = (int*)q; q += 256;
    float* part = (float*)q;
    int rc = VP_OK;
    do {
        tc::k_allele_center<<<cdiv(x->L * 32, 256), 256, 0, x->stream>>>(x->D, t.logpbar);
        if ((rc = check_launch(x, "k_allele_center"))) break;
        tc::k_build_counts<<<dim3((unsigned)(t.Npad / 128), groups, 1), 256, 0, x->stream>>>(
            x->D, t.C, t.CT, t.Apad, t.Npad, t.logpbar, part);
        if ((rc = check_launch(x, "k_build_counts"))) break;
        tc::k_center_sum<<<cdiv(x->N, 256), 256, 0, x->stream>>>(x->D, part, (int)groups, t.Npad, t.Bc);
        if ((rc = check_launch(x, "k_center_sum"))) break;
        if ((rc = make_map(&t.mapC, t.C, t.Npad, t.Apad, t.Apad, 128, t.bk))) break;
        rc = make_map(&t.mapCT, t.CT, t.Apad, t.Npad, t.Npad, 128, t.bk8, 1);
    } while (0);
    if (rc) {
        // nothing keeps the operands: a later call starts over
        x->allocs.pop_back();
        dev_free(p, x->stream);
        return rc;
    }
    t.ready = true;
    return VP_OK;
}

int tc_splits(int64_t tiles, int nsm) {
    // split the allele dimension so that the CTA count fills whole waves
    int best = 1;
    double beste = 0;
    for (int s = 1; s <= 24; ++s) {
        double ctas = (double)tiles * s, waves = ctas / nsm;
        double eff = waves / std::ceil(waves);
        if (eff > beste + 0.02) { beste = eff; best = s; }
        if (eff > 0.93) break;
    }
    return best;
}

// ---- launch configurations of the batched contractions and their tuner ----
// the likelihood-contraction tiles compiled in with two B operands (hi, lo):
// bf16 K elements per stage, 128-row tiles per CTA, cluster rows per CTA and
// per MMA
const int kTiles1[][4] = {{64, 2, 192, 192}, {64, 2, 144, 144}, {64, 1, 288, 144}, {32, 2, 192, 192}};
constexpr int kMaxStages = 6, kMaxSplits = 64;

// cluster rows of a chain group of the label draw (a chain of more rows is
// a group of its own: K <= 64 keeps the shared-memory sums of a tile of 32
// individuals within 48 KB)
constexpr int kSampleGroupRows = 160;


int64_t gemm1_tiles(const vp_ctx* x, int Rpad, const TcChoice& c) {
    return cdiv(x->tc.Npad, 128 * c.mt1) * (int64_t)(Rpad / c.bn1);
}

int choice_error(const vp_ctx* x, int Rpad, const TcChoice& c) {
    (void)x;
    bool tile = false;
    for (const auto& t : kTiles1) tile |= c.bk1 == t[0] && c.mt1 == t[1] && c.bn1 == t[2] && c.piece1 == t[3];
    if (!tile) {
        vp_set_error("likelihood tile (bk %d, row tiles %d, cols %d, piece %d) is not compiled in", c.bk1, c.mt1, c.bn1,
                     c.piece1);
        return VP_E_ARG;
    }
    if (Rpad % c.bn1) { vp_set_error("%d padded cluster rows are not whole groups of %d", Rpad, c.bn1); return VP_E_ARG; }
    if (c.st1 < 2 || c.st1 > kMaxStages || tc::gemm_smem_bytes(c.bn1, 2, c.st1, c.mt1, c.bk1, 2) > 227 * 1024) {
        vp_set_error("likelihood pipeline of %d stages does not fit", c.st1);
        return VP_E_ARG;
    }
    if (c.st2 < 2 || c.st2 > kMaxStages || tc::gemm_smem_bytes(192, 1, c.st2, 2, 128, 1) > 227 * 1024) {
        vp_set_error("count pipeline of %d stages does not fit", c.st2);
        return VP_E_ARG;
    }
    if (c.splits < 0 || c.splits > kMaxSplits || (c.gm1 != 0 && c.gm1 != 1) || (c.gm2 != 0 && c.gm2 != 1)) {
        vp_set_error("bad split count or CTA order");
        return VP_E_ARG;
    }
    return VP_OK;
}

// choices measured by vp_tune, per (individuals, padded alleles, cluster
// rows, SMs); with VP_TUNE_CACHE naming a file they are read from it at the
// first lookup and appended to it when measured
struct TuneKey {
    int64_t N, A;
    int R, nsm;
    bool operator==(const TuneKey& o) const { return N == o.N && A == o.A && R == o.R && nsm == o.nsm; }
};
std::mutex g_tune_mu;
std::vector<std::pair<TuneKey, TcChoice>> g_tuned;
bool g_tune_loaded = false;

void tune_put_locked(const TuneKey& k, const TcChoice& c) {
    for (auto& e : g_tuned)
        if (e.first == k) { e.second = c; return; }
    g_tuned.push_back({k, c});
}

void tune_load_locked() {
    if (g_tune_loaded) return;
    g_tune_loaded = true;
    const char* path = getenv("VP_TUNE_CACHE");
    FILE* f = path && *path ? fopen(path, "r") : nullptr;
    if (!f) return;
    long long N, A;
    TuneKey k;
    TcChoice c;
    while (fscanf(f, "%lld %lld %d %d %d %d %d %d %d %d %d %d %d", &N, &A, &k.R, &k.nsm, &c.bk1, &c.mt1, &c.bn1,
                  &c.piece1, &c.st1, &c.splits, &c.gm1, &c.st2, &c.gm2) == 13) {
        k.N = N; k.A = A;
        tune_put_locked(k, c);
    }
    fclose(f);
}

TuneKey tune_key(const vp_ctx* x, int R) { return TuneKey{x->N, x->tc.Apad, R, x->nsm}; }

TcChoice tuned_choice(const vp_ctx* x, int R) {
    std::lock_guard<std::mutex> g(g_tune_mu);
    tune_load_locked();
    const TuneKey k = tune_key(x, R);
    for (const auto& e : g_tuned)
        if (e.first == k) return e.second;
    return TcChoice{};
}

void tune_store(const vp_ctx* x, int R, const TcChoice& c) {
    std::lock_guard<std::mutex> g(g_tune_mu);
    tune_load_locked();
    const TuneKey k = tune_key(x, R);
    tune_put_locked(k, c);
    const char* path = getenv("VP_TUNE_CACHE");
    if (FILE* f = path && *path ? fopen(path, "a") : nullptr) {
        fprintf(f, "%lld %lld %d %d %d %d %d %d %d %d %d %d %d\n", (long long)k.N, (long long)k.A, k.R, k.nsm, c.bk1,
                c.mt1, c.bn1, c.piece1, c.st1, c.splits, c.gm1, c.st2, c.gm2);
        fclose(f);
    }
}

// the likelihood contraction of the current batch under choice c
// the likelihood contraction in `splits` split-K slices: all of them, or the
// `nz` slices from slice z0 on
int launch_gemm1(vp_ctx* x, const TcChoice& c, const CUtensorMap& A, const CUtensorMap& W0, const CUtensorMap& W1,
                 int splits, float* out, int z0 = 0, int nz = -1) {
    const TcOperands& t = x->tc;
    const TcBatch* b = x->batch;
    tc::GemmArgs g{};
    g.M = x->N; g.N = b->Rpad; g.kblocks = (int)(t.Apad / c.bk1);
    g.kb_per_split = (g.kblocks + splits - 1) / splits;
    g.BN = c.bn1; g.piece = c.piece1; g.nb = 2; g.mt = c.mt1; g.stages = c.st1; g.bk = c.bk1; g.esz = 2; g.mode = 0;
    g.group_major = c.gm1;
    g.out_f = out; g.ldo = b->Rpad; g.err = t.err;
    g.z0 = z0;
    const unsigned nzs = nz < 0 ? (unsigned)splits : (unsigned)nz;
    const unsigned mtiles = cdiv(t.Npad, 128 * c.mt1), groups = (unsigned)(b->Rpad / c.bn1);
    return launch_gemm(x, A, W0, W1, g, c.gm1 ? dim3(groups, mtiles, nzs) : dim3(mtiles, groups, nzs));
}

// copies each batch chain's header to the chain's own device header
__global__ void k_scatter_chains(const DevChain* src, DevChain* const* dst, int n) {
    static_assert(sizeof(DevChain) % 4 == 0, "DevChain copies as 32-bit words");
    if (blockIdx.x >= n) return;
    const uint32_t* a = reinterpret_cast<const uint32_t*>(src + blockIdx.x);
    uint32_t* d = reinterpret_cast<uint32_t*>(dst[blockIdx.x]);
    for (int j = threadIdx.x; j < (int)(sizeof(DevChain) / 4); j += blockDim.x) d[j] = a[j];
}

void free_batch(vp_ctx* x) {
    if (!x->batch) return;
    TcBatch* b = x->batch;
    const int n = (int)b->chains.size();
    std::vector<DevChain> hc(n);
    for (int i = 0; i < n; ++i) {
        vp_chain* c = b->chains[i];
        // hand each chain its counts back (stream-ordered after the batch's work)
        cudaMemcpyAsync(c->own_ni, c->h.Ni, (size_t)c->P.K * x->KT * 4, cudaMemcpyDeviceToDevice, x->stream);
        c->h.Ni = c->own_ni;
        hc[i] = c->h;
        if (c->graph) { cudaGraphExecDestroy(c->graph); c->graph = nullptr; }
    }
    cudaMemcpyAsync(b->dchains, hc.data(), n * sizeof(DevChain), cudaMemcpyHostToDevice, x->stream);
    k_scatter_chains<<<n, 128, 0, x->stream>>>(b->dchains, b->dptrs, n);
    x->launches++;
    if (b->graph) cudaGraphExecDestroy(b->graph);
    dev_free(b->mem, x->stream);
    delete b;
    x->batch = nullptr;
}

int make_batch(vp_ctx* x, vp_chain** cs, int n, const TcChoice* force) {
    if (x->batch) {
        TcBatch* b = x->batch;
        if (!force && (int)b->chains.size() == n && std::equal(b->chains.begin(), b->chains.end(), cs)) return VP_OK;
        free_batch(x);
    }
    int rc = tc_operands(x);
    if (rc) return rc;
    for (int i = 0; i < n; ++i) {
        const vp_params& P = cs[i]->P;
        if (P.admix || P.locpriori || P.fmodel || cs[i]->issued < cs[i]->h.nadmburnin || P.rng != VP_RNG_COUNTER) {
            vp_set_error("the tensor-core form runs no-admixture chains without location prior or F model, with "
                         "counter streams, past their admixture burn-in");
            return VP_E_ARG;
        }
    }
    auto* b = new TcBatch();
    b->chains.assign(cs, cs + n);
    std::vector<int32_t> rowchain, rowk, row0;
    for (int i = 0; i < n; ++i) {
        row0.push_back((int32_t)rowchain.size());
        for (int k = 0; k < cs[i]->P.K; ++k) { rowchain.push_back(i); rowk.push_back(k); }
    }
    b->R = (int)rowchain.size();
    // chain groups of the label draw: consecutive chains, at most
    // kSampleGroupRows cluster rows unless one chain has more
    std::vector<int4> sgrp;
    for (int i = 0; i < n; ++i) {
        const int K = cs[i]->P.K;
        if (sgrp.empty() || sgrp.back().w + K > kSampleGroupRows) sgrp.push_back(make_int4(i, i, row0[i], 0));
        sgrp.back().y = i + 1;
        sgrp.back().w += K;
    }
    b->nsgrp = (int)sgrp.size();
    for (const int4& gr : sgrp) b->sgrp_rows = std::max(b->sgrp_rows, gr.w);
    b->G = (b->R + b->BN - 1) / b->BN;
    b->Rpad = b->G * b->BN;
    const TcOperands& t = x->tc;
    b->cfg = force ? *force : tuned_choice(x, b->R);
    if (choice_error(x, b->Rpad, b->cfg)) {
        if (force) { delete b; return VP_E_ARG; }
        b->cfg = TcChoice{};
    }
    b->G1 = b->Rpad / b->cfg.bn1;
    b->splits = b->cfg.splits > 0 ? b->cfg.splits : tc_splits(gemm1_tiles(x, b->Rpad, b->cfg), x->nsm);
    const int64_t kblocks = t.Apad / b->cfg.bk1;
    b->splits = (int)std::min<int64_t>(b->splits, kblocks);
    b->splits = (int)cdiv(kblocks, cdiv(kblocks, b->splits));   // splits that hold k-blocks
    Carve probe{nullptr};
    auto lay = [&](Carve& cv) {
        b->dchains = cv.take<DevChain>(n);
        b->dptrs = cv.take<DevChain*>(n);
        b->lnlrec = cv.take<double>((int64_t)n * 128);
        b->rowchain = cv.take<int32_t>(b->R);
        b->rowk = cv.take<int32_t>(b->R);
        b->row0 = cv.take<int32_t>(n);
        b->sgrp = cv.take<int4>(b->nsgrp);
        b->Whi = cv.take<__nv_bfloat16>((int64_t)b->Rpad * t.Apad);
        b->Wlo = cv.take<__nv_bfloat16>((int64_t)b->Rpad * t.Apad);
        b->OH = cv.take<uint8_t>((int64_t)b->Rpad * t.Npad);
        b->LLpart = cv.take<float>((int64_t)b->splits * x->N * b->Rpad);
        b->NiAll = cv.take<int32_t>((int64_t)b->Rpad * x->KT);
    };
    lay(probe);
    cudaError_t e = dev_alloc(&b->mem, probe.off, x->device, x->stream);
    if (e != cudaSuccess) { delete b; vp_set_error("device allocation of %zu bytes for the batch: %s", probe.off, cudaGetErrorString(e)); return VP_E_MEM; }
    Carve cv{(char*)b->mem};
    lay(cv);
    // a failure before the chains' device headers are rewritten leaves the
    // chains as they were
    auto undo = [&](const char* what, cudaError_t err) {
        for (int i = 0; i < n; ++i) cs[i]->h.Ni = cs[i]->own_ni;
        dev_free(b->mem, x->stream);
        delete b;
        vp_set_error("%s failed: %s", what, cudaGetErrorString(err));
        return VP_E_CUDA;
    };
    if ((e = cudaMemsetAsync(b->mem, 0, probe.off, x->stream)) != cudaSuccess ||
        (e = cudaMemcpyAsync(b->rowchain, rowchain.data(), rowchain.size() * 4, cudaMemcpyHostToDevice, x->stream)) != cudaSuccess ||
        (e = cudaMemcpyAsync(b->rowk, rowk.data(), rowk.size() * 4, cudaMemcpyHostToDevice, x->stream)) != cudaSuccess ||
        (e = cudaMemcpyAsync(b->row0, row0.data(), row0.size() * 4, cudaMemcpyHostToDevice, x->stream)) != cudaSuccess ||
        (e = cudaMemcpyAsync(b->sgrp, sgrp.data(), sgrp.size() * sizeof(int4), cudaMemcpyHostToDevice, x->stream)) != cudaSuccess)
        return undo("batch upload", e);
    // the batch's count contraction writes every chain's Ni inside NiAll
    // (counts still pending are computed there below); the chains' device
    // headers are updated by one upload and a scatter kernel
    std::vector<DevChain> hc(n);
    std::vector<DevChain*> hp(n);
    for (int i = 0; i < n; ++i) {
        vp_chain* c = cs[i];
        int32_t* dst = b->NiAll + (int64_t)row0[i] * x->KT;
        if (!c->counts_pending &&
            (e = cudaMemcpyAsync(dst, c->h.Ni, (size_t)c->P.K * x->KT * 4, cudaMemcpyDeviceToDevice, x->stream)) != cudaSuccess)
            return undo("copy of a chain's counts into the batch", e);
        c->h.Ni = dst;
        hc[i] = c->h;
        hp[i] = c->d;
    }
    if ((e = cudaMemcpyAsync(b->dchains, hc.data(), n * sizeof(DevChain), cudaMemcpyHostToDevice, x->stream)) != cudaSuccess ||
        (e = cudaMemcpyAsync(b->dptrs, hp.data(), n * sizeof(DevChain*), cudaMemcpyHostToDevice, x->stream)) != cudaSuccess)
        return undo("batch header upload", e);
    k_scatter_chains<<<n, 128, 0, x->stream>>>(b->dchains, b->dptrs, n);
    x->launches++;
    if ((e = cudaGetLastError()) != cudaSuccess) return undo("launch of k_scatter_chains", e);
    for (int i = 0; i < n; ++i)
        if (cs[i]->graph) { cudaGraphExecDestroy(cs[i]->graph); cs[i]->graph = nullptr; }
    if ((rc = make_map(&b->mapC1, t.C, t.Npad, t.Apad, t.Apad, 128, b->cfg.bk1)) ||
        (rc = make_map(&b->mapWhi, b->Whi, b->Rpad, t.Apad, t.Apad, b->cfg.piece1, b->cfg.bk1)) ||
        (rc = make_map(&b->mapWlo, b->Wlo, b->Rpad, t.Apad, t.Apad, b->cfg.piece1, b->cfg.bk1)) ||
        (rc = make_map(&b->mapOH, b->OH, b->Rpad, t.Npad, t.Npad, b->piece, t.bk8, 1))) {
        x->batch = b;
        free_batch(x);
        return rc;
    }
    x->batch = b;
    // initial counts the chains left to the batch: one-hot rows of their
    // initial labels through the count contraction, for every chain at once
    bool pending = false;
    for (int i = 0; i < n; ++i) pending |= cs[i]->counts_pending;
    if (pending) {
        tc::BatchDev bd = batch_dev(x);
        LAUNCH(x, tc::k_onehot_from_z, (dim3(cdiv(x->N, 256), n, 1), 256, 0, x->stream), (bd));
        if ((rc = launch_counts_gemm(x))) return rc;
        for (int i = 0; i < n; ++i) cs[i]->counts_pending = false;
    }
    return VP_OK;
}

tc::BatchDev batch_dev(vp_ctx* x) {
    TcBatch* b = x->batch;
    tc::BatchDev d;
    d.chains = b->dchains; d.rowchain = b->rowchain; d.rowk = b->rowk; d.row0 = b->row0;
    d.R = b->R; d.Rpad = b->Rpad; d.nchains = (int)b->chains.size(); d.splits = b->splits;
    d.Apad = x->tc.Apad; d.Npad = x->tc.Npad; d.Whi = b->Whi; d.Wlo = b->Wlo; d.OH = b->OH;
    d.logpbar = x->tc.logpbar; d.Bc = x->tc.Bc; d.LLpart = b->LLpart;
    d.sgrp = b->sgrp; d.sgrp_ld = b->sgrp_rows | 1;
    return d;
}

// UpdateP blocks along the loci for `nloci` loci of R rows: between 2 and
// 16 (at most one block per 256 loci), chosen so that the blocks fill whole
// waves of the kernel's resident blocks
unsigned updatep_blocks(const vp_ctx* x, int64_t nloci, int R) {
    static const int per_sm = [] {
        int v = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, tc::k_update_p_tc, 256, 0) != cudaSuccess || v < 1) v = 4;
        return v;
    }();
    const double slots = (double)x->nsm * std::max(1, per_sm);
    const unsigned hi = std::max<unsigned>(1, std::min<unsigned>(16, cdiv(nloci, 256)));
    unsigned upx = 1;
    double best = -1;
    for (unsigned u = std::min(2u, hi); u <= hi; ++u) {
        const double w = (double)u * R / slots, eff = w / std::ceil(w);
        if (eff > best + 0.01) { best = eff; upx = u; }
    }
    return upx;
}

// branch streams and events for a sweep's fork and join
int fork_resources(vp_ctx* x, int nstreams, int nevents) {
    while ((int)x->fork.size() < nstreams) {
        cudaStream_t f;
        CK(cudaStreamCreateWithFlags(&f, cudaStreamNonBlocking));
        x->fork.push_back(f);
    }
    while ((int)x->fork_ev.size() < nevents) {
        cudaEvent_t e;
        CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        x->fork_ev.push_back(e);
    }
    return VP_OK;
}

// dynamic shared memory of an UpdateP block that lets at most `share` of
// them sit on an SM beside one CTA of the likelihood contraction (the
// contraction's issuing warps then share their schedulers with fewer ALU
// warps); 0 when the contraction leaves no room to divide
size_t updatep_share_smem(const vp_ctx* x, int share) {
    const TcChoice& c = x->batch->cfg;
    size_t g = tc::gemm_smem_bytes(c.bn1, 2, c.st1, c.mt1, c.bk1, 2);
    if (c.mt1 * c.bn1 > 256) g = std::max<size_t>(g, 115 * 1024);     // launch_gemm's TMEM rule
    int per_sm = 0, reserved = 0;
    if (cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, x->device) != cudaSuccess ||
        cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, x->device) != cudaSuccess)
        return 0;
    const int64_t room = (int64_t)per_sm - (int64_t)g - reserved;
    if (room <= 0) return 0;
    // a slot inside (room / (share + 1), room / share]: `share` slots fit, one more does not
    const int64_t slot = (room / (share + 1) + room / share) / 2;
    return (size_t)std::max<int64_t>(0, slot - reserved);
}

// launches go to another stream while in scope
struct OnStream {
    vp_ctx* x;
    cudaStream_t saved;
    OnStream(vp_ctx* x_, cudaStream_t f) : x(x_), saved(x_->stream) { x->stream = f; }
    ~OnStream() { x->stream = saved; }
};

// split-K slices of the likelihood contraction that run as separate ranges
int pipeline_ranges(const vp_ctx* x) {
    const TcBatch* b = x->batch;
    return x->tc_pipeline && b->splits > 1 ? b->splits : 1;
}

int launch_tc_sweep(vp_ctx* x) {
    TcBatch* b = x->batch;
    const int n = (int)b->chains.size();
    tc::BatchDev bd = batch_dev(x);
    cudaStream_t s = x->stream;
    const int nr = pipeline_ranges(x);
    if (nr == 1) {
        // UpdateP for all chains, with the split-bf16 centred log-frequency
        // rows (R rows x upx blocks, each thread walking many loci), then
        // the likelihood contraction
        const unsigned upx = updatep_blocks(x, x->L, b->R);
        prof_mark(x, true, PROF_UPDATEP_TC);
        LAUNCH(x, tc::k_update_p_tc, (dim3(upx, b->R, 1), 256, 0, s), (bd, (int64_t)0, x->L));
        prof_mark(x, false, PROF_UPDATEP_TC);
        prof_mark(x, true);
        int rc = launch_gemm1(x, b->cfg, b->mapC1, b->mapWhi, b->mapWlo, b->splits, b->LLpart);
        prof_mark(x, false);
        if (rc) return rc;
        b->gemm1_fn = x->last_gemm;
    } else {
        // by allele ranges, one per split-K slice of the likelihood
        // contraction: UpdateP of the ranges one after another on one
        // branch, each range's slice on a branch of its own once the range's
        // draws are written. The slices (tensor pipes, one CTA per SM) and
        // the next range's draws (ALUs, in the registers the contraction
        // leaves) share the SMs; the slices take precedence (graph node
        // priority). The slices write disjoint split-K partials, so the
        // labels are those of the single-launch order.
        const int ng = std::min(nr, 8);
        if (int rc = fork_resources(x, 1 + ng, 2 * nr + 3)) return rc;
        const size_t psm = updatep_share_smem(x, x->tc_pipeline);
        {
            static std::mutex mu;
            static std::vector<char> seen;
            if (first_on_device(mu, seen, x->device))
                CK(cudaFuncSetAttribute(tc::k_update_p_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024));
        }
        cudaEvent_t* ev = x->fork_ev.data();
        cudaStream_t ps = x->fork[0];
        CK(cudaEventRecord(ev[0], s));
        CK(cudaStreamWaitEvent(ps, ev[0], 0));
        const int64_t kbps = cdiv(x->tc.Apad / b->cfg.bk1, b->splits);
        const int64_t loci = kbps * b->cfg.bk1 / 2;          // biallelic: two allele columns per locus
        for (int r = 0; r < nr; ++r) {
            const int64_t l0 = r * loci, l1 = std::min<int64_t>(x->L, l0 + loci);
            {
                OnStream on(x, ps);
                if (r == 0) prof_mark(x, true, PROF_UPDATEP_TC);
                if (l1 > l0) {
                    // the first range runs alone: no cap
                    const unsigned upx = updatep_blocks(x, l1 - l0, b->R);
                    LAUNCH(x, tc::k_update_p_tc, (dim3(upx, b->R, 1), 256, r ? psm : 0, ps), (bd, l0, l1));
                }
                if (r == nr - 1) prof_mark(x, false, PROF_UPDATEP_TC);
                CK(cudaEventRecord(ev[1 + r], ps));
            }
            cudaStream_t gs = x->fork[1 + r % ng];
            CK(cudaStreamWaitEvent(gs, ev[1 + r], 0));
            {
                OnStream on(x, gs);
                if (r == 0) prof_mark(x, true);
                int rc = launch_gemm1(x, b->cfg, b->mapC1, b->mapWhi, b->mapWlo, b->splits, b->LLpart, r, 1);
                if (rc) return rc;
                CK(cudaEventRecord(ev[1 + nr + r], gs));
            }
        }
        b->gemm1_fn = x->last_gemm;
        for (int r = 0; r < nr; ++r) CK(cudaStreamWaitEvent(s, ev[1 + nr + r], 0));
        CK(cudaEventRecord(ev[1 + 2 * nr], ps));        // the UpdateP branch rejoins too
        CK(cudaStreamWaitEvent(s, ev[1 + 2 * nr], 0));
        prof_mark(x, false);
    }
    // labels of every chain, one-hot rows for the count contraction
    const size_t tsm = (size_t)tc::TS_TILE * (b->sgrp_rows | 1) * sizeof(float);
    LAUNCH(x, tc::k_sample_tc_tiles, (dim3(cdiv(x->N, tc::TS_TILE), b->nsgrp, 1), tc::TS_THREADS, tsm, s), (bd));
    // count contraction: Ni[row, a] = sum_i OH[row, i] C[i, a]
    if (int rc = launch_counts_gemm(x)) return rc;
    // Record for every chain, then m += 1
    unsigned ga = std::min<unsigned>(128, cdiv((int64_t)16 * x->KT, 256));
    LAUNCH(x, k_record_sweep, (dim3(ga, 1, n), 256, 0, s), (b->dchains, b->lnlrec));
    return VP_OK;
}

// graph node priorities of a captured sweep: the likelihood contraction's
// slices one level above the rest, which keep the context stream's priority
int set_node_priorities(vp_ctx* x, cudaGraph_t g, const void* hi_fn) {
    int least = 0, greatest = 0, base = 0;
    CK(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    CK(cudaStreamGetPriority(x->stream, &base));
    int hi = base, lo = base;
    if (base > greatest) hi = base - 1;        // numerically lower is more urgent
    else if (base < least) lo = base + 1;
    size_t nn = 0;
    CK(cudaGraphGetNodes(g, nullptr, &nn));
    std::vector<cudaGraphNode_t> nodes(nn);
    CK(cudaGraphGetNodes(g, nodes.data(), &nn));
    for (cudaGraphNode_t nd : nodes) {
        cudaGraphNodeType ty;
        CK(cudaGraphNodeGetType(nd, &ty));
        if (ty != cudaGraphNodeTypeKernel) continue;
        cudaKernelNodeParams kp{};
        CK(cudaGraphKernelNodeGetParams(nd, &kp));
        cudaLaunchAttributeValue v{};
        v.priority = kp.func == hi_fn ? hi : lo;
        CK(cudaGraphKernelNodeSetAttribute(nd, cudaLaunchAttributePriority, &v));
    }
    return VP_OK;
}

// the count contraction of the batch: Ni[row, a] = sum_i OH[row, i] C[i, a]
// into every chain's Ni (e4m3 operands, exact), or into `out` ([Rpad][KT])
int launch_counts_gemm(vp_ctx* x, int32_t* out) {
    TcBatch* b = x->batch;
    const TcOperands& t = x->tc;
    {
        tc::GemmArgs g{};
        g.M = (int)(2 * x->L); g.N = b->Rpad; g.kblocks = (int)(t.Npad / t.bk8); g.kb_per_split = g.kblocks;
        g.BN = b->BN; g.piece = b->piece; g.nb = 1; g.mt = b->mt2; g.stages = b->cfg.st2; g.bk = t.bk8; g.esz = 1;
        g.mode = 1; g.out_i = out ? out : b->NiAll; g.ldo = x->KT; g.err = t.err;
        const unsigned mtiles = cdiv(t.Apad, 128 * b->mt2);
        g.group_major = b->cfg.gm2 && mtiles <= 65535;     // grid.y limit; otherwise row tiles on x
        const dim3 grid = g.group_major ? dim3(b->G, mtiles, 1) : dim3(mtiles, b->G, 1);
        return launch_gemm(x, t.mapCT, b->mapOH, b->mapOH, g, grid);
    }
}

int run_tc(vp_ctx* x, vp_chain** cs, int n, int nsweeps) {
    int rc = make_batch(x, cs, n, nullptr);
    if (rc) return rc;
    TcBatch* b = x->batch;
    if (!b->graph) {
        cudaGraph_t g;
        x->prof_next = 0;
        x->prof_used = 0;
        CK(cudaStreamBeginCapture(x->stream, cudaStreamCaptureModeThreadLocal));
        int64_t before = x->launches;
        rc = launch_tc_sweep(x);
        cudaError_t e = cudaStreamEndCapture(x->stream, &g);
        if (rc) { if (e == cudaSuccess) cudaGraphDestroy(g); return rc; }
        if (e != cudaSuccess) { vp_set_error("graph capture failed: %s", cudaGetErrorString(e)); return VP_E_CUDA; }
        b->graph_nodes = (int)(x->launches - before);
        x->launches = before;
        const bool forked = pipeline_ranges(x) > 1;
        if (forked && (rc = set_node_priorities(x, g, b->gemm1_fn))) { cudaGraphDestroy(g); return rc; }
        e = cudaGraphInstantiate(&b->graph, g, forked ? cudaGraphInstantiateFlagUseNodePriority : 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) { vp_set_error("graph instantiate failed: %s", cudaGetErrorString(e)); return VP_E_CUDA; }
    }
    for (int i = 0; i < nsweeps; ++i) {
        CK(cudaGraphLaunch(b->graph, x->stream));
        x->launches += b->graph_nodes;
    }
    return VP_OK;
}

}  // namespace

namespace {
// mean device time of `iters` launches of fn after one untimed launch, on the
// context's stream; a launch whose pipeline wait gave up marks the candidate
// unusable (infinite time) and the flag is cleared
template <class F>
int time_candidate(vp_ctx* x, F fn, int iters, float* ms) {
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    if (cudaEventCreate(&e1) != cudaSuccess) { cudaEventDestroy(e0); vp_set_error("cudaEventCreate failed"); return VP_E_CUDA; }
    int rc = fn();
    if (!rc) {
        cudaEventRecord(e0, x->stream);
        for (int i = 0; i < iters && !rc; ++i) rc = fn();
        cudaEventRecord(e1, x->stream);
    }
    const cudaError_t e = cudaStreamSynchronize(x->stream);
    float t = 0.f;
    if (!rc && e == cudaSuccess) cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) { vp_set_error("tuning launch failed: %s", cudaGetErrorString(e)); return VP_E_CUDA; }
    if (rc) return rc;
    int flag = 0;
    CK(cudaMemcpy(&flag, x->tc.err, sizeof flag, cudaMemcpyDeviceToHost));
    if (flag) {
        CK(cudaMemset(x->tc.err, 0, sizeof flag));
        *ms = INFINITY;
        return VP_OK;
    }
    *ms = t / iters;
    return VP_OK;
}

// split counts to try: the whole-wave rule's, then the best wave fill, each
// a count whose splits all hold k-blocks
std::vector<int> split_candidates(const vp_ctx* x, int64_t tiles, int64_t kblocks, int keep) {
    auto norm = [&](int64_t s) { return (int)cdiv(kblocks, cdiv(kblocks, std::max<int64_t>(1, std::min(s, kblocks)))); };
    std::vector<int> out{norm(tc_splits(tiles, x->nsm))};
    std::vector<std::pair<double, int>> v;
    for (int s = 1; s <= std::min<int64_t>(kMaxSplits, kblocks); ++s) {
        if (norm(s) != s) continue;
        const double w = (double)tiles * s / x->nsm;
        v.push_back({-w / std::ceil(w), s});
    }
    std::sort(v.begin(), v.end());
    for (const auto& e : v) {
        if ((int)out.size() >= keep) break;
        if (std::find(out.begin(), out.end(), e.second) == out.end()) out.push_back(e.second);
    }
    return out;
}

bool same_gemm1(const TcChoice& a, const TcChoice& b) {
    return a.bk1 == b.bk1 && a.mt1 == b.mt1 && a.bn1 == b.bn1 && a.piece1 == b.piece1 && a.st1 == b.st1 &&
           a.splits == b.splits && a.gm1 == b.gm1;
}

// times the current batch's contractions under candidate configurations
// (effort 0: the current one; 1: its tile with every pipeline depth, split
// count and CTA order; 2: every compiled tile as well) and returns the
// fastest. The likelihood contraction writes a scratch buffer; the count
// contraction recomputes the chains' counts from their labels, which leaves
// them unchanged.
int tune_batch(vp_ctx* x, int effort, TcChoice* best, vp_tc_config* info) {
    TcBatch* b = x->batch;
    const TcOperands& t = x->tc;
    TcChoice cur = b->cfg;
    cur.splits = b->splits;
    std::vector<TcChoice> c1{cur};
    for (const auto& tl : kTiles1) {
        TcChoice c = cur;
        c.bk1 = tl[0]; c.mt1 = tl[1]; c.bn1 = tl[2]; c.piece1 = tl[3];
        const bool tile = c.bk1 == cur.bk1 && c.mt1 == cur.mt1 && c.bn1 == cur.bn1 && c.piece1 == cur.piece1;
        if (effort == 0 || (effort < 2 && !tile) || b->Rpad % c.bn1) continue;
        const std::vector<int> ss = split_candidates(x, gemm1_tiles(x, b->Rpad, c), t.Apad / c.bk1, 4);
        for (int st = 2; st <= kMaxStages; ++st) {
            if (tc::gemm_smem_bytes(c.bn1, 2, st, c.mt1, c.bk1, 2) > 227 * 1024) break;
            for (int gm = 0; gm < 2; ++gm)
                for (int sp : ss) {
                    TcChoice d = c;
                    d.st1 = st; d.gm1 = gm; d.splits = sp;
                    bool dup = false;
                    for (const auto& e : c1) dup |= same_gemm1(e, d);
                    if (!dup) c1.push_back(d);
                }
        }
    }
    int smax = 1;
    for (const auto& c : c1) smax = std::max(smax, c.splits);
    void* scratch = nullptr;
    cudaError_t e = dev_alloc(&scratch, (size_t)smax * x->N * b->Rpad * 4, x->device, x->stream);
    if (e != cudaSuccess) { vp_set_error("tuning scratch: %s", cudaGetErrorString(e)); return VP_E_MEM; }
    const int iters = effort ? 2 : 3;
    float best1 = INFINITY;
    TcChoice bc = cur;
    int rc = VP_OK;
    for (size_t i = 0; i < c1.size() && !rc; ++i) {
        const TcChoice& c = c1[i];
        CUtensorMap mA, mW0, mW1;
        if ((rc = make_map(&mA, t.C, t.Npad, t.Apad, t.Apad, 128, c.bk1)) ||
            (rc = make_map(&mW0, b->Whi, b->Rpad, t.Apad, t.Apad, c.piece1, c.bk1)) ||
            (rc = make_map(&mW1, b->Wlo, b->Rpad, t.Apad, t.Apad, c.piece1, c.bk1)))
            break;
        float ms = 0.f;
        rc = time_candidate(x, [&] { return launch_gemm1(x, c, mA, mW0, mW1, c.splits, (float*)scratch); }, iters, &ms);
        if (rc) break;
        // the label kernel reads every split's partial plane once
        const float score = ms + (float)((double)c.splits * x->N * b->Rpad * 4 / 6.0e9);
        if (i == 0) info->ms_likelihood_default = ms;
        if (score < best1) { best1 = score; bc = c; info->ms_likelihood = ms; }
    }
    dev_free(scratch, x->stream);
    if (rc) return rc;
    // count contraction: pipeline depth and CTA order, on one-hot rows of the
    // chains' current labels, into a scratch matrix (the chains' own counts
    // may come from per-copy draws that the labels do not give back)
    {
        tc::BatchDev bd = batch_dev(x);
        LAUNCH(x, tc::k_onehot_from_z, (dim3(cdiv(x->N, 256), (unsigned)b->chains.size(), 1), 256, 0, x->stream), (bd));
    }
    int32_t* ni_scratch = nullptr;
    e = dev_alloc((void**)&ni_scratch, (size_t)b->Rpad * x->KT * 4, x->device, x->stream);
    if (e != cudaSuccess) { vp_set_error("tuning scratch: %s", cudaGetErrorString(e)); return VP_E_MEM; }
    const TcChoice save = b->cfg;
    float best2 = INFINITY;
    int bst2 = save.st2, bgm2 = save.gm2, ncand = (int)c1.size();
    for (int pass = 0; pass < 2 && !rc; ++pass)
        for (int st = 2; st <= kMaxStages && !rc; ++st) {
            if (tc::gemm_smem_bytes(192, 1, st, 2, 128, 1) > 227 * 1024) break;
            for (int gm = 0; gm < 2 && !rc; ++gm) {
                const bool is_cur = st == save.st2 && gm == save.gm2;
                if (pass == 0 ? !is_cur : (is_cur || effort == 0)) continue;   // the current one first
                b->cfg.st2 = st;
                b->cfg.gm2 = gm;
                float ms = 0.f;
                rc = time_candidate(x, [&] { return launch_counts_gemm(x, ni_scratch); }, iters, &ms);
                ++ncand;
                if (rc) break;
                if (pass == 0) info->ms_counts_default = ms;
                if (ms < best2) { best2 = ms; bst2 = st; bgm2 = gm; info->ms_counts = ms; }
            }
        }
    b->cfg = save;
    dev_free(ni_scratch, x->stream);
    if (rc) return rc;
    *best = bc;
    best->st2 = bst2;
    best->gm2 = bgm2;
    info->candidates = ncand;
    return VP_OK;
}

void fill_config(const TcBatch* b, vp_tc_config* o) {
    o->bk = b->cfg.bk1; o->row_tiles = b->cfg.mt1; o->cols = b->cfg.bn1; o->piece = b->cfg.piece1;
    o->stages = b->cfg.st1; o->splits = b->splits; o->group_major = b->cfg.gm1;
    o->count_stages = b->cfg.st2; o->count_group_major = b->cfg.gm2;
}

int tc_chain_set(vp_chain** cs, int32_t n, vp_ctx** out) {
    if (!cs || n <= 0) { vp_set_error("no chains"); return VP_E_ARG; }
    for (int i = 0; i < n; ++i) {
        if (!cs[i] || cs[i]->ctx != cs[0]->ctx) { vp_set_error("the chains must share one context"); return VP_E_ARG; }
        if (cs[i]->P.form != VP_FORM_TC) { vp_set_error("chain %d is not a tensor-core chain", i); return VP_E_ARG; }
    }
    *out = cs[0]->ctx;
    return VP_OK;
}
}  // namespace

extern "C" int vp_tune(vp_chain** cs, int32_t n, int32_t effort, vp_tc_config* out) {
    vp_ctx* x = nullptr;
    if (int rc = tc_chain_set(cs, n, &x)) return rc;
    if (effort < 0 || effort > 2) { vp_set_error("effort must be 0, 1 or 2"); return VP_E_ARG; }
    cudaSetDevice(x->device);
    int rc = make_batch(x, cs, n, nullptr);
    if (rc) return rc;
    vp_tc_config info{};
    TcChoice best;
    if ((rc = tune_batch(x, effort, &best, &info))) return rc;
    if (effort > 0) {
        if ((rc = make_batch(x, cs, n, &best))) return rc;
        tune_store(x, x->batch->R, best);
    }
    if (out) {
        fill_config(x->batch, &info);
        *out = info;
    }
    return VP_OK;
}

extern "C" int vp_tc_configure(vp_chain** cs, int32_t n, const vp_tc_config* cfg) {
    vp_ctx* x = nullptr;
    if (int rc = tc_chain_set(cs, n, &x)) return rc;
    if (!cfg) { vp_set_error("null configuration"); return VP_E_ARG; }
    cudaSetDevice(x->device);
    TcChoice c;
    c.bk1 = cfg->bk; c.mt1 = cfg->row_tiles; c.bn1 = cfg->cols; c.piece1 = cfg->piece; c.st1 = cfg->stages;
    c.splits = cfg->splits; c.gm1 = cfg->group_major; c.st2 = cfg->count_stages; c.gm2 = cfg->count_group_major;
    return make_batch(x, cs, n, &c);
}

extern "C" int vp_tc_config_get(vp_chain** cs, int32_t n, vp_tc_config* out) {
    vp_ctx* x = nullptr;
    if (int rc = tc_chain_set(cs, n, &x)) return rc;
    if (!out) { vp_set_error("null output"); return VP_E_ARG; }
    cudaSetDevice(x->device);
    if (int rc = make_batch(x, cs, n, nullptr)) return rc;
    *out = vp_tc_config{};
    fill_config(x->batch, out);
    return VP_OK;
}

extern "C" int vp_tc_status(vp_ctx* x) {
    if (!x) { vp_set_error("null context"); return VP_E_ARG; }
    if (!x->tc.ready) return 0;
    // the context's stream is non-blocking: a copy on the default stream
    // would not wait for the kernels (or the initial clear) queued on it
    cudaSetDevice(x->device);
    CK(cudaStreamSynchronize(x->stream));
    int e = 0;
    CK(cudaMemcpy(&e, x->tc.err, sizeof(int), cudaMemcpyDeviceToHost));
    return e;
}

extern "C" int vp_debug_gemm_bf16(const uint16_t* A, const uint16_t* B0, const uint16_t* B1, int32_t M, int32_t N,
                                  int32_t K, int32_t BN, int32_t piece, int32_t splits, int32_t stages, int32_t mt,
                                  int32_t bk, float* D) {
    if (!A || !B0 || !D || M <= 0 || N <= 0 || K <= 0 || (bk != 32 && bk != 64) || K % bk || N % BN || BN % piece ||
        piece % 16 || piece > 256 || (mt != 1 && mt != 2) || BN * mt > 512 || splits < 1) {
        vp_set_error("vp_debug_gemm_bf16: bad shape");
        return VP_E_ARG;
    }
    vp_ctx tmp;
    cudaStreamCreateWithFlags(&tmp.stream, cudaStreamNonBlocking);
    const int64_t Mp = (M + 128 * mt - 1) / (128 * mt) * (128 * mt);
    void *dA, *dB0, *dB1 = nullptr, *dD;
    int* err;
    CK(cudaMalloc(&dA, (size_t)Mp * K * 2));
    CK(cudaMemset(dA, 0, (size_t)Mp * K * 2));
    CK(cudaMalloc(&dB0, (size_t)N * K * 2));
    CK(cudaMalloc(&dD, (size_t)splits * M * N * 4));
    CK(cudaMalloc(&err, 4));
    CK(cudaMemset(err, 0, 4));
    CK(cudaMemcpy(dA, A, (size_t)M * K * 2, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(dB0, B0, (size_t)N * K * 2, cudaMemcpyHostToDevice));
    if (B1) {
        CK(cudaMalloc(&dB1, (size_t)N * K * 2));
        CK(cudaMemcpy(dB1, B1, (size_t)N * K * 2, cudaMemcpyHostToDevice));
    }
    CUtensorMap ma, mb0, mb1;
    int rc = make_map(&ma, dA, Mp, K, K, 128, bk);
    if (!rc) rc = make_map(&mb0, dB0, N, K, K, piece, bk);
    if (!rc) rc = make_map(&mb1, B1 ? dB1 : dB0, N, K, K, piece, bk);
    if (!rc) {
        tc::GemmArgs g{};
        g.M = M; g.N = N; g.kblocks = K / bk; g.kb_per_split = (g.kblocks + splits - 1) / splits;
        g.BN = BN; g.piece = piece; g.nb = B1 ? 2 : 1; g.mt = mt; g.stages = stages; g.bk = bk; g.esz = 2; g.mode = 0;
        g.out_f = (float*)dD; g.ldo = N; g.err = err;
        rc = launch_gemm(&tmp, ma, mb0, mb1, g, dim3((unsigned)(Mp / (128 * mt)), N / BN, splits));
    }
    int e = 0;
    if (!rc) {
        cudaError_t ce = cudaStreamSynchronize(tmp.stream);
        if (ce != cudaSuccess) { vp_set_error("gemm: %s", cudaGetErrorString(ce)); rc = VP_E_CUDA; }
        else {
            cudaMemcpy(&e, err, 4, cudaMemcpyDeviceToHost);
            cudaMemcpy(D, dD, (size_t)splits * M * N * 4, cudaMemcpyDeviceToHost);
            if (e) { vp_set_error("gemm pipeline timed out (code %d)", e); rc = VP_E_CUDA; }
        }
    }
    cudaFree(dA); cudaFree(dB0); if (dB1) cudaFree(dB1); cudaFree(dD); cudaFree(err);
    cudaStreamDestroy(tmp.stream);
    tmp.stream = nullptr;
    return rc;
}

// Failure path of the tensor-core pipeline without a fault: one small
// contraction whose stage barriers expect 16 bytes more than their copies
// bring, so every pipeline wait runs out; then the same contraction with the
// right byte counts on the same device, checked against its exact result.
extern "C" int vp_debug_gemm_wait_timeout(int32_t* status_timeout, int32_t* status_after, double* max_err_after) {
    if (!status_timeout || !status_after || !max_err_after) { vp_set_error("null argument"); return VP_E_ARG; }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) { vp_set_error("no CUDA device"); return VP_E_NODEV; }
    constexpr int M = 256, N = 192, K = 256;
    // small integers times multiples of 1/8: every product and sum is exact in FP32
    std::vector<uint16_t> hA((size_t)M * K), hB((size_t)N * K);
    auto bf = [](float v) { uint32_t u; memcpy(&u, &v, 4); return (uint16_t)(u >> 16); };
    std::vector<double> ref((size_t)M * N, 0.0);
    for (int m = 0; m < M; ++m)
        for (int k = 0; k < K; ++k) hA[(size_t)m * K + k] = bf((float)((m * 7 + k * 3) % 3));
    for (int n = 0; n < N; ++n)
        for (int k = 0; k < K; ++k) hB[(size_t)n * K + k] = bf((float)(((n * 5 + k) % 17) - 8) / 8.f);
    for (int m = 0; m < M; ++m)
        for (int n = 0; n < N; ++n) {
            double t = 0;
            for (int k = 0; k < K; ++k) t += (double)((m * 7 + k * 3) % 3) * ((((n * 5 + k) % 17) - 8) / 8.0);
            ref[(size_t)m * N + n] = t;
        }
    vp_ctx tmp;
    CK(cudaStreamCreateWithFlags(&tmp.stream, cudaStreamNonBlocking));
    void *dA = nullptr, *dB = nullptr, *dD = nullptr;
    int* err = nullptr;
    int rc = VP_OK;
    std::vector<float> D((size_t)M * N);
    do {
        if (cudaMalloc(&dA, hA.size() * 2) != cudaSuccess || cudaMalloc(&dB, hB.size() * 2) != cudaSuccess ||
            cudaMalloc(&dD, D.size() * 4) != cudaSuccess || cudaMalloc(&err, 4) != cudaSuccess) {
            vp_set_error("allocation failed");
            rc = VP_E_MEM;
            break;
        }
        cudaMemcpy(dA, hA.data(), hA.size() * 2, cudaMemcpyHostToDevice);
        cudaMemcpy(dB, hB.data(), hB.size() * 2, cudaMemcpyHostToDevice);
        CUtensorMap ma, mb;
        if ((rc = make_map(&ma, dA, M, K, K, 128, 64)) || (rc = make_map(&mb, dB, N, K, K, 192, 64))) break;
        tc::GemmArgs g{};
        g.M = M; g.N = N; g.kblocks = K / 64; g.kb_per_split = g.kblocks;
        g.BN = 192; g.piece = 192; g.nb = 1; g.mt = 2; g.stages = 2; g.bk = 64; g.esz = 2; g.mode = 0;
        g.out_f = (float*)dD; g.ldo = N; g.err = err;
        for (int pass = 0; pass < 2 && !rc; ++pass) {
            g.tx_extra = pass == 0 ? 16 : 0;
            g.spin_limit = pass == 0 ? (1u << 12) : 0;   // short waits for the pass that times out
            cudaMemset(err, 0, 4);
            cudaMemset(dD, 0, D.size() * 4);
            if ((rc = launch_gemm(&tmp, ma, mb, mb, g, dim3(1, 1, 1)))) break;
            const cudaError_t ce = cudaStreamSynchronize(tmp.stream);
            if (ce != cudaSuccess) { vp_set_error("contraction failed: %s", cudaGetErrorString(ce)); rc = VP_E_CUDA; break; }
            int e = 0;
            cudaMemcpy(&e, err, 4, cudaMemcpyDeviceToHost);
            (pass == 0 ? *status_timeout : *status_after) = e;
        }
        if (rc) break;
        cudaMemcpy(D.data(), dD, D.size() * 4, cudaMemcpyDeviceToHost);
        double worst = 0;
        for (size_t j = 0; j < D.size(); ++j) worst = std::max(worst, std::abs((double)D[j] - ref[j]));
        *max_err_after = worst;
    } while (0);
    cudaFree(dA); cudaFree(dB); cudaFree(dD); cudaFree(err);
    cudaStreamDestroy(tmp.stream);
    return rc;
}

extern "C" int vp_debug_gemm_e4m3(const uint8_t* A, const uint8_t* B, int32_t M, int32_t N, int32_t K, int32_t BN,
                                  int32_t piece, int32_t stages, int32_t mt, float* D) {
    if (!A || !B || !D || M <= 0 || N <= 0 || K <= 0 || K % 128 || N % BN || BN % piece || piece % 16 || piece > 256 ||
        (mt != 1 && mt != 2) || BN * mt > 512) {
        vp_set_error("vp_debug_gemm_e4m3: bad shape");
        return VP_E_ARG;
    }
    vp_ctx tmp;
    cudaStreamCreateWithFlags(&tmp.stream, cudaStreamNonBlocking);
    const int64_t Mp = (M + 128 * mt - 1) / (128 * mt) * (128 * mt);
    void *dA = nullptr, *dB = nullptr, *dD = nullptr;
    int* err = nullptr;
    int rc = VP_OK;
    do {
        cudaError_t ce;
        if ((ce = cudaMalloc(&dA, (size_t)Mp * K)) != cudaSuccess || (ce = cudaMalloc(&dB, (size_t)N * K)) != cudaSuccess ||
            (ce = cudaMalloc(&dD, (size_t)M * N * 4)) != cudaSuccess || (ce = cudaMalloc(&err, 4)) != cudaSuccess) {
            vp_set_error("vp_debug_gemm_e4m3: %s", cudaGetErrorString(ce));
            rc = VP_E_MEM;
            break;
        }
        cudaMemset(dA, 0, (size_t)Mp * K);
        cudaMemset(err, 0, 4);
        cudaMemcpy(dA, A, (size_t)M * K, cudaMemcpyHostToDevice);
        cudaMemcpy(dB, B, (size_t)N * K, cudaMemcpyHostToDevice);
        CUtensorMap ma, mb;
        if ((rc = make_map(&ma, dA, Mp, K, K, 128, 128, 1)) || (rc = make_map(&mb, dB, N, K, K, piece, 128, 1))) break;
        tc::GemmArgs g{};
        g.M = M; g.N = N; g.kblocks = K / 128; g.kb_per_split = g.kblocks;
        g.BN = BN; g.piece = piece; g.nb = 1; g.mt = mt; g.stages = stages; g.bk = 128; g.esz = 1; g.mode = 0;
        g.out_f = (float*)dD; g.ldo = N; g.err = err; g.group_major = 1;   // the count contraction's order
        if ((rc = launch_gemm(&tmp, ma, mb, mb, g, dim3(N / BN, (unsigned)(Mp / (128 * mt)), 1)))) break;
        if ((ce = cudaStreamSynchronize(tmp.stream)) != cudaSuccess) {
            vp_set_error("gemm: %s", cudaGetErrorString(ce));
            rc = VP_E_CUDA;
            break;
        }
        int e = 0;
        cudaMemcpy(&e, err, 4, cudaMemcpyDeviceToHost);
        cudaMemcpy(D, dD, (size_t)M * N * 4, cudaMemcpyDeviceToHost);
        if (e) { vp_set_error("gemm pipeline timed out (code %d)", e); rc = VP_E_CUDA; }
    } while (0);
    cudaFree(dA); cudaFree(dB); cudaFree(dD); cudaFree(err);
    cudaStreamDestroy(tmp.stream);
    tmp.stream = nullptr;
    return rc;
}

extern "C" int vp_debug_gemm_time(int32_t M, int32_t N, int32_t K, int32_t BN, int32_t piece, int32_t splits,
                                  int32_t stages, int32_t mt, int32_t bk, int32_t esz, int32_t nb, int32_t mode,
                                  int32_t iters, double* ms) {
    if (!ms || M <= 0 || N <= 0 || K <= 0 || (esz != 1 && esz != 2) || (bk * esz != 64 && bk * esz != 128) || K % bk ||
        N % BN || BN % piece ||
        piece % 16 || piece > 256 || (mt != 1 && mt != 2) || BN * mt > 512 || splits < 1 || (nb != 1 && nb != 2) ||
        (mode != 0 && mode != 1) || (mode == 1 && splits != 1) || iters < 1) {
        vp_set_error("vp_debug_gemm_time: bad shape");
        return VP_E_ARG;
    }
    vp_ctx tmp;
    cudaStreamCreateWithFlags(&tmp.stream, cudaStreamNonBlocking);
    const int64_t Mp = (M + 128 * mt - 1) / (128 * mt) * (128 * mt);
    void *dA = nullptr, *dB = nullptr, *dD = nullptr;
    int* err = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = VP_OK;
    do {
        cudaError_t ce;
        const size_t outb = mode == 0 ? (size_t)splits * M * N * 4 : (size_t)N * M * 4;
        if ((ce = cudaMalloc(&dA, (size_t)Mp * K * esz)) != cudaSuccess ||
            (ce = cudaMalloc(&dB, (size_t)2 * N * K * esz)) != cudaSuccess ||
            (ce = cudaMalloc(&dD, outb)) != cudaSuccess || (ce = cudaMalloc(&err, 4)) != cudaSuccess) {
            vp_set_error("vp_debug_gemm_time: %s", cudaGetErrorString(ce));
            rc = VP_E_MEM;
            break;
        }
        // small values (bf16 0x3C3C ~ 0.0115, e4m3 0x3C = 1.5): the timing does not depend on them
        cudaMemsetAsync(dA, 0x3C, (size_t)Mp * K * esz, tmp.stream);
        cudaMemsetAsync(dB, 0x3C, (size_t)2 * N * K * esz, tmp.stream);
        cudaMemsetAsync(err, 0, 4, tmp.stream);
        CUtensorMap ma, mb0, mb1;
        const char* b1 = (const char*)dB + (size_t)N * K * esz;
        if ((rc = make_map(&ma, dA, Mp, K, K, 128, bk, esz)) || (rc = make_map(&mb0, dB, N, K, K, piece, bk, esz)) ||
            (rc = make_map(&mb1, b1, N, K, K, piece, bk, esz)))
            break;
        tc::GemmArgs g{};
        g.M = M; g.N = N; g.kblocks = K / bk; g.kb_per_split = (g.kblocks + splits - 1) / splits;
        g.BN = BN; g.piece = piece; g.nb = nb; g.mt = mt; g.stages = stages; g.bk = bk; g.esz = esz; g.mode = mode;
        g.out_f = (float*)dD; g.out_i = (int32_t*)dD; g.ldo = mode == 0 ? N : M; g.err = err;
        g.group_major = mode == 1 && Mp / (128 * mt) <= 65535;   // as the count contraction
        const dim3 grid = g.group_major ? dim3(N / BN, (unsigned)(Mp / (128 * mt)), splits)
                                        : dim3((unsigned)(Mp / (128 * mt)), N / BN, splits);
        if ((rc = launch_gemm(&tmp, ma, mb0, mb1, g, grid))) break;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        cudaEventRecord(e0, tmp.stream);
        for (int i = 0; i < iters && !rc; ++i) rc = launch_gemm(&tmp, ma, mb0, mb1, g, grid);
        cudaEventRecord(e1, tmp.stream);
        if (rc) break;
        if ((ce = cudaStreamSynchronize(tmp.stream)) != cudaSuccess) {
            vp_set_error("gemm: %s", cudaGetErrorString(ce));
            rc = VP_E_CUDA;
            break;
        }
        float t = 0;
        cudaEventElapsedTime(&t, e0, e1);
        *ms = t / iters;
        int e = 0;
        cudaMemcpy(&e, err, 4, cudaMemcpyDeviceToHost);
        if (e) { vp_set_error("gemm pipeline timed out (code %d)", e); rc = VP_E_CUDA; }
    } while (0);
    cudaStreamSynchronize(tmp.stream);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(dA); cudaFree(dB); cudaFree(dD); cudaFree(err);
    cudaStreamDestroy(tmp.stream);
    tmp.stream = nullptr;
    return rc;
}

extern "C" void* vp_stream(vp_ctx* x) { return x ? (void*)x->stream : nullptr; }

extern "C" int vp_release_memory(int device) {
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) { vp_set_error("no CUDA device"); return VP_E_NODEV; }
    if (device < 0 || device >= ndev) { vp_set_error("device %d out of range", device); return VP_E_ARG; }
    cudaMemPool_t pool = lib_pool(device);
    if (!pool) { vp_set_error("no memory pool on device %d", device); return VP_E_CUDA; }
    CK(cudaSetDevice(device));
    CK(cudaDeviceSynchronize());
    CK(cudaMemPoolTrimTo(pool, 0));
    return VP_OK;
}

extern "C" int vp_prof_enable(vp_ctx* x, int on) {
    if (!x) { vp_set_error("null context"); return VP_E_ARG; }
    if (on < 0 || on > PROF_UPDATEP_TC) { vp_set_error("profiling mode %d: 0, 1 or 2", on); return VP_E_ARG; }
    if (x->prof == on) return VP_OK;
    x->prof = on;
    // cached graphs were captured with or without the markers: re-capture
    if (x->pg) { cudaGraphExecDestroy(x->pg); x->pg = nullptr; x->pg_chains.clear(); }
    if (x->batch && x->batch->graph) { cudaGraphExecDestroy(x->batch->graph); x->batch->graph = nullptr; }
    return VP_OK;
}

extern "C" int vp_tc_pipeline(vp_ctx* x, int on) {
    if (!x) { vp_set_error("null context"); return VP_E_ARG; }
    if (on < 0 || on > 8) { vp_set_error("pipeline share %d: 0 (one pass) to 8", on); return VP_E_ARG; }
    if (x->tc_pipeline == on) return VP_OK;
    cudaSetDevice(x->device);
    CK(cudaStreamSynchronize(x->stream));
    x->tc_pipeline = on;
    // the cached sweep graph has the other shape: re-capture
    if (x->batch && x->batch->graph) { cudaGraphExecDestroy(x->batch->graph); x->batch->graph = nullptr; }
    return VP_OK;
}

extern "C" int vp_prof_read(vp_ctx* x, double* ms, int32_t* launches) {
    if (!x || !ms || !launches) { vp_set_error("null argument"); return VP_E_ARG; }
    CK(cudaStreamSynchronize(x->stream));
    double t = 0;
    for (int j = 0; j < x->prof_used; ++j) {
        float e = 0;
        CK(cudaEventElapsedTime(&e, x->prof_ev[2 * j], x->prof_ev[2 * j + 1]));
        t += e;
    }
    *ms = t;
    *launches = x->prof_used;
    return VP_OK;
}

// ===================== standalone likelihood call =====================
namespace {

// per-genotype log-probability table of the likelihood stream from the
// frequencies of K clusters over L biallelic loci (freq [K][2L])
__global__ void k_lt_from_freq(const float* freq, int K, int64_t L, int kp, float* lt) {
    int64_t kl = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (kl >= (int64_t)K * L) return;
    const int k = (int)(kl / L);
    const int64_t l = kl % L;
    const float l0 = ln_freq(freq[k * 2 * L + 2 * l]), l1 = ln_freq(freq[k * 2 * L + 2 * l + 1]);
    float* t = lt + l * 4 * kp + k;
    t[0] = l0 + l0;
    t[kp] = l0 + l1;
    t[2 * kp] = l1 + l1;
    t[3 * kp] = 0.f;
}

__global__ void k_ll_reduce(const DevChain* chains, double* ll) {
    const DevChain& c = chains[0];
    const int64_t n = (int64_t)c.D.N * c.K;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
        double v = 0;
        for (int ch = 0; ch < c.nchunk; ++ch) v += c.LLp[(int64_t)ch * n + j];
        ll[j] = v;
    }
}

struct LLPlan {
    DevChain h{};
    size_t scratch = 0;   // bytes: descriptor, table, partials
    int kc = 16, kgroups = 1;
    bool fma = false;
};

int ll_plan(int32_t N, int64_t L, int32_t K, int nsm, LLPlan* pl) {
    if (N <= 0 || L <= 0 || K < 1 || K > 64) { vp_set_error("loglik: bad sizes"); return VP_E_ARG; }
    DevChain& h = pl->h;
    h.D.N = N; h.D.L = L; h.D.KT = 2 * L; h.D.Nw = (N + 15) / 16; h.D.packed2 = 1; h.D.vmax = 2; h.D.maxK = 2;
    h.K = K;
    h.kp = (K + 3) & ~3;
    pl->fma = lf_form(K);
    pl->kc = ll_kc(pl->fma, K);
    pl->kgroups = (K + pl->kc - 1) / pl->kc;
    const int64_t nch = ll_chunks(pl->fma, pl->kc, pl->kgroups, N, L, nsm);
    h.lchunk = (int32_t)((L + nch - 1) / nch);
    h.nchunk = (int32_t)((L + h.lchunk - 1) / h.lchunk);
    Carve cv{nullptr};
    cv.take<DevChain>(1);
    cv.take<float>(L * 4 * h.kp);
    cv.take<double>((int64_t)h.nchunk * N * K);
    pl->scratch = cv.off + 256;
    return VP_OK;
}

// run the likelihood stream with the given scratch (device memory, plan size)
int ll_run(LLPlan& pl, const uint32_t* geno, const float* freq, double* ll, void* scratch, cudaStream_t s) {
    DevChain h = pl.h;
    Carve cv{(char*)(((uintptr_t)scratch + 255) & ~(uintptr_t)255)};
    DevChain* d = cv.take<DevChain>(1);
    h.lt = cv.take<float>(h.D.L * 4 * h.kp);
    h.LLp = cv.take<double>((int64_t)h.nchunk * h.D.N * h.K);
    h.D.g2 = geno;
    // the descriptor travels as the kernel's parameter: no host buffer has
    // to outlive the call
    k_set_chain<<<1, 128, 0, s>>>(d, h);
    k_lt_from_freq<<<cdiv((int64_t)h.K * h.D.L, 256), 256, 0, s>>>(freq, h.K, h.D.L, h.kp, h.lt);
    const dim3 g(cdiv(h.D.N, ll_individuals(pl.fma, pl.kc)), h.nchunk, pl.kgroups);
    if (pl.fma) {
        switch (pl.kc) {
            case 1: k_loglik_fma<1><<<g, LL_BLOCK, 0, s>>>(d, pl.kgroups, 1); break;
            case 2: k_loglik_fma<2><<<g, LL_BLOCK, 0, s>>>(d, pl.kgroups, 1); break;
            case 6: k_loglik_fma<6><<<g, LL_BLOCK, 0, s>>>(d, pl.kgroups, 1); break;
            default: k_loglik_fma<14><<<g, LL_BLOCK, 0, s>>>(d, pl.kgroups, 1); break;
        }
    } else {
        switch (pl.kc) {
            case 4: k_loglik<4><<<g, LT_BLOCK, 0, s>>>(d, pl.kgroups, 1); break;
            case 8: k_loglik<8><<<g, LT_BLOCK, 0, s>>>(d, pl.kgroups, 1); break;
            case 12: k_loglik<12><<<g, LT_BLOCK, 0, s>>>(d, pl.kgroups, 1); break;
            default: k_loglik<16><<<g, LT_BLOCK, 0, s>>>(d, pl.kgroups, 1); break;
        }
    }
    k_ll_reduce<<<std::min<unsigned>(1024, cdiv((int64_t)h.D.N * h.K, 256)), 256, 0, s>>>(d, ll);
    CK(cudaGetLastError());
    return VP_OK;
}

int device_sms() {
    int dev = 0, n = 132;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n;
}

}  // namespace

extern "C" int vp_loglik_packed2(const uint32_t* geno, int32_t n_ind, int64_t n_loc, const float* freq, int32_t K,
                                 double* ll, void* stream) {
    if (!geno || !freq || !ll) { vp_set_error("loglik: null pointer"); return VP_E_ARG; }
    LLPlan pl;
    int rc = ll_plan(n_ind, n_loc, K, device_sms(), &pl);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    void* scratch = nullptr;
    cudaError_t e = cudaMallocAsync(&scratch, pl.scratch, s);
    if (e != cudaSuccess) { vp_set_error("loglik scratch (%zu bytes): %s", pl.scratch, cudaGetErrorString(e)); return VP_E_MEM; }
    rc = ll_run(pl, geno, freq, ll, scratch, s);
    cudaFreeAsync(scratch, s);
    return rc;
}

// ===================== allocation-free likelihood call =====================
// Some callers may not allocate device memory at all: for example a host
// framework that has reserved the whole device budget up front and hands out
// only the buffers it owns, or a plugin whose host forbids allocation on its
// hot path. For them this variant of vp_loglik_packed2 takes its scratch (the
// per-genotype table and the per-chunk partial sums) from one fixed array in
// device memory, compiled into the library, instead of allocating.
//
// The array is VP_LOGLIK_NOALLOC_MAX_BYTES long and is held by every GPU that
// loads the library until the process exits. All calls on a device share it
// and it keeps whatever the previous call left there; every call writes the
// parts it reads before reading them, so nothing has to start at zero. Calls
// whose work overlaps on the GPU (issued on different streams without
// ordering between them) race on the array.
namespace {
#define VP_LOGLIK_NOALLOC_MAX_BYTES (32u << 20)
static __device__ __align__(256) unsigned char g_loglik_scratch[VP_LOGLIK_NOALLOC_MAX_BYTES];

// Device address of the array on each device. Host code cannot use the
// array's name as a device address, so the address is looked up once per
// device with that device current. The cached address belongs to the
// device's primary context: it is not valid after a device reset.
void* g_loglik_scratch_addr[64];
std::mutex g_loglik_scratch_mu;

int loglik_scratch_addr(void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) { vp_set_error("cudaGetDevice: %s", cudaGetErrorString(e)); return VP_E_CUDA; }
    if (dev < 0 || dev >= 64) { vp_set_error("device ordinal %d out of range", dev); return VP_E_ARG; }
    std::lock_guard<std::mutex> lk(g_loglik_scratch_mu);
    if (!g_loglik_scratch_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_loglik_scratch);
        if (e != cudaSuccess) { vp_set_error("cudaGetSymbolAddress: %s", cudaGetErrorString(e)); return VP_E_CUDA; }
        g_loglik_scratch_addr[dev] = p;
    }
    *out = g_loglik_scratch_addr[dev];
    return VP_OK;
}
}  // namespace

extern "C" int vp_loglik_packed2_noalloc(const uint32_t* geno, int32_t n_ind, int64_t n_loc, const float* freq,
                                         int32_t K, double* ll, void* stream) {
    if (!geno || !freq || !ll) { vp_set_error("loglik (no-alloc): null pointer"); return VP_E_ARG; }
    LLPlan pl;
    int rc = ll_plan(n_ind, n_loc, K, device_sms(), &pl);
    if (rc) return rc;
    if (pl.scratch > VP_LOGLIK_NOALLOC_MAX_BYTES) {
        vp_set_error("loglik (no-alloc): N=%d, L=%lld, K=%d needs %zu bytes of scratch; the fixed array holds %u",
                     n_ind, (long long)n_loc, K, pl.scratch, VP_LOGLIK_NOALLOC_MAX_BYTES);
        return VP_E_ARG;
    }
    void* scratch = nullptr;
    if ((rc = loglik_scratch_addr(&scratch))) return rc;
    return ll_run(pl, geno, freq, ll, scratch, (cudaStream_t)stream);
}
