// Kernels of one STRUCTURE sweep. Every kernel takes the chain descriptor from
// device memory (chains[blockIdx.z] for batched launches) and reads the sweep
// index m from the chain's control block, so the kernel sequence of a sweep is
// fixed and can be captured once in a CUDA graph and replayed: steps that do
// not apply at this m (Metropolis vs Gibbs Q, the no-admixture burn-in switch,
// thinning) return early on the device.
#pragma once
#include "vp_device.cuh"

namespace vp {

constexpr int KG = 16;          // clusters per thread in the likelihood kernels
constexpr int LL_BLOCK = 128;   // threads per CTA of the likelihood stream's FMA form
constexpr int LT_BLOCK = 256;   // threads (= individuals) per CTA of its table form
constexpr int SUB = 32;         // loci per FP32 sub-sum before folding into FP64

struct DevData {
    int32_t N, S, vmax, maxploidy, maxK, Nw, packed2;
    int32_t popcontig;    // every population's individuals are consecutive
    int64_t L, KT, coprime;
    const uint32_t* g2;   // [L][Nw]
    const uint8_t* gb;    // [L][N][vmax]
    const int32_t* k;
    const int64_t* off;
    const int64_t* vt;
    const int32_t* popid;
    const int32_t* pop_ind0;
    const int32_t* pop_nind;
    const float* totfreq;
    const int32_t* nhaplo;
    const int32_t* perm;   // [N] individuals in ascending ploidy, or null (one ploidy)
};

struct Ctl {
    int32_t m, nr, nlnl, done;     // done: blocks finished, for last-block reductions
    double r;
    double lnl;           // likelihood of the last sampled labels (no-admixture form)
};

struct DevChain {
    DevData D;
    int32_t K, admix, locpriori, fmodel, nburnin, nreps, nthinning, nadmburnin, writelnl;
    int32_t metrofreq, inferalpha, diffalpha, uniformalpha, fsame, difflambda, rlen, rng, nchunk, lchunk;
    int32_t zadm_tn, nlnlp, kp, nsampblk, zadm_lc;
    int32_t ntrace;       // capacity of lnlTrace in records
    double lambda, alpha, stdalpha, maxalpha, alphapriora, alphapriorb, maxr, epsr, epseta, epsgamma;
    double pmeanf, pstdf, stdf;
    uint64_t seed;
    Ctl* ctl;
    float *Freq, *FreqM, *FreqA, *Q, *Qprop, *Di, *lt, *fbuf;
    uint16_t* Z;
    int32_t *Mi, *Ni;
    int64_t* MiSum;
    double *LLp, *LL, *metro, *metrop, *Alpha, *Lambda, *f, *F, *Eta, *Gamma, *AlphaLocal, *SumAlpha;
    double *rout, *lnlTrace, *red, *lnlp;
    Rng64* rstate;
};

// step ids folded into Philox counters
enum : uint32_t { ST_INITZ = 1, ST_P = 2, ST_Q = 3, ST_METRO_P = 4, ST_METRO_A = 5, ST_A = 7, ST_INITADM = 8,
                  ST_ALPHA = 9, ST_ZSLICE = 10 };

__device__ __forceinline__ bool binaryq_at(const DevChain& c, int m) { return !c.admix && m >= c.nadmburnin; }
__device__ __forceinline__ bool metro_turn(const DevChain& c, int m) { return c.admix && c.metrofreq > 0 && m % c.metrofreq == 0; }
__device__ __forceinline__ bool record_at(const DevChain& c, int m) {
    return (c.writelnl && m < c.nburnin && m % c.nthinning == 0) || (m >= c.nburnin && (m - c.nburnin) % c.nthinning == 0);
}

// The block a kernel of the sweep works on. A launch of one chain (or of a
// tensor-core batch) uses the hardware indices. A cohort launch -- one launch
// of a kernel for the chains of several runs, each with its own dataset --
// passes a map with one entry per block: {the index that blockIdx.z would
// have in the chain's own launch, with the chain's slot in the cohort's
// DevChain array folded in; blockIdx.x and blockIdx.y of that launch; its
// gridDim.x}, so every chain's blocks do exactly the work, in the same
// decomposition and order, that its own launch would (no kernel of the sweep
// reads gridDim.y).
struct VBlock {
    int x, y, z, gx;
};
__device__ __forceinline__ VBlock vblock(const int4* map) {
    if (!map) return VBlock{(int)blockIdx.x, (int)blockIdx.y, (int)blockIdx.z, (int)gridDim.x};
    const int4 t = __ldg(map + blockIdx.x);
    return VBlock{t.y, t.z, t.x, t.w};
}
// a cohort keeps launching for runs whose sweeps are all done; their blocks
// return at once
__device__ __forceinline__ bool run_over(const DevChain& c) { return c.ctl->m >= c.nburnin + c.nreps; }

// ---------------------------------------------------------------------------
// block reductions
template <typename T>
__device__ T block_sum(T v, T* sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    int w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    __syncthreads();
    if ((threadIdx.x & 31) == 0) sh[w] = v;
    __syncthreads();
    T r = 0;
    if (threadIdx.x == 0)
        for (int j = 0; j < nw; ++j) r += sh[j];
    __syncthreads();
    return r;  // valid in thread 0
}

// the sum of n per-block partials by a whole block (thread j adds partials j,
// j + blockDim.x, ..., then one block reduction): the last block of a grid
// uses it instead of one thread walking every partial through a chain of
// dependent loads. Same order on every launch of a grid; valid in thread 0.
__device__ __forceinline__ double block_sum_partials(const double* p, int n, double* sh) {
    double v = 0;
    for (int j = threadIdx.x; j < n; j += blockDim.x) v += p[j];
    return block_sum(v, sh);
}

// ---------------------------------------------------------------------------
// initialisation: InitFix (src/structure.cpp:466-553), InitLocPriori (651-675),
// InitFmodel (677-708)
__global__ void k_init_state(const DevChain* chains) {
    const DevChain& c = chains[blockIdx.z];
    const DevData& D = c.D;
    const int K = c.K;
    int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, nt = (int64_t)gridDim.x * blockDim.x;
    for (int64_t l = tid; l < D.L; l += nt) {
        int k2 = D.k[l];
        float v = k2 == 2 ? 0.5f : (float)(1.0 / k2);
        // the chain's memory was zeroed when it was allocated: FreqM, Ni,
        // Mi, MiSum and Z start at zero without a store here
        for (int k = 0; k < K; ++k)
            for (int a = 0; a < k2; ++a) c.Freq[k * D.KT + D.off[l] + a] = c.fmodel ? (float)c.lambda : v;
        if (c.fmodel) {
            // the total-population frequencies are laid out in pre-sort order but
            // read with this (sorted) locus' offset and index, as in the reference
            const float* p2 = D.totfreq + D.off[l];
            int nh = D.nhaplo[l];
            for (int a = 0; a < k2; ++a)
                c.FreqA[D.off[l] + a] = (float)((c.lambda + p2[a] * nh) / (k2 * c.lambda + nh));
        }
    }
    for (int64_t j = tid; j < (int64_t)D.N * K; j += nt) c.Q[j] = (float)(1.0 / K);
    if (tid < K) {
        c.Alpha[tid] = c.alpha;
        c.Lambda[tid] = c.lambda;
        if (c.fmodel) { c.F[tid] = c.pmeanf; c.f[tid] = (1 - c.pmeanf) / c.pmeanf; }
        if (c.locpriori && !c.admix) c.Eta[tid] = (double)(1.0 / K);
    }
    if (c.locpriori)
        for (int64_t j = tid; j < (int64_t)D.S * K; j += nt) {
            c.AlphaLocal[j] = c.alpha;
            if (!c.admix) { c.Gamma[j] = (double)(1.0 / K); c.Di[j] = 0.f; }
        }
    if (c.locpriori)
        for (int64_t s = tid; s < D.S; s += nt) c.SumAlpha[s] = 0;
    for (int64_t j = tid; j < c.rlen; j += nt) c.rout[j] = 0;
    if (tid == 0) { c.ctl->m = 0; c.ctl->nr = 0; c.ctl->nlnl = 0; c.ctl->done = 0; c.ctl->r = 1; c.ctl->lnl = 0; }
}

// InitAdmix, single-label form (no admixture, no admixture burn-in):
// Z_i ~ U{0..K-1} from RNG(seed-1, SALT_INITADM), Mi[i, Z_i] = vt_i
// (src/structure.cpp:564-573)
__global__ void k_init_z_single(const DevChain* chains) {
    const DevChain& c = chains[blockIdx.z];
    const int K = c.K, N = c.D.N;
    if (c.rng == 0) {
        if (blockIdx.x || threadIdx.x) return;
        Rng64 r; r.init(c.seed - 1, VP_SALT_INITADM);
        for (int i = 0; i < N; ++i) {
            int z = (int)r.nextn(K);
            c.Z[i] = (uint16_t)z;
            c.Mi[i * K + z] = (int32_t)c.D.vt[i];
        }
    } else {
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
            Philox p; p.init(c.seed, ST_INITZ, (uint32_t)i, 0);
            int z = (int)(p.next() % (uint32_t)K);
            c.Z[i] = (uint16_t)z;
            c.Mi[i * K + z] = (int32_t)c.D.vt[i];
        }
    }
}

// ---------------------------------------------------------------------------
// genotype access
struct Copies {
    int n;
    uint8_t a[10];
};
__device__ __forceinline__ void load_copies(const DevData& D, int64_t l, int i, Copies& cp) {
    if (D.packed2) {
        int code = (D.g2[l * D.Nw + (i >> 4)] >> ((i & 15) * 2)) & 3;
        if (code == 3) { cp.n = 0; return; }
        cp.n = 2;
        cp.a[0] = code == 2 ? 1 : 0;
        cp.a[1] = code == 0 ? 0 : 1;
        return;
    }
    const uint8_t* g = D.gb + ((size_t)l * D.N + i) * D.vmax;
    int n = 0;
    if (g[0] != 0xFF)
        for (; n < D.vmax && g[n] != 0xFF; ++n) cp.a[n] = g[n];
    cp.n = n;
}

// InitAdmix, per-copy form: per locus RNG(seed + l, SALT_INITADM), one draw per
// typed copy (src/structure.cpp:617-645)
__global__ void k_init_admix(const DevChain* chains) {
    const DevChain& c = chains[blockIdx.z];
    const DevData& D = c.D;
    const int K = c.K;
    int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (l >= D.L) return;
    Rng64 r;
    if (c.rng == 0) r.init(c.seed + l, VP_SALT_INITADM);
    int64_t o = D.off[l];
    for (int i = 0; i < D.N; ++i) {
        Copies cp;
        load_copies(D, l, i, cp);
        if (!cp.n) continue;
        Philox ph;
        if (c.rng) ph.init(c.seed, ST_INITADM, (uint32_t)l, (uint32_t)i);
        for (int a = 0; a < cp.n; ++a) {
            int k2 = c.rng == 0 ? (int)r.nextn(K) : (int)(ph.next() % (uint32_t)K);
            atomicAdd(&c.Mi[i * K + k2], 1);
            atomicAdd(&c.Ni[k2 * D.KT + o + cp.a[a]], 1);
        }
    }
}

// ---------------------------------------------------------------------------
// UpdateP (src/structure.cpp:810-862): p_{k,l,.} ~ Dirichlet(prior + Ni).
// Also writes the lookup table the likelihood kernels read:
//   packed2: lt[(l*K + k)*4 + code] = code's log-probability (code 3 -> 0)
//   general: lt[k*KT + off_l + a]   = ln p
__device__ __forceinline__ float prior_of(const DevChain& c, int k, int64_t j) {
    if (!c.fmodel) return (float)c.Lambda[k];
    return c.FreqA[j] * (float)c.f[c.fsame ? 0 : k];
}
__device__ __forceinline__ void write_lt(const DevChain& c, int k, int64_t l, const float* p, int k2) {
    const DevData& D = c.D;
    if (D.packed2) {
        float l0 = ln_freq(p[0]), l1 = ln_freq(p[1]);
        float* t = c.lt + l * 4 * c.kp + k;
        t[0] = l0 + l0;
        t[c.kp] = l0 + l1;
        t[2 * c.kp] = l1 + l1;
        t[3 * c.kp] = 0.f;
    } else {
        for (int a = 0; a < k2; ++a) c.lt[k * D.KT + D.off[l] + a] = ln_freq(p[a]);
    }
}

// rebuild the lookup table from Freq (after a host-side state import)
__global__ void k_refresh_lt(const DevChain* chains) {
    const DevChain& c = chains[blockIdx.z];
    const DevData& D = c.D;
    int64_t kl = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (kl >= (int64_t)c.K * D.L) return;
    int k = (int)(kl / D.L);
    int64_t l = kl % D.L;
    write_lt(c, k, l, c.Freq + k * D.KT + D.off[l], D.k[l]);
}

// reference streams: 128 block streams RNG(seed + m*128 + b, SALT_UPDATEP),
// each serial over its share of the K*L range
__global__ void k_update_p_ref(const DevChain* chains, const int4* map = nullptr) {
    const VBlock vb = vblock(map);
    const DevChain& c = chains[vb.z];
    if (map && run_over(c)) return;
    const DevData& D = c.D;
    const int K = c.K, m = c.ctl->m;
    int b = threadIdx.x;
    if (b >= 128) return;
    int64_t kl0 = (int64_t)(b * K) * D.L / 128, kl1 = (int64_t)((b + 1) * K) * D.L / 128;
    Rng64 r;
    r.init(c.seed + (uint64_t)(m * 128 + b), VP_SALT_UPDATEP);
    float p[64];
    for (int64_t kl = kl0; kl < kl1; ++kl) {
        int k = (int)(kl / D.L);
        int64_t l = kl % D.L;
        int k2 = D.k[l];
        int64_t j = k * D.KT + D.off[l];
        double s = 0;
        for (int a = 0; a < k2; ++a) {
            double v = r.gamma((double)prior_of(c, k, D.off[l] + a) + (double)c.Ni[j + a]);
            p[a] = (float)v;
            s += v;
        }
        float inv = (float)(1.0 / s);
        for (int a = 0; a < k2; ++a) { p[a] *= inv; c.Freq[j + a] = p[a]; }
        write_lt(c, k, l, p, k2);
    }
}

// counter streams: one thread per (k, l)
__global__ void k_update_p_ctr(const DevChain* chains, const int4* map = nullptr) {
    const VBlock vb = vblock(map);
    const DevChain& c = chains[vb.z];
    if (map && run_over(c)) return;
    const DevData& D = c.D;
    const int K = c.K, m = c.ctl->m;
    int64_t kl = vb.x * (int64_t)blockDim.x + threadIdx.x;
    if (kl >= (int64_t)K * D.L) return;
    int k = (int)(kl / D.L);
    int64_t l = kl % D.L;
    int k2 = D.k[l];
    int64_t j = k * D.KT + D.off[l];
    Philox ph;
    ph.init(c.seed, ST_P | ((uint32_t)m << 4), (uint32_t)kl, (uint32_t)(kl >> 32));
    float p[64];
    if (k2 == 2) {
        // the same draws as the batched tensor-core UpdateP
        ph.dirichlet2(prior_of(c, k, D.off[l]) + (float)c.Ni[j], prior_of(c, k, D.off[l] + 1) + (float)c.Ni[j + 1], p[0],
                      p[1]);
    } else {
        float s = 0;
        for (int a = 0; a < k2; ++a) {
            float v = ph.gammaf(prior_of(c, k, D.off[l] + a) + (float)c.Ni[j + a]);
            p[a] = v;
            s += v;
        }
        const float inv = 1.f / s;
        for (int a = 0; a < k2; ++a) p[a] *= inv;
    }
    for (int a = 0; a < k2; ++a) c.Freq[j + a] = p[a];
    write_lt(c, k, l, p, k2);
}

// ---------------------------------------------------------------------------
// Log-likelihood of every individual under every cluster (the locus loop of
// UpdateQNoAdmix, src/structure.cpp:902-932): LL[i,k] = sum over loci and
// copies of ln p_{k,l,allele}. One thread per individual, 256 per CTA; grid.y
// splits the loci into chunks whose FP64 partials are summed in a fixed order
// by the sampling kernel. Biallelic diploid data: each 32-locus slice of the
// per-genotype log-probability table is staged in shared memory and folded
// into a table per locus pair (16 code pairs: the sum of the two loci's
// entries, rows placed by ll_pair_mul), so one 16-byte shared load and four
// adds serve two loci and four clusters; the slice's genotype words are staged transposed, so a thread
// takes the codes of four loci with one 16-byte load. FP32 sums over a slice
// are folded into Kahan-compensated FP32 totals (FP64 adds are slow on this
// part), converted to FP64 once per chunk.
// asynchronous global -> shared copies (cp.async); with ok false nothing is
// read and the destination is zero-filled
__device__ __forceinline__ void cp_async16(void* dst, const void* src, bool ok) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(d), "l"(src), "r"(ok ? 16 : 0) : "memory");
}
__device__ __forceinline__ void cp_async4(void* dst, const void* src, bool ok) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(d), "l"(src), "r"(ok ? 4 : 0) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

constexpr int LL_SL = 32;
template <int KC>
__device__ __forceinline__ void kahan_fold(float* acc, float* s, float* cmp) {
#pragma unroll
    for (int k = 0; k < KC; ++k) {
        float y = acc[k] - cmp[k];
        float t = s[k] + y;
        cmp[k] = (t - s[k]) - y;
        s[k] = t;
        acc[k] = 0.f;
    }
}
// row stride (floats) of the staged tables: 16-byte chunks in an odd count,
// so rows that differ by fewer than 8 land on different banks
template <int KC>
__host__ __device__ constexpr int ll_stride() { return (KC / 4) % 2 ? KC : KC + 4; }
// Row of code pair (a, b) in a locus pair's table: a + PB b. With PB = 11 the
// eight pairs without a missing code and other than (2, 2), the common ones,
// sit in eight different bank groups (each row an odd number of 16-byte
// chunks), so a quarter warp's gathers conflict only on rare pairs; the table
// spans 37 rows instead of 16, which static shared memory holds up to 12
// columns (16 columns keep a + 4b).
template <int KC>
__host__ __device__ constexpr int ll_pair_mul() { return KC <= 12 ? 11 : 4; }
template <int KC>
__host__ __device__ constexpr int ll_pair_rows() { return 3 + 3 * ll_pair_mul<KC>() + 1; }
template <int KC>
__global__ void __launch_bounds__(LT_BLOCK, 3) k_loglik(const DevChain* chains, int kgroups, int force, const int4* map = nullptr) {
    constexpr int TS = ll_stride<KC>();
    constexpr int GW = LT_BLOCK / 16;          // genotype words per CTA and locus
    constexpr int GS = LL_SL + 4;              // padded row of the transposed words
    __shared__ __align__(16) float sT[2][LL_SL][4][TS];       // two slices in flight
    constexpr int PB = ll_pair_mul<KC>();
    __shared__ __align__(16) float sP[LL_SL / 2][ll_pair_rows<KC>()][TS];
    __shared__ __align__(16) uint32_t sG[2][GW][GS];
    const VBlock vb = vblock(map);
    const DevChain& c = chains[vb.z / kgroups];
    if (map && run_over(c)) return;
    const int kg0 = (vb.z % kgroups) * KC;
    const DevData& D = c.D;
    const int K = c.K;
    if (!force && !binaryq_at(c, c.ctl->m)) return;
    const int i0 = vb.x * LT_BLOCK;
    const int i = i0 + threadIdx.x;
    const int64_t l0 = (int64_t)vb.y * c.lchunk;
    const int64_t l1 = min(D.L, l0 + c.lchunk);
    if (l0 >= D.L) return;
    float acc[KC], s[KC], cmp[KC];
#pragma unroll
    for (int k = 0; k < KC; ++k) { acc[k] = 0.f; s[k] = 0.f; cmp[k] = 0.f; }
    const bool live = i < D.N;
    if (D.packed2) {
        const int w0 = i0 >> 4;
        const int wsel = threadIdx.x >> 4, sh = (threadIdx.x & 15) * 2;
        // Each slice's table rows (16-byte chunks) and genotype words are
        // copied to shared memory asynchronously (cp.async) one slice ahead, so
        // their global latency is covered by the pair-table build and the adds
        // of the slice before. Rows and words past the chunk or the data are
        // zero-filled: a zero row adds nothing, whatever the code.
        constexpr int Q4 = KC / 4;                          // 16-byte chunks per table row
        auto issue = [&](int64_t ls, int buf) {
            const int nl = (int)min((int64_t)LL_SL, l1 - ls);
            for (int j = threadIdx.x; j < LL_SL * 4 * Q4; j += LT_BLOCK) {
                const int q = j % Q4, row = j / Q4;
                const bool ok = (row >> 2) < nl && kg0 + 4 * q < c.kp;
                const float* src = ok ? c.lt + ((ls << 2) + row) * c.kp + kg0 + 4 * q : c.lt;
                cp_async16(&sT[buf][row >> 2][row & 3][4 * q], src, ok);
            }
            for (int j = threadIdx.x; j < LL_SL * GW; j += LT_BLOCK) {
                const int ll = j % LL_SL, w = j / LL_SL;
                const bool ok = ll < nl && w0 + w < D.Nw;
                cp_async4(&sG[buf][w][ll], ok ? D.g2 + (ls + ll) * D.Nw + w0 + w : D.g2, ok);
            }
            cp_async_commit();
        };
        issue(l0, 0);
        int buf = 0;
        for (int64_t ls = l0; ls < l1; ls += LL_SL, buf ^= 1) {
            if (ls + LL_SL < l1) {
                issue(ls + LL_SL, buf ^ 1);
                cp_async_wait<1>();
            } else {
                cp_async_wait<0>();
            }
            __syncthreads();
            // pair rows: sP[p][a + PB b] = sT[2p][a] + sT[2p + 1][b]
            for (int j = threadIdx.x; j < (LL_SL / 2) * 16 * Q4; j += LT_BLOCK) {
                const int q = j % Q4, cp = (j / Q4) & 15, p = j / (16 * Q4);
                const float4 x = *reinterpret_cast<const float4*>(&sT[buf][2 * p][cp & 3][4 * q]);
                const float4 y = *reinterpret_cast<const float4*>(&sT[buf][2 * p + 1][cp >> 2][4 * q]);
                *reinterpret_cast<float4*>(&sP[p][(cp & 3) + PB * (cp >> 2)][4 * q]) =
                    make_float4(x.x + y.x, x.y + y.y, x.z + y.z, x.w + y.w);
            }
            __syncthreads();
            const uint4* gw = reinterpret_cast<const uint4*>(&sG[buf][wsel][0]);
#pragma unroll 2
            for (int q = 0; q < LL_SL / 4; ++q) {
                const uint4 g = gw[q];
                const int ca = ((g.x >> sh) & 3) + PB * ((g.y >> sh) & 3);
                const int cb = ((g.z >> sh) & 3) + PB * ((g.w >> sh) & 3);
                const float4* ta = reinterpret_cast<const float4*>(&sP[2 * q][ca][0]);
                const float4* tb = reinterpret_cast<const float4*>(&sP[2 * q + 1][cb][0]);
#pragma unroll
                for (int r = 0; r < KC / 4; ++r) {
                    const float4 va = ta[r], vb = tb[r];
                    acc[4 * r] += va.x; acc[4 * r + 1] += va.y; acc[4 * r + 2] += va.z; acc[4 * r + 3] += va.w;
                    acc[4 * r] += vb.x; acc[4 * r + 1] += vb.y; acc[4 * r + 2] += vb.z; acc[4 * r + 3] += vb.w;
                }
            }
            kahan_fold<KC>(acc, s, cmp);
            __syncthreads();   // sP and this buffer are rewritten next
        }
    } else {
        int cnt = 0;
        for (int64_t l = l0; l < l1; ++l) {
            Copies cp;
            if (live) load_copies(D, l, i, cp); else cp.n = 0;
            const float* t = c.lt + D.off[l];
            for (int a = 0; a < cp.n; ++a) {
#pragma unroll
                for (int k = 0; k < KC; ++k)
                    if (kg0 + k < K) acc[k] += __ldg(t + (int64_t)(kg0 + k) * D.KT + cp.a[a]);
            }
            if (++cnt == SUB) { cnt = 0; kahan_fold<KC>(acc, s, cmp); }
        }
        kahan_fold<KC>(acc, s, cmp);
    }
    if (!live) return;
    double* out = c.LLp + ((int64_t)vb.y * D.N + i) * K;
#pragma unroll
    for (int k = 0; k < KC; ++k)
        if (kg0 + k < K) out[kg0 + k] = (double)s[k] - (double)cmp[k];
}

// Likelihood stream for 2-bit biallelic diploid data as two FP32 FMAs per
// (individual, locus, cluster). The table's rows are T0 = 2 ln p0, T1 = ln p0 +
// ln p1, T2 = 2 ln p1 and 0 for a missing call, so a call of c copies adds
// typed * (a + c * b) with a = T0 and b = (T2 - T0) / 2 (the halving is
// exact). Each thread holds M individuals of one genotype word and KC
// clusters. A call's decode takes one logic op and two FMA-pipe ops: its two
// code bits, masked in place into the mantissa of 2^23, give c exactly after
// one FMA that rescales by 2^-2j and subtracts 2^(23-2j), and typed =
// saturate(3 - c) (the missing code 3 gives typed 0, so the finite a + 3b it
// meets adds nothing). The decode serves 2 KC FMAs; the slice's (a, b) pairs
// are shared-memory broadcasts. The slice's table rows and genotype
// words are copied to shared memory by cp.async one slice ahead. Sums over 32
// loci are folded into Kahan-compensated FP32 totals, converted to FP64 once
// per chunk, as in the table form.
template <int KC>
struct LfShape {
    static constexpr int M = KC <= 2 ? 16 : KC <= 6 ? 4 : 2;                 // individuals per thread
    static constexpr int SL = M >= 8 ? 32 : 64;                               // loci per staged slice
    static constexpr int GW = LL_BLOCK * M / 16;                              // genotype words per CTA and locus
    static constexpr int KQ = (KC + 3) / 4;                                   // 16-byte chunks of a staged row
};
// The FMA form runs where it measured ahead of the table form (N = 10,000
// over 58,027 loci, ms, FMA form / table form with 256-individual CTAs and
// the spread pair rows): K = 1 0.24 / 0.34, K = 2 0.32 / 0.33, K = 5, 6
// 0.49 / 0.52, K = 13, 14 0.98 / 1.00. The table form takes the rest: K = 3,
// 4, 7, 8 in 0.33 and 0.52 (the FMA form's 4- and 8-column kernels took 0.40
// and 0.65), K = 9..12 in 0.67 (its 10-column kernel 0.74), K = 15, 16 and
// K > 16. Its columns: K itself for K <= 2, else 6 or 14.
__host__ __device__ constexpr bool lf_form(int K) { return K <= 2 || K == 5 || K == 6 || K == 13 || K == 14; }
__host__ __device__ constexpr int lf_kc(int K) { return K <= 2 ? K : K <= 6 ? 6 : 14; }
__host__ __device__ constexpr int lf_individuals(int kc) { return LL_BLOCK * (kc <= 2 ? 16 : kc <= 6 ? 4 : 2); }
template <int KC>
__global__ void __launch_bounds__(LL_BLOCK) k_loglik_fma(const DevChain* chains, int kgroups, int force,
                                                         const int4* map = nullptr) {
    using S = LfShape<KC>;
    constexpr int M = S::M, SL = S::SL, GW = S::GW, KQ = S::KQ, GS = SL + 4;
    __shared__ __align__(16) float sT[2][SL][2][4 * KQ];   // rows T0 and T2 of the slice's loci
    __shared__ __align__(16) float2 sAB[SL][KC];            // (a, b)
    __shared__ __align__(16) uint32_t sG[2][GW][GS];        // genotype words, transposed
    const VBlock vb = vblock(map);
    const DevChain& c = chains[vb.z / kgroups];
    if (map && run_over(c)) return;
    const int kg0 = (vb.z % kgroups) * KC;
    const DevData& D = c.D;
    const int K = c.K;
    if (!force && !binaryq_at(c, c.ctl->m)) return;
    const int64_t l0 = (int64_t)vb.y * c.lchunk;
    const int64_t l1 = min(D.L, l0 + c.lchunk);
    if (l0 >= D.L) return;
    const int i0 = vb.x * LL_BLOCK * M;
    const int ib = i0 + threadIdx.x * M;
    const int w0 = i0 >> 4;
    const int wsel = (threadIdx.x * M) >> 4, sh = (ib & 15) * 2;
    float acc[M * KC], s[M * KC], cmp[M * KC];
#pragma unroll
    for (int j = 0; j < M * KC; ++j) { acc[j] = 0.f; s[j] = 0.f; cmp[j] = 0.f; }
    // rows and words past the chunk or the data are zero-filled; table columns
    // past kp are never read (their clusters' sums are not written)
    auto issue = [&](int64_t ls, int buf) {
        const int nl = (int)min((int64_t)SL, l1 - ls);
        for (int j = threadIdx.x; j < SL * 2 * KQ; j += LL_BLOCK) {
            const int q = j % KQ, r = (j / KQ) & 1, ll = j / (2 * KQ);
            const bool ok = ll < nl && kg0 + 4 * q < c.kp;
            const float* src = ok ? c.lt + (((ls + ll) << 2) + 2 * r) * c.kp + kg0 + 4 * q : c.lt;
            cp_async16(&sT[buf][ll][r][4 * q], src, ok);
        }
        for (int j = threadIdx.x; j < SL * GW; j += LL_BLOCK) {
            const int w = j % GW, ll = j / GW;
            const bool ok = ll < nl && w0 + w < D.Nw;
            cp_async4(&sG[buf][w][ll], ok ? D.g2 + (ls + ll) * D.Nw + w0 + w : D.g2, ok);
        }
        cp_async_commit();
    };
    issue(l0, 0);
    int buf = 0;
    for (int64_t ls = l0; ls < l1; ls += SL, buf ^= 1) {
        if (ls + SL < l1) {
            issue(ls + SL, buf ^ 1);
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncthreads();
        for (int j = threadIdx.x; j < SL * KC; j += LL_BLOCK) {
            const int k = j % KC, ll = j / KC;
            const float t0 = sT[buf][ll][0][k], t2 = sT[buf][ll][1][k];
            sAB[ll][k] = make_float2(t0, 0.5f * (t2 - t0));
        }
        __syncthreads();
        const uint32_t* gw = &sG[buf][wsel][0];
        // one locus a step, two in flight: the (a, b) registers of two loci
        // stay live, not of four
#pragma unroll 2
        for (int ll = 0; ll < SL; ++ll) {
            const uint32_t wd = gw[ll];
            float a[KC], b[KC];
            if constexpr (KC == 1) {
                const float2 v = sAB[ll][0];
                a[0] = v.x; b[0] = v.y;
            } else {
                const float4* ab = reinterpret_cast<const float4*>(&sAB[ll][0]);
#pragma unroll
                for (int k = 0; k < KC / 2; ++k) {
                    const float4 v = ab[k];
                    a[2 * k] = v.x; b[2 * k] = v.y; a[2 * k + 1] = v.z; b[2 * k + 1] = v.w;
                }
            }
            // this thread's codes from bit 0 (M = 16: individuals 8..15 from
            // the upper half word)
            const uint32_t ws = wd >> sh, wh = ws >> 16;
#pragma unroll
            for (int j = 0; j < M; ++j) {
                const int jj = j & 7;
                const uint32_t src = j < 8 ? ws : wh;
                const float x = __uint_as_float((src & (3u << (2 * jj))) | 0x4B000000u);
                const float gf = fmaf(x, 1.0f / (float)(1u << (2 * jj)), -(float)(1u << (23 - 2 * jj)));
                float tf;   // saturate(3 - c), the clamp folded into the subtraction
                asm("sub.sat.f32 %0, 0f40400000, %1;" : "=f"(tf) : "f"(gf));
#pragma unroll
                for (int k = 0; k < KC; ++k)
                    acc[j * KC + k] = fmaf(tf, fmaf(gf, b[k], a[k]), acc[j * KC + k]);
            }
            if ((ll & 31) == 31) kahan_fold<M * KC>(acc, s, cmp);
        }
        __syncthreads();   // sAB and this buffer are rewritten next
    }
    kahan_fold<M * KC>(acc, s, cmp);
#pragma unroll
    for (int j = 0; j < M; ++j) {
        const int i = ib + j;
        if (i >= D.N) break;
        double* out = c.LLp + ((int64_t)vb.y * D.N + i) * K;
#pragma unroll
        for (int k = 0; k < KC; ++k)
            if (kg0 + k < K) out[kg0 + k] = (double)s[j * KC + k] - (double)cmp[j * KC + k];
    }
}

// PolyLog (src/statistics.cpp:116-155): draw k with probability proportional
// to exp(LL_k - max); overwrites ll with the weights.
__device__ __forceinline__ int polylog(double* ll, int K, double u01, bool ref, Rng64* r) {
    double mx = -1.79769313486231570e+308, s = VP_MIN_FREQ * K;
    for (int k = 0; k < K; ++k) if (!(ll[k] < mx)) mx = ll[k];
    for (int k = 0; k < K; ++k) {
        double d = ll[k] - mx;
        ll[k] = d < -23 ? VP_MIN_FREQ : exp(d);
        s += ll[k];
    }
    double t = ref ? r->uniform(0, s) : u01 * s;
    for (int k = 0; k < K; ++k) {
        if (t < ll[k]) return k;
        t -= ll[k];
    }
    return K - 1;
}

// UpdateQNoAdmix label draw (src/structure.cpp:891-900) plus the state the
// reference rebuilds afterwards: Q one-hot, Mi[i, Z_i] = vt_i
// (src/structure.cpp:1305-1310), Di for the location prior (1151-1158) and the
// likelihood of the new labels, sum_i LL[i, Z_i], which is exactly what Record
// computes for a no-admixture sweep (src/structure.cpp:1902-1938).
// Reference streams are serial over individuals (one thread walks them all);
// counter streams use one thread per individual, and the last block to finish
// reduces the per-block likelihoods in a fixed order and rebuilds Di.
constexpr int SAMPLE_BLOCK = 256;
__device__ __forceinline__ bool last_block_done(Ctl* ctl, int nblocks) {
    __shared__ int is_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) is_last = atomicAdd(&ctl->done, 1) == nblocks - 1;
    __syncthreads();
    if (is_last) __threadfence();
    return is_last;
}
__device__ void sample_one(const DevChain& c, int i, int m, bool ref, Rng64* r, double* lnl) {
    const DevData& D = c.D;
    const int K = c.K, N = D.N;
    double ll[64];
    for (int k = 0; k < K; ++k) ll[k] = 0;
    for (int ch = 0; ch < c.nchunk; ++ch) {
        const double* p = c.LLp + ((int64_t)ch * N + i) * K;
        for (int k = 0; k < K; ++k) ll[k] += p[k];
    }
    for (int k = 0; k < K; ++k) c.LL[(int64_t)i * K + k] = ll[k];
    for (int k = 0; k < K; ++k) { c.Q[(int64_t)i * K + k] = 0.f; c.Mi[(int64_t)i * K + k] = 0; }
    if (D.vt[i] == 0) return;
    if (c.locpriori) {
        const double* g = c.Gamma + D.popid[i] * K;
        for (int k = 0; k < K; ++k) ll[k] += log(g[k]);
    }
    double u = 0;
    if (!ref) { Philox ph; ph.init(c.seed, ST_Q | ((uint32_t)m << 4), (uint32_t)i, 0); u = ph.uniformd(); }
    double keep[64];
    for (int k = 0; k < K; ++k) keep[k] = c.LL[(int64_t)i * K + k];
    int z = polylog(ll, K, u, ref, r);
    c.Q[(int64_t)i * K + z] = 1.f;
    c.Z[i] = (uint16_t)z;
    c.Mi[(int64_t)i * K + z] = (int32_t)D.vt[i];
    *lnl += keep[z];
}
// counter streams: one warp per individual. Lane k holds cluster k (and
// k + 32): it sums the chunk partials of its clusters in FP64, and the
// maximum (FP64), the normaliser and the categorical search (the first
// cluster whose cumulative weight exceeds the uniform) are warp reductions,
// a prefix scan and a ballot, the weights exp(LL_k - max) and the search in
// FP32. The counter-stream draw is not matched to the reference's stream.
// Returns, in every lane, LL[i, z] of the drawn label.
__device__ double sample_warp(const DevChain& c, int i, int m, int lane) {
    const DevData& D = c.D;
    const int K = c.K, N = D.N;
    const int k0 = lane, k1 = lane + 32;
    const bool h0 = k0 < K, h1 = k1 < K;
    double v0 = 0, v1 = 0;
    // unrolled so that the partials' loads are in flight together; the adds
    // keep chunk order
#pragma unroll 8
    for (int ch = 0; ch < c.nchunk; ++ch) {
        const double* p = c.LLp + ((int64_t)ch * N + i) * K;
        if (h0) v0 += p[k0];
        if (h1) v1 += p[k1];
    }
    double* LL = c.LL + (int64_t)i * K;
    float* Q = c.Q + (int64_t)i * K;
    int32_t* Mi = c.Mi + (int64_t)i * K;
    if (h0) LL[k0] = v0;
    if (h1) LL[k1] = v1;
    const int vt = (int)D.vt[i];
    if (vt == 0) {
        if (h0) { Q[k0] = 0.f; Mi[k0] = 0; }
        if (h1) { Q[k1] = 0.f; Mi[k1] = 0; }
        return 0;
    }
    double w0 = v0, w1 = v1;
    if (c.locpriori) {
        const double* g = c.Gamma + D.popid[i] * K;
        if (h0) w0 += log(g[k0]);
        if (h1) w1 += log(g[k1]);
    }
    // the maximum in FP64; the weights exp(LL_k - max), their prefix sums and
    // the draw in FP32 (FP64 arithmetic is slow on this part)
    double mx = fmax(h0 ? w0 : -1.79769313486231570e+308, h1 ? w1 : -1.79769313486231570e+308);
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    const float d0 = (float)(w0 - mx), d1 = (float)(w1 - mx);
    const float e0 = h0 ? (d0 < -23.f ? (float)VP_MIN_FREQ : __expf(d0)) : 0.f;
    const float e1 = h1 ? (d1 < -23.f ? (float)VP_MIN_FREQ : __expf(d1)) : 0.f;
    // inclusive prefix sums of the weights in cluster order
    float c0 = e0, c1 = e1;
    for (int o = 1; o < 32; o <<= 1) {
        const float a0 = __shfl_up_sync(0xffffffffu, c0, o), a1 = __shfl_up_sync(0xffffffffu, c1, o);
        if (lane >= o) { c0 += a0; c1 += a1; }
    }
    const float tot0 = __shfl_sync(0xffffffffu, c0, 31);
    c1 += tot0;
    const float s = __shfl_sync(0xffffffffu, c1, 31) + (float)(VP_MIN_FREQ * K);
    float u = 0.f;
    if (lane == 0) { Philox ph; ph.init(c.seed, ST_Q | ((uint32_t)m << 4), (uint32_t)i, 0); u = ph.uniformf(); }
    const float t = __shfl_sync(0xffffffffu, u, 0) * s;
    int z = K - 1;
    const unsigned b0 = __ballot_sync(0xffffffffu, h0 && t < c0);
    const unsigned b1 = __ballot_sync(0xffffffffu, h1 && t < c1);
    if (b0) z = __ffs(b0) - 1;
    else if (b1) z = 32 + __ffs(b1) - 1;
    if (h0) { Q[k0] = k0 == z ? 1.f : 0.f; Mi[k0] = k0 == z ? vt : 0; }
    if (h1) { Q[k1] = k1 == z ? 1.f : 0.f; Mi[k1] = k1 == z ? vt : 0; }
    if (lane == 0) c.Z[i] = (uint16_t)z;
    return __shfl_sync(0xffffffffu, z < 32 ? v0 : v1, z & 31);
}

__global__ void __launch_bounds__(SAMPLE_BLOCK) k_sample_noadmix(const DevChain* chains, int force, const int4* map = nullptr) {
    const VBlock vb = vblock(map);
    const DevChain& c = chains[vb.z];
    if (map && run_over(c)) return;
    const DevData& D = c.D;
    const int K = c.K, N = D.N, m = c.ctl->m;
    if (!force && !binaryq_at(c, m)) return;
    __shared__ double sh[32];
    const bool ref = c.rng == 0;
    if (force) {
        // likelihood only (parity tests): sum the chunk partials
        for (int i = vb.x * blockDim.x + threadIdx.x; i < N; i += vb.gx * blockDim.x)
            for (int k = 0; k < K; ++k) {
                double v = 0;
                for (int ch = 0; ch < c.nchunk; ++ch) v += c.LLp[((int64_t)ch * N + i) * K + k];
                c.LL[(int64_t)i * K + k] = v;
            }
        return;
    }
    if (ref) {
        if (vb.x) return;
        if (threadIdx.x == 0) {
            Rng64 r; r.init(c.seed + (uint64_t)m, VP_SALT_UPDATEQ);
            double lnl = 0;
            for (int i = 0; i < N; ++i) sample_one(c, i, m, true, &r, &lnl);
            c.ctl->lnl = lnl;
        }
    } else {
        const int lane = threadIdx.x & 31;
        const int i = vb.x * (SAMPLE_BLOCK / 32) + (threadIdx.x >> 5);
        double lnl = 0;
        if (i < N) lnl = sample_warp(c, i, m, lane);
        double t = block_sum(lane == 0 ? lnl : 0.0, sh);
        if (threadIdx.x == 0) c.lnlp[vb.x] = t;
        if (!last_block_done(c.ctl, vb.gx)) return;
        const double tot = block_sum_partials(c.lnlp, vb.gx, sh);
        if (threadIdx.x == 0) {
            c.ctl->lnl = tot;
            c.ctl->done = 0;
        }
    }
    if (c.locpriori) {
        __syncthreads();
        for (int j = threadIdx.x; j < D.S * K; j += blockDim.x) c.Di[j] = 0.f;
        __syncthreads();
        // Q is one-hot, so these float sums are exact small integers
        for (int i = threadIdx.x; i < N; i += blockDim.x)
            if (D.vt[i]) atomicAdd(&c.Di[D.popid[i] * K + c.Z[i]], 1.f);
    }
}

// UpdateZNoAdmix (src/structure.cpp:1257-1301): Ni[k,l,a] = copies of allele a
// at locus l among individuals labelled k. One warp per locus. Biallelic
// diploid data: lane j takes individuals j, j+32, ... (coalesced codes and
// labels) into a lane-private shared histogram (no atomics, no conflicts), and
// the warp reduces it. General data: per-warp shared histogram with atomics.
constexpr int COUNT_WARPS = 4;
__global__ void __launch_bounds__(COUNT_WARPS * 32) k_count_noadmix(const DevChain* chains, int force, const int4* map = nullptr) {
    extern __shared__ int32_t hist[];
    const VBlock vb = vblock(map);
    const DevChain& c = chains[vb.z];
    if (map && run_over(c)) return;
    const DevData& D = c.D;
    const int K = c.K;
    if (!force && !binaryq_at(c, c.ctl->m)) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t l = (int64_t)vb.x * COUNT_WARPS + warp;
    if (D.packed2) {
        int32_t* h = hist + warp * (2 * K * 32);
        for (int j = 0; j < 2 * K; ++j) h[j * 32 + lane] = 0;
        if (l < D.L) {
            const uint32_t* row = D.g2 + l * D.Nw;
            // four independent loads in flight per lane
            for (int i0 = lane; i0 < D.N; i0 += 128) {
                uint32_t w[4];
                int z[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int i = i0 + 32 * u;
                    w[u] = i < D.N ? __ldg(row + (i >> 4)) : 0xFFFFFFFFu;
                    z[u] = i < D.N ? (int)c.Z[i] : 0;
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int i = i0 + 32 * u;
                    const int code = (w[u] >> ((i & 15) * 2)) & 3;
                    if (code == 3) continue;
                    h[(z[u] * 2) * 32 + lane] += 2 - code;
                    h[(z[u] * 2 + 1) * 32 + lane] += code;
                }
            }
            const int64_t o = D.off[l];
            for (int j = 0; j < 2 * K; ++j) {
                int v = h[j * 32 + lane];
                for (int sft = 16; sft > 0; sft >>= 1) v += __shfl_xor_sync(0xffffffffu, v, sft);
                if (lane == 0) c.Ni[(j >> 1) * D.KT + o + (j & 1)] = v;
            }
        }
        return;
    }
    const int hsz = K * D.maxK;
    int32_t* h = hist + warp * hsz;
    for (int j = lane; j < hsz; j += 32) h[j] = 0;
    __syncwarp();
    if (l < D.L) {
        int k2 = D.k[l];
        for (int i = lane; i < D.N; i += 32) {
            Copies cp;
            load_copies(D, l, i, cp);
            int z = c.Z[i];
            for (int a = 0; a < cp.n; ++a) atomicAdd(&h[z * k2 + cp.a[a]], 1);
        }
    }
    __syncwarp();
    if (l < D.L) {
        int k2 = D.k[l];
        for (int j = lane; j < K * k2; j += 32) {
            int k = j / k2, a = j % k2;
            c.Ni[k * D.KT + D.off[l] + a] = h[k * k2 + a];
        }
    }
}

// UpdateZNoAdmix counts (src/structure.cpp:1257-1348) for 2-bit packed data,
// from bit planes, two genotype words (32 individuals) per 32-bit plane. With
// lo/hi the two bit planes of a word's codes (1 = one copy of allele 1, 2 =
// two, 3 = missing), each at the even bit positions, the planes of words 2p
// and 2p + 1 merge into one word (the second on the odd positions): LO, HI and
// MS = LO & HI. A CTA first writes, for each cluster k of its group and each
// word pair p, the mask with the bits of the pair's individuals labelled k
// (shared memory, KC x Np words), then walks loci with one warp per locus and
// the lanes over the locus's word pairs:
//   allele-1 copies in cluster k = popc(LO & m) + 2 popc(HI & m) - 3 popc(MS & m)
//   typed calls in cluster k     = n_k - popc(MS & m)
// and allele-0 copies = 2 x typed - allele-1 copies. Integer and exact; the
// same Ni as k_count_noadmix. grid.z = cluster groups of KC.
template <int KC>
__global__ void __launch_bounds__(256) k_count_packed(const DevChain* chains, int kgroups, int force, const int4* map = nullptr) {
    extern __shared__ uint32_t smask[];   // [KC][Np] masks, then [KC] cluster sizes
    const VBlock vb = vblock(map);
    const DevChain& c = chains[vb.z / kgroups];
    if (map && run_over(c)) return;
    const int kg0 = (vb.z % kgroups) * KC;
    const DevData& D = c.D;
    const int K = c.K, Nw = D.Nw, Np = (D.Nw + 1) >> 1;
    if (!force && !binaryq_at(c, c.ctl->m)) return;
    const int kn = min(KC, K - kg0);
    int32_t* nk = reinterpret_cast<int32_t*>(smask + (size_t)KC * Np);
    if (threadIdx.x < KC) nk[threadIdx.x] = 0;
    __syncthreads();
    int cnt[KC];
#pragma unroll
    for (int k = 0; k < KC; ++k) cnt[k] = 0;
    for (int p = threadIdx.x; p < Np; p += blockDim.x) {
        uint32_t mk[KC];
#pragma unroll
        for (int k = 0; k < KC; ++k) mk[k] = 0;
        for (int j = 0; j < 32; ++j) {
            const int i = 32 * p + j;   // word 2p + (j >> 4), position j & 15
            const int z = i < D.N ? (int)c.Z[i] - kg0 : -1;
            const uint32_t bit = 1u << (2 * (j & 15) + (j >> 4));
#pragma unroll
            for (int k = 0; k < KC; ++k)
                if (z == k) mk[k] |= bit;
        }
#pragma unroll
        for (int k = 0; k < KC; ++k) {
            smask[(size_t)k * Np + p] = mk[k];
            cnt[k] += __popc(mk[k]);
        }
    }
#pragma unroll
    for (int k = 0; k < KC; ++k)
        if (cnt[k]) atomicAdd(&nk[k], cnt[k]);
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarp = blockDim.x >> 5;
    for (int64_t l = (int64_t)vb.x * nwarp + warp; l < D.L; l += (int64_t)vb.gx * nwarp) {
        const uint32_t* row = D.g2 + l * Nw;
        int a1[KC], n3[KC];
#pragma unroll
        for (int k = 0; k < KC; ++k) { a1[k] = 0; n3[k] = 0; }
        // four word pairs per lane in flight: their eight loads first
        for (int p0 = lane; p0 < Np; p0 += 128) {
            uint32_t g0[4], g1[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int p = p0 + 32 * u;
                // a missing word past the row's end: its masks are 0
                g0[u] = p < Np ? __ldg(row + 2 * p) : 0xFFFFFFFFu;
                g1[u] = p < Np && 2 * p + 1 < Nw ? __ldg(row + 2 * p + 1) : 0xFFFFFFFFu;
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int p = p0 + 32 * u;
                if (p >= Np) break;
                // bit select: even positions from the first operand, odd from the second
                const uint32_t LO = (g0[u] & 0x55555555u) | ((g1[u] << 1) & 0xAAAAAAAAu);
                const uint32_t HI = ((g0[u] >> 1) & 0x55555555u) | (g1[u] & 0xAAAAAAAAu);
                const uint32_t MS = LO & HI;
#pragma unroll
                for (int k = 0; k < KC; ++k) {
                    if (k < kn) {
                        const uint32_t m = smask[(size_t)k * Np + p];
                        const int p3 = __popc(MS & m);
                        a1[k] += __popc(LO & m) + 2 * __popc(HI & m) - 3 * p3;
                        n3[k] += p3;
                    }
                }
            }
        }
#pragma unroll
        for (int k = 0; k < KC; ++k) {
            if (k < kn) {
                int v = a1[k], u = n3[k];
                for (int o = 16; o > 0; o >>= 1) {
                    v += __shfl_xor_sync(0xffffffffu, v, o);
                    u += __shfl_xor_sync(0xffffffffu, u, o);
                }
                if (lane == 0) {
                    const int64_t o2 = (int64_t)(kg0 + k) * D.KT + D.off[l];
                    c.Ni[o2] = 2 * (nk[k] - u) - v;
                    c.Ni[o2 + 1] = v;
                }
            }
        }
    }
}

// Dirichlet draw of one individual's admixture proportions from alpha + counts
__device__ __forceinline__ void dirichlet_ref(Rng64& r, float* q, const double* a, const int32_t* b, int K) {
    double s = 0;
    for (int k = 0; k < K; ++k) {
        double v = r.gamma(a[k] + (b ? (double)b[k] : 0.0));
        q[k] = (float)v;
        s += v;
    }
    float inv = (float)(1.0 / s);
    for (int k = 0; k < K; ++k) q[k] *= inv;
}
__device__ __forceinline__ void dirichlet_ctr(Philox& p, float* q, const double* a, const int32_t* b, int K) {
    float s = 0;
    for (int k = 0; k < K; ++k) {
        float v = p.gammaf((float)(a[k] + (b ? (double)b[k] : 0.0)));
        q[k] = v;
        s += v;
    }
    float inv = 1.f / s;
    for (int k = 0; k < K; ++k) q[k] *= inv;
}

// UpdateQAdmix (src/structure.cpp:984-1004): Q_i ~ Dirichlet(alpha + Mi_i),
// used by the admixture model and the no-admixture burn-in
__global__ void k_update_q_admix(const DevChain* chains, int force, const int4* map = nullptr) {
    const VBlock vb = vblock(map);
    const DevChain& c = chains[vb.z];
    if (map && run_over(c)) return;
    const DevData& D = c.D;
    const int K = c.K, m = c.ctl->m;
    if (!force) {
        if (c.admix && metro_turn(c, m)) return;
        if (!c.admix && m >= c.nadmburnin) return;
    }
    if (c.rng == 0) {
        if (vb.x || threadIdx.x) return;
        Rng64 r; r.init(c.seed + (uint64_t)m, VP_SALT_UPDATEQ);
        for (int i = 0; i < D.N; ++i)
            if (D.vt[i])
                dirichlet_ref(r, c.Q + (int64_t)i * K, c.locpriori ? c.AlphaLocal + D.popid[i] * K : c.Alpha,
                              c.Mi + (int64_t)i * K, K);
        return;
    }
    for (int i = vb.x * blockDim.x + threadIdx.x; i < D.N; i += vb.gx * blockDim.x) {
        if (!D.vt[i]) continue;
        Philox p; p.init(c.seed, ST_Q | ((uint32_t)m << 4), (uint32_t)i, 1);
        dirichlet_ctr(p, c.Q + (int64_t)i * K, c.locpriori ? c.AlphaLocal + D.popid[i] * K : c.Alpha,
                      c.Mi + (int64_t)i * K, K);
    }
}

// UpdateQMetro (src/structure.cpp:1006-1086): proposals Q'_i ~ Dirichlet(alpha)
__global__ void k_metro_propose(const DevChain* chains, int force, const int4* map = nullptr) {
    const VBlock vb = vblock(map);
    const DevChain& c = chains[vb.z];
    if (map && run_over(c)) return;
    const DevData& D = c.D;
    const int K = c.K, m = c.ctl->m;
    if (!force && !metro_turn(c, m)) return;
    if (c.rng == 0) {
        if (vb.x || threadIdx.x) return;
        Rng64 r; r.init(c.seed + (uint64_t)m, VP_SALT_UPDATEQ);
        for (int i = 0; i < D.N; ++i)
            if (D.vt[i])
                dirichlet_ref(r, c.Qprop + (int64_t)i * K, c.locpriori ? c.AlphaLocal + D.popid[i] * K : c.Alpha,
                              nullptr, K);
        *c.rstate = r;  // the acceptance draws continue this stream
        return;
    }
    for (int i = vb.x * blockDim.x + threadIdx.x; i < D.N; i += vb.gx * blockDim.x) {
        if (!D.vt[i]) continue;
        Philox p; p.init(c.seed, ST_METRO_P | ((uint32_t)m << 4), (uint32_t)i, 0);
        dirichlet_ctr(p, c.Qprop + (int64_t)i * K, c.locpriori ? c.AlphaLocal + D.popid[i] * K : c.Alpha,
                      nullptr, K);
    }
}

// log likelihood ratio of the proposals (UpdateQMetro, src/structure.cpp:
// 1006-1086): the sum over loci and copies of ln( sum_k q'_k p / sum_k q_k p ).
// Warp = 32 individuals (one per lane), CTA = 8 warps; grid.y = the locus
// ranges of the per-copy label kernel, whose partials k_metro_accept adds. A CTA stages each slice of
// ZA_LC loci's frequencies in shared memory ([ZA_LC][MK][KPAD], odd stride)
// and keeps Q and Q' rows in registers (K <= KM; EXACT: K == KM). FP32 sums
// over SUB loci fold into FP64 (the same operations in the same order for
// every K). Defined after the per-copy label kernel, whose slice constants it
// shares.
template <int KM, bool EXACT>
__global__ void __launch_bounds__(256) k_metro_ratio(const DevChain* chains, int force, const int4* map = nullptr);

__global__ void k_metro_accept(const DevChain* chains, int force, const int4* map = nullptr) {
    const VBlock vb = vblock(map);
    const DevChain& c = chains[vb.z];
    if (map && run_over(c)) return;
    const DevData& D = c.D;
    const int K = c.K, m = c.ctl->m;
    if (!force && !metro_turn(c, m)) return;
    const bool ref = c.rng == 0;
    if (ref && (vb.x || threadIdx.x)) return;
    Rng64 r;
    if (ref) r = *c.rstate;
    for (int i = ref ? 0 : vb.x * blockDim.x + threadIdx.x; i < D.N; i += ref ? 1 : vb.gx * blockDim.x) {
        double d = 0;
        const int nm = (int)((D.L + c.zadm_lc - 1) / c.zadm_lc);   // k_metro_ratio's locus ranges
        for (int ch = 0; ch < nm; ++ch) d += c.metrop[(int64_t)ch * D.N + i];
        c.metro[i] = d;
        if (D.vt[i] == 0) continue;
        double u;
        bool acc = d >= VP_NZERO;
        if (!acc) {
            if (ref) u = r.uniform();
            else { Philox p; p.init(c.seed, ST_METRO_A | ((uint32_t)m << 4), (uint32_t)i, 0); u = p.uniformd(); }
            acc = u < exp(d);
        }
        if (acc)
            for (int k = 0; k < K; ++k) c.Q[(int64_t)i * K + k] = c.Qprop[(int64_t)i * K + k];
    }
}

// Zero Mi and Ni ahead of the per-copy label draws
__global__ void k_zero_counts(const DevChain* chains, int force, const int4* map = nullptr) {
    const VBlock vb = vblock(map);
    const DevChain& c = chains[vb.z];
    if (map && run_over(c)) return;
    if (!force && binaryq_at(c, c.ctl->m)) return;
    int64_t tid = vb.x * (int64_t)blockDim.x + threadIdx.x, nt = (int64_t)vb.gx * blockDim.x;
    for (int64_t j = tid; j < (int64_t)c.D.N * c.K; j += nt) c.Mi[j] = 0;
    for (int64_t j = tid; j < (int64_t)c.K * c.D.KT; j += nt) c.Ni[j] = 0;
    for (int64_t j = tid; j < c.nlnlp; j += nt) c.lnlp[j] = 0;
}

// Poly over float weights (src/statistics.cpp:357-385) with the reference's
// float/double promotions
__device__ __forceinline__ int poly_f(const float* w, int K, float u01_or_neg, Rng32* r) {
    float sx = 0.f;
    for (int k = 0; k < K; ++k) sx += w[k];
    float s = sx + VP_MIN_FREQ * K;
    float t = r ? r->uniform(0.f, s) : u01_or_neg * s;
    for (int k = 0; k < K; ++k) {
        if (t < w[k] + VP_MIN_FREQ) return k;
        t -= w[k] + VP_MIN_FREQ;
    }
    return K - 1;
}

// UpdateZAdmix with reference streams (src/structure.cpp:1350-1438): one
// thread per locus walks all individuals with RNG<float>(seed + m*L + l,
// SALT_UPDATEZ), drawing maxploidy numbers per individual whether or not the
// copies are typed. Also sums ln(sum_k q_k p) over copies: the admixture
// likelihood Record needs (src/structure.cpp:1917-1925).
__global__ void k_update_z_admix_ref(const DevChain* chains, int force, const int4* map = nullptr) {
    const VBlock vb = vblock(map);
    const DevChain& c = chains[vb.z];
    if (map && run_over(c)) return;
    const DevData& D = c.D;
    const int K = c.K, m = c.ctl->m;
    if (!force && binaryq_at(c, m)) return;
    __shared__ double sh[32];
    int64_t l = vb.x * (int64_t)blockDim.x + threadIdx.x;
    double lnl = 0;
    if (l < D.L) {
        Rng32 r;
        r.init(c.seed + (uint64_t)((int64_t)m * D.L + l), VP_SALT_UPDATEZ);
        int64_t o = D.off[l];
        float w[64];
        for (int i = 0; i < D.N; ++i) {
            Copies cp;
            load_copies(D, l, i, cp);
            const float* q = c.Q + (int64_t)i * K;
            for (int a = 0; a < D.maxploidy; ++a) {
                if (a >= cp.n) { r.next(); continue; }
                float sx = 0.f;
                for (int k = 0; k < K; ++k) { w[k] = q[k] * c.Freq[k * D.KT + o + cp.a[a]]; sx += w[k]; }
                lnl += (double)logf(sx);
                int k2 = poly_f(w, K, 0.f, &r);
                atomicAdd(&c.Mi[i * K + k2], 1);
                c.Ni[k2 * D.KT + o + cp.a[a]]++;
            }
        }
    }
    double t = block_sum(lnl, sh);
    if (threadIdx.x == 0) c.lnlp[vb.x] = t;
}

// UpdateZAdmix with counter streams. Warp = 32 individuals (one per lane),
// CTA = 8 warps = 256 individuals; grid.y splits the loci into ranges that a
// CTA walks in slices of ZA_LC loci. A lane keeps its individual's Q row and
// its Mi counts in registers; the slice's frequencies are staged in shared
// memory. With at most ZA_PACKED = 32 (cluster, allele) bins, one per lane,
// the per-copy increments of Ni are reduced across the warp before they reach
// the slice histogram in shared memory: each lane's bin becomes a 1 in one of
// five 6-bit fields of a word and redux.sync adds the words of the 32 lanes
// (one reduction per five bins), then lane j adds bin j; with more bins (multi-
// allelic data) each copy adds to the shared histogram directly (measured
// faster there than grouping lanes with __match_any_sync). The slice
// histogram is flushed to Ni with one global atomic per non-zero entry. KM is
// the cluster count rounded up to a compiled size; EXACT means K == KM.
// Uniforms: one Philox stream per (individual, slice of ZA_LC loci); every
// locus takes vmax consecutive draws, used or not, so a block of four serves
// two diploid loci and a missing call shifts nothing.
// Record's likelihood, the sum of ln(sum_k q_k p) over copies, is formed only
// on sweeps that Record reads (thinning points) or when the step is forced.
constexpr int ZA_WARPS = 8;
constexpr int ZA_LC = 16;
constexpr int ZA_PACKED = 32;   // lane j flushes bin j
static_assert(ZA_PACKED <= 32, "one histogram bin per lane");
template <int KM, bool EXACT>
__global__ void __launch_bounds__(ZA_WARPS * 32) k_update_z_admix_ctr(const DevChain* chains, int force, const int4* map = nullptr) {
    extern __shared__ unsigned char smraw[];
    const VBlock vb = vblock(map);
    const DevChain& c = chains[vb.z];
    if (map && run_over(c)) return;
    const DevData& D = c.D;
    const int K = EXACT ? KM : c.K, m = c.ctl->m, MK = D.maxK;
    if (!force && binaryq_at(c, m)) return;
    __shared__ double sh[32];
    const int KPAD = K | 1;                                       // odd stride: no bank conflicts
    const int nbins = K * MK;
    const bool packed = nbins <= ZA_PACKED;
    float* sF = reinterpret_cast<float*>(smraw);                  // [ZA_LC][MK][KPAD]
    int32_t* hs = reinterpret_cast<int32_t*>(sF + ZA_LC * MK * KPAD);  // [ZA_LC][K][MK]
    const int lane = threadIdx.x & 31;
    const int slot = vb.x * (ZA_WARPS * 32) + threadIdx.x;
    const bool live = slot < D.N;
    const int i = live && D.perm ? D.perm[slot] : slot;   // ascending ploidy with mixed ploidy
    constexpr int NPK = (KM + 7) / 8;
    static_assert(ZA_LC * 10 < 256, "8-bit label counts per slice");
    float q[KM];
    int32_t mi[KM];
#pragma unroll
    for (int k = 0; k < KM; ++k) { q[k] = (live && (EXACT || k < K)) ? c.Q[(int64_t)i * K + k] : 0.f; mi[k] = 0; }
    const int64_t lb0 = (int64_t)vb.y * c.zadm_lc, lb1 = min(D.L, lb0 + c.zadm_lc);
    float ls = 0.f, lc = 0.f;  // Kahan sum of ln(sum_k q_k p)
    const bool rec = force || record_at(c, m);
    for (int64_t l0 = lb0; l0 < lb1; l0 += ZA_LC) {
        const int nl = (int)min((int64_t)ZA_LC, lb1 - l0);
        __syncthreads();
        for (int j = threadIdx.x; j < ZA_LC * MK * KPAD; j += blockDim.x) {
            int k = j % KPAD, a = (j / KPAD) % MK, ll = j / (KPAD * MK);
            float v = 0.f;
            if (ll < nl && k < K && a < D.k[l0 + ll]) v = __ldg(c.Freq + (int64_t)k * D.KT + D.off[l0 + ll] + a);
            sF[j] = v;
        }
        for (int j = threadIdx.x; j < ZA_LC * K * MK; j += blockDim.x) hs[j] = 0;
        __syncthreads();
        Philox ph;
        ph.init(c.seed, ST_ZSLICE | ((uint32_t)m << 4), (uint32_t)(l0 / ZA_LC), (uint32_t)i);
        uint64_t pk[NPK];
#pragma unroll
        for (int w = 0; w < NPK; ++w) pk[w] = 0;
        for (int ll = 0; ll < nl; ++ll) {
            const int64_t l = l0 + ll;
            Copies cp;
            if (live) load_copies(D, l, i, cp); else cp.n = 0;
            float lacc = 0.f;
            int32_t* hl = hs + ll * nbins;
            // with mixed ploidy the warp loops over its largest copy count;
            // every individual's stream still advances by vmax draws per locus
            const int nw = D.perm ? (int)__reduce_max_sync(0xffffffffu, (unsigned)cp.n) : D.vmax;
            for (int a = 0; a < nw; ++a) {
                const bool act = a < cp.n;
                const float u = ph.uniformf();
                int key = -1;
                if (act) {
                    const int al = cp.a[a];
                    const float* f = sF + (ll * MK + al) * KPAD;
                    // prefix sums of the weights q_k p_k (fused multiply-adds)
                    float sx = 0.f, pre[KM];
#pragma unroll
                    for (int k = 0; k < KM; ++k) {
                        if (EXACT || k < K) sx = __fmaf_rn(q[k], f[k], sx);
                        pre[k] = sx;
                    }
                    if (rec) lacc += logf(sx);
                    // Poly (src/statistics.cpp:357-385): the first cluster whose
                    // cumulative weight (each weight + 1e-10) exceeds the
                    // uniform times the total; the comparisons are independent
                    // of each other, the smallest passing cluster wins
                    const float t = u * (sx + (float)(VP_MIN_FREQ * K));
                    int k2 = K - 1;
#pragma unroll
                    for (int k = KM - 1; k >= 0; --k)
                        if ((EXACT || k < K) && t < __fmaf_rn((float)(k + 1), (float)VP_MIN_FREQ, pre[k])) k2 = k;
                    // this slice's label counts, 8 bits per cluster (at most
                    // ZA_LC x 10 copies per slice)
#pragma unroll
                    for (int w = 0; w < NPK; ++w)
                        if (w == (k2 >> 3)) pk[w] += 1ull << (8 * (k2 & 7));
                    key = k2 * MK + al;
                }
                if (packed) {
                    // every lane of the warp takes part (a < vmax is warp-uniform)
                    uint32_t mine = 0;
#pragma unroll
                    for (int w = 0; w < (ZA_PACKED + 4) / 5; ++w) {
                        if (w * 5 >= nbins) break;
                        const uint32_t v = (key >= 0 && key / 5 == w) ? 1u << (6 * (key % 5)) : 0u;
                        const uint32_t sw = __reduce_add_sync(0xffffffffu, v);
                        if (lane / 5 == w) mine = sw;
                    }
                    if (lane < nbins) {
                        const int cnt = (int)((mine >> (6 * (lane % 5))) & 63u);
                        if (cnt) atomicAdd(&hl[lane], cnt);
                    }
                } else if (act) {
                    atomicAdd(&hl[key], 1);
                }
            }
            ph.skip(D.vmax - nw);
            float y = lacc - lc, tt = ls + y;
            lc = (tt - ls) - y;
            ls = tt;
        }
#pragma unroll
        for (int k = 0; k < KM; ++k) mi[k] += (int32_t)((pk[k >> 3] >> (8 * (k & 7))) & 0xFFu);
        __syncthreads();
        for (int j = threadIdx.x; j < ZA_LC * K * MK; j += blockDim.x) {
            int v = hs[j];
            if (!v) continue;
            int a = j % MK, k = (j / MK) % K, ll = j / (MK * K);
            atomicAdd(&c.Ni[(int64_t)k * D.KT + D.off[l0 + ll] + a], v);
        }
    }
    if (live)
#pragma unroll
        for (int k = 0; k < KM; ++k)
            if ((EXACT || k < K) && mi[k]) atomicAdd(&c.Mi[(int64_t)i * K + k], mi[k]);
    double t = block_sum((double)ls - (double)lc, sh);
    if (threadIdx.x == 0) c.lnlp[vb.y * vb.gx + vb.x] = t;
}

template <int KM, bool EXACT>
__global__ void __launch_bounds__(256) k_metro_ratio(const DevChain* chains, int force, const int4* map) {
    extern __shared__ unsigned char smraw[];
    const VBlock vb = vblock(map);
    const DevChain& c = chains[vb.z];
    if (map && run_over(c)) return;
    const DevData& D = c.D;
    const int K = EXACT ? KM : c.K, m = c.ctl->m, MK = D.maxK;
    if (!force && !metro_turn(c, m)) return;
    const int KPAD = K | 1;
    float* sF = reinterpret_cast<float*>(smraw);   // [ZA_LC][MK][KPAD]
    const int slot = vb.x * blockDim.x + threadIdx.x;
    const bool live = slot < D.N;
    const int i = live && D.perm ? D.perm[slot] : slot;   // ascending ploidy with mixed ploidy
    float q1[KM], q0[KM];
#pragma unroll
    for (int k = 0; k < KM; ++k) {
        const bool on = live && (EXACT || k < K);
        q1[k] = on ? c.Qprop[(int64_t)i * K + k] : 0.f;
        q0[k] = on ? c.Q[(int64_t)i * K + k] : 0.f;
    }
    const int64_t lc0 = (int64_t)vb.y * c.zadm_lc, lc1 = min(D.L, lc0 + c.zadm_lc);
    double accd = 0;
    float acc = 0.f;
    int cnt = 0;
    for (int64_t l0 = lc0; l0 < lc1; l0 += ZA_LC) {
        const int nl = (int)min((int64_t)ZA_LC, lc1 - l0);
        __syncthreads();
        for (int j = threadIdx.x; j < ZA_LC * MK * KPAD; j += blockDim.x) {
            const int k = j % KPAD, a = (j / KPAD) % MK, ll = j / (KPAD * MK);
            float v = 0.f;
            if (ll < nl && k < K && a < D.k[l0 + ll]) v = __ldg(c.Freq + (int64_t)k * D.KT + D.off[l0 + ll] + a);
            sF[j] = v;
        }
        __syncthreads();
        for (int ll = 0; ll < nl; ++ll) {
            Copies cp;
            if (live) load_copies(D, l0 + ll, i, cp); else cp.n = 0;
            for (int a = 0; a < cp.n; ++a) {
                const float* f = sF + (ll * MK + cp.a[a]) * KPAD;
                float s1 = 0.f, s2 = 0.f;
#pragma unroll
                for (int k = 0; k < KM; ++k)
                    if (EXACT || k < K) {
                        s1 = __fmaf_rn(q1[k], f[k], s1);
                        s2 = __fmaf_rn(q0[k], f[k], s2);
                    }
                acc += logf(s1 / s2);
            }
            if (++cnt == SUB) { cnt = 0; accd += acc; acc = 0.f; }
        }
    }
    if (live) c.metrop[(int64_t)vb.y * D.N + i] = accd + (double)acc;
}

// ---------------------------------------------------------------------------
// exponent-split log product (src/math2.h:738-894, src/math2.cpp:1030-1116),
// serial, for the reference-stream Metropolis-Hastings steps
__device__ __forceinline__ void chargelog_f(int64_t& slog, double& prod, float v) {
    prod *= (double)v;
    if (prod < 1e-100 || prod > 1e100) {
        long long b = __double_as_longlong(prod);
        slog += ((b & 0x7FF0000000000000ll) >> 52) - 1023;
        prod = __longlong_as_double((b & (long long)0x800FFFFFFFFFFFFFull) | 0x3FF0000000000000ll);
    }
}
__device__ __forceinline__ void chargelog_d(int64_t& slog, double& prod, double v) {
    if (v < 1e-100 || v > 1e100) {
        long long b = __double_as_longlong(v);
        slog += ((b & 0x7FF0000000000000ll) >> 52) - 1023;
        v = __longlong_as_double((b & (long long)0x800FFFFFFFFFFFFFull) | 0x3FF0000000000000ll);
    }
    prod *= v;
    if (prod < 1e-100 || prod > 1e100) {
        long long b = __double_as_longlong(prod);
        slog += ((b & 0x7FF0000000000000ll) >> 52) - 1023;
        prod = __longlong_as_double((b & (long long)0x800FFFFFFFFFFFFFull) | 0x3FF0000000000000ll);
    }
}
__device__ __forceinline__ double closelog(int64_t slog, double prod) { return ((double)slog + log2(prod)) * 0.693147180559945; }
__device__ double logprod_f_serial(const float* a, int64_t n, int64_t sep) {
    int64_t s = 0; double p = 1;
    for (int64_t i = 0; i < n; ++i) chargelog_f(s, p, a[i * sep]);
    return closelog(s, p);
}
__device__ double logprod_d_serial(const double* a, int64_t n, int64_t sep) {
    int64_t s = 0; double p = 1;
    for (int64_t i = 0; i < n; ++i) chargelog_d(s, p, a[i * sep]);
    return closelog(s, p);
}

// Sums of ln Q that UpdateAlpha needs: one sequence per output
//   inferalpha, one alpha: ln prod Q over all N*K (1 output)
//   diffalpha:             ln prod Q[., k] (K outputs)
//   location prior+admix:  ln prod Q[i in s, k] (S*K outputs)
// Reference streams use the serial exponent-split product (a zero resets its
// running mantissa, as in the reference); counter streams a parallel sum.
constexpr int LPQ_BLOCKS = 64;
__global__ void k_logprod_q(const DevChain* chains, const int4* map = nullptr) {
    const VBlock vb = vblock(map);
    const DevChain& c = chains[vb.z];
    if (map && run_over(c)) return;
    const DevData& D = c.D;
    const int K = c.K, m = c.ctl->m;
    __shared__ double sh[32];
    int nseq, mode;
    if (c.locpriori && c.admix) { nseq = D.S * K; mode = 2; }
    else if (c.inferalpha && (c.admix || m < c.nadmburnin)) { nseq = c.diffalpha ? K : 1; mode = c.diffalpha; }
    else return;
    if (c.rng == 0) {
        // reference streams: the serial exponent-split product, one thread per sequence
        for (int s = vb.x * blockDim.x + threadIdx.x; s < nseq; s += vb.gx * blockDim.x) {
            const float* base; int64_t n, sep;
            if (mode == 2) { int sp = s / K, k = s % K; base = c.Q + (int64_t)D.pop_ind0[sp] * K + k; n = D.pop_nind[sp]; sep = K; }
            else if (mode == 1) { base = c.Q + s; n = D.N; sep = K; }
            else { base = c.Q; n = (int64_t)D.N * K; sep = 1; }
            c.red[s] = logprod_f_serial(base, n, sep);
        }
        return;
    }
    if (mode == 2 && D.popcontig) {
        // counter streams, one sequence per (location, cluster) over the
        // location's consecutive rows: one block per location, one block sum
        // per cluster (deterministic)
        for (int sp = vb.x; sp < D.S; sp += vb.gx) {
            const int64_t r0 = D.pop_ind0[sp], n = D.pop_nind[sp];
            for (int k = 0; k < K; ++k) {
                double v = 0;
                for (int64_t rr = threadIdx.x; rr < n; rr += blockDim.x) {
                    const float q = c.Q[(r0 + rr) * K + k];
                    v += q > 0.f ? (double)logf(q) : -709.0895657128241;
                }
                v = block_sum(v, sh);
                if (threadIdx.x == 0) c.red[sp * K + k] = v;
            }
        }
        return;
    }
    // counter streams: sum of ln Q per sequence, per-block partials reduced by
    // the last block in a fixed order
    double* part = c.red + (D.S * K + K + 1);   // [LPQ_BLOCKS][nseq]
    const int64_t NK = (int64_t)D.N * K;
    for (int s = 0; s < nseq; ++s) {
        double v = 0;
        const int64_t per = (NK + vb.gx - 1) / vb.gx;
        const int64_t j0 = vb.x * per, j1 = min(NK, j0 + per);
        for (int64_t j = j0 + threadIdx.x; j < j1; j += blockDim.x) {
            const int i = (int)(j / K), k = (int)(j % K);
            const int sq = mode == 2 ? D.popid[i] * K + k : mode == 1 ? k : 0;
            if (sq != s) continue;
            const float q = c.Q[j];
            v += q > 0.f ? (double)logf(q) : -709.0895657128241;
        }
        v = block_sum(v, sh);
        if (threadIdx.x == 0) part[vb.x * nseq + s] = v;
    }
    if (!last_block_done(c.ctl, vb.gx)) return;
    for (int s = threadIdx.x; s < nseq; s += blockDim.x) {
        double t = 0;
        for (int b2 = 0; b2 < (int)vb.gx; ++b2) t += part[b2 * nseq + s];
        c.red[s] = t;
    }
    if (threadIdx.x == 0) c.ctl->done = 0;
}

// UpdateAlpha (src/structure.cpp:1499-1594), reference stream
// RNG(seed + m, SALT_UPDATEALPHA), on one thread
// counter streams, location prior with admixture. The K global steps are
// independent of one another (each moves Alpha[k] against AlphaLocal[., k]):
// one thread per cluster, each on its own Philox stream. A location's K
// local steps share its SumAlpha and stay in order on one thread, but every
// term that does not involve SumAlpha (the proposal on its own Philox
// stream, ln(am/ao), lgamma(am), lgamma(ao), the ln Q sum) is formed first by
// one thread per (location, cluster); the ordered pass then adds the two
// SumAlpha lgamma terms and decides. Needs blockDim.x >= K.
__device__ void update_alpha_locprior_ctr(const DevChain& c, int m) {
    const DevData& D = c.D;
    const int K = c.K, S = D.S;
    const double r = c.ctl->r;
    const int t = threadIdx.x;
    if (t < K) {
        const int k = t;
        Philox ph;
        ph.init(c.seed, ST_ALPHA | ((uint32_t)m << 4), 0xFFFFFFFFu, 2u + (uint32_t)k);
        const double a0 = c.Alpha[k], am = a0 + c.stdalpha * ph.normald();
        if (am > 0 && am < c.maxalpha) {
            const double d = am - a0;
            double dlnL = S * (d * r * ref_mylog(r) + lgamma(r * a0) - lgamma(r * am));
            double lp = 0;   // ln of the product over locations of AlphaLocal[., k]
            for (int sl = 0; sl < S; ++sl) lp += ref_mylog(c.AlphaLocal[sl * K + k]);
            dlnL += r * d * lp;
            if (dlnL >= VP_NZERO || ph.uniformd() < exp(dlnL)) c.Alpha[k] = am;
        }
    }
    __syncthreads();
    // proposals and the SumAlpha-free part of each local log ratio, [S][K] x
    // (proposal, partial ratio, uniform), in the region of c.red that holds
    // k_logprod_q's block partials (reduced before this kernel runs)
    double* pre = c.red + ((int64_t)S * K + K + 1);
    for (int j = t; j < S * K; j += blockDim.x) {
        const int s = j / K, k = j % K;
        Philox ph;
        ph.init(c.seed, ST_ALPHA | ((uint32_t)m << 4), (uint32_t)s, 2u + (uint32_t)k);
        const double ao = c.AlphaLocal[j], am = ao + c.stdalpha * ph.normald();
        const double u = ph.uniformd();
        double part = 0.0;
        if (am > 0 && am < c.maxalpha) {
            const double d = am - ao;
            part = (r * c.Alpha[k] - 1) * ref_mylog(am / ao) - d * r + D.pop_nind[s] * (lgamma(ao) - lgamma(am)) +
                   d * c.red[j];
        }
        pre[3 * (int64_t)j] = am;
        pre[3 * (int64_t)j + 1] = part;
        pre[3 * (int64_t)j + 2] = u;
    }
    __syncthreads();
    for (int s = t; s < S; s += blockDim.x) {
        if (m % 10 == 0) {
            double tt = 0;
            for (int k = 0; k < K; ++k) tt += c.AlphaLocal[s * K + k];
            c.SumAlpha[s] = tt;
        }
        const int snind = D.pop_nind[s];
        for (int k = 0; k < K; ++k) {
            const int64_t j = (int64_t)s * K + k;
            const double ao = c.AlphaLocal[j], am = pre[3 * j];
            if (am > 0 && am < c.maxalpha) {
                const double d = am - ao;
                const double dlnL = pre[3 * j + 1] + snind * (lgamma(c.SumAlpha[s] + d) - lgamma(c.SumAlpha[s]));
                if (dlnL >= VP_NZERO || pre[3 * j + 2] < exp(dlnL)) {
                    c.AlphaLocal[j] = am;
                    c.SumAlpha[s] += d;
                }
            }
        }
    }
}

__global__ void k_update_alpha(const DevChain* chains, const int4* map = nullptr) {
    const VBlock vb = vblock(map);
    const DevChain& c = chains[vb.z];
    if (map && run_over(c)) return;
    if (vb.x) return;
    if (c.rng != 0 && c.locpriori && c.admix) {
        update_alpha_locprior_ctr(c, c.ctl->m);
        return;
    }
    if (threadIdx.x) return;
    const DevData& D = c.D;
    const int K = c.K, m = c.ctl->m, S = D.S, N = D.N;
    Rng64 rng; rng.init(c.seed + (uint64_t)m, VP_SALT_UPDATEALPHA);
    if (c.locpriori && c.admix) {
        double r = c.ctl->r;
        for (int k = 0; k < K; ++k) {
            double am = rng.normal(c.Alpha[k], c.stdalpha);
            if (am > 0 && am < c.maxalpha) {
                double d = am - c.Alpha[k];
                double dlnL = S * (d * r * ref_mylog(r) + lgamma(r * c.Alpha[k]) - lgamma(r * am));
                dlnL += r * d * logprod_d_serial(c.AlphaLocal + k, S, K);
                if (dlnL >= VP_NZERO || rng.uniform() < exp(dlnL)) c.Alpha[k] = am;
            }
        }
        if (m % 10 == 0)
            for (int s = 0; s < S; ++s) {
                double t = 0;
                for (int k = 0; k < K; ++k) t += c.AlphaLocal[s * K + k];
                c.SumAlpha[s] = t;
            }
        for (int s = 0; s < S; ++s) {
            int snind = D.pop_nind[s];
            for (int k = 0; k < K; ++k) {
                double ao = c.AlphaLocal[s * K + k], am = rng.normal(ao, c.stdalpha);
                if (am > 0 && am < c.maxalpha) {
                    double d = am - ao;
                    double dlnL = (r * c.Alpha[k] - 1) * ref_mylog(am / ao) - d * r +
                        snind * (lgamma(c.SumAlpha[s] + d) - lgamma(am) - lgamma(c.SumAlpha[s]) + lgamma(ao));
                    dlnL += d * c.red[s * K + k];
                    if (dlnL >= VP_NZERO || rng.uniform() < exp(dlnL)) {
                        c.AlphaLocal[s * K + k] = am;
                        c.SumAlpha[s] += d;
                    }
                }
            }
        }
        return;
    }
    if (!c.inferalpha) return;
    if (!c.admix && m >= c.nadmburnin) return;
    if (c.diffalpha) {
        double sumalpha = 0;
        for (int k = 0; k < K; ++k) sumalpha += c.Alpha[k];
        for (int k = 0; k < K; ++k) {
            double am = rng.normal(c.Alpha[k], c.stdalpha);
            if (am <= 0 || (am >= c.maxalpha && c.uniformalpha)) continue;
            double ao = c.Alpha[k], d = am - ao;
            double dlnL = c.uniformalpha ? 0 : ((c.alphapriora - 1) * ref_mylog(am / ao) + (ao - am) / c.alphapriorb);
            dlnL += (am - ao) * c.red[k] + (lgamma(sumalpha + d) - lgamma(sumalpha) - lgamma(am) + lgamma(ao)) * N;
            if (dlnL >= VP_NZERO || rng.uniform() < exp(dlnL)) c.Alpha[k] = am;
        }
    } else {
        double am = rng.normal(c.Alpha[0], c.stdalpha);
        if (am <= 0 || (am >= c.maxalpha && c.uniformalpha)) return;
        double ao = c.Alpha[0];
        double dlnL = c.uniformalpha ? 0 : ((c.alphapriora - 1) * ref_mylog(am / ao) + (ao - am) / c.alphapriorb);
        dlnL += (am - ao) * c.red[0] + (lgamma(K * am) - lgamma(K * ao) - K * lgamma(am) + K * lgamma(ao)) * N;
        if (dlnL >= VP_NZERO || rng.uniform() < exp(dlnL))
            for (int k = 0; k < K; ++k) c.Alpha[k] = am;
    }
}

// UpdateLocPriori (src/structure.cpp:1168-1255), one thread
__global__ void k_update_locpriori(const DevChain* chains, const int4* map = nullptr) {
    const VBlock vb = vblock(map);
    const DevChain& c = chains[vb.z];
    if (map && run_over(c)) return;
    if (threadIdx.x || vb.x || !c.locpriori) return;
    const DevData& D = c.D;
    const int K = c.K, S = D.S, m = c.ctl->m;
    Rng64 rng; rng.init(c.seed + (uint64_t)m, VP_SALT_UPDATELOC);
    double r = c.ctl->r, epsr = c.epsr;
    if (c.admix) {
        double rm = rng.uniform(r - epsr, r + epsr);
        if (rm > 0 && rm < c.maxr) {
            double dlnL = 0, d = rm - r, dt1 = rm * ref_mylog(rm) - r * ref_mylog(r);
            for (int k = 0; k < K; ++k) {
                dlnL += S * (c.Alpha[k] * dt1 - lgamma(rm * c.Alpha[k]) + lgamma(r * c.Alpha[k]));
                double sa = 0;
                for (int s = 0; s < S; ++s) sa += c.AlphaLocal[s * K + k];
                dlnL += c.Alpha[k] * d * logprod_d_serial(c.AlphaLocal + k, S, K) - sa * d;
            }
            if (dlnL >= VP_NZERO || rng.uniform() < exp(dlnL)) c.ctl->r = rm;
        }
        return;
    }
    double rm = rng.uniform(r - epsr, r + epsr);
    if (rm > 0 && rm < c.maxr) {
        double dlnL = lgamma(rm) - lgamma(r);
        for (int k = 0; k < K; ++k) dlnL += lgamma(r * c.Eta[k]) - lgamma(rm * c.Eta[k]);
        dlnL *= S;
        for (int k = 0; k < K; ++k) dlnL += (rm - r) * c.Eta[k] * logprod_d_serial(c.Gamma + k, S, K);
        if (dlnL >= VP_NZERO || rng.uniform() < exp(dlnL)) c.ctl->r = rm;
    }
    r = c.ctl->r;
    if (K >= 2) {
        int i1 = (int)rng.nextn(K), j1 = (int)rng.next_avoid(K, i1);
        double delta = rng.uniform(0, c.epseta);
        double e1 = c.Eta[i1] + delta, e2 = c.Eta[j1] - delta;
        if (e1 < 1 && e2 > 0) {
            double dlnL = S * (lgamma(r * c.Eta[i1]) + lgamma(r * c.Eta[j1]) - lgamma(r * e1) - lgamma(r * e2));
            dlnL += r * delta * (logprod_d_serial(c.Gamma + i1, S, K) - logprod_d_serial(c.Gamma + j1, S, K));
            if (dlnL >= VP_NZERO || rng.uniform() < exp(dlnL)) { c.Eta[i1] += delta; c.Eta[j1] -= delta; }
        }
        for (int s = 0; s < S; ++s) {
            int a = (int)rng.nextn(K), b = (int)rng.next_avoid(K, a);
            double dl = rng.uniform(0, c.epsgamma);
            double* G = c.Gamma + s * K;
            if (G[a] + dl < 1 && G[b] - dl > 0) {
                double dlnL = (r * c.Eta[a] - 1.0 + c.Di[s * K + a]) * ref_mylog(1 + dl / G[a]) +
                              (r * c.Eta[b] - 1.0 + c.Di[s * K + b]) * ref_mylog(1 - dl / G[b]);
                if (dlnL >= VP_NZERO || rng.uniform() < exp(dlnL)) { G[a] += dl; G[b] -= dl; }
            }
        }
    }
    if (m % 10 == 0) {
        // Unify (src/math2.cpp:2268-2285)
        double s = 0;
        for (int k = 0; k < K; ++k) s += c.Eta[k];
        double inv = 1.0 / (s + K * VP_MIN_FREQ);
        for (int k = 0; k < K; ++k) c.Eta[k] = (c.Eta[k] + VP_MIN_FREQ) * inv;
        for (int sp = 0; sp < S; ++sp) {
            double* G = c.Gamma + sp * K;
            double t = 0;
            for (int k = 0; k < K; ++k) t += G[k];
            double iv = 1.0 / (t + K * VP_MIN_FREQ);
            for (int k = 0; k < K; ++k) G[k] = (G[k] + VP_MIN_FREQ) * iv;
        }
    }
}

// UpdateA1 (src/structure.cpp:1646-1695): independent Dirichlet proposal of the
// ancestral frequencies at each locus. Reference streams: 32 block streams.
__device__ void update_a1_locus(const DevChain& c, int64_t l, Rng64* r, Philox* ph, float* pb, float* pc) {
    const DevData& D = c.D;
    const int K = c.K;
    int k2 = D.k[l];
    float* pa = c.FreqA + D.off[l];
    double lam = c.Lambda[0];
    for (int a = 0; a < k2; ++a) pb[a] = (float)lam;
    for (int k = 0; k < K; ++k) {
        const float* pk = c.Freq + k * D.KT + D.off[l];
        float fk = (float)c.f[k];
        for (int a = 0; a < k2; ++a) pb[a] += pk[a] * fk;
    }
    double s = 0;
    for (int a = 0; a < k2; ++a) {
        double v = r ? r->gamma((double)pb[a] * 1.0) : (double)ph->gammaf(pb[a]);
        pc[a] = (float)v;
        s += v;
    }
    float inv = (float)(1.0 / s);
    for (int a = 0; a < k2; ++a) pc[a] *= inv;
    double dlnL = 0;
    for (int a = 0; a < k2; ++a) dlnL += (pb[a] - lam) * (ref_mylog(pa[a] / pc[a]));
    for (int k = 0; k < K; ++k) {
        const float* pk = c.Freq + k * D.KT + D.off[l];
        double fr = c.f[k];
        for (int a = 0; a < k2; ++a)
            dlnL += lgamma(fr * pa[a]) - lgamma(fr * pc[a]) + fr * (pc[a] - pa[a]) * ref_mylog(pk[a]);
    }
    double u = dlnL >= VP_NZERO ? 0 : (r ? r->uniform() : ph->uniformd());
    if (dlnL >= VP_NZERO || u < exp(dlnL))
        for (int a = 0; a < k2; ++a) pa[a] = pc[a];
}

// UpdateA2 (src/structure.cpp:1745-1804): move mass delta between two alleles.
// The reference does not advance its frequency pointer on a rejected-bounds
// locus, so later loci of the same block read shifted frequencies; `pshift`
// carries that offset for the reference-stream form.
__device__ void update_a2_locus(const DevChain& c, int64_t l, int64_t pshift, Rng64* r, Philox* ph, bool* skipped) {
    const DevData& D = c.D;
    const int K = c.K;
    int k2 = D.k[l];
    float* pa = c.FreqA + D.off[l];
    const float* p = c.Freq + D.off[l] - pshift;
    double lam = c.Lambda[0];
    int m1, n1;
    double delta;
    if (r) {
        m1 = (int)r->nextn(k2); n1 = (int)r->next_avoid(k2, m1);
        delta = r->uniform(0, pow((double)D.N, -0.5));
    } else {
        m1 = (int)(ph->next() % (uint32_t)k2);
        n1 = (int)(ph->next() % (uint32_t)(k2 - 1)); if (n1 >= m1) n1++;
        delta = ph->uniformd() * pow((double)D.N, -0.5);
    }
    double pm0 = pa[m1], pm1 = pm0 + delta, pn0 = pa[n1], pn1 = pn0 - delta;
    *skipped = pm1 >= 1 || pn1 <= 0;
    if (*skipped) return;
    double dlnL = (lam - 1) * ref_mylog(pm1 * pn1 / pm0 / pn0);
    for (int k = 0; k < K; ++k) {
        double fr = c.f[k];
        dlnL += lgamma(fr * pm0) + lgamma(fr * pn0) - lgamma(fr * pm1) - lgamma(fr * pn1) +
                (fr * delta) * ref_mylog(p[k * D.KT + m1] / p[k * D.KT + n1]);
    }
    double u = dlnL >= VP_NZERO ? 0 : (r ? r->uniform() : ph->uniformd());
    if (dlnL >= VP_NZERO || u < exp(dlnL)) { pa[m1] = (float)pm1; pa[n1] = (float)pn1; }
}

__global__ void k_update_a(const DevChain* chains, const int4* map = nullptr) {
    const VBlock vb = vblock(map);
    const DevChain& c = chains[vb.z];
    if (map && run_over(c)) return;
    if (!c.fmodel) return;
    const DevData& D = c.D;
    const int m = c.ctl->m;
    const bool one = hash_ulong(c.seed + (uint64_t)m) & 1;
    if (c.rng == 0) {
        int b = vb.x * blockDim.x + threadIdx.x;
        if (b >= 32) return;
        int64_t l0 = b * D.L / 32, l1 = (b + 1) * D.L / 32;
        Rng64 r; r.init(c.seed + (uint64_t)(m * 32 + b), VP_SALT_UPDATEA);
        float* pb = c.fbuf + (D.maxK + 16) * b * 2;
        float* pc = pb + D.maxK + 16;
        int64_t pshift = 0;
        for (int64_t l = l0; l < l1; ++l) {
            if (one) update_a1_locus(c, l, &r, nullptr, pb, pc);
            else {
                bool sk;
                update_a2_locus(c, l, pshift, &r, nullptr, &sk);
                if (sk) pshift += D.k[l];
            }
        }
        return;
    }
    int64_t l = vb.x * (int64_t)blockDim.x + threadIdx.x;
    if (l >= D.L) return;
    Philox ph; ph.init(c.seed, ST_A | ((uint32_t)m << 4), (uint32_t)l, 0);
    float pb[64], pc[64];
    if (one) update_a1_locus(c, l, nullptr, &ph, pb, pc);
    else { bool sk; update_a2_locus(c, l, 0, nullptr, &ph, &sk); }
}

// UpdateF (src/structure.cpp:1806-1858): per-cluster F with a Normal random
// walk. One block per chain: thread 0 owns the stream, the block reduces the
// sum over all alleles for each proposal.
__global__ void k_update_f(const DevChain* chains, const int4* map = nullptr) {
    const VBlock vb = vblock(map);
    const DevChain& c = chains[vb.z];
    if (map && run_over(c)) return;
    if (!c.fmodel) return;
    const DevData& D = c.D;
    const int K = c.K, m = c.ctl->m;
    __shared__ double sh[32];
    __shared__ double s_fm, s_fo, s_Fm;
    __shared__ int s_go;
    Rng64 rng;
    if (threadIdx.x == 0) rng.init(c.seed + (uint64_t)m, VP_SALT_UPDATEF);
    for (int k = 0; k < K; ++k) {
        if (threadIdx.x == 0) {
            double Fo = c.F[k];
            double Fm = rng.normal(Fo, c.stdf);
            s_go = !(Fm < 0 || Fm > 1);
            s_Fm = Fm; s_fo = c.f[k]; s_fm = (1 - Fm) / Fm;
        }
        __syncthreads();
        if (!s_go) {
            if (c.fsame) return;
            __syncthreads();
            continue;
        }
        double fm = s_fm, fo = s_fo;
        double part = 0;
        for (int k2 = k; k2 < K; ++k2) {
            const float* p = c.Freq + k2 * D.KT;
            for (int64_t a = threadIdx.x; a < D.KT; a += blockDim.x) {
                float pa2 = c.FreqA[a];
                part += pa2 * (fm - fo) * ref_mylog(p[a]) + lgamma(fo * pa2) - lgamma(fm * pa2);
            }
            if (!c.fsame) break;
        }
        double tot = block_sum(part, sh);
        if (threadIdx.x == 0) {
            double Fo = c.F[k], Fm = s_Fm;
            double dlnL = c.pmeanf * (Fo - Fm) / (c.pstdf * c.pstdf) +
                          (c.pmeanf * c.pmeanf / (c.pstdf * c.pstdf) - 1) * ref_mylog(Fm / Fo) +
                          (c.fsame ? K : 1) * D.L * (lgamma(fm) - lgamma(fo));
            dlnL += tot;
            if (dlnL >= VP_NZERO || rng.uniform() < exp(dlnL)) {
                if (c.fsame) for (int j = 0; j < K; ++j) { c.F[j] = Fm; c.f[j] = fm; }
                else { c.F[k] = Fm; c.f[k] = fm; }
            }
        }
        __syncthreads();
        if (c.fsame) return;
    }
}

// Record (src/structure.cpp:1941-2045): likelihood trace, running sums of the
// likelihood and parameters, then m += 1. One block per chain.
// the scalar part of Record at sweep m, by one block
__device__ void record_scalars(const DevChain& c, int m, double* sh) {
    const DevData& D = c.D;
    const int K = c.K;
    if (record_at(c, m)) {
        double like;
        if (binaryq_at(c, m)) like = c.ctl->lnl;
        else {
            double v = 0;
            for (int j = threadIdx.x; j < c.nlnlp; j += blockDim.x) v += c.lnlp[j];
            like = block_sum(v, sh);
        }
        if (threadIdx.x == 0) {
            if (c.writelnl && c.ctl->nlnl < c.ntrace) c.lnlTrace[c.ctl->nlnl++] = like;
            if (m >= c.nburnin) {
                c.ctl->nr++;
                c.rout[0] += like;
                c.rout[1] += like * like;
                int nf = c.fmodel ? (c.fsame ? 1 : K) : 0;
                int na = c.admix ? (c.diffalpha ? K : 1) : 0;
                int nl = c.difflambda ? K : 1;
                for (int j = 0; j < nl; ++j) c.rout[4 + j] += c.Lambda[j];
                if (c.locpriori) {
                    c.rout[4 + nl] += c.ctl->r;
                    const double* g = c.admix ? c.Alpha : c.Eta;
                    for (int j = 0; j < K; ++j) c.rout[4 + nl + 1 + j] += g[j];
                    const double* gl = c.admix ? c.AlphaLocal : c.Gamma;
                    for (int j = 0; j < K * D.S; ++j) c.rout[4 + nl + 1 + K + j] += gl[j];
                } else if (c.admix)
                    for (int j = 0; j < na; ++j) c.rout[4 + nl + j] += c.Alpha[j];
                for (int j = 0; j < nf; ++j) c.rout[c.rlen - nf + j] += c.F[j];
            }
        }
    }
}

__global__ void k_record(const DevChain* chains) {
    const DevChain& c = chains[blockIdx.z];
    __shared__ double sh[32];
    record_scalars(c, c.ctl->m, sh);
}

// the element-wise part of Record: MiSum += Mi on every recorded sweep,
// FreqM += Freq after burn-in; the last kernel of a sweep also advances m
__global__ void k_accumulate(const DevChain* chains, int advance) {
    const DevChain& c = chains[blockIdx.z];
    const DevData& D = c.D;
    const int m = c.ctl->m;
    if (record_at(c, m)) {
        int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, nt = (int64_t)gridDim.x * blockDim.x;
        for (int64_t j = tid; j < (int64_t)D.N * c.K; j += nt) c.MiSum[j] += c.Mi[j];
        if (m >= c.nburnin)
            for (int64_t j = tid; j < (int64_t)c.K * D.KT; j += nt) c.FreqM[j] += c.Freq[j];
    }
}

__global__ void k_advance(const DevChain* chains) {
    const DevChain& c = chains[blockIdx.z];
    if (threadIdx.x == 0 && blockIdx.x == 0) c.ctl->m++;
}

// Record and the advance of m in one launch (the end of a captured sweep):
// every block adds its share of MiSum / FreqM; the last block to finish
// (after all blocks have read m) does the scalar Record and m += 1.
// With `exact` (the chains of a tensor-core batch), a recorded sweep's
// lnP(D) is formed from the counts: without admixture Record's sum over
// individuals and allele copies of ln p (src/structure.cpp:1902-1938) equals
// the sum over clusters, loci and alleles of Ni x ln p, with Ni the counts of
// the labels just drawn and p the frequencies they were drawn with. Each
// thread adds its products (all <= 0) with a compensated FP32 sum, the
// blocks' sums go to exact[chain][block] and the last block adds them in
// block order in FP64: within about 1e-7 relative. The batch's per-sweep sum
// from the likelihood contraction, whose FP32 accumulation over 10^5 and
// more alleles per split drifts by a few 1e-6 relative, serves the label
// draws only.
__global__ void k_record_sweep(const DevChain* chains, double* exact, const int4* map = nullptr) {
    const VBlock vb = vblock(map);
    const DevChain& c = chains[vb.z];
    if (map && run_over(c)) return;
    const DevData& D = c.D;
    __shared__ double sh[32];
    const int m = c.ctl->m;
    const bool rec = record_at(c, m);
    if (rec) {
        int64_t tid = vb.x * (int64_t)blockDim.x + threadIdx.x, nt = (int64_t)vb.gx * blockDim.x;
        for (int64_t j = tid; j < (int64_t)D.N * c.K; j += nt) c.MiSum[j] += c.Mi[j];
        const bool fm = m >= c.nburnin;
        if (exact) {
            float s = 0.f, cmp = 0.f;
            for (int64_t j = tid; j < (int64_t)c.K * D.KT; j += nt) {
                const float p = c.Freq[j];
                if (fm) c.FreqM[j] += p;
                const int n = c.Ni[j];
                if (n) {
                    const float y = (float)n * ln_freq(p) - cmp, t = s + y;
                    cmp = (t - s) - y;
                    s = t;
                }
            }
            const double bs = block_sum((double)s - (double)cmp, sh);
            if (threadIdx.x == 0) exact[(int64_t)vb.z * vb.gx + vb.x] = bs;
        } else if (fm) {
            for (int64_t j = tid; j < (int64_t)c.K * D.KT; j += nt) c.FreqM[j] += c.Freq[j];
        }
    }
    if (!last_block_done(c.ctl, vb.gx)) return;
    if (rec && exact) {
        const double t = block_sum_partials(exact + (int64_t)vb.z * vb.gx, vb.gx, sh);
        if (threadIdx.x == 0) c.ctl->lnl = t;
        __syncthreads();
    }
    record_scalars(c, m, sh);
    __syncthreads();
    if (threadIdx.x == 0) {
        c.ctl->done = 0;
        c.ctl->m = m + 1;
    }
}

// Arrange (src/structure.cpp:1860-1869)
__global__ void k_arrange(const DevChain* chains, double* ancestry) {
    const DevChain& c = chains[blockIdx.z];
    const DevData& D = c.D;
    const int K = c.K;
    int nr = c.ctl->nr;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < D.N; i += gridDim.x * blockDim.x) {
        double s = 0;
        for (int k = 0; k < K; ++k) s += (double)c.MiSum[(int64_t)i * K + k];
        double inv = 1.0 / (s + K * VP_MIN_FREQ);
        for (int k = 0; k < K; ++k) ancestry[(int64_t)i * K + k] = ((double)c.MiSum[(int64_t)i * K + k] + VP_MIN_FREQ) * inv;
    }
    float finv = (float)(1.0 / nr);
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < (int64_t)K * D.KT; j += (int64_t)gridDim.x * blockDim.x)
        c.FreqM[j] *= finv;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        double inv = 1.0 / nr;
        for (int j = 0; j < c.rlen; ++j) c.rout[j] *= inv;
        c.rout[2] = c.rout[1] - c.rout[0] * c.rout[0];
        c.rout[3] = c.rout[0] - c.rout[2] / 2;
    }
}

// ---------------------------------------------------------------------------
// Output reductions of WriteStructure (src/structure.cpp:293-324) on the mean
// frequencies of a finished run: for every pair j <= k of clusters,
//   G[k][j] = sum over loci of (1 - sum over alleles of p_k p_j)
// in FP64 from exact float x float products (the reference's SumProd /
// SumSquare of float frequencies into double). G[k][k] is the heterozygosity
// sum, so H[k] = G[k][k] / L and D[k][j] = G[k][j] / L - (H[k] + H[j]) / 2.
// grid.x = pair, grid.y = locus chunk; one FP64 partial per (pair, chunk),
// summed in a fixed order by k_divergence_finish.
constexpr int DIV_CHUNKS = 64;
__global__ void __launch_bounds__(256) k_divergence_pairs(const DevChain* chains, double* part) {
    const DevChain& c = chains[0];
    const DevData& D = c.D;
    __shared__ double sh[32];
    int q = blockIdx.x, k = 0;
    while (q > k) { q -= k + 1; ++k; }
    const int j = q;
    const float* pk = c.FreqM + (int64_t)k * D.KT;
    const float* pj = c.FreqM + (int64_t)j * D.KT;
    const int64_t per = (D.L + gridDim.y - 1) / gridDim.y;
    const int64_t l0 = (int64_t)blockIdx.y * per, l1 = min(D.L, l0 + per);
    double acc = 0;
    for (int64_t l = l0 + threadIdx.x; l < l1; l += blockDim.x) {
        const int64_t o = D.off[l];
        const int k2 = D.k[l];
        double sp = 0;
        for (int a = 0; a < k2; ++a) sp += (double)pk[o + a] * (double)pj[o + a];
        acc += 1 - sp;
    }
    const double t = block_sum(acc, sh);
    if (threadIdx.x == 0) part[(int64_t)blockIdx.x * gridDim.y + blockIdx.y] = t;
}
__global__ void k_divergence_finish(const DevChain* chains, const double* part, int nchunks, double* H, double* Dm) {
    const DevChain& c = chains[0];
    const int K = c.K;
    const double L = (double)c.D.L;
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        for (int k = 0; k < K; ++k) {
            const int q = k * (k + 1) / 2 + k;
            double g = 0;
            for (int b = 0; b < nchunks; ++b) g += part[(int64_t)q * nchunks + b];
            H[k] = g / L;
        }
        for (int k = 0; k < K; ++k)
            for (int j = 0; j <= k; ++j) {
                const int q = k * (k + 1) / 2 + j;
                double g = 0;
                for (int b = 0; b < nchunks; ++b) g += part[(int64_t)q * nchunks + b];
                Dm[j * K + k] = Dm[k * K + j] = g / L - (H[k] + H[j]) / 2;
            }
    }
}
// per-locus heterozygosity 1 - sum_a p^2 of every cluster (the diversity table)
__global__ void k_heterozygosity(const DevChain* chains, double* Hl) {
    const DevChain& c = chains[0];
    const DevData& D = c.D;
    const int64_t n = (int64_t)c.K * D.L;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        const int k = (int)(t / D.L);
        const int64_t l = t % D.L;
        const float* p = c.FreqM + (int64_t)k * D.KT + D.off[l];
        double ss = 0;
        for (int a = 0; a < D.k[l]; ++a) ss += (double)p[a] * (double)p[a];
        Hl[t] = 1 - ss;
    }
}

}  // namespace vp
