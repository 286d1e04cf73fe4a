// Tensor-core contraction for the batched no-admixture K-sweep (sm_103a).
//
//   D[m, n] = sum_k A[m, k] * (B0[n, k] + B1[n, k])        (B1 optional)
//
// A, B0, B1 are bf16, K-major (k contiguous) in global memory and are staged
// into shared memory by TMA, bk = 64 or 32 K elements per stage with the
// 128- or 64-byte swizzle (smaller stages keep more of them in flight); one
// thread issues tcgen05.mma (kind::f16, bf16 x bf16 -> f32) into a TMEM
// accumulator of 128 lanes x mt*BN columns; four epilogue warps read it back
// with tcgen05.ld.
// With B1 given, the hi and lo halves of a split-bf16 operand accumulate into
// the same FP32 accumulator.
//
// Warp roles (192 threads): warp 0 TMA producer, warp 1 TMEM allocator and MMA
// issuer, warps 2..5 epilogue (warp w reads TMEM lanes 32*(w%4)..+31).
// Every mbarrier wait is bounded: on time-out the CTA records an error code
// in *err, drains its own copies in flight (bounded), frees its TMEM and
// returns.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace vp {
namespace tc {

constexpr int BM = 128;
constexpr int NTHREADS = 192;
constexpr uint32_t SPIN_LIMIT = 1u << 22;

struct GemmArgs {
    int M, N;               // rows of A / D, columns of D (= rows of B)
    int kblocks;            // K / bk of the whole problem
    int kb_per_split;       // k-blocks handled by one CTA (grid.z splits K)
    int z0;                 // split index of grid.z = 0 (a launch of some of the splits)
    int BN;                 // columns per CTA (multiple of 16, <= 512)
    int piece;              // columns per MMA instruction (<= 256, multiple of 16)
    int nb;                 // 1 or 2 B operands
    int mt;                 // 128-row A tiles per CTA sharing the B tile (1 or 2)
    int stages;
    int bk;                 // K elements per stage (rows of bk * esz bytes: 128 or 64)
    int esz;                // element bytes: 2 bf16 (kind::f16), 1 e4m3 (kind::f8f6f4)
    int mode;               // 0: FP32 partials D[z][m][n]; 1: int32 transpose Dt[n][m] (no split)
    int group_major;        // 1: blockIdx.x is the column group and blockIdx.y the row tile, so the
                            //    groups that share an A tile run side by side and A streams from DRAM once
    float* out_f;           // mode 0: [splits][M][ldo]
    int32_t* out_i;         // mode 1: [N][ldo]
    int64_t ldo;
    int* err;
    int tx_extra;           // diagnostics only: bytes a stage barrier expects beyond what its copies
                            // bring (> 0 makes every stage wait run out: the time-out path under test)
    uint32_t spin_limit;    // polls per bounded wait (0: SPIN_LIMIT)
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
// bounded wait on a phase parity; returns false on time-out
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t limit = SPIN_LIMIT) {
    uint32_t addr = smem_u32(bar);
    for (uint32_t it = 0; it < limit; ++it) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(addr), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(
            smem_u32(dst)),
        "l"(map), "r"(smem_u32(bar)), "r"(x), "r"(y)
        : "memory");
}

// shared-memory matrix descriptor: K-major, rows of `row` bytes (128 or 64)
// with the matching swizzle, 8-row groups 8 rows apart (SBO), sm100
// descriptor version 1
__device__ __forceinline__ uint64_t sw_desc(uint32_t saddr, int row) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFF);
    d |= (uint64_t)1 << 16;                                 // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)((8 * row) >> 4) << 32;                  // stride byte offset
    d |= (uint64_t)1 << 46;                                 // version
    d |= (uint64_t)(row == 128 ? 2 : 4) << 61;              // SWIZZLE_128B or SWIZZLE_64B
    return d;
}

// instruction descriptor (D f32, both operands K-major, M = 128): bits 4-5
// D format (1 = f32), 7-9 A format and 10-12 B format (kind::f16: 1 = bf16;
// kind::f8f6f4: 0 = e4m3), 17-22 N/8, 24-28 M/16

// kind::f8f6f4 (e4m3 x e4m3 -> f32): 32 K elements (32 bytes) per instruction
__device__ __forceinline__ void mma_e4m3(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc));
}
__device__ __forceinline__ void mma_bf16(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc));
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

// dynamic shared memory: [stages][A tiles | B0 tile | B1 tile] (1024-aligned),
// then barriers.
// The tile shape is compile-time: one thread issues every MMA, and with the
// shape fixed each MMA is two descriptor additions and the instruction
// (rebuilding descriptors from runtime sizes made that thread, not the
// tensor core, the limit).
template <int BKT, int ESZ, int MT, int NB, int BNT, int PIECE>
__global__ void __launch_bounds__(NTHREADS, 1)
    k_gemm_bf16(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB0,
                const __grid_constant__ CUtensorMap mapB1, GemmArgs g) {
    constexpr int ROW = BKT * ESZ;    // bytes per K row of a stage
    static_assert((ROW == 64 || ROW == 128) && (ESZ == 1 || ESZ == 2), "stage depth");
    static_assert(BNT % PIECE == 0 && PIECE % 16 == 0 && PIECE <= 256 && MT * BNT <= 512, "tile");
    constexpr uint32_t A_TILE = BM * ROW;
    constexpr uint32_t A_BYTES = A_TILE * MT;
    constexpr uint32_t B_BYTES = BNT * ROW;
    constexpr uint32_t STAGE = A_BYTES + B_BYTES * NB;
    constexpr uint32_t NCOLS = MT * BNT <= 32 ? 32 : MT * BNT <= 64 ? 64 : MT * BNT <= 128 ? 128 : MT * BNT <= 256 ? 256 : 512;
    constexpr uint32_t FMT = ESZ == 2 ? 1u : 0u;   // bf16 / e4m3
    constexpr uint32_t IDESC = (1u << 4) | (FMT << 7) | (FMT << 10) | ((uint32_t)(PIECE >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int stages = g.stages;
    uint64_t* full = (uint64_t*)(smem + (size_t)STAGE * stages);
    uint64_t* empty = full + stages;
    uint64_t* accum = empty + stages;
    uint32_t* tmem_holder = (uint32_t*)(accum + 1);
    int* abort_flag = (int*)(tmem_holder + 1);

    const int m0 = (g.group_major ? blockIdx.y : blockIdx.x) * BM * MT;
    const int n0 = (g.group_major ? blockIdx.x : blockIdx.y) * BNT;
    const int split = blockIdx.z + g.z0;
    const int kb0 = split * g.kb_per_split;
    const int kb1 = min(g.kblocks, kb0 + g.kb_per_split);
    const int nk = kb1 - kb0;

    if (threadIdx.x == 0) {
        for (int s = 0; s < stages; ++s) { mbar_init(&full[s], 1); mbar_init(&empty[s], 1); }
        mbar_init(accum, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_holder)),
                     "r"(NCOLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_holder;

    const uint32_t lim = g.spin_limit ? g.spin_limit : SPIN_LIMIT;
    if (warp == 0) {
        // ---------------- TMA producer ----------------
        if (lane == 0 && nk > 0) {
            int issued = 0;
            for (int it = 0; it < nk; ++it) {
                const int s = it % stages;
                if (it >= stages && !mbar_wait(&empty[s], ((it / stages) & 1) ^ 1, lim)) {
                    atomicExch(g.err, 1);
                    *(volatile int*)abort_flag = 1;
                    break;
                }
                if (*(volatile int*)abort_flag) break;
                unsigned char* st = smem + (size_t)s * STAGE;
                mbar_expect_tx(&full[s], STAGE + g.tx_extra);
                const int kx = (kb0 + it) * BKT;
#pragma unroll
                for (int t = 0; t < MT; ++t) tma_load_2d(st + t * A_TILE, &mapA, &full[s], kx, m0 + t * BM);
#pragma unroll
                for (int b = 0; b < NB; ++b)
#pragma unroll
                    for (int p = 0; p < BNT; p += PIECE)
                        tma_load_2d(st + A_BYTES + b * B_BYTES + p * ROW, b == 0 ? &mapB0 : &mapB1, &full[s], kx,
                                    n0 + p);
                issued = it + 1;
            }
            // drain: every issued stage must have landed before the CTA may exit
            for (int it = (issued > stages ? issued - stages : 0); it < issued; ++it)
                mbar_wait(&full[it % stages], (it / stages) & 1, lim);
        }
    } else if (warp == 1) {
        // ---------------- MMA issuer ----------------
        if (lane == 0 && nk > 0) {
            // descriptor of stage 0 at its first byte; the tiles' offsets are
            // added to the address field in 16-byte units (a shared-memory
            // address below 256 KB never carries out of its 14 bits)
            const uint64_t d0 = sw_desc(smem_u32(smem), ROW);
            for (int it = 0; it < nk; ++it) {
                const int s = it % stages;
                if (!mbar_wait(&full[s], (it / stages) & 1, lim) || *(volatile int*)abort_flag) {
                    atomicExch(g.err, 2);
                    *(volatile int*)abort_flag = 1;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint64_t ds = d0 + (uint64_t)((s * STAGE) >> 4);
                const uint32_t acc0 = it != 0;
                // one MMA consumes 32 bytes of K: 16 bf16 or 32 e4m3
#pragma unroll
                for (int kk = 0; kk < ROW / 32; ++kk)
#pragma unroll
                    for (int t = 0; t < MT; ++t) {
                        const uint64_t ad = ds + (uint64_t)((t * A_TILE + kk * 32) >> 4);
#pragma unroll
                        for (int b = 0; b < NB; ++b)
#pragma unroll
                            for (int p = 0; p < BNT; p += PIECE) {
                                const uint64_t bd = ds + (uint64_t)((A_BYTES + b * B_BYTES + p * ROW + kk * 32) >> 4);
                                if (ESZ == 2) mma_bf16(tmem + (uint32_t)(t * BNT + p), ad, bd, IDESC, (kk | b) ? 1u : acc0);
                                else mma_e4m3(tmem + (uint32_t)(t * BNT + p), ad, bd, IDESC, (kk | b) ? 1u : acc0);
                            }
                    }
                mma_commit(&empty[s]);  // frees the stage once these MMAs have read it
            }
            // also on the error path: the commit arrives only once every MMA this
            // thread issued has finished writing TMEM
            mma_commit(accum);
        }
        if (lane == 0 && nk <= 0)
            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(accum)) : "memory");
    } else {
        // ---------------- epilogue ----------------
        const int q = warp & 3;  // TMEM lane quarter this warp may read
        const bool got = mbar_wait(accum, 0, lim);
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const bool valid = got && !*(volatile int*)abort_flag && nk > 0;
        if (!got) atomicExch(g.err, 3);
#pragma unroll
        for (int t = 0; t < MT; ++t) {
            const int row = m0 + t * BM + q * 32 + lane;
            for (int c0 = 0; c0 < BNT; c0 += 16) {
                float v[16];
                tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(t * BNT + c0), v);
                if (!valid) continue;
                if (g.mode == 0) {
                    if (row < g.M) {
                        float* o = g.out_f + ((int64_t)split * g.M + row) * g.ldo + n0 + c0;
#pragma unroll
                        for (int j = 0; j < 16; ++j)
                            if (n0 + c0 + j < g.N) o[j] = v[j];
                    }
                } else {
                    if (row < g.M)
#pragma unroll
                        for (int j = 0; j < 16; ++j)
                            if (n0 + c0 + j < g.N) g.out_i[(int64_t)(n0 + c0 + j) * g.ldo + row] = __float2int_rn(v[j]);
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 1) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(NCOLS));
    }
}

inline size_t gemm_smem_bytes(int BN, int nb, int stages, int mt, int bk, int esz) {
    size_t st = (size_t)BM * bk * esz * mt + (size_t)BN * bk * esz * nb;
    return st * stages + 1024 /*align slack*/ + 256 /*barriers*/;
}

}  // namespace tc
}  // namespace vp

#include <cuda_bf16.h>
#include "vp_kernels.cuh"

namespace vp {
namespace tc {

// ---- genotype-count operands of the batched K-sweep (biallelic diploid) ----
// C  [Npad][Apad]: C[i][2l+a]  copies of allele a at locus l in individual i (bf16)
// CT [Apad][Npad]: the transpose (alleles x individuals) as e4m3 bytes
// Missing calls and the padding are zero. 0, 1 and 2 are exact in both types.
constexpr uint8_t E4M3_ONE = 0x38, E4M3_TWO = 0x40;
// One CTA = 128 individuals x BUILD_TILES tiles of 64 loci. Per tile the
// 2-bit codes are decoded into shared memory and written as whole 128-byte
// lines of both layouts: CT rows (allele 2l+a, 128 individuals as e4m3
// bytes) and C rows (individual i, 64 loci x 2 alleles as bf16). The grid
// covers [Npad] x [Apad] entirely (padding individuals and loci are written
// as zeros), so the operands need no clearing beforehand. The same pass adds
// the centring constant's share of its loci, B_i += sum over non-missing
// calls of 2 ln pbar_0 + c (ln pbar_1 - ln pbar_0) (c copies of allele 1), per
// thread in FP32; the CTA's sums go to part[blockIdx.y][i] and k_center_sum
// adds them in FP64 in a fixed order.
constexpr int BUILD_TILES = 8;
__global__ void __launch_bounds__(256) k_build_counts(const DevData D, __nv_bfloat16* C, uint8_t* CT, int64_t Apad,
                                                      int64_t Npad, const float* logpbar, float* part) {
    __shared__ __align__(16) uint8_t code[64][128 + 16];   // [locus][individual]; 3 = missing or padding
    const int t = threadIdx.x;
    const int i0 = blockIdx.x * 128;
    const int seg = t & 15;          // C pieces: 8 columns = 4 loci x 2 alleles
    float acc[8];                    // B_i shares of rows (t >> 4) + 16 p
#pragma unroll
    for (int p = 0; p < 8; ++p) acc[p] = 0.f;
    // a tile's 512 packed words, two per thread (j = t, t + 256); the next
    // tile's are loaded while this tile's rows are written
    auto load_words = [&](int64_t lt0, uint32_t* wv) {
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int j = t + 256 * h, ll = j >> 3, w = j & 7;
            const int64_t l = lt0 + ll;
            const int wi = (i0 >> 4) + w;
            wv[h] = (l < D.L && wi < D.Nw) ? D.g2[l * D.Nw + wi] : 0xFFFFFFFFu;
        }
    };
    const int64_t lbase = (int64_t)blockIdx.y * BUILD_TILES * 64;
    uint32_t wcur[2];
    load_words(lbase, wcur);
    for (int tile = 0; tile < BUILD_TILES; ++tile) {
        const int64_t l0 = lbase + (int64_t)tile * 64;
        if (2 * l0 >= Apad) break;
        __syncthreads();
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int j = t + 256 * h, ll = j >> 3, w = j & 7;
            const uint32_t word = wcur[h];
            uint32_t q[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                uint32_t v = 0;
#pragma unroll
                for (int b = 0; b < 4; ++b) {
                    const int bb = u * 4 + b, i = i0 + w * 16 + bb;
                    v |= (i < D.N ? (word >> (2 * bb)) & 3u : 3u) << (8 * b);
                }
                q[u] = v;
            }
            *reinterpret_cast<uint4*>(&code[ll][w * 16]) = make_uint4(q[0], q[1], q[2], q[3]);
        }
        __syncthreads();
        uint32_t wnext[2] = {0xFFFFFFFFu, 0xFFFFFFFFu};
        if (tile + 1 < BUILD_TILES && 2 * (l0 + 64) < Apad) load_words(l0 + 64, wnext);
        // CT rows 2l+a: eight 16-byte pieces per row
        for (int j = t; j < 128 * 8; j += 256) {
            const int ra = j >> 3, pc = j & 7, ll = ra >> 1, a = ra & 1;
            const int64_t row = 2 * (l0 + ll) + a;
            if (row >= Apad) continue;
            const uint4 cw = *reinterpret_cast<const uint4*>(&code[ll][pc * 16]);
            const uint32_t in[4] = {cw.x, cw.y, cw.z, cw.w};
            // code c -> e4m3 copies of allele a: byte permutation tables
            // (allele 1: c; allele 0: 2 - c; missing: 0)
            const uint32_t lut = a ? 0x00403800u : 0x00003840u;
            uint32_t o[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const uint32_t v = in[u];
                const uint32_t sel = (v & 0xFu) | ((v >> 4) & 0xF0u) | ((v >> 8) & 0xF00u) | ((v >> 12) & 0xF000u);
                o[u] = __byte_perm(lut, 0u, sel);
            }
            *reinterpret_cast<uint4*>(CT + row * Npad + i0 + pc * 16) = make_uint4(o[0], o[1], o[2], o[3]);
        }
        // C rows: sixteen 16-byte pieces per row; this thread's column piece
        // is fixed (seg), its rows are (t >> 4) + 16 p
        const int64_t col = 2 * l0 + seg * 8;
        if (col < Apad) {
            float base[4], dif[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int64_t l = l0 + seg * 4 + u;
                const float p0 = l < D.L ? logpbar[2 * l] : 0.f, p1 = l < D.L ? logpbar[2 * l + 1] : 0.f;
                base[u] = 2.f * p0;
                dif[u] = p1 - p0;
            }
#pragma unroll
            for (int p = 0; p < 8; ++p) {
                const int ii = (t >> 4) + 16 * p;
                uint32_t w[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const uint32_t c = code[seg * 4 + u][ii];
                    // bf16 pairs (allele 0 low, allele 1 high) of (2-c, c); missing 0
                    w[u] = c == 0u ? 0x00004000u : c == 1u ? 0x3F803F80u : c == 2u ? 0x40000000u : 0u;
                    if (c != 3u) acc[p] += fmaf((float)c, dif[u], base[u]);
                }
                *reinterpret_cast<uint4*>(C + (int64_t)(i0 + ii) * Apad + col) = make_uint4(w[0], w[1], w[2], w[3]);
            }
        }
        wcur[0] = wnext[0];
        wcur[1] = wnext[1];
    }
    // the 16 column pieces of a row sit in 16 consecutive lanes
#pragma unroll
    for (int p = 0; p < 8; ++p) {
        float v = acc[p];
        for (int o = 8; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        const int i = i0 + (t >> 4) + 16 * p;
        if (seg == 0 && i < D.N) part[(int64_t)blockIdx.y * Npad + i] = v;
    }
}

// per-allele centring constant: ln of the dataset allele frequency (with a
// pseudo-count), and B[i] = sum_a C[i][a] * ln pbar_a, computed once
// one warp per locus: the lanes popcount the bit planes of the locus's
// packed words (codes 1 and 2 count copies of allele 1; 3 is missing or
// padding)
__global__ void k_allele_center(const DevData D, float* logpbar) {
    const int64_t l = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (l >= D.L) return;
    int n1 = 0, miss = 0;
    for (int w = lane; w < D.Nw; w += 32) {
        const uint32_t v = D.g2[l * D.Nw + w];
        const uint32_t lo = v & 0x55555555u, hi = (v >> 1) & 0x55555555u;
        n1 += __popc(lo & ~hi) + 2 * __popc(hi & ~lo);
        miss += __popc(lo & hi);
    }
    for (int o = 16; o > 0; o >>= 1) {
        n1 += __shfl_xor_sync(0xffffffffu, n1, o);
        miss += __shfl_xor_sync(0xffffffffu, miss, o);
    }
    if (lane) return;
    const int64_t t = 2 * ((int64_t)D.Nw * 16 - miss);
    logpbar[2 * l] = logf((float)(t - n1 + 1) / (float)(t + 2));
    logpbar[2 * l + 1] = logf((float)(n1 + 1) / (float)(t + 2));
}
// B[i] = sum_a C[i][a] ln pbar_a: the locus groups' FP32 shares written by
// k_build_counts, added in FP64 in group order (deterministic)
__global__ void k_center_sum(const DevData D, const float* part, int groups, int64_t Npad, double* Bc) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= D.N) return;
    double t = 0.0;
    for (int r = 0; r < groups; ++r) t += (double)part[(int64_t)r * Npad + i];
    Bc[i] = t;
}

struct BatchDev {
    const DevChain* chains;   // [nchains]
    const int32_t* rowchain;  // [R] chain of each cluster row
    const int32_t* rowk;      // [R] cluster index within its chain
    const int32_t* row0;      // [nchains] first row of each chain
    int R, Rpad, nchains, splits;
    int64_t Apad, Npad;
    __nv_bfloat16 *Whi, *Wlo;
    uint8_t* OH;              // [Rpad][Npad] one-hot labels, e4m3
    const float* logpbar;
    const double* Bc;
    const float* LLpart;      // [splits][N][Rpad]
    const int4* sgrp;         // chain groups of the label draw: {first chain, end chain, first row, rows}
    int sgrp_ld;              // shared-memory words per individual of a group's row sums
};

// UpdateP for every chain of the batch (counter streams, the same Philox
// counters as the per-chain kernel): p ~ Dirichlet(lambda + Ni), written to
// Freq and, centred and split into bf16 hi + lo, to the rows of W.
// grid.y = cluster row; a thread walks loci with a stride of the grid's
// width, so the chain's parameters are fetched once per thread, not per locus.
// Biallelic data: allele offsets are 2l. Loci [l0, l1): the sweep runs the
// step over allele ranges, each range's draws ahead of that range's slice of
// the likelihood contraction; every locus draws from its own counter, so the
// ranges give the values of one launch over all loci.
__global__ void __launch_bounds__(256) k_update_p_tc(BatchDev b, int64_t l0, int64_t l1) {
    const int r = blockIdx.y;
    const DevChain& c = b.chains[b.rowchain[r]];
    const int64_t L = c.D.L;
    const int k = b.rowk[r], m = c.ctl->m;
    const uint64_t seed = c.seed;
    const float lam = (float)c.Lambda[k];
    const int32_t* Ni = c.Ni + (int64_t)k * c.D.KT;
    float* Freq = c.Freq + (int64_t)k * c.D.KT;
    __nv_bfloat162* Whi = reinterpret_cast<__nv_bfloat162*>(b.Whi + (int64_t)r * b.Apad);
    __nv_bfloat162* Wlo = reinterpret_cast<__nv_bfloat162*>(b.Wlo + (int64_t)r * b.Apad);
    const float2* lpb = reinterpret_cast<const float2*>(b.logpbar);
    const int2* Ni2 = reinterpret_cast<const int2*>(Ni);
    float2* F2 = reinterpret_cast<float2*>(Freq);
    l1 = min(l1, L);
    for (int64_t l = l0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < l1; l += (int64_t)gridDim.x * blockDim.x) {
        const int64_t kl = (int64_t)k * L + l;
        Philox ph;
        ph.init(seed, ST_P | ((uint32_t)m << 4), (uint32_t)kl, (uint32_t)(kl >> 32));
        const int2 n = Ni2[l];
        float p0, p1;
        ph.dirichlet2(lam + (float)n.x, lam + (float)n.y, p0, p1);
        F2[l] = make_float2(p0, p1);
        const float2 lb = lpb[l];
        const float w0 = ln_freq_fast(p0) - lb.x, w1 = ln_freq_fast(p1) - lb.y;
        const __nv_bfloat16 h0 = __float2bfloat16(w0), h1 = __float2bfloat16(w1);
        Whi[l] = __halves2bfloat162(h0, h1);
        Wlo[l] = __halves2bfloat162(__float2bfloat16(w0 - __bfloat162float(h0)), __float2bfloat16(w1 - __bfloat162float(h1)));
    }
}

// one-hot rows of every chain's current labels (the initial counts of a
// batch: the count contraction of these rows is the no-admixture UpdateZ)
__global__ void k_onehot_from_z(BatchDev b) {
    const int ci = blockIdx.y;
    const DevChain& c = b.chains[ci];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.D.N) return;
    const int r0 = b.row0[ci], z = c.Z[i];
    for (int k = 0; k < c.K; ++k) b.OH[(int64_t)(r0 + k) * b.Npad + i] = k == z ? E4M3_ONE : 0;
}

// One (chain, individual). The split-K partials sum (`sums`, the chain's K
// values), in FP32, to the centred log-likelihood; the individual's constant
// B_i cancels from the label weights exp(LL_k - max), so the draw runs in
// FP32 on the centred sums (the GEMM accumulated them in FP32; a float
// uniform) and only LL itself, B_i + the centred sum, is formed in FP64.
// K <= KM with the values in registers; larger K goes through a separate
// (not inlined) copy with local arrays, so it does not raise the kernel's
// registers.
template <int KM, bool WIDE>
__device__ __forceinline__ double sample_tc_body(const BatchDev& b, const DevChain& c, int i, int m, int r0,
                                                 const float* sums) {
    const DevData& D = c.D;
    const int K = c.K;
    constexpr int UNR = WIDE ? 1 : KM;   // the wide copy keeps its loops rolled (arrays in local memory)
    float sf[KM];
    const double bc = b.Bc[i];
#pragma unroll UNR
    for (int k = 0; k < KM; ++k) {
        if (k >= K) break;
        const float v = sums[k];
        sf[k] = v;
        c.LL[(int64_t)i * K + k] = bc + (double)v;
    }
    int z = -1;
    double lnl = 0;
    if (D.vt[i]) {
        float mx = -3.402823466e+38f;
#pragma unroll UNR
        for (int k = 0; k < KM; ++k)
            if (k < K && !(sf[k] < mx)) mx = sf[k];
        float s = (float)(VP_MIN_FREQ * K);
#pragma unroll UNR
        for (int k = 0; k < KM; ++k)
            if (k < K) s += sf[k] - mx < -23.f ? (float)VP_MIN_FREQ : __expf(sf[k] - mx);
        Philox ph;
        ph.init(c.seed, ST_Q | ((uint32_t)m << 4), (uint32_t)i, 0);
        float t = ph.uniformf() * s;
        z = K - 1;
        bool found = false;
#pragma unroll UNR
        for (int k = 0; k < KM; ++k) {
            if (k < K && !found) {
                const float w = sf[k] - mx < -23.f ? (float)VP_MIN_FREQ : __expf(sf[k] - mx);
                if (t < w) { z = k; found = true; }
                else t -= w;
            }
        }
        float vz = 0.f;
#pragma unroll UNR
        for (int k = 0; k < KM; ++k)
            if (k == z) vz = sf[k];
        lnl = bc + (double)vz;
        c.Z[i] = (uint16_t)z;
    }
    const int vt = (int)D.vt[i];
#pragma unroll UNR
    for (int k = 0; k < KM; ++k) {
        if (k >= K) break;
        c.Q[(int64_t)i * K + k] = k == z ? 1.f : 0.f;
        c.Mi[(int64_t)i * K + k] = k == z ? vt : 0;
        b.OH[(int64_t)(r0 + k) * b.Npad + i] = k == z ? E4M3_ONE : 0;
    }
    return lnl;
}

__device__ __noinline__ double sample_tc_wide(const BatchDev& b, const DevChain& c, int i, int m, int r0,
                                              const float* sums) {
    return sample_tc_body<64, true>(b, c, i, m, r0, sums);
}

// Label draw for every (chain, individual) from the tensor-core likelihoods;
// also writes the one-hot label rows OH that the count contraction reads.
// A block takes TS_TILE individuals and one group of consecutive chains (grid.y; at most a few hundred cluster rows), so a
// c3 batch of 10,000 individuals and 100 chains runs about 1,250 blocks.
// The split-K partials of the group's rows are read as row segments
// (consecutive threads, consecutive rows; two in flight per thread) and
// summed in split order into shared memory, [individual][sgrp_ld] words (an
// odd stride: no bank conflicts); then warp w draws the labels of the
// group's chains w, w + 8, ... with lane = individual. Each chain's lnL
// partial of the tile goes to lnlp[tile]; the warp that writes a chain's
// last partial folds that chain's partials.
constexpr int TS_TILE = 32, TS_THREADS = 256;
__global__ void __launch_bounds__(TS_THREADS) k_sample_tc_tiles(BatchDev b) {
    extern __shared__ float rs[];
    const int4 gr = b.sgrp[blockIdx.y];
    const int N = b.chains[0].D.N;
    const int i0 = blockIdx.x * TS_TILE, ni = min(TS_TILE, N - i0);
    const int nr = gr.w, ld = b.sgrp_ld, tot = ni * nr;
    const int64_t plane = (int64_t)N * b.Rpad;
    const float* base = b.LLpart + (int64_t)i0 * b.Rpad + gr.z;
    for (int j = threadIdx.x; j < tot; j += 2 * TS_THREADS) {
        const int j2 = min(j + TS_THREADS, tot - 1);    // the last element again when past the end
        const int ia = j / nr, ra = j - ia * nr, ib = j2 / nr, rb = j2 - ib * nr;
        const float* pa = base + (int64_t)ia * b.Rpad + ra;
        const float* pb = base + (int64_t)ib * b.Rpad + rb;
        float va = 0.f, vb = 0.f;
#pragma unroll 4
        for (int s = 0; s < b.splits; ++s) {
            va += pa[s * plane];
            vb += pb[s * plane];
        }
        rs[ia * ld + ra] = va;
        rs[ib * ld + rb] = vb;
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int ci = gr.x + warp; ci < gr.y; ci += TS_THREADS / 32) {
        const DevChain& c = b.chains[ci];
        const int r0 = b.row0[ci], m = c.ctl->m;
        double lnl = 0;
        if (lane < ni) {
            const float* sums = rs + lane * ld + (r0 - gr.z);
            lnl = c.K <= 16 ? sample_tc_body<16, false>(b, c, i0 + lane, m, r0, sums)
                            : sample_tc_wide(b, c, i0 + lane, m, r0, sums);
        }
        for (int o = 16; o > 0; o >>= 1) lnl += __shfl_xor_sync(0xffffffffu, lnl, o);
        int last = 0;
        if (lane == 0) {
            c.lnlp[blockIdx.x] = lnl;
            __threadfence();
            last = atomicAdd(&c.ctl->done, 1) == (int)gridDim.x - 1;
        }
        if (__shfl_sync(0xffffffffu, last, 0)) {
            __threadfence();
            double t = 0;
            for (int j = lane; j < (int)gridDim.x; j += 32) t += __ldcg(c.lnlp + j);
            for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
            if (lane == 0) {
                c.ctl->lnl = t;
                c.ctl->done = 0;
            }
        }
    }
}

}  // namespace tc
}  // namespace vp
