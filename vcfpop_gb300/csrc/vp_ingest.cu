// VCF genotype ingest on the device: the data lines of a VCF (the text after
// the #CHROM header line) become the 2-bit packed genotype matrix of a
// biallelic diploid dataset, the store the STRUCTURE sweep reads.
//
// The reference reads VCF line by line on the host (LoadVCF / AddVCFGenotype,
// src/load.cpp; GENO_WRITER packs the genotype ids). Here the text is uploaded
// once and parsed in parallel:
//   0. upload: through two pinned staging buffers, the host copy of one
//      overlapping the DMA of the other;
//   1. line index: one warp per 4 KB chunk (coalesced 16-byte loads) counts
//      its line feeds, an exclusive scan of the counts, then the warp writes
//      the start offsets of its lines in order;
//   2. one CTA per line: the threads split the line's bytes, a block scan
//      numbers the tabs, the tab before field 5 (ALT) gives the allele count,
//      the FORMAT field must start with GT, and the owner of the tab before
//      each sample field decodes its call ("a/b" or "a|b", a and b in {0, 1,
//      .}, ending at ':', tab or end of line) into a shared-memory row of
//      packed words, written out coalesced.
// A line outside this fast path (not two alleles, a call that is not diploid
// 0/1, GT not the first FORMAT key, a wrong field count) is reported with its
// line number; the caller then uses a general reader.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "vp_callfilter.h"
#include "vp_internal.h"

namespace {

constexpr int CHUNK = 4096;
constexpr int PB = 256;  // threads per line CTA

#define CKI(call)                                                                 \
    do {                                                                          \
        cudaError_t e_ = (call);                                                  \
        if (e_ != cudaSuccess) {                                                  \
            vp_set_error("%s failed: %s", #call, cudaGetErrorString(e_));         \
            return VP_E_CUDA;                                                     \
        }                                                                         \
    } while (0)

// line feeds among the 16 bytes at p (bytes at or past n do not count)
__device__ __forceinline__ uint32_t lf_mask16(const char* t, int64_t p, int64_t n) {
    uint32_t m = 0;
    if (p + 16 <= n) {
        const uint4 v = *reinterpret_cast<const uint4*>(t + p);
        const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const uint32_t eq = __vcmpeq4(w[j], 0x0A0A0A0Au);   // 0xFF per matching byte
#pragma unroll
            for (int b = 0; b < 4; ++b) m |= ((eq >> (8 * b)) & 1u) << (4 * j + b);
        }
    } else {
        for (int j = 0; j < 16 && p + j < n; ++j) m |= (uint32_t)(t[p + j] == '\n') << j;
    }
    return m;
}

// one warp per chunk of CHUNK bytes: lane L reads 16 bytes at 16 * (32 * it + L)
__global__ void k_count_lf(const char* t, int64_t n, int64_t nchunks, int64_t* cnt) {
    const int64_t c = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (c >= nchunks) return;
    const int64_t s = c * CHUNK;
    int k = 0;
    for (int it = 0; it < CHUNK / 512; ++it) {
        const int64_t p = s + (int64_t)(it * 32 + lane) * 16;
        if (p < n) k += __popc(lf_mask16(t, p, n));
    }
    for (int o = 16; o > 0; o >>= 1) k += __shfl_xor_sync(0xffffffffu, k, o);
    if (lane == 0) cnt[c] = k;
}

// exclusive scan of n counts in one CTA (n up to a few million: chunked)
__global__ void k_scan(int64_t* v, int64_t n) {
    __shared__ int64_t sh[1024];
    __shared__ int64_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int64_t base = 0; base < n; base += 1024) {
        const int64_t i = base + threadIdx.x;
        const int64_t x = i < n ? v[i] : 0;
        sh[threadIdx.x] = x;
        __syncthreads();
        for (int o = 1; o < 1024; o <<= 1) {
            int64_t y = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
            __syncthreads();
            sh[threadIdx.x] += y;
            __syncthreads();
        }
        if (i < n) v[i] = carry + sh[threadIdx.x] - x;
        __syncthreads();
        if (threadIdx.x == 1023) carry += sh[1023];
        __syncthreads();
    }
}

// start offsets of the lines: line 0 at 0, line j + 1 after the j-th line
// feed; the warp of a chunk walks it in 512-byte steps, and a warp prefix
// sum of the lanes' counts puts their line feeds in order
__global__ void k_line_starts(const char* t, int64_t n, int64_t nchunks, const int64_t* pre, int64_t* start) {
    const int64_t c = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (c >= nchunks) return;
    const int64_t s = c * CHUNK;
    int64_t j = pre[c];
    for (int it = 0; it < CHUNK / 512; ++it) {
        const int64_t p = s + (int64_t)(it * 32 + lane) * 16;
        uint32_t m = p < n ? lf_mask16(t, p, n) : 0u;
        const int cntl = __popc(m);
        int incl = cntl;
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        int64_t q = j + incl - cntl;
        while (m) {
            const int b = __ffs(m) - 1;
            m &= m - 1;
            start[++q] = p + b + 1;
        }
        j += __shfl_sync(0xffffffffu, incl, 31);
    }
}

struct LineOut {
    int32_t* bad;     // [L] 0 = ok, else a reason code
    int32_t* nalt;    // [L] ALT alleles
};

// one CTA per line
__global__ void __launch_bounds__(PB) k_parse_lines(const char* t, const int64_t* start, int64_t L, int N, int Nw,
                                                    uint32_t* packed, LineOut out, vp_call_filter cf) {
    extern __shared__ uint32_t row[];   // [Nw]
    __shared__ int warp_tabs[PB / 32];
    __shared__ int err;
    __shared__ int nalt_s, dpid_s, gqid_s;
    __shared__ unsigned long long kept_s;
    const int64_t l = blockIdx.x;
    if (l >= L) return;
    const int64_t s = start[l];
    int64_t e = start[l + 1];
    // trim the line feed (and a carriage return before it)
    if (e > s && t[e - 1] == '\n') --e;
    if (e > s && t[e - 1] == '\r') --e;
    for (int w = threadIdx.x; w < Nw; w += PB) row[w] = 0;
    if (threadIdx.x == 0) { err = 0; nalt_s = 0; dpid_s = -1; gqid_s = -1; kept_s = 0; }
    const int64_t len = e - s;
    const int64_t seg = (len + PB - 1) / PB;
    const int64_t a = s + min(len, (int64_t)threadIdx.x * seg), b = s + min(len, (int64_t)(threadIdx.x + 1) * seg);
    int mine = 0;
    for (int64_t p = a; p < b; ++p) mine += t[p] == '\t';
    // block exclusive scan of the tab counts
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int incl = mine;
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) warp_tabs[warp] = incl;
    __syncthreads();
    int before = 0;
    for (int w = 0; w < warp; ++w) before += warp_tabs[w];
    int total = 0;
    for (int w = 0; w < PB / 32; ++w) total += warp_tabs[w];
    const int f0 = before + incl - mine;   // index of the next tab this thread meets
    if (threadIdx.x == 0 && total != 8 + N) err = 1;   // 9 fixed fields + N samples
    // the fixed fields first (ALT, FORMAT), then the calls
    int f = f0;
    for (int64_t p = a; p < b; ++p) {
        if (t[p] != '\t') continue;
        const int field = f + 1;    // the field that starts after this tab
        ++f;
        const char* q = t + p + 1;
        const int64_t room = e - (p + 1);
        if (field == 4) {          // ALT: alleles = commas + 1
            int commas = 0;
            for (int64_t r = 0; r < room && q[r] != '\t'; ++r) commas += q[r] == ',';
            nalt_s = commas + 1;
        } else if (field == 8) {   // FORMAT must start with GT
            int dp, gq;
            uint64_t kept;
            if (!vp::parse_format(q, room, &dp, &gq, &kept)) err = 2;
            dpid_s = dp;
            gqid_s = gq;
            kept_s = kept;
        }
    }
    __syncthreads();
    const int dpid = dpid_s, gqid = gqid_s;
    const uint64_t kept = kept_s;
    f = f0;
    for (int64_t p = a; p < b; ++p) {
        if (t[p] != '\t') continue;
        const int field = f + 1;
        ++f;
        const char* q = t + p + 1;
        const int64_t room = e - (p + 1);
        if (field >= 9) {
            const int i = field - 9;
            if (i >= N) { err = 1; continue; }
            // "x/y" or "x|y", x, y in {0, 1, .}, then ':' or tab or end of line
            if (room < 3 || (q[1] != '/' && q[1] != '|') || (room > 3 && q[3] != ':' && q[3] != '\t')) { err = 3; continue; }
            const char x = q[0], y = q[2];
            const bool mx = x == '.', my = y == '.';
            if ((!mx && x != '0' && x != '1') || (!my && y != '0' && y != '1')) { err = 3; continue; }
            uint32_t code = (mx || my) ? 3u : (uint32_t)((x - '0') + (y - '0'));
            if (code != 3u && vp::call_filtered(cf, t, p + 1, e, dpid, gqid, kept, 2)) code = 3u;
            atomicOr(&row[i >> 4], code << (2 * (i & 15)));
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int bad = err;
        if (!bad && nalt_s != 1) bad = 4;
        out.bad[l] = bad;
        out.nalt[l] = nalt_s;
    }
    // padding individuals of the last word are missing (3)
    for (int w = threadIdx.x; w < Nw; w += PB) {
        uint32_t v = row[w];
        const int i0 = w * 16;
        for (int j = 0; j < 16; ++j)
            if (i0 + j >= N) v |= 3u << (2 * j);
        packed[l * (int64_t)Nw + w] = v;
    }
}

// One CTA per line, any ploidy and allele count: the call of each sample
// ("a/b/c/..." or with '|', alleles 0..127, '.' for a missing copy, ending at
// ':', tab or end of line) becomes its allele indices in ascending order (the
// reference's unphased genotype, AddVCFGenotype in src/load.cpp), the first
// vmax of them stored, -1 for a missing call or an absent copy; ploidy0 gets
// the copies of each call on the first line (which sets each individual's
// ploidy) and nall[l] the alleles of the locus (REF plus the ALT commas + 1).
__global__ void __launch_bounds__(PB) k_parse_general(const char* t, const int64_t* start, int64_t L, int N, int vmax,
                                                      int8_t* G, int32_t* nall, int32_t* bad, int32_t* ploidy0,
                                                      int64_t line0, vp_call_filter cf) {
    __shared__ int warp_tabs[PB / 32];
    __shared__ int err;
    __shared__ int nall_s, dpid_s, gqid_s;
    __shared__ unsigned long long kept_s;
    const int64_t l = blockIdx.x;
    if (l >= L) return;
    const int64_t s = start[l];
    int64_t e = start[l + 1];
    if (e > s && t[e - 1] == '\n') --e;
    if (e > s && t[e - 1] == '\r') --e;
    if (threadIdx.x == 0) { err = 0; nall_s = 0; dpid_s = -1; gqid_s = -1; kept_s = 0; }
    const int64_t len = e - s;
    const int64_t seg = (len + PB - 1) / PB;
    const int64_t a = s + min(len, (int64_t)threadIdx.x * seg), b = s + min(len, (int64_t)(threadIdx.x + 1) * seg);
    int mine = 0;
    for (int64_t p = a; p < b; ++p) mine += t[p] == '\t';
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int incl = mine;
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) warp_tabs[warp] = incl;
    __syncthreads();
    int before = 0, total = 0;
    for (int w = 0; w < warp; ++w) before += warp_tabs[w];
    for (int w = 0; w < PB / 32; ++w) total += warp_tabs[w];
    const int f0 = before + incl - mine;
    if (threadIdx.x == 0 && total != 8 + N) err = 1;
    // the fixed fields first (ALT, FORMAT), then the calls
    int f = f0;
    for (int64_t p = a; p < b; ++p) {
        if (t[p] != '\t') continue;
        const int field = f + 1;
        ++f;
        const char* q = t + p + 1;
        const int64_t room = e - (p + 1);
        if (field == 4) {
            int commas = 0;
            for (int64_t r = 0; r < room && q[r] != '\t'; ++r) commas += q[r] == ',';
            nall_s = commas + 2;
        } else if (field == 8) {
            int dp, gq;
            uint64_t kept;
            if (!vp::parse_format(q, room, &dp, &gq, &kept)) err = 2;
            dpid_s = dp;
            gqid_s = gq;
            kept_s = kept;
        }
    }
    __syncthreads();
    const int dpid = dpid_s, gqid = gqid_s;
    const uint64_t kept = kept_s;
    f = f0;
    for (int64_t p = a; p < b; ++p) {
        if (t[p] != '\t') continue;
        const int field = f + 1;
        ++f;
        const char* q = t + p + 1;
        const int64_t room = e - (p + 1);
        if (field >= 9) {
            const int i = field - 9;
            if (i >= N) { err = 1; continue; }
            int al[16];
            int n = 0, cur = -1;
            bool miss = false, any = false;
            int64_t r = 0;
            for (; r < room && q[r] != ':' && q[r] != '\t'; ++r) {
                const char ch = q[r];
                if (ch == '/' || ch == '|') {
                    if (!any) miss = true;
                    else if (n < 16) al[n] = cur;
                    ++n;
                    cur = -1;
                    any = false;
                } else if (ch == '.') {
                    miss = true;
                    any = true;
                } else if (ch >= '0' && ch <= '9') {
                    cur = (cur < 0 ? 0 : cur * 10) + (ch - '0');
                    if (cur > 127) { err = 5; cur = 127; }
                    any = true;
                } else {
                    err = 3;
                }
            }
            if (!any) miss = true;
            else if (n < 16) al[n] = cur;
            ++n;
            if (n > 16) { err = 6; n = 16; }
            if (l == 0 && line0 == 0) ploidy0[i] = n;
            int8_t* out = G + ((size_t)l * N + i) * vmax;
            for (int c = 0; c < vmax; ++c) out[c] = -1;
            if (miss || vp::call_filtered(cf, t, p + 1, e, dpid, gqid, kept, n)) continue;
            // ascending order (insertion sort of at most 16)
            for (int x = 1; x < n; ++x) {
                const int v = al[x];
                int y = x - 1;
                while (y >= 0 && al[y] > v) { al[y + 1] = al[y]; --y; }
                al[y + 1] = v;
            }
            for (int c = 0; c < n && c < vmax; ++c) out[c] = (int8_t)al[c];
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        bad[l] = err;
        nall[l] = nall_s;
    }
}

// host text -> device through two pinned staging buffers: the host copy into
// one overlaps the DMA out of the other
int upload_staged(char* dst, const char* src, int64_t n, cudaStream_t st) {
    constexpr size_t STAGE = 32u << 20;
    char* stage[2] = {nullptr, nullptr};
    cudaEvent_t ev[2] = {nullptr, nullptr};
    int rc = VP_OK;
    if (cudaMallocHost((void**)&stage[0], STAGE) != cudaSuccess || cudaMallocHost((void**)&stage[1], STAGE) != cudaSuccess ||
        cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming) != cudaSuccess) {
        vp_set_error("pinned staging buffers for the upload could not be allocated");
        rc = VP_E_MEM;
    }
    int b = 0;
    bool used[2] = {false, false};
    for (int64_t off = 0; !rc && off < n; off += STAGE, b ^= 1) {
        const size_t len = (size_t)std::min<int64_t>(STAGE, n - off);
        if (used[b] && cudaEventSynchronize(ev[b]) != cudaSuccess) { vp_set_error("upload failed"); rc = VP_E_CUDA; break; }
        memcpy(stage[b], src + off, len);
        cudaError_t e = cudaMemcpyAsync(dst + off, stage[b], len, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaEventRecord(ev[b], st);
        if (e != cudaSuccess) { vp_set_error("upload failed: %s", cudaGetErrorString(e)); rc = VP_E_CUDA; break; }
        used[b] = true;
    }
    // the staging buffers are released only after their copies completed
    for (int j = 0; j < 2; ++j)
        if (used[j]) cudaEventSynchronize(ev[j]);
    for (int j = 0; j < 2; ++j) {
        if (ev[j]) cudaEventDestroy(ev[j]);
        if (stage[j]) cudaFreeHost(stage[j]);
    }
    return rc;
}

const char* reason(int code) {
    switch (code) {
        case 1: return "the number of fields is not 9 + the number of samples";
        case 2: return "GT is not the first FORMAT key";
        case 3: return "a call is not a diploid 0/1 genotype";
        case 4: return "the locus does not have exactly 2 alleles";
        case 5: return "an allele index above 127";
        case 6: return "a call with more than 16 copies";
    }
    return "unknown";
}

}  // namespace

namespace {

// the text on the device and the start offsets of its lines (L + 1 entries,
// the last the end of the text); with max_loci <= 0 only *n_loc is set
struct TextIndex {
    char* dt = nullptr;
    int64_t* cnt = nullptr;
    int64_t* starts = nullptr;
    int64_t L = 0;
    void release(cudaStream_t st) {
        if (starts) cudaFreeAsync(starts, st);
        if (cnt) cudaFreeAsync(cnt, st);
        if (dt) cudaFreeAsync(dt, st);
        starts = cnt = nullptr;
        dt = nullptr;
    }
};

int index_text(const char* text, size_t bytes, int64_t max_loci, cudaStream_t st, TextIndex& ix, int64_t* n_loc) {
    const int64_t n = (int64_t)bytes;
    const int64_t nchunks = (n + CHUNK - 1) / CHUNK;
    cudaError_t e;
    if ((e = cudaMallocAsync((void**)&ix.dt, n + 1, st)) != cudaSuccess ||
        (e = cudaMallocAsync((void**)&ix.cnt, (nchunks + 1) * 8, st)) != cudaSuccess) {
        vp_set_error("device allocation for the text failed: %s", cudaGetErrorString(e));
        return VP_E_MEM;
    }
    if (int rc = upload_staged(ix.dt, text, n, st)) return rc;
    const unsigned g = (unsigned)((nchunks * 32 + 255) / 256);
    k_count_lf<<<g, 256, 0, st>>>(ix.dt, n, nchunks, ix.cnt);
    cudaMemsetAsync(ix.cnt + nchunks, 0, 8, st);
    k_scan<<<1, 1024, 0, st>>>(ix.cnt, nchunks + 1);
    int64_t nlf = 0;
    if ((e = cudaMemcpyAsync(&nlf, ix.cnt + nchunks, 8, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (e = cudaStreamSynchronize(st)) != cudaSuccess) {
        vp_set_error("line index failed: %s", cudaGetErrorString(e));
        return VP_E_CUDA;
    }
    // a last line without a line feed counts too
    const bool tail = n > 0 && text[n - 1] != '\n';
    ix.L = nlf + (tail ? 1 : 0);
    *n_loc = ix.L;
    if (max_loci <= 0 || ix.L == 0) return VP_OK;
    if (ix.L > max_loci) { vp_set_error("%lld loci, buffer holds %lld", (long long)ix.L, (long long)max_loci); return VP_E_ARG; }
    if ((e = cudaMallocAsync((void**)&ix.starts, (nlf + 2) * 8, st)) != cudaSuccess) {
        vp_set_error("device allocation failed: %s", cudaGetErrorString(e));
        return VP_E_MEM;
    }
    cudaMemsetAsync(ix.starts, 0, 8, st);
    k_line_starts<<<g, 256, 0, st>>>(ix.dt, n, nchunks, ix.cnt, ix.starts);
    // the end of the last line (the host value must outlive the copy)
    static thread_local int64_t endv;
    endv = n;
    if ((e = cudaMemcpyAsync(ix.starts + ix.L, &endv, 8, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
        (e = cudaStreamSynchronize(st)) != cudaSuccess) {
        vp_set_error("line index failed: %s", cudaGetErrorString(e));
        return VP_E_CUDA;
    }
    return VP_OK;
}

int open_device(int device, cudaStream_t* st) {
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) { vp_set_error("no CUDA device"); return VP_E_NODEV; }
    if (device < 0 || device >= ndev) { vp_set_error("device %d out of range", device); return VP_E_ARG; }
    CKI(cudaSetDevice(device));
    CKI(cudaStreamCreateWithFlags(st, cudaStreamNonBlocking));
    return VP_OK;
}

}  // namespace

extern "C" int vp_vcf_pack2(const char* text, size_t bytes, int32_t n_ind, int device, uint32_t* packed,
                            int64_t max_loci, int64_t* line_start, int64_t* n_loc) {
    return vp_vcf_pack2_ex(text, bytes, n_ind, device, packed, max_loci, line_start, n_loc, nullptr);
}

extern "C" int vp_vcf_pack2_ex(const char* text, size_t bytes, int32_t n_ind, int device, uint32_t* packed,
                               int64_t max_loci, int64_t* line_start, int64_t* n_loc, const vp_call_filter* cf) {
    const vp_call_filter none{};
    if (!cf) cf = &none;
    if (!text || !n_loc || n_ind <= 0 || (max_loci > 0 && !packed)) { vp_set_error("bad arguments"); return VP_E_ARG; }
    const int Nw = (n_ind + 15) / 16;
    if ((size_t)Nw * 4 > 200 * 1024) { vp_set_error("too many samples for one line row in shared memory"); return VP_E_ARG; }
    cudaStream_t st;
    if (int rc0 = open_device(device, &st)) return rc0;
    TextIndex ix;
    int rc = VP_OK;
    do {
        if ((rc = index_text(text, bytes, max_loci, st, ix, n_loc))) break;
        const int64_t L = ix.L;
        if (max_loci <= 0 || L == 0) break;                       // size query
        cudaError_t e;
        uint32_t* dp = nullptr;
        int32_t* flags = nullptr;
        if ((e = cudaMallocAsync((void**)&dp, (size_t)L * Nw * 4, st)) != cudaSuccess ||
            (e = cudaMallocAsync((void**)&flags, (size_t)L * 8, st)) != cudaSuccess) {
            vp_set_error("device allocation failed: %s", cudaGetErrorString(e));
            rc = VP_E_MEM;
            if (dp) cudaFreeAsync(dp, st);
            break;
        }
        for (int64_t l0 = 0; l0 < L; l0 += 1 << 30) {
            const unsigned nb = (unsigned)std::min<int64_t>(L - l0, 1 << 30);
            k_parse_lines<<<nb, PB, (size_t)Nw * 4, st>>>(ix.dt, ix.starts + l0, nb, n_ind, Nw, dp + l0 * Nw,
                                                          LineOut{flags + l0, flags + L + l0}, *cf);
        }
        if ((e = cudaGetLastError()) != cudaSuccess) {
            vp_set_error("parse launch failed: %s", cudaGetErrorString(e));
            rc = VP_E_CUDA;
        }
        std::vector<int32_t> hb(L);
        if (!rc && ((e = cudaMemcpyAsync(packed, dp, (size_t)L * Nw * 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
                    (e = cudaMemcpyAsync(hb.data(), flags, (size_t)L * 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
                    (line_start && (e = cudaMemcpyAsync(line_start, ix.starts, (size_t)(L + 1) * 8, cudaMemcpyDeviceToHost,
                                                        st)) != cudaSuccess))) {
            vp_set_error("copy-out failed: %s", cudaGetErrorString(e));
            rc = VP_E_CUDA;
        }
        cudaFreeAsync(dp, st);
        cudaFreeAsync(flags, st);
        if (!rc && (e = cudaStreamSynchronize(st)) != cudaSuccess) {
            vp_set_error("parse failed: %s", cudaGetErrorString(e));
            rc = VP_E_CUDA;
        }
        if (!rc)
            for (int64_t l = 0; l < L; ++l)
                if (hb[l]) {
                    vp_set_error("data line %lld: %s", (long long)(l + 1), reason(hb[l]));
                    rc = VP_E_ARG;
                    break;
                }
    } while (0);
    ix.release(st);
    cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
    return rc;
}

extern "C" int vp_vcf_parse(const char* text, size_t bytes, int32_t n_ind, int32_t vmax, int device, int8_t* alleles,
                            int32_t* n_alleles, int32_t* ploidy, int64_t max_loci, int64_t* line_start, int64_t* n_loc) {
    return vp_vcf_parse_ex(text, bytes, n_ind, vmax, device, alleles, n_alleles, ploidy, max_loci, line_start, n_loc,
                           nullptr);
}

extern "C" int vp_vcf_parse_ex(const char* text, size_t bytes, int32_t n_ind, int32_t vmax, int device, int8_t* alleles,
                               int32_t* n_alleles, int32_t* ploidy, int64_t max_loci, int64_t* line_start,
                               int64_t* n_loc, const vp_call_filter* cf) {
    const vp_call_filter none{};
    if (!cf) cf = &none;
    if (!text || !n_loc || n_ind <= 0 || vmax < 1 || vmax > 16 ||
        (max_loci > 0 && (!alleles || !n_alleles || !ploidy))) {
        vp_set_error("bad arguments");
        return VP_E_ARG;
    }
    cudaStream_t st;
    if (int rc0 = open_device(device, &st)) return rc0;
    TextIndex ix;
    int rc = VP_OK;
    int8_t* dG = nullptr;
    int32_t* flags = nullptr;
    do {
        if ((rc = index_text(text, bytes, max_loci, st, ix, n_loc))) break;
        const int64_t L = ix.L;
        if (max_loci <= 0 || L == 0) break;
        cudaError_t e;
        const size_t gb = (size_t)L * n_ind * vmax;
        if ((e = cudaMallocAsync((void**)&dG, gb, st)) != cudaSuccess ||
            (e = cudaMallocAsync((void**)&flags, (size_t)L * 8 + (size_t)n_ind * 4, st)) != cudaSuccess) {
            vp_set_error("device allocation failed: %s", cudaGetErrorString(e));
            rc = VP_E_MEM;
            break;
        }
        int32_t* dnall = flags + L;
        int32_t* dploidy = flags + 2 * L;
        cudaMemsetAsync(dploidy, 0, (size_t)n_ind * 4, st);
        for (int64_t l0 = 0; l0 < L; l0 += 1 << 30) {
            const unsigned nb = (unsigned)std::min<int64_t>(L - l0, 1 << 30);
            k_parse_general<<<nb, PB, 0, st>>>(ix.dt, ix.starts + l0, nb, n_ind, vmax, dG + (size_t)l0 * n_ind * vmax,
                                               dnall + l0, flags + l0, dploidy, l0, *cf);
        }
        if ((e = cudaGetLastError()) != cudaSuccess) {
            vp_set_error("parse launch failed: %s", cudaGetErrorString(e));
            rc = VP_E_CUDA;
            break;
        }
        std::vector<int32_t> hb(L);
        if ((e = cudaMemcpyAsync(alleles, dG, gb, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
            (e = cudaMemcpyAsync(n_alleles, dnall, (size_t)L * 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
            (e = cudaMemcpyAsync(ploidy, dploidy, (size_t)n_ind * 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
            (e = cudaMemcpyAsync(hb.data(), flags, (size_t)L * 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
            (line_start && (e = cudaMemcpyAsync(line_start, ix.starts, (size_t)(L + 1) * 8, cudaMemcpyDeviceToHost,
                                                st)) != cudaSuccess) ||
            (e = cudaStreamSynchronize(st)) != cudaSuccess) {
            vp_set_error("parse failed: %s", cudaGetErrorString(e));
            rc = VP_E_CUDA;
            break;
        }
        for (int64_t l = 0; l < L; ++l)
            if (hb[l]) {
                vp_set_error("data line %lld: %s", (long long)(l + 1), reason(hb[l]));
                rc = VP_E_ARG;
                break;
            }
    } while (0);
    if (dG) cudaFreeAsync(dG, st);
    if (flags) cudaFreeAsync(flags, st);
    ix.release(st);
    cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
    return rc;
}

// ---------------------------------------------------------------------------
// Locus filter on the packed matrix. One warp per locus: the lanes count the
// four 2-bit codes of their words (popcounts of the low and high bit planes),
// lane 0 derives the reference's statistics for a biallelic diploid locus
// (counts c0 = 0/0, c1 = 0/1, c2 = 1/1):
//   n = c0 + c1 + c2, nhaplo = 2n, allele counts 2c0 + c1 and c1 + 2c2,
//   frequencies as Unify gives them ((count + 1e-10) / (2n + 2e-10)),
//   k = alleles above 1e-10, ptype = n / N, and for k = 2: bmaf, he = 1 - a2,
//   ho = c1 / n (HIndex 1 for a heterozygote), pic, ae = 1 / a2, I.
namespace {
__device__ __forceinline__ float rlog(float x) { return logf(x); }
__device__ __forceinline__ double rlog(double x) { return log(x); }

// CalcDiversity's statistics for one biallelic diploid locus in the
// reference's REAL (float under -g_float=single): allele counts in REAL,
// Unify in double stored in REAL, CountK above 1e-10, then the statistics
template <typename REAL>
__device__ void locus_stats(int c0, int c1, int c2, int N, int& k, double& ptype, double& bmaf, double& he, double& ho,
                            double& pic, double& ae, double& I, double& pval) {
    const double nan = __longlong_as_double(0x7ff8000000000000ll);
    const int n = c0 + c1 + c2;
    ptype = (double)((REAL)n / (REAL)N);
    k = 0;
    bmaf = he = ho = pic = ae = I = pval = nan;
    if (n == 0) return;
    REAL fre[2] = {(REAL)(2 * c0 + c1), (REAL)(c1 + 2 * c2)};
    const double invsum = 1.0 / ((double)fre[0] + (double)fre[1] + 2 * 1e-10);
    fre[0] = (REAL)(((double)fre[0] + 1e-10) * invsum);
    fre[1] = (REAL)(((double)fre[1] + 1e-10) * invsum);
    k = (fre[0] > 1e-10) + (fre[1] > 1e-10);
    if (k < 2) return;
    const REAL hoR = (REAL)(2.0 * c1) / (REAL)(2.0 * n);
    const int nh = 2 * n;
    REAL Iv = 0, b = 1, a2 = 0, picv = 0;
    for (int a = 0; a < 2; ++a) {
        const REAL af = fre[a];
        if (af * nh < 1e-5) continue;
        if (af > 1e-5) Iv += -af * rlog(af);
        if (b > af) b = af;
        a2 += af * af;
        if (a == 0 && fre[1] > 0) picv += 2 * af * fre[1] * (1 - af * fre[1]);
    }
    if (b > 0.5) b = 1 - b;
    bmaf = b;
    he = (REAL)(1 - a2);
    ho = hoR;
    pic = picv;
    ae = (REAL)(1 / a2);
    I = Iv;
    // HWE G-test (src/diversity.cpp:337-492): the expected count of each
    // observed genotype, GFZ x n (HWE coefficient x frequencies in double,
    // stored in REAL); an expectation below 5 collapses the two alleles into
    // one and leaves no test (NaN). With two alleles df = 1, and the p-value
    // is 1 - the chi-square CDF, 1 - erf(sqrt(G / 2)).
    const int gc[3] = {c0, c1, c2};
    REAL G = 0;
    for (int g = 0; g < 3; ++g) {
        if (!gc[g]) continue;
        const double gf = g == 1 ? 2.0 * (double)fre[1] * (double)fre[0] : (double)fre[g >> 1] * (double)fre[g >> 1];
        const REAL obs = (REAL)gc[g], ex = (REAL)(gf * n);
        if (ex < 5) return;
        G += 2 * obs * rlog(obs / ex);
    }
    pval = (REAL)(1.0 - erf(sqrt(0.5 * (double)G)));
}

__device__ __forceinline__ bool outside(double v, double lo, double hi) { return v < lo || v > hi; }

__global__ void k_locus_filter(const uint32_t* packed, int64_t L, int N, int Nw, vp_locus_filter f, uint8_t* keep,
                               double* stats) {
    const int64_t l = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (l >= L) return;
    const uint32_t* row = packed + l * Nw;
    int c1 = 0, c2 = 0, c3 = 0;
    for (int w = lane; w < Nw; w += 32) {
        const uint32_t v = row[w];
        const uint32_t lo = v & 0x55555555u, hi = (v >> 1) & 0x55555555u;
        c1 += __popc(lo & ~hi);
        c2 += __popc(hi & ~lo);
        c3 += __popc(lo & hi);
    }
    for (int o = 16; o > 0; o >>= 1) {
        c1 += __shfl_xor_sync(0xffffffffu, c1, o);
        c2 += __shfl_xor_sync(0xffffffffu, c2, o);
        c3 += __shfl_xor_sync(0xffffffffu, c3, o);
    }
    if (lane) return;
    const int c0 = Nw * 16 - c1 - c2 - c3;  // padding calls are coded missing (3)
    const int n = c0 + c1 + c2;
    double ptype, bmaf, he, ho, pic, ae, I, pval;
    int k;
    if (f.single) locus_stats<float>(c0, c1, c2, N, k, ptype, bmaf, he, ho, pic, ae, I, pval);
    else locus_stats<double>(c0, c1, c2, N, k, ptype, bmaf, he, ho, pic, ae, I, pval);
    const bool fail = k == 0 || (f.bmaf_b && k == 2 && outside(bmaf, f.bmaf_min, f.bmaf_max)) ||
                      (f.k_b && (k < f.k_min || k > f.k_max)) || (f.n_b && (n < f.n_min || n > f.n_max)) ||
                      (f.ptype_b && outside(ptype, f.ptype_min, f.ptype_max)) ||
                      (f.he_b && outside(he, f.he_min, f.he_max)) || (f.ho_b && outside(ho, f.ho_min, f.ho_max)) ||
                      (f.pic_b && outside(pic, f.pic_min, f.pic_max)) || (f.ae_b && outside(ae, f.ae_min, f.ae_max)) ||
                      (f.I_b && outside(I, f.I_min, f.I_max)) ||
                      (f.pval_b && pval != -1 && outside(pval, f.pval_min, f.pval_max));
    keep[l] = fail ? 0 : 1;
    if (stats) {
        double* o = stats + l * VP_LOCUS_STATS;
        o[0] = n; o[1] = k; o[2] = ptype; o[3] = bmaf; o[4] = he; o[5] = ho; o[6] = pic; o[7] = ae; o[8] = I;
        o[9] = pval;
    }
}
}  // namespace

extern "C" int vp_locus_filter_pack2(const uint32_t* packed, int64_t n_loc, int32_t n_ind, const vp_locus_filter* f,
                                     int device, uint8_t* keep, double* stats) {
    if (!packed || !f || !keep || n_loc < 0 || n_ind <= 0) { vp_set_error("bad arguments"); return VP_E_ARG; }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) { vp_set_error("no CUDA device"); return VP_E_NODEV; }
    if (device < 0 || device >= ndev) { vp_set_error("device %d out of range", device); return VP_E_ARG; }
    if (n_loc == 0) return VP_OK;
    CKI(cudaSetDevice(device));
    const int Nw = (n_ind + 15) / 16;
    cudaStream_t st;
    CKI(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    const size_t pb = (size_t)n_loc * Nw * 4, sb = stats ? (size_t)n_loc * VP_LOCUS_STATS * 8 : 0;
    char* buf = nullptr;
    int rc = VP_OK;
    cudaError_t e = cudaMallocAsync((void**)&buf, pb + 256 + (size_t)n_loc + 256 + sb, st);
    if (e != cudaSuccess) { vp_set_error("device allocation failed: %s", cudaGetErrorString(e)); rc = VP_E_MEM; }
    if (!rc) {
        uint32_t* dp = (uint32_t*)buf;
        uint8_t* dk = (uint8_t*)(buf + (pb + 255) / 256 * 256);
        double* ds = stats ? (double*)(buf + (pb + 255) / 256 * 256 + ((size_t)n_loc + 255) / 256 * 256) : nullptr;
        rc = upload_staged((char*)dp, (const char*)packed, (int64_t)pb, st);
        if (!rc) {
            k_locus_filter<<<(unsigned)((n_loc * 32 + 255) / 256), 256, 0, st>>>(dp, n_loc, n_ind, Nw, *f, dk, ds);
            if ((e = cudaGetLastError()) != cudaSuccess ||
                (e = cudaMemcpyAsync(keep, dk, (size_t)n_loc, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
                (ds && (e = cudaMemcpyAsync(stats, ds, sb, cudaMemcpyDeviceToHost, st)) != cudaSuccess) ||
                (e = cudaStreamSynchronize(st)) != cudaSuccess) {
                vp_set_error("locus filter failed: %s", cudaGetErrorString(e));
                rc = VP_E_CUDA;
            }
        }
        cudaFreeAsync(buf, st);
    }
    cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
    return rc;
}
