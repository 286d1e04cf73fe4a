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

// ---------------------------------------------------------------------------
// Locus statistics of any ploidy and allele count (the general genotype
// layout G[L][N][vmax], allele indices 0..63, up to 10 copies). The
// reference computes them over the locus' genotype table (DIVERSITY::
// CalcDiversity, src/diversity.cpp:144-492), whose genotypes appear in the
// order the loader first met them (src/load.cpp:2180-2230); its REAL sums run
// in that order. One warp per locus builds the table: 32 calls at a time,
// each lane looks its call's key up, the lanes with a new key group by key
// (__match_any_sync) and the first lane of each group appends it, in lane
// order, so the table keeps the order of first appearance; the counts are
// atomics. A locus holds at most N distinct genotypes, so each block's table
// lives in global scratch of N entries, with an open-addressing map from key
// to slot; a map entry carries the stamp of the locus (or collapse round)
// that wrote it, so nothing is cleared between loci. Lane 0 then derives the
// statistics and runs the HWE test with the reference's allele collapsing.
namespace {

// a call's key: copies in bits 0-3, allele j in bits 4 + 6j (0: missing;
// a call with an allele index outside the locus' kall alleles counts as
// missing)
__device__ __forceinline__ uint64_t call_key(const int8_t* g, int vmax, int kall) {
    if (g[0] < 0) return 0;
    uint64_t k = 0;
    int v = 0;
    for (; v < vmax && g[v] >= 0; ++v) {
        if (g[v] >= kall) return 0;
        k |= (uint64_t)g[v] << (4 + 6 * v);
    }
    return k | (uint64_t)v;
}

// key -> slot map: entries (stamp << 32 | slot), empty unless the stamp is
// the current one; read past L1 (__ldcg), written by atomics
struct SlotMap {
    unsigned long long* e;
    uint32_t mask;
    uint32_t stamp;
};
// the 64-bit finalizer of MurmurHash3 (Appleby)
__device__ __forceinline__ uint32_t key_hash(uint64_t k) {
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdull;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ull;
    k ^= k >> 33;
    return (uint32_t)k;
}
// the slot of key k among keys[], or -1
__device__ int map_find(const SlotMap& m, const uint64_t* keys, uint64_t k) {
    uint32_t h = key_hash(k) & m.mask;
    for (uint32_t n = 0; n <= m.mask; ++n, h = (h + 1) & m.mask) {
        const unsigned long long e = __ldcg(m.e + h);
        if ((uint32_t)(e >> 32) != m.stamp) return -1;
        const int s = (int)(uint32_t)e;
        if (__ldcg(keys + s) == k) return s;
    }
    return -1;
}
// key k (absent from the map) -> slot; lanes of one warp may insert
// distinct keys at once
__device__ void map_insert(const SlotMap& m, uint64_t k, int slot) {
    const unsigned long long v = ((unsigned long long)m.stamp << 32) | (uint32_t)slot;
    uint32_t h = key_hash(k) & m.mask;
    for (uint32_t n = 0; n <= m.mask; ++n, h = (h + 1) & m.mask) {
        unsigned long long e = __ldcg(m.e + h);
        while ((uint32_t)(e >> 32) != m.stamp) {
            const unsigned long long old = atomicCAS(m.e + h, e, v);
            if (old == e) return;
            e = old;
        }
    }
}

// one pass of the warp over the calls of a locus: with INSERT new keys join
// the table (tk, tc: T entries) in order of first appearance, with COUNT
// every call adds 1 to its key's count
template <bool INSERT, bool COUNT>
__device__ void table_pass(const int8_t* G, int N, int vmax, int kall, uint64_t* tk, uint32_t* tc, int& T,
                           const SlotMap& m) {
    const int lane = threadIdx.x & 31;
    for (int i0 = 0; i0 < N; i0 += 32) {
        const int i = i0 + lane;
        const uint64_t k = i < N ? call_key(G + (size_t)i * vmax, vmax, kall) : 0;
        int slot = k ? map_find(m, tk, k) : -1;
        if (INSERT) {
            const bool isnew = k && slot < 0;
            const unsigned peers = __match_any_sync(0xffffffffu, isnew ? k : ~0ull);
            const bool leader = isnew && (__ffs(peers) - 1) == lane;
            const unsigned leaders = __ballot_sync(0xffffffffu, leader);
            if (leaders) {
                if (leader) {
                    const int s = T + __popc(leaders & ((1u << lane) - 1u));
                    __stcg(tk + s, k);
                    __stcg(tc + s, 0u);
                    __threadfence_block();
                    map_insert(m, k, s);
                }
                __threadfence_block();
                __syncwarp();
                if (isnew) slot = map_find(m, tk, k);
                T += __popc(leaders);
            }
        }
        if (COUNT && slot >= 0) atomicAdd(tc + slot, 1u);
        __syncwarp();
    }
    __threadfence_block();
    __syncwarp();
}

// the dosage pattern of a key: distinct alleles by descending copy count,
// ties by the larger allele first (GENOTYPE::GENOTYPE, src/function.cpp
// :259-337)
struct GtPattern {
    int v, na;
    int al[10], key[10], cnt[10];
};
__device__ void gt_pattern(uint64_t k, GtPattern& p) {
    p.v = (int)(k & 15);
    for (int j = 0; j < p.v; ++j) p.al[j] = (int)((k >> (4 + 6 * j)) & 63);
    p.na = 0;
    for (int i = 0; i < p.v; ++i) {
        bool isnew = true;
        for (int j = i - 1; j >= 0; --j)
            if (p.al[i] == p.al[j]) { isnew = false; break; }
        if (!isnew) continue;
        int ac = 1;
        for (int j = i + 1; j < p.v; ++j) ac += p.al[j] == p.al[i];
        p.key[p.na] = p.al[i];
        p.cnt[p.na++] = ac;
    }
    for (int i = 0; i < p.na; ++i)
        for (int j = i + 1; j < p.na; ++j)
            if (p.cnt[i] < p.cnt[j] || (p.cnt[i] == p.cnt[j] && p.key[i] < p.key[j])) {
                int t = p.cnt[i]; p.cnt[i] = p.cnt[j]; p.cnt[j] = t;
                t = p.key[i]; p.key[i] = p.key[j]; p.key[j] = t;
            }
}
// GENOTYPE::HIndex as the reference's table holds it: a 15-decimal literal,
// the double nearest round(p / q x 10^15) / 10^15 (0 for one copy)
__device__ double gt_hindex(const GtPattern& p) {
    const long long q = (long long)p.v * (p.v - 1);
    if (q == 0) return 0;
    long long same = 0;
    for (int i = 0; i < p.na; ++i) same += (long long)p.cnt[i] * (p.cnt[i] - 1);
    const long long n15 = (2 * (q - same) * 1000000000000000LL + q) / (2 * q);
    return (double)n15 / 1e15;
}
// GENOTYPE::HWECoef: v! / prod cnt!
__device__ double gt_hwecoef(const GtPattern& p) {
    double f = 1;
    for (int i = 2; i <= p.v; ++i) f *= i;
    for (int a = 0; a < p.na; ++a)
        for (int i = 2; i <= p.cnt[a]; ++i) f /= i;
    return f;
}
// IntegerPower (src/math2.h:307-350) in double
__device__ double ipow(double x, int n) {
    switch (n) {
        case 0: return 1;
        case 1: return x;
        case 2: return x * x;
        case 3: return x * x * x;
        case 4: { const double x2 = x * x; return x2 * x2; }
        case 5: { const double x2 = x * x; return x2 * x2 * x; }
        case 6: { const double x3 = x * x * x; return x3 * x3; }
        case 7: { const double x3 = x * x * x; return x3 * x3 * x; }
        case 8: { const double x2 = x * x, x4 = x2 * x2; return x4 * x4; }
        case 9: { const double x3 = x * x * x; return x3 * x3 * x3; }
        case 10: { const double x2 = x * x, x4 = x2 * x2; return x4 * x4 * x2; }
        default: return pow(x, (double)n);
    }
}
// the chi-square upper tail: 1 - erf(sqrt(x / 2)) for df = 1 (as the
// biallelic kernel), else 1 - P(df / 2, x / 2), the regularized lower
// incomplete gamma function by its series below a + 1 and its continued
// fraction above (Numerical Recipes, 6.2)
__device__ double chi2_upper(double x, int df) {
    if (df == 1) return 1.0 - erf(sqrt(0.5 * x));
    const double a = 0.5 * df, z = 0.5 * x;
    if (z <= 0) return 1;
    const double lg = lgamma(a);
    if (z < a + 1) {
        double ap = a, sum = 1.0 / a, del = sum;
        for (int n = 0; n < 1000; ++n) {
            ap += 1;
            del *= z / ap;
            sum += del;
            if (fabs(del) < fabs(sum) * 1e-16) break;
        }
        return 1.0 - sum * exp(-z + a * log(z) - lg);
    }
    double b = z + 1 - a, c = 1.0 / 1e-300, d = 1.0 / b, h = d;
    for (int i = 1; i < 1000; ++i) {
        const double an = -i * (i - a);
        b += 2;
        d = an * d + b;
        if (fabs(d) < 1e-300) d = 1e-300;
        c = b + an / c;
        if (fabs(c) < 1e-300) c = 1e-300;
        d = 1.0 / d;
        const double del = d * c;
        h *= del;
        if (fabs(del - 1) < 1e-16) break;
    }
    return exp(-z + a * log(z) - lg) * h;
}

// CalcDiversity over a genotype table (keys tk, counts tc, T entries), k2
// alleles, ni individuals; k1/c1 and k2b/c2 (T entries each) hold the
// collapsed tables of the HWE test, cm maps their keys (a new stamp per
// round). out: n, k, ptype, bmaf, he, ho, pic, ae, I, pval (NaN where the
// reference leaves them undefined).
template <typename REAL>
__device__ void general_stats(const uint64_t* tk, const uint32_t* tc, int T, uint64_t* k1, uint32_t* c1,
                              uint64_t* k2b, uint32_t* c2, SlotMap& cm, int k2, int ni, double* out) {
    const double MINF = 1e-10, NANV = __longlong_as_double(0x7ff8000000000000ll);
    REAL fre[64], ho = 0, how = 0;
    for (int a = 0; a < k2; ++a) fre[a] = 0;
    int n = 0, nhaplo = 0, minp = 100, maxp = 0;
    bool varploidy = false;
    GtPattern p;
    for (int gi = 0; gi < T; ++gi) {
        const unsigned c = __ldcg(tc + gi);
        if (!c) continue;
        gt_pattern(__ldcg(tk + gi), p);
        const int v = p.v;
        nhaplo += v * c;
        maxp = max(maxp, v);
        minp = min(minp, v);
        if (maxp != minp) varploidy = true;
        ho += gt_hindex(p) * c * v * (v - 1);
        how += c * v * (v - 1);
        n += c;
        for (int i = 0; i < v; ++i) fre[p.al[i]] += c;
    }
    const REAL ptype = n / (REAL)ni;
    {   // Unify (src/math2.cpp:2268-2304)
        double s = 0;
        for (int a = 0; a < k2; ++a) s += fre[a];
        const double invsum = 1.0 / (s + k2 * MINF);
        for (int a = 0; a < k2; ++a) fre[a] = (REAL)(((double)fre[a] + MINF) * invsum);
    }
    int k = 0;
    if (n)
        for (int a = 0; a < k2; ++a) k += fre[a] > MINF;
    double bmaf = NANV, he = NANV, hoo = NANV, pic = NANV, ae = NANV, I = NANV, pval = NANV;
    if (k >= 2) {
        hoo = ho / how;
        REAL b = 1, a2 = 0, picv = 0, Iv = 0;
        const int nh = (int)(nhaplo + 0.5);
        for (int a = 0; a < k2; ++a) {
            const REAL af = fre[a];
            if (af * nh < 1e-5) continue;
            if (af > 1e-5) Iv += -af * rlog(af);
            if (b > af) b = af;
            a2 += af * af;
            for (int c = a + 1; c < k2; ++c)
                if (fre[c] > 0) picv += 2 * af * fre[c] * (1 - af * fre[c]);
        }
        if (b > 0.5) b = 1 - b;
        bmaf = b;
        he = (REAL)(1 - a2);
        ae = (REAL)(1 / a2);
        I = Iv;
        pic = picv;
        if (!varploidy) {
            // the HWE G-test with allele collapsing (src/diversity.cpp:337-492),
            // genotype model 0: expected counts HWECoef x prod f^count x n
            const int ploidy = maxp;
            const uint64_t* ck = tk;
            const uint32_t* cc = tc;
            int n1 = T;
            REAL f1[64], f2[64];
            int amap[64];
            for (int a = 0; a < k2; ++a) f1[a] = fre[a];
            uint64_t* dk = k1;
            uint32_t* dc = c1;
            REAL G = 0;
            bool flag = false;
            for (int kk = k2; kk >= 1 && !flag; kk = (kk <= k ? kk - 1 : k)) {
                if (kk == 1) break;
                for (int a = 0; a < kk; ++a) f2[a] = 0;
                if (kk <= k) {
                    flag = true;
                    G = 0;
                    for (int gi = 0; gi < n1; ++gi) {
                        const uint32_t cgi = __ldcg(cc + gi);
                        if (!cgi) continue;
                        gt_pattern(__ldcg(ck + gi), p);
                        double gfz = gt_hwecoef(p);
                        for (int ai = p.na - 1; ai >= 0; --ai) gfz *= ipow((double)f1[p.key[ai]], p.cnt[ai]);
                        const REAL obs = (REAL)cgi, ex = (REAL)(gfz * n);
                        if (ex < 5) { flag = false; break; }
                        G += 2 * obs * rlog(obs / ex);
                    }
                }
                if (flag) {
                    double bin = 1;   // Binomial(ploidy + kk - 1, ploidy) by factorials
                    for (int i = 2; i <= ploidy + kk - 1; ++i) bin *= i;
                    for (int i = 2; i <= ploidy; ++i) bin /= i;
                    for (int i = 2; i <= kk - 1; ++i) bin /= i;
                    pval = (REAL)chi2_upper((double)G, (int)(bin - kk + 0.5));
                    break;
                }
                if (kk <= k) {
                    // merge the two rarest alleles (GetMinID: the first minimum)
                    int m1 = 0;
                    for (int a = 1; a < kk; ++a) if (f1[m1] > f1[a]) m1 = a;
                    f1[m1]++;
                    int m2 = 0;
                    for (int a = 1; a < kk; ++a) if (f1[m2] > f1[a]) m2 = a;
                    f1[m1]--;
                    if (m1 > m2) { const int t = m1; m1 = m2; m2 = t; }
                    for (int j = 0, q = 0; j < kk; ++j) {
                        if (j == m2) { amap[j] = m1; f2[m1] = f1[m1] + f1[m2]; }
                        else { amap[j] = q; f2[q++] = f1[j]; }
                    }
                } else {
                    // absent alleles onto the most frequent one (GetMaxID: the first maximum)
                    int m1 = 0;
                    for (int a = 1; a < kk; ++a) if (f1[m1] < f1[a]) m1 = a;
                    for (int j = 0, q = 0; j < kk; ++j) amap[j] = f1[j] < MINF ? -1 : q++;
                    for (int j = 0; j < kk; ++j) amap[j] = amap[j] == -1 ? amap[m1] : amap[j];
                }
                // the collapsed table, in order of first mapping
                int n2 = 0;
                ++cm.stamp;
                for (int gi = 0; gi < n1; ++gi) {
                    const uint32_t cgi = __ldcg(cc + gi);
                    if (!cgi) continue;
                    gt_pattern(__ldcg(ck + gi), p);
                    int al[10];
                    for (int ai = 0; ai < ploidy; ++ai) al[ai] = amap[p.al[ai]];
                    for (int x = 1; x < ploidy; ++x) {
                        const int y0 = al[x];
                        int y = x - 1;
                        while (y >= 0 && al[y] > y0) { al[y + 1] = al[y]; --y; }
                        al[y + 1] = y0;
                    }
                    uint64_t nk = (uint64_t)ploidy;
                    for (int j = 0; j < ploidy; ++j) {
                        f2[al[j]] += cgi;
                        nk |= (uint64_t)(al[j] & 63) << (4 + 6 * j);
                    }
                    const int found = map_find(cm, dk, nk);
                    if (found < 0) {
                        __stcg(dk + n2, nk);
                        __stcg(dc + n2, cgi);
                        map_insert(cm, nk, n2);
                        ++n2;
                    } else {
                        __stcg(dc + found, __ldcg(dc + found) + cgi);
                    }
                }
                {
                    double s = 0;
                    for (int a = 0; a < kk; ++a) s += f2[a];
                    const double invsum = 1.0 / (s + kk * MINF);
                    for (int a = 0; a < kk; ++a) f2[a] = (REAL)(((double)f2[a] + MINF) * invsum);
                }
                for (int a = 0; a < kk; ++a) f1[a] = f2[a];
                // the new table becomes the current one; the other buffer is next
                ck = dk;
                cc = dc;
                n1 = n2;
                if (dk == k1) { dk = k2b; dc = c2; } else { dk = k1; dc = c1; }
            }
        }
    }
    out[0] = n; out[1] = k; out[2] = ptype; out[3] = bmaf; out[4] = he; out[5] = hoo; out[6] = pic;
    out[7] = ae; out[8] = I; out[9] = pval;
}

// one warp (= block) per locus, grid-stride; scratch per block: three
// tables of N keys and N counts, two maps of H entries (H a power of two,
// at least 2N; zeroed once: stamp 0 is never current)
__global__ void __launch_bounds__(32) k_locus_filter_general(const int8_t* G, const int8_t* Gt, int64_t L, int N,
                                                             int vmax, const int32_t* nall, vp_locus_filter f,
                                                             uint64_t* keys, uint32_t* counts,
                                                             unsigned long long* maps, uint32_t H, uint8_t* keep,
                                                             double* stats) {
    const int lane = threadIdx.x;
    uint64_t* tk = keys + (size_t)blockIdx.x * 3 * N;
    uint64_t* k1 = tk + N;
    uint64_t* k2 = k1 + N;
    uint32_t* tc = counts + (size_t)blockIdx.x * 3 * N;
    uint32_t* c1 = tc + N;
    uint32_t* c2 = c1 + N;
    SlotMap tm{maps + (size_t)blockIdx.x * 2 * H, H - 1, 0};
    SlotMap cm{tm.e + H, H - 1, 0};
    for (int64_t l = blockIdx.x; l < L; l += gridDim.x) {
        tm.stamp = (uint32_t)(l / gridDim.x) + 1;    // a new stamp for each locus of this block
        const int8_t* g = G + (size_t)l * N * vmax;
        const int kall = nall[l];
        int T = 0;
        if (Gt) {
            table_pass<true, false>(Gt + (size_t)l * N * vmax, N, vmax, kall, tk, tc, T, tm);
            table_pass<false, true>(g, N, vmax, kall, tk, tc, T, tm);
        } else {
            table_pass<true, true>(g, N, vmax, kall, tk, tc, T, tm);
        }
        if (lane == 0) {
            double o[VP_LOCUS_STATS];
            if (f.single) general_stats<float>(tk, tc, T, k1, c1, k2, c2, cm, nall[l], N, o);
            else general_stats<double>(tk, tc, T, k1, c1, k2, c2, cm, nall[l], N, o);
            const int k = (int)o[1], n = (int)o[0];
            const bool fail = k == 0 || (f.bmaf_b && k == 2 && outside(o[3], f.bmaf_min, f.bmaf_max)) ||
                              (f.k_b && (k < f.k_min || k > f.k_max)) || (f.n_b && (n < f.n_min || n > f.n_max)) ||
                              (f.ptype_b && outside(o[2], f.ptype_min, f.ptype_max)) ||
                              (f.he_b && outside(o[4], f.he_min, f.he_max)) ||
                              (f.ho_b && outside(o[5], f.ho_min, f.ho_max)) ||
                              (f.pic_b && outside(o[6], f.pic_min, f.pic_max)) ||
                              (f.ae_b && outside(o[7], f.ae_min, f.ae_max)) ||
                              (f.I_b && outside(o[8], f.I_min, f.I_max)) ||
                              (f.pval_b && o[9] != -1 && outside(o[9], f.pval_min, f.pval_max));
            keep[l] = fail ? 0 : 1;
            if (stats)
                for (int j = 0; j < VP_LOCUS_STATS; ++j) stats[l * VP_LOCUS_STATS + j] = o[j];
        }
        __syncwarp();
    }
}

}  // namespace

extern "C" int vp_locus_filter_general(const int8_t* alleles, const int8_t* alleles_table, int64_t n_loc,
                                       int32_t n_ind, int32_t vmax, const int32_t* n_alleles,
                                       const vp_locus_filter* f, int device, uint8_t* keep, double* stats) {
    if (!alleles || !n_alleles || !f || !keep || n_loc < 0 || n_ind <= 0 || vmax < 1 || vmax > 10) {
        vp_set_error("bad arguments");
        return VP_E_ARG;
    }
    // the genotype tables' hash maps index their entries with 32-bit masks
    if (n_ind > (1 << 28)) {
        vp_set_error("%d individuals: at most 2^28 for the genotype tables", n_ind);
        return VP_E_ARG;
    }
    for (int64_t l = 0; l < n_loc; ++l)
        if (n_alleles[l] < 1 || n_alleles[l] > 64) {
            vp_set_error("locus %lld has %d alleles (1 to 64)", (long long)(l + 1), n_alleles[l]);
            return VP_E_ARG;
        }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) { vp_set_error("no CUDA device"); return VP_E_NODEV; }
    if (device < 0 || device >= ndev) { vp_set_error("device %d out of range", device); return VP_E_ARG; }
    if (n_loc == 0) return VP_OK;
    CKI(cudaSetDevice(device));
    cudaStream_t st;
    CKI(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    const size_t gb = (size_t)n_loc * n_ind * vmax, tb = alleles_table ? gb : 0, kb = (size_t)n_loc * 4,
                 sb = stats ? (size_t)n_loc * VP_LOCUS_STATS * 8 : 0;
    // hash entries: a power of two, at least twice the individuals
    uint32_t H = 64;
    while ((uint64_t)H < 2ull * (uint64_t)n_ind) H <<= 1;
    int nsm = 132;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device);
    // a warp per block, 16 blocks per SM, scratch held under 2 GiB (fewer
    // blocks than SMs for very large samples)
    const int64_t per_block = (int64_t)n_ind * 3 * 12 + (int64_t)H * 16;
    const unsigned grid = (unsigned)std::max<int64_t>(
        1, std::min<int64_t>({n_loc, (int64_t)nsm * 16, (2ll << 30) / per_block}));
    const size_t xb = (size_t)grid * 3 * n_ind * 8, cb = (size_t)grid * 3 * n_ind * 4, mb = (size_t)grid * 2 * H * 8;
    auto up = [](size_t x) { return (x + 255) / 256 * 256; };
    char* buf = nullptr;
    int rc = VP_OK;
    cudaError_t e = cudaMallocAsync((void**)&buf, up(gb) + up(tb) + up(kb) + up((size_t)n_loc) + up(sb) + up(xb) +
                                                      up(cb) + mb, st);
    if (e != cudaSuccess) { vp_set_error("device allocation failed: %s", cudaGetErrorString(e)); rc = VP_E_MEM; }
    std::vector<uint8_t> hk;
    if (!rc) {
        char* q = buf;
        int8_t* dg = (int8_t*)q; q += up(gb);
        int8_t* dt = alleles_table ? (int8_t*)q : nullptr; q += up(tb);
        int32_t* dn = (int32_t*)q; q += up(kb);
        uint8_t* dk = (uint8_t*)q; q += up((size_t)n_loc);
        double* ds = stats ? (double*)q : nullptr; q += up(sb);
        uint64_t* xk = (uint64_t*)q; q += up(xb);
        uint32_t* xc = (uint32_t*)q; q += up(cb);
        unsigned long long* xm = (unsigned long long*)q;
        rc = upload_staged((char*)dg, (const char*)alleles, (int64_t)gb, st);
        if (!rc && dt) rc = upload_staged((char*)dt, (const char*)alleles_table, (int64_t)tb, st);
        if (!rc) {
            hk.resize(n_loc);
            if ((e = cudaMemcpyAsync(dn, n_alleles, kb, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
                (e = cudaMemsetAsync(xm, 0, mb, st)) != cudaSuccess) {
                vp_set_error("upload failed: %s", cudaGetErrorString(e));
                rc = VP_E_CUDA;
            } else {
                k_locus_filter_general<<<grid, 32, 0, st>>>(dg, dt, n_loc, n_ind, vmax, dn, *f, xk, xc, xm, H, dk, ds);
                if ((e = cudaGetLastError()) != cudaSuccess ||
                    (e = cudaMemcpyAsync(hk.data(), dk, (size_t)n_loc, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
                    (ds && (e = cudaMemcpyAsync(stats, ds, sb, cudaMemcpyDeviceToHost, st)) != cudaSuccess) ||
                    (e = cudaStreamSynchronize(st)) != cudaSuccess) {
                    vp_set_error("locus filter failed: %s", cudaGetErrorString(e));
                    rc = VP_E_CUDA;
                }
            }
        }
        cudaFreeAsync(buf, st);
    }
    cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
    if (!rc) memcpy(keep, hk.data(), (size_t)n_loc);
    return rc;
}
