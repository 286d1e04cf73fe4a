// Internal types shared by the host translation units of the library.
#pragma once
#include <stdint.h>

#include <atomic>
#include <string>
#include <vector>

#include "../../include/vcfpop_structure.h"

// host buffer that is page-locked when a CUDA device is present (so uploads
// run at full copy-engine speed), plain heap memory otherwise
template <typename T>
struct HostBuf {
    T* p = nullptr;
    size_t n = 0;
    bool pinned = false;
    HostBuf() = default;
    HostBuf(const HostBuf&) = delete;
    HostBuf& operator=(const HostBuf&) = delete;
    ~HostBuf() { release(); }
    void release();
    void resize(size_t m);
    T* data() { return p; }
    const T* data() const { return p; }
    size_t size() const { return n; }
    T& operator[](size_t i) { return p[i]; }
    const T& operator[](size_t i) const { return p[i]; }
};

struct vp_dataset {
    std::atomic<int> refs{1};      // the caller's handle plus each server request holding it
    int32_t N = 0, S = 0, vmax = 0, maxploidy = 0, maxK = 0, Nw = 0;
    int64_t L = 0, KT = 0, coprime = 1;
    bool packed2 = false;
    HostBuf<uint32_t> g2;          // packed2: [L][Nw] 2-bit codes, sorted locus order
    std::vector<uint8_t> gb;       // general: [L][N][vmax] allele per copy, 0xFF none
    std::vector<int32_t> k;        // [L] alleles
    std::vector<int64_t> off;      // [L] allele offsets
    std::vector<int64_t> vt;       // [N] typed copies per individual
    std::vector<int64_t> order;    // [L] sorted position -> input locus
    std::vector<int32_t> popid, pop_ind0, pop_nind;
    std::vector<int32_t> perm;     // individuals in ascending ploidy (empty: one ploidy)
    std::vector<float> totfreq;    // [KT] total-population frequency, pre-sort layout
    std::vector<int32_t> nhaplo;   // [L] typed copies per locus, pre-sort order
    std::vector<int64_t> kdis;     // [maxK+1] loci with k alleles
};

void vp_set_error(const char* fmt, ...);

// device bytes a request (its context's uploads plus one chain) will hold;
// -1 when the parameters are invalid
int64_t vp_request_bytes(const vp_dataset* ds, const vp_params* P, int nsm);
// vp_open with the context's stream at a CUDA stream priority (lower numbers
// run first; 0 is the default)
int vp_open_ex(const vp_dataset* ds, int device, int priority, vp_ctx** out);
// one more reference to a dataset; vp_dataset_free drops one
void vp_dataset_retain(const vp_dataset* ds);
// vp_finish without the final wait
int vp_finish_issue(vp_chain** cs, int32_t n);
// sweeps issued so far and in total for one chain
void vp_chain_progress(const vp_chain* c, int64_t* issued, int64_t* total);
// the dataset a chain's context holds, and the chain's parameters
const vp_dataset* vp_chain_dataset(const vp_chain* c);
void vp_chain_params(const vp_chain* c, vp_params* p);
// vp_cohort_open with the cohort's stream at a CUDA stream priority
int vp_cohort_open_ex(int device, int priority, vp_cohort** out);
// a hash of the launches of one sweep of the chain (kernels, shapes, scalar
// arguments): chains with equal signatures merge every launch of a cohort
uint64_t vp_chain_sweep_signature(vp_chain* c);
