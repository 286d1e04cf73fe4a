// Internal types shared by the host translation units of the library.
#pragma once
#include <stdint.h>
#include <string>
#include <vector>

#include "../../include/vcfpop_structure.h"

struct vp_dataset {
    int32_t N = 0, S = 0, vmax = 0, maxploidy = 0, maxK = 0, Nw = 0;
    int64_t L = 0, KT = 0, coprime = 1;
    bool packed2 = false;
    std::vector<uint32_t> g2;      // packed2: [L][Nw] 2-bit codes, sorted locus order
    std::vector<uint8_t> gb;       // general: [L][N][vmax] allele per copy, 0xFF none
    std::vector<int32_t> k;        // [L] alleles
    std::vector<int64_t> off;      // [L] allele offsets
    std::vector<int64_t> vt;       // [N] typed copies per individual
    std::vector<int64_t> order;    // [L] sorted position -> input locus
    std::vector<int32_t> popid, pop_ind0, pop_nind;
    std::vector<float> totfreq;    // [KT] total-population frequency, pre-sort layout
    std::vector<int32_t> nhaplo;   // [L] typed copies per locus, pre-sort order
    std::vector<int64_t> kdis;     // [maxK+1] loci with k alleles
};

void vp_set_error(const char* fmt, ...);
