// The reference's genotype filter (-f_dp, -f_gq, -f_ploidy) on the text of a
// VCF data line, shared by the device parsers (vp_ingest.cu) and the driver's
// host reader (vp_cli.cpp) so that both read a call the same way.
#pragma once
#include <cstdint>

#include "../../include/vcfpop_structure.h"

#ifdef __CUDACC__
#define VP_HD __host__ __device__
#else
#define VP_HD
#endif

namespace vp {

// The loader rewrites each data line before it reads the calls
// (src/load.cpp:2130-2257): of the FORMAT keys it keeps GT, DP and GQ
// (two bytes, case as written, then ':' or a tab; AD only for allelic-depth
// modes, which do not apply here), and each call keeps the values of those
// keys, in order. The genotype filter then finds DP and GQ among the kept
// keys (LOCUS::GetFormatId) and reads each call's value with ReadIntegerKeep,
// which scans the rewritten text: values of dropped keys are not there.
//
// The FORMAT field at q (up to a tab or the end of the line): GT must be its
// first key; dp and gq get the indices (in this FORMAT) of its first DP and
// GQ keys (-1: absent); bit j of kept is set when key j is kept (keys past 63
// are not).
VP_HD inline bool parse_format(const char* q, int64_t room, int* dp, int* gq, uint64_t* kept) {
    *dp = -1;
    *gq = -1;
    *kept = 0;
    if (!(room >= 2 && q[0] == 'G' && q[1] == 'T' && (room == 2 || q[2] == ':' || q[2] == '\t'))) return false;
    int idx = 0;
    int64_t s0 = 0;
    for (int64_t r = 0;; ++r) {
        const bool last = r >= room || q[r] == '\t';
        if (!last && q[r] != ':') continue;
        if (r - s0 == 2 && idx < 64) {
            const char a = q[s0], b = q[s0 + 1];
            const bool isgt = a == 'G' && b == 'T', isdp = a == 'D' && b == 'P', isgq = a == 'G' && b == 'Q';
            if (isgt || isdp || isgq) *kept |= 1ull << idx;
            if (isdp && *dp < 0) *dp = idx;
            if (isgq && *gq < 0) *gq = idx;
        }
        if (last) break;
        ++idx;
        s0 = r + 1;
    }
    return true;
}

// ReadIntegerKeep (src/string2.cpp:711-727) from key j0 of the call at p:
// characters up to the first digit or '-' are skipped (so a '.' value reads
// the next number further on: a later kept key of this call or a later
// call), then the digits are read, wrapping like the reference's int.
// Characters of keys the rewrite dropped are not seen. The reference's scan
// has no bound; here the end of the line e stops it, with 0 when no digit
// follows.
VP_HD inline int read_int_keep(const char* t, int64_t p, int64_t e, int j0, uint64_t kept) {
    int j = j0;
    auto next = [&](char* c) {          // the next character of the rewritten text, or 0 past e
        for (;;) {
            if (p >= e) { ++p; *c = '\0'; return; }
            const char x = t[p++];
            if (x == ':') { ++j; *c = x; return; }
            if (x == '\t') { j = 0; *c = x; return; }
            if (j < 64 && ((kept >> j) & 1)) { *c = x; return; }
        }
    };
    int sign = 0;
    char c;
    next(&c);
    while (c < '0' || c > '9') {
        if (p > e) return 0;
        if (c == '-') {
            sign = 1;
            next(&c);
            break;
        }
        next(&c);
    }
    uint32_t x = 0;
    while (c >= '0' && c <= '9') {
        x = x * 10u + (uint32_t)(c - '0');
        next(&c);
    }
    return sign ? -(int)x : (int)x;
}

// The genotype filter (-f with -f_dp, -f_gq, -f_ploidy; AddVCFGenotype,
// src/load.cpp:3545-3566) on a typed call of v copies starting at t[p]
// (its keys end at a tab or at e): true when the call becomes missing. A DP
// or GQ key counts only where the call has it (dpid < fmtc among the kept
// keys, which is the same as among all keys: a call's keys are a prefix of
// FORMAT); DP is compared as an unsigned value (-1 skips it), GQ as a signed
// one.
VP_HD inline bool call_filtered(const vp_call_filter& cf, const char* t, int64_t p, int64_t e, int dpid, int gqid,
                                uint64_t kept, int v) {
    if (cf.ploidy_b && (v < cf.ploidy_min || v > cf.ploidy_max)) return true;
    if (!cf.dp_b && !cf.gq_b) return false;
    int64_t sdp = -1, sgq = -1;
    int fmtc = 1;
    for (int64_t r = p; r < e && t[r] != '\t'; ++r)
        if (t[r] == ':') {
            if (fmtc == dpid) sdp = r + 1;
            if (fmtc == gqid) sgq = r + 1;
            ++fmtc;
        }
    if (cf.dp_b && dpid >= 0 && dpid < fmtc) {
        const uint32_t dp = (uint32_t)read_int_keep(t, sdp, e, dpid, kept);
        if (dp != 0xFFFFFFFFu && (dp < (uint32_t)cf.dp_min || dp > (uint32_t)cf.dp_max)) return true;
    }
    if (cf.gq_b && gqid >= 0 && gqid < fmtc) {
        const int gq = read_int_keep(t, sgq, e, gqid, kept);
        if (gq != -1 && (gq < cf.gq_min || gq > cf.gq_max)) return true;
    }
    return false;
}

}  // namespace vp
