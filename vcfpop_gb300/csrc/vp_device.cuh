// Device-side primitives of the STRUCTURE sweep: seeding hashes, the two
// random-number families, the reference's polynomial sine, and the
// exponent-split log used for zero frequencies.
//
// "Reference streams" (REF mode) follow vcfpop's generators exactly so that a
// step fed the same state draws the same uniforms as the reference:
//   RNG<double>  xorshift128+ seeded by MurmurHash64   (src/statistics.cpp:62-87)
//   RNG<float>   xorshift96   seeded by MurmurHash32   (src/statistics.cpp:330-355)
// "Counter streams" (CTR mode) are Philox-4x32-10 (Salmon et al., SC'11),
// keyed by the chain seed with the counter naming (sweep, step, element), so
// every draw site is independent and the steps run fully in parallel.
#pragma once
#include <stdint.h>
#include <cuda_runtime.h>

#define VP_MIN_FREQ 1e-10
#define VP_NZERO (-1e-10)

// salts of the reference's streams (src/global.h:70-80)
#define VP_SALT_INITADM   0xDA310D821043E1D3ull
#define VP_SALT_UPDATEQ   0xE7853EB09C92935Aull
#define VP_SALT_UPDATEZ   0x9B83516C63E249C3ull
#define VP_SALT_UPDATEP   0xD4EA1DB746DF14E3ull
#define VP_SALT_UPDATEA   0x49913AD9EDBD2EB8ull
#define VP_SALT_UPDATELOC 0x95EE7991226E2D14ull
#define VP_SALT_UPDATEALPHA 0x8A26E2C4D1BC5E54ull
#define VP_SALT_UPDATEF   0xF82104A5ADDAAF9Full

namespace vp {

// ---------------- hashing (src/hash.cpp:9-16, 219-223, 432-474) ----------------
__host__ __device__ inline uint32_t crc32c_u64(uint32_t crc, uint64_t v) {
    for (int b = 0; b < 8; ++b) {
        crc ^= (uint32_t)(v & 0xFF);
        v >>= 8;
        for (int j = 0; j < 8; ++j) crc = (crc >> 1) ^ (0x82F63B78u & (0u - (crc & 1u)));
    }
    return crc;
}
__host__ __device__ inline uint32_t hash_ulong(uint64_t v) { return crc32c_u64(0xB385FDA9u, v); }
__host__ __device__ inline uint32_t murmur_mix(uint32_t data, uint32_t seed) {
    const uint32_t m = 0x5bd1e995u;
    uint32_t s = seed ^ 4u, a = data;
    a *= m; a ^= a >> 24; a *= m; s *= m; a ^= s;
    a ^= a >> 13; a *= m; a ^= a >> 15;
    return a;
}
__host__ __device__ inline uint64_t murmur64(uint64_t data, uint64_t seed) {
    uint32_t d0 = (uint32_t)data, d1 = (uint32_t)(data >> 32);
    uint32_t s0 = (uint32_t)seed, s1 = (uint32_t)(seed >> 32);
    d1 = (~d0) ^ d1; s1 = (~s0) ^ s1;
    return ((uint64_t)murmur_mix(d1, s1) << 32) | (uint64_t)murmur_mix(d0, s0);
}
__host__ __device__ inline uint32_t murmur32(uint64_t data, uint64_t seed) {
    return murmur_mix((~(uint32_t)data) ^ (uint32_t)(data >> 32), (~(uint32_t)seed) ^ (uint32_t)(seed >> 32));
}

// ---------------- the reference's polynomial sine/cosine ----------------
// Box-Muller in the reference uses its own polynomials (src/math2.h:1087-1140),
// so REF mode must evaluate the same ones to draw the same normals.
__host__ __device__ inline double ref_cos_core(double x) {
    double x2 = x * x, x4 = x2 * x2, x8 = x4 * x4;
    return (-2.7236370439787708e-7 * x2 + 2.4799852696610628e-5) * x8 +
           (-1.3888885054799695e-3 * x2 + 4.1666666636943683e-2) * x4 +
           (-4.9999999999963024e-1 * x2 + 1.0000000000000000e+0);
}
__host__ __device__ inline double ref_sin_core(double x) {
    double x2 = x * x, x4 = x2 * x2;
    return ((2.7181216275479732e-6 * x2 - 1.9839312269456257e-4) * x4 +
            (8.3333293048425631e-3 * x2 - 1.6666666640797048e-1)) * x2 * x + x;
}
__host__ __device__ inline double ref_sin(double x) {
    double t0 = floor(fabs(x * 6.3661977236758138e-1) + 0.5);
    double q = (x * 6.3661977236758138e-1 < 0.0) ? -t0 : t0;
    int quadrant = (int)q;
    double t = x - q * 1.5707963267923333e+00;
    t = t - q * 2.5633441515945189e-12;
    t = (quadrant & 1) ? ref_cos_core(t) : ref_sin_core(t);
    return (quadrant & 2) ? -t : t;
}
__host__ __device__ inline double ref_cos(double x) { return ref_sin(x + (3.14159265358979323846264338328 / 2)); }

// natural log with the reference's bounds (src/math2.h:608-615)
__device__ inline double ref_mylog(double v) {
    if (v < 1e-300) return -6.90775527898214000E+02;
    if (v > 1e300) return +6.90775527898214000E+02;
    return log(v);
}

// ln of a float frequency as the reference's exponent-split product sees it:
// a zero contributes 2^-1023 (src/math2.h:738-780).
__device__ inline float ln_freq(float p) {
    return p > 0.f ? logf(p) : -709.0895657128241f;
}
// the same with the hardware logarithm (absolute error about 2^-21), for the
// centred tensor-core weights, which serve the label draws only (a recorded
// lnP(D) is formed from the counts with ln_freq)
__device__ inline float ln_freq_fast(float p) {
    return p > 0.f ? __logf(p) : -709.0895657128241f;
}

// ---------------- RNG<double>: xorshift128+ ----------------
struct Rng64 {
    uint64_t x, y;
    double U1, U2;
    bool cached;
    __device__ inline void init(uint64_t s, uint64_t salt) {
        s = murmur64(s, salt);
        x = 0x159A55E5075BCD15ull ^ s;
        y = 0x054913331F123BB5ull ^ (s << 6);
        cached = false;
    }
    __device__ inline uint64_t next() {
        uint64_t a = x, b = y;
        x = b;
        a ^= a << 23; a ^= a >> 18; a ^= b; a ^= b >> 5;
        y = a;
        return a + b;
    }
    __device__ inline double uniform(double mn = 0, double mx = 1) {
        uint64_t u = next();
        double re = __longlong_as_double((long long)(0x3FF0000000000000ull | (u & 0x000FFFFFFFFFFFFFull)));
        return (re - 1.0) * (mx - mn) + mn;
    }
    // Box-Muller keeping the second value (src/statistics.cpp:185-202). The
    // reference marks "no cached value" by writing 0xFFFFFFFF into the low word
    // of U1; a computed U1 whose low word is exactly that value is likewise
    // treated as absent.
    __device__ inline double normal(double mean = 0, double sd = 1) {
        if (cached) {
            double re = U1 * ref_sin(U2);
            cached = false;
            return re * sd + mean;
        }
        double v1 = uniform(), v2 = uniform();
        double s = -2.0 * log(v1);
        U1 = s > 0 ? sqrt(s) : (s > -VP_MIN_FREQ ? 0.0 : __longlong_as_double(0x7ff8000000000000ll));
        U2 = 2.0 * 3.14159265358979323846264338328 * v2;
        cached = ((uint32_t)__double_as_longlong(U1)) != 0xFFFFFFFFu;
        return U1 * ref_cos(U2) * sd + mean;
    }
    // Marsaglia-Tsang with the alpha<1 boost (src/statistics.cpp:212-242)
    __device__ inline double gamma(double alpha) {
        double boost = 1.0;
        bool small = alpha < 1;
        double a = small ? 1.0 + alpha : alpha;
        double t, v, u;
        double d = a - 0.333333333333333;
        double c = 1.0 / (sqrt(d) * 3.0);
        // bounded: valid shapes accept within a few attempts (the reference's
        // draws are reproduced exactly); a NaN shape would otherwise loop forever
        for (int attempt = 0; attempt < 4096; ++attempt) {
            int tries = 0;
            do {
                t = normal();
                v = 1.0 + c * t;
            } while (v <= 0 && ++tries < 4096);
            v = v * v * v;
            u = uniform();
            if (u < 1.0 - 0.0331 * t * t * t * t) break;
            if (log(u) < 0.5 * t * t + d * (1.0 - v + log(v))) break;
        }
        double g = d * v;
        if (small) boost = pow(uniform(), 1.0 / alpha);
        return g * boost;
    }
    __device__ inline uint64_t nextn(uint64_t mx) { return next() % mx; }
    __device__ inline uint64_t next_avoid(uint64_t mx, uint64_t av) {
        uint64_t a = nextn(mx - 1);
        if (a >= av) a++;
        return a;
    }
};

// ---------------- RNG<float>: xorshift96 ----------------
struct Rng32 {
    uint32_t x, y, z;
    __device__ inline void init(uint64_t seed, uint64_t salt) {
        uint32_t s = murmur32(seed, salt);
        x = 0x075BCD15u ^ s;
        y = 0x159A55E5u ^ (s << 3);
        z = 0x1F123BB5u ^ (s << 6);
    }
    __device__ inline uint32_t next() {
        x ^= x << 16; x ^= x >> 5; x ^= x << 1;
        uint32_t t = x; x = y; y = z; z = t ^ x ^ y;
        return z;
    }
    __device__ inline float uniform(float mn, float mx) {
        uint32_t u = next();
        float re = __uint_as_float(0x3F800000u | (u & 0x007FFFFFu));
        return (re - 1.0f) * (mx - mn) + mn;
    }
};

// ---------------- Philox-4x32-10 counter streams ----------------
struct Philox {
    uint4 ctr;
    uint2 key;
    uint4 buf;
    int pos;
    __device__ inline void init(uint64_t seed, uint32_t a, uint32_t b, uint32_t c) {
        key = make_uint2((uint32_t)seed, (uint32_t)(seed >> 32));
        ctr = make_uint4(a, b, c, 0);
        pos = 4;
    }
    __device__ static inline uint4 round10(uint4 c, uint2 k) {
#pragma unroll
        for (int r = 0; r < 10; ++r) {
            uint32_t hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
            uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
            c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
            k.x += 0x9E3779B9u; k.y += 0xBB67AE85u;
        }
        return c;
    }
    // pos counts the draws taken from buf; at 4 or more the next draw starts
    // a new block, pos - 4 draws past its start (skip() only moves pos)
    __device__ inline uint32_t next() {
        if (pos >= 4) {
            ctr.w += (uint32_t)((pos - 4) >> 2);
            buf = round10(ctr, key);
            ctr.w++;
            pos = (pos - 4) & 3;
        }
        uint32_t r = pos == 0 ? buf.x : pos == 1 ? buf.y : pos == 2 ? buf.z : buf.w;
        pos++;
        return r;
    }
    __device__ inline void skip(int n) { pos += n; }
    // the stream's first block, consumed whole (right after init)
    __device__ inline uint4 first_block() {
        buf = round10(ctr, key);
        ctr.w++;
        pos = 4;
        return buf;
    }
    // uniform in (0, 1]
    __device__ static inline float to_uniformf(uint32_t x) { return ((float)(x >> 8) + 1.0f) * (1.0f / 16777216.0f); }
    __device__ inline float uniformf() { return to_uniformf(next()); }
    __device__ inline double uniformd() {
        uint64_t h = next(), l = next();
        return ((double)(((h << 32) | l) >> 11) + 1.0) * (1.0 / 9007199254740992.0);
    }
    // standard normal in double precision (Box-Muller on two double uniforms)
    __device__ inline double normald() {
        const double u1 = uniformd(), u2 = uniformd();
        return sqrt(-2.0 * log(u1)) * cospi(2.0 * u2);
    }
    __device__ inline float normalf() {
        float u1 = uniformf(), u2 = uniformf();
        float r = sqrtf(-2.0f * logf(u1));
        return r * cospif(2.0f * u2);
    }
    // Marsaglia-Tsang gamma(alpha, 1) in single precision; alpha<1 boosted
    __device__ inline float gammaf(float alpha) {
        bool small = alpha < 1.f;
        float a = small ? alpha + 1.f : alpha;
        float d = a - 1.f / 3.f, c = rsqrtf(9.f * d);
        float v;
        for (int it = 0; it < 64; ++it) {
            float t = normalf();
            v = 1.f + c * t;
            if (v <= 0.f) continue;
            v = v * v * v;
            float u = uniformf();
            if (u < 1.f - 0.0331f * t * t * t * t) break;
            if (logf(u) < 0.5f * t * t + d * (1.f - v + logf(v))) break;
        }
        float g = d * v;
        if (small) g *= powf(uniformf(), 1.f / alpha);
        return g;
    }
    // Two independent gamma(a0, 1), gamma(a1, 1) draws (a Beta draw for a
    // biallelic locus), on a stream fresh from init. The first Marsaglia-Tsang
    // attempt of both takes the stream's first Philox block: the cosine and sine normals of one Box-Muller pair and
    // two acceptance uniforms; an attempt that is rejected (rare for shapes
    // >= 1) continues as gammaf does, on further blocks. The Box-Muller
    // radius and angle use the hardware approximations (__logf, __sincosf of
    // an angle in [-pi, pi)): the counter streams are not matched to the
    // reference's draws, and these calls are the bulk of the kernel's issue.
    __device__ inline void gamma2(float a0, float a1, float& g0, float& g1) {
        const bool s0 = a0 < 1.f, s1 = a1 < 1.f;
        const float b0 = s0 ? a0 + 1.f : a0, b1 = s1 ? a1 + 1.f : a1;
        const float d0 = b0 - 1.f / 3.f, c0 = rsqrtf(9.f * d0);
        const float d1 = b1 - 1.f / 3.f, c1 = rsqrtf(9.f * d1);
        // the first block of the stream gives the four uniforms directly; a
        // rejected attempt continues with the next block
        const uint4 b4 = first_block();
        const float u1 = to_uniformf(b4.x), u2 = to_uniformf(b4.y), u3 = to_uniformf(b4.z), u4 = to_uniformf(b4.w);
        const float r = sqrtf(-2.0f * __logf(u1));
        float sn, cs;
        __sincosf(6.283185307179586f * u2 - 3.141592653589793f, &sn, &cs);
        const bool ok0 = mt_accept(d0, c0, r * cs, u3, g0);
        const bool ok1 = mt_accept(d1, c1, r * sn, u4, g1);
        if (!ok0) g0 = mt_more(d0, c0);
        if (!ok1) g1 = mt_more(d1, c1);
        if (s0) g0 *= powf(uniformf(), 1.f / a0);
        if (s1) g1 *= powf(uniformf(), 1.f / a1);
    }
    // Beta(a0, a1) as the normalised pair of gamma2, (p0, p1) summing to 1:
    // the biallelic Dirichlet draw of UpdateP, shared by the per-chain and
    // batched kernels so that both give the same frequencies
    __device__ inline void dirichlet2(float a0, float a1, float& p0, float& p1) {
        float g0, g1;
        gamma2(a0, a1, g0, g1);
        const float inv = __fdividef(1.f, g0 + g1);
        p0 = g0 * inv;
        p1 = g1 * inv;
    }
    // one Marsaglia-Tsang attempt with normal t and uniform u
    __device__ static inline bool mt_accept(float d, float c, float t, float u, float& g) {
        float v = 1.f + c * t;
        if (v <= 0.f) return false;
        v = v * v * v;
        g = d * v;
        if (u < 1.f - 0.0331f * t * t * t * t) return true;
        return __logf(u) < 0.5f * t * t + d * (1.f - v + __logf(v));
    }
    __device__ inline float mt_more(float d, float c) {
        float g = d;
        for (int it = 0; it < 64; ++it)
            if (mt_accept(d, c, normalf(), uniformf(), g)) break;
        return g;
    }
};

}  // namespace vp
