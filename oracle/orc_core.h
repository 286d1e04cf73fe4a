/*
 * ORACLE (test infrastructure only) -- CPU restatement of the reference's
 * hashing, random-number and log-product primitives used by its STRUCTURE path.
 *
 * Nothing in the product links this file. Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg call it, to check and time the GPU library
 * against it.
 *
 * Each function names the reference file:line it restates (vcfpop v1.08b,
 * paths relative to the project's src/ folder). Arithmetic follows the
 * reference's scalar path (-g_simd=none) operation by operation, including the
 * float/double promotions, so that a build with -ffp-contract=off and no
 * fast-math reproduces the reference's results bit for bit on the same libm.
 */
#ifndef ORC_CORE_H
#define ORC_CORE_H
#include <stdint.h>
#include <math.h>
#include <string.h>
#include <float.h>

#define ORC_MIN_FREQ 1e-10           /* global.h:60 */
#define ORC_NZERO (-1e-10)           /* global.h:50 */
#define ORC_DBL_UNDERFLOW 1e-100     /* global.h:54 */
#define ORC_DBL_OVERFLOW 1e100       /* global.h:55 */
#define ORC_PI 3.14159265358979323846264338328 /* global.h:37 */

/* Salts, global.h:70-80 */
#define SALT_INITADM   0xDA310D821043E1D3ull
#define SALT_UPDATEQ   0xE7853EB09C92935Aull
#define SALT_UPDATEZ   0x9B83516C63E249C3ull
#define SALT_UPDATEP   0xD4EA1DB746DF14E3ull
#define SALT_UPDATEA   0x49913AD9EDBD2EB8ull
#define SALT_UPDATELOC 0x95EE7991226E2D14ull
#define SALT_UPDATEALPHA 0x8A26E2C4D1BC5E54ull
#define SALT_UPDATELAMBDA 0x67099E2FE2510092ull
#define SALT_UPDATEF   0xF82104A5ADDAAF9Full

/* ---- hashing (hash.cpp) ---- */

/* CRC32C of one 64-bit word, as SSE4.2 crc32 / ARMv8 crc32cd: hash.cpp:9-16 */
static inline uint32_t orc_crc32c_u64(uint32_t crc, uint64_t v) {
    for (int b = 0; b < 8; ++b) {
        crc ^= (uint32_t)(v & 0xFF);
        v >>= 8;
        for (int j = 0; j < 8; ++j) crc = (crc >> 1) ^ (0x82F63B78u & (0u - (crc & 1u)));
    }
    return crc;
}
/* HashULong with HASH64 undefined (vcfpop.h:546-550): hash.cpp:219-223 */
static inline uint32_t orc_hash_ulong(uint64_t v) { return orc_crc32c_u64(0xB385FDA9u, v); }

/* MurmurHash2 one-word mix: hash.cpp:432-452 */
static inline uint32_t orc_murmur2(uint32_t data, uint32_t seed) {
    const uint32_t m = 0x5bd1e995u;
    uint32_t s = seed ^ 4u, a = data;
    a *= m; a ^= a >> 24; a *= m; s *= m; a ^= s;
    a ^= a >> 13; a *= m; a ^= a >> 15;
    return a;
}
/* MurmurHash64: hash.cpp:455-464 */
static inline uint64_t orc_murmur64(uint64_t data, uint64_t seed) {
    uint32_t d0 = (uint32_t)data, d1 = (uint32_t)(data >> 32);
    uint32_t s0 = (uint32_t)seed, s1 = (uint32_t)(seed >> 32);
    d1 = (~d0) ^ d1; s1 = (~s0) ^ s1;
    return ((uint64_t)orc_murmur2(d1, s1) << 32) | (uint64_t)orc_murmur2(d0, s0);
}
/* MurmurHash32: hash.cpp:467-473 */
static inline uint32_t orc_murmur32(uint64_t data, uint64_t seed) {
    uint32_t a32 = (~(uint32_t)data) ^ (uint32_t)(data >> 32);
    uint32_t s32 = (~(uint32_t)seed) ^ (uint32_t)(seed >> 32);
    return orc_murmur2(a32, s32);
}

/* ---- math helpers (math2.h) ---- */

/* MyLog: math2.h:608-615 */
static inline double orc_mylog(double v) {
    if (v < 1e-300) return -6.90775527898214000E+02;
    if (v > 1e300) return +6.90775527898214000E+02;
    return log(v);
}
/* MySqrt: math2.h:295-303 */
static inline double orc_mysqrt(double v) {
    if (v > 0) return sqrt(v);
    if (v > -ORC_MIN_FREQ) return 0;
    return NAN;
}
/* The reference's own polynomial sine/cosine (math2.h:1087-1140); Normal()
 * uses them instead of libm, so the oracle must too. */
static inline double orc_coscore(double x) {
    double x2 = x * x, x4 = x2 * x2, x8 = x4 * x4;
    return (-2.7236370439787708e-7 * x2 + 2.4799852696610628e-5) * x8 +
           (-1.3888885054799695e-3 * x2 + 4.1666666636943683e-2) * x4 +
           (-4.9999999999963024e-1 * x2 + 1.0000000000000000e+0);
}
static inline double orc_sincore(double x) {
    double x2 = x * x, x4 = x2 * x2;
    return ((2.7181216275479732e-6 * x2 - 1.9839312269456257e-4) * x4 +
            (8.3333293048425631e-3 * x2 - 1.6666666640797048e-1)) * x2 * x + x;
}
static inline double orc_myrint(double x) {
    double t = floor(fabs(x) + 0.5);
    return (x < 0.0) ? -t : t;
}
static inline double orc_mysin(double x) {
    double q = orc_myrint(x * 6.3661977236758138e-1);
    int quadrant = (int)q;
    double t = x - q * 1.5707963267923333e+00;
    t = t - q * 2.5633441515945189e-12;
    t = (quadrant & 1) ? orc_coscore(t) : orc_sincore(t);
    return (quadrant & 2) ? -t : t;
}
static inline double orc_mycos(double x) { return orc_mysin(x + (ORC_PI / 2)); }

/* ---- exponent-split running product (math2.h:716-902) ---- */
static inline void orc_add_exponent_d(int64_t* slog, double* val) {
    int64_t vv; memcpy(&vv, val, 8);
    *slog += ((vv & 0x7FF0000000000000ll) >> 52) - 1023;
    vv = (vv & (int64_t)0x800FFFFFFFFFFFFFull) | 0x3FF0000000000000ll;
    memcpy(val, &vv, 8);
}
/* ChargeLog(int64&, double&, double): math2.h:762-771 */
static inline void orc_chargelog_d(int64_t* slog, double* prod, double val) {
    if (val < ORC_DBL_UNDERFLOW || val > ORC_DBL_OVERFLOW) orc_add_exponent_d(slog, &val);
    *prod *= val;
    if (*prod < ORC_DBL_UNDERFLOW || *prod > ORC_DBL_OVERFLOW) orc_add_exponent_d(slog, prod);
}
/* ChargeLog(int64&, double&, float): math2.h:774-780 */
static inline void orc_chargelog_f(int64_t* slog, double* prod, float val) {
    *prod *= val;
    if (*prod < ORC_DBL_UNDERFLOW || *prod > ORC_DBL_OVERFLOW) orc_add_exponent_d(slog, prod);
}
/* CloseLog: math2.h:889-894 (result in natural log) */
static inline double orc_closelog(int64_t slog, double prod) {
    return ((double)slog + log2(prod)) * 0.693147180559945;
}
/* LogProd(float*, n, sep) / LogProd(double*, n, sep): math2.cpp:1030-1116 scalar arms */
static inline double orc_logprod_f(const float* A, int64_t n, int64_t sep) {
    int64_t slog = 0; double prod = 1;
    for (int64_t i = 0; i < n; ++i, A += sep) orc_chargelog_f(&slog, &prod, *A);
    return orc_closelog(slog, prod);
}
static inline double orc_logprod_d(const double* A, int64_t n, int64_t sep) {
    int64_t slog = 0; double prod = 1;
    for (int64_t i = 0; i < n; ++i, A += sep) orc_chargelog_d(&slog, &prod, *A);
    return orc_closelog(slog, prod);
}
/* LogProdDiv(double*, double*, n, sep): math2.cpp:1118-1143 */
static inline double orc_logproddiv_d(const double* A, const double* B, int64_t n, int64_t sep) {
    int64_t s1 = 0, s2 = 0; double p1 = 1, p2 = 1;
    for (int64_t i = 0; i < n; ++i, A += sep, B += sep) {
        orc_chargelog_d(&s1, &p1, *A);
        orc_chargelog_d(&s2, &p2, *B);
    }
    return orc_closelog(s1, p1) - orc_closelog(s2, p2);
}
/* Sum(double*, n, sep): math2.cpp scalar arm */
static inline double orc_sum_d(const double* A, int64_t n, int64_t sep) {
    double re = 0;
    for (int64_t i = 0; i < n; ++i, A += sep) re += *A;
    return re;
}
static inline double orc_sum_f(const float* A, int64_t n) {
    double re = 0;
    for (int64_t i = 0; i < n; ++i) re += A[i];
    return re;
}
/* Unify(double*, n): math2.cpp:2268-2285 */
static inline void orc_unify_d(double* A, int64_t n) {
    double invsum = 1.0 / (orc_sum_d(A, n, 1) + n * ORC_MIN_FREQ);
    for (int64_t i = 0; i < n; ++i) A[i] = (A[i] + ORC_MIN_FREQ) * invsum;
}
/* Unify(float*, n): math2.cpp:2288-2305 */
static inline void orc_unify_f(float* A, int64_t n) {
    double invsum = 1.0 / (orc_sum_f(A, n) + n * ORC_MIN_FREQ);
    for (int64_t i = 0; i < n; ++i) A[i] = (float)(((double)A[i] + ORC_MIN_FREQ) * invsum);
}

/* ---- RNG<double>: xorshift128+ (statistics.cpp:62-320) ---- */
typedef struct { uint64_t x, y; double U1, U2; } orc_rng64;

static inline void orc_rng64_init(orc_rng64* r, uint64_t s, uint64_t salt) {
    s = orc_murmur64(s, salt);
    r->x = 0x159A55E5075BCD15ull ^ s;
    r->y = 0x054913331F123BB5ull ^ (s << 6);
    uint64_t u; memcpy(&u, &r->U1, 8);
    u = (u & 0xFFFFFFFF00000000ull) | 0xFFFFFFFFull; /* *(uint*)&U1 = 0xFFFFFFFF */
    memcpy(&r->U1, &u, 8);
}
static inline uint64_t orc_rng64_next(orc_rng64* r) {
    uint64_t a = r->x, b = r->y;
    r->x = b;
    a ^= a << 23; a ^= a >> 18; a ^= b; a ^= b >> 5;
    r->y = a;
    return a + b;
}
/* Uniform: statistics.cpp:168-174 */
static inline double orc_rng64_uniform(orc_rng64* r, double mn, double mx) {
    uint64_t u = orc_rng64_next(r), b = 0x3FF0000000000000ull | (u & 0x000FFFFFFFFFFFFFull);
    double re; memcpy(&re, &b, 8);
    return (re - 1.0) * (mx - mn) + mn;
}
static inline int orc_u1_cached(const orc_rng64* r) {
    uint32_t lo; memcpy(&lo, &r->U1, 4);
    return lo != 0xFFFFFFFFu;
}
/* Normal (Box-Muller with a cached second value): statistics.cpp:185-202 */
static inline double orc_rng64_normal(orc_rng64* r, double mean, double sd) {
    if (orc_u1_cached(r)) {
        double re = r->U1 * orc_mysin(r->U2);
        uint32_t ff = 0xFFFFFFFFu; memcpy(&r->U1, &ff, 4);
        return re * sd + mean;
    }
    volatile double v1 = orc_rng64_uniform(r, 0, 1);
    volatile double v2 = orc_rng64_uniform(r, 0, 1);
    r->U1 = orc_mysqrt(-2.0 * log(v1));
    r->U2 = 2.0 * ORC_PI * v2;
    return r->U1 * orc_mycos(r->U2) * sd + mean;
}
/* Gamma (Marsaglia-Tsang; boost for alpha<1): statistics.cpp:212-242 */
static double orc_rng64_gamma(orc_rng64* r, double alpha, double beta) {
    if (alpha < 1) {
        volatile double v1 = orc_rng64_gamma(r, 1.0 + alpha, beta);
        volatile double v2 = pow(orc_rng64_uniform(r, 0, 1), 1.0 / alpha);
        return v1 * v2;
    }
    double t, v, u;
    double d = alpha - 0.333333333333333;
    double c = 1.0 / (sqrt(d) * 3.0);
    for (;;) {
        do {
            t = orc_rng64_normal(r, 0, 1);
            volatile double v1 = c * t;
            v = 1.0 + v1;
        } while (v <= 0);
        v = v * v * v;
        u = orc_rng64_uniform(r, 0, 1);
        if (u < 1.0 - 0.0331 * t * t * t * t) break;
        if (log(u) < 0.5 * t * t + d * (1.0 - v + log(v))) break;
    }
    return beta * d * v;
}
/* Poly(double*, n): statistics.cpp:89-114 */
static inline int orc_rng64_poly(orc_rng64* r, const double* a, int n) {
    double s = orc_sum_d(a, n, 1) + ORC_MIN_FREQ * n;
    double t = orc_rng64_uniform(r, 0, s);
    for (int i = 0; i < n; ++i) {
        if (t < a[i] + ORC_MIN_FREQ) return i;
        t -= a[i] + ORC_MIN_FREQ;
    }
    return n - 1;
}
/* PolyLog(double*, n), overwrites a: statistics.cpp:116-155 */
static inline int orc_rng64_polylog(orc_rng64* r, double* a, int n) {
    double maxval = -DBL_MAX, s = ORC_MIN_FREQ * n;
    for (int i = 0; i < n; ++i) { if (a[i] < maxval) continue; maxval = a[i]; }
    for (int i = 0; i < n; ++i) {
        double diff = a[i] - maxval;
        a[i] = diff < -23 ? ORC_MIN_FREQ : exp(diff);
        s += a[i];
    }
    double rr = orc_rng64_uniform(r, 0, s);
    for (int i = 0; i < n; ++i) {
        if (rr < a[i]) return i;
        rr -= a[i];
    }
    return n - 1;
}
/* Next / NextAvoid: statistics.cpp:301-320 */
static inline uint64_t orc_rng64_nextn(orc_rng64* r, uint64_t mx) { return orc_rng64_next(r) % mx; }
static inline uint64_t orc_rng64_nextavoid(orc_rng64* r, uint64_t mx, uint64_t av) {
    uint64_t a = orc_rng64_nextn(r, mx - 1);
    if (a >= av) a++;
    return a;
}

/* ---- RNG<float>: xorshift96 (statistics.cpp:330-393) ---- */
typedef struct { uint32_t x, y, z; } orc_rng32;
static inline void orc_rng32_init(orc_rng32* r, uint64_t seed, uint64_t salt) {
    uint32_t s = orc_murmur32(seed, salt);
    r->x = 0x075BCD15u ^ s;
    r->y = 0x159A55E5u ^ (s << 3);
    r->z = 0x1F123BB5u ^ (s << 6);
}
static inline uint32_t orc_rng32_next(orc_rng32* r) {
    uint32_t t;
    r->x ^= r->x << 16; r->x ^= r->x >> 5; r->x ^= r->x << 1;
    t = r->x; r->x = r->y; r->y = r->z; r->z = t ^ r->x ^ r->y;
    return r->z;
}
static inline float orc_rng32_uniform(orc_rng32* r, float mn, float mx) {
    uint32_t u = orc_rng32_next(r), b = 0x3F800000u | (u & 0x007FFFFFu);
    float re; memcpy(&re, &b, 4);
    return (re - 1.0f) * (mx - mn) + mn;
}
/* Poly(float*, n) with Sumx: statistics.cpp:357-385, math2.cpp:1233-1250 */
static inline int orc_rng32_poly(orc_rng32* r, const float* a, int n) {
    float s = 0, sx = 0;
    for (int i = 0; i < n; ++i) sx += a[i];
    s = sx + ORC_MIN_FREQ * n;
    float t = orc_rng32_uniform(r, 0, s);
    for (int i = 0; i < n; ++i) {
        if (t < a[i] + ORC_MIN_FREQ) return i;
        t -= a[i] + ORC_MIN_FREQ;
    }
    return n - 1;
}

#endif
