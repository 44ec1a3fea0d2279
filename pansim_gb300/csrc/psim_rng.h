// Counter-based random draws and the deterministic math shared by the CUDA
// kernels and the host code of pansim_gb300.
//
// The reference draws from a per-thread curand XORWOW state on the GPU
// (include/tools/randomGenerator.h:31-94, src/tools/randomGenerator.cpp:10-15)
// and from per-OpenMP-thread std::mt19937_64 generators seeded by
// std::random_device on the CPU; neither stream is reproducible across
// back ends or runs.  Here every draw comes from a stateless Philox4x32-10
// stream (Salmon, Moraes, Dror, Shaw: "Parallel random numbers: as easy as
// 1, 2, 3", SC'11) keyed by the run seed and addressed by
// (agent, tick, phase, block).  A stream yields 32-bit words in order; the
// four RandomGenerator entry points map onto it as:
//   randomUnit()        -> psim_u01:     53-bit double in [0,1) from 2 words
//   randomReal(max)     -> max * psim_u01
//   randomUnsigned(m)   -> psim_below:   floor(word * m / 2^32), no word if m==0
//   geometric(p)        -> psim_geometric: failures before the first success of
//                          Bernoulli trials "word < thr(p)", thr = floor(p*2^32)
// All of these are exact integer / IEEE operations, so the same stream gives
// bit-identical results on the host and on the device.
//
// psim_one_minus_exp() evaluates 1 - exp(-x) for x >= 0 with explicit fma()
// Horner steps (Taylor series of expm1 and of exp after an ln2 range
// reduction), so it too is bit-identical on host and device.
#pragma once
#include <stdint.h>
#include <math.h>

#if defined(__CUDACC__)
#define PSIM_HD __host__ __device__ __forceinline__
#else
#define PSIM_HD static inline
#endif

#define PSIM_PHILOX_M0 0xD2511F53u
#define PSIM_PHILOX_M1 0xCD9E8D57u
#define PSIM_PHILOX_W0 0x9E3779B9u
#define PSIM_PHILOX_W1 0xBB67AE85u

// Stream phases: the third counter word.  Each phase has its own stream per
// (agent, tick) so that draws of one policy never shift another's.
enum {
    PSIM_PHASE_MOVE = 1,      // movement at timestamp t
    PSIM_PHASE_INFECT = 2,    // infection at timestamp t, + variant
    PSIM_PHASE_PROGRESS = 16, // daily progression at the midnight timestamp
    PSIM_PHASE_TEST = 17,     // daily testing at the midnight timestamp
    PSIM_PHASE_IMMUNIZE = 18, // daily immunization
    PSIM_PHASE_PLAN_SWQ = 19, // planLocations: school/work quarantine lookups
    PSIM_PHASE_PLAN_UNDERAGE = 20,
    PSIM_PHASE_PLAN_NOWORK = 21,
    PSIM_PHASE_TEST_FLAG = 22, // testing: flagLocations lookups
    PSIM_PHASE_EXPOSE = 23,    // closure rule ExposeToMutation at the midnight timestamp
    PSIM_PHASE_IMM_CATEGORY = 24, // immunization categories, + category pass (10 passes)
    PSIM_PHASE_IMM_BOOSTER = 40,  // immunization boosters, + round
    PSIM_PHASE_IMM_PRIMARY = 56,  // immunization first doses, + category
    PSIM_PHASE_OTHER_DISEASE = 66 // non-COVID hospitalization and death at the midnight timestamp
};

typedef struct psim_ctr4 {
    uint32_t v[4];
} psim_ctr4;

PSIM_HD uint32_t psim_mulhi32(uint32_t a, uint32_t b) {
    return (uint32_t)(((uint64_t)a * (uint64_t)b) >> 32);
}

// Philox4x32 with 10 rounds.
PSIM_HD psim_ctr4 psim_philox4x32_10(psim_ctr4 c, uint32_t k0, uint32_t k1) {
#if defined(__CUDACC__)
#pragma unroll
#endif
    for (int r = 0; r < 10; ++r) {
        if (r > 0) {
            k0 += PSIM_PHILOX_W0;
            k1 += PSIM_PHILOX_W1;
        }
        uint32_t hi0 = psim_mulhi32(PSIM_PHILOX_M0, c.v[0]);
        uint32_t lo0 = PSIM_PHILOX_M0 * c.v[0];
        uint32_t hi1 = psim_mulhi32(PSIM_PHILOX_M1, c.v[2]);
        uint32_t lo1 = PSIM_PHILOX_M1 * c.v[2];
        psim_ctr4 n;
        n.v[0] = hi1 ^ c.v[1] ^ k0;
        n.v[1] = lo1;
        n.v[2] = hi0 ^ c.v[3] ^ k1;
        n.v[3] = lo0;
        c = n;
    }
    return c;
}

// A sequential word stream over consecutive Philox blocks.
typedef struct psim_stream {
    uint32_t k0, k1;
    uint32_t c0, c1, c2, blk;
    uint32_t buf[4];
    uint32_t idx;
} psim_stream;

PSIM_HD void psim_stream_init(psim_stream* s, uint64_t seed, uint32_t agent, uint32_t tick, uint32_t phase) {
    s->k0 = (uint32_t)seed;
    s->k1 = (uint32_t)(seed >> 32);
    s->c0 = agent;
    s->c1 = tick;
    s->c2 = phase;
    s->blk = 0;
    s->idx = 4;
    s->buf[0] = s->buf[1] = s->buf[2] = s->buf[3] = 0;
}

PSIM_HD uint32_t psim_next_u32(psim_stream* s) {
    if (s->idx >= 4) {
        psim_ctr4 c;
        c.v[0] = s->c0;
        c.v[1] = s->c1;
        c.v[2] = s->c2;
        c.v[3] = s->blk;
        psim_ctr4 o = psim_philox4x32_10(c, s->k0, s->k1);
        s->buf[0] = o.v[0];
        s->buf[1] = o.v[1];
        s->buf[2] = o.v[2];
        s->buf[3] = o.v[3];
        s->blk += 1;
        s->idx = 0;
    }
    return s->buf[s->idx++];
}

// 53-bit uniform double in [0, 1).
PSIM_HD double psim_u01_from(uint32_t a, uint32_t b) {
    return ((double)(a >> 5) * 67108864.0 + (double)(b >> 6)) * (1.0 / 9007199254740992.0);
}

PSIM_HD double psim_u01(psim_stream* s) {
    uint32_t a = psim_next_u32(s);
    uint32_t b = psim_next_u32(s);
    return psim_u01_from(a, b);
}

// Uniform integer in [0, m); consumes no word when m == 0 (the reference
// returns 0 before drawing, include/tools/randomGenerator.h:61-63).
PSIM_HD uint32_t psim_below(psim_stream* s, uint32_t m) {
    if (m == 0) return 0u;
    uint32_t w = psim_next_u32(s);
    return (uint32_t)(((uint64_t)w * (uint64_t)m) >> 32);
}

// Bernoulli threshold for success probability p: P(word < thr) = thr / 2^32.
PSIM_HD uint32_t psim_geometric_threshold(double p) {
    if (!(p > 0.0)) return 0u;
    if (p >= 1.0) return 0xFFFFFFFFu;
    double t = floor(p * 4294967296.0);
    if (t < 1.0) t = 1.0;
    return (uint32_t)t;
}

#define PSIM_GEOMETRIC_MAX_TRIALS (1u << 24)

// Number of failures before the first success (support 0,1,2,...), the same
// support as std::geometric_distribution.  Bounded at 2^24 trials.
PSIM_HD int psim_geometric(psim_stream* s, uint32_t thr) {
    if (thr == 0xFFFFFFFFu) return 0;
    uint32_t k = 0;
    while (k < PSIM_GEOMETRIC_MAX_TRIALS) {
        if (psim_next_u32(s) < thr) break;
        ++k;
    }
    return (int)k;
}

// Single-shot uniform for (seed, agent, tick, phase): the first two words of
// the stream's first block.
PSIM_HD double psim_u01_once(uint64_t seed, uint32_t agent, uint32_t tick, uint32_t phase) {
    psim_ctr4 c;
    c.v[0] = agent;
    c.v[1] = tick;
    c.v[2] = phase;
    c.v[3] = 0u;
    psim_ctr4 o = psim_philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    return psim_u01_from(o.v[0], o.v[1]);
}

// fma() is the correctly rounded IEEE fused multiply-add on both sides.
#define PSIM_FMA(a, b, c) fma((a), (b), (c))

// 1 - exp(-x) for x >= 0, deterministic across host and device.
PSIM_HD double psim_one_minus_exp(double x) {
    if (!(x > 0.0)) return 0.0;
    if (x >= 40.0) return 1.0;
    if (x < 0.5) {
        // -expm1(-x) = sum_{k>=1} (-1)^(k+1) x^k / k!
        double p = 0x1.2f49b46814157p-57;     // k = 19
        p = PSIM_FMA(p, x, -0x1.6827863b97d97p-53);
        p = PSIM_FMA(p, x, 0x1.952c77030ad4ap-49);
        p = PSIM_FMA(p, x, -0x1.ae7f3e733b81fp-45);
        p = PSIM_FMA(p, x, 0x1.ae7f3e733b81fp-41);
        p = PSIM_FMA(p, x, -0x1.93974a8c07c9dp-37);
        p = PSIM_FMA(p, x, 0x1.6124613a86d09p-33);
        p = PSIM_FMA(p, x, -0x1.1eed8eff8d898p-29);
        p = PSIM_FMA(p, x, 0x1.ae64567f544e4p-26);
        p = PSIM_FMA(p, x, -0x1.27e4fb7789f5cp-22);
        p = PSIM_FMA(p, x, 0x1.71de3a556c734p-19);
        p = PSIM_FMA(p, x, -0x1.a01a01a01a01ap-16);
        p = PSIM_FMA(p, x, 0x1.a01a01a01a01ap-13);
        p = PSIM_FMA(p, x, -0x1.6c16c16c16c17p-10);
        p = PSIM_FMA(p, x, 0x1.1111111111111p-7);
        p = PSIM_FMA(p, x, -0x1.5555555555555p-5);
        p = PSIM_FMA(p, x, 0x1.5555555555555p-3);
        p = PSIM_FMA(p, x, -0x1.0000000000000p-1);
        p = PSIM_FMA(p, x, 0x1.0000000000000p+0);
        return p * x;
    }
    // exp(-x) = 2^-n * exp(-y), x = n*ln2 + y, |y| <= ln2/2
    double n = floor(PSIM_FMA(x, 0x1.71547652b82fep+0, 0.5));
    double y = PSIM_FMA(-n, 0x1.62e42fee00000p-1, x);
    y = PSIM_FMA(-n, 0x1.a39ef35793c76p-33, y);
    double z = -y;
    // exp(z) = sum_{k>=0} z^k / k!, |z| <= 0.35
    double e = 0x1.ae7f3e733b81fp-45;     // 1/16!
    e = PSIM_FMA(e, z, 0x1.ae7f3e733b81fp-41);  // 1/15!
    e = PSIM_FMA(e, z, 0x1.93974a8c07c9dp-37);  // 1/14!
    e = PSIM_FMA(e, z, 0x1.6124613a86d09p-33);  // 1/13!
    e = PSIM_FMA(e, z, 0x1.1eed8eff8d898p-29);  // 1/12!
    e = PSIM_FMA(e, z, 0x1.ae64567f544e4p-26);  // 1/11!
    e = PSIM_FMA(e, z, 0x1.27e4fb7789f5cp-22);  // 1/10!
    e = PSIM_FMA(e, z, 0x1.71de3a556c734p-19);  // 1/9!
    e = PSIM_FMA(e, z, 0x1.a01a01a01a01ap-16);  // 1/8!
    e = PSIM_FMA(e, z, 0x1.a01a01a01a01ap-13);  // 1/7!
    e = PSIM_FMA(e, z, 0x1.6c16c16c16c17p-10);  // 1/6!
    e = PSIM_FMA(e, z, 0x1.1111111111111p-7);   // 1/5!
    e = PSIM_FMA(e, z, 0x1.5555555555555p-5);   // 1/4!
    e = PSIM_FMA(e, z, 0x1.5555555555555p-3);   // 1/3!
    e = PSIM_FMA(e, z, 0x1.0000000000000p-1);   // 1/2!
    e = PSIM_FMA(e, z, 1.0);
    e = PSIM_FMA(e, z, 1.0);
    // scale by 2^-n exactly (n in [1, 58])
    double scale = 1.0;
    int ni = (int)n;
    for (int i = 0; i < ni; ++i) scale *= 0.5;
    return 1.0 - e * scale;
}

// 1 - exp(-x) for x >= 0 in FP32, deterministic across host and device
// (explicit fmaf Horner steps; Taylor series of -expm1 below 0.5, of exp
// after a two-part ln2 range reduction above).  Relative error a few ulp,
// and no cancellation at small x.
PSIM_HD float psim_one_minus_expf(float x) {
    if (!(x > 0.0f)) return 0.0f;
    if (x >= 20.0f) return 1.0f;
    if (x < 0.5f) {
        float p = 0x1.ae6456p-26f;               // k = 11
        p = fmaf(p, x, -0x1.27e4fcp-22f);
        p = fmaf(p, x, 0x1.71de3ap-19f);
        p = fmaf(p, x, -0x1.a01a02p-16f);
        p = fmaf(p, x, 0x1.a01a02p-13f);
        p = fmaf(p, x, -0x1.6c16c2p-10f);
        p = fmaf(p, x, 0x1.111112p-7f);
        p = fmaf(p, x, -0x1.555556p-5f);
        p = fmaf(p, x, 0x1.555556p-3f);
        p = fmaf(p, x, -0x1.0p-1f);
        p = fmaf(p, x, 1.0f);
        return p * x;
    }
    const float n = floorf(fmaf(x, 0x1.715476p+0f, 0.5f));
    float y = fmaf(-n, 0x1.63p-1f, x);
    y = fmaf(-n, -0x1.bd0106p-13f, y);
    const float z = -y;
    float e = 0x1.27e4fcp-22f;                   // 1/10!
    e = fmaf(e, z, 0x1.71de3ap-19f);
    e = fmaf(e, z, 0x1.a01a02p-16f);
    e = fmaf(e, z, 0x1.a01a02p-13f);
    e = fmaf(e, z, 0x1.6c16c2p-10f);
    e = fmaf(e, z, 0x1.111112p-7f);
    e = fmaf(e, z, 0x1.555556p-5f);
    e = fmaf(e, z, 0x1.555556p-3f);
    e = fmaf(e, z, 0x1.0p-1f);
    e = fmaf(e, z, 1.0f);
    e = fmaf(e, z, 1.0f);
    float scale = 1.0f;
    const int ni = (int)n;
    for (int i = 0; i < ni; ++i) scale *= 0.5f;
    return 1.0f - e * scale;
}

// The infection ratio of a location (infectionPolicies.h:523-546):
// r = 1 - exp(-k * (S / n) * w * season * dt) with S the exact fixed-point
// sum, every step one IEEE single-precision operation.
PSIM_HD float psim_hazard_x(long long fix, unsigned n, float k_f, float w, float season, unsigned dt, float* x_out) {
    if (fix == 0 || n == 0) {
        *x_out = 0.0f;
        return 0.0f;
    }
    float S = (float)fix;
    S = S * 0x1p-40f;
    float x = S / (float)n;
    x = k_f * x;
    x = x * w;
    x = x * season;
    x = x * (float)dt;
    *x_out = x;
    return psim_one_minus_expf(x);
}

PSIM_HD float psim_hazard(long long fix, unsigned n, float k_f, float w, float season, unsigned dt) {
    float x;
    return psim_hazard_x(fix, n, k_f, w, season, dt, &x);
}

// Fixed-point scale for per-location infectiousness sums: every FP32 value
// >= 2^-17 converts exactly, so the int64 sum is exact and independent of
// summation order.
#define PSIM_FIX_SCALE_F 1099511627776.0f   /* 2^40 */
#define PSIM_FIX_INV 9.094947017729282379150390625e-13 /* 2^-40 */
