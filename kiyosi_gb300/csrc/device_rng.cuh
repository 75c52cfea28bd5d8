// Device random streams: kiyosi's PCG32 / Box-Muller normals and scrambled Sobol points,
// reproduced bit-exactly in their integer words on sm_103a.
//
// FP64 transforms follow the reference's arithmetic step for step (the FP64 translation
// unit is compiled with --fmad=false, so only the explicit fma() calls fuse, exactly
// where the reference calls mul_add).  FP32 transforms start from the same integers.
#pragma once
#include <cstdint>

namespace kgpu {

constexpr int kBlockSize = 256;            // BLOCK_SIZE, engines/monte_carlo.rs:20
constexpr uint64_t kPcgMultiplier = 6364136223846793005ULL;
constexpr int kSobolBits = 52;

// ------------------------------------------------------------------------------------
// PCG-XSH-RR 64/32 (engines/monte_carlo.rs:2224-2277)
// ------------------------------------------------------------------------------------
struct Pcg {
    uint64_t state;
    uint64_t inc;
};

__host__ __device__ __forceinline__ uint32_t pcg_next(Pcg& g) {
    uint64_t previous = g.state;
    g.state = previous * kPcgMultiplier + g.inc;
    uint32_t x = uint32_t(((previous >> 18) ^ previous) >> 27);
    uint32_t r = uint32_t(previous >> 59);
#ifdef __CUDA_ARCH__
    return __funnelshift_r(x, x, r);
#else
    return (x >> r) | (x << ((32 - r) & 31));
#endif
}

// Pcg32::new (monte_carlo.rs:2247-2256)
__host__ __device__ __forceinline__ Pcg pcg_new(uint64_t seed, uint64_t stream) {
    Pcg g{0, (stream << 1) | 1};
    pcg_next(g);
    g.state += seed;
    pcg_next(g);
    return g;
}

// Pcg32::advance (monte_carlo.rs:2233-2245): O(log distance) affine squaring.
__host__ __device__ __forceinline__ void pcg_advance(Pcg& g, uint64_t distance) {
    uint64_t multiplier = kPcgMultiplier, inc = g.inc;
    while (distance != 0) {
        if (distance & 1) g.state = g.state * multiplier + inc;
        inc = inc * (multiplier + 1);
        multiplier = multiplier * multiplier;
        distance >>= 1;
    }
}

// The 52 random bits of Pcg32::uniform (monte_carlo.rs:2272-2276).
__host__ __device__ __forceinline__ uint64_t pcg_bits52(Pcg& g) {
    uint64_t hi = pcg_next(g);
    uint64_t lo = pcg_next(g);
    return (hi << 20) | (lo >> 12);
}

// ------------------------------------------------------------------------------------
// FP64 Box-Muller exactly as sample_normal (monte_carlo.rs:1830-1845).
// ------------------------------------------------------------------------------------
__device__ __forceinline__ double uniform52(uint64_t bits) {
    return (double(bits) + 0.5) / 4503599627370496.0;
}

// sin_cos_turns (monte_carlo.rs:1852-1894): turn-space quadrant reduction and Taylor
// polynomials with separately rounded products and sums.
__device__ __forceinline__ void sin_cos_turns(double turns, double* s, double* c) {
    const double tau = 6.283185307179586;
    uint32_t quadrant = __double2uint_rz(__dadd_rn(__dmul_rn(turns, 4.0), 0.5));
    double angle = __dmul_rn(tau, __dadd_rn(turns, -__dmul_rn(0.25, double(quadrant))));
    double sq = __dmul_rn(angle, angle);
    double ps = -1.0 / 1307674368000.0;
    ps = __dadd_rn(__dmul_rn(ps, sq), 1.0 / 6227020800.0);
    ps = __dadd_rn(__dmul_rn(ps, sq), -1.0 / 39916800.0);
    ps = __dadd_rn(__dmul_rn(ps, sq), 1.0 / 362880.0);
    ps = __dadd_rn(__dmul_rn(ps, sq), -1.0 / 5040.0);
    ps = __dadd_rn(__dmul_rn(ps, sq), 1.0 / 120.0);
    ps = __dadd_rn(__dmul_rn(ps, sq), -1.0 / 6.0);
    double pc = 1.0 / 20922789888000.0;
    pc = __dadd_rn(__dmul_rn(pc, sq), -1.0 / 87178291200.0);
    pc = __dadd_rn(__dmul_rn(pc, sq), 1.0 / 479001600.0);
    pc = __dadd_rn(__dmul_rn(pc, sq), -1.0 / 3628800.0);
    pc = __dadd_rn(__dmul_rn(pc, sq), 1.0 / 40320.0);
    pc = __dadd_rn(__dmul_rn(pc, sq), -1.0 / 720.0);
    pc = __dadd_rn(__dmul_rn(pc, sq), 1.0 / 24.0);
    pc = __dadd_rn(__dmul_rn(pc, sq), -0.5);
    // The reference folds from 0.0: 0*sq + k0 = k0 exactly, as above.
    double sn = __dadd_rn(angle, __dmul_rn(__dmul_rn(angle, sq), ps));
    double cs = __dadd_rn(1.0, __dmul_rn(sq, pc));
    if (quadrant & 1) {
        double t = sn;
        sn = cs;
        cs = -t;
    }
    if (quadrant & 2) {
        sn = -sn;
        cs = -cs;
    }
    *s = sn;
    *c = cs;
}

// `exact_radius` selects the FP32 radius's square root (below); FP64 is always IEEE.
__device__ __forceinline__ void box_muller(uint64_t b1, uint64_t b2, double* cosine, double* sine,
                                           bool /*exact_radius*/ = false) {
    double radius = sqrt(__dmul_rn(-2.0, log(uniform52(b1))));
    double s, c;
    sin_cos_turns(uniform52(b2), &s, &c);
    *cosine = __dmul_rn(radius, c);
    *sine = __dmul_rn(radius, s);
}

// FP32 Box-Muller on the same 52-bit integers.  The angle is reduced to [-1/2, 1/2]
// turns before the hardware sine/cosine, whose absolute error on [-pi, pi] is ~2^-21.
// (k + 1/2) 2^-52 in single precision from a 52-bit integer, converting 32-bit halves
// (a 64-bit integer conversion is a multi-instruction sequence).
__device__ __forceinline__ float unit52f(uint64_t k) {
    const float hi = __uint2float_rn(uint32_t(k >> 20));
    const float lo = __uint2float_rn(uint32_t(k & 0xFFFFF));
    return fmaf(hi, 0x1p-32f, fmaf(lo, 0x1p-52f, 0x1p-53f));
}

// FP32 square root on the SFU (PTX sqrt.approx.f32, one MUFU operation; sqrt(+0) = +0):
// IEEE sqrtf adds a Newton correction and a special-case branch to it, about eight more
// instructions for a last-bit difference that FP32 paths do not need.
__device__ __forceinline__ float sqrt_approx(float x) {
    float r;
    asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// The radius takes the SFU square root unless `exact_radius` asks for IEEE sqrtf.  Both
// were measured: the SFU root made the one-thread-per-path Heston Asian 7% faster and the
// path-major shared-grid walk 10% slower (the compiler schedules that walk differently),
// so the shared-grid kernel asks for the IEEE root.
__device__ __forceinline__ void box_muller(uint64_t b1, uint64_t b2, float* cosine, float* sine,
                                           bool exact_radius = false) {
    float u1 = unit52f(b1);
    float u2 = unit52f(b2);
    const float r2 = -2.0f * __logf(u1);
    float radius = exact_radius ? sqrtf(r2) : sqrt_approx(r2);
    // u2 - rint(u2) for u2 in [0, 1] (rint(0.5) = 0) as a compare and select; the
    // result is the same float for every u2 in that range.
    float turns = u2 > 0.5f ? u2 - 1.0f : u2;
    float s, c;
    __sincosf(6.28318530717958647692f * turns, &s, &c);
    *cosine = radius * c;
    *sine = radius * s;
}

// ------------------------------------------------------------------------------------
// Inverse normal CDF.
// ------------------------------------------------------------------------------------
// FP64: Cephes ndtri as restated in engines/monte_carlo/sobol.rs:253-346.
__device__ __forceinline__ double ndtri_poly(double v, const double* c, int n, double leading) {
    double r = leading;
    for (int i = 0; i < n; ++i) r = __dadd_rn(__dmul_rn(r, v), c[i]);
    return r;
}

__device__ inline double inverse_normal_cdf(double probability) {
    const double P0[] = {-59.96335010141079, 98.00107541859997, -56.67628574690703,
                         13.931260938727968, -1.2391658386738125};
    const double Q0[] = {1.9544885833814176, 4.676279128988815,  86.36024213908905,
                         -225.46268785411937, 200.26021238006066, -82.03722561683334,
                         15.90562251262117,   -1.1833162112133};
    const double P1[] = {4.0554489230596245,  31.525109459989388,  57.16281922464213,
                         44.08050738932008,   14.684956192885803,  2.1866330685079025,
                         -0.1402560791713545, -0.03504246268278482, -0.0008574567851546854};
    const double Q1[] = {15.779988325646675,   45.39076351288792,   41.3172038254672,
                         15.04253856929075,    2.504649462083094,   -0.14218292285478779,
                         -0.03808064076915783, -0.0009332594808954574};
    const double P2[] = {3.2377489177694603,     6.915228890689842,     3.9388102529247444,
                         1.3330346081580755,     0.20148538954917908,   0.012371663481782003,
                         0.00030158155350823543, 2.6580697468673755e-06, 6.239745391849833e-09};
    const double Q2[] = {6.02427039364742,       3.6798356385616087,     1.3770209948908132,
                         0.21623699359449663,    0.013420400608854318,   0.00032801446468212774,
                         2.8924786474538068e-06, 6.790194080099813e-09};
    const double tail_boundary = 0.1353352832366127;
    bool upper = probability > 1.0 - tail_boundary;
    double tail = upper ? 1.0 - probability : probability;
    if (tail > tail_boundary) {
        double centered = tail - 0.5;
        double square = __dmul_rn(centered, centered);
        double ratio = __ddiv_rn(ndtri_poly(square, P0, 5, 0.0), ndtri_poly(square, Q0, 8, 1.0));
        return __dmul_rn(__dadd_rn(centered, __dmul_rn(__dmul_rn(centered, square), ratio)),
                         sqrt(2.0 * 3.141592653589793));
    }
    double root = sqrt(__dmul_rn(-2.0, log(tail)));
    double inverse = __ddiv_rn(1.0, root);
    double ratio = root < 8.0
                       ? __ddiv_rn(ndtri_poly(inverse, P1, 9, 0.0), ndtri_poly(inverse, Q1, 8, 1.0))
                       : __ddiv_rn(ndtri_poly(inverse, P2, 9, 0.0), ndtri_poly(inverse, Q2, 8, 1.0));
    double correction = __dmul_rn(inverse, ratio);
    double quantile = __dadd_rn(__dadd_rn(root, -__ddiv_rn(log(root), root)), -correction);
    return upper ? quantile : -quantile;
}

__device__ __forceinline__ double sobol_normal(uint64_t bits, double) {
    return inverse_normal_cdf(uniform52(bits));
}

// FP32: lower-tail probability t formed exactly from the integer (1 - u is exact
// there), x = 1 - 2t, w = -ln(4 t (1 - t)); Phi^{-1}(t) = -sqrt(2) x p(w) with p a
// two-piece polynomial fitted by fit_normal_quantile.py (max abs error 1.1e-5 over the
// whole 52-bit range, ~1e-7 for |z| < 3).  The tail piece is needed by 0.7% of draws
// and sits behind a branch.
// Normal quantile from a lower-tail probability t in (0, 1/2] (see above).
__device__ __forceinline__ float normal_from_tail(float t, bool upper) {
    const float x = fmaf(-2.0f, t, 1.0f);
    const float w = -__logf(4.0f * t * (1.0f - t));
    const float v1 = w - 2.5f;
    float p = 3.194503809e-08f;
    p = fmaf(p, v1, 3.488168990e-07f);
    p = fmaf(p, v1, -3.563068968e-06f);
    p = fmaf(p, v1, -4.445640587e-06f);
    p = fmaf(p, v1, 2.187011429e-04f);
    p = fmaf(p, v1, -1.253577486e-03f);
    p = fmaf(p, v1, -4.177785603e-03f);
    p = fmaf(p, v1, 2.466406437e-01f);
    p = fmaf(p, v1, 1.501409427e+00f);
    if (w >= 5.0f) {  // |z| > 2.7: rare, so the warp seldom diverges here
        const float v2 = w * rsqrtf(w) - 3.0f;
        float p2 = 1.884356591e-05f;
        p2 = fmaf(p2, v2, -2.298956430e-04f);
        p2 = fmaf(p2, v2, 1.165614206e-03f);
        p2 = fmaf(p2, v2, -3.248520120e-03f);
        p2 = fmaf(p2, v2, 5.754719426e-03f);
        p2 = fmaf(p2, v2, -7.795813414e-03f);
        p2 = fmaf(p2, v2, 9.445793138e-03f);
        p2 = fmaf(p2, v2, 1.001694350e+00f);
        p = fmaf(p2, v2, 2.832976957e+00f);
    }
    const float z = 1.41421356237309505f * x * p;
    return upper ? z : -z;
}

// Two quantiles at once: normal_from_tail's central-piece operations in their packed
// FP32x2 forms (each lane of FFMA2 / FMUL2 / FADD2 is the IEEE single-precision
// operation, so each result equals normal_from_tail's); an element that needs the tail
// piece (w >= 5, and `need`) is evaluated by normal_from_tail itself.
__device__ __forceinline__ float2 normal_from_tail_pair(float2 t, bool upper0, bool upper1, bool need0,
                                                        bool need1) {
    const float2 x = __ffma2_rn(make_float2(-2.0f, -2.0f), t, make_float2(1.0f, 1.0f));
    const float2 rest = __fadd2_rn(make_float2(1.0f, 1.0f), make_float2(-t.x, -t.y));
    const float2 prod = __fmul2_rn(__fmul2_rn(make_float2(4.0f, 4.0f), t), rest);
    const float2 w = make_float2(-__logf(prod.x), -__logf(prod.y));
    const float2 v1 = __fadd2_rn(w, make_float2(-2.5f, -2.5f));
    auto c = [](float k) { return make_float2(k, k); };
    float2 p = c(3.194503809e-08f);
    p = __ffma2_rn(p, v1, c(3.488168990e-07f));
    p = __ffma2_rn(p, v1, c(-3.563068968e-06f));
    p = __ffma2_rn(p, v1, c(-4.445640587e-06f));
    p = __ffma2_rn(p, v1, c(2.187011429e-04f));
    p = __ffma2_rn(p, v1, c(-1.253577486e-03f));
    p = __ffma2_rn(p, v1, c(-4.177785603e-03f));
    p = __ffma2_rn(p, v1, c(2.466406437e-01f));
    p = __ffma2_rn(p, v1, c(1.501409427e+00f));
    float2 z = __fmul2_rn(__fmul2_rn(c(1.41421356237309505f), x), p);
    z.x = upper0 ? z.x : -z.x;
    z.y = upper1 ? z.y : -z.y;
    if (need0 && w.x >= 5.0f) z.x = normal_from_tail(t.x, upper0);
    if (need1 && w.y >= 5.0f) z.y = normal_from_tail(t.y, upper1);
    return z;
}

// Lower-tail probability from the top 32 bits k32 of the 52-bit tail integer: the
// unknown low 20 bits are taken at their midpoint.
__device__ __forceinline__ float normal_from_tail32(uint32_t k32, bool upper) {
    return normal_from_tail(fmaf(__uint2float_rn(k32), 0x1p-32f, 0x1p-33f), upper);
}

__device__ __forceinline__ float sobol_normal(uint64_t bits, float) {
    const uint64_t half = uint64_t(1) << 51;
    const bool upper = bits >= half;
    const uint64_t k = upper ? ((uint64_t(1) << 52) - 1 - bits) : bits;
    return normal_from_tail(unit52f(k), upper);
}

}  // namespace kgpu
