// Shared device helpers for libbz (sm_103a): constants, Philox4x32-10, uniform and
// normal conventions, exact reference index arithmetic, decoupled look-back.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "bz.h"

namespace bz {

// electron_kernel_numba.py:13-24 (same expressions, so the float64 values match).
__host__ __device__ inline double q_e() { return 1.602 * 1e-19; }
__host__ __device__ inline double m_e() { return 9.10938 * 1e-31; }
__host__ __device__ inline double m_n() { return 6.6 * 1e-26; }
__host__ __device__ inline double j_ev() { return 6.241509 * 1e18; }
constexpr double E_ION = 15.76;
constexpr double EPS_DEAD = 0.01;  // velocity given to w<=0 particles inside the kernel
constexpr double X_DEAD = 0.00000001;  // where the reference parks absorbed particles

// --------------------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as
// 1, 2, 3", SC'11): 10 rounds of two 32x32->64 multiplies, Weyl key schedule.
// --------------------------------------------------------------------------------------
struct u32x4 { uint32_t x, y, z, w; };

template <int ROUNDS = 10>
__device__ __forceinline__ u32x4 philox_r(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0,
                                          uint32_t k1) {
#pragma unroll
    for (int r = 0; r < ROUNDS; ++r) {
        // one 32x32 -> 64-bit product per multiplier gives both halves
        const uint64_t p0 = uint64_t(0xD2511F53u) * c0;
        const uint64_t p1 = uint64_t(0xCD9E8D57u) * c2;
        const uint32_t hi0 = uint32_t(p0 >> 32), lo0 = uint32_t(p0);
        const uint32_t hi1 = uint32_t(p1 >> 32), lo1 = uint32_t(p1);
        c0 = hi1 ^ c1 ^ k0;
        c1 = lo1;
        c2 = hi0 ^ c3 ^ k1;
        c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return {c0, c1, c2, c3};
}
__device__ __forceinline__ u32x4 philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0,
                                        uint32_t k1) {
    return philox_r<10>(c0, c1, c2, c3, k0, k1);
}

// Rounds of the push's draws (gas velocity, collision, ionization). Salmon et al. report
// Philox4x32 with 7 rounds as the smallest round count that passes all of TestU01's
// BigCrush ("Crush-resistant", SC'11 Table 2) and recommend 10 as a margin; the push, whose
// runtime these rounds dominate after the memory traffic, uses 7, and so do the resampling
// draws (RS_ROUNDS). The energy redraws, the minibatches and the known-answer checks keep 10.
constexpr int PUSH_ROUNDS = 7;
constexpr int RS_ROUNDS = 7;

// The same generator with the round keys precomputed (k + r*W, r = 0..9): when they sit
// in the kernel's parameter space the XORs read them directly and no key schedule runs.
template <int ROUNDS = 10>
__device__ __forceinline__ u32x4 philox_rk(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, const uint32_t *rk0,
                                           const uint32_t *rk1) {
    static_assert(ROUNDS >= 1 && ROUNDS <= 10, "ten round keys");
#pragma unroll
    for (int r = 0; r < ROUNDS; ++r) {
        const uint64_t p0 = uint64_t(0xD2511F53u) * c0;
        const uint64_t p1 = uint64_t(0xCD9E8D57u) * c2;
        const uint32_t hi0 = uint32_t(p0 >> 32), lo0 = uint32_t(p0);
        const uint32_t hi1 = uint32_t(p1 >> 32), lo1 = uint32_t(p1);
        c0 = hi1 ^ c1 ^ rk0[r];
        c1 = lo1;
        c2 = hi0 ^ c3 ^ rk1[r];
        c3 = lo0;
    }
    return {c0, c1, c2, c3};
}
// Two independent counters (differing only in the last word) through the same rounds, one
// round of each after the other: the two dependency chains interleave, so a warp has a
// second multiply to issue while the first one's result is pending.
template <int ROUNDS = 10>
__device__ __forceinline__ void philox_rk_x2(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3a, uint32_t c3b,
                                             const uint32_t *rk0, const uint32_t *rk1, u32x4 &ra, u32x4 &rb) {
    static_assert(ROUNDS >= 1 && ROUNDS <= 10, "ten round keys");
    uint32_t a0 = c0, a1 = c1, a2 = c2, a3 = c3a;
    uint32_t b0 = c0, b1 = c1, b2 = c2, b3 = c3b;
#pragma unroll
    for (int r = 0; r < ROUNDS; ++r) {
        const uint64_t pa0 = uint64_t(0xD2511F53u) * a0, pa1 = uint64_t(0xCD9E8D57u) * a2;
        const uint64_t pb0 = uint64_t(0xD2511F53u) * b0, pb1 = uint64_t(0xCD9E8D57u) * b2;
        const uint32_t na0 = uint32_t(pa1 >> 32) ^ a1 ^ rk0[r], na2 = uint32_t(pa0 >> 32) ^ a3 ^ rk1[r];
        const uint32_t nb0 = uint32_t(pb1 >> 32) ^ b1 ^ rk0[r], nb2 = uint32_t(pb0 >> 32) ^ b3 ^ rk1[r];
        a1 = uint32_t(pa1); a3 = uint32_t(pa0); a0 = na0; a2 = na2;
        b1 = uint32_t(pb1); b3 = uint32_t(pb0); b0 = nb0; b2 = nb2;
    }
    ra = {a0, a1, a2, a3};
    rb = {b0, b1, b2, b3};
}
inline void philox_round_keys(uint64_t seed, uint32_t *rk0, uint32_t *rk1) {
    uint32_t k0 = uint32_t(seed), k1 = uint32_t(seed >> 32);
    for (int r = 0; r < 10; ++r, k0 += 0x9E3779B9u, k1 += 0xBB67AE85u) {
        rk0[r] = k0;
        rk1[r] = k1;
    }
}

// A uniform and its complement, both exact: float path u = ((r>>9)+0.5)*2^-23;
// double path u = ((hi26<<26 | lo26) + 0.5)*2^-52. Keeping 1-u exact lets sin(chi)
// = 2 sqrt(u(1-u)) keep full relative accuracy near the poles.
template <typename T> struct Uni { T u, c; };

__device__ __forceinline__ Uni<float> uni_f(uint32_t r) {
    // k = r >> 9 spliced into the mantissa of 1.0 gives 1 + k 2^-23 exactly; subtracting
    // 1 - 2^-24 (exact, Sterbenz) leaves u = (2k + 1) 2^-24. Its complement
    // (2^24 - 2k - 1) 2^-24 has 24 significant bits at most, so 1 - u is exact too.
    const float one_minus = 0x1.fffffep-1f;  // 1 - 2^-24
    const float u = __int_as_float(0x3F800000u | (r >> 9)) - one_minus;
    return {u, 1.0f - u};
}
__device__ __forceinline__ Uni<double> uni_d(uint32_t a, uint32_t b) {
    // u = (2k + 1) 2^-53 with k < 2^52; 1 - u has 53 significant bits at most: exact
    uint64_t k = (uint64_t(a >> 6) << 26) | uint64_t(b >> 6);
    const double u = (double(k) + 0.5) * 0x1p-52;
    return {u, 1.0 - u};
}

// the 23 bits of three Philox words that uni_f leaves unused (their low 9, 9 and 5 bits),
// placed where uni_f reads: an independent uniform without another Philox call
__device__ __forceinline__ uint32_t low_bits_word(uint32_t a, uint32_t b, uint32_t c) {
    return (a << 23) | ((b & 511u) << 14) | ((c & 511u) << 5);
}

// Key and step words of the stream: key = seed, counter = (slot, step lo, step hi, tag).
struct Rng {
    uint32_t k0, k1, s0, s1;
};
__device__ __forceinline__ Rng make_rng(const bz_params &p) {
    uint64_t st = p.step_ptr ? *p.step_ptr : p.step;
    return {uint32_t(p.seed), uint32_t(p.seed >> 32), uint32_t(st), uint32_t(st >> 32)};
}

// Four uniforms for (slot, step, tag): one Philox call (float) or two (double).
template <typename T> struct Draw4 { Uni<T> v[4]; };

__device__ __forceinline__ void draw4(const Rng &g, uint32_t slot, uint32_t tag, Draw4<float> &d) {
    u32x4 r = philox(slot, g.s0, g.s1, tag, g.k0, g.k1);
    d.v[0] = uni_f(r.x); d.v[1] = uni_f(r.y); d.v[2] = uni_f(r.z); d.v[3] = uni_f(r.w);
}
__device__ __forceinline__ void draw4(const Rng &g, uint32_t slot, uint32_t tag, Draw4<double> &d) {
    u32x4 a = philox(slot, g.s0, g.s1, tag, g.k0, g.k1);
    u32x4 b = philox(slot, g.s0, g.s1, tag | (1u << 8), g.k0, g.k1);
    d.v[0] = uni_d(a.x, a.y); d.v[1] = uni_d(a.z, a.w); d.v[2] = uni_d(b.x, b.y); d.v[3] = uni_d(b.z, b.w);
}
// the same draws with precomputed round keys
// (and a ninth uniform from the second draw's unused low bits)
__device__ __forceinline__ void draw4x2(const Rng &g, const uint32_t *rk0, const uint32_t *rk1, uint32_t slot,
                                        uint32_t tag_a, uint32_t tag_b, Draw4<float> &da, Draw4<float> &db,
                                        Uni<float> &low_b) {
    u32x4 a, b;
    philox_rk_x2<PUSH_ROUNDS>(slot, g.s0, g.s1, tag_a, tag_b, rk0, rk1, a, b);
    da.v[0] = uni_f(a.x); da.v[1] = uni_f(a.y); da.v[2] = uni_f(a.z); da.v[3] = uni_f(a.w);
    db.v[0] = uni_f(b.x); db.v[1] = uni_f(b.y); db.v[2] = uni_f(b.z); db.v[3] = uni_f(b.w);
    low_b = uni_f(low_bits_word(b.x, b.y, b.z));
}
__device__ __forceinline__ void draw4(const Rng &g, const uint32_t *rk0, const uint32_t *rk1, uint32_t slot,
                                      uint32_t tag, Draw4<float> &d) {
    u32x4 r = philox_rk<PUSH_ROUNDS>(slot, g.s0, g.s1, tag, rk0, rk1);
    d.v[0] = uni_f(r.x); d.v[1] = uni_f(r.y); d.v[2] = uni_f(r.z); d.v[3] = uni_f(r.w);
}
__device__ __forceinline__ void draw4(const Rng &g, const uint32_t *rk0, const uint32_t *rk1, uint32_t slot,
                                      uint32_t tag, Draw4<double> &d) {
    u32x4 a = philox_rk<PUSH_ROUNDS>(slot, g.s0, g.s1, tag, rk0, rk1);
    u32x4 b = philox_rk<PUSH_ROUNDS>(slot, g.s0, g.s1, tag | (1u << 8), rk0, rk1);
    d.v[0] = uni_d(a.x, a.y); d.v[1] = uni_d(a.z, a.w); d.v[2] = uni_d(b.x, b.y); d.v[3] = uni_d(b.z, b.w);
}

// The hardware approximations (one MUFU instruction each) in their flush-to-zero forms:
// without .ftz a subnormal input is first scaled into the normal range, which costs several
// instructions per call. Every caller here passes a normal number, or one whose flush to
// zero gives the same result downstream (stated at the call), and for normal inputs the two
// forms return the same value.
__device__ __forceinline__ float lg2_ftz(float x) {
    float y;
    asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float ex2_ftz(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float rsqrt_ftz(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float rcp_ftz(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float sin_ftz(float x) {
    float y;
    asm("sin.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float cos_ftz(float x) {
    float y;
    asm("cos.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

__device__ __forceinline__ void sincospi_t(float a, float *s, float *c) { sincospif(a, s, c); }
__device__ __forceinline__ void sincospi_t(double a, double *s, double *c) { sincospi(a, s, c); }

// sin and cos of 2*pi*u, u in (0,1). float: the hardware approximation on the argument
// reduced to (-pi, pi), where its absolute error is below 2^-21.4 (sin(2 pi u) =
// -sin(2 pi (u - 1/2))); double: sincospi.
__device__ __forceinline__ void sincos2pi(float u, float *s, float *c) {
    const float a = 6.28318530717958647692f * (u - 0.5f);  // |a| < pi: normal or zero
    *s = -sin_ftz(a);
    *c = -cos_ftz(a);
}
__device__ __forceinline__ void sincos2pi(double u, double *s, double *c) { sincospi(2.0 * u, s, c); }

// w > min_wt as the reference tests it in float64: for float32 w the same as
// w >= wmin_f, the smallest float above min_wt (formed on the host)
__device__ __forceinline__ bool above_min(float w, double, float wmin_f) { return w >= wmin_f; }
__device__ __forceinline__ bool above_min(double w, double min_wt, float) { return w > min_wt; }

static inline float float_above(double m) {
    float t = float(m);
    if (double(t) <= m) t = nextafterf(t, INFINITY);
    return t;
}

// square root of a positive argument: x * rsqrt(x) in float (relative error ~1e-7),
// correctly rounded in double
// (float callers pass squared speeds floored at 1e-30, energies above a threshold and
// products of two uniforms: normal numbers)
__device__ __forceinline__ float sqrt_pos(float x) { return x * rsqrt_ftz(x); }
__device__ __forceinline__ double sqrt_pos(double x) { return sqrt(x); }

// Two standard normals times sigma from two float uniforms by Box-Muller (radius
// sqrt(-2 ln a), angle 2 pi b), with the hardware log2, reciprocal root, sine and cosine.
// -ln a comes from the log2 where a <= 1 - 2^-6 (|ln a| > 0.0157: the log2's absolute error
// of 2^-22.6 is then below 1e-5 of it) and from the series of -ln(1 - c) in the exact
// complement c = 1 - a above (relative truncation error c^4 / 5 < 1.2e-8), so the radius
// keeps its relative accuracy down to the smallest one; both are normal numbers (a <= 1 -
// 2^-24), as x rsqrt(x) needs.
__device__ __forceinline__ void box_muller_f(Uni<float> a, Uni<float> b, float sigma, float &g0, float &g1) {
    const float c = a.c;
    // 2 (c + c^2/2 + c^3/3 + c^4/4) = -2 ln(1 - c) for small c
    const float ser = c * fmaf(c, fmaf(c, fmaf(c, 0.5f, 0.6666667f), 1.0f), 2.0f);
    const float r2 = c < 0.015625f ? ser : -1.3862944f * lg2_ftz(a.u);  // -2 ln 2 log2(a)
    const float r = sigma * sqrt_pos(r2);
    float s, co;
    sincos2pi(b.u, &s, &co);
    g0 = r * co;
    g1 = r * s;
}

// Box-Muller pair from uniforms (a, b): r = sqrt(-2 ln a), angle 2 pi b.
template <typename T> __device__ __forceinline__ void box_muller(T a, T b, T &g0, T &g1) {
    T r = sqrt_pos(T(-2) * log(a));
    T s, c;
    sincos2pi(b, &s, &c);
    g0 = r * c;
    g1 = r * s;
}

// --------------------------------------------------------------------------------------
// Reference index arithmetic, exact. The reference forms these in float64 from
// float64 positions; here x is float32 or float64. A float32 candidate is used
// unless it lies near a boundary, where the float64 expression is evaluated.
// --------------------------------------------------------------------------------------
// The float candidate s carries a relative error below 2^-23 (~1.2e-7): the float
// reciprocal or slope and the product or fma are each rounded once to float, and the
// float64 expression itself is within a few 2^-53 of the exact value. mag bounds the
// magnitudes that were summed into s (|s| when nothing cancels), so a distance from s
// to the nearest integer above 2.5e-7*mag + 1e-7 (twice the bound, plus room for the
// roundings of the test itself) guarantees that truncating s gives the float64 result.
__device__ __forceinline__ bool safe_trunc(float s, float mag) {
    float fr = s - floorf(s);
    float m = fmaf(mag, 2.5e-7f, 1e-7f);
    return fr > m && fr < 1.0f - m;
}
// int(x / dx) (boltzmann.py:657): E-field face of the pre-push position.
template <typename T> __device__ __forceinline__ int face_index(T x, double dx, float inv_dx_f) {
    if (sizeof(T) == 4) {
        float s = float(x) * inv_dx_f;
        if (safe_trunc(s, fabsf(s))) return int(s);
    }
    return int(double(x) / dx);
}
// int((x + 0.5 dx) / dx) (boltzmann.py:658): binning cell.
template <typename T> __device__ __forceinline__ int cell_index(T x, double dx, float inv_dx_f) {
    if (sizeof(T) == 4) {
        float s = fmaf(float(x), inv_dx_f, 0.5f);
        if (safe_trunc(s, fmaf(fabsf(float(x)), inv_dx_f, 0.5f))) return int(s);
    }
    return int((double(x) + 0.5 * dx) / dx);
}
// int(int(((x + dx/2)/(L+dx)) * float(M)) / bnf) (post_processing_1D.py:44, kernels-new.cu:65,
// redcheck block = fine / bnf): deposit node.
struct NodeMap {
    double half_dx, Lp, fM;  // 0.5*dx, L+dx, (double)(float)M
    float a, b;              // float candidate: node ~= x*a + b
    int bnf;
};
// formed on the host and passed to the kernels (its float64 divisions stay off the GPU)
inline NodeMap make_node_map(const bz_params &p) {
    NodeMap m;
    int M = p.bnf * p.n_nodes;
    m.half_dx = 0.5 * p.dx;
    m.Lp = p.L + p.dx;
    m.fM = double(float(M));
    m.a = float(m.fM / m.Lp / p.bnf);
    m.b = float(m.half_dx * m.fM / m.Lp / p.bnf);
    m.bnf = p.bnf;
    return m;
}
template <typename T> __device__ __forceinline__ int node_index(T x, const NodeMap &m);
// deposit node of a particle for each motion mode (out-of-range values are dropped by the
// callers; in an ensemble x is the swarm index)
template <typename T> __device__ __forceinline__ int deposit_node(int advect, T x, const NodeMap &m) {
    return advect == BZ_ADVECT_1D ? node_index(x, m) : (advect == BZ_ADVECT_ENSEMBLE ? int(x) : 0);
}
// the same for a position known to be positive (an alive particle: 0 < x < L)
template <typename T> __device__ __forceinline__ int node_index_pos(T x, const NodeMap &m);
template <typename T> __device__ __forceinline__ int deposit_node_pos(int advect, T x, const NodeMap &m) {
    return advect == BZ_ADVECT_1D ? node_index_pos(x, m) : (advect == BZ_ADVECT_ENSEMBLE ? int(x) : 0);
}
// binning cell of a particle for each motion mode
template <typename T> __device__ __forceinline__ int bin_cell(int advect, T x, double dx, float inv_dx_f) {
    return advect == BZ_ADVECT_1D ? cell_index(x, dx, inv_dx_f) : (advect == BZ_ADVECT_ENSEMBLE ? int(x) : 0);
}
template <typename T> __device__ __forceinline__ int node_index(T x, const NodeMap &m) {
    if (sizeof(T) == 4) {
        float s = fmaf(float(x), m.a, m.b);
        if (safe_trunc(s, fmaf(fabsf(float(x)), m.a, m.b))) return int(s);
    }
    double tx = (double(x) + m.half_dx) / m.Lp;
    int fine = int(tx * m.fM);
    return fine / m.bnf;
}
template <typename T> __device__ __forceinline__ int node_index_pos(T x, const NodeMap &m) {
    if (sizeof(T) == 4) {
        const float s = fmaf(float(x), m.a, m.b);  // x > 0 and m.a, m.b > 0: nothing cancels
        if (safe_trunc(s, s)) return int(s);
    }
    double tx = (double(x) + m.half_dx) / m.Lp;
    int fine = int(tx * m.fM);
    return fine / m.bnf;
}

// --------------------------------------------------------------------------------------
// Decoupled look-back over tiles for two counters (survivors, children).
// status word: [63:62] flag (1 aggregate, 2 inclusive prefix), [61:31] c, [30:0] s.
// --------------------------------------------------------------------------------------
constexpr uint64_t LB_AGG = 1ull << 62;
constexpr uint64_t LB_PRE = 2ull << 62;
constexpr uint64_t LB_MASK = (1ull << 31) - 1;

__device__ __forceinline__ void st_release(uint64_t *p, uint64_t v) {
    asm volatile("st.release.gpu.global.b64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ uint64_t ld_acquire(const uint64_t *p) {
    uint64_t v;
    asm volatile("ld.acquire.gpu.global.b64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ uint64_t lb_pack(uint64_t flag, uint32_t s, uint32_t c) {
    return flag | (uint64_t(c & LB_MASK) << 31) | uint64_t(s & LB_MASK);
}

// Iteration limits of the bounded device-side waits: each wait's own default, overridden
// process-wide by bz_set_wait_limit (0 keeps the defaults); launches pass the value.
constexpr uint32_t WAIT_LIMIT_DEFAULT = 1u << 22;  // look-back polls
uint32_t host_wait_limit(uint32_t dflt = WAIT_LIMIT_DEFAULT);

// Called by warp 0 of the block that owns ``tile``. Publishes (s, c) as the tile
// aggregate, waits for predecessors (at most ``wait_limit`` polls in all), publishes the
// inclusive prefix and returns the exclusive prefix in (*ps, *pc) on lane 0. A wait that
// runs out counts the missing tiles as empty and raises BZ_DEV_LOOKBACK.
__device__ inline void lookback(uint64_t *status_arr, int tile, uint32_t s, uint32_t c, uint32_t *ps, uint32_t *pc,
                                uint32_t *err, uint32_t wait_limit) {
    const int lane = threadIdx.x & 31;
    if (tile == 0) {
        if (lane == 0) {
            st_release(&status_arr[0], lb_pack(LB_PRE, s, c));
            *ps = 0; *pc = 0;
        }
        return;
    }
    if (lane == 0) st_release(&status_arr[tile], lb_pack(LB_AGG, s, c));
    uint32_t acc_s = 0, acc_c = 0;
    int base = tile - 1;
    uint32_t spins = 0;
    bool timed_out = false;
    while (true) {
        int t = base - lane;
        uint64_t v = (t >= 0) ? ld_acquire(&status_arr[t]) : LB_PRE;  // before tile 0: empty prefix
        uint64_t flag = v & (3ull << 62);
        unsigned pre = __ballot_sync(0xffffffffu, flag == LB_PRE);
        int stop = pre ? (__ffs(pre) - 1) : 31;  // nearest predecessor holding an inclusive prefix
        unsigned needed = (stop == 31) ? 0xffffffffu : ((1u << (stop + 1)) - 1u);
        unsigned not_ready = __ballot_sync(0xffffffffu, flag == 0) & needed;
        if (not_ready && !timed_out) {
            if (++spins > wait_limit) {
                timed_out = true;  // give up waiting: count missing tiles as empty, flag it
                if (lane == 0) atomicOr(err, BZ_DEV_LOOKBACK);
            } else {
                __nanosleep(64);
                continue;
            }
        }
        uint32_t vs = uint32_t(v & LB_MASK), vc = uint32_t((v >> 31) & LB_MASK);
        if (lane > stop || flag == 0) { vs = 0; vc = 0; }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            vs += __shfl_xor_sync(0xffffffffu, vs, o);
            vc += __shfl_xor_sync(0xffffffffu, vc, o);
        }
        acc_s += vs;
        acc_c += vc;
        if (pre) break;
        base -= 32;
    }
    if (lane == 0) {
        st_release(&status_arr[tile], lb_pack(LB_PRE, acc_s + s, acc_c + c));
        *ps = acc_s;
        *pc = acc_c;
    }
}

__host__ __device__ inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// The resampling trigger of one (cell, bin) key with n particles and target T
// (boltzmann.py:894-916; 3bin :1063-1113, 5bin :1256-1334): too few (0 < n < split_below T)
// or too many (n >= merge_at T) sets need_any; too many in the last bin sets need_last,
// the one test that decides under BZ_QUIRK_TRIGGER_LAST.
__device__ __forceinline__ void rs_key_need(int64_t n, int64_t T, bool last_bin, double split_below, double merge_at,
                                            int &need_any, int &need_last) {
    if (n > 0 && double(n) < split_below * double(T)) need_any = 1;
    if (double(n) >= merge_at * double(T)) {
        need_any = 1;
        if (last_bin) need_last = 1;
    }
}

inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

}  // namespace bz
