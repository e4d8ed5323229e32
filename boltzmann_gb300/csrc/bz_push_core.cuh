// Shared pieces of the electron push: per-particle push + Monte-Carlo collision
// (electron_kernel_numba.py:38-287), used by the dense, reference-ordered push
// (bz_push.cu) and by the segmented push of the solver (bz_segments.cu).
#pragma once
#include <algorithm>

#include "bz_common.cuh"

namespace bz {

constexpr int PT = 256;            // threads per CTA
constexpr int PI = 4;              // consecutive particles per thread per tile
constexpr int PTILE = PT * PI;     // particles per tile
constexpr int PWARPS = PT / 32;

template <typename T> struct SoA { T *x, *vx, *vy, *vz, *w; };

// The reference's cross-section fits (electron_kernel_numba.py:66-174), float64.
static __constant__ double c_el_a[12] = {-0.02704763, -0.08847237, -0.37608274, -1.4874467, -0.9870356, 14.28063581,
                                  -2.12069169, -0.3585636, 1.25262128, -2.28332905, -1.47508661, -0.11090525};
static __constant__ double c_el_b[12] = {-0.23720051, -0.6084786, -1.8167778, -4.82420619, -4.2206026, 18.92275458,
                                  0.7555105, 0.79246666, -0.40002029, 4.89566076, 2.82263476, -0.77506081};
static __constant__ double c_el_c[12] = {-19.67900951, -20.24111992, -21.51414308, -23.55745478, -23.44715988,
                                  -14.70556113, -19.71943671, -19.71260274, -19.48909003, -21.46789173,
                                  -20.1928456, -17.81752307};
static __constant__ double c_el_e[11] = {0.000780396, 0.006098667, 0.0476269, 0.1015574, 0.1943527, 0.2995781,
                                  1.097156, 2.339524, 4.988691, 10.63765, 22.68322};
static __constant__ double c_io_a[8] = {-2149239.99337822, -227229.83440255, -20173.68563579, -1838.90888364,
                                 -186.98923927, -24.48843901, -4.33101714, -0.68345667};
static __constant__ double c_io_b[8] = {5150451.29014456, 545171.14839945, 48599.13254342, 4491.58838596,
                                 477.04784782, 69.43965607, 14.47124519, 2.6053539};
static __constant__ double c_io_c[8] = {-3085665.64874862, -327016.69508374, -29290.96100603, -2763.82866252,
                                 -324.75732578, -69.145292411, -31.66224458, -21.99823511};
static __constant__ double c_io_e[7] = {15.77742, 15.81964, 15.96196, 16.44162, 18.05837, 23.50771, 41.87498};

__device__ inline void sigma_fits(double e, double &s_el, double &s_ion) {
    double le = log10(e);
    int k = 0;
    while (k < 11 && !(e < c_el_e[k])) ++k;
    s_el = pow(10.0, (c_el_a[k] * le + c_el_b[k]) * le + c_el_c[k]);
    double lg = 0.0;  // at e == 15.76 no piece matches and the reference's sum is 0
    if (E_ION < e && e < c_io_e[0]) {
        lg = (c_io_a[0] * le + c_io_b[0]) * le + c_io_c[0];
    } else {
        for (int j = 1; j < 8; ++j) {
            bool hi_ok = (j == 7) || (e < c_io_e[j]);
            if (c_io_e[j - 1] <= e && hi_ok) { lg = (c_io_a[j] * le + c_io_b[j]) * le + c_io_c[j]; break; }
        }
    }
    double s2 = pow(10.0, lg);
    s_ion = (e < E_ION) ? 0.0 : s2;
}

// Per-launch constants derived on the host.
template <typename T> struct PushConst {
    T efac;         // 0.5 m_e j_ev: |v|^2 (m^2/s^2) -> eV
    T c100dt;       // 100 dt: m/s -> cm per step
    T kick;         // dt (q/m) 100: V/cm -> m/s per step
    T f_el;         // sqrt(1 - 2 m_e/m_n)
    T e2v;          // 2/(j_ev m_e): eV -> (m/s)^2
    T gas_sigma;
    T L;
    float inv_dx_f;
    float xs_inv_d, xs_off;  // t = log2(e)*xs_inv_d - xs_off
    double efac_d, e2v_d, c100dt_d;
    T p_null;       // 1 - exp(-dt nu_max) (null collision)
    T inv_nu_max;
    T dt, e_exc;    // dt and the excitation threshold in the working precision
    NodeMap nm;     // deposit node map
    uint32_t rk0[10], rk1[10];  // Philox round keys of the seed
    float efac_h, efac_l;       // 0.5 m_e j_ev as an unevaluated sum of two floats
    float exc_h, exc_l, ion_h, ion_l;  // the excitation and ionization thresholds, likewise
    T wall_lo, wall_hi;         // L*1e-3, L*(1-1e-3): closer to a wall the float64 test decides
    float xs_last;              // xs_n - 1 (float), the table's last index
    int xs_imax, face_max;      // xs_n - 2, n_faces - 1
};

template <typename T> struct Item {
    T x, vx, vy, vz;      // state after the step (w unchanged)
    T cx, cvx, cvy, cvz;  // child
    T e, ce;              // energies (eV) after the step, for the deposit
    bool alive, child, ionized, excited;
};

template <typename T>
__device__ __forceinline__ void iso_dir(Uni<T> a, Uni<T> b, T vn, T &vx, T &vy, T &vz) {
    // cos(chi) = 2a-1, sin(chi) = 2 sqrt(a(1-a)), phi = 2 pi b (electron_kernel_numba.py:202-209)
    T cc = a.u - a.c;
    T sc = T(2) * sqrt_pos(a.u * a.c);
    T sp, cp;
    sincos2pi(b.u, &sp, &cp);
    vx = vn * sc * cp;
    vy = vn * sc * sp;
    vz = vn * cc;
}

// e - thr for a float32 relative velocity (ax, ay, az) without the cancellation of a float
// subtraction: the squared speed and the energy as unevaluated sums of two floats (exact
// products by fma and exact sums, Dekker 1971 / Knuth TAOCP 4.2.2), then the threshold's
// high part subtracted exactly (both within a factor of two: Sterbenz). Absolute error
// about 1e-14 e. The rounded operations are spelled out so that none is contracted.
__device__ __forceinline__ float excess_energy_f(float ax, float ay, float az, float efh, float efl, float th,
                                                 float tl) {
    const float p1 = __fmul_rn(ax, ax), e1 = fmaf(ax, ax, -p1);
    const float p2 = __fmul_rn(ay, ay), e2 = fmaf(ay, ay, -p2);
    const float p3 = __fmul_rn(az, az), e3 = fmaf(az, az, -p3);
    const float s1 = __fadd_rn(p1, p2), b1 = __fsub_rn(s1, p1);
    const float t1 = __fadd_rn(__fsub_rn(p1, __fsub_rn(s1, b1)), __fsub_rn(p2, b1));
    const float s2 = __fadd_rn(s1, p3), b2 = __fsub_rn(s2, s1);
    const float t2 = __fadd_rn(__fsub_rn(s1, __fsub_rn(s2, b2)), __fsub_rn(p3, b2));
    const float vh = s2, vl = __fadd_rn(__fadd_rn(__fadd_rn(t1, t2), __fadd_rn(e1, e2)), e3);
    const float eh = __fmul_rn(efh, vh);
    const float el = __fadd_rn(fmaf(efh, vh, -eh), fmaf(efh, vl, __fmul_rn(efl, vh)));
    return __fadd_rn(__fsub_rn(eh, th), __fsub_rn(el, tl));
}

// 1 - exp(-x), x >= 0. float: the hardware exponential, absolute error ~2e-7 (the
// collision test compares this probability with a uniform, so an absolute error is what
// matters); double: expm1.
// (exp(-x) = 2^(-x log2 e); a result flushed to zero leaves P = 1, as its float32 value is)
__device__ __forceinline__ float coll_prob(float x) { return 1.0f - ex2_ftz(x * -1.4426950408889634f); }
__device__ __forceinline__ double coll_prob(double x) { return -expm1(-x); }

__device__ __forceinline__ float fdiv_fast(float a, float b) { return a * rcp_ftz(b); }  // b: a normal sum of n sigma
__device__ __forceinline__ double fdiv_fast(double a, double b) { return a / b; }

template <typename T> __device__ __forceinline__ Uni<T> uni_from_replay(double r) {
    return {T(r), T(1.0 - r)};
}

enum { P_NONE = 0, P_ELASTIC = 1, P_EXCITE = 2, P_IONIZE = 3 };

// The reference's test (electron_kernel_numba.py:195-212): elastic if u < r0, then the
// next process if r0 < u < r1, and so on; strict inequalities as in the reference.
template <typename U> __device__ __forceinline__ int choose(U u, U r0, U r1, U r2) {
    if (u < r0) return P_ELASTIC;
    if (r0 < u && u < r1) return P_EXCITE;
    if (r1 < u && u < r2) return P_IONIZE;
    return P_NONE;
}

// ADV >= 0: the motion mode (ADV) and the direct collision probability fixed at compile time
template <typename T, bool REPLAY, int XS, int ADV = -1>
__device__ __forceinline__ void push_item(const bz_params &p, const PushConst<T> &k, const Rng &rng, uint32_t slot, T x, T vx, T vy,
                                          T vz, const T *E_s, const float4 *xs_s, const double *R,
                                          const double *gas, Item<T> &o) {
    const int advect = ADV >= 0 ? ADV : p.advect;
    const int coll_model = ADV >= 0 ? int(BZ_COLL_DIRECT) : p.coll_model;
    // gas velocity (boltzmann.py:589, electron_kernel_numba.py:51-53) and uniforms
    T g0 = 0, g1 = 0, g2 = 0;
    Uni<T> u0, u1, u2, u3;
    Uni<T> u5{T(0.5), T(0.5)};  // the child's azimuth (float32: the collision draw's unused low bits)
    double r0_replay = 0.0;
    if (REPLAY) {
        g0 = T(gas[size_t(slot) * 3 + 0]);
        g1 = T(gas[size_t(slot) * 3 + 1]);
        g2 = T(gas[size_t(slot) * 3 + 2]);
        r0_replay = R[size_t(slot) * 7 + 0];
        u0 = uni_from_replay<T>(r0_replay);
        u1 = uni_from_replay<T>(R[size_t(slot) * 7 + 1]);
        u2 = uni_from_replay<T>(R[size_t(slot) * 7 + 2]);
        u3 = uni_from_replay<T>(R[size_t(slot) * 7 + 3]);
    } else {
        Draw4<T> dg, d;
        if constexpr (sizeof(T) == 4) {
            // gas-velocity and collision uniforms from one interleaved pair of Philox calls;
            // the ionization child's azimuth from the collision words' unused low bits (no
            // third Philox call)
            draw4x2(rng, k.rk0, k.rk1, slot, 0u, 1u, dg, d, u5);
        } else {
            draw4(rng, k.rk0, k.rk1, slot, 0u, dg);
            draw4(rng, k.rk0, k.rk1, slot, 1u, d);
        }
        if constexpr (sizeof(T) == 4) {
            // Box-Muller pairs from the gas draw's words (0, 1) and (2, 3), as in float64
            if (k.gas_sigma > T(0)) {
                float h;
                box_muller_f(dg.v[0], dg.v[1], k.gas_sigma, g0, g1);
                box_muller_f(dg.v[2], dg.v[3], k.gas_sigma, g2, h);
            }
        } else if (k.gas_sigma > T(0)) {
            T h;
            box_muller(dg.v[0].u, dg.v[1].u, g0, g1);
            box_muller(dg.v[2].u, dg.v[3].u, g2, h);
            g0 *= k.gas_sigma; g1 *= k.gas_sigma; g2 *= k.gas_sigma;
        }
        u0 = d.v[0]; u1 = d.v[1]; u2 = d.v[2]; u3 = d.v[3];
        r0_replay = double(u0.u);
    }
    // the field at the pre-push face (electron_kernel_numba.py:257-263), read first: it
    // depends on x only, and its shared-memory load overlaps the collision arithmetic
    int face = 0;
    if (advect == BZ_ADVECT_ENSEMBLE) {
        face = min(max(int(x), 0), k.face_max);
    } else if (advect) {
        face = face_index(x, p.dx, k.inv_dx_f);
        face = min(max(face, 0), k.face_max);
    }
    const T Ef = E_s[face];
    // energy of the gas-relative velocity (electron_kernel_numba.py:55-63)
    T ax = vx - g0, ay = vy - g1, az = vz - g2;
    T v2 = ax * ax + ay * ay + az * az;
    // (float: floored at 1e-30, a normal number, for the flush-to-zero reciprocal root)
    T vmag = sqrt_pos(sizeof(T) == 4 ? (v2 > T(1e-30) ? v2 : T(1e-30)) : (v2 > T(0) ? v2 : T(1e-30)));
    T e = k.efac * v2;
    int proc;
    if (XS == BZ_XS_REF_FITS) {
        // the reference's fits and collision test, in float64 (electron_kernel_numba.py:64-198)
        double ad = double(ax), bd = double(ay), cd = double(az);
        double v2d = ad * ad + bd * bd + cd * cd;
        double vm = sqrt(v2d);
        double ed = k.efac_d * v2d;
        double s0, s2;
        sigma_fits(ed, s0, s2);
        s0 *= p.nn;
        s2 *= p.nn;
        double q0, q2;
        if (coll_model == BZ_COLL_DIRECT) {
            double st = s0 + s2;
            double P = 1.0 - exp(-p.dt * vm * st);
            double pc = P * (1.0 / st);
            q0 = s0 * pc;
            q2 = q0 + s2 * pc;
        } else {
            double c = (1.0 - exp(-p.dt * p.nu_max)) * vm / p.nu_max;
            q0 = s0 * c;
            q2 = q0 + s2 * c;
        }
        proc = choose<double>(r0_replay, q0, q0, q2);
        vmag = T(vm);
    } else {
        // n*sigma table, linear in log2(e) on the log grid
        // (a subnormal energy flushes to log2 = -inf, which the clamp below turns into the
        // table's first point, where any energy below its start lands)
        float lt = fmaf(lg2_ftz(float(e)), k.xs_inv_d, -k.xs_off);
        lt = fminf(fmaxf(lt, 0.0f), k.xs_last);
        int i = min(int(lt), k.xs_imax);
        float f = lt - float(i);
        float4 a = xs_s[i], b = xs_s[i + 1];
        T s0 = T(fmaf(f, b.x - a.x, a.x));
        T s1 = T(fmaf(f, b.y - a.y, a.y));
        T s2 = T(fmaf(f, b.z - a.z, a.z));
        if (e < k.e_exc) s1 = T(0);
        if (e < T(E_ION)) s2 = T(0);
        T r0, r1, r2;
        if (coll_model == BZ_COLL_DIRECT) {
            T st = s0 + s1 + s2;
            T P = coll_prob(k.dt * vmag * st);
            T pc = fdiv_fast(P, st);
            r0 = s0 * pc;
            r1 = r0 + s1 * pc;
            r2 = r1 + s2 * pc;
        } else {
            T c = k.p_null * vmag * k.inv_nu_max;
            r0 = s0 * c;
            r1 = r0 + s1 * c;
            r2 = r1 + s2 * c;
        }
        proc = choose<T>(u0.u, r0, r1, r2);
    }
    o.child = false;
    o.ionized = false;
    o.excited = (proc == P_EXCITE);
    // speed after a collision: elastic |v| (1 - 2 m_e/m_n)^1/2 (electron_kernel_numba.py:197-209)
    T vn = vmag * k.f_el;
    if (proc >= P_EXCITE) {
        // energy left after the threshold: in the working precision when e - threshold
        // keeps at least a quarter of e, else without the subtraction's cancellation
        // (float32: two-float arithmetic; float64: the float64 expression);
        // excitation loses e_exc (the reference has no excitation: sigma_g1 = 0),
        // ionization shares e - 15.76 equally (electron_kernel_numba.py:211-255)
        // (the float thresholds are the float64 ones rounded on the host, so no float64
        // conversion runs here)
        const bool ex = proc == P_EXCITE;
        T thr;
        if constexpr (sizeof(T) == 4) thr = ex ? k.exc_h : k.ion_h;
        else thr = ex ? p.e_exc : E_ION;
        if (sizeof(T) == 8 || e - thr >= T(0.25) * e) {
            T en = ex ? (e - thr) : T(0.5) * (e - thr);
            vn = sqrt_pos(en * k.e2v);
        } else if constexpr (sizeof(T) == 4) {
            float d = fabsf(excess_energy_f(ax, ay, az, k.efac_h, k.efac_l, ex ? k.exc_h : k.ion_h,
                                            ex ? k.exc_l : k.ion_l));
            if (!ex) d = 0.5f * d;
            vn = sqrt_pos(d * k.e2v);
        }
    }
    // one isotropic redirection for every process, computed in every lane and kept where the
    // particle collided: with a collision probability of 0.2-0.3 per step nearly every warp
    // has a colliding lane, so a branch around it would save nothing
    T nvx, nvy, nvz;
    {
        T ix, iy, iz;
        iso_dir(u1, u2, vn, ix, iy, iz);
        const bool coll = proc != P_NONE;
        nvx = coll ? ix : vx;
        nvy = coll ? iy : vy;
        nvz = coll ? iz : vz;
    }
    if (proc == P_IONIZE) {
        // the new electron: same position and weight, its own isotropic direction
        if (REPLAY) {
            u5 = uni_from_replay<T>(R[size_t(slot) * 7 + 5]);
        } else if constexpr (sizeof(T) == 8) {
            Draw4<T> d;
            draw4(rng, k.rk0, k.rk1, slot, 2u, d);
            u5 = d.v[0];
        }
        iso_dir(u3, u5, vn, o.cvx, o.cvy, o.cvz);
        o.cx = x;
        o.child = true;
        o.ionized = true;
        o.ce = k.efac * (o.cvx * o.cvx + o.cvy * o.cvy + o.cvz * o.cvz);
    }
    // drift with the post-collision velocity, kick with E at the pre-push face,
    // absorbing walls (electron_kernel_numba.py:257-276)
    T xn = x;
    bool valid = true;
    if (advect == BZ_ADVECT_1D) {
        xn = x + k.c100dt * nvx;
        if (xn < k.wall_lo || xn > k.wall_hi) {
            // near a wall: decide in float64 like the reference
            double xd = double(x) + k.c100dt_d * double(nvx);
            valid = (0.0 < xd) && (xd < p.L);
            xn = T(xd);
        }
    }
    nvx -= k.kick * Ef;
    o.alive = valid;
    o.x = xn; o.vx = nvx; o.vy = nvy; o.vz = nvz;
    o.e = k.efac * (nvx * nvx + nvy * nvy + nvz * nvz);
}

template <typename T> struct AccT { using t = T; };

static int g_num_sms = 0;
inline int num_sms() {
    if (g_num_sms == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
        if (g_num_sms <= 0) g_num_sms = 1;
    }
    return g_num_sms;
}

template <typename T> inline PushConst<T> make_push_const(const bz_params &p) {
    PushConst<T> k;
    double me = m_e(), jev = j_ev(), qe = q_e(), mn = m_n();
    k.efac = T(0.5 * me * jev);
    k.efac_d = 0.5 * me * jev;
    k.c100dt = T(100 * p.dt);
    k.c100dt_d = 100 * p.dt;
    k.kick = T(p.dt * (qe / me) * 100);
    k.f_el = T(sqrt(1 - (2 * me / mn)));
    k.e2v = T(2.0 / (jev * me));
    k.e2v_d = 2.0 / (jev * me);
    auto split = [](double v, float &h, float &l) { h = float(v); l = float(v - double(h)); };
    split(k.efac_d, k.efac_h, k.efac_l);
    split(p.e_exc, k.exc_h, k.exc_l);
    split(E_ION, k.ion_h, k.ion_l);
    k.gas_sigma = T(p.gas_sigma);
    k.L = T(p.L);
    k.inv_dx_f = float(1.0 / p.dx);
    if (p.xs_n >= 2 && p.xs_emax > p.xs_emin && p.xs_emin > 0) {
        double inv_d = double(p.xs_n - 1) / log2(p.xs_emax / p.xs_emin);
        k.xs_inv_d = float(inv_d);
        k.xs_off = float(log2(p.xs_emin) * inv_d);
    } else {
        k.xs_inv_d = 0.f;
        k.xs_off = 0.f;
    }
    k.p_null = T(p.nu_max > 0 ? -expm1(-p.dt * p.nu_max) : 0.0);
    k.inv_nu_max = T(p.nu_max > 0 ? 1.0 / p.nu_max : 0.0);
    k.dt = T(p.dt);
    k.e_exc = T(p.e_exc);
    k.nm = make_node_map(p);
    philox_round_keys(p.seed, k.rk0, k.rk1);
    k.wall_lo = T(p.L) * T(1e-3);
    k.wall_hi = T(p.L) * T(1 - 1e-3);
    k.xs_last = float(p.xs_n - 1);
    k.xs_imax = p.xs_n - 2;
    k.face_max = p.n_faces - 1;
    return k;
}

// The dense push through the segmented kernel (bz_segments.cu): BZ_ERR_WORKSPACE when the
// workspace is smaller than bz_push_workspace_fast_*, and the caller pushes with k_push.
template <typename T>
int dense_push_segmented(const bz_params &p, SoA<T> in, const int32_t *n_in, int64_t in_cap, SoA<T> out, int64_t cap,
                         int32_t *counts, const T *E, const double *R, const double *gas, double *moments, void *ws,
                         size_t ws_bytes, uint32_t *status, cudaStream_t st);

}  // namespace bz
