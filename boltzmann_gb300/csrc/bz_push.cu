// Fused electron push + Monte-Carlo collision + moment deposit + compaction.
//
// One persistent launch per step. Each CTA takes tiles of PTILE particles from an
// atomic ticket, so a tile's predecessors are always running or done and the
// decoupled look-back that orders the output cannot wait on an unscheduled CTA.
// Per particle (electron_kernel_numba.py:38-287): gas-velocity subtraction, energy,
// cross sections (n*sigma table in shared memory, or the reference's fits in FP64),
// collision test and process choice, isotropic scatter (elastic / excitation /
// ionization with an appended child), drift with the post-collision velocity, kick
// with E at the pre-push face, absorbing walls. Survivors are written in input order
// and children in parent order after them, the order reshuffle_data_atomics
// (post_processing_1D.py:26-38) leaves. The deposit of post_processing
// (post_processing_1D.py:44-57, kernels-new.cu:56-132) is accumulated in a per-CTA
// shared-memory grid and merged into the float64 moments once per CTA.
#include <algorithm>
#include <cstdio>
#include <mutex>

#include "bz_common.cuh"

namespace bz {

constexpr int PT = 256;            // threads per CTA
constexpr int PI = 4;              // consecutive particles per thread per tile
constexpr int PTILE = PT * PI;     // particles per tile
constexpr int PWARPS = PT / 32;

template <typename T> struct SoA { T *x, *vx, *vy, *vz, *w; };

// The reference's cross-section fits (electron_kernel_numba.py:66-174), float64.
__constant__ double c_el_a[12] = {-0.02704763, -0.08847237, -0.37608274, -1.4874467, -0.9870356, 14.28063581,
                                  -2.12069169, -0.3585636, 1.25262128, -2.28332905, -1.47508661, -0.11090525};
__constant__ double c_el_b[12] = {-0.23720051, -0.6084786, -1.8167778, -4.82420619, -4.2206026, 18.92275458,
                                  0.7555105, 0.79246666, -0.40002029, 4.89566076, 2.82263476, -0.77506081};
__constant__ double c_el_c[12] = {-19.67900951, -20.24111992, -21.51414308, -23.55745478, -23.44715988,
                                  -14.70556113, -19.71943671, -19.71260274, -19.48909003, -21.46789173,
                                  -20.1928456, -17.81752307};
__constant__ double c_el_e[11] = {0.000780396, 0.006098667, 0.0476269, 0.1015574, 0.1943527, 0.2995781,
                                  1.097156, 2.339524, 4.988691, 10.63765, 22.68322};
__constant__ double c_io_a[8] = {-2149239.99337822, -227229.83440255, -20173.68563579, -1838.90888364,
                                 -186.98923927, -24.48843901, -4.33101714, -0.68345667};
__constant__ double c_io_b[8] = {5150451.29014456, 545171.14839945, 48599.13254342, 4491.58838596,
                                 477.04784782, 69.43965607, 14.47124519, 2.6053539};
__constant__ double c_io_c[8] = {-3085665.64874862, -327016.69508374, -29290.96100603, -2763.82866252,
                                 -324.75732578, -69.145292411, -31.66224458, -21.99823511};
__constant__ double c_io_e[7] = {15.77742, 15.81964, 15.96196, 16.44162, 18.05837, 23.50771, 41.87498};

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
};

template <typename T> struct Item {
    T x, vx, vy, vz;      // state after the step (w unchanged)
    T cx, cvx, cvy, cvz;  // child
    T e, ce;              // energies (eV) after the step, for the deposit
    bool alive, child, ionized;
};

template <typename T>
__device__ __forceinline__ void iso_dir(Uni<T> a, Uni<T> b, T vn, T &vx, T &vy, T &vz) {
    // cos(chi) = 2a-1, sin(chi) = 2 sqrt(a(1-a)), phi = 2 pi b (electron_kernel_numba.py:202-209)
    T cc = a.u - a.c;
    T sc = T(2) * sqrt(a.u * a.c);
    T sp, cp;
    sincos2pi(b.u, &sp, &cp);
    vx = vn * sc * cp;
    vy = vn * sc * sp;
    vz = vn * cc;
}

__device__ __forceinline__ float fdiv_fast(float a, float b) { return __fdividef(a, b); }
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

template <typename T, bool REPLAY, int XS>
__device__ __forceinline__ void push_item(const bz_params &p, const PushConst<T> &k, const Rng &rng, uint32_t slot, T x, T vx, T vy,
                                          T vz, const T *E_s, const float4 *xs_s, const double *R,
                                          const double *gas, Item<T> &o) {
    // gas velocity (boltzmann.py:589, electron_kernel_numba.py:51-53) and uniforms
    T g0 = 0, g1 = 0, g2 = 0;
    Uni<T> u0, u1, u2, u3;
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
        if (k.gas_sigma > T(0)) {
            Draw4<T> d;
            draw4(rng, slot, 0u, d);
            T h;
            box_muller(d.v[0].u, d.v[1].u, g0, g1);
            box_muller(d.v[2].u, d.v[3].u, g2, h);
            g0 *= k.gas_sigma; g1 *= k.gas_sigma; g2 *= k.gas_sigma;
        }
        Draw4<T> d;
        draw4(rng, slot, 1u, d);
        u0 = d.v[0]; u1 = d.v[1]; u2 = d.v[2]; u3 = d.v[3];
        r0_replay = double(u0.u);
    }
    // energy of the gas-relative velocity (electron_kernel_numba.py:55-63)
    T ax = vx - g0, ay = vy - g1, az = vz - g2;
    T v2 = ax * ax + ay * ay + az * az;
    T vmag = sqrt(v2);
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
        if (p.coll_model == BZ_COLL_DIRECT) {
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
        float lt = fmaf(__log2f(float(e)), k.xs_inv_d, -k.xs_off);
        lt = fminf(fmaxf(lt, 0.0f), float(p.xs_n - 1));
        int i = min(int(lt), p.xs_n - 2);
        float f = lt - float(i);
        float4 a = xs_s[i], b = xs_s[i + 1];
        T s0 = T(fmaf(f, b.x - a.x, a.x));
        T s1 = T(fmaf(f, b.y - a.y, a.y));
        T s2 = T(fmaf(f, b.z - a.z, a.z));
        if (e < T(p.e_exc)) s1 = T(0);
        if (e < T(E_ION)) s2 = T(0);
        T r0, r1, r2;
        if (p.coll_model == BZ_COLL_DIRECT) {
            T st = s0 + s1 + s2;
            T P = -expm1(-T(p.dt) * vmag * st);
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
    T nvx = vx, nvy = vy, nvz = vz;
    if (proc == P_ELASTIC) {
        // |v| (1 - 2 m_e/m_n)^1/2, isotropic (electron_kernel_numba.py:197-209)
        iso_dir(u1, u2, vmag * k.f_el, nvx, nvy, nvz);
    } else if (proc != P_NONE) {
        // energy left after the threshold: in the working precision when e - threshold
        // keeps at least a quarter of e, else in float64 (the subtraction cancels)
        const double thr = (proc == P_EXCITE) ? p.e_exc : E_ION;
        T vn;
        if (sizeof(T) == 8 || e - T(thr) >= T(0.25) * e) {
            T en = (proc == P_EXCITE) ? (e - T(thr)) : T(0.5) * (e - T(thr));
            vn = sqrt(en * k.e2v);
        } else {
            double ed = k.efac_d * (double(ax) * double(ax) + double(ay) * double(ay) + double(az) * double(az));
            double en = (proc == P_EXCITE) ? fabs(ed - thr) : fabs(0.5 * (ed - thr));
            vn = T(sqrt(en * k.e2v_d));
        }
        if (proc == P_EXCITE) {
            // lose e_exc, isotropic (the reference has no excitation: sigma_g1 = 0)
            iso_dir(u1, u2, vn, nvx, nvy, nvz);
        } else {
            // ionization, equal sharing of e - 15.76 (electron_kernel_numba.py:211-255)
            iso_dir(u1, u2, vn, nvx, nvy, nvz);
            Uni<T> u5;
            if (REPLAY) {
                u5 = uni_from_replay<T>(R[size_t(slot) * 7 + 5]);
            } else {
                Draw4<T> d;
                draw4(rng, slot, 2u, d);
                u5 = d.v[0];
            }
            iso_dir(u3, u5, vn, o.cvx, o.cvy, o.cvz);
            o.cx = x;
            o.child = true;
            o.ionized = true;
            o.ce = k.efac * (o.cvx * o.cvx + o.cvy * o.cvy + o.cvz * o.cvz);
        }
    }
    // drift with the post-collision velocity, kick with E at the pre-push face,
    // absorbing walls (electron_kernel_numba.py:257-276)
    T xn = x;
    int face = 0;
    bool valid = true;
    if (p.advect) {
        xn = x + k.c100dt * nvx;
        face = face_index(x, p.dx, k.inv_dx_f);
        face = min(max(face, 0), p.n_faces - 1);
        if (xn < k.L * T(1e-3) || xn > k.L * T(1 - 1e-3)) {
            // near a wall: decide in float64 like the reference
            double xd = double(x) + k.c100dt_d * double(nvx);
            valid = (0.0 < xd) && (xd < p.L);
            xn = T(xd);
        }
    }
    nvx -= k.kick * E_s[face];
    o.alive = valid;
    o.x = xn; o.vx = nvx; o.vy = nvy; o.vz = nvz;
    o.e = k.efac * (nvx * nvx + nvy * nvy + nvz * nvz);
}

template <typename T> struct AccT { using t = T; };

template <typename T, bool REPLAY, int XS, bool DEPOSIT>
#ifndef BZ_PUSH_MINB
#define BZ_PUSH_MINB 3
#endif
__global__ void __launch_bounds__(PT, BZ_PUSH_MINB) k_push(bz_params p, PushConst<T> kc, SoA<T> in, const int32_t *n_in,
                                             int64_t in_cap, SoA<T> out, int64_t cap, int32_t *counts, const T *E,
                                             const double *R, const double *gas, double *moments,
                                             unsigned int *ticket, uint64_t *tile_status, int max_tiles,
                                             uint32_t *status) {
    using A = typename AccT<T>::t;
    extern __shared__ __align__(16) unsigned char smem[];
    const int nf = p.advect ? p.n_faces : 1;
    const int nnodes = p.n_nodes;
    const int xsn = (XS == BZ_XS_TABLE) ? p.xs_n : 0;
    float4 *xs_s = reinterpret_cast<float4 *>(smem);
    A *mom_s = reinterpret_cast<A *>(smem + size_t(xsn) * sizeof(float4));
    T *E_s = reinterpret_cast<T *>(reinterpret_cast<unsigned char *>(mom_s) + (DEPOSIT ? size_t(3) * nnodes * sizeof(A) : 0));
    __shared__ int s_tile;
    __shared__ uint32_t s_ps, s_pc;
    __shared__ uint32_t s_warp[PWARPS];

    for (int i = threadIdx.x; i < nf; i += PT) E_s[i] = E[i];
    if (XS == BZ_XS_TABLE)
        for (int i = threadIdx.x; i < xsn; i += PT)
            xs_s[i] = make_float4(p.xs_table[i], p.xs_table[xsn + i], p.xs_table[2 * xsn + i], 0.0f);
    if (DEPOSIT)
        for (int i = threadIdx.x; i < 3 * nnodes; i += PT) mom_s[i] = A(0);
    const NodeMap nm = make_node_map(p);
    const Rng rng = make_rng(p);
    int n = *n_in;
    if (n < 0 || int64_t(n) > in_cap) {
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(status, BZ_DEV_CAPACITY);
        n = n < 0 ? 0 : int(in_cap);
    }
    const int ntiles = int(ceil_div(n, PTILE));
    if (ntiles > max_tiles) {
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(status, BZ_DEV_CAPACITY);
        return;
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t err = 0;
    while (true) {
        if (threadIdx.x == 0) s_tile = int(atomicAdd(ticket, 1u));
        __syncthreads();
        const int tile = s_tile;
        if (tile >= ntiles) break;
        const int64_t base = int64_t(tile) * PTILE + int64_t(threadIdx.x) * PI;
        T x[PI], vx[PI], vy[PI], vz[PI], w[PI];
        if (base + PI <= n && sizeof(T) == 4) {
            float4 a = *reinterpret_cast<const float4 *>(in.x + base);
            float4 b = *reinterpret_cast<const float4 *>(in.vx + base);
            float4 c = *reinterpret_cast<const float4 *>(in.vy + base);
            float4 d = *reinterpret_cast<const float4 *>(in.vz + base);
            float4 f = *reinterpret_cast<const float4 *>(in.w + base);
            x[0] = a.x; x[1] = a.y; x[2] = a.z; x[3] = a.w;
            vx[0] = b.x; vx[1] = b.y; vx[2] = b.z; vx[3] = b.w;
            vy[0] = c.x; vy[1] = c.y; vy[2] = c.z; vy[3] = c.w;
            vz[0] = d.x; vz[1] = d.y; vz[2] = d.z; vz[3] = d.w;
            w[0] = f.x; w[1] = f.y; w[2] = f.z; w[3] = f.w;
        } else {
#pragma unroll
            for (int j = 0; j < PI; ++j) {
                int64_t i = base + j;
                bool ok = i < n;
                x[j] = ok ? in.x[i] : T(0);
                vx[j] = ok ? in.vx[i] : T(0);
                vy[j] = ok ? in.vy[i] : T(0);
                vz[j] = ok ? in.vz[i] : T(0);
                w[j] = ok ? in.w[i] : T(0);
            }
        }
        Item<T> it[PI];
        uint32_t ns = 0, nc = 0;
#pragma unroll
        for (int j = 0; j < PI; ++j) {
            it[j].alive = false;
            it[j].child = false;
            it[j].ionized = false;
            if (w[j] > T(0)) {
                push_item<T, REPLAY, XS>(p, kc, rng, uint32_t(base + j), x[j], vx[j], vy[j], vz[j], E_s, xs_s, R, gas,
                                         it[j]);
                ns += it[j].alive;
                nc += it[j].child;
                if (!(isfinite(it[j].vx) && isfinite(it[j].vy) && isfinite(it[j].vz))) err |= BZ_DEV_NONFINITE;
                if (DEPOSIT) {
                    if (it[j].alive) {
                        int nd = p.advect ? node_index(it[j].x, nm) : 0;
                        if (nd >= 0 && nd < nnodes) {
                            atomicAdd(&mom_s[nd], A(w[j]));
                            if (it[j].ionized) atomicAdd(&mom_s[nnodes + nd], A(w[j]));
                            atomicAdd(&mom_s[2 * nnodes + nd], A(w[j] * it[j].e));
                        }
                    } else if (it[j].ionized && (p.flags & BZ_QUIRK_DEAD_IONFLAG)) {
                        atomicAdd(&mom_s[nnodes + 0], A(1));
                    }
                    if (it[j].child) {
                        int nd = p.advect ? node_index(it[j].cx, nm) : 0;
                        if (nd >= 0 && nd < nnodes) {
                            atomicAdd(&mom_s[nd], A(w[j]));
                            atomicAdd(&mom_s[2 * nnodes + nd], A(w[j] * it[j].ce));
                        }
                    }
                }
            }
        }
        // block-wide exclusive scan of (ns, nc) packed as 16+16 bits
        uint32_t v = ns | (nc << 16);
        uint32_t incl = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        if (lane == 31) s_warp[warp] = incl;
        __syncthreads();
        if (warp == 0) {
            uint32_t wv = lane < PWARPS ? s_warp[lane] : 0u;
            uint32_t wi = wv;
#pragma unroll
            for (int o = 1; o < PWARPS; o <<= 1) {
                uint32_t t = __shfl_up_sync(0xffffffffu, wi, o);
                if (lane >= o) wi += t;
            }
            uint32_t tot = __shfl_sync(0xffffffffu, wi, PWARPS - 1);
            if (lane < PWARPS) s_warp[lane] = wi - wv;  // exclusive warp offsets
            lookback(tile_status, tile, tot & 0xffffu, tot >> 16, &s_ps, &s_pc, status);
            if (lane == 0 && tile == ntiles - 1) {
                counts[0] = int32_t(s_ps + (tot & 0xffffu));
                counts[1] = int32_t(s_pc + (tot >> 16));
                counts[2] = counts[0] + counts[1];
            }
        }
        __syncthreads();
        uint32_t excl = s_warp[warp] + incl - v;
        int64_t ps = int64_t(s_ps) + (excl & 0xffffu);
        int64_t pc = int64_t(s_pc) + (excl >> 16);
#pragma unroll
        for (int j = 0; j < PI; ++j) {
            if (it[j].alive) {
                if (ps < cap) {
                    out.x[ps] = it[j].x; out.vx[ps] = it[j].vx; out.vy[ps] = it[j].vy; out.vz[ps] = it[j].vz;
                    out.w[ps] = w[j];
                } else {
                    err |= BZ_DEV_CAPACITY;
                }
                ++ps;
            }
            if (it[j].child) {
                int64_t q = cap - 1 - pc;  // children staged at the tail in reverse order
                if (q >= 0) {
                    out.x[q] = it[j].cx; out.vx[q] = it[j].cvx; out.vy[q] = it[j].cvy; out.vz[q] = it[j].cvz;
                    out.w[q] = w[j];
                } else {
                    err |= BZ_DEV_CAPACITY;
                }
                ++pc;
            }
        }
        __syncthreads();  // s_tile / s_warp reuse
    }
    if (err) atomicOr(status, err);
    if (DEPOSIT) {
        __syncthreads();
        for (int i = threadIdx.x; i < 3 * nnodes; i += PT) {
            A val = mom_s[i];
            if (val != A(0)) {
                int col = i / nnodes, nd = i - col * nnodes;
                int dst = (col == 2 ? 3 : col) * nnodes + nd;
                atomicAdd(&moments[dst], double(val));
            }
        }
    }
}

// Move the children from the staging tail (reverse order) to out[ns .. ns+nc).
template <typename T>
__global__ void k_append_children(SoA<T> out, int64_t cap, int32_t *counts, uint32_t *status) {
    const int64_t ns = counts[0], nc = counts[1];
    if (ns + 2 * nc > cap) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            atomicOr(status, BZ_DEV_CAPACITY);
            counts[1] = 0;
            counts[2] = int32_t(ns < cap ? ns : cap);
        }
        return;
    }
    for (int64_t j = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; j < nc; j += int64_t(gridDim.x) * blockDim.x) {
        int64_t src = cap - 1 - j, dst = ns + j;
        out.x[dst] = out.x[src]; out.vx[dst] = out.vx[src]; out.vy[dst] = out.vy[src];
        out.vz[dst] = out.vz[src]; out.w[dst] = out.w[src];
    }
}

// --------------------------------------------------------------------------------------
// host side
// --------------------------------------------------------------------------------------
static int g_num_sms = 0;
static int num_sms() {
    if (g_num_sms == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
        if (g_num_sms <= 0) g_num_sms = 1;
    }
    return g_num_sms;
}

template <typename T> PushConst<T> make_push_const(const bz_params &p) {
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
    return k;
}

struct PushWsLayout {
    static constexpr size_t ticket_bytes = 256;
    static size_t tiles(int64_t capacity) { return size_t(ceil_div(std::max<int64_t>(capacity, 1), PTILE)); }
    static size_t bytes(int64_t capacity) { return ticket_bytes + 8 * tiles(capacity); }
};

template <typename T, bool REPLAY, int XS, bool DEPOSIT>
static int launch_push_t(const bz_params &p, SoA<T> in, const int32_t *n_in, int64_t in_cap, SoA<T> out, int64_t cap,
                         int32_t *counts, const T *E, const double *R, const double *gas, double *moments,
                         void *ws, size_t ws_bytes, uint32_t *status, cudaStream_t st) {
    using A = typename AccT<T>::t;
    const int nf = p.advect ? p.n_faces : 1;
    const int xsn = (XS == BZ_XS_TABLE) ? p.xs_n : 0;
    size_t smem = size_t(xsn) * sizeof(float4) + (DEPOSIT ? size_t(3) * p.n_nodes * sizeof(A) : 0) +
                  size_t(nf) * sizeof(T);
    auto kern = k_push<T, REPLAY, XS, DEPOSIT>;
    if (smem > 48 * 1024) {
        if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)) != cudaSuccess)
            return BZ_ERR_UNSUPPORTED;
    }
    // prefer shared memory over L1 so that shared memory never limits the resident CTAs
    cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, PT, smem) != cudaSuccess || per_sm < 1)
        return BZ_ERR_UNSUPPORTED;
    // max tiles the workspace can order
    int64_t max_tiles = int64_t((ws_bytes - PushWsLayout::ticket_bytes) / 8);
    unsigned char *wsb = static_cast<unsigned char *>(ws);
    unsigned int *ticket = reinterpret_cast<unsigned int *>(wsb);
    uint64_t *tile_status = reinterpret_cast<uint64_t *>(wsb + PushWsLayout::ticket_bytes);
    if (cudaMemsetAsync(ws, 0, ws_bytes, st) != cudaSuccess) return BZ_ERR_CUDA;
    if (cudaMemsetAsync(counts, 0, 3 * sizeof(int32_t), st) != cudaSuccess) return BZ_ERR_CUDA;
    int grid = num_sms() * per_sm;
    int64_t tiles_cap = std::max<int64_t>(1, std::min<int64_t>(max_tiles, int64_t(1) << 30));
    if (grid > tiles_cap) grid = int(tiles_cap);
    PushConst<T> kc = make_push_const<T>(p);
    kern<<<grid, PT, smem, st>>>(p, kc, in, n_in, in_cap, out, cap, counts, E, R, gas, moments, ticket, tile_status,
                                 int(std::min<int64_t>(max_tiles, INT32_MAX)), status);
    if (cudaGetLastError() != cudaSuccess) return BZ_ERR_CUDA;
    k_append_children<T><<<num_sms() * 2, 256, 0, st>>>(out, cap, counts, status);
    if (cudaGetLastError() != cudaSuccess) return BZ_ERR_CUDA;
    return BZ_OK;
}

template <typename T, typename P>
static int push_entry(const bz_params *pp, P in_, const int32_t *n_in, int64_t in_cap, P out_, int64_t cap,
                      int32_t *counts,
                      const T *E, const double *R, const double *gas, double *moments, void *ws, size_t ws_bytes,
                      uint32_t *status, void *stream) {
    if (!pp || !n_in || !counts || !E || !ws || !status || cap <= 0 || in_cap < 0) return BZ_ERR_ARG;
    const bz_params &p = *pp;
    if (!in_.x || !in_.vx || !in_.vy || !in_.vz || !in_.w || !out_.x || !out_.vx || !out_.vy || !out_.vz || !out_.w)
        return BZ_ERR_ARG;
    if ((R == nullptr) != (gas == nullptr)) return BZ_ERR_ARG;
    if (p.advect && (p.n_faces < 1 || p.dx <= 0 || p.L <= 0)) return BZ_ERR_ARG;
    if (p.n_nodes < 1 || p.bnf < 1) return BZ_ERR_ARG;
    if (p.xs_mode == BZ_XS_TABLE && (p.xs_n < 2 || !p.xs_table || !(p.xs_emax > p.xs_emin) || p.xs_emin <= 0))
        return BZ_ERR_ARG;
    if (p.xs_mode != BZ_XS_TABLE && p.xs_mode != BZ_XS_REF_FITS) return BZ_ERR_ARG;
    if (p.coll_model == BZ_COLL_NULL && !(p.nu_max > 0)) return BZ_ERR_ARG;
    if (ws_bytes < PushWsLayout::bytes(1)) return BZ_ERR_WORKSPACE;
    // vector loads need 16-byte aligned arrays
    auto al = [](const void *q) { return (reinterpret_cast<uintptr_t>(q) & 15u) == 0; };
    if (sizeof(T) == 4 && !(al(in_.x) && al(in_.vx) && al(in_.vy) && al(in_.vz) && al(in_.w))) return BZ_ERR_ARG;
    SoA<T> in{in_.x, in_.vx, in_.vy, in_.vz, in_.w};
    SoA<T> out{out_.x, out_.vx, out_.vy, out_.vz, out_.w};
    cudaStream_t st = as_stream(stream);
    const bool replay = R != nullptr;
    const bool dep = moments != nullptr;
#define BZ_PUSH_CASE(RP, XSM, DP)                                                                                   \
    if (replay == RP && p.xs_mode == XSM && dep == DP)                                                             \
        return launch_push_t<T, RP, XSM, DP>(p, in, n_in, in_cap, out, cap, counts, E, R, gas, moments, ws, ws_bytes,      \
                                             status, st);
    BZ_PUSH_CASE(false, BZ_XS_TABLE, true)
    BZ_PUSH_CASE(false, BZ_XS_TABLE, false)
    BZ_PUSH_CASE(false, BZ_XS_REF_FITS, true)
    BZ_PUSH_CASE(false, BZ_XS_REF_FITS, false)
    BZ_PUSH_CASE(true, BZ_XS_TABLE, true)
    BZ_PUSH_CASE(true, BZ_XS_TABLE, false)
    BZ_PUSH_CASE(true, BZ_XS_REF_FITS, true)
    BZ_PUSH_CASE(true, BZ_XS_REF_FITS, false)
#undef BZ_PUSH_CASE
    return BZ_ERR_ARG;
}

}  // namespace bz

extern "C" {

size_t bz_push_workspace(int64_t capacity) { return bz::PushWsLayout::bytes(capacity); }

int bz_push_collide_f32(const bz_params *p, bz_particles_f32 in, const int32_t *n_in, int64_t in_capacity,
                        bz_particles_f32 out, int64_t out_capacity, int32_t *counts, const float *E, const double *replay_R,
                        const double *replay_gas, double *moments, void *workspace, size_t workspace_bytes,
                        uint32_t *status, void *stream) {
    return bz::push_entry<float>(p, in, n_in, in_capacity, out, out_capacity, counts, E, replay_R, replay_gas, moments, workspace,
                                 workspace_bytes, status, stream);
}

int bz_push_collide_f64(const bz_params *p, bz_particles_f64 in, const int32_t *n_in, int64_t in_capacity,
                        bz_particles_f64 out, int64_t out_capacity, int32_t *counts, const double *E, const double *replay_R,
                        const double *replay_gas, double *moments, void *workspace, size_t workspace_bytes,
                        uint32_t *status, void *stream) {
    return bz::push_entry<double>(p, in, n_in, in_capacity, out, out_capacity, counts, E, replay_R, replay_gas, moments, workspace,
                                  workspace_bytes, status, stream);
}

const char *bz_version(void) { return "libbz 0.1 sm_103a"; }

}  // extern "C"

// ------------------------------------------------------------------------------------
// Allocation-free variant of the push: the look-back scratch (a tile ticket and one
// status word per 1024-particle tile) lives in a fixed array compiled into the library,
// so a caller that cannot allocate device memory only passes inputs and outputs.
// ------------------------------------------------------------------------------------
namespace bz {

static_assert(BZ_PUSH_NOALLOC_MAX_PARTICLES % PTILE == 0, "scratch holds whole tiles");
static_assert(PushWsLayout::ticket_bytes == 256, "scratch header matches the workspace layout");

// One copy per GPU that loads the library, alive until the process exits.
static __device__ __align__(256) unsigned char g_push_noalloc_scratch[BZ_PUSH_NOALLOC_SCRATCH_BYTES];

// Device address of the scratch array on the current device. The array's name in host
// code only stands in for the symbol, so the address is asked of the runtime once per
// device (with that device current) and remembered.
constexpr int kMaxDevices = 64;
static std::mutex g_noalloc_mu;
static void *g_noalloc_ptr[kMaxDevices] = {};

static int noalloc_scratch(void **out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) return BZ_ERR_CUDA;
    if (dev < 0 || dev >= kMaxDevices) return BZ_ERR_UNSUPPORTED;
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void *ptr = nullptr;
        if (cudaGetSymbolAddress(&ptr, g_push_noalloc_scratch) != cudaSuccess || !ptr) return BZ_ERR_CUDA;
        g_noalloc_ptr[dev] = ptr;
    }
    *out = g_noalloc_ptr[dev];
    return BZ_OK;
}

}  // namespace bz

extern "C" {

int bz_push_collide_f32_noalloc(const bz_params *p, bz_particles_f32 in, const int32_t *n_in, int64_t in_capacity,
                                bz_particles_f32 out, int64_t out_capacity, int32_t *counts, const float *E,
                                const double *replay_R, const double *replay_gas, double *moments, uint32_t *status,
                                void *stream) {
    if (in_capacity > BZ_PUSH_NOALLOC_MAX_PARTICLES) return BZ_ERR_TOO_LARGE;
    void *scratch = nullptr;
    int rc = bz::noalloc_scratch(&scratch);
    if (rc != BZ_OK) return rc;
    // the scratch is cleared by the launch (cudaMemsetAsync on the caller's stream)
    return bz::push_entry<float>(p, in, n_in, in_capacity, out, out_capacity, counts, E, replay_R, replay_gas,
                                 moments, scratch, BZ_PUSH_NOALLOC_SCRATCH_BYTES, status, stream);
}

}  // extern "C"
