/* FP64 CPU restatement of the reference's electron PIC-MCC hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the oracle the CUDA kernels are checked against, and the
 * CPU baseline timed beside them. Each function cites the reference lines it restates
 * (paths within jfabell/boltzmann, 1bin variant unless stated).
 *
 * Parity pins: tests/test_oracle_golden.py checks every function here against vectors
 * produced by running the reference's own Python source (tests/golden/make_golden.py).
 */
#include "bz_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* electron_kernel_numba.py:13-24 */
#define REF_L_UNUSED 2.54
static double c_qe(void) { return 1.602 * pow(10.0, -19.0); }
static double c_me(void) { return 9.10938 * pow(10.0, -31.0); }
static double c_mn(void) { return 6.6 * pow(10.0, -26.0); }
static double c_jev(void) { return 6.241509 * 1e18; }
#define E_ION 15.76
#define EPS_DEAD 0.01

/* ------------------------------------------------------------------------------------ */
/* Philox4x32-10                                                                         */
/* ------------------------------------------------------------------------------------ */
/* Philox4x32 with a given number of rounds (10: Philox4x32-10) */
void orc_philox_rounds(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4], int rounds) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < rounds; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        c0 = hi1 ^ c1 ^ k0;
        c1 = lo1;
        c2 = hi0 ^ c3 ^ k1;
        c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}
void orc_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) { orc_philox_rounds(ctr, key, out, 10); }

/* Rounds of the push's draws (tags 0-2: gas velocity, collision, ionization), as in the
 * kernels: Philox4x32-7. Resampling draws (tag 3) keep 10. */
#define PUSH_ROUNDS 7

/* Uniform conventions shared with the CUDA kernels (exact in the target type, and so is
 * the complement 1-u):
 *   float path : u = ((r >> 9) + 0.5) * 2^-23
 *   double path: u = (((r_a >> 6) << 26 | (r_b >> 6)) + 0.5) * 2^-52           */
static void draw_u(const orc_params *p, uint64_t slot, uint32_t tag, double *u, int nu) {
    const int rounds = tag <= 2u ? PUSH_ROUNDS : 10;
    uint32_t key[2] = {(uint32_t)p->seed, (uint32_t)(p->seed >> 32)};
    uint32_t ctr[4] = {(uint32_t)slot, (uint32_t)p->step, (uint32_t)(p->step >> 32), tag};
    uint32_t r[4];
    if (p->precision == 64) {
        int k = 0;
        for (uint32_t c = 0; k < nu; ++c) {
            ctr[3] = tag | (c << 8);
            orc_philox_rounds(ctr, key, r, rounds);
            for (int j = 0; j < 2 && k < nu; ++j, ++k) {
                uint64_t m = ((uint64_t)(r[2 * j] >> 6) << 26) | (uint64_t)(r[2 * j + 1] >> 6);
                u[k] = ((double)m + 0.5) * 0x1p-52;
            }
        }
    } else {
        orc_philox_rounds(ctr, key, r, rounds);
        for (int k = 0; k < nu && k < 4; ++k) u[k] = ((double)(r[k] >> 9) + 0.5) * 0x1p-23;
    }
}

/* The raw words of a float-path draw (tag <= 2: the push's rounds). */
static void draw_raw(const orc_params *p, uint64_t slot, uint32_t tag, uint32_t r[4]) {
    uint32_t key[2] = {(uint32_t)p->seed, (uint32_t)(p->seed >> 32)};
    uint32_t ctr[4] = {(uint32_t)slot, (uint32_t)p->step, (uint32_t)(p->step >> 32), tag};
    orc_philox_rounds(ctr, key, r, tag <= 2u ? PUSH_ROUNDS : 10);
}

/* Box-Muller: (r cos 2πb, r sin 2πb) with r = sqrt(-2 ln a). */
static void box_muller(double a, double b, double *g0, double *g1) {
    double r = sqrt(-2.0 * log(a));
    *g0 = r * cos(2.0 * M_PI * b);
    *g1 = r * sin(2.0 * M_PI * b);
}

/* ------------------------------------------------------------------------------------ */
/* cross sections                                                                        */
/* ------------------------------------------------------------------------------------ */
/* electron_kernel_numba.py:66-127, elastic fit: 12 log10-quadratic pieces. */
static const double EL_A[12] = {-0.02704763, -0.08847237, -0.37608274, -1.4874467, -0.9870356, 14.28063581,
                                -2.12069169, -0.3585636, 1.25262128, -2.28332905, -1.47508661, -0.11090525};
static const double EL_B[12] = {-0.23720051, -0.6084786, -1.8167778, -4.82420619, -4.2206026, 18.92275458,
                                0.7555105, 0.79246666, -0.40002029, 4.89566076, 2.82263476, -0.77506081};
static const double EL_C[12] = {-19.67900951, -20.24111992, -21.51414308, -23.55745478, -23.44715988, -14.70556113,
                                -19.71943671, -19.71260274, -19.48909003, -21.46789173, -20.1928456, -17.81752307};
static const double EL_E[11] = {0.000780396, 0.006098667, 0.0476269, 0.1015574, 0.1943527, 0.2995781,
                                1.097156, 2.339524, 4.988691, 10.63765, 22.68322};
/* electron_kernel_numba.py:129-174, ionization fit: 8 pieces above 15.76 eV. */
static const double IO_A[8] = {-2149239.99337822, -227229.83440255, -20173.68563579, -1838.90888364,
                               -186.98923927, -24.48843901, -4.33101714, -0.68345667};
static const double IO_B[8] = {5150451.29014456, 545171.14839945, 48599.13254342, 4491.58838596,
                               477.04784782, 69.43965607, 14.47124519, 2.6053539};
static const double IO_C[8] = {-3085665.64874862, -327016.69508374, -29290.96100603, -2763.82866252,
                               -324.75732578, -69.145292411, -31.66224458, -21.99823511};
static const double IO_E[7] = {15.77742, 15.81964, 15.96196, 16.44162, 18.05837, 23.50771, 41.87498};

static void sigma_fits(double e, double *s_el, double *s_ion) {
    double le = log10(e);
    int k = 0;
    while (k < 11 && !(e < EL_E[k])) ++k;
    double lg0 = (EL_A[k] * le + EL_B[k]) * le + EL_C[k];
    *s_el = pow(10.0, lg0);
    double lg2 = 0.0; /* no piece matches at e == 15.76 exactly: log = 0 (electron_kernel_numba.py:164) */
    if (E_ION < e && e < IO_E[0]) lg2 = (IO_A[0] * le + IO_B[0]) * le + IO_C[0];
    else {
        for (int j = 1; j < 8; ++j) {
            int hi_ok = (j == 7) ? 1 : (e < IO_E[j]);
            if (IO_E[j - 1] <= e && hi_ok) { lg2 = (IO_A[j] * le + IO_B[j]) * le + IO_C[j]; break; }
        }
    }
    double s2 = pow(10.0, lg2);
    if (e < E_ION) s2 = 0.0;
    *s_ion = s2;
}

/* n*sigma table lookup, linear in log2(e) on a log grid (same arithmetic as the kernels). */
static void sigma_table(const orc_params *p, double e, double *ns) {
    int n = p->xs_n;
    double inv_d = (double)(n - 1) / log2(p->xs_emax / p->xs_emin);
    double t = (log2(e) - log2(p->xs_emin)) * inv_d;
    if (!(t > 0.0)) t = 0.0;
    if (t > (double)(n - 1)) t = (double)(n - 1);
    int i = (int)t;
    if (i > n - 2) i = n - 2;
    double f = t - i;
    for (int k = 0; k < 3; ++k) {
        double a = p->xs_table[k * n + i], b = p->xs_table[k * n + i + 1];
        ns[k] = a + f * (b - a);
    }
}

/* ------------------------------------------------------------------------------------ */
/* push + collide (electron_kernel_numba.py:38-287)                                      */
/* ------------------------------------------------------------------------------------ */
typedef struct { double x, y, z, vx, vy, vz, w, e, flag; int child, exc; double cx, cy, cz, cvx, cvy, cvz, ce, cw, margin; } push_out;

static void push_one(const orc_params *p, int64_t i, const double *in_d, const double *in_t, const double *E,
                     const double *R, const double *gas, push_out *o) {
    const double q_e = c_qe(), m_e = c_me(), m_n = c_mn(), j_ev = c_jev();
    const double efac = 0.5 * m_e * j_ev;
    double d_w = in_t[0];
    int nz = d_w > 0;
    double xx = in_d[0], xy = in_d[1], xz = in_d[2];
    double vx = in_d[3] * nz + EPS_DEAD * (1 - nz);
    double vy = in_d[4] * nz + EPS_DEAD * (1 - nz);
    double vz = in_d[5] * nz + EPS_DEAD * (1 - nz);
    double Ru[6];
    double g[3];
    if (p->rng_mode == 0) {
        for (int k = 0; k < 6; ++k) Ru[k] = R[i * 7 + k];
        for (int k = 0; k < 3; ++k) g[k] = gas[i * 3 + k];
    } else {
        double ug[4], uc[4], ui[1];
        g[0] = g[1] = g[2] = 0.0;
        if (p->precision == 64) {
            /* float64: Box-Muller from the gas draw, the child's azimuth from tag 2 */
            if (p->gas_sigma > 0) {
                draw_u(p, (uint64_t)i, 0u, ug, 4);
                double g3;
                box_muller(ug[0], ug[1], &g[0], &g[1]);
                box_muller(ug[2], ug[3], &g[2], &g3);
                for (int k = 0; k < 3; ++k) g[k] *= p->gas_sigma;
            }
            draw_u(p, (uint64_t)i, 2u, ui, 1);
        } else {
            /* float32: Box-Muller pairs from the gas draw's words (0, 1) and (2, 3), as in
             * float64; the child's azimuth from the bits of the collision draw's first three
             * words that its uniforms leave unused (the low 9, 9 and 5), placed where a
             * float-path uniform takes its 23 bits */
            draw_u(p, (uint64_t)i, 0u, ug, 4);
            if (p->gas_sigma > 0) {
                double g3;
                box_muller(ug[0], ug[1], &g[0], &g[1]);
                box_muller(ug[2], ug[3], &g[2], &g3);
                for (int k = 0; k < 3; ++k) g[k] *= p->gas_sigma;
            }
            uint32_t rc[4];
            draw_raw(p, (uint64_t)i, 1u, rc);
            const uint32_t r5 = (rc[0] << 23) | ((rc[1] & 511u) << 14) | ((rc[2] & 511u) << 5);
            ui[0] = ((double)(r5 >> 9) + 0.5) * 0x1p-23;
        }
        draw_u(p, (uint64_t)i, 1u, uc, 4);
        Ru[0] = uc[0]; Ru[1] = uc[1]; Ru[2] = uc[2]; Ru[3] = uc[3]; Ru[4] = 0.0; Ru[5] = ui[0];
    }
    double ax = vx - g[0], ay = vy - g[1], az = vz - g[2];
    double e_el = ax * ax + ay * ay + az * az;
    double v_mag = sqrt(e_el);
    e_el = efac * e_el;
    double s0, s1 = 0.0, s2;
    if (p->xs_mode == 1) {
        sigma_fits(e_el, &s0, &s2);
        s0 *= p->nn;
        s2 *= p->nn;
    } else {
        double ns[3];
        sigma_table(p, e_el, ns);
        s0 = ns[0]; s1 = ns[1]; s2 = ns[2];
        if (e_el < p->e_exc) s1 = 0.0; /* no process below its threshold */
        if (e_el < E_ION) s2 = 0.0;
    }
    double r0, r1, r2;
    if (p->coll_model == 0) {
        double sig_tot = s0 + s1 + s2;
        double P = 1.0 - exp(-p->dt * v_mag * sig_tot);
        double pcst = P * (1.0 / sig_tot);
        r0 = s0 * pcst;
        r1 = r0 + s1 * pcst;
        r2 = r1 + s2 * pcst;
    } else {
        double P = 1.0 - exp(-p->dt * p->nu_max);
        double c = P * v_mag / p->nu_max;
        r0 = s0 * c;
        r1 = r0 + s1 * c;
        r2 = r1 + s2 * c;
    }
    o->child = 0;
    o->exc = 0;
    o->flag = 0.0;
    double u0 = Ru[0];
    /* distance of the decision uniform to the nearest process boundary */
    o->margin = fmin(fmin(fabs(u0 - r0), fabs(u0 - r1)), fabs(u0 - r2));
    if (u0 < r0) {
        /* elastic, electron_kernel_numba.py:197-209 */
        double cos_chi = 2 * Ru[1] - 1;
        double chi = acos(cos_chi);
        double phi = 2 * M_PI * Ru[2];
        double vn = v_mag * sqrt(1 - (2 * m_e / m_n));
        vx = vn * sin(chi) * cos(phi);
        vy = vn * sin(chi) * sin(phi);
        vz = vn * cos(chi);
    } else if (r0 < u0 && u0 < r1) {
        /* excitation (table mode only; the reference has none): loss e_exc, isotropic */
        if ((e_el - p->e_exc) < 0.05 * e_el) o->margin = 0.0; /* ill-conditioned in float32 */
        o->exc = 1;
        double cos_chi = 2 * Ru[1] - 1;
        double chi = acos(cos_chi);
        double phi = 2 * M_PI * Ru[2];
        double en = fabs(e_el - p->e_exc);
        double vn = sqrt(2 * en / (j_ev * m_e));
        vx = vn * sin(chi) * cos(phi);
        vy = vn * sin(chi) * sin(phi);
        vz = vn * cos(chi);
    } else if (r1 < u0 && u0 < r2) {
        /* ionization, electron_kernel_numba.py:211-255 */
        if ((e_el - E_ION) < 0.05 * e_el) o->margin = 0.0; /* ill-conditioned in float32 */
        double cos_chi = 2 * Ru[1] - 1;
        double chi = acos(cos_chi);
        double phi = 2 * M_PI * Ru[2];
        double e_ej = fabs(0.5 * (e_el - E_ION));
        double vn = sqrt(2 * e_ej / (j_ev * m_e));
        vx = vn * sin(chi) * cos(phi);
        vy = vn * sin(chi) * sin(phi);
        vz = vn * cos(chi);
        o->flag = 1.0;
        cos_chi = 2 * Ru[3] - 1;
        chi = acos(cos_chi);
        phi = 2 * M_PI * Ru[5];
        double tvx = vn * sin(chi) * cos(phi);
        double tvy = vn * sin(chi) * sin(phi);
        double tvz = vn * cos(chi);
        o->child = 1;
        o->cx = xx; o->cy = xy; o->cz = xz;
        o->cvx = tvx; o->cvy = tvy; o->cvz = tvz;
        o->ce = efac * (tvx * tvx + tvy * tvy + tvz * tvz);
        o->cw = d_w;
    }
    int idx = 0;
    if (p->advect == 2) {
        /* ensemble of 0-D swarms: x holds the swarm index, the swarm's field is E[x] */
        idx = (int)xx;
        if (idx < 0) idx = 0;
        if (idx > p->n_faces - 1) idx = p->n_faces - 1;
    } else if (p->advect) {
        /* X-ADV (electron_kernel_numba.py:258-260) with the post-collision velocity */
        double x_old = xx;
        xx += 100 * p->dt * vx;
        xy += 100 * p->dt * vy;
        xz += 100 * p->dt * vz;
        /* E at the pre-push cell int(x/dx) (boltzmann.py:657) */
        idx = (int)(x_old / p->dx);
        if (idx < 0) idx = 0;
        if (idx > p->n_faces - 1) idx = p->n_faces - 1;
    }
    vx -= p->dt * (q_e / m_e) * (100 * E[idx]);
    int valid = p->advect == 1 ? ((0 < xx && xx < p->L) && d_w > 0) : (d_w > 0);
    if (p->advect == 1) o->margin = fmin(o->margin, fmin(fabs(xx), fabs(xx - p->L)) / p->L);
    o->w = valid * d_w;
    o->x = valid * xx + (1 - valid) * 0.00000001;
    o->y = valid * xy;
    o->z = valid * xz;
    vx = valid * vx;
    vy = valid * vy;
    vz = valid * vz;
    o->e = efac * (vx * vx + vy * vy + vz * vz);
    o->vx = vx; o->vy = vy; o->vz = vz;
}

int64_t orc_push(const orc_params *p, int64_t n, double *data, double *tosum, const double *E,
                 const double *R, const double *gas) {
    return orc_push_margin(p, n, data, tosum, E, R, gas, NULL);
}

int64_t orc_push_margin(const orc_params *p, int64_t n, double *data, double *tosum, const double *E,
                        const double *R, const double *gas, double *margin) {
    int64_t nni = 0;
    for (int64_t i = 0; i < n; ++i) {
        push_out o;
        push_one(p, i, data + i * 6, tosum + i * 4, E, R, gas, &o);
        if (margin) margin[i] = o.margin;
        if (o.child) {
            int64_t wi = n + nni++;
            double *d = data + wi * 6, *t = tosum + wi * 4;
            d[3] = o.cvx; d[4] = o.cvy; d[5] = o.cvz;
            d[0] = o.cx; d[1] = o.cy; d[2] = o.cz;
            t[3] = o.ce;
            t[0] = o.cw;
        }
        double *d = data + i * 6, *t = tosum + i * 4;
        if (o.flag != 0.0) t[1] = 1.0;
        if (p->moment_exc) t[2] = (o.exc && o.w > 0) ? 1.0 : 0.0; /* survivors only, like the kernels */
        t[0] = o.w;
        d[0] = o.x; d[1] = o.y; d[2] = o.z;
        t[3] = o.e;
        d[3] = o.vx; d[4] = o.vy; d[5] = o.vz;
    }
    return nni;
}

/* ------------------------------------------------------------------------------------ */
/* deposit: post_processing_1D.py:44-62 + kernels-new.cu reda (:56-73) / redcheck (:8-50) */
/* ------------------------------------------------------------------------------------ */
/* fine deposit bin int(((x + dx/2)/(L + dx)) * float(M)) (post_processing_1D.py:44); in an
 * ensemble the swarm index times bnf (its node), for one 0-D swarm bin 0 */
static int fine_bin(const orc_params *p, double x, double half, double Lp, double fM) {
    if (p->advect == 1) return (int)(((x + half) / Lp) * fM);
    if (p->advect == 2) return (int)x * p->bnf;
    return 0;
}

static void deposit_impl(const orc_params *p, int64_t n_total, const double *data, const double *tosum,
                         double *moments, int weight_cols) {
    int RN = p->n_nodes;
    int M = p->bnf * RN;
    double *fine = (double *)calloc((size_t)M * 4, sizeof(double));
    double half = 0.5 * p->dx, Lp = p->L + p->dx;
    double fM = (double)(float)M;
    for (int64_t i = 0; i < n_total; ++i) {
        const double *t = tosum + i * 4;
        double v[4] = {t[0], t[1], t[2], t[3]};
        if (weight_cols && t[0] > 0.0) { v[1] = t[1] * t[0]; v[2] = t[2] * t[0]; v[3] = t[3] * t[0]; }
        int b = fine_bin(p, data[i * 6], half, Lp, fM);
        if (b < 0 || b >= M) continue;
        for (int j = 0; j < 4; ++j) fine[(size_t)b * 4 + j] += v[j];
    }
    if (M / RN > 1) {
        int bloks = (int)ceil((double)M / RN);
        for (int k = 0; k < RN; ++k) {
            double bb[64][4];
            for (int t2 = 0; t2 < bloks && t2 < 64; ++t2)
                for (int j = 0; j < 4; ++j) bb[t2][j] = (k * bloks + t2 < M) ? fine[(size_t)(k * bloks + t2) * 4 + j] : 0.0;
            for (int s = bloks / 2; s > 0; s >>= 1)
                for (int t2 = 0; t2 < s; ++t2)
                    for (int j = 0; j < 4; ++j) bb[t2][j] += bb[t2 + s][j];
            for (int j = 0; j < 4; ++j) moments[j * RN + k] = bb[0][j];
        }
    } else {
        for (int k = 0; k < RN; ++k)
            for (int j = 0; j < 4; ++j) moments[j * RN + k] = fine[(size_t)k * 4 + j];
    }
    free(fine);
}

void orc_deposit(const orc_params *p, int64_t n_total, const double *data, const double *tosum, double *moments) {
    deposit_impl(p, n_total, data, tosum, moments, 1);
}

int64_t orc_post(const orc_params *p, int64_t n_total, double *data, double *tosum, double *moments) {
    /* cols 1..3 scaled by w for w>0, deposited, col 3 divided back (post_processing_1D.py:50-62) */
    for (int64_t i = 0; i < n_total; ++i) {
        double *t = tosum + i * 4;
        if (t[0] > 0.0) { t[1] *= t[0]; t[2] *= t[0]; t[3] *= t[0]; }
    }
    deposit_impl(p, n_total, data, tosum, moments, 0);
    for (int64_t i = 0; i < n_total; ++i) {
        double *t = tosum + i * 4;
        if (t[0] > 0.0) t[3] = t[3] / t[0];
    }
    /* reshuffle_data_atomics (post_processing_1D.py:26-38): keep w > 0 in order */
    int64_t na = 0;
    for (int64_t i = 0; i < n_total; ++i) {
        if (tosum[i * 4] > 0.0) {
            if (na != i) { memmove(data + na * 6, data + i * 6, 6 * sizeof(double)); memmove(tosum + na * 4, tosum + i * 4, 4 * sizeof(double)); }
            ++na;
        }
    }
    for (int64_t i = na; i < n_total; ++i) { memset(data + i * 6, 0, 6 * sizeof(double)); memset(tosum + i * 4, 0, 4 * sizeof(double)); }
    return na;
}

/* ------------------------------------------------------------------------------------ */
/* binning: bin_particles.py:7-22 (1bin), 3bin :7-37, 5bin :7-49                          */
/* ------------------------------------------------------------------------------------ */
static double energy_col(double vx, double vy, double vz, double w) {
    double e = 0.5 * c_me() * c_jev() * (vx * vx + vy * vy + vz * vz);
    if (w > 0.0) e = (e * w) / w; /* post_processing_1D.py:53,62 */
    return e;
}

void orc_bin(const orc_params *p, int64_t n, const double *x, const double *vx, const double *vy,
             const double *vz, const double *w, int nb, const double *edges, int64_t max_ppc,
             int64_t *counts, int64_t *lists) {
    int RN = p->n_nodes;
    for (int64_t k = 0; k < (int64_t)nb * RN; ++k) counts[k] = 0;
    for (int64_t k = 0; k < (int64_t)nb * max_ppc * RN; ++k) lists[k] = -1;
    for (int64_t j = 0; j < n; ++j) {
        if (!(w[j] > 0)) continue;
        int64_t cc = p->advect == 1 ? (int64_t)((x[j] + 0.5 * p->dx) / p->dx) : (p->advect == 2 ? (int64_t)x[j] : 0);
        if (cc < 0 || cc > RN - 1) continue;
        int b = 0;
        if (nb > 1) {
            double e = energy_col(vx[j], vy[j], vz[j], w[j]);
            b = -1;
            for (int k = 0; k < nb - 1; ++k) if (e < edges[k]) { b = k; break; }
            if (b < 0) { if (e >= edges[nb - 2]) b = nb - 1; else continue; }
        }
        int64_t slot = counts[(int64_t)b * RN + cc]++;
        if (slot < max_ppc) lists[((int64_t)b * max_ppc + slot) * RN + cc] = j;
    }
}

/* ------------------------------------------------------------------------------------ */
/* ES-WPNC resampling: boltzmann.py:799-890                                              */
/* ------------------------------------------------------------------------------------ */
static int64_t lower_bound(const double *a, int64_t n, double v) { /* searchsorted side='left' */
    int64_t lo = 0, hi = n;
    while (lo < hi) { int64_t m = (lo + hi) / 2; if (a[m] < v) lo = m + 1; else hi = m; }
    return lo;
}
static int64_t upper_bound(const double *a, int64_t n, double v) { /* searchsorted side='right' */
    int64_t lo = 0, hi = n;
    while (lo < hi) { int64_t m = (lo + hi) / 2; if (a[m] <= v) lo = m + 1; else hi = m; }
    return lo;
}

void orc_eedf(const orc_params *p, int64_t n, const double *x, const double *vx, const double *vy,
              const double *vz, const double *w, int nbins, double emin, double emax, double *hist) {
    int RN = p->n_nodes;
    int M = p->bnf * RN;
    double half = 0.5 * p->dx, Lp = p->L + p->dx, fM = (double)(float)M;
    double efac = 0.5 * c_me() * c_jev(), lemin = log(emin), scale = (double)nbins / log(emax / emin);
    for (int64_t j = 0; j < n; ++j) {
        if (!(w[j] > 0)) continue;
        int fb = fine_bin(p, x[j], half, Lp, fM);
        if (fb < 0 || fb >= M) continue;
        int nd = fb / p->bnf;
        double e = efac * (vx[j] * vx[j] + vy[j] * vy[j] + vz[j] * vz[j]);
        if (!(e > 0)) continue;
        double t = (log(e) - lemin) * scale;
        if (!(t >= 0 && t < nbins)) continue;
        hist[(int64_t)nd * nbins + (int)floor(t)] += w[j];
    }
}

static int cmp_i64(const void *a, const void *b) {
    int64_t x = *(const int64_t *)a, y = *(const int64_t *)b;
    return (x > y) - (x < y);
}

int64_t orc_resample(const orc_params *p, int64_t n, double *data, double *tosum, int nb,
                     const int64_t *targets, double min_wt, const int64_t *max_ppc,
                     const int64_t *counts, const int64_t *lists, int64_t list_stride,
                     const double *u, int64_t n_u, int64_t *n_used, int flags, const double *thr) {
    const double m_e = c_me(), j_ev = c_jev();
    int RN = p->n_nodes;
    /* split below thr[0]*T, merge at thr[1]*T down to int(thr[2]*T) survivors;
     * the reference's 0.5, 3 and 0.6 (boltzmann.py:807, 826, 829) when thr is NULL */
    const double split_below = thr ? thr[0] : 0.5, merge_at = thr ? thr[1] : 3.0,
                 merge_keep = thr ? thr[2] : 0.6;
    int64_t Nc = n;
    int64_t ui = 0;
    /* list_stride = max list length stored per (bin, cell) */
    for (int cc = 0; cc < RN; ++cc) {
        for (int b = 0; b < nb; ++b) {
            const int64_t tk = (flags & 0x10) ? (int64_t)cc * nb + b : b; /* per-key or per-bin */
            int64_t T = targets[tk];
            int64_t cnt = counts[(int64_t)b * RN + cc];
            const int64_t *lst = lists + (int64_t)b * list_stride * RN; /* [slot][cell] */
#define LIST(s) lst[(int64_t)(s) * RN + cc]
            /* too few: split (boltzmann.py:806-823) */
            if (0 < cnt && (double)cnt < split_below * (double)T) {
                int64_t nhw = 0;
                int64_t *hw = (int64_t *)malloc(sizeof(int64_t) * (size_t)cnt);
                for (int64_t s = 0; s < cnt; ++s) { int64_t id = LIST(s); if (tosum[id * 4] > min_wt) hw[nhw++] = id; }
                if (nhw > 0) {
                    int64_t m = 2 * T - cnt;
                    double *cdf = (double *)malloc(sizeof(double) * (size_t)nhw);
                    double sw = 0.0;
                    for (int64_t k = 0; k < nhw; ++k) sw += tosum[hw[k] * 4];
                    double acc = 0.0;
                    for (int64_t k = 0; k < nhw; ++k) { acc += tosum[hw[k] * 4] / sw; cdf[k] = acc; }
                    double last = cdf[nhw - 1];
                    for (int64_t k = 0; k < nhw; ++k) cdf[k] /= last;
                    int64_t *keep = (int64_t *)malloc(sizeof(int64_t) * (size_t)(m > 0 ? m : 1));
                    for (int64_t k = 0; k < m; ++k) {
                        double uu = (ui < n_u) ? u[ui] : 0.5;
                        ++ui;
                        int64_t ix = upper_bound(cdf, nhw, uu);
                        if (ix > nhw - 1) ix = nhw - 1;
                        keep[k] = hw[ix];
                    }
                    qsort(keep, (size_t)m, sizeof(int64_t), cmp_i64);
                    for (int64_t k = 0; k < m;) {
                        int64_t id = keep[k], c = 0;
                        while (k < m && keep[k] == id) { ++c; ++k; }
                        int64_t tgt = (flags & 1) ? hw[id % nhw] : id;
                        tosum[tgt * 4] = tosum[tgt * 4] / (double)(c + 1);
                        for (int64_t r = 0; r < c; ++r) {
                            memcpy(data + (Nc + r) * 6, data + tgt * 6, 6 * sizeof(double));
                            memcpy(tosum + (Nc + r) * 4, tosum + tgt * 4, 4 * sizeof(double));
                        }
                        Nc += c;
                    }
                    free(keep);
                    free(cdf);
                }
                free(hw);
            }
            /* too many: merge (boltzmann.py:826-877) */
            if ((double)cnt >= merge_at * (double)T) {
                int64_t np_ = cnt < max_ppc[tk] ? cnt : max_ppc[tk];
                int64_t K = (int64_t)(merge_keep * (double)T);
                double W = 0.0, sx = 0.0, sy = 0.0, sz = 0.0, se = 0.0;
                for (int64_t s = 0; s < np_; ++s) W += tosum[LIST(s) * 4];
                for (int64_t s = 0; s < np_; ++s) { int64_t id = LIST(s); sx += data[id * 6 + 3] * tosum[id * 4]; }
                for (int64_t s = 0; s < np_; ++s) { int64_t id = LIST(s); sy += data[id * 6 + 4] * tosum[id * 4]; }
                for (int64_t s = 0; s < np_; ++s) { int64_t id = LIST(s); sz += data[id * 6 + 5] * tosum[id * 4]; }
                for (int64_t s = 0; s < np_; ++s) { int64_t id = LIST(s); se += tosum[id * 4] * tosum[id * 4 + 3] / W; }
                double ux = sx / W, uy = sy / W, uz = sz / W;
                double T_cell = (2.0 / 3.0) * se;
                double wbar = W / (double)K;
                double *cdf = (double *)malloc(sizeof(double) * (size_t)np_);
                double acc = 0.0;
                for (int64_t s = 0; s < np_; ++s) { acc += tosum[LIST(s) * 4] / W; cdf[s] = acc; }
                for (int64_t k = 0; k < K; ++k) {
                    double uu = (ui < n_u) ? u[ui] : 0.5;
                    ++ui;
                    double Rv = (1.0 / (double)K) * (uu + (double)k);
                    int64_t ix = lower_bound(cdf, np_, Rv);
                    ix = ix % np_; /* CuPy wraps ids_LE[len] to ids_LE[0] */
                    int64_t id = LIST(ix);
                    memcpy(data + (Nc + k) * 6, data + id * 6, 6 * sizeof(double));
                    memcpy(tosum + (Nc + k) * 4, tosum + id * 4, 4 * sizeof(double));
                    tosum[(Nc + k) * 4] = wbar;
                }
                for (int64_t s = 0; s < np_; ++s) { int64_t id = LIST(s); memset(data + id * 6, 0, 6 * sizeof(double)); memset(tosum + id * 4, 0, 4 * sizeof(double)); }
                double hx = 0, hy = 0, hz = 0, he = 0;
                for (int64_t k = 0; k < K; ++k) he += tosum[(Nc + k) * 4] * tosum[(Nc + k) * 4 + 3];
                for (int64_t k = 0; k < K; ++k) hx += data[(Nc + k) * 6 + 3] * tosum[(Nc + k) * 4];
                for (int64_t k = 0; k < K; ++k) hy += data[(Nc + k) * 6 + 4] * tosum[(Nc + k) * 4];
                for (int64_t k = 0; k < K; ++k) hz += data[(Nc + k) * 6 + 5] * tosum[(Nc + k) * 4];
                double Te_hat = (2.0 / 3.0) * he / W;
                hx /= W; hy /= W; hz /= W;
                double Tfac;
                if (flags & 2) {
                    /* energy-conserving: scale only the thermal part (kept about its own mean) */
                    double half_m = 0.5 * m_e * j_ev;
                    /* survivors that are all one particle have no kept thermal part (the
                       subtraction leaves rounding, below 1e-12 of their energy): factor 1; an
                       original thermal part below zero by rounding counts as zero */
                    double th_o = 1.5 * T_cell - half_m * (ux * ux + uy * uy + uz * uz);
                    double th_k = 1.5 * Te_hat - half_m * (hx * hx + hy * hy + hz * hz);
                    Tfac = th_k > 1e-12 * 1.5 * Te_hat ? sqrt((th_o > 0.0 ? th_o : 0.0) / th_k) : 1.0;
                } else {
                    Tfac = sqrt(T_cell / Te_hat);
                }
                for (int64_t k = 0; k < K; ++k) {
                    double *d = data + (Nc + k) * 6;
                    d[3] = ux + (d[3] - hx) * Tfac;
                    d[4] = uy + (d[4] - hy) * Tfac;
                    d[5] = uz + (d[5] - hz) * Tfac;
                    tosum[(Nc + k) * 4 + 3] = 0.5 * m_e * j_ev * (d[3] * d[3] + d[4] * d[4] + d[5] * d[5]);
                }
                free(cdf);
                Nc += K;
            }
#undef LIST
        }
    }
    if (n_used) *n_used = ui;
    /* compaction of w != 0 (boltzmann.py:879-890) */
    int64_t na = 0;
    for (int64_t i = 0; i < Nc; ++i) {
        if (tosum[i * 4] != 0.0) {
            if (na != i) { memmove(data + na * 6, data + i * 6, 6 * sizeof(double)); memmove(tosum + na * 4, tosum + i * 4, 4 * sizeof(double)); }
            ++na;
        }
    }
    for (int64_t i = na; i < Nc; ++i) { memset(data + i * 6, 0, 6 * sizeof(double)); memset(tosum + i * 4, 0, 4 * sizeof(double)); }
    return na;
}

/* ------------------------------------------------------------------------------------ */
/* Poisson (EF_kernel_1D.py:7-44) and ion fluid (heavies_kernel_1D.py:4-64)               */
/* ------------------------------------------------------------------------------------ */
void orc_poisson(int N, double dx, double eps0, double V0, double freq, double t, const double *ne,
                 const double *ni, double *V, double *E) {
    /* banded Cholesky of tridiag(-1, 2, -1)/dx^2 (boltzmann.py:744-755) */
    int n = N - 1;
    double *d = (double *)malloc(sizeof(double) * (size_t)n);
    double *l = (double *)calloc((size_t)n, sizeof(double));
    double *y = (double *)malloc(sizeof(double) * (size_t)n);
    double *rhs = (double *)malloc(sizeof(double) * (size_t)n);
    double a = 2.0 / (dx * dx), b = -1.0 / (dx * dx);
    d[0] = sqrt(a);
    for (int i = 1; i < n; ++i) { l[i] = b / d[i - 1]; d[i] = sqrt(a - l[i] * l[i]); }
    for (int i = 0; i < n; ++i) rhs[i] = (1.0 / eps0) * (ni[i + 1] - ne[i + 1]);
    double vs = V0 * sin(2 * M_PI * freq * t);
    rhs[0] = rhs[0] + (1.0 / (dx * dx)) * vs;
    y[0] = rhs[0] / d[0];
    for (int i = 1; i < n; ++i) y[i] = (1.0 / d[i]) * (rhs[i] - l[i] * y[i - 1]);
    V[n - 1] = y[n - 1] / d[n - 1];
    for (int i = 1; i < n; ++i) V[n - 1 - i] = (1.0 / d[n - 1 - i]) * (y[n - 1 - i] - l[n - 1 - i + 1] * V[n - 1 - i + 1]);
    for (int i = 0; i < N - 2; ++i) E[i + 1] = -(V[i + 1] - V[i]) / dx;
    E[0] = -(V[0] - vs) / dx;
    E[N - 1] = -(0 - V[N - 2]) / dx;
    free(d); free(l); free(y); free(rhs);
}

int orc_fluid(int N, double dx, double dt, double mu_i, double D_i, const double *E, double *ni, double *Ji) {
    int brk = 0;
    double *rhs = (double *)malloc(sizeof(double) * (size_t)(N + 1));
    double e0 = E[0] > 0 ? E[0] : 0.0, eN = E[N - 1] < 0 ? E[N - 1] : 0.0;
    ni[0] = ni[1] * ((D_i / dx - 0.5 * mu_i * e0) / (D_i / dx + 0.5 * mu_i * e0));
    ni[N] = ni[N - 1] * ((D_i / dx + 0.5 * mu_i * eN) / (D_i / dx - 0.5 * mu_i * eN));
    for (int i = 0; i < N; ++i) Ji[i] = (mu_i * (0.5 * (ni[i] + ni[i + 1])) * E[i] - D_i * (ni[i + 1] - ni[i]) / dx);
    for (int i = 1; i < N; ++i) {
        rhs[i] = ni[i] - dt * (Ji[i] - Ji[i - 1]) / dx;
        if (rhs[i] < 0 && ni[i] > 0) brk = 1;
        ni[i] = rhs[i];
    }
    ni[0] = ni[1] * ((D_i / dx - 0.5 * mu_i * e0) / (D_i / dx + 0.5 * mu_i * e0));
    ni[N] = ni[N - 1] * ((D_i / dx + 0.5 * mu_i * eN) / (D_i / dx - 0.5 * mu_i * eN));
    free(rhs);
    return brk;
}

/* ------------------------------------------------------------------------------------ */
/* OpenMP full step: the CPU baseline                                                    */
/* ------------------------------------------------------------------------------------ */
int64_t orc_step_omp(const orc_params *p, int64_t n, int64_t cap, double *data, double *tosum,
                     double *data_tmp, double *tosum_tmp, const double *E, double *moments, int nthreads) {
    int RN = p->n_nodes;
    int M = p->bnf * RN;
    double half = 0.5 * p->dx, Lp = p->L + p->dx;
    double fM = (double)(float)M;
    int nt = nthreads > 0 ? nthreads : 1;
    /* every particle may leave one child: the output needs 2n rows, the temporaries 2n */
    if (n < 0 || 2 * n > cap) return -1;
    int64_t *cnt_s = (int64_t *)calloc((size_t)nt + 1, sizeof(int64_t));
    int64_t *cnt_c = (int64_t *)calloc((size_t)nt + 1, sizeof(int64_t));
    double *fine = (double *)calloc((size_t)nt * M * 4, sizeof(double));
    int64_t chunk = (n + nt - 1) / nt;
    (void)cap;
#pragma omp parallel num_threads(nt)
    {
#ifdef _OPENMP
        int tid = omp_get_thread_num();
#else
        int tid = 0;
#endif
        int64_t lo = tid * chunk, hi = lo + chunk < n ? lo + chunk : n;
        double *my = fine + (size_t)tid * M * 4;
        int64_t ns = 0, nc = 0;
        push_out o;
        /* pass 1: push + collide + deposit into a private fine grid, write survivors and
         * children to the temporaries at this thread's chunk offsets */
        for (int64_t i = lo; i < hi; ++i) {
            push_one(p, i, data + i * 6, tosum + i * 4, E, NULL, NULL, &o);
            int b;
            if (o.w > 0) {
                b = fine_bin(p, o.x, half, Lp, fM);
                if (b >= 0 && b < M) {
                    my[b * 4 + 0] += o.w; my[b * 4 + 1] += o.flag * o.w; my[b * 4 + 3] += o.e * o.w;
                    if (p->moment_exc && o.exc) my[b * 4 + 2] += o.w;
                }
                double *d = data_tmp + (lo + ns) * 6, *t = tosum_tmp + (lo + ns) * 4;
                d[0] = o.x; d[1] = o.y; d[2] = o.z; d[3] = o.vx; d[4] = o.vy; d[5] = o.vz;
                t[0] = o.w; t[1] = 0; t[2] = 0; t[3] = o.e;
                ++ns;
            } else if (o.flag != 0.0) {
                b = fine_bin(p, o.x, half, Lp, fM);
                if (b >= 0 && b < M) my[b * 4 + 1] += o.flag;
            }
            if (o.child) {
                b = fine_bin(p, o.cx, half, Lp, fM);
                if (b >= 0 && b < M) { my[b * 4 + 0] += o.cw; my[b * 4 + 3] += o.ce * o.cw; }
                /* children are parked in the second half of the temporaries (capacity 2n) */
                double *d = data_tmp + (n + lo + nc) * 6, *t = tosum_tmp + (n + lo + nc) * 4;
                d[0] = o.cx; d[1] = o.cy; d[2] = o.cz; d[3] = o.cvx; d[4] = o.cvy; d[5] = o.cvz;
                t[0] = o.cw; t[1] = 0; t[2] = 0; t[3] = o.ce;
                ++nc;
            }
        }
        cnt_s[tid + 1] = ns;
        cnt_c[tid + 1] = nc;
    }
    for (int t = 0; t < nt; ++t) { cnt_s[t + 1] += cnt_s[t]; cnt_c[t + 1] += cnt_c[t]; }
    int64_t total_s = cnt_s[nt];
#pragma omp parallel num_threads(nt)
    {
#ifdef _OPENMP
        int tid = omp_get_thread_num();
#else
        int tid = 0;
#endif
        int64_t lo = tid * chunk, hi = lo + chunk < n ? lo + chunk : n;
        int64_t ns = cnt_s[tid + 1] - cnt_s[tid], nc = cnt_c[tid + 1] - cnt_c[tid];
        if (lo < hi) {
            memcpy(data + cnt_s[tid] * 6, data_tmp + lo * 6, (size_t)ns * 6 * sizeof(double));
            memcpy(tosum + cnt_s[tid] * 4, tosum_tmp + lo * 4, (size_t)ns * 4 * sizeof(double));
            memcpy(data + (total_s + cnt_c[tid]) * 6, data_tmp + (n + lo) * 6, (size_t)nc * 6 * sizeof(double));
            memcpy(tosum + (total_s + cnt_c[tid]) * 4, tosum_tmp + (n + lo) * 4, (size_t)nc * 4 * sizeof(double));
        }
    }
    /* merge private grids and form node moments (race-free redcheck) */
    int bloks = M / RN;
    for (int k = 0; k < RN; ++k)
        for (int j = 0; j < 4; ++j) {
            double s = 0.0;
            for (int t = 0; t < nt; ++t)
                for (int q = 0; q < bloks; ++q) s += fine[(size_t)t * M * 4 + (size_t)(k * bloks + q) * 4 + j];
            moments[j * RN + k] = s;
        }
    int64_t nnew = total_s + cnt_c[nt];
    free(cnt_s); free(cnt_c); free(fine);
    return nnew;
}
