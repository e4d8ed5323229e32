/* CPU restatement (FP64) of the reference's electron PIC-MCC hot path.
 *
 * TEST INFRASTRUCTURE: this is the oracle that the CUDA kernels are checked against
 * and the CPU baseline that the benchmark reports beside them. Nothing on the
 * product path links it.
 *
 * Layout follows the reference: array-of-structures FP64,
 *   data[i*6 + {0:x, 1:y, 2:z, 3:vx, 4:vy, 5:vz}]   (boltzmann.py:271)
 *   tosum[i*4 + {0:w, 1:ionflag, 2:unused, 3:energy eV}] (boltzmann.py:272)
 * x in cm, v in m/s, E in V/cm, neutral density in m^-3 (the kernel's ``nn``).
 */
#ifndef BZ_ORACLE_H
#define BZ_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_params {
    int n_faces;        /* N: length of E (faces)                         */
    int n_nodes;        /* N+1: deposit nodes and binning cells           */
    int bnf;            /* fine bins per node in the deposit              */
    double L, dx, dt;   /* cm, cm, s                                      */
    double nn;          /* neutral density, m^-3                          */
    int xs_mode;        /* 0: n*sigma table, 1: reference fits            */
    int coll_model;     /* 0: direct probability (reference), 1: null collision */
    int advect;         /* 1: 1D advection + absorbing walls, 0: 0-D swarm */
    int rng_mode;       /* 0: replay R[n][7] and gas[n][3]; 1: Philox     */
    int precision;      /* uniform convention for Philox: 32 (float) or 64 (double) */
    uint64_t seed, step;
    double gas_sigma;   /* std dev of each gas velocity component, m/s (Philox mode) */
    /* n*sigma table: [3][xs_n] float32 (elastic, excitation, ionization), m^-1 */
    int xs_n;
    double xs_emin, xs_emax;
    const float *xs_table;
    double nu_max;      /* null-collision bound, s^-1 (coll_model 1) */
    double e_exc;       /* excitation threshold and loss, eV (table mode) */
    int moment_exc;     /* 1: tosum column 2 holds this step's excitation flag (deposited as sum w) */
} orc_params;

/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11). */
void orc_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
void orc_philox_rounds(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4], int rounds);

/* electron_kernel_numba.py:38-287 for particles 0..n-1; children appended at n+k in
 * parent order. Returns the number of children (the reference's curr_count). */
int64_t orc_push(const orc_params *p, int64_t n, double *data, double *tosum, const double *E,
                 const double *R, const double *gas);

/* orc_push, and margin[i] = distance of particle i's decision uniform to the nearest
 * process boundary, or of its new position to a wall (/L), whichever is smaller: where
 * float32 and float64 arithmetic may legitimately decide differently. It is 0 for an
 * inelastic collision within 5% of its threshold, where e - threshold amplifies the
 * rounding of float32 inputs beyond 1e-6 of the scattered speed. */
int64_t orc_push_margin(const orc_params *p, int64_t n, double *data, double *tosum, const double *E,
                        const double *R, const double *gas, double *margin);

/* post_processing_1D.py:40-68 with kernels-new.cu reda/redcheck (race-free): moments
 * out[4][n_nodes] = (ne, ni_src, ns_src, nrg); compacts w>0 in place; returns Nnew. */
int64_t orc_post(const orc_params *p, int64_t n_total, double *data, double *tosum, double *moments);

/* Deposit only (no compaction, no tosum mutation): the moments post_processing would
 * produce for this state. */
void orc_deposit(const orc_params *p, int64_t n_total, const double *data, const double *tosum,
                 double *moments);

/* define_particle_bins (bin_particles.py:7-22 and the 3/5-bin versions) for SoA input.
 * Energy is taken as the reference holds it at binning time: ((e*w)/w).
 * counts[nb][n_nodes] (every live particle, also beyond max_ppc);
 * lists[nb][max_ppc][n_nodes] particle indices in ascending order (-1 where empty). */
void orc_bin(const orc_params *p, int64_t n, const double *x, const double *vx, const double *vy,
             const double *vz, const double *w, int nb, const double *edges, int64_t max_ppc,
             int64_t *counts, int64_t *lists);

/* _do_resampling (boltzmann.py:799-890; 3bin :813-1060; 5bin :843-1253), AoS state.
 * counts/lists from orc_bin. Random numbers are consumed from u[] in processing order
 * (cell ascending, bins ascending in energy; split draws then merge draws).
 * flags bit0: reproduce the reference's split indexing (HW_ids[unique_ids[v]] with
 * CuPy's wrap-around); bit1: energy-conserving merge rescale (thermal part only);
 * bit4: targets and max_ppc per (cell, bin) key, index cell*nb + bin.
 * thr = {split_below, merge_at, merge_keep}, or NULL for the reference's 0.5, 3, 0.6.
 * Returns the particle count after the final compaction; *n_used = uniforms consumed. */
int64_t orc_resample(const orc_params *p, int64_t n, double *data, double *tosum, int nb,
                     const int64_t *targets, double min_wt, const int64_t *max_ppc,
                     const int64_t *counts, const int64_t *lists, int64_t list_stride,
                     const double *u, int64_t n_u, int64_t *n_used, int flags, const double *thr);

/* Energy distribution per deposit node (the swarm in an ensemble): hist[n_nodes][nbins]
 * += w in bin floor(nbins ln(e/emin)/ln(emax/emin)); energies outside [emin, emax) skipped. */
void orc_eedf(const orc_params *p, int64_t n, const double *x, const double *vx, const double *vy,
              const double *vz, const double *w, int nbins, double emin, double emax, double *hist);

/* EF_kernel_1D.py:7-44 with the banded Cholesky factor of boltzmann.py:744-755. */
void orc_poisson(int N, double dx, double eps0, double V0, double freq, double t, const double *ne,
                 const double *ni, double *V /*N-1*/, double *E /*N*/);

/* heavies_kernel_1D.py:4-64 (ion part; the never-sourced species is zero). Returns break_flag. */
int orc_fluid(int N, double dx, double dt, double mu_i, double D_i, const double *E, double *ni,
              double *Ji);

/* Full-step CPU baseline (OpenMP over particles): push (Philox, table) + deposit +
 * compaction, the reference's step order. data/tosum have capacity cap >= 2n; the
 * temporaries hold 2n rows. Returns Nnew, or -1 (nothing written) when 2n > cap. */
int64_t orc_step_omp(const orc_params *p, int64_t n, int64_t cap, double *data, double *tosum,
                     double *data_tmp, double *tosum_tmp, const double *E, double *moments,
                     int nthreads);

#ifdef __cplusplus
}
#endif
#endif
