/* libbz: GB300 (sm_103a) electron PIC-MCC hot path behind a C ABI.
 *
 * Drop-in replacement for the device work that jfabell/boltzmann's solver class binds
 * in BoltzmannDSMC._init_kernels (boltzmann.py:758-795). Every function:
 *   - takes plain device pointers owned by the caller (any allocator: torch, cudaMalloc);
 *   - enqueues work on the caller's stream (``stream`` is a cudaStream_t) and does not
 *     synchronise; particle counts live in device memory, so a whole step can be
 *     captured in a CUDA graph;
 *   - returns a bz_status code (0 = enqueued); conditions found on the device
 *     (capacity exhausted, look-back timeout, NaN) are OR-ed into the caller's
 *     ``status`` word as BZ_DEV_* bits, which the host reads when it wants to.
 * Errors never trap or abort on the device.
 *
 * Particle state is structure-of-arrays (x, vx, vy, vz, w), all float32 (``_f32``
 * entry points) or all float64 (``_f64``), with x in cm, v in m/s and w in the
 * reference's density units. The reference keeps y, z positions that no 1D quantity
 * reads (boltzmann.py:271); they are not stored.
 */
#ifndef BZ_H
#define BZ_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* host-side return codes */
enum bz_status {
    BZ_OK = 0,
    BZ_ERR_ARG = 1,       /* null pointer, bad size or mode            */
    BZ_ERR_CUDA = 2,      /* a CUDA call failed (launch, memset)        */
    BZ_ERR_WORKSPACE = 3, /* workspace smaller than bz_*_workspace says  */
    BZ_ERR_UNSUPPORTED = 4,
    BZ_ERR_TOO_LARGE = 5  /* input larger than a fixed-size entry point supports */
};

/* device-side status bits (OR-ed into *status) */
#define BZ_DEV_CAPACITY 0x1u   /* output capacity exceeded; extra particles dropped */
#define BZ_DEV_LOOKBACK 0x2u   /* a look-back wait hit its iteration limit            */
#define BZ_DEV_NONFINITE 0x4u  /* non-finite velocity or weight produced               */
#define BZ_DEV_BINRANGE 0x8u   /* a live particle outside every cell / energy bin        */

/* reference behaviours reproduced on request (bz_params.flags) */
#define BZ_QUIRK_SPLIT_WRAP 0x1u     /* split copies HW_ids[id % nHW] (boltzmann.py:820-822, CuPy wrap) */
#define BZ_QUIRK_DEAD_IONFLAG 0x2u   /* an ionized particle that leaves adds 1 to ni_src[0]
                                        (unweighted ion flag at x=1e-8, post_processing_1D.py:50-55) */
#define BZ_QUIRK_TRIGGER_LAST 0x4u   /* resampling decided by the last bin's max test only
                                        (boltzmann.py:913-916, 3bin :1108-1111, 5bin :1329-1334) */
#define BZ_FIX_MERGE_ENERGY 0x8u     /* merge rescales the thermal part only: energy conserving */
#define BZ_PER_KEY_TARGETS 0x10u     /* resampling targets and max_ppc are given per (cell, bin) key
                                        (key = cell*nbins + bin) instead of per bin */
#define BZ_MOMENT_EXCITATION 0x20u   /* the push's deposit adds sum(w) of the particles that excited
                                        this step to moments row 2 (ns_src, always 0 in the reference) */
#define BZ_CLEAR_MOMENTS 0x40u       /* the push clears moments (4 x n_nodes float64) before it
                                        accumulates into them (a memset on the caller's stream) */
#define BZ_RESAMPLE_IN_PLACE 0x80u   /* bz_seg_resample_*: the result stays in s (bz_seg_place_*: the
                                        appended particles into free slots, merged ones left as w = 0);
                                        out is only the scratch of a repack when they do not fit */

/* particle motion (bz_params.advect) */
#define BZ_ADVECT_NONE 0      /* one 0-D swarm: no drift, E[0] everywhere, every particle in node/cell 0 */
#define BZ_ADVECT_1D 1        /* 1D drift with absorbing walls at 0 and L; E at face int(x/dx) */
#define BZ_ADVECT_ENSEMBLE 2  /* independent 0-D swarms: x holds the swarm index s (an integer value);
                                 no drift; swarm s sees E[s] and deposits / bins into node / cell s */

/* cross-section modes */
#define BZ_XS_TABLE 0     /* n*sigma tables on a log energy grid (elastic, excitation, ionization) */
#define BZ_XS_REF_FITS 1  /* the reference's log10-quadratic fits, evaluated in FP64
                             (electron_kernel_numba.py:66-174) */
/* collision models */
#define BZ_COLL_DIRECT 0  /* P = 1-exp(-n sigma_tot v dt), process by R0 (electron_kernel_numba.py:187-198) */
#define BZ_COLL_NULL 1    /* null collision with bound nu_max */

typedef struct bz_params {
    /* grid: N faces (E), N+1 nodes (deposit / binning cells) */
    int32_t n_faces;
    int32_t n_nodes;
    int32_t bnf;        /* fine bins per node of the reference deposit (post_processing bnf) */
    int32_t advect;     /* BZ_ADVECT_*: 1D advection, one 0-D swarm, or an ensemble of swarms */
    double L, dx;       /* cm */
    /* physics */
    double dt;          /* s */
    double nn;          /* neutral density, m^-3 */
    double gas_sigma;   /* std dev of each gas velocity component, m/s (0: off) */
    double e_exc;       /* excitation threshold and energy loss, eV */
    double nu_max;      /* null-collision bound, s^-1 */
    int32_t xs_mode;    /* BZ_XS_* */
    int32_t coll_model; /* BZ_COLL_* */
    int32_t xs_n;       /* points of the n*sigma table */
    int32_t flags;      /* BZ_QUIRK_* | BZ_FIX_* */
    double xs_emin, xs_emax;  /* eV, log grid end points */
    const float *xs_table;    /* device, [3][xs_n], n*sigma in m^-1 (elastic, excitation, ionization) */
    /* counter-based random numbers: Philox4x32-10 keyed by seed, counter (slot, step) */
    uint64_t seed;
    uint64_t step;
    const uint64_t *step_ptr; /* device; when set, the step is read from it (CUDA graph replay) */
} bz_params;

typedef struct bz_particles_f32 { float *x, *vx, *vy, *vz, *w; } bz_particles_f32;
typedef struct bz_particles_f64 { double *x, *vx, *vy, *vz, *w; } bz_particles_f64;

/* ---------------------------------------------------------------------------------- */
/* push + collide (+ fused deposit and compaction)                                     */
/* ---------------------------------------------------------------------------------- */
/* Replaces electron_kernel (electron_kernel_numba.py:291-303) together with the
 * deposit and per-step compaction of post_processing (post_processing_1D.py:40-68,
 * reduction/__init__.py:3-11 -> kernels-new.cu calls).
 *
 * in[0 .. *n_in) is pushed and collided; particles that stay alive are written to
 * out[0 .. ns) in input order, then the ionization children in parent order,
 * out[ns .. ns+nc): the reference's order after reshuffle_data_atomics. counts[0] = ns,
 * counts[1] = nc, counts[2] = ns+nc. Input particles with w <= 0 are dropped.
 * moments (optional, [4][n_nodes] float64, accumulated into: zero it first) receives
 * (sum w, sum w*ionflag, 0, sum w*energy) at node int(((x+dx/2)/(L+dx))*bnf*n_nodes)/bnf,
 * the reference's ne, ni_src, ns_src, nrg before the division by the host.
 * Random numbers: Philox (replay_R == NULL) or replayed, R[i][7] and gas[i][3]
 * float64 arrays in the reference's layout (electron_kernel_numba.py:195-238, boltzmann.py:589).
 * in and out must not overlap. A count above in_capacity is clamped to it and
 * BZ_DEV_CAPACITY is raised; out_capacity must leave room for ns + 2*nc (children are
 * staged at the tail before they are moved behind the survivors). */
size_t bz_push_workspace(int64_t capacity);
/* With a workspace of this many bytes (or more) the same call pushes through the segmented
 * kernel instead: the input read as segments of 2048 particles (each particle keeps its
 * index as its Philox counter, so the results are the same), pushed into segments held in
 * the workspace (about 40 * in_capacity bytes in float32), then gathered into the order
 * above; no tile waits for its predecessors' counts. Particles beyond out_capacity are
 * dropped with BZ_DEV_CAPACITY (children first); n_nodes is bz_params.n_nodes. */
size_t bz_push_workspace_fast_f32(int64_t in_capacity, int32_t n_nodes);
size_t bz_push_workspace_fast_f64(int64_t in_capacity, int32_t n_nodes);
int bz_push_collide_f32(const bz_params *p, bz_particles_f32 in, const int32_t *n_in, int64_t in_capacity,
                        bz_particles_f32 out, int64_t out_capacity, int32_t *counts,
                        const float *E, const double *replay_R, const double *replay_gas,
                        double *moments, void *workspace, size_t workspace_bytes,
                        uint32_t *status, void *stream);
int bz_push_collide_f64(const bz_params *p, bz_particles_f64 in, const int32_t *n_in, int64_t in_capacity,
                        bz_particles_f64 out, int64_t out_capacity, int32_t *counts,
                        const double *E, const double *replay_R, const double *replay_gas,
                        double *moments, void *workspace, size_t workspace_bytes,
                        uint32_t *status, void *stream);

/* Deposit only: the moments post_processing forms for a state (kernels-new.cu:56-132,
 * race-free). ionflag (optional, uint8 per particle) is the reference's tosum[:,1]. */
int bz_deposit_f32(const bz_params *p, bz_particles_f32 s, const int32_t *n, int64_t capacity,
                   const uint8_t *ionflag, double *moments, void *stream);
int bz_deposit_f64(const bz_params *p, bz_particles_f64 s, const int32_t *n, int64_t capacity,
                   const uint8_t *ionflag, double *moments, void *stream);

/* ---------------------------------------------------------------------------------- */
/* binning: cell x energy-bin key, stable counting sort                                 */
/* ---------------------------------------------------------------------------------- */
/* Replaces define_particle_bins (bin_particles.py:7-22; 3bin/5bin :7-49) and the table
 * fills of _check_for_resampling (boltzmann.py:898-903). Key = cell*nbins + ebin with
 * cell = int((x+dx/2)/dx) (boltzmann.py:658) and ebin from the energy against
 * edges[nbins-1] (eV, ascending). Live particles only (w > 0).
 * perm[0 .. live) lists particle indices sorted by key, ascending index within a key;
 * offsets[k] / counts[k] give key k's slice; hw_counts[k] counts particles with
 * w > min_wt (split candidates, boltzmann.py:809). nkeys = n_nodes*nbins <= 65535. */
size_t bz_bin_workspace(int64_t capacity, int32_t nkeys);
int bz_bin_f32(const bz_params *p, bz_particles_f32 s, const int32_t *n, int64_t capacity, int32_t nbins,
               const double *edges, double min_wt, int32_t *perm, int32_t *offsets, int32_t *counts,
               int32_t *hw_counts, void *workspace, size_t workspace_bytes, uint32_t *status, void *stream);
int bz_bin_f64(const bz_params *p, bz_particles_f64 s, const int32_t *n, int64_t capacity, int32_t nbins,
               const double *edges, double min_wt, int32_t *perm, int32_t *offsets, int32_t *counts,
               int32_t *hw_counts, void *workspace, size_t workspace_bytes, uint32_t *status, void *stream);

/* ---------------------------------------------------------------------------------- */
/* ES-WPNC resampling                                                                   */
/* ---------------------------------------------------------------------------------- */
/* Replaces _check_for_resampling + _do_resampling (boltzmann.py:799-916; 3bin
 * :813-1113; 5bin :843-1334): per (cell, bin), split when 0 < n < split_below*T and a
 * particle has w > min_wt (draw 2T-n copies with probability w), merge when
 * n >= merge_at*T (keep int(merge_keep*T) by stratified sampling, weight W/K, velocity
 * rescale). targets[nbins], max_ppc[nbins] as the reference (T, 10T).
 * Appended particles go to s[*n ..) in (cell, bin) order; merged originals get w = 0;
 * then the state is compacted into ``out`` (w != 0 kept in order, boltzmann.py:879-890).
 * Random numbers: Philox (replay_u == NULL) or replay_u[] consumed in processing order
 * (per key: split draws or merge draws). need_out[0] = 1 when resampling ran.
 * capacity bounds both s and out.
 * cons_diag (optional, [nkeys][BZ_CONS_DIAG_STRIDE] float64, zeroed for keys that do not
 * merge): W, px, py, pz, sum w*energy of the merged originals; the same of the survivors
 * as stored (weights and velocities in the state's precision); the same of the survivors
 * as formed in float64 before they are stored (K * W/K and the rescaled velocities). */
#define BZ_CONS_DIAG_STRIDE 15
size_t bz_resample_workspace(int64_t capacity, int32_t nkeys);
int bz_resample_f32(const bz_params *p, bz_particles_f32 s, const int32_t *n, int64_t capacity,
                    bz_particles_f32 out, int32_t *n_out, int32_t nbins, const int32_t *targets,
                    const int32_t *max_ppc, double min_wt, double split_below, double merge_at,
                    double merge_keep, const int32_t *perm, const int32_t *offsets, const int32_t *counts,
                    const int32_t *hw_counts, const double *replay_u, int32_t *need_out, double *cons_diag,
                    void *workspace, size_t workspace_bytes, uint32_t *status, void *stream);
int bz_resample_f64(const bz_params *p, bz_particles_f64 s, const int32_t *n, int64_t capacity,
                    bz_particles_f64 out, int32_t *n_out, int32_t nbins, const int32_t *targets,
                    const int32_t *max_ppc, double min_wt, double split_below, double merge_at,
                    double merge_keep, const int32_t *perm, const int32_t *offsets, const int32_t *counts,
                    const int32_t *hw_counts, const double *replay_u, int32_t *need_out, double *cons_diag,
                    void *workspace, size_t workspace_bytes, uint32_t *status, void *stream);

/* Order-preserving compaction of w != 0 (boltzmann.py:879-883). */
size_t bz_compact_workspace(int64_t capacity);
int bz_compact_f32(bz_particles_f32 in, const int32_t *n, int64_t in_capacity, bz_particles_f32 out,
                   int64_t out_capacity, int32_t *n_out, void *workspace, size_t workspace_bytes,
                   uint32_t *status, void *stream);
int bz_compact_f64(bz_particles_f64 in, const int32_t *n, int64_t in_capacity, bz_particles_f64 out,
                   int64_t out_capacity, int32_t *n_out, void *workspace, size_t workspace_bytes,
                   uint32_t *status, void *stream);

/* ---------------------------------------------------------------------------------- */
/* grid: ion fluid and Poisson (FP64, device resident)                                  */
/* ---------------------------------------------------------------------------------- */
/* Host-side grid update of the step loop (boltzmann.py:643-647): ni += ni_src,
 * Te = (2/3) nrg/ne (NaN -> 0), g2 += ni_src, from moments[4][n_nodes]. */
int bz_grid_update(int32_t n_nodes, const double *moments, double *ni, double *Te, double *g2, void *stream);
/* Ion-source rate closure (no counterpart in the reference, whose ion source is always the
 * push's counted ionizations, post_processing_1D.py:50-55 -> boltzmann.py:643): replaces
 * moments row 1 (ni_src) by rate[i] * moments row 0 (ne) for every node, rate[n_nodes] the
 * ionizations per electron per step (k_ion n_gas dt, e.g. from the learned start-up's
 * network). Launched between the push and the grid step. */
int bz_ion_source_closure(int32_t n_nodes, const double *rate, double *moments, void *stream);
/* heavies_kernel_fluid (heavies_kernel_1D.py:4-64), ion part; break flag -> *brk. */
int bz_ion_fluid(int32_t N, double dx, double dt, double mu_i, double D_i, const double *E, double *ni,
                 double *Ji, int32_t *brk, void *stream);
/* EF_kernel (EF_kernel_1D.py:7-44) with the banded Cholesky factor of boltzmann.py:744-755.
 * bz_poisson_factor (once per grid, synchronous) writes the factor chol_diag[N-1],
 * chol_lower[N-1] and the solve plan[4*(N-1)]: the substitutions' prefix products and
 * scaled reciprocals, so that each solve is two prefix sums. bz_poisson: t is read from
 * *t_dev when t_dev != NULL (graph capture), else t_host. Writes V[N-1] and E (float64
 * [N]); E32 (optional) receives a float32 copy for the float32 push. */
int bz_poisson_factor(int32_t N, double dx, double *chol_diag, double *chol_lower, double *plan);
int bz_poisson(int32_t N, double dx, double eps0, double V0, double freq, double t_host, const double *t_dev,
               const double *ne, const double *ni, const double *plan, double *V, double *E, float *E32,
               void *stream);
/* The grid part of one step in one launch, in the step loop's order (boltzmann.py:643-678):
 * bz_grid_update (ni += ni_src, Te, g2), the clock (*t_dev += dt, *step_dev += 1),
 * bz_ion_fluid with the field of the last solve, bz_poisson at the new time (moments row 0
 * is ne). Te, g2, step_dev, E32 and brk may be NULL. */
int bz_field_step(int32_t N, double dx, double dt, double mu_i, double D_i, double eps0, double V0, double freq,
                  const double *moments, double *ni, double *Te, double *g2, double *t_dev, uint64_t *step_dev,
                  const double *plan, double *V, double *E, float *E32, double *Ji, int32_t *brk, void *stream);
/* Step clock on the device (graph-capturable): *t_dev += dt, *step_dev += 1 (either may be NULL). */
int bz_advance_clock(double *t_dev, uint64_t *step_dev, double dt, void *stream);
/* bz_field_step over G = ceil((N-1)/64) CTAs with barriers over all of them between the
 * phases: the float64 work is spread over G SMs. Where G <= 16 (N <= 1025) and the device
 * can form such a cluster, the CTAs are one thread-block cluster and the barriers are the
 * cluster's hardware barrier; otherwise one cooperative launch with grid-wide barriers.
 * Same results up to the association of the Poisson substitution sums. workspace:
 * bz_field_step_coop_workspace(N) bytes; BZ_ERR_TOO_LARGE when the cooperative CTAs cannot
 * all be resident. */
size_t bz_field_step_coop_workspace(int32_t N);
int bz_field_step_coop(int32_t N, double dx, double dt, double mu_i, double D_i, double eps0, double V0,
                       double freq, const double *moments, double *ni, double *Te, double *g2, double *t_dev,
                       uint64_t *step_dev, const double *plan, double *V, double *E, float *E32, double *Ji,
                       int32_t *brk, void *workspace, size_t workspace_bytes, void *stream);
/* Which form bz_field_step_coop takes: 0 the cluster form where it fits, else the
 * cooperative one (default); 1 always cooperative; 2 always the cluster form
 * (BZ_ERR_UNSUPPORTED where it does not fit). Process-wide. */
int bz_field_step_select(int32_t mode);
int bz_field_step_selected(void);

/* ---------------------------------------------------------------------------------- */
/* segmented particle state (the solver's hot loop)                                      */
/* ---------------------------------------------------------------------------------- */
/* No counterpart in the reference; a layout of the same particles. nseg segments of
 * 2*half slots (half a multiple of 4); segment s holds run 0 at slots
 * [s*2*half, s*2*half + counts[2s]) and run 1 at [s*2*half + half, ... + counts[2s+1]).
 * The segmented push processes every segment with one warp and needs no ordering
 * between segments; within a segment the output order is the reference's (survivors of
 * run 0 then run 1 in order into run 0, children in parent order into run 1). A segment
 * must hold at most half particles before a push; a push that leaves a segment above
 * half sets BZ_SEG_NEEDS_REPACK in *seg_flags, and bz_seg_repack_* (conditional on that
 * flag when only_if is given) spreads the particles evenly again. */
typedef struct bz_segments_f32 { float *x, *vx, *vy, *vz, *w; int32_t *counts; int32_t nseg, half; } bz_segments_f32;
typedef struct bz_segments_f64 { double *x, *vx, *vy, *vz, *w; int32_t *counts; int32_t nseg, half; } bz_segments_f64;
#define BZ_SEG_NEEDS_REPACK 0x1u

/* Push + collide (+ deposit) of a segmented state into another (same nseg, half); the
 * per-particle arithmetic of bz_push_collide_*. Philox counters use the input slot.
 * Slots with w <= 0 (left by merges) are dropped, not pushed. n_pushed (optional, device)
 * accumulates the number of input particles pushed (w > 0). Slots are
 * indexed with 32 bits: nseg * 2 * half above 2^32 - 1 returns BZ_ERR_TOO_LARGE. */
size_t bz_seg_push_workspace(void);
/* A workspace of this many bytes (or more) also holds, for the float32 push with an n*sigma
 * table, the direct collision model, 1D drift and a deposit (the tuned kernels), one float2
 * (sum w, sum w*energy) per node for every CTA: the deposit then accumulates there by vector
 * reductions in L2 instead of by shared-memory atomics (float32 per-CTA sums as before,
 * merged into the float64 moments at the CTA's end). Any workspace of at least
 * bz_seg_push_workspace() bytes works; the larger one is faster. */
size_t bz_seg_push_workspace_nodes(int32_t n_nodes);
int bz_seg_push_collide_f32(const bz_params *p, bz_segments_f32 in, bz_segments_f32 out, const float *E,
                            const double *replay_R, const double *replay_gas, double *moments,
                            uint64_t *n_pushed, void *workspace, size_t workspace_bytes, uint32_t *seg_flags,
                            uint32_t *status, void *stream);
int bz_seg_push_collide_f64(const bz_params *p, bz_segments_f64 in, bz_segments_f64 out, const double *E,
                            const double *replay_R, const double *replay_gas, double *moments,
                            uint64_t *n_pushed, void *workspace, size_t workspace_bytes, uint32_t *seg_flags,
                            uint32_t *status, void *stream);
/* CTA shapes of the float32 table + deposit segmented push (threads per CTA, particles
 * per lane per round, CTAs per SM the registers are budgeted for, whether the next
 * round is prefetched into registers). Shape 0 is the default; bz_seg_push_select sets
 * the shape later launches use (process-wide; select before capturing a graph) in the
 * 1D-drift and ensemble modes with the direct collision probability, whose kernels have
 * both modes fixed at compile time; other modes run shape 0. Results do not depend on the
 * shape except for the summation order of the float moments. */
int32_t bz_seg_push_shapes(void);
int bz_seg_push_shape_info(int32_t shape, int32_t *threads, int32_t *per_lane, int32_t *min_blocks,
                           int32_t *prefetch);
int bz_seg_push_select(int32_t shape);
int32_t bz_seg_push_selected(void);
/* All particles with w != 0 of *in (segment order, run 0 then run 1; in may be NULL)
 * followed by app[0 .. *app_n) (may be absent: app_n NULL), spread over out's segments,
 * ceil(total/nseg) each in run 0. Skipped entirely when only_if != NULL and its
 * BZ_SEG_NEEDS_REPACK bit is clear; clears *seg_flags when it runs (if given). */
size_t bz_seg_repack_workspace(int32_t nseg_in);
int bz_seg_repack_f32(const bz_segments_f32 *in, bz_particles_f32 app, const int32_t *app_n,
                      int64_t app_capacity, bz_segments_f32 out, void *workspace, size_t workspace_bytes,
                      const uint32_t *only_if, uint32_t *seg_flags, uint32_t *status, void *stream);
int bz_seg_repack_f64(const bz_segments_f64 *in, bz_particles_f64 app, const int32_t *app_n,
                      int64_t app_capacity, bz_segments_f64 out, void *workspace, size_t workspace_bytes,
                      const uint32_t *only_if, uint32_t *seg_flags, uint32_t *status, void *stream);
/* Repack s through scratch (same geometry) and back into s, in one launch: what a caller
 * whose graph fixes the buffer roles needs after a push that filled a segment. Same
 * workspace (bz_seg_repack_workspace(s.nseg)), only_if and seg_flags rules. */
int bz_seg_rebalance_f32(bz_segments_f32 s, bz_segments_f32 scratch, void *workspace, size_t workspace_bytes,
                         const uint32_t *only_if, uint32_t *seg_flags, uint32_t *status, void *stream);
int bz_seg_rebalance_f64(bz_segments_f64 s, bz_segments_f64 scratch, void *workspace, size_t workspace_bytes,
                         const uint32_t *only_if, uint32_t *seg_flags, uint32_t *status, void *stream);
/* Places app[0 .. *app_n) (capped at app_capacity) into s in place, the step after a
 * resampling's merges and splits: into the free slots of run 1 of each segment, after its n1
 * particles. Segment k, with live_k slots of w != 0, takes at most
 * min(half - n1_k, half - live_k), so that the next push cannot overflow it: first up to
 * ceil(total / nseg) live particles in all, then what is left in segment order; app order
 * is kept within each of the two passes. Slots with w = 0 stay (a push or repack drops
 * them). When the particles do not fit that way, or a segment holds more than half live
 * particles, s and app are repacked through scratch (s's geometry) and back into s instead,
 * evenly as bz_seg_repack_* spreads them. Either way *seg_flags (if given) is cleared.
 * Workspace: bz_seg_place_workspace(s.nseg) bytes. BZ_ERR_TOO_LARGE when
 * 2 * nseg * half exceeds INT32_MAX. */
size_t bz_seg_place_workspace(int32_t nseg);
int bz_seg_place_f32(bz_segments_f32 s, bz_particles_f32 app, const int32_t *app_n, int64_t app_capacity,
                     bz_segments_f32 scratch, void *workspace, size_t workspace_bytes, uint32_t *seg_flags,
                     uint32_t *status, void *stream);
int bz_seg_place_f64(bz_segments_f64 s, bz_particles_f64 app, const int32_t *app_n, int64_t app_capacity,
                     bz_segments_f64 scratch, void *workspace, size_t workspace_bytes, uint32_t *seg_flags,
                     uint32_t *status, void *stream);
/* Moments (sum w, 0, 0, sum w*energy) of a segmented state (no ion flags are stored). */
int bz_seg_deposit_f32(const bz_params *p, bz_segments_f32 s, double *moments, void *stream);
int bz_seg_deposit_f64(const bz_params *p, bz_segments_f64 s, double *moments, void *stream);
/* Electron energy distribution: adds sum(w) per (node, energy bin) to hist[n_nodes][nbins]
 * (float64, accumulated; zero it first). Bin k covers [emin r^k, emin r^(k+1)) eV with
 * r = (emax/emin)^(1/nbins), i.e. k = floor(nbins ln(e/emin) / ln(emax/emin)) with e in
 * float64 from the stored velocities; energies outside [emin, emax) are not counted. The
 * node is the deposit node (the swarm in an ensemble). */
int bz_seg_eedf_f32(const bz_params *p, bz_segments_f32 s, int32_t nbins, double emin, double emax, double *hist,
                    void *stream);
int bz_seg_eedf_f64(const bz_params *p, bz_segments_f64 s, int32_t nbins, double emin, double emax, double *hist,
                    void *stream);
/* Binning of a segmented state: as bz_bin_*, perm holds slot indices. */
size_t bz_seg_bin_workspace(int32_t nseg, int64_t capacity);
int bz_seg_bin_f32(const bz_params *p, bz_segments_f32 s, int32_t nbins, const double *edges, double min_wt,
                   int32_t *perm, int32_t *offsets, int32_t *counts, int32_t *hw_counts, void *workspace,
                   size_t workspace_bytes, uint32_t *status, void *stream);
int bz_seg_bin_f64(const bz_params *p, bz_segments_f64 s, int32_t nbins, const double *edges, double min_wt,
                   int32_t *perm, int32_t *offsets, int32_t *counts, int32_t *hw_counts, void *workspace,
                   size_t workspace_bytes, uint32_t *status, void *stream);
/* Binning of a segmented state that also evaluates the resampling trigger (the rule of
 * bz_seg_resample_*: targets per bin, or per key with BZ_PER_KEY_TARGETS; BZ_QUIRK_TRIGGER_LAST
 * in p->flags) from the counts before it sorts: *need_out (device, may be NULL) gets 1 or 0,
 * and when it is 0 the sort is skipped, so perm and offsets are valid only when resampling
 * will run. counts and hw_counts are always complete. Workspace: bz_seg_bin_workspace. */
int bz_seg_bin_check_f32(const bz_params *p, bz_segments_f32 s, int32_t nbins, const double *edges, double min_wt,
                         int32_t *perm, int32_t *offsets, int32_t *counts, int32_t *hw_counts, const int32_t *targets,
                         double split_below, double merge_at, int32_t *need_out, void *workspace,
                         size_t workspace_bytes, uint32_t *status, void *stream);
int bz_seg_bin_check_f64(const bz_params *p, bz_segments_f64 s, int32_t nbins, const double *edges, double min_wt,
                         int32_t *perm, int32_t *offsets, int32_t *counts, int32_t *hw_counts, const int32_t *targets,
                         double split_below, double merge_at, int32_t *need_out, void *workspace,
                         size_t workspace_bytes, uint32_t *status, void *stream);
/* ES-WPNC resampling of a segmented state: as bz_resample_*, with the appended particles
 * collected in app (capacity app_capacity) and everything repacked into out; with
 * BZ_RESAMPLE_IN_PLACE in p->flags the result stays in s instead (bz_seg_place_* with out
 * as its scratch: out then needs s's geometry). */
size_t bz_seg_resample_workspace(int32_t nseg, int64_t capacity, int32_t nkeys);
int bz_seg_resample_f32(const bz_params *p, bz_segments_f32 s, bz_particles_f32 app, int64_t app_capacity,
                        bz_segments_f32 out, int32_t nbins, const int32_t *targets, const int32_t *max_ppc,
                        double min_wt, double split_below, double merge_at, double merge_keep,
                        const int32_t *perm, const int32_t *offsets, const int32_t *counts,
                        const int32_t *hw_counts, const double *replay_u, int32_t *need_out,
                        double *cons_diag, void *workspace, size_t workspace_bytes, uint32_t *seg_flags,
                        uint32_t *status, void *stream);
int bz_seg_resample_f64(const bz_params *p, bz_segments_f64 s, bz_particles_f64 app, int64_t app_capacity,
                        bz_segments_f64 out, int32_t nbins, const int32_t *targets, const int32_t *max_ppc,
                        double min_wt, double split_below, double merge_at, double merge_keep,
                        const int32_t *perm, const int32_t *offsets, const int32_t *counts,
                        const int32_t *hw_counts, const double *replay_u, int32_t *need_out,
                        double *cons_diag, void *workspace, size_t workspace_bytes, uint32_t *seg_flags,
                        uint32_t *status, void *stream);

/* ---------------------------------------------------------------------------------- */
/* bounded device-side waits                                                            */
/* ---------------------------------------------------------------------------------- */
/* No counterpart in the reference (its only device-side check is the ion fluid's break
 * flag, heavies_kernel_1D.py:44-46). Every wait on the device is bounded: the look-back of
 * bz_push_collide_* and bz_compact_* (default 2^22 polls) and the tensor-core completion
 * waits of the network kernels (default 2^24 polls). A wait that runs out raises
 * BZ_DEV_LOOKBACK (the network kernels: in bz_mlp_status), stops waiting and returns.
 * bz_set_wait_limit sets one limit for all of them (0 restores the defaults);
 * process-wide, read by later launches. */
int bz_set_wait_limit(uint32_t spins);
uint32_t bz_wait_limit(void);
/* The look-back on its own, for checks of its timeout: ntiles - first_tile single-warp
 * CTAs take tiles first_tile, first_tile+1, ... and each publishes one survivor;
 * prefix[tile] receives the exclusive prefix it sees (0xffffffff for tiles nobody took).
 * first_tile = 1 leaves tile 0 unpublished, so the waits that reach it run out and count
 * it as empty. workspace: bz_lookback_selftest_workspace(ntiles) bytes. */
size_t bz_lookback_selftest_workspace(int32_t ntiles);
int bz_lookback_selftest(int32_t ntiles, int32_t first_tile, uint32_t *prefix, void *workspace,
                         size_t workspace_bytes, uint32_t *status, void *stream);
/* The network kernels' tensor-core completion wait on its own (one CTA: TMEM allocated,
 * mbarrier for one arrival, the bounded wait, TMEM freed). arrive = 1: the arrival comes
 * and *done = 1; arrive = 0: nothing arrives, the wait runs out, *done = 2 and
 * BZ_DEV_LOOKBACK is raised in bz_mlp_status. done is a device pointer. */
int bz_mlp_wait_selftest(int32_t arrive, uint32_t *done, void *stream);

/* ---------------------------------------------------------------------------------- */
/* allocation-free push                                                                 */
/* ---------------------------------------------------------------------------------- */
/* No counterpart in the reference. The same fused push + collide + deposit + compaction
 * as bz_push_collide_f32, for callers that cannot allocate device memory: code running
 * inside a host process whose allocator it does not own (a plugin loaded into another
 * solver, or a tool that must not grow the pool of a framework sharing the GPU) and
 * code that must not call cudaMalloc at all. Instead of a caller workspace it uses one
 * scratch array compiled into the library (BZ_PUSH_NOALLOC_SCRATCH_BYTES, 512 KiB plus
 * a 256-byte header), which the CUDA runtime places on every GPU that loads the library
 * and keeps until the process exits. Limits and behaviour:
 *   - in_capacity may not exceed BZ_PUSH_NOALLOC_MAX_PARTICLES (64 Mi particles);
 *     larger inputs return BZ_ERR_TOO_LARGE and nothing is launched;
 *   - the first call in a CUDA context looks up the array's device address in that
 *     context (with it current) and remembers it under the context's unique id, so hosts
 *     that make their own contexts or reset the device get the right address; make that
 *     first call before capturing any stream;
 *   - every call on a device shares the one array and clears it first, so calls that
 *     overlap on the GPU (two streams, or two threads) race: serialise them;
 *   - nothing is allocated: no cudaMalloc, no cudaFree, no allocating library call. */
#define BZ_PUSH_NOALLOC_MAX_PARTICLES (64ll * 1024 * 1024)
#define BZ_PUSH_NOALLOC_SCRATCH_BYTES (256 + 8 * (BZ_PUSH_NOALLOC_MAX_PARTICLES / 1024))
int bz_push_collide_f32_noalloc(const bz_params *p, bz_particles_f32 in, const int32_t *n_in,
                                int64_t in_capacity, bz_particles_f32 out, int64_t out_capacity,
                                int32_t *counts, const float *E, const double *replay_R,
                                const double *replay_gas, double *moments, uint32_t *status,
                                void *stream);
/* The scratch array's device address in the current context (the set-up of the first
 * call, run now if it has not run yet); for checks that a context switch is seen. */
int bz_push_noalloc_scratch_address(void **address);

/* ---------------------------------------------------------------------------------------
 * Surrogate network of the learned CCP start-up (no counterpart in the reference: its
 * runs always start from the plain initial state, boltzmann.py:271-312). A fully
 * connected network of BZ_MLP_LAYERS weight layers: BZ_MLP_IN inputs (the features,
 * zero-padded), BZ_MLP_LAYERS-1 hidden layers of BZ_MLP_HIDDEN GELU units (tanh form),
 * BZ_MLP_OUT linear outputs (zero-padded). Matrix products take BF16 operands and
 * accumulate in FP32 on the tensor cores; biases, pre-activations, outputs, gradients
 * and the Adam state are FP32.
 *
 * Parameters: one FP32 array of BZ_MLP_NPARAM values, layer by layer: W_l (out_l x in_l,
 * row-major) followed by b_l (out_l). The BF16 copies `wb` (same layout, the bias slots
 * unused) and `wt` (each W_l transposed, in_l x out_l, at W_l's offset) are what the
 * kernels read; bz_mlp_sync and bz_mlp_adam keep them equal to round(W) in BF16.
 * Rows: x is n x BZ_MLP_IN FP32 (16-byte aligned), y n x BZ_MLP_OUT FP32; the saved
 * pre-activations z are (BZ_MLP_LAYERS-1) x n x BZ_MLP_HIDDEN FP32.
 * ------------------------------------------------------------------------------------- */
#define BZ_MLP_IN 16
#define BZ_MLP_HIDDEN 128
#define BZ_MLP_OUT 80
#define BZ_MLP_LAYERS 5
#define BZ_MLP_NPARAM 62032 /* 16*128+128 + 3*(128*128+128) + 128*80+80 */
int32_t bz_mlp_param_count(void);
/* kernels of bz_mlp_forward / bz_mlp_train_step: 0 = warp-level mma.sync (m16n8k16)
 * throughout; 1 = forward on tcgen05.mma with a TMEM accumulator (one CTA per 128 rows),
 * backward on mma.sync (default: the faster training step); 2 = forward and backward on
 * tcgen05 (deterministic gradients) */
int bz_mlp_select(int32_t path);
int32_t bz_mlp_selected(void);
/* device-side conditions of the network kernels since the last call (BZ_DEV_LOOKBACK: a
 * bounded tensor-core wait gave up); synchronous, clears them */
int bz_mlp_status(uint32_t *out);
/* wb/wt from the FP32 parameters */
int bz_mlp_sync(const float *params, uint16_t *wb, uint16_t *wt, void *stream);
/* y = f(x[idx[r]]) for r < n (idx NULL: row r); z (NULL: not kept) receives the hidden
 * layers' pre-activations for a following bz_mlp_backward */
int bz_mlp_forward(const uint16_t *wb, const float *params, const float *x, const int32_t *idx, int32_t n,
                   float *y, float *z, void *stream);
/* loss = sum_r sum_c wcol[c] (y - t[idx[r]])^2 / (2 n) added to *loss; its gradient with
 * respect to every parameter added to grad (FP32, BZ_MLP_NPARAM). With a workspace of
 * bz_mlp_backward_workspace(n) bytes the products run on tcgen05 and every CTA writes its
 * own partial gradient, summed in a fixed order (deterministic); without one (NULL), on
 * mma.sync with FP32 atomics. */
size_t bz_mlp_backward_workspace(int32_t n);
int bz_mlp_backward(const uint16_t *wb, const uint16_t *wt, const float *params, const float *x,
                    const float *t, const float *wcol, const int32_t *idx, int32_t n, const float *y,
                    const float *z, float *grad, float *loss, void *workspace, size_t workspace_bytes,
                    void *stream);
/* one Adam step (Kingma & Ba 2015) with bias correction for step `step` (1-based) and
 * decoupled weight decay on the weights; clears grad and refreshes wb/wt */
int bz_mlp_adam(float *params, float *grad, float *m, float *v, uint16_t *wb, uint16_t *wt, int64_t step,
                float lr, float beta1, float beta2, float eps, float weight_decay, void *stream);
/* n indices uniform in [0, n_rows) from Philox (seed, step): a training minibatch */
int bz_mlp_batch(int32_t n_rows, int32_t n, uint64_t seed, uint64_t step, int32_t *idx, void *stream);
/* batch + forward (z kept) + backward + Adam: one training step (four launches);
 * ws: bz_mlp_train_workspace(n) bytes */
size_t bz_mlp_train_workspace(int32_t n);
int bz_mlp_train_step(float *params, float *grad, float *m, float *v, uint16_t *wb, uint16_t *wt,
                      const float *x, const float *t, const float *wcol, int32_t n_rows, int32_t n,
                      uint64_t seed, int64_t step, float lr, float beta1, float beta2, float eps,
                      float weight_decay, float *loss, void *workspace, size_t workspace_bytes, void *stream);

/* Sets every live particle's velocity from a tabulated energy distribution of its key (its
 * deposit node; in an ensemble its swarm): cdf is n_keys x nbins FP64, the cumulative
 * weight fractions of nbins log-spaced bins over [emin, emax) eV (last entry 1; a key
 * whose last entry is not positive keeps its particles as they are). Energy: the bin by
 * inverse CDF, log-uniform within it, times energy_scale[key] (optional, n_keys FP64);
 * direction isotropic; Philox (seed, slot). */
int bz_seg_sample_energy_f32(const bz_params *p, bz_segments_f32 s, int32_t n_keys, int32_t nbins, double emin,
                             double emax, const double *cdf, const double *energy_scale, uint64_t seed,
                             void *stream);
int bz_seg_sample_energy_f64(const bz_params *p, bz_segments_f64 s, int32_t n_keys, int32_t nbins, double emin,
                             double emax, const double *cdf, const double *energy_scale, uint64_t seed,
                             void *stream);

/* Philox4x32-10 (Salmon et al. 2011) of n counters ctr[n][4] under keys key[n][2] into
 * out[n][4], all device pointers, through the device code the kernels draw from: variant 0
 * the plain rounds, 1 and 2 the two outputs of the interleaved pair with precomputed round
 * keys (both given the same counter); variant 3 the interleaved pair with the push's round
 * count (7, Philox4x32-7). For known-answer checks of the generator. */
int bz_philox4x32_10(const uint32_t *ctr, const uint32_t *key, int32_t n, int32_t variant, uint32_t *out,
                     void *stream);

/* library identification */
const char *bz_version(void);

#ifdef __cplusplus
}
#endif
#endif
