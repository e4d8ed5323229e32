// Device-resident grid step: host-side grid update of the step loop, ion drift-
// diffusion and Poisson solve, all float64, so that a CCP step needs no host round trip.
// This file is compiled without FMA contraction so the float64 operation order of the
// reference's numba code (EF_kernel_1D.py, heavies_kernel_1D.py) is kept.
#include <cooperative_groups.h>

#include "bz_common.cuh"

namespace bz {

// boltzmann.py:643-647, nodes i = first, first + stride, ...
__device__ __forceinline__ void grid_update_body(int nn, const double *mom, double *ni, double *Te, double *g2,
                                                 int first, int stride) {
    for (int i = first; i < nn; i += stride) {
        double ne = mom[i], src = mom[nn + i], nrg = mom[3 * nn + i];
        if (ni) ni[i] = ni[i] + src;
        if (Te) {
            double t = (2. / 3.) * nrg / ne;
            Te[i] = isfinite(t) ? t : (isnan(t) ? 0.0 : (t > 0 ? 1.7976931348623157e308 : -1.7976931348623157e308));
        }
        if (g2) g2[i] = g2[i] + src;
    }
}

__global__ void k_grid_update(int nn, const double *mom, double *ni, double *Te, double *g2) {
    grid_update_body(nn, mom, ni, Te, g2, threadIdx.x + blockIdx.x * blockDim.x, blockDim.x * gridDim.x);
}

// heavies_kernel_1D.py:4-64, ion part, by one whole CTA; the boundary nodes depend on the
// interior update, so the phases are separated by barriers.
__device__ void ion_fluid_body(int N, double dx, double dt, double mu_i, double D_i, const double *E, double *ni,
                               double *Ji, int32_t *brk, int *s_brk_p) {
    int &s_brk = *s_brk_p;
    if (threadIdx.x == 0) {
        s_brk = 0;
        double e0 = fmax(E[0], 0.0), eN = fmin(E[N - 1], 0.0);
        ni[0] = ni[1] * ((D_i / dx - 0.5 * mu_i * e0) / (D_i / dx + 0.5 * mu_i * e0));
        ni[N] = ni[N - 1] * ((D_i / dx + 0.5 * mu_i * eN) / (D_i / dx - 0.5 * mu_i * eN));
    }
    __syncthreads();
    for (int i = threadIdx.x; i < N; i += blockDim.x)
        Ji[i] = (mu_i * (0.5 * (ni[i] + ni[i + 1])) * E[i] - D_i * (ni[i + 1] - ni[i]) / dx);
    __syncthreads();
    int b = 0;
    for (int i = 1 + threadIdx.x; i < N; i += blockDim.x) {
        double r = ni[i] - dt * (Ji[i] - Ji[i - 1]) / dx;
        if (r < 0 && ni[i] > 0) b = 1;
        ni[i] = r;  // each node reads only fluxes, which are final
    }
    if (b) atomicOr(&s_brk, 1);
    __syncthreads();
    if (threadIdx.x == 0) {
        double e0 = fmax(E[0], 0.0), eN = fmin(E[N - 1], 0.0);
        ni[0] = ni[1] * ((D_i / dx - 0.5 * mu_i * e0) / (D_i / dx + 0.5 * mu_i * e0));
        ni[N] = ni[N - 1] * ((D_i / dx + 0.5 * mu_i * eN) / (D_i / dx - 0.5 * mu_i * eN));
        if (brk) *brk = s_brk;
    }
}

__global__ void __launch_bounds__(1024) k_ion_fluid(int N, double dx, double dt, double mu_i, double D_i,
                                                    const double *E, double *ni, double *Ji, int32_t *brk) {
    __shared__ int s_brk;
    ion_fluid_body(N, dx, dt, mu_i, D_i, E, ni, Ji, brk, &s_brk);
}

// banded Cholesky factor of tridiag(-1, 2, -1)/dx^2 (what boltzmann.py:744-755 gets from
// scipy.linalg.cholesky_banded): d[0] = sqrt(a), l[i] = b/d[i-1], d[i] = sqrt(a - l[i]^2).
// The two substitutions of the solve are first-order recurrences z_i = a_i z_{i-1} + b_i
// with constant a_i, so they are precomputed here as prefix products: forward
// y_i = (r_i - l_i y_{i-1})/d_i = P_i sum_{k<=i} r_k g_k with P_i = prod_{k=1..i}(-l_k/d_k),
// g_k = 1/(d_k P_k); backward V_i = (y_i - l_{i+1} V_{i+1})/d_i = Q_i sum_{k>=i} y_k h_k with
// Q_i = prod_{k=i..n-2}(-l_{k+1}/d_k), h_k = 1/(d_k Q_k). For this matrix P_i =
// sqrt(2/((i+1)(i+2))) and Q_i = (i+1)/n: no overflow, no cancellation in the products.
// plan = [P | g | Q | h], n = N-1 each. One thread: called once per grid.
__global__ void k_poisson_factor(int N, double dx, double *d, double *l, double *plan) {
    if (threadIdx.x || blockIdx.x) return;
    int n = N - 1;
    double a = 2. / (dx * dx), b = -1. / (dx * dx);
    d[0] = sqrt(a);
    l[0] = 0.0;
    for (int i = 1; i < n; ++i) {
        l[i] = b / d[i - 1];
        d[i] = sqrt(a - l[i] * l[i]);
    }
    double *P = plan, *g = plan + n, *Q = plan + 2 * n, *h = plan + 3 * n;
    double pr = 1.0;
    for (int i = 0; i < n; ++i) {
        if (i > 0) pr = pr * (-l[i] / d[i]);
        P[i] = pr;
        g[i] = 1.0 / (d[i] * pr);
    }
    pr = 1.0;
    for (int i = n - 1; i >= 0; --i) {
        if (i < n - 1) pr = pr * (-l[i + 1] / d[i]);
        Q[i] = pr;
        h[i] = 1.0 / (d[i] * pr);
    }
}

constexpr int PS_T = 1024;

// inclusive block-wide sum of v over PS_T threads in index order
__device__ double block_inclusive_sum(double v, double *sh) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        double t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    if (lane == 31) sh[warp] = v;
    __syncthreads();
    if (warp == 0) {
        double w = sh[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            double t = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += t;
        }
        sh[lane] = w;
    }
    __syncthreads();
    if (warp > 0) v += sh[warp - 1];
    __syncthreads();
    return v;
}

// EF_kernel_1D.py:26-42: forward and backward substitution with the factor (as the two
// prefix sums of the plan), then face fields. One CTA, float64; rows in chunks of PS_T
// with the running sum carried between chunks. y (the forward result) lives in E until
// the faces overwrite it.
struct PoissonShared { double sh[32]; double carry, vs; };

__device__ void poisson_body(int N, double dx, double eps0, double V0, double freq, double t_host,
                             const double *t_dev, const double *ne, const double *ni, const double *plan, double *V,
                             double *E, float *E32, double *y, PoissonShared &S) {
    double *sh = S.sh;
    double &carry = S.carry, &vs_s = S.vs;
    const int n = N - 1;
    const double *P = plan, *g = plan + n, *Q = plan + 2 * n, *h = plan + 3 * n;
    // electrode voltage, evaluated once (float64 sin is costly on this part's narrow FP64 pipe)
    if (threadIdx.x == 0) {
        const double t = t_dev ? *t_dev : t_host;
        vs_s = V0 * sin(2 * 3.141592653589793 * freq * t);
        carry = 0.0;
    }
    __syncthreads();
    const double vs = vs_s;
    // forward: r_i = (ni - ne)/eps0 (+ boundary term at i = 0); y_i = P_i sum_{k<=i} r_k g_k
    for (int c0 = 0; c0 < n; c0 += PS_T) {
        const int i = c0 + threadIdx.x;
        double c = 0.0;
        if (i < n) {
            double r = (1.0 / eps0) * (ni[i + 1] - ne[i + 1]);
            if (i == 0) r = r + (1.0 / (dx * dx)) * vs;
            c = r * g[i];
        }
        const double s = block_inclusive_sum(c, sh) + carry;
        if (i < n) y[i] = P[i] * s;
        __syncthreads();
        if (i == min(c0 + PS_T, n) - 1) carry = s;
        __syncthreads();
    }
    // backward: V_i = Q_i sum_{k>=i} y_k h_k (rows taken from the end)
    if (threadIdx.x == 0) carry = 0.0;
    __syncthreads();
    for (int c0 = 0; c0 < n; c0 += PS_T) {
        const int j = c0 + threadIdx.x;  // j-th row from the end
        const int i = n - 1 - j;
        const double c = (j < n) ? y[i] * h[i] : 0.0;
        const double s = block_inclusive_sum(c, sh) + carry;
        if (j < n) V[i] = Q[i] * s;
        __syncthreads();
        if (j == min(c0 + PS_T, n) - 1) carry = s;
        __syncthreads();
    }
    // faces (EF_kernel_1D.py:39-42)
    for (int i = threadIdx.x; i < N; i += PS_T) {
        double e;
        if (i == 0) e = -(V[0] - vs) / dx;
        else if (i == N - 1) e = -(0 - V[N - 2]) / dx;
        else e = -(V[i] - V[i - 1]) / dx;
        E[i] = e;
        if (E32) E32[i] = float(e);
    }
}

__global__ void __launch_bounds__(PS_T) k_poisson(int N, double dx, double eps0, double V0, double freq,
                                                  double t_host, const double *t_dev, const double *ne,
                                                  const double *ni, const double *plan, double *V, double *E,
                                                  float *E32, double *y) {
    __shared__ PoissonShared S;
    poisson_body(N, dx, eps0, V0, freq, t_host, t_dev, ne, ni, plan, V, E, E32, y, S);
}

// The whole grid part of a step in one CTA (the order of the step loop,
// boltzmann.py:643-678): grid update, clock, ion fluid with the field of the last solve,
// Poisson with the new time and densities. One launch instead of four.
__global__ void __launch_bounds__(PS_T) k_field_step(int N, double dx, double dt, double mu_i, double D_i,
                                                     double eps0, double V0, double freq, const double *mom,
                                                     double *ni, double *Te, double *g2, double *t_dev,
                                                     uint64_t *step_dev, const double *plan, double *V,
                                                     double *E, float *E32, double *Ji, int32_t *brk) {
    __shared__ PoissonShared S;
    __shared__ int s_brk;
    const int nn = N + 1;
    grid_update_body(nn, mom, ni, Te, g2, threadIdx.x, blockDim.x);
    if (threadIdx.x == 0) {
        if (t_dev) *t_dev = *t_dev + dt;
        if (step_dev) *step_dev = *step_dev + 1;
    }
    __syncthreads();
    ion_fluid_body(N, dx, dt, mu_i, D_i, E, ni, Ji, brk, &s_brk);
    __syncthreads();
    // E is the forward substitution's scratch: the fluid above has read the old field
    poisson_body(N, dx, eps0, V0, freq, 0.0, t_dev, mom, ni, plan, V, E, E32, E, S);
}

// The same grid step spread over G CTAs, phases separated by barriers over all G CTAs:
// float64 throughput is per SM on this part, and one CTA spent most of its time waiting on
// its SM's narrow float64 pipe. CTA b owns Poisson rows [b*FM_T, (b+1)*FM_T); each
// substitution is a CTA-local scan plus the sum of the other CTAs' totals (in CTA order),
// so the result equals the one-CTA kernel's up to the association of the float64 sums.
// CLUSTER: the G CTAs form one thread-block cluster (G <= 16, i.e. up to 1025 nodes) and
// the barriers are the cluster's hardware barrier, whose release/acquire at cluster scope
// orders the global-memory phases; otherwise a cooperative launch and grid-wide barriers.
constexpr int FM_T = 64;

__device__ double cta64_inclusive_sum(double v, double *sh) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        double t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    if (lane == 31) sh[warp] = v;
    __syncthreads();
    if (warp == 1) v += sh[0];
    __syncthreads();
    return v;
}

// The ion flux through face i (heavies_kernel_1D.py:36-37) with the boundary densities of
// faces 0 and N-1 formed where they are needed (heavies_kernel_1D.py:22-33).
__device__ __forceinline__ double face_flux(int i, int N, double dx, double mu_i, double D_i, double e0, double eN,
                                            const double *ni, const double *E) {
    const double a = (i == 0) ? ni[1] * ((D_i / dx - 0.5 * mu_i * e0) / (D_i / dx + 0.5 * mu_i * e0)) : ni[i];
    const double c = (i + 1 == N) ? ni[N - 1] * ((D_i / dx + 0.5 * mu_i * eN) / (D_i / dx - 0.5 * mu_i * eN))
                                  : ni[i + 1];
    return (mu_i * (0.5 * (a + c)) * E[i] - D_i * (c - a) / dx);
}

template <bool CLUSTER>
__device__ __forceinline__ void phase_sync() {
    if constexpr (CLUSTER) cooperative_groups::this_cluster().sync();
    else cooperative_groups::this_grid().sync();
}

template <bool CLUSTER>
__global__ void __launch_bounds__(FM_T) k_field_step_mc(int N, double dx, double dt, double mu_i, double D_i,
                                                        double eps0, double V0, double freq, const double *mom,
                                                        double *ni, double *Te, double *g2, double *t_dev,
                                                        uint64_t *step_dev, const double *plan, double *V, double *E,
                                                        float *E32, double *Ji, int32_t *brk, double *tot,
                                                        int32_t *flag) {
    __shared__ double sh[2];
    __shared__ double s_vs;
    __shared__ double s_c[FM_T];
    const int G = gridDim.x, b = blockIdx.x, t = threadIdx.x;
    const int gt = b * FM_T + t, GT = G * FM_T;
    const int nn = N + 1, n = N - 1;
    const double tnew = *t_dev + dt;  // every thread reads the clock before it is advanced
    // grid update (boltzmann.py:643-647)
    grid_update_body(nn, mom, ni, Te, g2, gt, GT);
    if (gt == 0) *flag = 0;
    if (t == 0) s_vs = V0 * sin(2 * 3.141592653589793 * freq * tnew);
    phase_sync<CLUSTER>();
    if (gt == 0) {
        *t_dev = tnew;
        if (step_dev) *step_dev = *step_dev + 1;
    }
    // ion fluid (heavies_kernel_1D.py:4-64). G*FM_T >= N-1, so thread gt owns at most one
    // interior node j = gt+1: it forms both fluxes of that node itself (the left one is also
    // its left neighbour's right flux, the same arithmetic on the same operands), writes
    // face j (and face 0 for j = 1) and keeps the new density in a register — the Poisson
    // row j-1 below is this thread's too. The densities reach memory only after the next
    // barrier, when no thread reads the old ones any more; the boundary densities are
    // formed by the threads that own nodes 1 and N-1.
    const double e0 = fmax(E[0], 0.0), eN = fmin(E[N - 1], 0.0);
    const int j = 1 + gt;
    double nj = 0.0;
    if (j < N) {
        const double JL = face_flux(j - 1, N, dx, mu_i, D_i, e0, eN, ni, E);
        const double JR = face_flux(j, N, dx, mu_i, D_i, e0, eN, ni, E);
        if (j == 1) Ji[0] = JL;
        Ji[j] = JR;
        const double old = ni[j];
        nj = old - dt * (JR - JL) / dx;
        if (nj < 0 && old > 0) atomicOr(flag, 1);
    }
    const double vs = s_vs;
    const double *P = plan, *g = plan + n, *Q = plan + 2 * n, *h = plan + 3 * n;
    const double *ne = mom;
    // forward substitution: y_i = P_i sum_{k<=i} r_k g_k (EF_kernel_1D.py:26-42)
    const int i = b * FM_T + t;  // = gt: row i uses node i+1 = j
    double c = 0.0;
    if (i < n) {
        double r = (1.0 / eps0) * (nj - ne[i + 1]);
        if (i == 0) r = r + (1.0 / (dx * dx)) * vs;
        c = r * g[i];
    }
    const double sf = cta64_inclusive_sum(c, sh);
    if (t == FM_T - 1) tot[b] = sf;
    phase_sync<CLUSTER>();
    if (j < N) {
        ni[j] = nj;
        if (j == 1) ni[0] = nj * ((D_i / dx - 0.5 * mu_i * e0) / (D_i / dx + 0.5 * mu_i * e0));
        if (j == N - 1) ni[N] = nj * ((D_i / dx + 0.5 * mu_i * eN) / (D_i / dx - 0.5 * mu_i * eN));
    }
    if (gt == 0 && brk) *brk = *flag;
    double carry = 0.0;
    for (int k = 0; k < b; ++k) carry += tot[k];
    const double y = (i < n) ? P[i] * (sf + carry) : 0.0;
    // backward: V_i = Q_i sum_{k>=i} y_k h_k, the CTA's rows scanned from the end
    s_c[t] = (i < n) ? y * h[i] : 0.0;
    __syncthreads();
    const int tr = FM_T - 1 - t, ir = b * FM_T + tr;  // this thread's row in the backward scan
    const double sb = cta64_inclusive_sum(s_c[tr], sh);
    if (t == FM_T - 1) tot[G + b] = sb;
    phase_sync<CLUSTER>();
    double carry_b = 0.0;
    for (int k = G - 1; k > b; --k) carry_b += tot[G + k];
    if (ir < n) V[ir] = Q[ir] * (sb + carry_b);
    phase_sync<CLUSTER>();
    // faces (EF_kernel_1D.py:39-42)
    for (int f = gt; f < N; f += GT) {
        double e;
        if (f == 0) e = -(V[0] - vs) / dx;
        else if (f == N - 1) e = -(0 - V[N - 2]) / dx;
        else e = -(V[f] - V[f - 1]) / dx;
        E[f] = e;
        if (E32) E32[f] = float(e);
    }
}

// 0: the cluster form where it fits, else the cooperative one; 1: cooperative; 2: cluster
static int g_field_mode = 0;

// Can G CTAs of the cluster form run as one cluster on the current device? (G <= 8 is
// portable; up to 16 needs the non-portable size, granted per kernel.) Cached per
// (device, G).
static bool field_cluster_ok(int G) {
    static int cached_dev = -1, cached_G = -1;
    static bool cached = false;
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev == cached_dev && G == cached_G) return cached;
    cached_dev = dev;
    cached_G = G;
    cached = false;
    if (G < 1 || G > 16) return false;
    if (G > 8 && cudaFuncSetAttribute(k_field_step_mc<true>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) !=
                     cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = unsigned(G);
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(G);
    cfg.blockDim = dim3(FM_T);
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int nclusters = 0;
    if (cudaOccupancyMaxActiveClusters(&nclusters, k_field_step_mc<true>, &cfg) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    cached = nclusters > 0;
    return cached;
}

// rate closure of the ion source: ni_src = nu_i ne per node (moments row 1 from row 0)
__global__ void k_ion_source_closure(int nn, const double *rate, double *mom) {
    for (int i = threadIdx.x + blockIdx.x * blockDim.x; i < nn; i += blockDim.x * gridDim.x)
        mom[nn + i] = rate[i] * mom[i];
}

__global__ void k_advance_clock(double *t, uint64_t *step, double dt) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        if (t) *t = *t + dt;
        if (step) *step = *step + 1;
    }
}

}  // namespace bz

extern "C" {
int bz_grid_update(int32_t n_nodes, const double *moments, double *ni, double *Te, double *g2, void *stream) {
    if (n_nodes < 1 || !moments) return BZ_ERR_ARG;
    bz::k_grid_update<<<(n_nodes + 255) / 256, 256, 0, bz::as_stream(stream)>>>(n_nodes, moments, ni, Te, g2);
    return cudaGetLastError() == cudaSuccess ? BZ_OK : BZ_ERR_CUDA;
}
int bz_ion_source_closure(int32_t n_nodes, const double *rate, double *moments, void *stream) {
    if (n_nodes < 1 || !rate || !moments) return BZ_ERR_ARG;
    bz::k_ion_source_closure<<<(n_nodes + 255) / 256, 256, 0, bz::as_stream(stream)>>>(n_nodes, rate, moments);
    return cudaGetLastError() == cudaSuccess ? BZ_OK : BZ_ERR_CUDA;
}
int bz_ion_fluid(int32_t N, double dx, double dt, double mu_i, double D_i, const double *E, double *ni, double *Ji,
                 int32_t *brk, void *stream) {
    if (N < 2 || !E || !ni || !Ji) return BZ_ERR_ARG;
    bz::k_ion_fluid<<<1, 1024, 0, bz::as_stream(stream)>>>(N, dx, dt, mu_i, D_i, E, ni, Ji, brk);
    return cudaGetLastError() == cudaSuccess ? BZ_OK : BZ_ERR_CUDA;
}
int bz_poisson_factor(int32_t N, double dx, double *chol_diag, double *chol_lower, double *plan) {
    if (N < 3 || !chol_diag || !chol_lower || !plan) return BZ_ERR_ARG;
    bz::k_poisson_factor<<<1, 32>>>(N, dx, chol_diag, chol_lower, plan);
    if (cudaGetLastError() != cudaSuccess) return BZ_ERR_CUDA;
    return cudaDeviceSynchronize() == cudaSuccess ? BZ_OK : BZ_ERR_CUDA;
}
int bz_poisson(int32_t N, double dx, double eps0, double V0, double freq, double t_host, const double *t_dev,
               const double *ne, const double *ni, const double *plan, double *V, double *E, float *E32,
               void *stream) {
    if (N < 3 || !ne || !ni || !plan || !V || !E) return BZ_ERR_ARG;
    // E doubles as the scratch of the forward substitution: it is written only after
    // the backward substitution has consumed y (both inside the same CTA).
    bz::k_poisson<<<1, bz::PS_T, 0, bz::as_stream(stream)>>>(N, dx, eps0, V0, freq, t_host, t_dev, ne, ni, plan, V,
                                                              E, E32, E);
    return cudaGetLastError() == cudaSuccess ? BZ_OK : BZ_ERR_CUDA;
}
int bz_field_step(int32_t N, double dx, double dt, double mu_i, double D_i, double eps0, double V0, double freq,
                  const double *moments, double *ni, double *Te, double *g2, double *t_dev, uint64_t *step_dev,
                  const double *plan, double *V, double *E, float *E32, double *Ji, int32_t *brk, void *stream) {
    if (N < 3 || !moments || !ni || !t_dev || !plan || !V || !E || !Ji) return BZ_ERR_ARG;
    bz::k_field_step<<<1, bz::PS_T, 0, bz::as_stream(stream)>>>(N, dx, dt, mu_i, D_i, eps0, V0, freq, moments, ni,
                                                                 Te, g2, t_dev, step_dev, plan, V, E, E32, Ji, brk);
    return cudaGetLastError() == cudaSuccess ? BZ_OK : BZ_ERR_CUDA;
}
size_t bz_field_step_coop_workspace(int32_t N) {
    if (N < 3) return 0;
    const int G = int(bz::ceil_div(N - 1, bz::FM_T));
    return size_t(2 * G + 2) * sizeof(double);
}
int bz_field_step_coop(int32_t N, double dx, double dt, double mu_i, double D_i, double eps0, double V0, double freq,
                       const double *moments, double *ni, double *Te, double *g2, double *t_dev, uint64_t *step_dev,
                       const double *plan, double *V, double *E, float *E32, double *Ji, int32_t *brk,
                       void *workspace, size_t workspace_bytes, void *stream) {
    if (N < 3 || !moments || !ni || !t_dev || !plan || !V || !E || !Ji || !workspace) return BZ_ERR_ARG;
    if (workspace_bytes < bz_field_step_coop_workspace(N)) return BZ_ERR_WORKSPACE;
    int G = int(bz::ceil_div(N - 1, bz::FM_T));
    double *tot = static_cast<double *>(workspace);
    int32_t *flag = reinterpret_cast<int32_t *>(tot + 2 * G);
    void *args[] = {&N, &dx, &dt, &mu_i, &D_i, &eps0, &V0, &freq, (void *)&moments, &ni, &Te, &g2, &t_dev,
                    &step_dev, (void *)&plan, &V, &E, &E32, &Ji, &brk, &tot, &flag};
    if (bz::g_field_mode != 1 && bz::field_cluster_ok(G)) {
        cudaLaunchConfig_t cfg = {};
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = unsigned(G);
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.gridDim = dim3(G);
        cfg.blockDim = dim3(bz::FM_T);
        cfg.dynamicSmemBytes = 0;
        cfg.stream = bz::as_stream(stream);
        cfg.attrs = at;
        cfg.numAttrs = 1;
        cudaError_t e = cudaLaunchKernelExC(&cfg, (const void *)bz::k_field_step_mc<true>, args);
        return e == cudaSuccess ? BZ_OK : BZ_ERR_CUDA;
    }
    if (bz::g_field_mode == 2) return BZ_ERR_UNSUPPORTED;  // the cluster form was asked for and is not possible
    int dev = 0, per_sm = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, bz::k_field_step_mc<false>, bz::FM_T, 0) !=
            cudaSuccess ||
        G > per_sm * sms)
        return BZ_ERR_TOO_LARGE;  // every CTA must be resident for the grid-wide barriers
    cudaError_t e = cudaLaunchCooperativeKernel((const void *)bz::k_field_step_mc<false>, dim3(G), dim3(bz::FM_T),
                                                args, 0, bz::as_stream(stream));
    return e == cudaSuccess ? BZ_OK : BZ_ERR_CUDA;
}
int bz_field_step_select(int32_t mode) {
    if (mode < 0 || mode > 2) return BZ_ERR_ARG;
    bz::g_field_mode = mode;
    return BZ_OK;
}
int bz_field_step_selected(void) { return bz::g_field_mode; }
int bz_advance_clock(double *t_dev, uint64_t *step_dev, double dt, void *stream) {
    if (!t_dev && !step_dev) return BZ_ERR_ARG;
    bz::k_advance_clock<<<1, 32, 0, bz::as_stream(stream)>>>(t_dev, step_dev, dt);
    return cudaGetLastError() == cudaSuccess ? BZ_OK : BZ_ERR_CUDA;
}
}
