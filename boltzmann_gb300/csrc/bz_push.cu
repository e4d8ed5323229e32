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
#include <cuda.h>

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <mutex>

#include "bz_push_core.cuh"

namespace bz {


template <typename T, bool REPLAY, int XS, bool DEPOSIT>
#ifndef BZ_PUSH_MINB
#define BZ_PUSH_MINB 3
#endif
__global__ void __launch_bounds__(PT, BZ_PUSH_MINB) k_push(bz_params p, PushConst<T> kc, SoA<T> in, const int32_t *n_in,
                                             int64_t in_cap, SoA<T> out, int64_t cap, int32_t *counts, const T *E,
                                             const double *R, const double *gas, double *moments,
                                             unsigned int *ticket, uint64_t *tile_status, int max_tiles,
                                             uint32_t *status, uint32_t wait_limit) {
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
    const NodeMap &nm = kc.nm;
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
            it[j].excited = false;
            if (w[j] > T(0)) {
                push_item<T, REPLAY, XS>(p, kc, rng, uint32_t(base + j), x[j], vx[j], vy[j], vz[j], E_s, xs_s, R, gas,
                                         it[j]);
                ns += it[j].alive;
                nc += it[j].child;
                if (!(isfinite(it[j].vx) && isfinite(it[j].vy) && isfinite(it[j].vz))) err |= BZ_DEV_NONFINITE;
                if (DEPOSIT) {
                    if (it[j].alive) {
                        int nd = deposit_node(p.advect, it[j].x, nm);
                        if (nd >= 0 && nd < nnodes) {
                            atomicAdd(&mom_s[nd], A(w[j]));
                            if (it[j].ionized) atomicAdd(&mom_s[nnodes + nd], A(w[j]));
                            atomicAdd(&mom_s[2 * nnodes + nd], A(w[j] * it[j].e));
                            if (it[j].excited && (p.flags & BZ_MOMENT_EXCITATION))
                                atomicAdd(&moments[2 * nnodes + nd], double(w[j]));  // rare: straight to the grid
                        }
                    } else if (it[j].ionized && (p.flags & BZ_QUIRK_DEAD_IONFLAG)) {
                        atomicAdd(&mom_s[nnodes + 0], A(1));
                    }
                    if (it[j].child) {
                        int nd = deposit_node(p.advect, it[j].cx, nm);
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
            lookback(tile_status, tile, tot & 0xffffu, tot >> 16, &s_ps, &s_pc, status, wait_limit);
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
                                 int(std::min<int64_t>(max_tiles, INT32_MAX)), status, host_wait_limit());
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
    if (p.advect < BZ_ADVECT_NONE || p.advect > BZ_ADVECT_ENSEMBLE) return BZ_ERR_ARG;
    if (p.advect == BZ_ADVECT_1D && (p.n_faces < 1 || p.dx <= 0 || p.L <= 0)) return BZ_ERR_ARG;
    if (p.advect == BZ_ADVECT_ENSEMBLE && p.n_faces < 1) return BZ_ERR_ARG;
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
    if (dep && (p.flags & BZ_CLEAR_MOMENTS) &&
        cudaMemsetAsync(moments, 0, sizeof(double) * 4 * size_t(p.n_nodes), st) != cudaSuccess)
        return BZ_ERR_CUDA;
    // with a workspace of bz_push_workspace_fast_* bytes: the segmented kernel and a gather
    // into the reference order (no tile waits for its predecessors)
    {
        const int rc = dense_push_segmented<T>(p, in, n_in, in_cap, out, cap, counts, E, R, gas, moments, ws, ws_bytes,
                                               status, st);
        if (rc != BZ_ERR_WORKSPACE) return rc;
    }
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

// Philox4x32-10 of n (counter, key) pairs through the device code the kernels use:
// variant 0 the plain rounds, 1 and 2 the two halves of the interleaved pair with round
// keys (philox_rk_x2, whose second counter differs in word 3: here the same counter), 3 the
// interleaved pair with the push's round count.
__global__ void k_philox(const uint32_t *ctr, const uint32_t *key, int n, int variant, uint32_t *out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t *c = ctr + 4 * size_t(i), *k = key + 2 * size_t(i);
    u32x4 r;
    if (variant == 0) {
        r = philox(c[0], c[1], c[2], c[3], k[0], k[1]);
    } else {
        uint32_t rk0[10], rk1[10];
        for (int j = 0; j < 10; ++j) {
            rk0[j] = k[0] + uint32_t(j) * 0x9E3779B9u;
            rk1[j] = k[1] + uint32_t(j) * 0xBB67AE85u;
        }
        u32x4 a, b;
        if (variant == 3) philox_rk_x2<PUSH_ROUNDS>(c[0], c[1], c[2], c[3], c[3], rk0, rk1, a, b);
        else philox_rk_x2(c[0], c[1], c[2], c[3], c[3], rk0, rk1, a, b);
        r = variant == 2 ? b : a;
    }
    uint32_t *o = out + 4 * size_t(i);
    o[0] = r.x; o[1] = r.y; o[2] = r.z; o[3] = r.w;
}

static std::atomic<uint32_t> g_wait_limit{0};
uint32_t host_wait_limit(uint32_t dflt) {
    const uint32_t v = g_wait_limit.load(std::memory_order_relaxed);
    return v ? v : dflt;
}

// The look-back wait on its own: CTAs take tiles first_tile, first_tile+1, ... from a
// ticket and each publishes one survivor; prefix[tile] receives the exclusive prefix the
// look-back gives. With first_tile = 1 no CTA owns tile 0, so every wait that reaches
// tile 0 runs out after wait_limit polls, counts it as empty and raises BZ_DEV_LOOKBACK.
__global__ void k_lookback_selftest(unsigned int *ticket, uint64_t *tile_status, int first_tile, int ntiles,
                                    uint32_t *prefix, uint32_t *status, uint32_t wait_limit) {
    if (threadIdx.x >= 32) return;
    int tile = 0;
    if (threadIdx.x == 0) tile = int(atomicAdd(ticket, 1u)) + first_tile;
    tile = __shfl_sync(0xffffffffu, tile, 0);
    if (tile >= ntiles) return;
    uint32_t ps = 0, pc = 0;
    lookback(tile_status, tile, 1u, 0u, &ps, &pc, status, wait_limit);
    if (threadIdx.x == 0) prefix[tile] = ps;
}

}  // namespace bz

extern "C" {

int bz_set_wait_limit(uint32_t spins) {
    bz::g_wait_limit.store(spins, std::memory_order_relaxed);
    return BZ_OK;
}
uint32_t bz_wait_limit(void) { return bz::g_wait_limit.load(std::memory_order_relaxed); }

size_t bz_lookback_selftest_workspace(int32_t ntiles) {
    return bz::PushWsLayout::ticket_bytes + 8 * size_t(ntiles > 0 ? ntiles : 1);
}

int bz_lookback_selftest(int32_t ntiles, int32_t first_tile, uint32_t *prefix, void *workspace, size_t workspace_bytes,
                         uint32_t *status, void *stream) {
    if (ntiles < 1 || ntiles > (1 << 20) || first_tile < 0 || first_tile > 1 || !prefix || !workspace || !status)
        return BZ_ERR_ARG;
    if (workspace_bytes < bz_lookback_selftest_workspace(ntiles)) return BZ_ERR_WORKSPACE;
    cudaStream_t st = bz::as_stream(stream);
    if (cudaMemsetAsync(workspace, 0, bz_lookback_selftest_workspace(ntiles), st) != cudaSuccess) return BZ_ERR_CUDA;
    if (cudaMemsetAsync(prefix, 0xff, sizeof(uint32_t) * size_t(ntiles), st) != cudaSuccess) return BZ_ERR_CUDA;
    unsigned char *w = static_cast<unsigned char *>(workspace);
    const int ctas = ntiles - first_tile;
    if (ctas > 0)
        bz::k_lookback_selftest<<<ctas, 32, 0, st>>>(reinterpret_cast<unsigned int *>(w),
                                                     reinterpret_cast<uint64_t *>(w + bz::PushWsLayout::ticket_bytes),
                                                     first_tile, ntiles, prefix, status, bz::host_wait_limit());
    return cudaGetLastError() == cudaSuccess ? BZ_OK : BZ_ERR_CUDA;
}

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

int bz_philox4x32_10(const uint32_t *ctr, const uint32_t *key, int32_t n, int32_t variant, uint32_t *out,
                     void *stream) {
    if (n < 0 || variant < 0 || variant > 3 || (n > 0 && (!ctr || !key || !out))) return BZ_ERR_ARG;
    if (n == 0) return BZ_OK;
    bz::k_philox<<<int(bz::ceil_div(n, 256)), 256, 0, bz::as_stream(stream)>>>(ctr, key, n, variant, out);
    return cudaGetLastError() == cudaSuccess ? BZ_OK : BZ_ERR_CUDA;
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

// Device address of the scratch array in the current CUDA context. The array's name in
// host code only stands in for the symbol, so the address is asked of the runtime once per
// context (with that context current) and remembered under the context's unique id: a
// host that creates its own contexts, switches between them or resets the device gets
// the address that belongs to the context it launches in (an id is never reused).
using PfnCtxGetCurrent = CUresult (*)(CUcontext *);
using PfnCtxGetId = CUresult (*)(CUcontext, unsigned long long *);
constexpr int kCtxCache = 64;
static std::mutex g_noalloc_mu;
static unsigned long long g_noalloc_ctx[kCtxCache] = {};
static void *g_noalloc_ptr[kCtxCache] = {};
static int g_noalloc_next = 0;

static int current_context_id(unsigned long long *id) {
    static PfnCtxGetCurrent get_cur = nullptr;
    static PfnCtxGetId get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_cur = reinterpret_cast<PfnCtxGetCurrent>(f);
        f = nullptr;
        q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<PfnCtxGetId>(f);
    });
    if (!get_cur || !get_id) return BZ_ERR_CUDA;
    CUcontext ctx = nullptr;
    if (get_cur(&ctx) != CUDA_SUCCESS) return BZ_ERR_CUDA;
    if (!ctx) {  // nothing current yet: make the current device's primary context current
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess || cudaSetDevice(dev) != cudaSuccess) return BZ_ERR_CUDA;
        if (get_cur(&ctx) != CUDA_SUCCESS || !ctx) return BZ_ERR_CUDA;
    }
    return get_id(ctx, id) == CUDA_SUCCESS ? BZ_OK : BZ_ERR_CUDA;
}

static int noalloc_scratch(void **out) {
    unsigned long long id = 0;
    int rc = current_context_id(&id);
    if (rc != BZ_OK) return rc;
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    for (int i = 0; i < kCtxCache; ++i)
        if (g_noalloc_ptr[i] && g_noalloc_ctx[i] == id) {
            *out = g_noalloc_ptr[i];
            return BZ_OK;
        }
    void *ptr = nullptr;
    if (cudaGetSymbolAddress(&ptr, g_push_noalloc_scratch) != cudaSuccess || !ptr) return BZ_ERR_CUDA;
    g_noalloc_ctx[g_noalloc_next] = id;  // the oldest entry makes room
    g_noalloc_ptr[g_noalloc_next] = ptr;
    g_noalloc_next = (g_noalloc_next + 1) % kCtxCache;
    *out = ptr;
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
    // only the prefix this input needs is used, and cleared by the launch (cudaMemsetAsync
    // on the caller's stream)
    const size_t used = bz::PushWsLayout::bytes(in_capacity);
    return bz::push_entry<float>(p, in, n_in, in_capacity, out, out_capacity, counts, E, replay_R, replay_gas,
                                 moments, scratch, used, status, stream);
}

int bz_push_noalloc_scratch_address(void **address) {
    if (!address) return BZ_ERR_ARG;
    return bz::noalloc_scratch(address);
}

}  // extern "C"
