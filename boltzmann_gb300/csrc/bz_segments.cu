// Segmented particle layout for the solver's hot loop.
//
// The dense push (bz_push.cu) keeps the reference's global order (survivors, then
// children) with a decoupled look-back across tiles; measured on GB300, waiting for
// predecessor tiles halves its throughput. Here the particles live in nseg segments of
// 2*half slots. Segment s holds two runs: run 0 at slots [s*2h, s*2h + n0) and run 1 at
// [s*2h + h, s*2h + h + n1). One warp pushes one whole segment: survivors of run 0 and
// run 1 (in that order) go to run 0 of the same output segment, children (parent order)
// to run 1. No two warps share anything but the shared-memory deposit grid, so the loop
// has no barrier and no inter-warp wait. Within one segment the order is exactly the
// reference's (reshuffle_data_atomics keeps survivors in order, then appends children).
// A segment whose input holds at most half particles cannot overflow: every particle
// leaves at most one survivor and one child. After a push, a segment above half raises
// BZ_SEG_NEEDS_REPACK; k_seg_repack* then spreads all particles evenly again.
#include <algorithm>
#include <type_traits>

#include <cooperative_groups.h>

#include "bz_push_core.cuh"

namespace bz {

// CTA shapes of the push: threads per CTA, consecutive particles per lane per round and
// the minimum resident CTAs per SM the registers are budgeted for. Entry 0 is the
// default; bz_seg_push_select() picks another for the float32 table + deposit push (the
// solver's hot loop), which is what the autotuner times.
// prefetch: the next round's particle is loaded into registers while this round computes
// (one particle per lane only; costs five registers, so it pairs with 64-register shapes).
struct SegShape { int threads, per_lane, min_blocks; bool prefetch; };
// The last two take four consecutive particles per lane with 128-bit loads of each column.
constexpr SegShape kSegShapes[] = {{512, 1, 2, true},  {320, 1, 4, true},  {640, 1, 2, true},
                                   {384, 1, 3, true},  {448, 1, 2, true},  {320, 1, 4, false},
                                   {256, 2, 4, false}, {256, 1, 4, true},  {256, 4, 2, false},
                                   {128, 4, 4, false}};
constexpr int kSegNumShapes = int(sizeof(kSegShapes) / sizeof(kSegShapes[0]));
static int g_seg_shape = 0;

// The CTA's moment grid in shared memory: (sum w, sum w e) interleaved per node, then sum w
// of the ionizing particles; a node's two sums are added one after the other. (One 64-bit
// compare-and-swap for both float32 sums took fewer instructions but was slower where many
// lanes of a warp hit one node, as right after a resampling step appends cell-ordered
// copies: 628 -> 820 us for that push.)
template <typename A> __device__ __forceinline__ void dep_pair(A *g, int nd, A a, A b) {
    atomicAdd(&g[2 * nd], a);
    atomicAdd(&g[2 * nd + 1], b);
}
// The float32 alternative when the caller's workspace holds a grid per CTA in global memory:
// a node's two sums as one vector reduction, performed in L2 without a return value, so the
// lane does not wait for it (a float add to shared memory is a compare-and-swap loop on this
// part, with retries where lanes of a warp meet on a node).
// (written as a global-space reduction: a vector atomic on a generic pointer is not)
__device__ __forceinline__ void dep_red(float2 *g, int nd, float a, float b) {
    asm volatile("red.relaxed.gpu.global.add.v2.f32 [%0], {%1, %2};" ::"l"(__cvta_generic_to_global(g + nd)), "f"(a),
                 "f"(b)
                 : "memory");
}

constexpr size_t SEG_PUSH_TICKET_BYTES = 256;  // the push's segment ticket (cleared per launch)

template <typename T> struct Seg {
    SoA<T> a;
    int32_t *cnt;  // [2*nseg]
    int nseg, half;
};

__device__ __forceinline__ int64_t seg_slot(int seg, int run, int half, int j) {
    return int64_t(seg) * (2 * int64_t(half)) + int64_t(run) * half + j;
}
// the same slot as a 32-bit index: the push's launcher checks that every slot fits (an
// unsigned 32-bit index lets each array access be one wide multiply-add on its base)
__device__ __forceinline__ uint32_t seg_slot32(int seg, int run, int half, int j) {
    return uint32_t(seg) * (2u * uint32_t(half)) + uint32_t(run) * uint32_t(half) + uint32_t(j);
}

// ADV >= 0: the motion mode (ADV) and the direct collision probability are known at compile
// time (the CCP's hot loop: 1D drift; the swarm ensemble), so their tests leave the loop (4%
// of the CCP push's time); ADV < 0 reads both from the parameters. GRED: the float32 deposit
// goes to this CTA's grid in global memory (gdep, from the workspace) by vector reductions
template <typename T, bool REPLAY, int XS, bool DEPOSIT, int SG_T, int SG_I, int MINB, bool PF, int ADV, bool GRED>
__global__ void __launch_bounds__(SG_T, MINB)
    k_seg_push(bz_params p, PushConst<T> kc, Seg<T> in, Seg<T> out, const T *E, const double *R, const double *gas,
               double *moments, unsigned long long *n_pushed, unsigned int *ticket, uint32_t *seg_flags,
               uint32_t *status, float2 *gdep, uint32_t in_stride) {
    using A = typename AccT<T>::t;
    const int advect = ADV >= 0 ? ADV : p.advect;
    constexpr int SG_R = 32 * SG_I;  // particles per warp round
    extern __shared__ __align__(16) unsigned char smem[];
    const int nf = advect ? p.n_faces : 1;
    const int nnodes = p.n_nodes;
    const int xsn = (XS == BZ_XS_TABLE) ? p.xs_n : 0;
    float4 *xs_s = reinterpret_cast<float4 *>(smem);
    A *mom_s = reinterpret_cast<A *>(smem + size_t(xsn) * sizeof(float4));
    T *E_s = reinterpret_cast<T *>(reinterpret_cast<unsigned char *>(mom_s) +
                                   (DEPOSIT ? size_t(3) * nnodes * sizeof(A) : 0));
    for (int i = threadIdx.x; i < nf; i += SG_T) E_s[i] = E[i];
    if (XS == BZ_XS_TABLE)
        for (int i = threadIdx.x; i < xsn; i += SG_T)
            xs_s[i] = make_float4(p.xs_table[i], p.xs_table[xsn + i], p.xs_table[2 * xsn + i], 0.0f);
    if (DEPOSIT)
        for (int i = threadIdx.x; i < 3 * nnodes; i += SG_T) mom_s[i] = A(0);
    // GRED: (sum w, sum w e) in this CTA's grid in global memory (the ionized particles' sums
    // and the rare paths stay in shared memory)
    static_assert(!GRED || (DEPOSIT && sizeof(T) == 4 && ADV == BZ_ADVECT_1D), "global grid: float32 1D deposit");
    float2 *gd = nullptr;
    if constexpr (GRED) {
        gd = gdep + size_t(blockIdx.x) * size_t(nnodes);
        for (int i = threadIdx.x; i < nnodes; i += SG_T) gd[i] = make_float2(0.f, 0.f);
    }
    __syncthreads();
    const NodeMap &nm = kc.nm;
    const Rng rng = make_rng(p);
    const int lane = threadIdx.x & 31;
    const int H = in.half;
    uint32_t err = 0;
    uint32_t pushed = 0;  // particles with w > 0 this lane pushed (slots emptied by merges are not counted)
    bool overfull = false;
    while (true) {
        int seg = 0;
        if (lane == 0) seg = int(atomicAdd(ticket, 1u));
        seg = __shfl_sync(0xffffffffu, seg, 0);
        if (seg >= in.nseg) break;
        uint32_t ns_off = 0, nc_off = 0;  // warp-uniform running output offsets
        for (int run = 0; run < 2; ++run) {
            int cnt = in.cnt[2 * seg + run];
            if (cnt < 0 || cnt > H) {  // corrupt count: touch nothing beyond the run
                err |= BZ_DEV_CAPACITY;
                cnt = cnt < 0 ? 0 : H;
            }
            // input slot (and Philox counter) of the run's first particle: segments in_stride
            // slots apart (2 half; half for a dense array read as segments with run 1 empty)
            const uint32_t rbase = uint32_t(seg) * in_stride + uint32_t(run) * uint32_t(H);
            // one particle of the run (zeros past its end)
            auto fetch = [&](int j, T &a, T &b, T &c, T &d, T &e) {
                const bool ok = j < cnt;
                const uint32_t q = rbase + uint32_t(j);
                a = ok ? in.a.x[q] : T(0);
                b = ok ? in.a.vx[q] : T(0);
                c = ok ? in.a.vy[q] : T(0);
                d = ok ? in.a.vz[q] : T(0);
                e = ok ? in.a.w[q] : T(0);
            };
            T px = T(0), pvx = T(0), pvy = T(0), pvz = T(0), pw = T(0);  // the next round (prefetch)
            if constexpr (PF) fetch(lane, px, pvx, pvy, pvz, pw);
            for (int r0 = 0; r0 < cnt; r0 += SG_R) {
                const int j0 = r0 + lane * SG_I;
                T x[SG_I], vx[SG_I], vy[SG_I], vz[SG_I], w[SG_I];
                bool vec = false;
                if constexpr (PF) {
                    static_assert(SG_I == 1, "prefetch takes one particle per lane");
                    x[0] = px; vx[0] = pvx; vy[0] = pvy; vz[0] = pvz; w[0] = pw;
                    fetch(r0 + SG_R + lane, px, pvx, pvy, pvz, pw);
                    vec = true;
                } else if constexpr (SG_I == 4 && sizeof(T) == 4) {
                  if (j0 + SG_I <= cnt && (H % 4) == 0) {
                    vec = true;
                    const uint32_t b = rbase + uint32_t(j0);
                    float4 qa = *reinterpret_cast<const float4 *>(in.a.x + b);
                    float4 qb = *reinterpret_cast<const float4 *>(in.a.vx + b);
                    float4 qc = *reinterpret_cast<const float4 *>(in.a.vy + b);
                    float4 qd = *reinterpret_cast<const float4 *>(in.a.vz + b);
                    float4 qf = *reinterpret_cast<const float4 *>(in.a.w + b);
                    x[0] = qa.x; x[1] = qa.y; x[2] = qa.z; x[3] = qa.w;
                    vx[0] = qb.x; vx[1] = qb.y; vx[2] = qb.z; vx[3] = qb.w;
                    vy[0] = qc.x; vy[1] = qc.y; vy[2] = qc.z; vy[3] = qc.w;
                    vz[0] = qd.x; vz[1] = qd.y; vz[2] = qd.z; vz[3] = qd.w;
                    w[0] = qf.x; w[1] = qf.y; w[2] = qf.z; w[3] = qf.w;
                  }
                } else if constexpr (SG_I == 2 && sizeof(T) == 4) {
                  if (j0 + SG_I <= cnt && (H % 2) == 0) {
                    vec = true;
                    const uint32_t b = rbase + uint32_t(j0);
                    float2 qa = *reinterpret_cast<const float2 *>(in.a.x + b);
                    float2 qb = *reinterpret_cast<const float2 *>(in.a.vx + b);
                    float2 qc = *reinterpret_cast<const float2 *>(in.a.vy + b);
                    float2 qd = *reinterpret_cast<const float2 *>(in.a.vz + b);
                    float2 qf = *reinterpret_cast<const float2 *>(in.a.w + b);
                    x[0] = qa.x; x[1] = qa.y;
                    vx[0] = qb.x; vx[1] = qb.y;
                    vy[0] = qc.x; vy[1] = qc.y;
                    vz[0] = qd.x; vz[1] = qd.y;
                    w[0] = qf.x; w[1] = qf.y;
                  }
                }
                if (!vec) {
#pragma unroll
                    for (int k = 0; k < SG_I; ++k) {
                        const bool ok = j0 + k < cnt;
                        const uint32_t b = rbase + uint32_t(j0 + k);
                        x[k] = ok ? in.a.x[b] : T(0);
                        vx[k] = ok ? in.a.vx[b] : T(0);
                        vy[k] = ok ? in.a.vy[b] : T(0);
                        vz[k] = ok ? in.a.vz[b] : T(0);
                        w[k] = ok ? in.a.w[b] : T(0);
                    }
                }
                Item<T> it[SG_I];
#pragma unroll
                for (int k = 0; k < SG_I; ++k) {
                    it[k].alive = false;
                    it[k].child = false;
                    it[k].ionized = false;
                    it[k].excited = false;
                    if (w[k] > T(0)) {
                        ++pushed;
                        push_item<T, REPLAY, XS, ADV>(p, kc, rng, rbase + uint32_t(j0 + k), x[k], vx[k], vy[k], vz[k], E_s,
                                                 xs_s, R, gas, it[k]);
                        // one test for the three components (a sum of finite speeds stays finite)
                        if (!isfinite(it[k].vx + it[k].vy + it[k].vz)) err |= BZ_DEV_NONFINITE;
                        if (DEPOSIT) {
                            const bool alive = it[k].alive;
                            // an alive particle lies inside (0, L): its node needs no |x|
                            const int nd = alive ? deposit_node_pos(advect, it[k].x, nm) : -1;
                            const bool in_grid = nd >= 0 && nd < nnodes;
                            if (in_grid && advect != BZ_ADVECT_ENSEMBLE) {  // ensembles: warp-summed below
                                if constexpr (GRED)
                                    dep_red(gd, nd, float(w[k]), float(w[k] * it[k].e));
                                else
                                    dep_pair(mom_s, nd, A(w[k]), A(w[k] * it[k].e));
                                if (it[k].ionized) atomicAdd(&mom_s[2 * nnodes + nd], A(w[k]));
                            }
                            // rarely taken, one test for all: an excitation counted into the
                            // grid, an ionized particle that was absorbed, an ionization's child
                            const bool exc = in_grid && it[k].excited && (p.flags & BZ_MOMENT_EXCITATION);
                            const bool dead_ion = !alive && it[k].ionized && (p.flags & BZ_QUIRK_DEAD_IONFLAG);
                            if (exc || dead_ion || it[k].child) {
                                if (exc) atomicAdd(&moments[2 * nnodes + nd], double(w[k]));  // straight to the grid
                                if (dead_ion) atomicAdd(&mom_s[2 * nnodes + 0], A(1));
                                if (it[k].child) {
                                    const int cn = deposit_node_pos(advect, it[k].cx, nm);
                                    if (cn >= 0 && cn < nnodes) dep_pair(mom_s, cn, A(w[k]), A(w[k] * it[k].ce));
                                }
                            }
                        }
                    }
                }
                if (DEPOSIT && advect == BZ_ADVECT_ENSEMBLE) {
                    // in an ensemble a warp's particles usually belong to one swarm: when all
                    // lanes deposit to the same node, sum over the warp first (one atomic per
                    // moment instead of 32 colliding ones)
#pragma unroll
                    for (int k = 0; k < SG_I; ++k) {
                        int nd = it[k].alive ? int(it[k].x) : -1;
                        if (nd >= nnodes) nd = -1;
                        A c0 = nd >= 0 ? A(w[k]) : A(0);
                        A c1 = (nd >= 0 && it[k].ionized) ? A(w[k]) : A(0);
                        A c2 = nd >= 0 ? A(w[k] * it[k].e) : A(0);
                        const int nd0 = __shfl_sync(0xffffffffu, nd, 0);
                        if (__all_sync(0xffffffffu, nd == nd0)) {
#pragma unroll
                            for (int o = 16; o > 0; o >>= 1) {
                                c0 += __shfl_xor_sync(0xffffffffu, c0, o);
                                c1 += __shfl_xor_sync(0xffffffffu, c1, o);
                                c2 += __shfl_xor_sync(0xffffffffu, c2, o);
                            }
                            if (lane == 0 && nd0 >= 0) {
                                dep_pair(mom_s, nd0, c0, c2);
                                if (c1 != A(0)) atomicAdd(&mom_s[2 * nnodes + nd0], c1);
                            }
                        } else if (nd >= 0) {
                            dep_pair(mom_s, nd, c0, c2);
                            if (c1 != A(0)) atomicAdd(&mom_s[2 * nnodes + nd], c1);
                        }
                    }
                }
                // output offsets in input order (lane-major, then k): one ballot per flag and
                // k; the lanes below contribute popc(mask & lanes_below)
                const uint32_t below = (1u << lane) - 1u;
                uint32_t ps = ns_off, pc = nc_off, ts = 0, tc = 0;
#pragma unroll
                for (int k = 0; k < SG_I; ++k) {
                    const uint32_t ma = __ballot_sync(0xffffffffu, it[k].alive);
                    const uint32_t mc = __ballot_sync(0xffffffffu, it[k].child);
                    ps += __popc(ma & below);
                    pc += __popc(mc & below);
                    ts += __popc(ma);
                    tc += __popc(mc);
                }
#pragma unroll
                for (int k = 0; k < SG_I; ++k) {
                    if (it[k].alive) {
                        if (ps < uint32_t(H)) {
                            const uint32_t q = seg_slot32(seg, 0, H, int(ps));
                            out.a.x[q] = it[k].x; out.a.vx[q] = it[k].vx; out.a.vy[q] = it[k].vy;
                            out.a.vz[q] = it[k].vz; out.a.w[q] = w[k];
                        } else {
                            err |= BZ_DEV_CAPACITY;
                        }
                        ++ps;
                    }
                    if (it[k].child) {
                        if (pc < uint32_t(H)) {
                            const uint32_t q = seg_slot32(seg, 1, H, int(pc));
                            out.a.x[q] = it[k].cx; out.a.vx[q] = it[k].cvx; out.a.vy[q] = it[k].cvy;
                            out.a.vz[q] = it[k].cvz; out.a.w[q] = w[k];
                        } else {
                            err |= BZ_DEV_CAPACITY;
                        }
                        ++pc;
                    }
                }
                ns_off += ts;
                nc_off += tc;
            }
        }
        if (lane == 0) {
            out.cnt[2 * seg] = int32_t(min(ns_off, uint32_t(H)));
            out.cnt[2 * seg + 1] = int32_t(min(nc_off, uint32_t(H)));
        }
        if (ns_off + nc_off > uint32_t(H)) overfull = true;  // next push could overflow: repack first
    }
    if (err) atomicOr(status, err);
    if (overfull && lane == 0) atomicOr(seg_flags, BZ_SEG_NEEDS_REPACK);
    if (n_pushed) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) pushed += __shfl_xor_sync(0xffffffffu, pushed, o);
        if (lane == 0 && pushed) atomicAdd(n_pushed, (unsigned long long)pushed);
    }
    if (DEPOSIT) {
        if constexpr (GRED) __threadfence();  // this CTA's reductions are performed before the reads below
        __syncthreads();
        if constexpr (GRED) {
            for (int i = threadIdx.x; i < nnodes; i += SG_T) {
                const float2 v = __ldcg(gd + i);  // from L2
                if (v.x != 0.f) atomicAdd(&moments[i], double(v.x));
                if (v.y != 0.f) atomicAdd(&moments[3 * nnodes + i], double(v.y));
            }
        }
        for (int i = threadIdx.x; i < 3 * nnodes; i += SG_T) {
            A val = mom_s[i];
            if (val != A(0)) {
                // (sum w, sum w e) pairs -> moments rows 0 and 3; sum w of the ionizing -> row 1
                const int row = i < 2 * nnodes ? ((i & 1) ? 3 : 0) : 1;
                const int nd = i < 2 * nnodes ? (i >> 1) : i - 2 * nnodes;
                atomicAdd(&moments[row * nnodes + nd], double(val));
            }
        }
    }
}

// ------------------------------------------------------------------------------------
// repack: all particles with w != 0, in order (segment by segment, run 0 then run 1,
// then an optional dense append buffer), spread evenly over the output segments
// (fill = ceil(total / nseg) in run 0). Count -> scan -> scatter -> set counts, as the
// phases of one cooperative kernel separated by grid-wide barriers (the launch
// guarantees that every CTA is resident); deterministic. Conditional on the request flag:
// every CTA reads it at entry and it is cleared only after the last barrier.
// ------------------------------------------------------------------------------------
constexpr int RP_T = 256;

__device__ __forceinline__ bool repack_skip(const uint32_t *only_if) {
    return only_if && !(*only_if & BZ_SEG_NEEDS_REPACK);
}

template <typename T>
__device__ __forceinline__ void repack_put(Seg<T> &out, int64_t v, int fill, T x, T vx, T vy, T vz, T w,
                                           uint32_t &err) {
    if (v < 0 || v > int64_t(UINT32_MAX)) {  // slot indices fit 32 bits (checked at the entry points)
        err |= BZ_DEV_CAPACITY;
        return;
    }
    const uint32_t vv = uint32_t(v), f = uint32_t(fill);
    const uint32_t sq = vv / f;  // 32-bit division: a fraction of the 64-bit one's instructions
    const int seg = int(sq), j = int(vv - sq * f);
    if (seg < out.nseg && j < out.half) {
        const int64_t q = seg_slot(seg, 0, out.half, j);
        out.a.x[q] = x; out.a.vx[q] = vx; out.a.vy[q] = vy; out.a.vz[q] = vz; out.a.w[q] = w;
    } else {
        err |= BZ_DEV_CAPACITY;
    }
}

__device__ __forceinline__ int repack_fill(int64_t total, int nseg) {
    return int(max(int64_t(1), (total + nseg - 1) / nseg));
}

template <typename T>
__global__ void __launch_bounds__(RP_T) k_seg_repack(Seg<T> in, SoA<T> app, const int32_t *app_n, int64_t app_cap,
                                                     Seg<T> out, Seg<T> back, int32_t *live, int32_t *pre,
                                                     const uint32_t *only_if, uint32_t *seg_flags, uint32_t *status) {
    cooperative_groups::grid_group grid = cooperative_groups::this_grid();
    if (repack_skip(only_if)) return;  // uniform: the flag is cleared after the last barrier
    __shared__ int64_t part[RP_T];
    const int lane = threadIdx.x & 31;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int m = in.nseg;
    // 1. live particles per input segment
    for (int seg = gw; seg < m; seg += warps) {
        int c = 0;
        for (int run = 0; run < 2; ++run) {
            const int cnt = min(max(in.cnt[2 * seg + run], 0), in.half);
            const int64_t b = seg_slot(seg, run, in.half, 0);
#pragma unroll 8
            for (int j = lane; j < cnt; j += 32) c += (in.a.w[b + j] != T(0));
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
        if (lane == 0) live[seg] = c;
    }
    grid.sync();
    // 2. exclusive scan (CTA 0): pre[0..m), pre[m] = live total, pre[m+1] = + appended
    if (blockIdx.x == 0) {
        const int per = (m + RP_T - 1) / RP_T;
        const int lo = threadIdx.x * per, hi = min(m, lo + per);
        int64_t sum = 0;
        int k = lo;
        for (; k + 8 <= hi; k += 8) {  // eight independent loads in flight
            int32_t v[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) v[u] = live[k + u];
#pragma unroll
            for (int u = 0; u < 8; ++u) sum += v[u];
        }
        for (; k < hi; ++k) sum += live[k];
        part[threadIdx.x] = sum;
        __syncthreads();
        for (int o = 1; o < RP_T; o <<= 1) {
            const int64_t t = threadIdx.x >= o ? part[threadIdx.x - o] : 0;
            __syncthreads();
            part[threadIdx.x] += t;
            __syncthreads();
        }
        int64_t run = part[threadIdx.x] - sum;
        k = lo;
        for (; k + 8 <= hi; k += 8) {
            int32_t v[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) v[u] = live[k + u];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                pre[k + u] = int32_t(run);
                run += v[u];
            }
        }
        for (; k < hi; ++k) { pre[k] = int32_t(run); run += live[k]; }
        if (threadIdx.x == RP_T - 1) {
            const int64_t a = app_n ? min(int64_t(max(*app_n, 0)), app_cap) : 0;
            pre[m] = int32_t(part[RP_T - 1]);
            pre[m + 1] = int32_t(part[RP_T - 1] + a);
        }
    }
    grid.sync();
    // 3. scatter: input segments (warp per segment, ballot compaction), then the appended
    const int64_t total = pre[m + 1];
    const int fill = repack_fill(total, out.nseg);
    uint32_t err = 0;
    for (int seg = gw; seg < m; seg += warps) {
        int64_t off = pre[seg];
        for (int run = 0; run < 2; ++run) {
            const int cnt = min(max(in.cnt[2 * seg + run], 0), in.half);
            const int64_t b = seg_slot(seg, run, in.half, 0);
            // four rounds of 32 at a time: their weights, then the kept particles' other
            // columns, are loaded together (independent loads in flight), then written in
            // round order
            for (int j0 = 0; j0 < cnt; j0 += 4 * 32) {
                T wv[4], xx[4], a1[4], a2[4], a3[4];
                bool keep[4];
                unsigned mk[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int j = j0 + u * 32 + lane;
                    wv[u] = j < cnt ? in.a.w[b + j] : T(0);
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int j = j0 + u * 32 + lane;
                    keep[u] = j < cnt && wv[u] != T(0);
                    mk[u] = __ballot_sync(0xffffffffu, keep[u]);
                    xx[u] = keep[u] ? in.a.x[b + j] : T(0);
                    a1[u] = keep[u] ? in.a.vx[b + j] : T(0);
                    a2[u] = keep[u] ? in.a.vy[b + j] : T(0);
                    a3[u] = keep[u] ? in.a.vz[b + j] : T(0);
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    if (keep[u]) {
                        const int64_t v = off + __popc(mk[u] & ((1u << lane) - 1u));
                        repack_put(out, v, fill, xx[u], a1[u], a2[u], a3[u], wv[u], err);
                    }
                    off += __popc(mk[u]);
                }
            }
        }
    }
    if (app_n) {
        const int64_t base = pre[m];
        const int64_t na = total - base;
        for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < na && i < app_cap;
             i += int64_t(gridDim.x) * blockDim.x)
            repack_put(out, base + i, fill, app.x[i], app.vx[i], app.vy[i], app.vz[i], app.w[i], err);
    }
    if (err) atomicOr(status, err);
    grid.sync();
    // 4. output counts
    for (int s2 = blockIdx.x * blockDim.x + threadIdx.x; s2 < out.nseg; s2 += gridDim.x * blockDim.x) {
        const int64_t c = min(max(total - int64_t(s2) * fill, int64_t(0)), int64_t(min(fill, out.half)));
        out.cnt[2 * s2] = int32_t(c);
        out.cnt[2 * s2 + 1] = 0;
    }
    // 5. optionally copy the balanced layout back (same geometry): run 0 of every segment
    if (back.nseg > 0) {
        grid.sync();
        const int64_t nslots = int64_t(out.nseg) * fill;
        for (int64_t v = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; v < min(nslots, total);
             v += int64_t(gridDim.x) * blockDim.x) {
            const int seg = int(v / fill), j = int(v - int64_t(seg) * fill);
            if (j >= out.half) continue;  // an overflowing layout was already reported
            const int64_t q = seg_slot(seg, 0, out.half, j);
            back.a.x[q] = out.a.x[q]; back.a.vx[q] = out.a.vx[q]; back.a.vy[q] = out.a.vy[q];
            back.a.vz[q] = out.a.vz[q]; back.a.w[q] = out.a.w[q];
        }
        for (int s2 = blockIdx.x * blockDim.x + threadIdx.x; s2 < 2 * out.nseg; s2 += gridDim.x * blockDim.x)
            back.cnt[s2] = out.cnt[s2];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0 && seg_flags) *seg_flags = 0u;  // the request is served
}

// ------------------------------------------------------------------------------------
// place: the particles a resampling step appended (app[0 .. n_app)) go into the free slots
// of run 1 of the segments, in place, instead of a full repack of everything. Segment k
// (live_k slots with w != 0, n1_k slots in run 1) takes at most
// cap_k = min(half - n1_k, half - live_k) of them: its run 1 has the room, and its live
// particles plus the placed ones fill at most one output run of the next push, so that push
// cannot overflow. A first pass gives each segment up to fill = ceil(total / nseg) live
// particles in all, a second hands out what is left in segment order; app order is kept
// within each pass (app[0 .. A1) in the first, app[A1 ..) in the second). Slots emptied by
// merges (w = 0) stay: the next push or repack drops them. When the particles do not fit
// that way, or a segment already holds more than half live particles, nothing is placed
// and the fallback word gets BZ_SEG_NEEDS_REPACK for a conditional repack of the segments
// and app together. Each CTA owns a contiguous range of segments through all phases:
// live counts | totals and CTA-local scans of the shares | CTA offsets and copies, with
// grid-wide barriers between them (cooperative launch) and the per-CTA partial sums as the
// only exchange; deterministic.
// ------------------------------------------------------------------------------------
struct PlaceWs {
    size_t live, loc1, loce, part, misc, total;
    static int max_ctas(int nseg) { return int(ceil_div(std::max(nseg, 1), RP_T / 32)); }
    explicit PlaceWs(int nseg) {
        auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
        const size_t m = size_t(std::max(nseg, 1));
        live = 0;
        loc1 = al(4 * m);
        loce = loc1 + al(4 * m);
        part = loce + al(4 * m);
        misc = part + al(8 * 4 * size_t(max_ctas(nseg)));  // four int64 partials per CTA
        total = misc + 256;
    }
};
// misc[0]: the fallback word

// segment k's first-pass share and its room beyond it
__device__ __forceinline__ void place_share(int live, int n1, int half, int fill, int &a1, int &room) {
    const int cap = max(0, min(half - n1, half - live));
    a1 = min(max(fill - live, 0), cap);
    room = cap - a1;
}

// exclusive block scan (RP_T threads) of two int64 values; ta, tb get the block totals
__device__ __forceinline__ void rp_scan2(int64_t &a, int64_t &b, int64_t &ta, int64_t &tb, int64_t *sa, int64_t *sb) {
    const int t = threadIdx.x;
    sa[t] = a;
    sb[t] = b;
    __syncthreads();
    for (int o = 1; o < RP_T; o <<= 1) {
        const int64_t xa = t >= o ? sa[t - o] : 0, xb = t >= o ? sb[t - o] : 0;
        __syncthreads();
        sa[t] += xa;
        sb[t] += xb;
        __syncthreads();
    }
    ta = sa[RP_T - 1];
    tb = sb[RP_T - 1];
    a = sa[t] - a;
    b = sb[t] - b;
    __syncthreads();
}

__device__ __forceinline__ int nz4(float4 v) { return (v.x != 0.f) + (v.y != 0.f) + (v.z != 0.f) + (v.w != 0.f); }
__device__ __forceinline__ int nz4(double2 v) { return (v.x != 0.0) + (v.y != 0.0); }

// slots with w != 0 among w[b .. b + cnt), this lane's share (16-byte loads when w is aligned)
template <typename T> __device__ __forceinline__ int count_live(const T *w, uint32_t b, int cnt, int lane) {
    using V = typename std::conditional<sizeof(T) == 4, float4, double2>::type;
    constexpr int PER = 16 / int(sizeof(T));
    int c = 0, j0 = 0;
    if ((reinterpret_cast<uintptr_t>(w) & 15u) == 0) {  // b is a multiple of 4 (half is)
        const V *p = reinterpret_cast<const V *>(w + b);
        const int nv = cnt / PER;
#pragma unroll 4
        for (int i = lane; i < nv; i += 32) c += nz4(p[i]);
        j0 = nv * PER;
    }
    for (int j = j0 + lane; j < cnt; j += 32) c += (w[b + uint32_t(j)] != T(0));
    return c;
}

template <typename T>
__global__ void __launch_bounds__(RP_T) k_seg_place(Seg<T> s, SoA<T> app, const int32_t *app_n, int64_t app_cap,
                                                    int32_t *live, int32_t *loc1, int32_t *loce, int64_t *part,
                                                    int32_t *misc, uint32_t *seg_flags) {
    cooperative_groups::grid_group grid = cooperative_groups::this_grid();
    __shared__ int64_t sa[RP_T], sb[RP_T];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    constexpr int NW = RP_T / 32;
    const int G = gridDim.x, b = blockIdx.x;
    const int m = s.nseg, H = s.half;
    const int S = (m + G - 1) / G;  // this CTA's segments: [lo, hi)
    const int lo = min(m, b * S), hi = min(m, lo + S);
    int64_t *p_live = part, *p_bad = part + G, *p_a1 = part + 2 * G, *p_room = part + 3 * G;
    auto n1_of = [&](int k) { return min(max(s.cnt[2 * k + 1], 0), H); };
    // nothing appended and no repack requested (a resampling step whose check found nothing,
    // or merges only): nothing to place or rebalance (the same for every CTA: both words
    // change only after the last barrier below)
    if (*app_n <= 0 && !(seg_flags && (*seg_flags & BZ_SEG_NEEDS_REPACK))) {
        if (b == 0 && t == 0) misc[0] = 0;
        return;
    }
    // 1. live particles per segment (warp per segment) and the CTA's sum
    int64_t my_live = 0, my_bad = 0;
    for (int seg = lo + warp; seg < hi; seg += NW) {
        int c = 0;
        for (int run = 0; run < 2; ++run)
            c += count_live(s.a.w, seg_slot32(seg, run, H, 0), min(max(s.cnt[2 * seg + run], 0), H), lane);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
        if (lane == 0) {
            live[seg] = c;
            my_live += c;
            my_bad |= c > H;
        }
    }
    {
        int64_t tl, tb;
        rp_scan2(my_live, my_bad, tl, tb, sa, sb);
        if (t == 0) {
            p_live[b] = tl;
            p_bad[b] = tb;
        }
    }
    grid.sync();
    // 2. totals (every CTA from the same partials), then this CTA's shares, scanned locally
    int64_t TL = 0, BAD = 0;
    for (int i = t; i < G; i += RP_T) {
        TL += p_live[i];
        BAD += p_bad[i];
    }
    {
        int64_t x = TL, y = BAD;
        rp_scan2(x, y, TL, BAD, sa, sb);
    }
    const int64_t na = min(int64_t(max(*app_n, 0)), app_cap);
    const int fill = int(max(int64_t(1), (TL + na + m - 1) / m));
    int64_t c1 = 0, ce = 0;
    for (int base = lo; base < hi; base += RP_T) {
        const int k = base + t;
        int a1 = 0, room = 0;
        if (k < hi) place_share(live[k], n1_of(k), H, fill, a1, room);
        int64_t x1 = a1, xe = room, t1, te;
        rp_scan2(x1, xe, t1, te, sa, sb);
        if (k < hi) {
            loc1[k] = int32_t(c1 + x1);
            loce[k] = int32_t(ce + xe);
        }
        c1 += t1;
        ce += te;
    }
    if (t == 0) {
        p_a1[b] = c1;
        p_room[b] = ce;
    }
    grid.sync();
    // 3. the CTA's offsets in both passes and the totals, the decision, the copies
    int64_t A1 = 0, R = 0, pre1 = 0, pree = 0;
    for (int i = t; i < G; i += RP_T) {
        const int64_t v1 = p_a1[i], ve = p_room[i];
        A1 += v1;
        R += ve;
        if (i < b) {
            pre1 += v1;
            pree += ve;
        }
    }
    {
        int64_t x = A1, y = R;
        rp_scan2(x, y, A1, R, sa, sb);
        x = pre1;
        y = pree;
        rp_scan2(x, y, pre1, pree, sa, sb);
    }
    const bool fallback = BAD != 0 || A1 + R < na;  // the same in every CTA
    if (b == 0 && t == 0) {
        misc[0] = fallback ? int32_t(BZ_SEG_NEEDS_REPACK) : 0;
        // every segment will hold at most half live particles: a pending request is served
        if (!fallback && seg_flags) *seg_flags = 0u;
    }
    if (fallback) return;  // the conditional repack takes s and app together
    for (int seg = lo + warp; seg < hi; seg += NW) {
        const int n1 = n1_of(seg);
        int a1, room;
        place_share(live[seg], n1, H, fill, a1, room);
        const int64_t s1 = pre1 + loc1[seg], s2 = A1 + pree + loce[seg];
        const int len1 = int(max(int64_t(0), min(int64_t(a1), na - s1)));
        const int len2 = A1 < na ? int(max(int64_t(0), min(int64_t(room), na - s2))) : 0;
        const int len = len1 + len2;
        const uint32_t base = seg_slot32(seg, 1, H, n1);
        // four rounds of 32 at a time: all their loads in flight before the stores
        for (int j0 = 0; j0 < len; j0 += 4 * 32) {
            T xx[4], a1v[4], a2v[4], a3v[4], wv[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int j = j0 + u * 32 + lane;
                if (j < len) {
                    const int64_t i = j < len1 ? s1 + j : s2 + (j - len1);
                    xx[u] = app.x[i]; a1v[u] = app.vx[i]; a2v[u] = app.vy[i]; a3v[u] = app.vz[i]; wv[u] = app.w[i];
                }
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int j = j0 + u * 32 + lane;
                if (j < len) {
                    const uint32_t q = base + uint32_t(j);
                    s.a.x[q] = xx[u]; s.a.vx[q] = a1v[u]; s.a.vy[q] = a2v[u]; s.a.vz[q] = a3v[u]; s.a.w[q] = wv[u];
                }
            }
        }
        __syncwarp();  // every lane has read n1
        if (lane == 0) s.cnt[2 * seg + 1] = n1 + len;
    }
}

// moments of a segmented state (post_processing_1D.py:44-57), one warp per segment
template <typename T>
__global__ void __launch_bounds__(256) k_seg_deposit(bz_params p, NodeMap nm, Seg<T> s, double *moments) {
    extern __shared__ __align__(16) unsigned char smem[];
    T *m = reinterpret_cast<T *>(smem);
    const int nn = p.n_nodes;
    for (int i = threadIdx.x; i < 3 * nn; i += blockDim.x) m[i] = T(0);
    __syncthreads();
    const T efac = T(0.5 * m_e() * j_ev());
    const int lane = threadIdx.x & 31;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    for (int seg = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; seg < s.nseg; seg += warps) {
        for (int run = 0; run < 2; ++run) {
            const int cnt = min(max(s.cnt[2 * seg + run], 0), s.half);
            const int64_t b = seg_slot(seg, run, s.half, 0);
            for (int j = lane; j < cnt; j += 32) {
                const T wi = s.a.w[b + j];
                if (!(wi > T(0))) continue;
                const int nd = deposit_node(p.advect, s.a.x[b + j], nm);
                if (nd < 0 || nd >= nn) continue;
                const T vx = s.a.vx[b + j], vy = s.a.vy[b + j], vz = s.a.vz[b + j];
                atomicAdd(&m[nd], wi);
                atomicAdd(&m[2 * nn + nd], wi * efac * (vx * vx + vy * vy + vz * vz));
            }
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 3 * nn; i += blockDim.x) {
        const T v = m[i];
        if (v != T(0)) {
            const int col = i / nn, nd = i - col * nn;
            atomicAdd(&moments[(col == 2 ? 3 : col) * nn + nd], double(v));
        }
    }
}

// ------------------------------------------------------------------------------------
// host side
// ------------------------------------------------------------------------------------
template <typename T, typename S> static bool seg_ok(const S &s) {
    return s.x && s.vx && s.vy && s.vz && s.w && s.counts && s.nseg > 0 && s.half > 0 && (s.half % 4) == 0;
}
template <typename T, typename S> static Seg<T> to_seg(const S &s) {
    return Seg<T>{SoA<T>{s.x, s.vx, s.vy, s.vz, s.w}, s.counts, s.nseg, s.half};
}

template <typename T, bool REPLAY, int XS, bool DEPOSIT, int SG_T = kSegShapes[0].threads,
          int SG_I = kSegShapes[0].per_lane, int MINB = kSegShapes[0].min_blocks, bool PF = kSegShapes[0].prefetch,
          int ADV = -1, bool GRED = false>
static int launch_seg_push(const bz_params &p, Seg<T> in, Seg<T> out, const T *E, const double *R, const double *gas,
                           double *moments, uint64_t *n_pushed, void *ws, size_t ws_bytes, uint32_t *seg_flags,
                           uint32_t *status, cudaStream_t st, uint32_t in_stride) {
    using A = typename AccT<T>::t;
    const int nf = p.advect ? p.n_faces : 1;
    const int xsn = (XS == BZ_XS_TABLE) ? p.xs_n : 0;
    const size_t smem = size_t(xsn) * sizeof(float4) + (DEPOSIT ? size_t(3) * p.n_nodes * sizeof(A) : 0) +
                        size_t(nf) * sizeof(T);
    auto kern = k_seg_push<T, REPLAY, XS, DEPOSIT, SG_T, SG_I, MINB, PF, ADV, GRED>;
    if (smem > 48 * 1024 &&
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)) != cudaSuccess)
        return BZ_ERR_UNSUPPORTED;
    cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, SG_T, smem) != cudaSuccess || per_sm < 1)
        return BZ_ERR_UNSUPPORTED;
    int grid = num_sms() * per_sm;
    grid = std::max(1, std::min(grid, int(ceil_div(in.nseg, SG_T / 32))));
    // GRED: the per-CTA grids follow the ticket in the workspace; without the room for them the
    // caller takes a kernel with the deposit in shared memory instead
    float2 *gdep = nullptr;
    if (GRED) {
        if (ws_bytes < SEG_PUSH_TICKET_BYTES + size_t(grid) * size_t(p.n_nodes) * sizeof(float2)) return BZ_ERR_WORKSPACE;
        gdep = reinterpret_cast<float2 *>(static_cast<unsigned char *>(ws) + SEG_PUSH_TICKET_BYTES);
    }
    if (cudaMemsetAsync(ws, 0, SEG_PUSH_TICKET_BYTES, st) != cudaSuccess) return BZ_ERR_CUDA;
    kern<<<grid, SG_T, smem, st>>>(p, make_push_const<T>(p), in, out, E, R, gas, moments,
                                   reinterpret_cast<unsigned long long *>(n_pushed), static_cast<unsigned int *>(ws),
                                   seg_flags, status, gdep, in_stride);
    return cudaGetLastError() == cudaSuccess ? BZ_OK : BZ_ERR_CUDA;
}

template <typename T>
static int seg_push_run(const bz_params &p, Seg<T> in, uint32_t in_stride, Seg<T> out, const T *E, const double *R,
                        const double *gas, double *moments, uint64_t *n_pushed, void *ws, size_t ws_bytes,
                        uint32_t *seg_flags, uint32_t *status, cudaStream_t st);

template <typename T, typename S>
static int seg_push_entry(const bz_params *pp, S in_, S out_, const T *E, const double *R, const double *gas,
                          double *moments, uint64_t *n_pushed, void *ws, size_t ws_bytes, uint32_t *seg_flags,
                          uint32_t *status,
                          void *stream) {
    if (!pp || !E || !ws || !status || !seg_flags || !seg_ok<T>(in_) || !seg_ok<T>(out_)) return BZ_ERR_ARG;
    if (in_.nseg != out_.nseg || in_.half != out_.half) return BZ_ERR_ARG;
    if (int64_t(in_.nseg) * 2 * in_.half > int64_t(UINT32_MAX)) return BZ_ERR_TOO_LARGE;  // 32-bit slot indices
    if (ws_bytes < SEG_PUSH_TICKET_BYTES) return BZ_ERR_WORKSPACE;
    if ((R == nullptr) != (gas == nullptr)) return BZ_ERR_ARG;
    const bz_params &p = *pp;
    if (p.advect < BZ_ADVECT_NONE || p.advect > BZ_ADVECT_ENSEMBLE) return BZ_ERR_ARG;
    if (p.advect == BZ_ADVECT_1D && (p.n_faces < 1 || p.dx <= 0 || p.L <= 0)) return BZ_ERR_ARG;
    if (p.advect == BZ_ADVECT_ENSEMBLE && p.n_faces < 1) return BZ_ERR_ARG;
    if (p.n_nodes < 1 || p.bnf < 1) return BZ_ERR_ARG;
    if (p.xs_mode == BZ_XS_TABLE && (p.xs_n < 2 || !p.xs_table || !(p.xs_emax > p.xs_emin) || p.xs_emin <= 0))
        return BZ_ERR_ARG;
    if (p.xs_mode != BZ_XS_TABLE && p.xs_mode != BZ_XS_REF_FITS) return BZ_ERR_ARG;
    if (p.coll_model == BZ_COLL_NULL && !(p.nu_max > 0)) return BZ_ERR_ARG;
    auto al = [](const void *q) { return (reinterpret_cast<uintptr_t>(q) & 15u) == 0; };
    if (sizeof(T) == 4 && !(al(in_.x) && al(in_.vx) && al(in_.vy) && al(in_.vz) && al(in_.w))) return BZ_ERR_ARG;
    return seg_push_run<T>(p, to_seg<T>(in_), 2u * uint32_t(in_.half), to_seg<T>(out_), E, R, gas, moments, n_pushed,
                           ws, ws_bytes, seg_flags, status, as_stream(stream));
}

// the push of validated segments (in_stride: slots between the input segments' starts)
template <typename T>
static int seg_push_run(const bz_params &p, Seg<T> in, uint32_t in_stride, Seg<T> out, const T *E, const double *R,
                        const double *gas, double *moments, uint64_t *n_pushed, void *ws, size_t ws_bytes,
                        uint32_t *seg_flags, uint32_t *status, cudaStream_t st) {
    const bool replay = R != nullptr, dep = moments != nullptr;
    if (dep && (p.flags & BZ_CLEAR_MOMENTS) &&
        cudaMemsetAsync(moments, 0, sizeof(double) * 4 * size_t(p.n_nodes), st) != cudaSuccess)
        return BZ_ERR_CUDA;
    if constexpr (sizeof(T) == 4) {
        if (!replay && p.xs_mode == BZ_XS_TABLE && dep) {  // the hot loop: tunable CTA shape
            // the CCP's hot loop (1D drift) and the swarm ensemble, with the direct collision
            // probability, take kernels with both modes fixed at compile time in the selected
            // shape; other modes (one 0-D swarm, null collision) the default shape's general kernel
            const int adv = p.coll_model != BZ_COLL_DIRECT ? -1 : p.advect;
#define BZ_SEG_SHAPE(K)                                                                                            \
    case K:                                                                                                        \
        if (adv == BZ_ADVECT_1D) {                                                                                 \
            const int rc = launch_seg_push<T, false, BZ_XS_TABLE, true, kSegShapes[K].threads,                     \
                                           kSegShapes[K].per_lane, kSegShapes[K].min_blocks, kSegShapes[K].prefetch, \
                                           BZ_ADVECT_1D, true>(p, in, out, E, R, gas, moments, n_pushed, ws,          \
                                                               ws_bytes, seg_flags, status, st, in_stride);         \
            if (rc != BZ_ERR_WORKSPACE) return rc;                                                                 \
            break; /* no room for the per-CTA grids: the general kernel below */                                    \
        }                                                                                                          \
        if (adv == BZ_ADVECT_ENSEMBLE)                                                                             \
            return launch_seg_push<T, false, BZ_XS_TABLE, true, kSegShapes[K].threads, kSegShapes[K].per_lane,       \
                                   kSegShapes[K].min_blocks, kSegShapes[K].prefetch, BZ_ADVECT_ENSEMBLE>(            \
                p, in, out, E, R, gas, moments, n_pushed, ws, ws_bytes, seg_flags, status, st, in_stride);         \
        break;
            switch (g_seg_shape) {
                BZ_SEG_SHAPE(0)
                BZ_SEG_SHAPE(1)
                BZ_SEG_SHAPE(2)
                BZ_SEG_SHAPE(3)
                BZ_SEG_SHAPE(4)
                BZ_SEG_SHAPE(5)
                BZ_SEG_SHAPE(6)
                BZ_SEG_SHAPE(7)
                BZ_SEG_SHAPE(8)
                BZ_SEG_SHAPE(9)
                default: break;
            }
#undef BZ_SEG_SHAPE
        }
    }
    static_assert(kSegNumShapes == 10, "one case per CTA shape");
#define BZ_SEG_CASE(RP, XSM, DP)                                                                                    \
    if (replay == RP && p.xs_mode == XSM && dep == DP)                                                             \
        return launch_seg_push<T, RP, XSM, DP>(p, in, out, E, R, gas, moments, n_pushed, ws, ws_bytes, seg_flags,     \
                                               status, st, in_stride);
    BZ_SEG_CASE(false, BZ_XS_TABLE, true)
    BZ_SEG_CASE(false, BZ_XS_TABLE, false)
    BZ_SEG_CASE(false, BZ_XS_REF_FITS, true)
    BZ_SEG_CASE(false, BZ_XS_REF_FITS, false)
    BZ_SEG_CASE(true, BZ_XS_TABLE, true)
    BZ_SEG_CASE(true, BZ_XS_TABLE, false)
    BZ_SEG_CASE(true, BZ_XS_REF_FITS, true)
    BZ_SEG_CASE(true, BZ_XS_REF_FITS, false)
#undef BZ_SEG_CASE
    return BZ_ERR_ARG;
}

struct RepackWs {
    size_t live, pre, total;
    explicit RepackWs(int nseg) {
        auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
        live = 0;
        pre = al(4 * size_t(nseg));
        total = pre + al(4 * (size_t(nseg) + 2));
    }
};

template <typename T, typename S, typename P>
static int seg_repack_entry(const S *in_, P app_, const int32_t *app_n, int64_t app_cap, S out_, void *ws,
                            size_t ws_bytes, const uint32_t *only_if, uint32_t *seg_flags, uint32_t *status,
                            void *stream, const S *back_ = nullptr) {
    if (!ws || !status || !seg_ok<T>(out_)) return BZ_ERR_ARG;
    if (back_ && (!seg_ok<T>(*back_) || back_->nseg != out_.nseg || back_->half != out_.half)) return BZ_ERR_ARG;
    if (in_ && !seg_ok<T>(*in_)) return BZ_ERR_ARG;
    const bool has_app = app_n != nullptr;
    if (has_app && (!app_.x || !app_.vx || !app_.vy || !app_.vz || !app_.w || app_cap < 0)) return BZ_ERR_ARG;
    if (!in_ && !has_app) return BZ_ERR_ARG;
    const int nseg_in = in_ ? in_->nseg : 0;
    RepackWs L(nseg_in);
    if (ws_bytes < L.total) return BZ_ERR_WORKSPACE;
    unsigned char *b = static_cast<unsigned char *>(ws);
    int32_t *live = reinterpret_cast<int32_t *>(b + L.live);
    int32_t *pre = reinterpret_cast<int32_t *>(b + L.pre);
    Seg<T> in = in_ ? to_seg<T>(*in_) : Seg<T>{SoA<T>{nullptr, nullptr, nullptr, nullptr, nullptr}, nullptr, 0, 4};
    Seg<T> out = to_seg<T>(out_);
    Seg<T> back = back_ ? to_seg<T>(*back_) : Seg<T>{SoA<T>{nullptr, nullptr, nullptr, nullptr, nullptr}, nullptr, 0, 4};
    SoA<T> app{app_.x, app_.vx, app_.vy, app_.vz, app_.w};
    auto kern = k_seg_repack<T>;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, RP_T, 0) != cudaSuccess || per_sm < 1)
        return BZ_ERR_UNSUPPORTED;
    const int need = std::max(1, int(ceil_div(std::max(nseg_in, out.nseg), RP_T / 32)));
    const int grid = std::max(1, std::min(num_sms() * per_sm, need));
    void *args[] = {&in,   &app, (void *)&app_n, &app_cap, &out, &back, &live, &pre, (void *)&only_if, &seg_flags,
                    &status};
    if (cudaLaunchCooperativeKernel(reinterpret_cast<void *>(kern), dim3(grid), dim3(RP_T), args, 0,
                                    as_stream(stream)) != cudaSuccess)
        return BZ_ERR_CUDA;
    return BZ_OK;
}

template <typename T, typename S, typename P>
static int seg_place_entry(S s_, P app_, const int32_t *app_n, int64_t app_cap, S scratch_, void *ws,
                           size_t ws_bytes, uint32_t *seg_flags, uint32_t *status, void *stream) {
    if (!ws || !status || !app_n || !seg_ok<T>(s_) || !seg_ok<T>(scratch_)) return BZ_ERR_ARG;
    if (scratch_.nseg != s_.nseg || scratch_.half != s_.half) return BZ_ERR_ARG;
    if (!app_.x || !app_.vx || !app_.vy || !app_.vz || !app_.w || app_cap < 0) return BZ_ERR_ARG;
    if (int64_t(s_.nseg) * 2 * s_.half > int64_t(INT32_MAX)) return BZ_ERR_TOO_LARGE;  // int32 shares and offsets
    PlaceWs L(s_.nseg);
    const size_t rws = RepackWs(s_.nseg).total;
    if (ws_bytes < L.total + rws) return BZ_ERR_WORKSPACE;
    unsigned char *b = static_cast<unsigned char *>(ws);
    int32_t *live = reinterpret_cast<int32_t *>(b + L.live);
    int32_t *loc1 = reinterpret_cast<int32_t *>(b + L.loc1);
    int32_t *loce = reinterpret_cast<int32_t *>(b + L.loce);
    int64_t *part = reinterpret_cast<int64_t *>(b + L.part);
    int32_t *misc = reinterpret_cast<int32_t *>(b + L.misc);
    Seg<T> s = to_seg<T>(s_);
    SoA<T> app{app_.x, app_.vx, app_.vy, app_.vz, app_.w};
    auto kern = k_seg_place<T>;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, RP_T, 0) != cudaSuccess || per_sm < 1)
        return BZ_ERR_UNSUPPORTED;
    const int grid = std::max(1, std::min(num_sms() * per_sm, PlaceWs::max_ctas(s.nseg)));
    void *args[] = {&s, &app, (void *)&app_n, &app_cap, &live, &loc1, &loce, &part, &misc, &seg_flags};
    if (cudaLaunchCooperativeKernel(reinterpret_cast<void *>(kern), dim3(grid), dim3(RP_T), args, 0,
                                    as_stream(stream)) != cudaSuccess)
        return BZ_ERR_CUDA;
    // when they did not fit: the segments and app together through scratch and back
    return seg_repack_entry<T>(&s_, app_, app_n, app_cap, scratch_, b + L.total, rws,
                               reinterpret_cast<const uint32_t *>(misc), seg_flags, status, stream, &s_);
}

// ------------------------------------------------------------------------------------
// The dense push (bz_push_collide_*: survivors in input order, then children in parent
// order, the order reshuffle_data_atomics leaves, post_processing_1D.py:26-38) through the
// segmented kernel: the input array read as segments of DENSE_HALF particles (run 1 empty,
// so a particle's Philox counter stays its index in the array), pushed into segments in
// the workspace, then gathered into the reference's order. No tile waits for its
// predecessors' counts (the look-back of k_push), at the price of one more pass over the
// output (20 B read and 20 B written per particle).
// ------------------------------------------------------------------------------------
constexpr int DENSE_HALF = 2048;
struct DenseWs {
    int nseg;
    size_t push, cin, cout, part, flags, cols, col_bytes, total;
    DenseWs(int64_t in_cap, int n_nodes, size_t elem) {
        auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
        nseg = int(std::max<int64_t>(1, ceil_div(std::max<int64_t>(in_cap, 1), DENSE_HALF)));
        push = 0;
        cin = push + al(bz_seg_push_workspace_nodes(n_nodes));
        cout = cin + al(8 * size_t(nseg));
        part = cout + al(8 * size_t(nseg));
        flags = part + al(16 * size_t(PlaceWs::max_ctas(nseg)));  // two int64 partials per gather CTA
        cols = flags + 256;
        col_bytes = al(size_t(nseg) * 2 * DENSE_HALF * elem);
        total = cols + 5 * col_bytes;
    }
};

// input counts of the array read as segments: min(half, n - k half) in run 0, run 1 empty
__global__ void k_dense_in_counts(const int32_t *n_in, int64_t in_cap, int nseg, int half, int32_t *cin,
                                  uint32_t *status) {
    int64_t n = *n_in;
    if (n < 0 || n > in_cap) {  // as k_push: flag it and take what the array holds
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(status, BZ_DEV_CAPACITY);
        n = n < 0 ? 0 : in_cap;
    }
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nseg; k += gridDim.x * blockDim.x) {
        cin[2 * k] = int32_t(min(int64_t(half), max(int64_t(0), n - int64_t(k) * half)));
        cin[2 * k + 1] = 0;
    }
}

// Segments -> the reference's order: survivors of segment 0, 1, ... then children of
// segment 0, 1, ...; the counts [survivors, children, total] as k_push leaves them. Each CTA
// owns a contiguous range of segments: its sums | every CTA's offsets from all partials,
// then per chunk of RP_T segments a block scan and a warp per segment copying its runs
// (cooperative launch).
template <typename T>
__global__ void __launch_bounds__(RP_T) k_dense_gather(Seg<T> s, SoA<T> out, int64_t cap, int32_t *counts,
                                                       int64_t *part, uint32_t *status) {
    cooperative_groups::grid_group grid = cooperative_groups::this_grid();
    __shared__ int64_t sa[RP_T], sb[RP_T], o_s[RP_T], o_c[RP_T];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    constexpr int NW = RP_T / 32;
    const int G = gridDim.x, b = blockIdx.x, m = s.nseg, H = s.half;
    const int S = (m + G - 1) / G;
    const int lo = min(m, b * S), hi = min(m, lo + S);
    auto cnt_of = [&](int k, int run) { return min(max(s.cnt[2 * k + run], 0), H); };
    {
        int64_t ls = 0, lc = 0, ts, tc;
        for (int k = lo + t; k < hi; k += RP_T) {
            ls += cnt_of(k, 0);
            lc += cnt_of(k, 1);
        }
        rp_scan2(ls, lc, ts, tc, sa, sb);
        if (t == 0) {
            part[2 * b] = ts;
            part[2 * b + 1] = tc;
        }
    }
    grid.sync();
    int64_t TS = 0, TC = 0, ps = 0, pc = 0;
    for (int i = t; i < G; i += RP_T) {
        const int64_t a = part[2 * i], c = part[2 * i + 1];
        TS += a;
        TC += c;
        if (i < b) {
            ps += a;
            pc += c;
        }
    }
    {
        int64_t x = TS, y = TC;
        rp_scan2(x, y, TS, TC, sa, sb);
        x = ps;
        y = pc;
        rp_scan2(x, y, ps, pc, sa, sb);
    }
    uint32_t err = 0;
    for (int base = lo; base < hi; base += RP_T) {
        const int k = base + t;
        int64_t xs = k < hi ? cnt_of(k, 0) : 0, xc = k < hi ? cnt_of(k, 1) : 0, t1, t2;
        rp_scan2(xs, xc, t1, t2, sa, sb);
        o_s[t] = ps + xs;       // survivors from here
        o_c[t] = TS + pc + xc;  // children after every survivor
        __syncthreads();
        const int nk = min(RP_T, hi - base);
        for (int q = warp; q < nk; q += NW) {
            const int kk = base + q;
            for (int run = 0; run < 2; ++run) {
                const int c = cnt_of(kk, run);
                const int64_t d0 = run ? o_c[q] : o_s[q];
                const uint32_t s0 = seg_slot32(kk, run, H, 0);
                // four rounds of 32 at a time: their loads in flight before the stores
                for (int j0 = 0; j0 < c; j0 += 4 * 32) {
                    T xx[4], a1[4], a2[4], a3[4], wv[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const int j = j0 + u * 32 + lane;
                        if (j < c) {
                            const uint32_t q0 = s0 + uint32_t(j);
                            xx[u] = s.a.x[q0]; a1[u] = s.a.vx[q0]; a2[u] = s.a.vy[q0]; a3[u] = s.a.vz[q0];
                            wv[u] = s.a.w[q0];
                        }
                    }
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const int j = j0 + u * 32 + lane;
                        if (j < c) {
                            const int64_t d = d0 + j;
                            if (d < cap) {
                                out.x[d] = xx[u]; out.vx[d] = a1[u]; out.vy[d] = a2[u]; out.vz[d] = a3[u];
                                out.w[d] = wv[u];
                            } else {
                                err |= BZ_DEV_CAPACITY;
                            }
                        }
                    }
                }
            }
        }
        ps += t1;
        pc += t2;
        __syncthreads();  // o_s and o_c are rewritten by the next chunk
    }
    if (err) atomicOr(status, err);
    if (b == 0 && t == 0) {
        const int64_t ns = min(TS, cap), nc = max(int64_t(0), min(TC, cap - ns));
        counts[0] = int32_t(ns);
        counts[1] = int32_t(nc);
        counts[2] = int32_t(ns + nc);
    }
}

template <typename T>
int dense_push_segmented(const bz_params &p, SoA<T> in, const int32_t *n_in, int64_t in_cap, SoA<T> out, int64_t cap,
                         int32_t *counts, const T *E, const double *R, const double *gas, double *moments, void *ws,
                         size_t ws_bytes, uint32_t *status, cudaStream_t st) {
    const DenseWs L(in_cap, p.n_nodes, sizeof(T));
    // without the room, or beyond 32-bit slots and counts: the caller runs the look-back push
    if (ws_bytes < L.total) return BZ_ERR_WORKSPACE;
    if (int64_t(L.nseg) * 2 * DENSE_HALF > int64_t(UINT32_MAX) || cap > int64_t(INT32_MAX)) return BZ_ERR_WORKSPACE;
    unsigned char *b = static_cast<unsigned char *>(ws);
    int32_t *cin = reinterpret_cast<int32_t *>(b + L.cin);
    int32_t *cout = reinterpret_cast<int32_t *>(b + L.cout);
    int64_t *part = reinterpret_cast<int64_t *>(b + L.part);
    uint32_t *flags = reinterpret_cast<uint32_t *>(b + L.flags);
    T *col[5];
    for (int k = 0; k < 5; ++k) col[k] = reinterpret_cast<T *>(b + L.cols + size_t(k) * L.col_bytes);
    Seg<T> sin{in, cin, L.nseg, DENSE_HALF};
    Seg<T> sout{SoA<T>{col[0], col[1], col[2], col[3], col[4]}, cout, L.nseg, DENSE_HALF};
    k_dense_in_counts<<<int(std::min<int64_t>(ceil_div(L.nseg, 256), 1024)), 256, 0, st>>>(n_in, in_cap, L.nseg,
                                                                                            DENSE_HALF, cin, status);
    if (cudaGetLastError() != cudaSuccess) return BZ_ERR_CUDA;
    if (cudaMemsetAsync(flags, 0, sizeof(uint32_t), st) != cudaSuccess) return BZ_ERR_CUDA;
    bz_params pp = p;
    pp.flags &= ~uint32_t(BZ_CLEAR_MOMENTS);  // the dense entry has cleared them
    int rc = seg_push_run<T>(pp, sin, uint32_t(DENSE_HALF), sout, E, R, gas, moments, nullptr, b + L.push,
                             L.cin - L.push, flags, status, st);
    if (rc != BZ_OK) return rc;
    auto kern = k_dense_gather<T>;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, RP_T, 0) != cudaSuccess || per_sm < 1)
        return BZ_ERR_UNSUPPORTED;
    const int grid = std::max(1, std::min(num_sms() * per_sm, PlaceWs::max_ctas(L.nseg)));
    void *args[] = {&sout, &out, &cap, &counts, &part, &status};
    if (cudaLaunchCooperativeKernel(reinterpret_cast<void *>(kern), dim3(grid), dim3(RP_T), args, 0, st) != cudaSuccess)
        return BZ_ERR_CUDA;
    return BZ_OK;
}
template int dense_push_segmented<float>(const bz_params &, SoA<float>, const int32_t *, int64_t, SoA<float>, int64_t,
                                         int32_t *, const float *, const double *, const double *, double *, void *,
                                         size_t, uint32_t *, cudaStream_t);
template int dense_push_segmented<double>(const bz_params &, SoA<double>, const int32_t *, int64_t, SoA<double>,
                                          int64_t, int32_t *, const double *, const double *, const double *, double *,
                                          void *, size_t, uint32_t *, cudaStream_t);

// energy distribution per node (swarm): one warp per segment. The bin is taken from a
// float log2 unless it lies within 1e-4 of a bin edge, where it is recomputed in float64
// (the float estimate is off by far less than that).
template <typename T>
__global__ void __launch_bounds__(256) k_seg_eedf(bz_params p, NodeMap nm, Seg<T> s, int nbins, float a_f, float b_f,
                                                  double lemin, double scale, double *hist) {
    const double efac = 0.5 * m_e() * j_ev();
    const float efac_f = float(efac);
    const int lane = threadIdx.x & 31;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    const int nn = p.n_nodes;
    for (int seg = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; seg < s.nseg; seg += warps) {
        for (int run = 0; run < 2; ++run) {
            const int cnt = min(max(s.cnt[2 * seg + run], 0), s.half);
            const int64_t b = seg_slot(seg, run, s.half, 0);
            for (int j = lane; j < cnt; j += 32) {
                const T wi = s.a.w[b + j];
                if (!(wi > T(0))) continue;
                const int nd = deposit_node(p.advect, s.a.x[b + j], nm);
                if (nd < 0 || nd >= nn) continue;
                const T vx = s.a.vx[b + j], vy = s.a.vy[b + j], vz = s.a.vz[b + j];
                const float v2 = float(vx) * float(vx) + float(vy) * float(vy) + float(vz) * float(vz);
                if (!(v2 > 0.f)) continue;
                const float t = fmaf(__log2f(efac_f * v2), a_f, -b_f);
                if (!(t > -1.f && t < float(nbins) + 1.f)) continue;  // far outside [emin, emax)
                const float fr = t - floorf(t);
                int k;
                if (fr > 1e-4f && fr < 1.f - 1e-4f) {
                    k = int(floorf(t));
                } else {
                    const double e = efac * (double(vx) * double(vx) + double(vy) * double(vy) + double(vz) * double(vz));
                    if (!(e > 0.0)) continue;
                    k = int(floor((log(e) - lemin) * scale));
                }
                if (k < 0 || k >= nbins) continue;
                atomicAdd(&hist[int64_t(nd) * nbins + k], double(wi));
            }
        }
    }
}

template <typename T, typename S>
static int seg_eedf_entry(const bz_params *pp, S s_, int nbins, double emin, double emax, double *hist, void *stream) {
    if (!pp || !hist || !seg_ok<T>(s_) || nbins < 1 || !(emin > 0) || !(emax > emin)) return BZ_ERR_ARG;
    const bz_params &p = *pp;
    if (p.n_nodes < 1 || p.bnf < 1 || (p.advect == BZ_ADVECT_1D && (p.dx <= 0 || p.L <= 0))) return BZ_ERR_ARG;
    const double scale = double(nbins) / log(emax / emin);  // bins per e-fold
    const int blocks = std::max(1, std::min(num_sms() * 8, int(ceil_div(s_.nseg, 8))));
    k_seg_eedf<T><<<blocks, 256, 0, as_stream(stream)>>>(p, make_node_map(p), to_seg<T>(s_), nbins,
                                                         float(scale * log(2.0)), float(log(emin) * scale),
                                                         log(emin), scale, hist);
    return cudaGetLastError() == cudaSuccess ? BZ_OK : BZ_ERR_CUDA;
}

// velocities drawn from a tabulated energy distribution per key (the learned start-up):
// bin by inverse CDF, energy log-uniform within the bin, isotropic direction
template <typename T>
__global__ void __launch_bounds__(256) k_seg_sample_energy(bz_params p, NodeMap nm, Seg<T> s, int nkeys, int nbins,
                                                           double lemin, double dle, const double *cdf,
                                                           const double *escale, Rng g) {
    const double e2v = 2.0 / (j_ev() * m_e());  // eV -> (m/s)^2
    const int lane = threadIdx.x & 31;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    for (int seg = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; seg < s.nseg; seg += warps) {
        for (int run = 0; run < 2; ++run) {
            const int cnt = min(max(s.cnt[2 * seg + run], 0), s.half);
            const int64_t b = seg_slot(seg, run, s.half, 0);
            for (int j = lane; j < cnt; j += 32) {
                if (!(s.a.w[b + j] > T(0))) continue;
                const int key = deposit_node(p.advect, s.a.x[b + j], nm);
                if (key < 0 || key >= nkeys) continue;
                const double *c = cdf + int64_t(key) * nbins;
                const double tot = c[nbins - 1];
                if (!(tot > 0.0)) continue;
                const uint32_t slot = uint32_t(b + j);
                const u32x4 q = philox(slot, g.s0, g.s1, 0x65656400u, g.k0, g.k1);
                const u32x4 r = philox(slot, g.s0, g.s1, 0x65656401u, g.k0, g.k1);
                const double ub = uni_d(q.x, q.y).u * tot;
                int lo = 0, hi = nbins - 1;  // first bin whose cumulative fraction exceeds ub
                while (lo < hi) {
                    const int m = (lo + hi) >> 1;
                    if (c[m] > ub) hi = m; else lo = m + 1;
                }
                double e = exp(lemin + (double(lo) + uni_d(q.z, q.w).u) * dle);
                if (escale) e *= escale[key];
                const double sp = sqrt(e * e2v);
                const Uni<double> a = uni_d(r.x, r.y), bb = uni_d(r.z, r.w);
                const double cc = a.u - a.c, sc = 2.0 * sqrt(a.u * a.c);
                double sph, cph;
                sincospi(2.0 * bb.u, &sph, &cph);
                s.a.vx[b + j] = T(sp * sc * cph);
                s.a.vy[b + j] = T(sp * sc * sph);
                s.a.vz[b + j] = T(sp * cc);
            }
        }
    }
}

template <typename T, typename S>
static int seg_sample_energy_entry(const bz_params *pp, S s_, int nkeys, int nbins, double emin, double emax,
                                   const double *cdf, const double *escale, uint64_t seed, void *stream) {
    if (!pp || !cdf || !seg_ok<T>(s_) || nkeys < 1 || nbins < 1 || !(emin > 0) || !(emax > emin)) return BZ_ERR_ARG;
    const bz_params &p = *pp;
    if (p.advect == BZ_ADVECT_1D && (p.dx <= 0 || p.L <= 0 || p.bnf < 1 || p.n_nodes < 1)) return BZ_ERR_ARG;
    const int blocks = std::max(1, std::min(num_sms() * 8, int(ceil_div(s_.nseg, 8))));
    const Rng g{uint32_t(seed), uint32_t(seed >> 32), 0u, 0u};
    k_seg_sample_energy<T><<<blocks, 256, 0, as_stream(stream)>>>(p, make_node_map(p), to_seg<T>(s_), nkeys, nbins,
                                                                  log(emin), log(emax / emin) / nbins, cdf, escale,
                                                                  g);
    return cudaGetLastError() == cudaSuccess ? BZ_OK : BZ_ERR_CUDA;
}

template <typename T, typename S>
static int seg_deposit_entry(const bz_params *pp, S s_, double *moments, void *stream) {
    if (!pp || !moments || !seg_ok<T>(s_)) return BZ_ERR_ARG;
    const bz_params &p = *pp;
    if (p.n_nodes < 1 || p.bnf < 1 || (p.advect == BZ_ADVECT_1D && (p.dx <= 0 || p.L <= 0))) return BZ_ERR_ARG;
    const size_t smem = size_t(3) * p.n_nodes * sizeof(T);
    auto kern = k_seg_deposit<T>;
    if (smem > 48 * 1024 &&
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)) != cudaSuccess)
        return BZ_ERR_UNSUPPORTED;
    const int blocks = std::max(1, std::min(num_sms() * 4, int(ceil_div(s_.nseg, 8))));
    kern<<<blocks, 256, smem, as_stream(stream)>>>(p, make_node_map(p), to_seg<T>(s_), moments);
    return cudaGetLastError() == cudaSuccess ? BZ_OK : BZ_ERR_CUDA;
}

}  // namespace bz

extern "C" {

size_t bz_seg_push_workspace(void) { return bz::SEG_PUSH_TICKET_BYTES; }
size_t bz_seg_push_workspace_nodes(int32_t n_nodes) {
    // the ticket, then one float2 per node for every CTA the push can launch (at most 8 per SM)
    return bz::SEG_PUSH_TICKET_BYTES + size_t(bz::num_sms()) * 8 * size_t(std::max(n_nodes, 0)) * sizeof(float2);
}
int32_t bz_seg_push_shapes(void) { return bz::kSegNumShapes; }
int bz_seg_push_shape_info(int32_t shape, int32_t *threads, int32_t *per_lane, int32_t *min_blocks,
                           int32_t *prefetch) {
    if (shape < 0 || shape >= bz::kSegNumShapes) return BZ_ERR_ARG;
    if (threads) *threads = bz::kSegShapes[shape].threads;
    if (per_lane) *per_lane = bz::kSegShapes[shape].per_lane;
    if (min_blocks) *min_blocks = bz::kSegShapes[shape].min_blocks;
    if (prefetch) *prefetch = bz::kSegShapes[shape].prefetch ? 1 : 0;
    return BZ_OK;
}
int bz_seg_push_select(int32_t shape) {
    if (shape < 0 || shape >= bz::kSegNumShapes) return BZ_ERR_ARG;
    bz::g_seg_shape = shape;
    return BZ_OK;
}
int32_t bz_seg_push_selected(void) { return bz::g_seg_shape; }
size_t bz_seg_repack_workspace(int32_t nseg_in) { return bz::RepackWs(nseg_in).total; }

int bz_seg_push_collide_f32(const bz_params *p, bz_segments_f32 in, bz_segments_f32 out, const float *E,
                            const double *replay_R, const double *replay_gas, double *moments, uint64_t *n_pushed,
                            void *workspace, size_t workspace_bytes, uint32_t *seg_flags, uint32_t *status,
                            void *stream) {
    return bz::seg_push_entry<float>(p, in, out, E, replay_R, replay_gas, moments, n_pushed, workspace,
                                     workspace_bytes, seg_flags, status, stream);
}
int bz_seg_push_collide_f64(const bz_params *p, bz_segments_f64 in, bz_segments_f64 out, const double *E,
                            const double *replay_R, const double *replay_gas, double *moments, uint64_t *n_pushed,
                            void *workspace, size_t workspace_bytes, uint32_t *seg_flags, uint32_t *status,
                            void *stream) {
    return bz::seg_push_entry<double>(p, in, out, E, replay_R, replay_gas, moments, n_pushed, workspace,
                                      workspace_bytes, seg_flags, status, stream);
}
int bz_seg_repack_f32(const bz_segments_f32 *in, bz_particles_f32 app, const int32_t *app_n, int64_t app_capacity,
                      bz_segments_f32 out, void *workspace, size_t workspace_bytes, const uint32_t *only_if,
                      uint32_t *seg_flags, uint32_t *status, void *stream) {
    return bz::seg_repack_entry<float>(in, app, app_n, app_capacity, out, workspace, workspace_bytes, only_if,
                                       seg_flags, status, stream);
}
int bz_seg_repack_f64(const bz_segments_f64 *in, bz_particles_f64 app, const int32_t *app_n, int64_t app_capacity,
                      bz_segments_f64 out, void *workspace, size_t workspace_bytes, const uint32_t *only_if,
                      uint32_t *seg_flags, uint32_t *status, void *stream) {
    return bz::seg_repack_entry<double>(in, app, app_n, app_capacity, out, workspace, workspace_bytes, only_if,
                                        seg_flags, status, stream);
}
int bz_seg_rebalance_f32(bz_segments_f32 s, bz_segments_f32 scratch, void *workspace, size_t workspace_bytes,
                         const uint32_t *only_if, uint32_t *seg_flags, uint32_t *status, void *stream) {
    return bz::seg_repack_entry<float>(&s, bz_particles_f32{}, nullptr, 0, scratch, workspace, workspace_bytes,
                                       only_if, seg_flags, status, stream, &s);
}
int bz_seg_rebalance_f64(bz_segments_f64 s, bz_segments_f64 scratch, void *workspace, size_t workspace_bytes,
                         const uint32_t *only_if, uint32_t *seg_flags, uint32_t *status, void *stream) {
    return bz::seg_repack_entry<double>(&s, bz_particles_f64{}, nullptr, 0, scratch, workspace, workspace_bytes,
                                        only_if, seg_flags, status, stream, &s);
}
size_t bz_seg_place_workspace(int32_t nseg) { return bz::PlaceWs(nseg).total + bz::RepackWs(nseg).total; }
size_t bz_push_workspace_fast_f32(int64_t in_capacity, int32_t n_nodes) {
    return bz::DenseWs(in_capacity, n_nodes, sizeof(float)).total;
}
size_t bz_push_workspace_fast_f64(int64_t in_capacity, int32_t n_nodes) {
    return bz::DenseWs(in_capacity, n_nodes, sizeof(double)).total;
}
int bz_seg_place_f32(bz_segments_f32 s, bz_particles_f32 app, const int32_t *app_n, int64_t app_capacity,
                     bz_segments_f32 scratch, void *workspace, size_t workspace_bytes, uint32_t *seg_flags,
                     uint32_t *status, void *stream) {
    return bz::seg_place_entry<float>(s, app, app_n, app_capacity, scratch, workspace, workspace_bytes, seg_flags,
                                      status, stream);
}
int bz_seg_place_f64(bz_segments_f64 s, bz_particles_f64 app, const int32_t *app_n, int64_t app_capacity,
                     bz_segments_f64 scratch, void *workspace, size_t workspace_bytes, uint32_t *seg_flags,
                     uint32_t *status, void *stream) {
    return bz::seg_place_entry<double>(s, app, app_n, app_capacity, scratch, workspace, workspace_bytes, seg_flags,
                                       status, stream);
}
int bz_seg_deposit_f32(const bz_params *p, bz_segments_f32 s, double *moments, void *stream) {
    return bz::seg_deposit_entry<float>(p, s, moments, stream);
}
int bz_seg_deposit_f64(const bz_params *p, bz_segments_f64 s, double *moments, void *stream) {
    return bz::seg_deposit_entry<double>(p, s, moments, stream);
}
int bz_seg_eedf_f32(const bz_params *p, bz_segments_f32 s, int32_t nbins, double emin, double emax, double *hist,
                    void *stream) {
    return bz::seg_eedf_entry<float>(p, s, nbins, emin, emax, hist, stream);
}
int bz_seg_eedf_f64(const bz_params *p, bz_segments_f64 s, int32_t nbins, double emin, double emax, double *hist,
                    void *stream) {
    return bz::seg_eedf_entry<double>(p, s, nbins, emin, emax, hist, stream);
}
int bz_seg_sample_energy_f32(const bz_params *p, bz_segments_f32 s, int32_t n_keys, int32_t nbins, double emin,
                             double emax, const double *cdf, const double *energy_scale, uint64_t seed,
                             void *stream) {
    return bz::seg_sample_energy_entry<float>(p, s, n_keys, nbins, emin, emax, cdf, energy_scale, seed, stream);
}
int bz_seg_sample_energy_f64(const bz_params *p, bz_segments_f64 s, int32_t n_keys, int32_t nbins, double emin,
                             double emax, const double *cdf, const double *energy_scale, uint64_t seed,
                             void *stream) {
    return bz::seg_sample_energy_entry<double>(p, s, n_keys, nbins, emin, emax, cdf, energy_scale, seed, stream);
}

}  // extern "C"
