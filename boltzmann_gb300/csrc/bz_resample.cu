// ES-WPNC particle resampling (split / merge per cell and energy bin) and the
// order-preserving compaction that follows it.
//
// _check_for_resampling / _do_resampling (boltzmann.py:799-916; 3bin :813-1113;
// 5bin :843-1334) loop over cells on the host with many small CuPy calls. Here:
//   k_rs_decide  : one CTA classifies every (cell, bin) key, computes the append and
//                  random-draw offsets (processing order = key order) and the trigger;
//   k_rs_apply   : one CTA per key with work, float64 sums / scans / searches;
//   k_compact    : decoupled look-back stream compaction of w != 0.
#include <algorithm>

#include "bz_common.cuh"

namespace bz {

template <typename T> struct SoAR { T *x, *vx, *vy, *vz, *w; };

constexpr int RS_T = 256;
// a key's cumulative-weight table lives in shared memory when it has at most RS_CDF
// entries (the binary searches of the draws then hit shared memory), else in the scratch
constexpr int RS_CDF = 4096;
enum { ACT_NONE = 0, ACT_SPLIT = 1, ACT_MERGE = 2 };

struct RsWs {
    size_t act, app_off, draw_off, misc, cdf, cnt, total;
    RsWs(int64_t cap, int nkeys) {
        size_t k = size_t(nkeys) + 1, c = size_t(std::max<int64_t>(cap, 1));
        auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
        act = 0;
        app_off = act + al(4 * k);
        draw_off = app_off + al(4 * k);
        misc = draw_off + al(4 * k);
        cdf = misc + 256;
        cnt = cdf + al(8 * c);
        // six int32 regions of the key's list length: draw counts, candidate ids, copy
        // targets, and for the split's divisions the target groups (starts, fill, members)
        total = cnt + al(24 * c);
    }
};

constexpr size_t RS_APPLY_SMEM = RS_CDF * (sizeof(double) + sizeof(int32_t));

// misc[0] = total appended, misc[1] = need flag
__global__ void __launch_bounds__(1024) k_rs_decide(const int32_t *counts, const int32_t *hw_counts, int n_nodes,
                                                    int nb, const int32_t *targets, double split_below,
                                                    double merge_at, double merge_keep, int flags, int32_t *act,
                                                    int32_t *app_off, int32_t *draw_off, int32_t *misc,
                                                    int32_t *need_out) {
    __shared__ int64_t pa[65], pd[65];  // per-warp sums, then the warps' offsets, then the totals
    __shared__ int s_need_last, s_need_any;
    const int nkeys = n_nodes * nb;
    if (threadIdx.x == 0) { s_need_last = 0; s_need_any = 0; }
    __syncthreads();
    const int per = (nkeys + 1023) / 1024;
    const int lo = threadIdx.x * per, hi = min(nkeys, lo + per);
    int64_t sa = 0, sd = 0;
    int need_last = 0, need_any = 0;
    const bool per_key = (flags & BZ_PER_KEY_TARGETS) != 0;
    for (int k = lo; k < hi; ++k) {
        int b = k % nb;
        int64_t n = counts[k];
        int64_t T = targets[per_key ? k : b];
        int a = ACT_NONE;
        int64_t app = 0;
        if (n > 0 && double(n) < split_below * double(T) && hw_counts[k] > 0) {
            a = ACT_SPLIT;
            app = 2 * T - n;  // boltzmann.py:814
        } else if (double(n) >= merge_at * double(T)) {
            a = ACT_MERGE;
            app = int64_t(merge_keep * double(T));  // boltzmann.py:829
        }
        rs_key_need(n, T, b == nb - 1, split_below, merge_at, need_any, need_last);
        act[k] = a;
        sa += app;
        sd += app;
    }
    if (need_last) atomicOr(&s_need_last, 1);
    if (need_any) atomicOr(&s_need_any, 1);
    // exclusive scans of the appended and drawn counts over the 1024 threads' spans: within
    // each warp by shuffles, then over the 32 warp sums
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int64_t ia = sa, id = sd;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int64_t xa = __shfl_up_sync(0xffffffffu, ia, o), xd = __shfl_up_sync(0xffffffffu, id, o);
        if (lane >= o) {
            ia += xa;
            id += xd;
        }
    }
    if (lane == 31) {
        pa[warp] = ia;
        pd[warp] = id;
    }
    __syncthreads();
    if (warp == 0) {
        const int64_t wa = pa[lane], wd = pd[lane];
        int64_t xa = wa, xd = wd;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int64_t ya = __shfl_up_sync(0xffffffffu, xa, o), yd = __shfl_up_sync(0xffffffffu, xd, o);
            if (lane >= o) {
                xa += ya;
                xd += yd;
            }
        }
        pa[32 + lane] = xa - wa;  // the warps before this one
        pd[32 + lane] = xd - wd;
        if (lane == 31) {
            pa[64] = xa;  // the totals
            pd[64] = xd;
        }
    }
    __syncthreads();
    // the reference decides with its last max test only (boltzmann.py:913-916)
    const int need = (flags & BZ_QUIRK_TRIGGER_LAST) ? s_need_last : s_need_any;
    int64_t ra = pa[32 + warp] + ia - sa, rd = pd[32 + warp] + id - sd;
    for (int k = lo; k < hi; ++k) {
        if (!need) act[k] = ACT_NONE;
        int a = act[k];
        app_off[k] = int32_t(ra);
        draw_off[k] = int32_t(rd);
        if (a != ACT_NONE) {
            int b = k % nb;
            int64_t n = counts[k], T = targets[per_key ? k : b];
            int64_t app = (a == ACT_SPLIT) ? 2 * T - n : int64_t(merge_keep * double(T));
            ra += app;
            rd += app;
        }
    }
    if (threadIdx.x == 1023) {
        misc[0] = need ? int32_t(pa[64]) : 0;
        misc[1] = need;
        if (need_out) need_out[0] = need;
    }
}

// uniform number j of key k: replayed, or Philox 52-bit (two per call)
__device__ __forceinline__ double rs_uniform(const Rng &g, const double *replay_u, int64_t draw_base, int key,
                                             int j) {
    if (replay_u) return replay_u[draw_base + j];
    u32x4 r = philox_r<RS_ROUNDS>(uint32_t(key), uint32_t(j >> 1), g.s0, 3u | (g.s1 << 8), g.k0, g.k1);
    return (j & 1) ? uni_d(r.z, r.w).u : uni_d(r.x, r.y).u;
}

// Binary searches over a non-decreasing table of non-negative doubles. For non-negative
// IEEE doubles the order of the bit patterns as integers is the order of the values, so
// the comparisons run on the integer pipe instead of GB300's narrow float64 pipe.
__device__ __forceinline__ int lower_bound_d(const double *a, int n, double v) {
    const long long vb = __double_as_longlong(v);
    int lo = 0, hi = n;
    while (lo < hi) { int m = (lo + hi) >> 1; if (__double_as_longlong(a[m]) < vb) lo = m + 1; else hi = m; }
    return lo;
}
__device__ __forceinline__ int upper_bound_d(const double *a, int n, double v) {
    const long long vb = __double_as_longlong(v);
    int lo = 0, hi = n;
    while (lo < hi) { int m = (lo + hi) >> 1; if (__double_as_longlong(a[m]) <= vb) lo = m + 1; else hi = m; }
    return lo;
}

// The split's draws in the integer domain. A Philox draw is u = (2k+1) 2^-53 with k the
// 52-bit integer of two output words (rs_uniform). With X = cdf 2^53 (exact: a power-of-two
// scaling) and H = 2 floor(X) + [X not an integer], cdf > u holds exactly when H > 2(2k+1),
// so the binary search for the first cumulative weight above u runs on 64-bit integers
// and gives the index the float64 search gives.
// H is formed from the bits of c (0 <= c <= 1) with integer operations only: c = M 2^(e-1075)
// with M = 2^52 + mantissa, so X = M 2^(e-1022).
__device__ __forceinline__ uint64_t cdf_key(double c) {
    const uint64_t b = uint64_t(__double_as_longlong(c));
    const int e = int(b >> 52);
    if (e == 0) return b ? 1ull : 0ull;  // zero, or a subnormal (0 < X < 1)
    const uint64_t M = (b & ((1ull << 52) - 1)) | (1ull << 52);
    const int sh = 1022 - e;
    if (sh <= 0) return 2ull * (M << (-sh));  // c >= 1/2: X is an integer
    if (sh >= 64) return 1ull;                // 0 < X < 1
    return 2ull * (M >> sh) + ((M & ((1ull << sh) - 1)) ? 1ull : 0ull);
}
__device__ __forceinline__ int draw_index(const uint64_t *H, int n, uint32_t a, uint32_t b) {
    const uint64_t k = (uint64_t(a >> 6) << 26) | uint64_t(b >> 6);
    const uint64_t v = 4ull * k + 2ull;  // 2 (2k + 1)
    int lo = 0, hi = n;
    while (lo < hi) { int m = (lo + hi) >> 1; if (H[m] <= v) lo = m + 1; else hi = m; }
    return lo < n ? lo : n - 1;
}

// Sums of float32 terms as unevaluated pairs of floats (hi + lo): products made exact by
// the fma error term, additions by the two-sum error term (Dekker 1971; Knuth, TAOCP
// 4.2.2), renormalised after every addition, so each addition errs by about 2^-48 of the
// running sum. They keep this part's narrow float64 pipe out of the per-particle sums; the
// rounded operations are spelled out so that none is contracted into an fma.
struct FF { float hi, lo; };
__device__ __forceinline__ void ff_add(FF &a, float x, float xl) {
    const float s = __fadd_rn(a.hi, x), bb = __fsub_rn(s, a.hi);
    const float err = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(x, bb));
    const float lo = __fadd_rn(a.lo, __fadd_rn(err, xl));
    const float h = __fadd_rn(s, lo);
    a.lo = __fsub_rn(lo, __fsub_rn(h, s));
    a.hi = h;
}
__device__ __forceinline__ void ff_add_prod(FF &a, float x, float y) {  // a += x y
    const float p = __fmul_rn(x, y);
    ff_add(a, p, fmaf(x, y, -p));
}
__device__ __forceinline__ double ff_value(const FF &a) { return double(a.hi) + double(a.lo); }

// block helpers (RS_T threads)
template <typename V> __device__ V block_sum(V v, V *sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    V t = V(0);
    if (threadIdx.x < RS_T / 32) t = sh[threadIdx.x];
    if (warp == 0) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (lane == 0) sh[0] = t;
    }
    __syncthreads();
    V r = sh[0];
    __syncthreads();
    return r;
}

// exclusive scan over the block in thread order; returns the exclusive prefix, *total
template <typename V> __device__ V block_excl_scan(V v, V *sh, V *total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    V incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        V t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    __syncthreads();
    if (lane == 31) sh[warp] = incl;
    __syncthreads();
    if (threadIdx.x == 0) {
        V run = V(0);
        for (int w = 0; w < RS_T / 32; ++w) { V t = sh[w]; sh[w] = run; run += t; }
        sh[RS_T / 32] = run;
    }
    __syncthreads();
    V r = sh[warp] + incl - v;
    *total = sh[RS_T / 32];
    __syncthreads();
    return r;
}

// N block-wide sums with one set of barriers (sh: RS_T/32 * N doubles)
template <int N> __device__ void block_sum_n(double (&v)[N], double *sh) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < N; ++i)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[i] += __shfl_xor_sync(0xffffffffu, v[i], o);
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int i = 0; i < N; ++i) sh[warp * N + i] = v[i];
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int i = 0; i < N; ++i) {
            double t = lane < RS_T / 32 ? sh[lane * N + i] : 0.0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
            v[i] = t;
        }
        if (lane == 0)
#pragma unroll
            for (int i = 0; i < N; ++i) sh[i] = v[i];
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < N; ++i) v[i] = sh[i];
    __syncthreads();
}

// N block-wide sums of float pairs on the float32 pipe (xor-shuffle reductions of the pairs
// within each warp and then across the warps), returned in float64 to every thread: one
// conversion per sum instead of float64 adds in every thread (shf: RS_T/32 * N float2,
// shd: N doubles)
template <int N> __device__ void block_sum_ff(FF (&v)[N], double (&out)[N], float2 *shf, double *shd) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < N; ++i)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            ff_add(v[i], __shfl_xor_sync(0xffffffffu, v[i].hi, o), __shfl_xor_sync(0xffffffffu, v[i].lo, o));
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int i = 0; i < N; ++i) shf[warp * N + i] = make_float2(v[i].hi, v[i].lo);
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int i = 0; i < N; ++i) {
            FF t{0.f, 0.f};
            if (lane < RS_T / 32) t = FF{shf[lane * N + i].x, shf[lane * N + i].y};
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
                ff_add(t, __shfl_xor_sync(0xffffffffu, t.hi, o), __shfl_xor_sync(0xffffffffu, t.lo, o));
            if (lane == 0) shd[i] = ff_value(t);
        }
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < N; ++i) out[i] = shd[i];
    __syncthreads();
}

// cdf[j] = carry + sum_{i<=j} val(j) for j < len, RS_ITEMS consecutive entries per thread
// and one block scan per RS_T*RS_ITEMS entries
constexpr int RS_ITEMS = 8;
// Threads and warps past the end do no float64 arithmetic (small keys would otherwise pay
// for a whole block's padding on this part's narrow float64 pipe).
template <typename F> __device__ void block_cumsum(int len, F val, double *cdf, double *sh) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double carry = 0.0;
    for (int c0 = 0; c0 < len; c0 += RS_T * RS_ITEMS) {
        const int j0 = c0 + threadIdx.x * RS_ITEMS;
        const bool warp_live = c0 + warp * 32 * RS_ITEMS < len;
        double v[RS_ITEMS];
        double local = 0.0;
        if (j0 < len) {
#pragma unroll
            for (int i = 0; i < RS_ITEMS; ++i) {
                v[i] = j0 + i < len ? val(j0 + i) : 0.0;
                local += v[i];
            }
        }
        double incl = local;
        if (warp_live) {
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const double t = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += t;
            }
        }
        __syncthreads();
        if (lane == 31) sh[warp] = warp_live ? incl : 0.0;
        __syncthreads();
        if (threadIdx.x == 0) {
            double run = 0.0;
            for (int w = 0; w < RS_T / 32; ++w) { const double t = sh[w]; sh[w] = run; run += t; }
            sh[RS_T / 32] = run;
        }
        __syncthreads();
        if (j0 < len) {
            double acc = carry + (sh[warp] + incl - local);  // the block scan's association
#pragma unroll
            for (int i = 0; i < RS_ITEMS; ++i) {
                acc += v[i];
                if (j0 + i < len) cdf[j0 + i] = acc;
            }
        }
        carry += sh[RS_T / 32];
        __syncthreads();
    }
}

// in-place exclusive scan of a[0, n) (int32), RS_ITEMS consecutive entries per thread and
// one block scan per RS_T * RS_ITEMS entries; the result also into b when given; returns
// the total to every thread. Ends without a barrier: callers synchronise before reading.
__device__ int64_t block_scan_inplace(int32_t *a, int32_t *b, int n, int64_t *shi) {
    int64_t carry = 0;
    for (int c0 = 0; c0 < n; c0 += RS_T * RS_ITEMS) {
        const int j0 = c0 + threadIdx.x * RS_ITEMS;
        int v[RS_ITEMS];
        int local = 0;
#pragma unroll
        for (int i = 0; i < RS_ITEMS; ++i) {
            v[i] = j0 + i < n ? a[j0 + i] : 0;
            local += v[i];
        }
        int64_t tot;
        int64_t acc = carry + block_excl_scan<int64_t>(local, shi, &tot);
#pragma unroll
        for (int i = 0; i < RS_ITEMS; ++i)
            if (j0 + i < n) {
                a[j0 + i] = int32_t(acc);
                if (b) b[j0 + i] = int32_t(acc);
                acc += v[i];
            }
        carry += tot;
    }
    return carry;
}

template <typename T>
__global__ void __launch_bounds__(RS_T) k_rs_apply(bz_params p, SoAR<T> s, const int32_t *n_ptr, int64_t cap, int nb,
                                                   const int32_t *targets, const int32_t *max_ppc, double min_wt,
                                                   float wmin_f, double merge_keep, const int32_t *perm, const int32_t *offsets,
                                                   const int32_t *counts, const int32_t *act, const int32_t *app_off,
                                                   const int32_t *draw_off, const double *replay_u, double *ws_cdf,
                                                   int32_t *ws_cnt, double *cons_diag, SoAR<T> app, int64_t app_cap,
                                                   uint32_t *status) {
    __shared__ double shd[RS_T / 32 + 1];
    __shared__ double shv[RS_T / 32 * 5];
    __shared__ int64_t shi[RS_T / 32 + 1];
    const int key = blockIdx.x;
    const int a = act[key];
    if (a == ACT_NONE) return;
    const Rng rng = make_rng(p);
    const int b = key % nb;
    const int n_k = counts[key];
    const int off = offsets[key];
    // appended particles go behind the n particles of s, or into app when it is given
    const bool to_app = app.w != nullptr;
    if (int64_t(off) + n_k > cap || (!to_app && int64_t(*n_ptr) > cap)) {  // inconsistent bins: touch nothing
        if (threadIdx.x == 0) atomicOr(status, BZ_DEV_CAPACITY);
        return;
    }
    const int64_t base = (to_app ? 0 : int64_t(*n_ptr)) + app_off[key];
    SoAR<T> dst = to_app ? app : s;
    const int64_t dcap = to_app ? app_cap : cap;
    const int tk = (p.flags & BZ_PER_KEY_TARGETS) ? key : b;  // target / max_ppc entry
    const int64_t T_ = targets[tk];
    const double efac = 0.5 * m_e() * j_ev();
    extern __shared__ double cdf_sh[];  // RS_CDF doubles, then RS_CDF int32 draw counts
    int32_t *cnt_sh = reinterpret_cast<int32_t *>(cdf_sh + RS_CDF);
    // table length: the split's candidates (at most n_k) or the merge's first max_ppc
    const int tab_len = (a == ACT_SPLIT) ? n_k : min(n_k, int(max_ppc[tk]));
    double *cdf = tab_len <= RS_CDF ? cdf_sh : ws_cdf + off;
    int32_t *cnt = ws_cnt + off;
    if (a == ACT_SPLIT) {
        // ---- split (boltzmann.py:806-823): candidates w > min_wt, in index order
        int nhw = 0;
        double W = 0.0;
        // compact candidates into cnt[] (their particle ids) and their weights, in float64,
        // into the table (kept for the cumsum): RS_ITEMS consecutive entries per thread and one
        // block scan per RS_T * RS_ITEMS entries
        for (int c0 = 0; c0 < n_k; c0 += RS_T * RS_ITEMS) {
            const int j0 = c0 + threadIdx.x * RS_ITEMS;
            int ids[RS_ITEMS];
            T wv[RS_ITEMS];
            uint32_t hwm = 0;
            int local = 0;
#pragma unroll
            for (int i = 0; i < RS_ITEMS; ++i) {
                ids[i] = j0 + i < n_k ? perm[off + j0 + i] : -1;
                wv[i] = ids[i] >= 0 ? s.w[ids[i]] : T(0);
                if (ids[i] >= 0 && above_min(wv[i], min_wt, wmin_f)) {
                    hwm |= 1u << i;
                    ++local;
                }
            }
            int64_t tot;
            int64_t pos = block_excl_scan<int64_t>(local, shi, &tot);
#pragma unroll
            for (int i = 0; i < RS_ITEMS; ++i)
                if ((hwm >> i) & 1u) {
                    const double wd = double(wv[i]);
                    cnt[nhw + pos] = ids[i];
                    cdf[nhw + pos] = wd;
                    W += wd;
                    ++pos;
                }
            nhw += int(tot);
        }
        __syncthreads();
        if (nhw == 0) return;
        W = block_sum<double>(W, shd);
        // cdf = cumsum(w/W), then / cdf[-1] (CuPy RandomState.choice with p); the
        // divisions are multiplications by the reciprocal (within 2 ulp; float64 division
        // is many instructions on this part's narrow float64 pipe)
        const double inv_W = 1.0 / W;
        block_cumsum(nhw, [&](int j) { return cdf[j] * inv_W; }, cdf, shd);  // in place
        __syncthreads();
        const double inv_last = 1.0 / cdf[nhw - 1];
        // Scratch of this key. A table that fits shared memory (small) keeps the draw counts
        // there too, so cnt keeps the candidate ids and, once the draws are made, the table's
        // space holds the target groups' starts and fill pointers; otherwise the draw counts,
        // a copy of the ids and the groups live in the scratch. gmem (the groups' members),
        // tgt (each entry's target) and wgt (the weight of each entry's copies) are scratch.
        const bool small = nhw <= RS_CDF;
        int32_t *dcnt = small ? cnt_sh : cnt;
        int32_t *hw_ids = small ? cnt : ws_cnt + cap + off;
        int32_t *tgt = ws_cnt + 2 * cap + off;
        int32_t *gstart = small ? reinterpret_cast<int32_t *>(cdf_sh) : ws_cnt + 3 * cap + off;
        int32_t *gfill = small ? reinterpret_cast<int32_t *>(cdf_sh) + nhw : ws_cnt + 4 * cap + off;
        int32_t *gmem = ws_cnt + 5 * cap + off;
        T *wgt = reinterpret_cast<T *>(ws_cdf + off);
        const bool ints = replay_u == nullptr;  // Philox draws: the table as integer keys
        uint64_t *H = reinterpret_cast<uint64_t *>(cdf);
        for (int j = threadIdx.x; j < nhw; j += RS_T) {
            const double c = cdf[j] * inv_last;
            if (ints) H[j] = cdf_key(c);
            else cdf[j] = c;
            if (!small) hw_ids[j] = cnt[j];
        }
        __syncthreads();
        for (int j = threadIdx.x; j < nhw; j += RS_T) dcnt[j] = 0;
        __syncthreads();
        const int m = int(2 * T_ - n_k);
        if (ints) {
            // draws 2i and 2i+1 come from one Philox call (rs_uniform's stream)
            for (int i = threadIdx.x; 2 * i < m; i += RS_T) {
                const u32x4 r = philox_r<RS_ROUNDS>(uint32_t(key), uint32_t(i), rng.s0, 3u | (rng.s1 << 8), rng.k0,
                                                    rng.k1);
                atomicAdd(&dcnt[draw_index(H, nhw, r.x, r.y)], 1);
                if (2 * i + 1 < m) atomicAdd(&dcnt[draw_index(H, nhw, r.z, r.w)], 1);
            }
        } else {
            for (int k = threadIdx.x; k < m; k += RS_T) {
                const double u = replay_u[draw_off[key] + k];
                int ix = upper_bound_d(cdf, nhw, u);
                if (ix > nhw - 1) ix = nhw - 1;
                atomicAdd(&dcnt[ix], 1);
            }
        }
        __syncthreads();
        // the divisions. Entry j (a candidate drawn c > 0 times) divides its target's weight
        // by c+1 and its copies carry the result. The target is candidate j itself, or with
        // the reference's indexing candidate (id of j) mod nhw (HW_ids[unique_ids[v]], CuPy
        // wrapping the index, boltzmann.py:818-823), so several entries may share a target and
        // divide its weight in turn, in entry order. Entries are grouped by target (counting
        // sort), and each target's group is worked through by one thread in entry order,
        // all targets at once.
        const bool wrap = (p.flags & BZ_QUIRK_SPLIT_WRAP) != 0;
        for (int j = threadIdx.x; j < nhw; j += RS_T) gstart[j] = 0;  // the table is no longer read
        __syncthreads();
        for (int j = threadIdx.x; j < nhw; j += RS_T)
            if (dcnt[j]) atomicAdd(&gstart[wrap ? hw_ids[j] % nhw : j], 1);
        __syncthreads();
        block_scan_inplace(gstart, gfill, nhw, shi);  // group sizes -> group starts (and fill pointers)
        __syncthreads();
        for (int j = threadIdx.x; j < nhw; j += RS_T)
            if (dcnt[j]) gmem[atomicAdd(&gfill[wrap ? hw_ids[j] % nhw : j], 1)] = j;
        __syncthreads();
        #pragma unroll 4
        for (int g = threadIdx.x; g < nhw; g += RS_T) {
            const int g0 = gstart[g], g1 = gfill[g];  // after the fill, gfill[g] is the group's end
            if (g1 == g0) continue;
            for (int a1 = g0 + 1; a1 < g1; ++a1) {  // entry order (groups are a few entries)
                const int e = gmem[a1];
                int a2 = a1 - 1;
                while (a2 >= g0 && gmem[a2] > e) { gmem[a2 + 1] = gmem[a2]; --a2; }
                gmem[a2 + 1] = e;
            }
            const int t = hw_ids[g];
            T wcur = s.w[t];
            for (int a1 = g0; a1 < g1; ++a1) {
                const int j = gmem[a1];
                // w / (c+1) rounded to the state's precision. For float32 the float division
                // gives it directly: a float over an integer below 2^28 never lies close enough
                // to a float rounding midpoint (closer than 2^-53 relative without being on it)
                // for the float64 quotient, rounded again, to differ
                if constexpr (sizeof(T) == 4) wcur = __fdiv_rn(wcur, float(dcnt[j] + 1));
                else wcur = wcur / T(dcnt[j] + 1);
                wgt[j] = wcur;
                tgt[j] = t;
            }
            s.w[t] = wcur;
        }
        __syncthreads();
        // copies, in entry order: the counts become each entry's first output slot (one block
        // scan in place), then every warp works through chunks of 32 entries on its own, with
        // no block barrier: the chunk's slots are one contiguous range, which the warp fills 32
        // slots at a time with coalesced stores, each lane finding the entry of its slot by a
        // binary search over the lanes' first slots and taking the entry's values by shuffles.
        // The slots and their values are the ones a loop over each entry's copies writes.
        const int total = int(block_scan_inplace(dcnt, nullptr, nhw, shi));
        __syncthreads();
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        // one chunk's entry per lane: its first slot, its count and its copy's values
        struct Chunk { int st, en; T x, vx, vy, vz, w; };
        auto load_chunk = [&](int c0) {
            Chunk k{0, 0, T(0), T(0), T(0), T(0), T(0)};
            const int j = c0 + lane;
            if (c0 < nhw && j < nhw) {
                k.st = dcnt[j];
                k.en = j + 1 < nhw ? dcnt[j + 1] : total;
                if (k.en > k.st) {
                    const int t = tgt[j];
                    k.x = s.x[t]; k.vx = s.vx[t]; k.vy = s.vy[t]; k.vz = s.vz[t]; k.w = wgt[j];
                }
            }
            return k;
        };
        Chunk nxt = load_chunk(warp * 32);
        for (int c0 = warp * 32; c0 < nhw; c0 += RS_T) {
            const Chunk cur = nxt;
            nxt = load_chunk(c0 + RS_T);  // the next chunk's gathers are in flight while this one is written
            const int j = c0 + lane;
            const bool valid = j < nhw;
            const int st = cur.st, en = cur.en;
            const T xx = cur.x, a1 = cur.vx, a2 = cur.vy, a3 = cur.vz, ww = cur.w;
            const int last = min(31, nhw - 1 - c0);                      // the chunk's last entry
            const int wlo = __shfl_sync(0xffffffffu, st, 0);
            const int wn = __shfl_sync(0xffffffffu, en, last) - wlo;      // the chunk's slots
            const int rel = valid ? st - wlo : 0x7fffffff;                 // this entry's first slot
            for (int q0 = 0; q0 < wn; q0 += 32) {
                const int q = q0 + lane;
                int src = 0;  // the last lane whose first slot is at or below q (it has copies)
#pragma unroll
                for (int step = 16; step > 0; step >>= 1) {
                    const int e = __shfl_sync(0xffffffffu, rel, src + step);
                    if (e <= q) src += step;
                }
                const T vx0 = __shfl_sync(0xffffffffu, xx, src), vx1 = __shfl_sync(0xffffffffu, a1, src);
                const T vx2 = __shfl_sync(0xffffffffu, a2, src), vx3 = __shfl_sync(0xffffffffu, a3, src);
                const T vw = __shfl_sync(0xffffffffu, ww, src);
                if (q < wn) {
                    const int64_t d = base + wlo + q;
                    if (d < dcap) {
                        dst.x[d] = vx0; dst.vx[d] = vx1; dst.vy[d] = vx2; dst.vz[d] = vx3; dst.w[d] = vw;
                    } else {
                        atomicOr(status, BZ_DEV_CAPACITY);
                    }
                }
            }
        }
        return;
    }
    // ---- merge (boltzmann.py:826-877)
    const int np_ = min(n_k, int(max_ppc[tk]));
    const int K = int(merge_keep * double(T_));
    if (K > np_) {  // survivors need their own scratch slots (max_ppc >= merge_keep*T)
        if (threadIdx.x == 0) atomicOr(status, BZ_DEV_CAPACITY);
        return;
    }
    double W = 0, px = 0, py = 0, pz = 0, ew = 0;
    if constexpr (sizeof(T) == 4) {
        // float32 state: each thread's five sums as pairs of floats (sum w |v|^2 here, times
        // efac in float64 once per thread), then float64 across the block
        FF fW{0.f, 0.f}, fx{0.f, 0.f}, fy{0.f, 0.f}, fz{0.f, 0.f}, fe{0.f, 0.f};
        #pragma unroll 2
        for (int j = threadIdx.x; j < np_; j += RS_T) {
            const int id = perm[off + j];
            const float w = s.w[id], vx = s.vx[id], vy = s.vy[id], vz = s.vz[id];
            cdf[j] = double(w);  // kept for the cumsum
            ff_add(fW, w, 0.f);
            ff_add_prod(fx, vx, w);
            ff_add_prod(fy, vy, w);
            ff_add_prod(fz, vz, w);
            FF v2{__fmul_rn(vx, vx), fmaf(vx, vx, -__fmul_rn(vx, vx))};
            ff_add_prod(v2, vy, vy);
            ff_add_prod(v2, vz, vz);
            const float ph = __fmul_rn(w, v2.hi);
            ff_add(fe, ph, __fadd_rn(fmaf(w, v2.hi, -ph), __fmul_rn(w, v2.lo)));
        }
        FF f[5] = {fW, fx, fy, fz, fe};
        double m[5];
        block_sum_ff<5>(f, m, reinterpret_cast<float2 *>(shv), shd);
        W = m[0]; px = m[1]; py = m[2]; pz = m[3]; ew = efac * m[4];
    } else {
        #pragma unroll 4
        for (int j = threadIdx.x; j < np_; j += RS_T) {
            int id = perm[off + j];
            double w = s.w[id], vx = s.vx[id], vy = s.vy[id], vz = s.vz[id];
            cdf[j] = w;  // kept for the cumsum
            W += w;
            px += vx * w;
            py += vy * w;
            pz += vz * w;
            ew += w * (efac * (vx * vx + vy * vy + vz * vz));
        }
        double m[5] = {W, px, py, pz, ew};
        block_sum_n<5>(m, shv);
        W = m[0]; px = m[1]; py = m[2]; pz = m[3]; ew = m[4];
    }
    const double inv_W = 1.0 / W;
    const double ux = px / W, uy = py / W, uz = pz / W;
    const double T_cell = (2.0 / 3.0) * (ew / W);
    // cdf = cumsum(w/W) (not renormalised), stratified R_k = (1/K)(u_k + k)
    block_cumsum(np_, [&](int j) { return cdf[j] * inv_W; }, cdf, shd);  // in place
    __syncthreads();
    const double wbar = W / double(K);
    const T wbar_t = T(wbar);
    double hx = 0, hy = 0, hz = 0, he = 0;
    const double invK = 1.0 / double(K);
    if constexpr (sizeof(T) == 4) {
        // float32 state: the survivors all weigh W/K, so their mean velocity is (sum v)/K and
        // their energy W/K efac sum |v|^2: the sums as pairs of floats, then float64 once
        FF sx{0.f, 0.f}, sy{0.f, 0.f}, sz{0.f, 0.f}, s2{0.f, 0.f};
        #pragma unroll 2
        for (int k = threadIdx.x; k < K; k += RS_T) {
            double u = rs_uniform(rng, replay_u, draw_off[key], key, k);
            double R = invK * (u + double(k));
            int ix = lower_bound_d(cdf, np_, R);
            ix = ix % np_;  // CuPy wraps ids[len] to ids[0]
            int id = perm[off + ix];
            cnt[k] = id;
            const float vx = s.vx[id], vy = s.vy[id], vz = s.vz[id];
            ff_add(sx, vx, 0.f);
            ff_add(sy, vy, 0.f);
            ff_add(sz, vz, 0.f);
            ff_add_prod(s2, vx, vx);
            ff_add_prod(s2, vy, vy);
            ff_add_prod(s2, vz, vz);
        }
        FF f[4] = {sx, sy, sz, s2};
        double m[4];
        block_sum_ff<4>(f, m, reinterpret_cast<float2 *>(shv), shd);
        hx = m[0] * invK; hy = m[1] * invK; hz = m[2] * invK; he = wbar * (efac * m[3]);
    } else {
        #pragma unroll 4
        for (int k = threadIdx.x; k < K; k += RS_T) {
            double u = rs_uniform(rng, replay_u, draw_off[key], key, k);
            double R = invK * (u + double(k));
            int ix = lower_bound_d(cdf, np_, R);
            ix = ix % np_;  // CuPy wraps ids[len] to ids[0]
            int id = perm[off + ix];
            cnt[k] = id;
            double vx = s.vx[id], vy = s.vy[id], vz = s.vz[id];
            hx += vx * wbar;
            hy += vy * wbar;
            hz += vz * wbar;
            he += wbar * (efac * (vx * vx + vy * vy + vz * vz));
        }
        double m[4] = {hx, hy, hz, he};
        block_sum_n<4>(m, shv);
        hx = m[0] / W; hy = m[1] / W; hz = m[2] / W; he = m[3];
    }
    const double Te_hat = (2.0 / 3.0) * he / W;
    double Tfac;
    if (p.flags & BZ_FIX_MERGE_ENERGY) {
        // scale the thermal part only: sum w e about the kept mean equals the original
        // thermal energy, so total energy is conserved (the reference's factor includes
        // the drift energy, boltzmann.py:861-869)
        // (survivors that are all one particle have no kept thermal part to scale: what
        // the subtraction leaves is rounding, below 1e-12 of their energy, and the factor
        // stays 1; an original thermal part below zero by rounding counts as zero)
        double th_o = ew - efac * W * (ux * ux + uy * uy + uz * uz);
        double th_k = he - efac * W * (hx * hx + hy * hy + hz * hz);
        Tfac = th_k > 1e-12 * he ? sqrt(fmax(th_o, 0.0) / th_k) : 1.0;
    } else {
        Tfac = sqrt(T_cell / Te_hat);
    }
    __syncthreads();  // every read of the originals is done before they are zeroed / overwritten
    double aW = 0, ax = 0, ay = 0, az = 0, ae = 0;  // the survivors as stored
    double fx = 0, fy = 0, fz = 0, fe = 0;          // the survivors as formed in float64
    #pragma unroll 4
    for (int k = threadIdx.x; k < K; k += RS_T) {
        int id = cnt[k];
        T xx = s.x[id];
        double vx = ux + (double(s.vx[id]) - hx) * Tfac;
        double vy = uy + (double(s.vy[id]) - hy) * Tfac;
        double vz = uz + (double(s.vz[id]) - hz) * Tfac;
        T tx = T(vx), ty = T(vy), tz = T(vz);
        int64_t q = base + k;
        if (q < dcap) {
            dst.x[q] = xx; dst.vx[q] = tx; dst.vy[q] = ty; dst.vz[q] = tz; dst.w[q] = wbar_t;
        } else {
            atomicOr(status, BZ_DEV_CAPACITY);
        }
        if (cons_diag) {
            fx += wbar * vx;
            fy += wbar * vy;
            fz += wbar * vz;
            fe += wbar * (efac * (vx * vx + vy * vy + vz * vz));
            double wd = double(wbar_t), dx = tx, dy = ty, dz = tz;
            aW += wd;
            ax += wd * dx;
            ay += wd * dy;
            az += wd * dz;
            ae += wd * (efac * (dx * dx + dy * dy + dz * dz));
        }
    }
    __syncthreads();
    #pragma unroll 4
    for (int j = threadIdx.x; j < np_; j += RS_T) s.w[perm[off + j]] = T(0);
    if (cons_diag) {
        double m[5] = {aW, ax, ay, az, ae};
        block_sum_n<5>(m, shv);
        aW = m[0]; ax = m[1]; ay = m[2]; az = m[3]; ae = m[4];
        double f[4] = {fx, fy, fz, fe};
        block_sum_n<4>(f, shv);
        if (threadIdx.x == 0) {
            double *d = cons_diag + size_t(key) * BZ_CONS_DIAG_STRIDE;
            d[0] = W; d[1] = px; d[2] = py; d[3] = pz; d[4] = ew;
            d[5] = aW; d[6] = ax; d[7] = ay; d[8] = az; d[9] = ae;
            d[10] = wbar * double(K); d[11] = f[0]; d[12] = f[1]; d[13] = f[2]; d[14] = f[3];
        }
    }
}

// the apply kernel's dynamic shared memory (the table and the draw counts) is above the
// default 48 KB: allowed once per precision
template <typename T> static bool rs_apply_smem_ok() {
    static const bool ok = cudaFuncSetAttribute(k_rs_apply<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                int(RS_APPLY_SMEM)) == cudaSuccess;
    return ok;
}

// ------------------------------------------------------------------------------------
// order-preserving compaction of w != 0 (boltzmann.py:879-883)
// ------------------------------------------------------------------------------------
constexpr int CT = 256, CI = 4, CTILE = CT * CI;

template <typename T>
__global__ void __launch_bounds__(CT) k_compact(SoAR<T> in, const int32_t *n_ptr, const int32_t *extra,
                                                int64_t in_cap, SoAR<T> out, int64_t out_cap, int32_t *n_out,
                                                unsigned int *ticket, uint64_t *tile_status, int max_tiles,
                                                uint32_t *status, uint32_t wait_limit) {
    __shared__ int s_tile;
    __shared__ uint32_t s_ps, s_pc, s_warp[CT / 32];
    int64_t n = int64_t(max(*n_ptr, 0)) + (extra ? int64_t(max(*extra, 0)) : 0);
    if (n > in_cap) {
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(status, BZ_DEV_CAPACITY);
        n = in_cap;
    }
    const int ntiles = int(ceil_div(n, CTILE));
    if (ntiles > max_tiles) {
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(status, BZ_DEV_CAPACITY);
        return;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    while (true) {
        if (threadIdx.x == 0) s_tile = int(atomicAdd(ticket, 1u));
        __syncthreads();
        const int tile = s_tile;
        if (tile >= ntiles) break;
        const int64_t b0 = int64_t(tile) * CTILE + int64_t(threadIdx.x) * CI;
        uint32_t keep = 0;
#pragma unroll
        for (int j = 0; j < CI; ++j) {
            int64_t i = b0 + j;
            if (i < n && in.w[i] != T(0)) keep |= 1u << j;
        }
        uint32_t v = __popc(keep), incl = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        if (lane == 31) s_warp[warp] = incl;
        __syncthreads();
        if (warp == 0) {
            uint32_t wv = lane < CT / 32 ? s_warp[lane] : 0u, wi = wv;
#pragma unroll
            for (int o = 1; o < CT / 32; o <<= 1) {
                uint32_t t = __shfl_up_sync(0xffffffffu, wi, o);
                if (lane >= o) wi += t;
            }
            uint32_t tot = __shfl_sync(0xffffffffu, wi, CT / 32 - 1);
            if (lane < CT / 32) s_warp[lane] = wi - wv;
            lookback(tile_status, tile, tot, 0u, &s_ps, &s_pc, status, wait_limit);
            if (lane == 0 && tile == ntiles - 1) *n_out = int32_t(min(int64_t(s_ps + tot), out_cap));
        }
        __syncthreads();
        int64_t pos = int64_t(s_ps) + s_warp[warp] + incl - v;
#pragma unroll
        for (int j = 0; j < CI; ++j) {
            if (keep & (1u << j)) {
                int64_t i = b0 + j;
                if (pos < out_cap) {
                    out.x[pos] = in.x[i]; out.vx[pos] = in.vx[i]; out.vy[pos] = in.vy[i]; out.vz[pos] = in.vz[i];
                    out.w[pos] = in.w[i];
                } else {
                    atomicOr(status, BZ_DEV_CAPACITY);
                }
                ++pos;
            }
        }
        __syncthreads();
    }
}

struct CompactWs {
    static size_t bytes(int64_t cap) { return 256 + 8 * size_t(ceil_div(std::max<int64_t>(cap, 1), CTILE)); }
};

template <typename T>
static int launch_compact(SoAR<T> in, const int32_t *n, const int32_t *extra, int64_t in_cap, SoAR<T> out,
                          int64_t out_cap, int32_t *n_out, void *ws, size_t ws_bytes, uint32_t *status,
                          cudaStream_t st) {
    if (ws_bytes < CompactWs::bytes(1)) return BZ_ERR_WORKSPACE;
    if (cudaMemsetAsync(ws, 0, ws_bytes, st) != cudaSuccess) return BZ_ERR_CUDA;
    if (cudaMemsetAsync(n_out, 0, sizeof(int32_t), st) != cudaSuccess) return BZ_ERR_CUDA;
    int dev = 0, sms = 1, per_sm = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_compact<T>, CT, 0);
    int64_t max_tiles = int64_t((ws_bytes - 256) / 8);
    unsigned char *b = static_cast<unsigned char *>(ws);
    k_compact<T><<<sms * std::max(per_sm, 1), CT, 0, st>>>(in, n, extra, in_cap, out, out_cap, n_out,
                                                           reinterpret_cast<unsigned int *>(b),
                                                           reinterpret_cast<uint64_t *>(b + 256),
                                                           int(std::min<int64_t>(max_tiles, INT32_MAX)), status,
                                                           host_wait_limit());
    return cudaGetLastError() == cudaSuccess ? BZ_OK : BZ_ERR_CUDA;
}

template <typename T, typename P>
static int resample_entry(const bz_params *pp, P s_, const int32_t *n, int64_t cap, P out_, int32_t *n_out, int nb,
                          const int32_t *targets, const int32_t *max_ppc, double min_wt, double split_below,
                          double merge_at, double merge_keep, const int32_t *perm, const int32_t *offsets,
                          const int32_t *counts, const int32_t *hw_counts, const double *replay_u,
                          int32_t *need_out, double *cons_diag, void *ws, size_t ws_bytes, uint32_t *status,
                          void *stream) {
    if (!pp || !n || cap <= 0 || !n_out || !targets || !max_ppc || !perm || !offsets || !counts || !hw_counts ||
        !ws || !status)
        return BZ_ERR_ARG;
    if (!s_.x || !s_.vx || !s_.vy || !s_.vz || !s_.w || !out_.x || !out_.vx || !out_.vy || !out_.vz || !out_.w)
        return BZ_ERR_ARG;
    const bz_params &p = *pp;
    if (nb < 1 || p.n_nodes < 1 || !(merge_at > split_below) || !(merge_keep > 0)) return BZ_ERR_ARG;
    const int nkeys = p.n_nodes * nb;
    RsWs L(cap, nkeys);
    size_t cws = CompactWs::bytes(cap);
    if (ws_bytes < L.total + cws) return BZ_ERR_WORKSPACE;
    unsigned char *b = static_cast<unsigned char *>(ws);
    int32_t *act = reinterpret_cast<int32_t *>(b + L.act);
    int32_t *app_off = reinterpret_cast<int32_t *>(b + L.app_off);
    int32_t *draw_off = reinterpret_cast<int32_t *>(b + L.draw_off);
    int32_t *misc = reinterpret_cast<int32_t *>(b + L.misc);
    double *cdf = reinterpret_cast<double *>(b + L.cdf);
    int32_t *cnt = reinterpret_cast<int32_t *>(b + L.cnt);
    cudaStream_t st = as_stream(stream);
    k_rs_decide<<<1, 1024, 0, st>>>(counts, hw_counts, p.n_nodes, nb, targets, split_below, merge_at, merge_keep,
                                    p.flags, act, app_off, draw_off, misc, need_out);
    if (cons_diag && cudaMemsetAsync(cons_diag, 0, sizeof(double) * BZ_CONS_DIAG_STRIDE * nkeys, st) != cudaSuccess) return BZ_ERR_CUDA;
    if (!rs_apply_smem_ok<T>()) return BZ_ERR_UNSUPPORTED;
    SoAR<T> s{s_.x, s_.vx, s_.vy, s_.vz, s_.w};
    SoAR<T> o{out_.x, out_.vx, out_.vy, out_.vz, out_.w};
    k_rs_apply<T><<<nkeys, RS_T, RS_APPLY_SMEM, st>>>(p, s, n, cap, nb, targets, max_ppc, min_wt,
                                                                float_above(min_wt), merge_keep, perm, offsets,
                                          counts, act, app_off, draw_off, replay_u, cdf, cnt, cons_diag,
                                          SoAR<T>{nullptr, nullptr, nullptr, nullptr, nullptr}, 0, status);
    if (cudaGetLastError() != cudaSuccess) return BZ_ERR_CUDA;
    return launch_compact<T>(s, n, misc, cap, o, cap, n_out, b + L.total, ws_bytes - L.total, status, st);
}

template <typename T, typename S, typename P>
static int seg_resample_entry(const bz_params *pp, S s_, P app_, int64_t app_cap, S out_, int nb,
                              const int32_t *targets, const int32_t *max_ppc, double min_wt, double split_below,
                              double merge_at, double merge_keep, const int32_t *perm, const int32_t *offsets,
                              const int32_t *counts, const int32_t *hw_counts, const double *replay_u,
                              int32_t *need_out, double *cons_diag, void *ws, size_t ws_bytes, uint32_t *seg_flags,
                              uint32_t *status, void *stream);

}  // namespace bz

extern "C" {
size_t bz_seg_resample_workspace(int32_t nseg, int64_t capacity, int32_t nkeys) {
    return bz::RsWs(capacity, nkeys).total + std::max(bz_seg_repack_workspace(nseg), bz_seg_place_workspace(nseg));
}
int bz_seg_resample_f32(const bz_params *p, bz_segments_f32 s, bz_particles_f32 app, int64_t app_capacity,
                        bz_segments_f32 out, int32_t nbins, const int32_t *targets, const int32_t *max_ppc,
                        double min_wt, double split_below, double merge_at, double merge_keep, const int32_t *perm,
                        const int32_t *offsets, const int32_t *counts, const int32_t *hw_counts,
                        const double *replay_u, int32_t *need_out, double *cons_diag, void *workspace,
                        size_t workspace_bytes, uint32_t *seg_flags, uint32_t *status, void *stream) {
    return bz::seg_resample_entry<float>(p, s, app, app_capacity, out, nbins, targets, max_ppc, min_wt, split_below,
                                         merge_at, merge_keep, perm, offsets, counts, hw_counts, replay_u, need_out,
                                         cons_diag, workspace, workspace_bytes, seg_flags, status, stream);
}
int bz_seg_resample_f64(const bz_params *p, bz_segments_f64 s, bz_particles_f64 app, int64_t app_capacity,
                        bz_segments_f64 out, int32_t nbins, const int32_t *targets, const int32_t *max_ppc,
                        double min_wt, double split_below, double merge_at, double merge_keep, const int32_t *perm,
                        const int32_t *offsets, const int32_t *counts, const int32_t *hw_counts,
                        const double *replay_u, int32_t *need_out, double *cons_diag, void *workspace,
                        size_t workspace_bytes, uint32_t *seg_flags, uint32_t *status, void *stream) {
    return bz::seg_resample_entry<double>(p, s, app, app_capacity, out, nbins, targets, max_ppc, min_wt, split_below,
                                          merge_at, merge_keep, perm, offsets, counts, hw_counts, replay_u, need_out,
                                          cons_diag, workspace, workspace_bytes, seg_flags, status, stream);
}
}  // extern "C"

namespace bz {
template <typename T, typename S, typename P>
static int seg_resample_entry(const bz_params *pp, S s_, P app_, int64_t app_cap, S out_, int nb,
                              const int32_t *targets, const int32_t *max_ppc, double min_wt, double split_below,
                              double merge_at, double merge_keep, const int32_t *perm, const int32_t *offsets,
                              const int32_t *counts, const int32_t *hw_counts, const double *replay_u,
                              int32_t *need_out, double *cons_diag, void *ws, size_t ws_bytes, uint32_t *seg_flags,
                              uint32_t *status, void *stream) {
    if (!pp || !targets || !max_ppc || !perm || !offsets || !counts || !hw_counts || !ws || !status) return BZ_ERR_ARG;
    if (!s_.x || !s_.vx || !s_.vy || !s_.vz || !s_.w || !s_.counts || s_.nseg <= 0 || s_.half <= 0) return BZ_ERR_ARG;
    if (!app_.x || !app_.vx || !app_.vy || !app_.vz || !app_.w || app_cap <= 0) return BZ_ERR_ARG;
    const bz_params &p = *pp;
    if (nb < 1 || p.n_nodes < 1 || !(merge_at > split_below) || !(merge_keep > 0)) return BZ_ERR_ARG;
    const int nkeys = p.n_nodes * nb;
    const int64_t cap = int64_t(s_.nseg) * 2 * s_.half;
    RsWs L(cap, nkeys);
    const bool in_place = (p.flags & BZ_RESAMPLE_IN_PLACE) != 0;
    if (in_place && (out_.nseg != s_.nseg || out_.half != s_.half)) return BZ_ERR_ARG;
    const size_t rws = in_place ? bz_seg_place_workspace(s_.nseg) : bz_seg_repack_workspace(s_.nseg);
    if (ws_bytes < L.total + rws) return BZ_ERR_WORKSPACE;
    unsigned char *b = static_cast<unsigned char *>(ws);
    int32_t *act = reinterpret_cast<int32_t *>(b + L.act);
    int32_t *app_off = reinterpret_cast<int32_t *>(b + L.app_off);
    int32_t *draw_off = reinterpret_cast<int32_t *>(b + L.draw_off);
    int32_t *misc = reinterpret_cast<int32_t *>(b + L.misc);
    double *cdf = reinterpret_cast<double *>(b + L.cdf);
    int32_t *cnt = reinterpret_cast<int32_t *>(b + L.cnt);
    cudaStream_t st = as_stream(stream);
    k_rs_decide<<<1, 1024, 0, st>>>(counts, hw_counts, p.n_nodes, nb, targets, split_below, merge_at, merge_keep,
                                    p.flags, act, app_off, draw_off, misc, need_out);
    if (cons_diag && cudaMemsetAsync(cons_diag, 0, sizeof(double) * BZ_CONS_DIAG_STRIDE * nkeys, st) != cudaSuccess) return BZ_ERR_CUDA;
    if (!rs_apply_smem_ok<T>()) return BZ_ERR_UNSUPPORTED;
    SoAR<T> s{s_.x, s_.vx, s_.vy, s_.vz, s_.w};
    SoAR<T> app{app_.x, app_.vx, app_.vy, app_.vz, app_.w};
    k_rs_apply<T><<<nkeys, RS_T, RS_APPLY_SMEM, st>>>(p, s, nullptr, cap, nb, targets, max_ppc, min_wt,
                                                                float_above(min_wt), merge_keep, perm, offsets,
                                          counts, act, app_off, draw_off, replay_u, cdf, cnt, cons_diag, app, app_cap,
                                          status);
    if (cudaGetLastError() != cudaSuccess) return BZ_ERR_CUDA;
    int rc;
    if (in_place) {
        // the appended particles into the free slots of s (out: the scratch of a repack when
        // they do not fit)
        if (sizeof(T) == 4)
            rc = bz_seg_place_f32(*reinterpret_cast<const bz_segments_f32 *>(&s_),
                                  *reinterpret_cast<const bz_particles_f32 *>(&app_), misc, app_cap,
                                  *reinterpret_cast<const bz_segments_f32 *>(&out_), b + L.total, rws, seg_flags,
                                  status, stream);
        else
            rc = bz_seg_place_f64(*reinterpret_cast<const bz_segments_f64 *>(&s_),
                                  *reinterpret_cast<const bz_particles_f64 *>(&app_), misc, app_cap,
                                  *reinterpret_cast<const bz_segments_f64 *>(&out_), b + L.total, rws, seg_flags,
                                  status, stream);
        return rc;
    }
    // everything left in s (w != 0) followed by the appended particles, spread over out
    if (sizeof(T) == 4)
        rc = bz_seg_repack_f32(reinterpret_cast<const bz_segments_f32 *>(&s_),
                               *reinterpret_cast<const bz_particles_f32 *>(&app_), misc, app_cap,
                               *reinterpret_cast<const bz_segments_f32 *>(&out_), b + L.total, rws, nullptr, seg_flags,
                               status, stream);
    else
        rc = bz_seg_repack_f64(reinterpret_cast<const bz_segments_f64 *>(&s_),
                               *reinterpret_cast<const bz_particles_f64 *>(&app_), misc, app_cap,
                               *reinterpret_cast<const bz_segments_f64 *>(&out_), b + L.total, rws, nullptr, seg_flags,
                               status, stream);
    return rc;
}

}  // namespace bz

extern "C" {
size_t bz_resample_workspace(int64_t capacity, int32_t nkeys) {
    return bz::RsWs(capacity, nkeys).total + bz::CompactWs::bytes(capacity);
}
int bz_resample_f32(const bz_params *p, bz_particles_f32 s, const int32_t *n, int64_t capacity, bz_particles_f32 out,
                    int32_t *n_out, int32_t nbins, const int32_t *targets, const int32_t *max_ppc, double min_wt,
                    double split_below, double merge_at, double merge_keep, const int32_t *perm,
                    const int32_t *offsets, const int32_t *counts, const int32_t *hw_counts, const double *replay_u,
                    int32_t *need_out, double *cons_diag, void *workspace, size_t workspace_bytes, uint32_t *status,
                    void *stream) {
    return bz::resample_entry<float>(p, s, n, capacity, out, n_out, nbins, targets, max_ppc, min_wt, split_below,
                                     merge_at, merge_keep, perm, offsets, counts, hw_counts, replay_u, need_out,
                                     cons_diag, workspace, workspace_bytes, status, stream);
}
int bz_resample_f64(const bz_params *p, bz_particles_f64 s, const int32_t *n, int64_t capacity, bz_particles_f64 out,
                    int32_t *n_out, int32_t nbins, const int32_t *targets, const int32_t *max_ppc, double min_wt,
                    double split_below, double merge_at, double merge_keep, const int32_t *perm,
                    const int32_t *offsets, const int32_t *counts, const int32_t *hw_counts, const double *replay_u,
                    int32_t *need_out, double *cons_diag, void *workspace, size_t workspace_bytes, uint32_t *status,
                    void *stream) {
    return bz::resample_entry<double>(p, s, n, capacity, out, n_out, nbins, targets, max_ppc, min_wt, split_below,
                                      merge_at, merge_keep, perm, offsets, counts, hw_counts, replay_u, need_out,
                                      cons_diag, workspace, workspace_bytes, status, stream);
}
size_t bz_compact_workspace(int64_t capacity) { return bz::CompactWs::bytes(capacity); }
int bz_compact_f32(bz_particles_f32 in, const int32_t *n, int64_t in_capacity, bz_particles_f32 out,
                   int64_t out_capacity, int32_t *n_out, void *workspace, size_t workspace_bytes, uint32_t *status,
                   void *stream) {
    if (!n || !n_out || !workspace || !status || in_capacity < 0 || out_capacity < 0) return BZ_ERR_ARG;
    if (!in.x || !in.vx || !in.vy || !in.vz || !in.w || !out.x || !out.vx || !out.vy || !out.vz || !out.w)
        return BZ_ERR_ARG;
    bz::SoAR<float> a{in.x, in.vx, in.vy, in.vz, in.w}, b{out.x, out.vx, out.vy, out.vz, out.w};
    return bz::launch_compact<float>(a, n, nullptr, in_capacity, b, out_capacity, n_out, workspace, workspace_bytes,
                                     status, bz::as_stream(stream));
}
int bz_compact_f64(bz_particles_f64 in, const int32_t *n, int64_t in_capacity, bz_particles_f64 out,
                   int64_t out_capacity, int32_t *n_out, void *workspace, size_t workspace_bytes, uint32_t *status,
                   void *stream) {
    if (!n || !n_out || !workspace || !status || in_capacity < 0 || out_capacity < 0) return BZ_ERR_ARG;
    if (!in.x || !in.vx || !in.vy || !in.vz || !in.w || !out.x || !out.vx || !out.vy || !out.vz || !out.w)
        return BZ_ERR_ARG;
    bz::SoAR<double> a{in.x, in.vx, in.vy, in.vz, in.w}, b{out.x, out.vx, out.vy, out.vz, out.w};
    return bz::launch_compact<double>(a, n, nullptr, in_capacity, b, out_capacity, n_out, workspace,
                                      workspace_bytes, status, bz::as_stream(stream));
}
}
