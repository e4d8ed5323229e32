// Cell x energy-bin binning as a stable counting sort.
//
// Replaces define_particle_bins (bin_particles.py:7-22; 3bin/5bin :7-49), whose atomic
// appends give a nondeterministic order, with a deterministic one: particles sorted by
// key = cell*nbins + ebin, ascending particle index within a key (the order the
// reference's serial semantics would give). Keys are 16-bit; the sort is an LSD radix
// sort with 8-bit digits (one or two passes). Each pass: per-tile digit histograms,
// a scan in (digit, tile) order, and a stable scatter in which every warp ranks its
// own contiguous segment with __match_any_sync. Per-key counts and split-candidate
// counts are formed in the key pass with shared-memory histograms.
#include <algorithm>

#include "bz_common.cuh"

namespace bz {

constexpr int RB_T = 512;               // threads per tile CTA
constexpr int RB_I = 8;                 // items per thread
constexpr int RB_TILE = RB_T * RB_I;    // 4096 items per tile
constexpr int RB_W = RB_T / 32;         // warps
constexpr int RB_SEG = RB_TILE / RB_W;  // items per warp segment (256)
constexpr int RADIX = 256;

// energy as the reference holds it when binning: tosum[:,3] = ((e*w)/w) after
// post_processing (post_processing_1D.py:53,62), e = 0.5 m_e j_ev (vx^2+vy^2+vz^2)
template <typename T>
__device__ __forceinline__ int energy_bin(T vx, T vy, T vz, T w, int nb, const double *edges_s,
                                          const float *edges_f, float efac_f, double efac_d) {
    if (nb == 1) return 0;
    if (sizeof(T) == 4) {
        float e = efac_f * (float(vx) * float(vx) + float(vy) * float(vy) + float(vz) * float(vz));
        bool safe = true;
        int b = nb - 1;
        for (int k = nb - 2; k >= 0; --k) {
            const float ed = edges_f[k];
            if (fabsf(e - ed) <= 1e-5f * fabsf(ed) + 1e-30f) safe = false;
            if (e < ed) b = k;
        }
        if (safe && isfinite(e)) return b;
    }
    double dvx = double(vx), dvy = double(vy), dvz = double(vz), dw = double(w);
    double e = efac_d * (dvx * dvx + dvy * dvy + dvz * dvz);
    if (dw > 0) e = (e * dw) / dw;
    for (int k = 0; k < nb - 1; ++k)
        if (e < edges_s[k]) return k;
    if (e >= edges_s[nb - 2]) return nb - 1;
    return -1;  // NaN energy: in no bin (every comparison of the reference fails)
}


template <typename T>
__global__ void __launch_bounds__(RB_T) k_bin_keys(bz_params p, const T *x, const T *vx, const T *vy, const T *vz,
                                                   const T *w, const int32_t *n_ptr, int64_t cap, int nb,
                                                   const double *edges, double min_wt, float wmin_f,
                                                   float inv_dx_f, uint16_t *keys, uint32_t *hist, int32_t *counts,
                                                   int32_t *hw_counts, int nkeys, uint32_t *status) {
    extern __shared__ __align__(16) unsigned char smem[];
    uint32_t *c_s = reinterpret_cast<uint32_t *>(smem);  // [nkeys] counts
    uint32_t *h_s = c_s + nkeys;                          // [nkeys] hw counts
    uint32_t *d_s = h_s + nkeys;                          // [RADIX] low-digit histogram
    __shared__ double edges_s[16];
    __shared__ float edges_f[16];
    const int n = int(min(int64_t(max(*n_ptr, 0)), cap));
    const int ntiles = int(ceil_div(n, RB_TILE));
    if (int(blockIdx.x) >= ntiles) return;
    for (int i = threadIdx.x; i < 2 * nkeys + RADIX; i += RB_T) c_s[i] = 0;
    if (threadIdx.x < 16) {
        edges_s[threadIdx.x] = threadIdx.x < nb - 1 ? edges[threadIdx.x] : 0.0;
        edges_f[threadIdx.x] = float(edges_s[threadIdx.x]);
    }
    __syncthreads();
    const float efac_f = float(0.5 * m_e() * j_ev());
    const double efac_d = 0.5 * m_e() * j_ev();
    uint32_t err = 0;
    const int64_t t0 = int64_t(blockIdx.x) * RB_TILE;
    for (int j = threadIdx.x; j < RB_TILE; j += RB_T) {
        int64_t i = t0 + j;
        if (i >= n) break;
        T wi = w[i];
        int key = nkeys;  // invalid: sorted past every bin
        if (wi > T(0)) {
            int cell = bin_cell(p.advect, x[i], p.dx, inv_dx_f);
            int b = energy_bin(vx[i], vy[i], vz[i], wi, nb, edges_s, edges_f, efac_f, efac_d);
            if (cell >= 0 && cell < p.n_nodes && b >= 0) {
                key = cell * nb + b;
                atomicAdd(&c_s[key], 1u);
                if (above_min(wi, min_wt, wmin_f)) atomicAdd(&h_s[key], 1u);
            } else {
                err |= BZ_DEV_BINRANGE;
            }
        }
        keys[i] = uint16_t(key);
        atomicAdd(&d_s[key & 0xff], 1u);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < nkeys; k += RB_T) {
        if (c_s[k]) atomicAdd(reinterpret_cast<unsigned int *>(&counts[k]), c_s[k]);
        if (h_s[k]) atomicAdd(reinterpret_cast<unsigned int *>(&hw_counts[k]), h_s[k]);
    }
    for (int d = threadIdx.x; d < RADIX; d += RB_T) hist[size_t(blockIdx.x) * RADIX + d] = d_s[d];
    if (err) atomicOr(status, err);
}

__global__ void __launch_bounds__(RB_T) k_radix_hist(const uint16_t *keys, const int32_t *n_ptr, int64_t cap,
                                                     int shift, uint32_t *hist) {
    __shared__ uint32_t d_s[RADIX];
    const int n = int(min(int64_t(max(*n_ptr, 0)), cap));
    const int ntiles = int(ceil_div(n, RB_TILE));
    // the live tile count is known only here: a grid of a few CTAs per SM loops over them
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        for (int i = threadIdx.x; i < RADIX; i += RB_T) d_s[i] = 0;
        __syncthreads();
        const int64_t t0 = int64_t(tile) * RB_TILE;
        for (int j = threadIdx.x; j < RB_TILE; j += RB_T) {
            int64_t i = t0 + j;
            if (i >= n) break;
            atomicAdd(&d_s[(keys[i] >> shift) & 0xff], 1u);
        }
        __syncthreads();
        for (int d = threadIdx.x; d < RADIX; d += RB_T) hist[size_t(tile) * RADIX + d] = d_s[d];
        __syncthreads();
    }
}

// hist[t][d] -> global exclusive offset of (digit d, tile t) in (digit, tile) order, in two
// passes of one CTA per digit: the column totals, then each column's exclusive scan plus
// the totals of the digits below it (integer sums: the result does not depend on the order).
constexpr int RS_COL_T = 256;

__device__ __forceinline__ uint32_t cta_sum_u32(uint32_t v, uint32_t *sh) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    uint32_t t = 0;
    for (int w = 0; w < RS_COL_T / 32; ++w) t += sh[w];
    __syncthreads();
    return t;
}

__global__ void __launch_bounds__(RS_COL_T) k_radix_colsum(const uint32_t *hist, const int32_t *n_ptr, int64_t cap,
                                                          uint32_t *totals) {
    __shared__ uint32_t sh[RS_COL_T / 32];
    const int n = int(min(int64_t(max(*n_ptr, 0)), cap));
    const int ntiles = int(ceil_div(n, RB_TILE));
    const int d = blockIdx.x;
    uint32_t s = 0;
    for (int t = threadIdx.x; t < ntiles; t += RS_COL_T) s += hist[size_t(t) * RADIX + d];
    s = cta_sum_u32(s, sh);
    if (threadIdx.x == 0) totals[d] = s;
}

__global__ void __launch_bounds__(RS_COL_T) k_radix_colscan(uint32_t *hist, const int32_t *n_ptr, int64_t cap,
                                                           const uint32_t *totals) {
    __shared__ uint32_t sh[RS_COL_T / 32];
    const int n = int(min(int64_t(max(*n_ptr, 0)), cap));
    const int ntiles = int(ceil_div(n, RB_TILE));
    const int d = blockIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t b = 0;
    for (int k = threadIdx.x; k < d; k += RS_COL_T) b += totals[k];
    uint32_t carry = cta_sum_u32(b, sh);  // the digits below d
    constexpr int PER = 8;                // consecutive tiles per thread in a chunk
    for (int c0 = 0; c0 < ntiles; c0 += RS_COL_T * PER) {
        const int t0 = c0 + threadIdx.x * PER;
        uint32_t v[PER], local = 0;
#pragma unroll
        for (int u = 0; u < PER; ++u) {
            v[u] = t0 + u < ntiles ? hist[size_t(t0 + u) * RADIX + d] : 0u;
            local += v[u];
        }
        uint32_t incl = local;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        if (lane == 31) sh[warp] = incl;
        __syncthreads();
        uint32_t before = 0, chunk = 0;
        for (int w = 0; w < RS_COL_T / 32; ++w) {
            if (w < warp) before += sh[w];
            chunk += sh[w];
        }
        uint32_t run = carry + before + incl - local;
#pragma unroll
        for (int u = 0; u < PER; ++u) {
            if (t0 + u < ntiles) hist[size_t(t0 + u) * RADIX + d] = run;
            run += v[u];
        }
        carry += chunk;
        __syncthreads();  // sh is rewritten by the next chunk
    }
}

// Stable scatter by the digit at ``shift``. vals_in == nullptr means identity values.
// The tile is first sorted by digit in shared memory (each warp ranks its contiguous run
// with __match_any_sync), then written out digit run by digit run, so that consecutive
// threads write consecutive addresses (runs of ~tile/256 items) instead of scattering
// every item to its own sector.
constexpr size_t RB_SCATTER_SMEM = sizeof(uint32_t) * (RB_W * RADIX + 2 * RADIX) + RB_TILE * (2 + 4);

__global__ void __launch_bounds__(RB_T) k_radix_scatter(const uint16_t *keys_in, const uint32_t *vals_in,
                                                        const int32_t *n_ptr, int64_t cap, int shift,
                                                        const uint32_t *offsets, uint16_t *keys_out,
                                                        uint32_t *vals_out) {
    extern __shared__ __align__(16) unsigned char smem[];
    uint32_t (*cnt)[RADIX] = reinterpret_cast<uint32_t (*)[RADIX]>(smem);
    uint32_t *lbase = reinterpret_cast<uint32_t *>(smem) + RB_W * RADIX;  // tile-local start of each digit
    uint32_t *gshift = lbase + RADIX;                                      // global start - local start
    uint32_t *v_s = gshift + RADIX;
    uint16_t *k_s = reinterpret_cast<uint16_t *>(v_s + RB_TILE);
    const int n = int(min(int64_t(max(*n_ptr, 0)), cap));
    const int ntiles = int(ceil_div(n, RB_TILE));
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // a grid of a few CTAs per SM loops over the live tiles (their count is known only here)
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        for (int i = threadIdx.x; i < RB_W * RADIX; i += RB_T) (&cnt[0][0])[i] = 0;
        __syncthreads();
        const int64_t tile0 = int64_t(tile) * RB_TILE;
        const int tile_n = int(min(int64_t(RB_TILE), int64_t(n) - tile0));
        const int64_t seg0 = tile0 + int64_t(warp) * RB_SEG;
        uint16_t k[RB_I];
        uint32_t v[RB_I];
        const unsigned lt_mask = (1u << lane) - 1u;
#pragma unroll
        for (int r = 0; r < RB_I; ++r) {
            int64_t i = seg0 + r * 32 + lane;
            bool ok = i < n;
            k[r] = ok ? keys_in[i] : uint16_t(0);
            v[r] = ok ? (vals_in ? vals_in[i] : uint32_t(i)) : 0u;
            unsigned act = __ballot_sync(0xffffffffu, ok);
            if (ok) {
                int dg = (k[r] >> shift) & 0xff;
                unsigned peers = __match_any_sync(act, dg);
                if (lane == __ffs(peers) - 1) cnt[warp][dg] += __popc(peers);
            }
            __syncwarp();
        }
        __syncthreads();
        // per digit: the tile's total, its local start (exclusive scan over digits, one warp),
        // and the warps' local starts
        if (warp == 0) {
            uint32_t carry = 0;
            for (int d0 = 0; d0 < RADIX; d0 += 32) {
                const int dg = d0 + lane;
                uint32_t tot = 0;
                for (int ww = 0; ww < RB_W; ++ww) tot += cnt[ww][dg];
                uint32_t incl = tot;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
                    if (lane >= o) incl += t;
                }
                lbase[dg] = carry + incl - tot;
                carry += __shfl_sync(0xffffffffu, incl, 31);
            }
        }
        __syncthreads();
        for (int dg = threadIdx.x; dg < RADIX; dg += RB_T) {
            uint32_t run = lbase[dg];
            gshift[dg] = offsets[size_t(tile) * RADIX + dg] - run;
            for (int ww = 0; ww < RB_W; ++ww) {
                uint32_t t = cnt[ww][dg];
                cnt[ww][dg] = run;
                run += t;
            }
        }
        __syncthreads();
        // the tile sorted by digit, in shared memory
#pragma unroll
        for (int r = 0; r < RB_I; ++r) {
            int64_t i = seg0 + r * 32 + lane;
            bool ok = i < n;
            unsigned act = __ballot_sync(0xffffffffu, ok);
            if (ok) {
                int dg = (k[r] >> shift) & 0xff;
                unsigned peers = __match_any_sync(act, dg);
                uint32_t pos = cnt[warp][dg] + __popc(peers & lt_mask);
                k_s[pos] = k[r];
                v_s[pos] = v[r];
                __syncwarp(act);
                if (lane == __ffs(peers) - 1) cnt[warp][dg] += __popc(peers);
            }
            __syncwarp();
        }
        __syncthreads();
        // out, in tile order: each digit's run lands contiguously at its global position
        for (int p = threadIdx.x; p < tile_n; p += RB_T) {
            const uint16_t key = k_s[p];
            const uint32_t g = gshift[(key >> shift) & 0xff] + uint32_t(p);
            keys_out[g] = key;
            vals_out[g] = v_s[p];
        }
        __syncthreads();  // the next tile reuses the shared arrays
    }
}

// the scatter's dynamic shared memory is above the default 48 KB limit
static bool scatter_smem_ok() {
    return cudaFuncSetAttribute(k_radix_scatter, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                int(RB_SCATTER_SMEM)) == cudaSuccess;
}

// Grids of the histogram and scatter passes: as many CTAs as can be resident at once
// (they loop over the live tiles), never more than the tiles of the capacity.
static int radix_grid(int64_t cap, bool scatter) {
    static int per_sm[2] = {0, 0};
    int &k = per_sm[scatter ? 1 : 0];
    if (k == 0) {
        int b = 0;
        cudaError_t e = scatter ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_radix_scatter, RB_T,
                                                                                int(RB_SCATTER_SMEM))
                                : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_radix_hist, RB_T, 0);
        if (e != cudaSuccess) cudaGetLastError();
        k = std::max(1, b);
    }
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return int(std::max<int64_t>(1, std::min<int64_t>(ceil_div(cap, RB_TILE), int64_t(sms) * k)));
}

// offsets[k] = exclusive scan of counts[0..nkeys), offsets[nkeys] = live total.
__global__ void __launch_bounds__(1024) k_key_offsets(const int32_t *counts, int nkeys, int32_t *offsets) {
    // chunks of 1024 x 8 consecutive entries: each thread loads its eight at once (neighbouring
    // threads' spans are adjacent, so a warp reads 1 KB in one sweep), a warp-shuffle scan
    // and one over the 32 warps' sums give the offsets, a carry links the chunks
    constexpr int PER = 8, CHUNK = 1024 * PER;
    __shared__ int32_t wsum[32];
    __shared__ int32_t chunk_total;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    int32_t carry = 0;
    for (int base = 0; base < nkeys; base += CHUNK) {
        const int k0 = base + t * PER;
        int32_t v[PER], local = 0;
#pragma unroll
        for (int u = 0; u < PER; ++u) {
            v[u] = k0 + u < nkeys ? counts[k0 + u] : 0;
            local += v[u];
        }
        int32_t incl = local;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int32_t x = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += x;
        }
        if (lane == 31) wsum[warp] = incl;
        __syncthreads();
        if (warp == 0) {
            const int32_t ws = wsum[lane];
            int32_t wi = ws;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int32_t x = __shfl_up_sync(0xffffffffu, wi, o);
                if (lane >= o) wi += x;
            }
            wsum[lane] = wi - ws;  // the warps before this one
        }
        __syncthreads();
        int32_t run = carry + wsum[warp] + incl - local;
#pragma unroll
        for (int u = 0; u < PER; ++u) {
            if (k0 + u < nkeys) offsets[k0 + u] = run;
            run += v[u];
        }
        if (t == 1023) chunk_total = run;  // carry + the whole chunk
        __syncthreads();
        carry = chunk_total;
        __syncthreads();  // wsum and chunk_total are rewritten by the next chunk
    }
    if (t == 0) offsets[nkeys] = carry;
}

struct BinWs {
    size_t keys_a, keys_b, vals_a, hist, total;
    BinWs(int64_t cap) {
        size_t c = size_t(std::max<int64_t>(cap, 1));
        size_t nt = size_t(ceil_div(int64_t(c), RB_TILE));
        keys_a = 0;
        keys_b = keys_a + ((c * 2 + 255) & ~size_t(255));
        vals_a = keys_b + ((c * 2 + 255) & ~size_t(255));
        hist = vals_a + ((c * 4 + 255) & ~size_t(255));
        total = hist + (nt + 1) * RADIX * 4;  // the tiles' digit counts, then the digit totals
    }
};

template <typename T, typename P>
static int bin_entry(const bz_params *pp, P s, const int32_t *n, int64_t cap, int nb, const double *edges,
                     double min_wt, int32_t *perm, int32_t *offsets, int32_t *counts, int32_t *hw_counts, void *ws,
                     size_t ws_bytes, uint32_t *status, void *stream) {
    if (!pp || !n || cap <= 0 || !perm || !offsets || !counts || !hw_counts || !ws || !status) return BZ_ERR_ARG;
    if (!s.x || !s.vx || !s.vy || !s.vz || !s.w) return BZ_ERR_ARG;
    const bz_params &p = *pp;
    if (nb < 1 || nb > 16 || (nb > 1 && !edges) || p.n_nodes < 1 || (p.advect == BZ_ADVECT_1D && p.dx <= 0)) return BZ_ERR_ARG;
    const int nkeys = p.n_nodes * nb;
    if (nkeys >= 65535) return BZ_ERR_UNSUPPORTED;
    BinWs L(cap);
    if (ws_bytes < L.total) return BZ_ERR_WORKSPACE;
    unsigned char *b = static_cast<unsigned char *>(ws);
    uint16_t *keys_a = reinterpret_cast<uint16_t *>(b + L.keys_a);
    uint16_t *keys_b = reinterpret_cast<uint16_t *>(b + L.keys_b);
    uint32_t *vals_a = reinterpret_cast<uint32_t *>(b + L.vals_a);
    uint32_t *hist = reinterpret_cast<uint32_t *>(b + L.hist);
    uint32_t *dig_tot = hist + size_t(ceil_div(std::max<int64_t>(cap, 1), RB_TILE)) * RADIX;
    cudaStream_t st = as_stream(stream);
    const int grid = int(ceil_div(cap, RB_TILE));
    if (cudaMemsetAsync(counts, 0, sizeof(int32_t) * nkeys, st) != cudaSuccess) return BZ_ERR_CUDA;
    if (cudaMemsetAsync(hw_counts, 0, sizeof(int32_t) * nkeys, st) != cudaSuccess) return BZ_ERR_CUDA;
    size_t smem = sizeof(uint32_t) * (2 * size_t(nkeys) + RADIX);
    auto kk = k_bin_keys<T>;
    if (smem > 48 * 1024 &&
        cudaFuncSetAttribute(kk, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)) != cudaSuccess)
        return BZ_ERR_UNSUPPORTED;
    kk<<<grid, RB_T, smem, st>>>(p, s.x, s.vx, s.vy, s.vz, s.w, n, cap, nb, edges, min_wt, float_above(min_wt),
                                 float(1.0 / p.dx), keys_a, hist, counts, hw_counts,
                                 nkeys, status);
    const bool two = nkeys >= RADIX;  // invalid key = nkeys must be ordered too
    k_radix_colsum<<<RADIX, RS_COL_T, 0, st>>>(hist, n, cap, dig_tot);
    k_radix_colscan<<<RADIX, RS_COL_T, 0, st>>>(hist, n, cap, dig_tot);
    if (!scatter_smem_ok()) return BZ_ERR_UNSUPPORTED;
    k_radix_scatter<<<radix_grid(cap, true), RB_T, RB_SCATTER_SMEM, st>>>(keys_a, nullptr, n, cap, 0, hist, keys_b,
                                                         two ? vals_a : reinterpret_cast<uint32_t *>(perm));
    if (two) {
        k_radix_hist<<<radix_grid(cap, false), RB_T, 0, st>>>(keys_b, n, cap, 8, hist);
        k_radix_colsum<<<RADIX, RS_COL_T, 0, st>>>(hist, n, cap, dig_tot);
    k_radix_colscan<<<RADIX, RS_COL_T, 0, st>>>(hist, n, cap, dig_tot);
        k_radix_scatter<<<radix_grid(cap, true), RB_T, RB_SCATTER_SMEM, st>>>(keys_b, vals_a, n, cap, 8, hist, keys_a,
                                                             reinterpret_cast<uint32_t *>(perm));
    }
    k_key_offsets<<<1, 1024, 0, st>>>(counts, nkeys, offsets);
    return cudaGetLastError() == cudaSuccess ? BZ_OK : BZ_ERR_CUDA;
}

// ------------------------------------------------------------------------------------
// segmented state: keys are written densely (segment order, run 0 then run 1) together
// with each particle's slot, and the same radix passes sort the slots.
// ------------------------------------------------------------------------------------
__global__ void k_seg_totals(const int32_t *cnt, int nseg, int half, int32_t *tot) {
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nseg; s += gridDim.x * blockDim.x)
        tot[s] = min(max(cnt[2 * s], 0), half) + min(max(cnt[2 * s + 1], 0), half);
}

template <typename T>
__global__ void __launch_bounds__(256) k_seg_bin_keys(bz_params p, const T *x, const T *vx, const T *vy, const T *vz,
                                                      const T *w, const int32_t *cnt, int nseg, int half,
                                                      const int32_t *pre, int nb, const double *edges, double min_wt,
                                                      float wmin_f, float inv_dx_f, uint16_t *keys, uint32_t *slots,
                                                      int32_t *counts,
                                                      int32_t *hw_counts, int nkeys, uint32_t *status) {
    extern __shared__ __align__(16) unsigned char smem[];
    uint32_t *c_s = reinterpret_cast<uint32_t *>(smem);
    uint32_t *h_s = c_s + nkeys;
    __shared__ double edges_s[16];
    __shared__ float edges_f[16];
    for (int i = threadIdx.x; i < 2 * nkeys; i += blockDim.x) c_s[i] = 0;
    if (threadIdx.x < 16) {
        edges_s[threadIdx.x] = threadIdx.x < nb - 1 ? edges[threadIdx.x] : 0.0;
        edges_f[threadIdx.x] = float(edges_s[threadIdx.x]);
    }
    __syncthreads();
    const float efac_f = float(0.5 * m_e() * j_ev());
    const double efac_d = 0.5 * m_e() * j_ev();
    const int lane = threadIdx.x & 31;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    uint32_t err = 0;
    for (int seg = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; seg < nseg; seg += warps) {
        int64_t v0 = pre[seg];
        for (int run = 0; run < 2; ++run) {
            const int c = min(max(cnt[2 * seg + run], 0), half);
            const int64_t b = int64_t(seg) * 2 * half + int64_t(run) * half;
            // four rounds of 32 particles at a time, all five columns loaded together (the
            // loads do not wait on the weight test), then keyed in order
            for (int j0 = 0; j0 < c; j0 += 4 * 32) {
                T wv[4], xv[4], ux[4], uy[4], uz[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int j = j0 + u * 32 + lane;
                    const bool ok = j < c;
                    const int64_t i = b + j;
                    wv[u] = ok ? w[i] : T(0);
                    xv[u] = ok ? x[i] : T(0);
                    ux[u] = ok ? vx[i] : T(0);
                    uy[u] = ok ? vy[i] : T(0);
                    uz[u] = ok ? vz[i] : T(0);
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int j = j0 + u * 32 + lane;
                    if (j < c) {
                        int key = nkeys;
                        if (wv[u] > T(0)) {
                            int cell = bin_cell(p.advect, xv[u], p.dx, inv_dx_f);
                            int e = energy_bin(ux[u], uy[u], uz[u], wv[u], nb, edges_s, edges_f, efac_f, efac_d);
                            if (cell >= 0 && cell < p.n_nodes && e >= 0) {
                                key = cell * nb + e;
                                atomicAdd(&c_s[key], 1u);
                                if (above_min(wv[u], min_wt, wmin_f)) atomicAdd(&h_s[key], 1u);
                            } else {
                                err |= BZ_DEV_BINRANGE;
                            }
                        }
                        keys[v0 + j] = uint16_t(key);
                        slots[v0 + j] = uint32_t(b + j);
                    }
                }
            }
            v0 += c;
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < nkeys; k += blockDim.x) {
        if (c_s[k]) atomicAdd(reinterpret_cast<unsigned int *>(&counts[k]), c_s[k]);
        if (h_s[k]) atomicAdd(reinterpret_cast<unsigned int *>(&hw_counts[k]), h_s[k]);
    }
    if (err) atomicOr(status, err);
}

struct SegBinWs {
    size_t keys_a, keys_b, vals_a, slots, hist, tot, pre, total;
    SegBinWs(int nseg, int64_t cap) {
        auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
        size_t c = size_t(std::max<int64_t>(cap, 1));
        size_t nt = size_t(ceil_div(int64_t(c), RB_TILE));
        keys_a = 0;
        keys_b = keys_a + al(2 * c);
        vals_a = keys_b + al(2 * c);
        slots = vals_a + al(4 * c);
        hist = slots + al(4 * c);
        tot = hist + al((nt + 1) * RADIX * 4);  // the tiles' digit counts, then the digit totals
        pre = tot + al(4 * size_t(nseg));
        total = pre + al(4 * (size_t(nseg) + 2));  // the offsets, the live total, the count to sort
    }
};

// The resampling trigger from the key counts (the rule k_rs_decide applies), before the
// sort: n_sort gets the live total when resampling will run and 0 when it will not, so the
// radix passes that read it have nothing to do in a step whose check finds nothing.
__global__ void __launch_bounds__(1024) k_bin_need(const int32_t *counts, int nkeys, int nb, const int32_t *targets,
                                                   double split_below, double merge_at, int flags,
                                                   const int32_t *n_live, int32_t *n_sort, int32_t *need_out) {
    const bool per_key = (flags & BZ_PER_KEY_TARGETS) != 0;
    int need_any = 0, need_last = 0;
    for (int k = threadIdx.x; k < nkeys; k += blockDim.x) {
        const int b = k % nb;
        rs_key_need(counts[k], targets[per_key ? k : b], b == nb - 1, split_below, merge_at, need_any, need_last);
    }
    need_any = __syncthreads_or(need_any);
    need_last = __syncthreads_or(need_last);
    if (threadIdx.x == 0) {
        const int need = (flags & BZ_QUIRK_TRIGGER_LAST) ? need_last : need_any;
        *n_sort = need ? *n_live : 0;
        if (need_out) *need_out = need;
    }
}

// the trigger's inputs for a binning that sorts only when resampling will run
struct BinCheck {
    const int32_t *targets;
    double split_below, merge_at;
    int32_t *need_out;
};

template <typename T, typename S>
static int seg_bin_entry(const bz_params *pp, S s, int nb, const double *edges, double min_wt, int32_t *perm,
                         int32_t *offsets, int32_t *counts, int32_t *hw_counts, void *ws, size_t ws_bytes,
                         uint32_t *status, void *stream, const BinCheck *chk = nullptr) {
    if (!pp || !perm || !offsets || !counts || !hw_counts || !ws || !status) return BZ_ERR_ARG;
    if (!s.x || !s.vx || !s.vy || !s.vz || !s.w || !s.counts || s.nseg <= 0 || s.half <= 0) return BZ_ERR_ARG;
    if (chk && (!chk->targets || !(chk->merge_at > chk->split_below))) return BZ_ERR_ARG;
    const bz_params &p = *pp;
    if (nb < 1 || nb > 16 || (nb > 1 && !edges) || p.n_nodes < 1 || (p.advect == BZ_ADVECT_1D && p.dx <= 0)) return BZ_ERR_ARG;
    const int nkeys = p.n_nodes * nb;
    if (nkeys >= 65535) return BZ_ERR_UNSUPPORTED;
    const int64_t cap = int64_t(s.nseg) * 2 * s.half;
    if (cap > int64_t(UINT32_MAX)) return BZ_ERR_UNSUPPORTED;
    SegBinWs L(s.nseg, cap);
    if (ws_bytes < L.total) return BZ_ERR_WORKSPACE;
    unsigned char *b = static_cast<unsigned char *>(ws);
    uint16_t *keys_a = reinterpret_cast<uint16_t *>(b + L.keys_a);
    uint16_t *keys_b = reinterpret_cast<uint16_t *>(b + L.keys_b);
    uint32_t *vals_a = reinterpret_cast<uint32_t *>(b + L.vals_a);
    uint32_t *slots = reinterpret_cast<uint32_t *>(b + L.slots);
    uint32_t *hist = reinterpret_cast<uint32_t *>(b + L.hist);
    uint32_t *dig_tot = hist + size_t(ceil_div(std::max<int64_t>(cap, 1), RB_TILE)) * RADIX;
    int32_t *tot = reinterpret_cast<int32_t *>(b + L.tot);
    int32_t *pre = reinterpret_cast<int32_t *>(b + L.pre);
    cudaStream_t st = as_stream(stream);
    if (cudaMemsetAsync(counts, 0, sizeof(int32_t) * nkeys, st) != cudaSuccess) return BZ_ERR_CUDA;
    if (cudaMemsetAsync(hw_counts, 0, sizeof(int32_t) * nkeys, st) != cudaSuccess) return BZ_ERR_CUDA;
    k_seg_totals<<<int(std::min<int64_t>(ceil_div(s.nseg, 256), 4096)), 256, 0, st>>>(s.counts, s.nseg, s.half, tot);
    k_key_offsets<<<1, 1024, 0, st>>>(tot, s.nseg, pre);
    const int32_t *n = pre + s.nseg;  // live total on the device
    size_t smem = sizeof(uint32_t) * 2 * size_t(nkeys);
    auto kk = k_seg_bin_keys<T>;
    if (smem > 48 * 1024 &&
        cudaFuncSetAttribute(kk, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)) != cudaSuccess)
        return BZ_ERR_UNSUPPORTED;
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int kb = std::max(1, std::min(sms * 4, int(ceil_div(s.nseg, 8))));
    kk<<<kb, 256, smem, st>>>(p, s.x, s.vx, s.vy, s.vz, s.w, s.counts, s.nseg, s.half, pre, nb, edges, min_wt,
                              float_above(min_wt), float(1.0 / p.dx), keys_a,
                              slots, counts, hw_counts, nkeys, status);
    if (chk) {
        // the trigger first: the passes below sort nothing when it finds nothing to resample
        int32_t *n_sort = pre + s.nseg + 1;
        k_bin_need<<<1, 1024, 0, st>>>(counts, nkeys, nb, chk->targets, chk->split_below, chk->merge_at, p.flags, n,
                                       n_sort, chk->need_out);
        n = n_sort;
    }
    const bool two = nkeys >= RADIX;
    k_radix_hist<<<radix_grid(cap, false), RB_T, 0, st>>>(keys_a, n, cap, 0, hist);
    k_radix_colsum<<<RADIX, RS_COL_T, 0, st>>>(hist, n, cap, dig_tot);
    k_radix_colscan<<<RADIX, RS_COL_T, 0, st>>>(hist, n, cap, dig_tot);
    if (!scatter_smem_ok()) return BZ_ERR_UNSUPPORTED;
    k_radix_scatter<<<radix_grid(cap, true), RB_T, RB_SCATTER_SMEM, st>>>(keys_a, slots, n, cap, 0, hist, keys_b,
                                                         two ? vals_a : reinterpret_cast<uint32_t *>(perm));
    if (two) {
        k_radix_hist<<<radix_grid(cap, false), RB_T, 0, st>>>(keys_b, n, cap, 8, hist);
        k_radix_colsum<<<RADIX, RS_COL_T, 0, st>>>(hist, n, cap, dig_tot);
    k_radix_colscan<<<RADIX, RS_COL_T, 0, st>>>(hist, n, cap, dig_tot);
        k_radix_scatter<<<radix_grid(cap, true), RB_T, RB_SCATTER_SMEM, st>>>(keys_b, vals_a, n, cap, 8, hist, keys_a,
                                                             reinterpret_cast<uint32_t *>(perm));
    }
    k_key_offsets<<<1, 1024, 0, st>>>(counts, nkeys, offsets);
    return cudaGetLastError() == cudaSuccess ? BZ_OK : BZ_ERR_CUDA;
}

}  // namespace bz

extern "C" {
size_t bz_bin_workspace(int64_t capacity, int32_t nkeys) {
    (void)nkeys;
    return bz::BinWs(capacity).total;
}
int bz_bin_f32(const bz_params *p, bz_particles_f32 s, const int32_t *n, int64_t capacity, int32_t nbins,
               const double *edges, double min_wt, int32_t *perm, int32_t *offsets, int32_t *counts,
               int32_t *hw_counts, void *workspace, size_t workspace_bytes, uint32_t *status, void *stream) {
    return bz::bin_entry<float>(p, s, n, capacity, nbins, edges, min_wt, perm, offsets, counts, hw_counts, workspace,
                                workspace_bytes, status, stream);
}
size_t bz_seg_bin_workspace(int32_t nseg, int64_t capacity) { return bz::SegBinWs(nseg, capacity).total; }
int bz_seg_bin_f32(const bz_params *p, bz_segments_f32 s, int32_t nbins, const double *edges, double min_wt,
                   int32_t *perm, int32_t *offsets, int32_t *counts, int32_t *hw_counts, void *workspace,
                   size_t workspace_bytes, uint32_t *status, void *stream) {
    return bz::seg_bin_entry<float>(p, s, nbins, edges, min_wt, perm, offsets, counts, hw_counts, workspace,
                                    workspace_bytes, status, stream);
}
int bz_seg_bin_check_f32(const bz_params *p, bz_segments_f32 s, int32_t nbins, const double *edges, double min_wt,
                         int32_t *perm, int32_t *offsets, int32_t *counts, int32_t *hw_counts, const int32_t *targets,
                         double split_below, double merge_at, int32_t *need_out, void *workspace,
                         size_t workspace_bytes, uint32_t *status, void *stream) {
    const bz::BinCheck chk{targets, split_below, merge_at, need_out};
    return bz::seg_bin_entry<float>(p, s, nbins, edges, min_wt, perm, offsets, counts, hw_counts, workspace,
                                    workspace_bytes, status, stream, &chk);
}
int bz_seg_bin_check_f64(const bz_params *p, bz_segments_f64 s, int32_t nbins, const double *edges, double min_wt,
                         int32_t *perm, int32_t *offsets, int32_t *counts, int32_t *hw_counts, const int32_t *targets,
                         double split_below, double merge_at, int32_t *need_out, void *workspace,
                         size_t workspace_bytes, uint32_t *status, void *stream) {
    const bz::BinCheck chk{targets, split_below, merge_at, need_out};
    return bz::seg_bin_entry<double>(p, s, nbins, edges, min_wt, perm, offsets, counts, hw_counts, workspace,
                                     workspace_bytes, status, stream, &chk);
}
int bz_seg_bin_f64(const bz_params *p, bz_segments_f64 s, int32_t nbins, const double *edges, double min_wt,
                   int32_t *perm, int32_t *offsets, int32_t *counts, int32_t *hw_counts, void *workspace,
                   size_t workspace_bytes, uint32_t *status, void *stream) {
    return bz::seg_bin_entry<double>(p, s, nbins, edges, min_wt, perm, offsets, counts, hw_counts, workspace,
                                     workspace_bytes, status, stream);
}
int bz_bin_f64(const bz_params *p, bz_particles_f64 s, const int32_t *n, int64_t capacity, int32_t nbins,
               const double *edges, double min_wt, int32_t *perm, int32_t *offsets, int32_t *counts,
               int32_t *hw_counts, void *workspace, size_t workspace_bytes, uint32_t *status, void *stream) {
    return bz::bin_entry<double>(p, s, n, capacity, nbins, edges, min_wt, perm, offsets, counts, hw_counts, workspace,
                                 workspace_bytes, status, stream);
}
}
