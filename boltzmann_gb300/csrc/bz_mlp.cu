// Surrogate network of the learned CCP start-up: BF16 x BF16 -> FP32 tensor-core
// products, FP32 epilogues, FP32 master weights and Adam. The forward pass runs on
// tcgen05.mma with a TMEM accumulator (k_mlp_fwd_tc, the default) or on warp-level
// mma.sync m16n8k16 (k_mlp_fwd); the backward pass uses mma.sync.
//
// Network: BZ_MLP_IN (16) inputs -> 4 hidden layers of 128 GELU units -> BZ_MLP_OUT (80)
// linear outputs. Every weight matrix lives in shared memory for the whole kernel, rows
// padded by 8 BF16 (16 bytes) so that the fragment loads of a warp hit 32 different
// banks. A warp owns 16 rows of the batch; its activations stay in a per-warp shared
// tile between layers, so the forward pass reads x once and writes y (and, for
// training, the FP32 pre-activations) once.
//
// Fragment layout of mma.sync.m16n8k16.row.col (PTX ISA, "Matrix fragments for
// mma.m16n8k16"), g = lane/4, t = lane%4:
//   A (16x16, row-major): a0 = A[g][2t..2t+1], a1 = A[g+8][2t..], a2 = A[g][2t+8..],
//                         a3 = A[g+8][2t+8..]
//   B (16x8, k x n):      b0 = B[2t..2t+1][g], b1 = B[2t+8..2t+9][g]
//   C (16x8, FP32):       c0,c1 = C[g][2t..2t+1], c2,c3 = C[g+8][2t..2t+1]
// B[k][n] = W[n][k] for y = x W^T, so W stored row-major (out x in) gives B fragments as
// single 32-bit loads; the backward pass's dA = dZ W reads the transposed copy.
#include <cuda_bf16.h>

#include <algorithm>

#include "bz_common.cuh"

namespace bz {

constexpr int MLP_IN = BZ_MLP_IN;
constexpr int MLP_H = BZ_MLP_HIDDEN;
constexpr int MLP_OUT = BZ_MLP_OUT;
constexpr int MLP_NL = BZ_MLP_LAYERS;

__host__ __device__ constexpr int mlp_in(int l) { return l == 0 ? MLP_IN : MLP_H; }
__host__ __device__ constexpr int mlp_out(int l) { return l == MLP_NL - 1 ? MLP_OUT : MLP_H; }
__host__ __device__ constexpr int mlp_woff(int l) {
    return l == 0 ? 0 : mlp_woff(l - 1) + mlp_in(l - 1) * mlp_out(l - 1) + mlp_out(l - 1);
}
__host__ __device__ constexpr int mlp_boff(int l) { return mlp_woff(l) + mlp_in(l) * mlp_out(l); }
constexpr int MLP_NPARAM = mlp_woff(MLP_NL);
static_assert(MLP_NPARAM == BZ_MLP_NPARAM, "parameter count");
static_assert(MLP_IN % 16 == 0 && MLP_H % 16 == 0 && MLP_OUT % 16 == 0, "dimensions are whole k-steps");

// shared-memory copies: W_l as out_l rows of in_l + 8, W_l^T as in_l rows of out_l + 8
__host__ __device__ constexpr int ws_stride(int l) { return mlp_in(l) + 8; }
__host__ __device__ constexpr int ws_off(int l) { return l == 0 ? 0 : ws_off(l - 1) + mlp_out(l - 1) * ws_stride(l - 1); }
__host__ __device__ constexpr int wts_stride(int l) { return mlp_out(l) + 8; }
__host__ __device__ constexpr int wts_off(int l) {  // layers 1.. only (layer 0's input gradient is not needed)
    return l <= 1 ? 0 : wts_off(l - 1) + mlp_in(l - 1) * wts_stride(l - 1);
}
__host__ __device__ constexpr int bs_off(int l) { return l == 0 ? 0 : bs_off(l - 1) + mlp_out(l - 1); }
constexpr int WS_TOTAL = ws_off(MLP_NL);
constexpr int WTS_TOTAL = wts_off(MLP_NL);
constexpr int BS_TOTAL = bs_off(MLP_NL);
constexpr int AS = MLP_H + 8;  // row stride of a warp's activation tile (BF16)

constexpr int MF_WARPS = 8;    // forward: 8 warps, 128 rows per tile
constexpr int MB_WARPS = 4;    // backward: 4 warps, 64 rows per tile
constexpr int MB_ROWS = 16 * MB_WARPS;
constexpr int RS = MB_ROWS + 8;  // row stride of the transposed tiles (BF16)

constexpr size_t FWD_SMEM = size_t(WS_TOTAL) * 2 + size_t(BS_TOTAL) * 4 + size_t(MF_WARPS) * 16 * AS * 2;
constexpr size_t BWD_SMEM = size_t(WTS_TOTAL) * 2 + size_t(MB_WARPS) * 16 * AS * 2 + size_t(MLP_H) * RS * 2 * 2;
static_assert(FWD_SMEM <= 227 * 1024 && BWD_SMEM <= 227 * 1024, "shared memory");

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t *>(&v);
}
__device__ __forceinline__ float bf16_to_f(__nv_bfloat16 v) { return __bfloat162float(v); }

__device__ __forceinline__ void mma_bf16(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// GELU, tanh form (Hendrycks & Gimpel 2016): 0.5 z (1 + tanh(c (z + 0.044715 z^3))),
// c = sqrt(2/pi); and its derivative. tanh is the hardware approximation (tanh.approx.f32,
// relative error about 2^-11, below the BF16 rounding that every activation gets next).
constexpr float GELU_C = 0.7978845608028654f;
constexpr float GELU_A = 0.044715f;
__device__ __forceinline__ float tanh_hw(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float gelu(float z) {
    const float u = GELU_C * fmaf(GELU_A * z * z, z, z);
    return 0.5f * z * (1.0f + tanh_hw(u));
}
__device__ __forceinline__ float gelu_grad(float z) {
    const float u = GELU_C * fmaf(GELU_A * z * z, z, z);
    const float th = tanh_hw(u);
    return 0.5f * (1.0f + th) + 0.5f * z * (1.0f - th * th) * GELU_C * fmaf(3.0f * GELU_A, z * z, 1.0f);
}

// 16 rows x N outputs of one warp: acc = bias + A (16 x K, shared, stride AS) * W^T
// (W: N x K in shared memory, stride K + 8)
template <int K, int N>
__device__ __forceinline__ void warp_gemm_bias(const __nv_bfloat16 *A, const __nv_bfloat16 *W, const float *bias,
                                               int lane, float (&acc)[N / 8][4]) {
    constexpr int NT = N / 8;
    constexpr int WS32 = (K + 8) / 2;
    constexpr int AS32 = AS / 2;
    const int g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int nt = 0; nt < NT; ++nt) {
        const int c = nt * 8 + 2 * t;
        acc[nt][0] = bias ? bias[c] : 0.0f;
        acc[nt][1] = bias ? bias[c + 1] : 0.0f;
        acc[nt][2] = acc[nt][0];
        acc[nt][3] = acc[nt][1];
    }
    const uint32_t *A32 = reinterpret_cast<const uint32_t *>(A);
    const uint32_t *W32 = reinterpret_cast<const uint32_t *>(W);
#pragma unroll
    for (int k0 = 0; k0 < K; k0 += 16) {
        const int kc = k0 / 2 + t;
        const uint32_t a0 = A32[g * AS32 + kc], a1 = A32[(g + 8) * AS32 + kc];
        const uint32_t a2 = A32[g * AS32 + kc + 4], a3 = A32[(g + 8) * AS32 + kc + 4];
#pragma unroll
        for (int nt = 0; nt < NT; ++nt) {
            const int n = nt * 8 + g;
            mma_bf16(acc[nt], a0, a1, a2, a3, W32[n * WS32 + kc], W32[n * WS32 + kc + 4]);
        }
    }
}

// one forward layer of a warp: pre-activations (optionally saved), then GELU into the
// activation tile (hidden) or the output rows (last)
template <int L, bool SAVE>
__device__ __forceinline__ void fwd_layer(const __nv_bfloat16 *ws, const float *bs, __nv_bfloat16 *act, int lane,
                                          int row0, int n, float *z, float *y) {
    constexpr int K = mlp_in(L), N = mlp_out(L);
    float acc[N / 8][4];
    warp_gemm_bias<K, N>(act, ws + ws_off(L), bs + bs_off(L), lane, acc);
    __syncwarp();  // every lane has read the tile before it is overwritten
    const int g = lane >> 2, t = lane & 3;
    const int r0 = row0 + g, r1 = row0 + g + 8;
    uint32_t *act32 = reinterpret_cast<uint32_t *>(act);
#pragma unroll
    for (int nt = 0; nt < N / 8; ++nt) {
        const int c = nt * 8 + 2 * t;
        if (L == MLP_NL - 1) {
            if (r0 < n) *reinterpret_cast<float2 *>(y + size_t(r0) * MLP_OUT + c) = make_float2(acc[nt][0], acc[nt][1]);
            if (r1 < n) *reinterpret_cast<float2 *>(y + size_t(r1) * MLP_OUT + c) = make_float2(acc[nt][2], acc[nt][3]);
        } else {
            if (SAVE) {
                float *zl = z + size_t(L) * n * MLP_H;
                if (r0 < n) *reinterpret_cast<float2 *>(zl + size_t(r0) * MLP_H + c) = make_float2(acc[nt][0], acc[nt][1]);
                if (r1 < n) *reinterpret_cast<float2 *>(zl + size_t(r1) * MLP_H + c) = make_float2(acc[nt][2], acc[nt][3]);
            }
            act32[g * (AS / 2) + c / 2] = pack_bf16(gelu(acc[nt][0]), gelu(acc[nt][1]));
            act32[(g + 8) * (AS / 2) + c / 2] = pack_bf16(gelu(acc[nt][2]), gelu(acc[nt][3]));
        }
    }
    __syncwarp();
}

// x rows (gathered through idx) into a warp's tile as BF16; rows past n are zero
__device__ __forceinline__ void load_x_tile(const float *x, const int32_t *idx, int row0, int n, int lane,
                                            __nv_bfloat16 *act) {
    static_assert(MLP_IN == 16, "one row = two lanes of 8 features");
    const int rr = lane >> 1, half = lane & 1;
    const int r = row0 + rr;
    float4 a = make_float4(0.f, 0.f, 0.f, 0.f), b = a;
    if (r < n) {
        const int src = idx ? idx[r] : r;
        const float4 *p = reinterpret_cast<const float4 *>(x + size_t(src) * MLP_IN + half * 8);
        a = p[0];
        b = p[1];
    }
    uint4 q;
    q.x = pack_bf16(a.x, a.y);
    q.y = pack_bf16(a.z, a.w);
    q.z = pack_bf16(b.x, b.y);
    q.w = pack_bf16(b.z, b.w);
    *reinterpret_cast<uint4 *>(act + rr * AS + half * 8) = q;
}

// BF16 matrix rows x cols (row-major, global) into shared memory with a padded stride:
// 16-byte asynchronous copies (cp.async), all in flight at once; the caller waits
// (cp_async_wait_all) and synchronises the block before reading
__device__ __forceinline__ void cp_async16(void *smem_dst, const void *gsrc) {
    const uint32_t d = static_cast<uint32_t>(__cvta_generic_to_shared(smem_dst));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
}
__device__ __forceinline__ void copy_padded(const uint16_t *src, int rows, int cols, __nv_bfloat16 *dst, int stride) {
    const int chunks = cols / 8;
    for (int e = threadIdx.x; e < rows * chunks; e += blockDim.x) {
        const int r = e / chunks, c = e - r * chunks;
        cp_async16(dst + r * stride + c * 8, src + size_t(r) * cols + c * 8);
    }
}

template <bool SAVE>
__global__ void __launch_bounds__(32 * MF_WARPS, 1)
    k_mlp_fwd(const uint16_t *wb, const float *prm, const float *x, const int32_t *idx, int n, float *y, float *z) {
    extern __shared__ __align__(16) unsigned char smem[];
    __nv_bfloat16 *ws = reinterpret_cast<__nv_bfloat16 *>(smem);
    float *bs = reinterpret_cast<float *>(smem + size_t(WS_TOTAL) * 2);
    __nv_bfloat16 *acts = reinterpret_cast<__nv_bfloat16 *>(smem + size_t(WS_TOTAL) * 2 + size_t(BS_TOTAL) * 4);
#pragma unroll
    for (int l = 0; l < MLP_NL; ++l) {
        copy_padded(wb + mlp_woff(l), mlp_out(l), mlp_in(l), ws + ws_off(l), ws_stride(l));
        for (int i = threadIdx.x; i < mlp_out(l); i += blockDim.x) bs[bs_off(l) + i] = prm[mlp_boff(l) + i];
    }
    cp_async_wait_all();
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __nv_bfloat16 *act = acts + warp * 16 * AS;
    const int tiles = int(ceil_div(n, 16 * MF_WARPS));
    for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const int row0 = tile * 16 * MF_WARPS + warp * 16;
        if (row0 >= n) continue;  // warp-uniform; no block barrier below
        load_x_tile(x, idx, row0, n, lane, act);
        __syncwarp();
        fwd_layer<0, SAVE>(ws, bs, act, lane, row0, n, z, y);
        fwd_layer<1, SAVE>(ws, bs, act, lane, row0, n, z, y);
        fwd_layer<2, SAVE>(ws, bs, act, lane, row0, n, z, y);
        fwd_layer<3, SAVE>(ws, bs, act, lane, row0, n, z, y);
        fwd_layer<4, SAVE>(ws, bs, act, lane, row0, n, z, y);
    }
}

// ------------------------------------------------------------------------------------
// forward on the 5th-generation tensor cores (tcgen05): one CTA of 4 warps per tile of 128
// rows. The weights sit in shared memory in the canonical K-major layout without swizzle
// (8-row x 16-byte core matrices; element (r, k) at (r/8)*SBO + (k/8)*128 + (r%8)*16 +
// (k%8)*2 bytes, SBO = 16*K), the tile's activations likewise; one thread issues the
// layer's K/16 tcgen05.mma (M = 128, N = 128 or 80, BF16 x BF16 -> FP32) into a
// 128-column TMEM accumulator and commits them to an mbarrier; every warp then reads its
// 32 TMEM lanes (= its 32 rows) with tcgen05.ld, adds the bias, applies GELU and writes the
// next layer's operand back to shared memory (or the output rows). Waits are bounded: on
// a timeout the kernel raises a status bit and stops.
// ------------------------------------------------------------------------------------
constexpr int TC_ROWS = 128;
constexpr int TC_THREADS = 256;  // backward: warps w and w+4 share TMEM lanes 32*(w%4).. and split the columns
// forward: 16 warps, four per TMEM lane quarter (warps w, w+4, w+8, w+12 read lanes 32*(w%4)..
// and take a quarter of the 16-column chunks each): the epilogue, not the tensor core, sets
// the forward's time, so it gets four warps per row block
constexpr int TCF_THREADS = 512;
constexpr int TCF_GROUPS = TCF_THREADS / TC_ROWS;
constexpr uint32_t TC_WAIT_LIMIT = 1u << 24;
__host__ __device__ constexpr int wc_off(int l) { return l == 0 ? 0 : wc_off(l - 1) + mlp_out(l - 1) * mlp_in(l - 1) * 2; }
constexpr int WC_BYTES = wc_off(MLP_NL);
constexpr int TC_ACT_BYTES = TC_ROWS * MLP_H * 2;
constexpr size_t TC_SMEM = 1024 + size_t(WC_BYTES) + TC_ACT_BYTES + BS_TOTAL * 4 + 64;
static_assert(TC_SMEM <= 227 * 1024, "shared memory");
static_assert(TC_THREADS == 2 * TC_ROWS && TCF_THREADS >= 2 * TC_ROWS && MLP_IN == 16,
              "two threads per row: the 16 inputs as two 16-byte chunks");

__device__ uint32_t g_mlp_status = 0;

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return uint32_t(__cvta_generic_to_shared(p)); }
// shared-memory matrix descriptor: start address, leading (K-direction) and stride
// (8-row direction) byte offsets, descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return uint64_t((saddr & 0x3FFFFu) >> 4) | (uint64_t(lbo >> 4) << 16) | (uint64_t(sbo >> 4) << 32) |
           (1ull << 46);
}
// instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both K-major
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(N >> 3) << 17) | (uint32_t(M >> 4) << 24);
}
__device__ __forceinline__ void tc_mma(uint32_t tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}
__device__ __forceinline__ void tc_commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
                 : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t phase, uint32_t limit) {
    for (uint32_t it = 0; it < limit; ++it) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(mbar), "r"(phase)
            : "memory");
        if (done) return true;
    }
    return false;
}
// 16 consecutive FP32 accumulator columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// byte offset of the 16-byte chunk (row r, k = 8*c8 .. 8*c8+7) in the canonical layout of a
// matrix with K columns
__device__ __forceinline__ int canon_off(int r, int c8, int K) { return (r >> 3) * (16 * K) + c8 * 128 + (r & 7) * 16; }

template <int L, bool SAVE>
__device__ __forceinline__ bool tc_layer(unsigned char *wc, unsigned char *act, const float *bs, uint32_t tmem,
                                         uint32_t mbar, uint32_t &phase, uint32_t wl, int row0, int n, float *z, float *y) {
    constexpr int K = mlp_in(L), N = mlp_out(L);
    const int tid = threadIdx.x, warp = tid >> 5;
    // every thread's operand writes are complete and visible to the tensor core
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    if (tid == 0) {
        tc_fence_after();
        const uint32_t a0 = smem_u32(act), b0 = smem_u32(wc + wc_off(L));
        constexpr uint32_t idesc = idesc_bf16(TC_ROWS, N);
#pragma unroll
        for (int kk = 0; kk < K / 16; ++kk)
            tc_mma(tmem, umma_desc(a0 + kk * 256, 128, 16 * K), umma_desc(b0 + kk * 256, 128, 16 * K), idesc,
                   kk > 0 ? 1u : 0u);
        tc_commit(mbar);
    }
    // one decision for the whole block (every thread reaches this barrier)
    const bool ok = __syncthreads_and(mbar_wait(mbar, phase, wl)) != 0;
    phase ^= 1u;
    if (!ok) return false;
    tc_fence_after();
    // epilogue: this thread owns row 32*(warp%4) + lane (its TMEM lane) and a quarter of the
    // 16-column chunks (warps 0-3 the first, 4-7 the second, ...)
    constexpr int NCH = N / 16, HALF = (NCH + TCF_GROUPS - 1) / TCF_GROUPS;  // chunks per warp group
    const int lo = min(NCH, (warp >> 2) * HALF), hi = min(NCH, lo + HALF);
    const int rl = 32 * (warp & 3) + (tid & 31);
    const uint32_t tl = tmem + (uint32_t(32 * (warp & 3)) << 16);
    const int r = row0 + rl;
    const float *b = bs + bs_off(L);
    // one 16-column chunk at a time: 16 accumulators live
#pragma unroll
    for (int j = 0; j < HALF; ++j) {
        if (lo + j >= hi) break;
        const int c0 = (lo + j) * 16;
        float v[16];
        tmem_ld16(tl + uint32_t(c0), v);
        tmem_wait_ld();
#pragma unroll
        for (int c = 0; c < 16; ++c) v[c] += b[c0 + c];
        if (L == MLP_NL - 1) {
            if (r < n) {
                float4 *yr = reinterpret_cast<float4 *>(y + size_t(r) * MLP_OUT + c0);
#pragma unroll
                for (int c = 0; c < 16; c += 4) yr[c / 4] = make_float4(v[c], v[c + 1], v[c + 2], v[c + 3]);
            }
        } else {
            if (SAVE && r < n) {
                float4 *zr = reinterpret_cast<float4 *>(z + (size_t(L) * n + r) * MLP_H + c0);
#pragma unroll
                for (int c = 0; c < 16; c += 4) zr[c / 4] = make_float4(v[c], v[c + 1], v[c + 2], v[c + 3]);
            }
            // the next layer's A operand (K = 128): two 16-byte chunks of 8 activations
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const float *a = v + 8 * h;
                uint4 q;
                q.x = pack_bf16(gelu(a[0]), gelu(a[1]));
                q.y = pack_bf16(gelu(a[2]), gelu(a[3]));
                q.z = pack_bf16(gelu(a[4]), gelu(a[5]));
                q.w = pack_bf16(gelu(a[6]), gelu(a[7]));
                *reinterpret_cast<uint4 *>(act + canon_off(rl, c0 / 8 + h, MLP_H)) = q;
            }
        }
    }
    return true;
}

template <bool SAVE>
__global__ void __launch_bounds__(TCF_THREADS, 1)
    k_mlp_fwd_tc(const uint16_t *wb, const float *prm, const float *x, const int32_t *idx, int n, float *y, float *z,
                 uint32_t wl) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    // 1024-byte aligned operand region
    unsigned char *base = smem_raw + ((1024 - (smem_u32(smem_raw) & 1023u)) & 1023u);
    unsigned char *wc = base;
    unsigned char *act = wc + WC_BYTES;
    float *bs = reinterpret_cast<float *>(act + TC_ACT_BYTES);
    uint64_t *mbar_p = reinterpret_cast<uint64_t *>(bs + BS_TOTAL + (BS_TOTAL & 1));
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(mbar_p + 1);
    const int tid = threadIdx.x, warp = tid >> 5;
    // weights into the canonical layout (asynchronous 16-byte copies), biases
#pragma unroll
    for (int l = 0; l < MLP_NL; ++l) {
        const int K = mlp_in(l), N = mlp_out(l), chunks = K / 8;
        for (int e = tid; e < N * chunks; e += TCF_THREADS) {
            const int r = e / chunks, c8 = e - r * chunks;
            cp_async16(wc + wc_off(l) + canon_off(r, c8, K), wb + mlp_woff(l) + size_t(r) * K + c8 * 8);
        }
        for (int i = tid; i < N; i += TCF_THREADS) bs[bs_off(l) + i] = prm[mlp_boff(l) + i];
    }
    const uint32_t mbar = smem_u32(mbar_p);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 128;" ::"r"(smem_u32(tmem_slot))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    cp_async_wait_all();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    uint32_t phase = 0;
    bool ok = true;
    const int tiles = int(ceil_div(n, TC_ROWS));
    for (int tile = blockIdx.x; tile < tiles && ok; tile += gridDim.x) {
        const int row0 = tile * TC_ROWS;
        // the tile's inputs (K = 16): one 16-byte chunk (8 features) per thread of the first 256
        if (tid < 2 * TC_ROWS) {
            const int rl = tid & (TC_ROWS - 1), c8 = tid / TC_ROWS;
            const int r = row0 + rl;
            float4 q0 = make_float4(0.f, 0.f, 0.f, 0.f), q1 = q0;
            if (r < n) {
                const float4 *p = reinterpret_cast<const float4 *>(x + size_t(idx ? idx[r] : r) * MLP_IN + 8 * c8);
                q0 = p[0];
                q1 = p[1];
            }
            uint4 u;
            u.x = pack_bf16(q0.x, q0.y);
            u.y = pack_bf16(q0.z, q0.w);
            u.z = pack_bf16(q1.x, q1.y);
            u.w = pack_bf16(q1.z, q1.w);
            *reinterpret_cast<uint4 *>(act + canon_off(rl, c8, MLP_IN)) = u;
        }
        ok = tc_layer<0, SAVE>(wc, act, bs, tmem, mbar, phase, wl, row0, n, z, y) &&
             tc_layer<1, SAVE>(wc, act, bs, tmem, mbar, phase, wl, row0, n, z, y) &&
             tc_layer<2, SAVE>(wc, act, bs, tmem, mbar, phase, wl, row0, n, z, y) &&
             tc_layer<3, SAVE>(wc, act, bs, tmem, mbar, phase, wl, row0, n, z, y) &&
             tc_layer<4, SAVE>(wc, act, bs, tmem, mbar, phase, wl, row0, n, z, y);
        // every TMEM read and shared write of this tile is done before the next one
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
    }
    if (!ok && tid == 0) atomicOr(&g_mlp_status, BZ_DEV_LOOKBACK);
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 128;" ::"r"(tmem) : "memory");
}

// ------------------------------------------------------------------------------------
// backward. Per tile of 64 rows, from the output layer down:
//   dZ_4 = wcol (y - t) / n;   for l = 4..0:
//     dW_l += dZ_l^T A_{l-1}   (A_{-1} = x; the CTA's 64 rows are the k dimension)
//     db_l += column sums of dZ_l
//     dZ_{l-1} = (dZ_l W_l) * gelu'(z_{l-1})   (l >= 1)
// dZ is kept as BF16 twice: row-major per warp (A operand of dZ W) and transposed for the
// whole tile (A operand of dZ^T A); A_{l-1} is rebuilt from the saved z as BF16, transposed
// (B operand). Partial dW, db of a tile are added to grad with FP32 atomics.
// ------------------------------------------------------------------------------------
struct BwdSmem {
    __nv_bfloat16 *wt, *dz, *dzT, *aT;
};

// dW_l += dZ^T (out x 64) * A (64 x in), partial over the tile, added to grad
template <int L>
__device__ __forceinline__ void bwd_weight_grad(const BwdSmem &s, int warp, int lane, float *grad) {
    constexpr int NO = mlp_out(L), NI = mlp_in(L);
    constexpr int MT = NO / 16, NT = NI / 8;
    constexpr int NCH = NT < 8 ? NT : 8;  // n-tiles per pass (8 x 4 accumulators)
    const int g = lane >> 2, t = lane & 3;
    const uint32_t *D32 = reinterpret_cast<const uint32_t *>(s.dzT);
    const uint32_t *X32 = reinterpret_cast<const uint32_t *>(s.aT);
    constexpr int RS32 = RS / 2;
    for (int m = warp; m < MT; m += MB_WARPS) {
#pragma unroll
        for (int n0 = 0; n0 < NT; n0 += NCH) {
            float acc[NCH][4];
#pragma unroll
            for (int j = 0; j < NCH; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
#pragma unroll
            for (int k0 = 0; k0 < MB_ROWS; k0 += 16) {
                const int kc = k0 / 2 + t;
                const int o = m * 16 + g;
                const uint32_t a0 = D32[o * RS32 + kc], a1 = D32[(o + 8) * RS32 + kc];
                const uint32_t a2 = D32[o * RS32 + kc + 4], a3 = D32[(o + 8) * RS32 + kc + 4];
#pragma unroll
                for (int j = 0; j < NCH; ++j) {
                    const int i = (n0 + j) * 8 + g;
                    mma_bf16(acc[j], a0, a1, a2, a3, X32[i * RS32 + kc], X32[i * RS32 + kc + 4]);
                }
            }
            float *gw = grad + mlp_woff(L);
#pragma unroll
            for (int j = 0; j < NCH; ++j) {
                const int i = (n0 + j) * 8 + 2 * t;
                const int o = m * 16 + g;
                atomicAdd(gw + o * NI + i, acc[j][0]);
                atomicAdd(gw + o * NI + i + 1, acc[j][1]);
                atomicAdd(gw + (o + 8) * NI + i, acc[j][2]);
                atomicAdd(gw + (o + 8) * NI + i + 1, acc[j][3]);
            }
        }
    }
    // db_l: column sums of dZ over the tile's rows
    for (int o = threadIdx.x; o < NO; o += blockDim.x) {
        float sum = 0.f;
        for (int r = 0; r < MB_ROWS; ++r) sum += bf16_to_f(s.dzT[o * RS + r]);
        if (sum != 0.f) atomicAdd(grad + mlp_boff(L) + o, sum);
    }
}

// the transposed BF16 activations A_{L-1} of the tile (B operand of the weight gradient):
// four consecutive features per thread and item, four items in flight per thread
template <int L>
__device__ __forceinline__ void bwd_build_aT(const BwdSmem &s, const float *x, const int32_t *idx, const float *z,
                                             int n, int tile_row0) {
    constexpr int NI = mlp_in(L), NI4 = NI / 4, TOT = MB_ROWS * NI4, U = 4;
    for (int e0 = threadIdx.x; e0 < TOT; e0 += U * blockDim.x) {
        float4 v[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int e = e0 + u * blockDim.x;
            const int rr = e / NI4, i4 = e - rr * NI4;
            const int r = tile_row0 + rr;
            v[u] = make_float4(0.f, 0.f, 0.f, 0.f);
            if (e < TOT && r < n) {
                const float *src = (L == 0) ? x + size_t(idx ? idx[r] : r) * MLP_IN + 4 * i4
                                            : z + (size_t(L > 0 ? L - 1 : 0) * n + r) * MLP_H + 4 * i4;
                v[u] = *reinterpret_cast<const float4 *>(src);
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int e = e0 + u * blockDim.x;
            if (e >= TOT) break;
            const int rr = e / NI4, i4 = e - rr * NI4;
            const bool ok = tile_row0 + rr < n;
            float a0 = v[u].x, a1 = v[u].y, a2 = v[u].z, a3 = v[u].w;
            if (L > 0 && ok) { a0 = gelu(a0); a1 = gelu(a1); a2 = gelu(a2); a3 = gelu(a3); }
            s.aT[(4 * i4 + 0) * RS + rr] = __float2bfloat16_rn(a0);
            s.aT[(4 * i4 + 1) * RS + rr] = __float2bfloat16_rn(a1);
            s.aT[(4 * i4 + 2) * RS + rr] = __float2bfloat16_rn(a2);
            s.aT[(4 * i4 + 3) * RS + rr] = __float2bfloat16_rn(a3);
        }
    }
}

// store one warp's dZ values (accumulator layout) row-major and transposed
__device__ __forceinline__ void put_dz(const BwdSmem &s, int warp, int lane, int c, float d00, float d01, float d10,
                                       float d11) {
    const int g = lane >> 2;
    uint32_t *dz32 = reinterpret_cast<uint32_t *>(s.dz + warp * 16 * AS);
    const uint32_t p0 = pack_bf16(d00, d01), p1 = pack_bf16(d10, d11);
    dz32[g * (AS / 2) + c / 2] = p0;
    dz32[(g + 8) * (AS / 2) + c / 2] = p1;
    const __nv_bfloat162 q0 = *reinterpret_cast<const __nv_bfloat162 *>(&p0);
    const __nv_bfloat162 q1 = *reinterpret_cast<const __nv_bfloat162 *>(&p1);
    const int rl = warp * 16 + g;
    s.dzT[c * RS + rl] = q0.x;
    s.dzT[(c + 1) * RS + rl] = q0.y;
    s.dzT[c * RS + rl + 8] = q1.x;
    s.dzT[(c + 1) * RS + rl + 8] = q1.y;
}

// dZ_{L-1} = (dZ_L W_L) * gelu'(z_{L-1}) for one warp's 16 rows
template <int L>
__device__ __forceinline__ void bwd_input_grad(const BwdSmem &s, int warp, int lane, const float *z, int n,
                                               int row0) {
    constexpr int NO = mlp_out(L), NI = mlp_in(L);
    float acc[NI / 8][4];
    warp_gemm_bias<NO, NI>(s.dz + warp * 16 * AS, s.wt + wts_off(L), nullptr, lane, acc);
    __syncthreads();  // the whole tile is done with dZ_L (weight gradient, this product)
    const int g = lane >> 2, t = lane & 3;
    const int r0 = row0 + g, r1 = row0 + g + 8;
    const float *zl = z + size_t(L - 1) * n * MLP_H;
#pragma unroll
    for (int nt = 0; nt < NI / 8; ++nt) {
        const int c = nt * 8 + 2 * t;
        float2 z0 = make_float2(0.f, 0.f), z1 = z0;
        const bool ok0 = r0 < n, ok1 = r1 < n;
        if (ok0) z0 = *reinterpret_cast<const float2 *>(zl + size_t(r0) * MLP_H + c);
        if (ok1) z1 = *reinterpret_cast<const float2 *>(zl + size_t(r1) * MLP_H + c);
        put_dz(s, warp, lane, c, ok0 ? acc[nt][0] * gelu_grad(z0.x) : 0.f, ok0 ? acc[nt][1] * gelu_grad(z0.y) : 0.f,
               ok1 ? acc[nt][2] * gelu_grad(z1.x) : 0.f, ok1 ? acc[nt][3] * gelu_grad(z1.y) : 0.f);
    }
}

template <int L>
__device__ __forceinline__ void bwd_layer(const BwdSmem &s, int warp, int lane, const float *x, const int32_t *idx,
                                          const float *z, int n, int tile_row0, float *grad) {
    bwd_build_aT<L>(s, x, idx, z, n, tile_row0);
    __syncthreads();  // aT and dzT of the tile are complete
    bwd_weight_grad<L>(s, warp, lane, grad);
    if constexpr (L > 0) bwd_input_grad<L>(s, warp, lane, z, n, tile_row0 + warp * 16);
    __syncthreads();  // dZ_{L-1} complete; aT free again
}

__global__ void __launch_bounds__(32 * MB_WARPS, 1)
    k_mlp_bwd(const uint16_t *wt, const float *x, const float *tg, const float *wcol, const int32_t *idx, int n,
              const float *y, const float *z, float *grad, float *loss) {
    extern __shared__ __align__(16) unsigned char smem[];
    BwdSmem s;
    s.wt = reinterpret_cast<__nv_bfloat16 *>(smem);
    s.dz = s.wt + WTS_TOTAL;
    s.dzT = s.dz + MB_WARPS * 16 * AS;
    s.aT = s.dzT + MLP_H * RS;
#pragma unroll
    for (int l = 1; l < MLP_NL; ++l)
        copy_padded(wt + mlp_woff(l), mlp_in(l), mlp_out(l), s.wt + wts_off(l), wts_stride(l));
    for (int i = threadIdx.x; i < MLP_H * RS; i += blockDim.x) s.dzT[i] = __float2bfloat16_rn(0.f);
    cp_async_wait_all();
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int g = lane >> 2, t = lane & 3;
    const float inv_n = 1.0f / float(n);
    float lsum = 0.f;
    const int tiles = int(ceil_div(n, MB_ROWS));
    for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const int tile_row0 = tile * MB_ROWS;
        const int row0 = tile_row0 + warp * 16;
        // dZ_4 = wcol (y - t) / n, and the loss
        for (int nt = 0; nt < MLP_OUT / 8; ++nt) {
            const int c = nt * 8 + 2 * t;
            float d[4];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int r = row0 + g + 8 * h;
                float e0 = 0.f, e1 = 0.f;
                if (r < n) {
                    const float *tr = tg + size_t(idx ? idx[r] : r) * MLP_OUT;
                    e0 = (y[size_t(r) * MLP_OUT + c] - tr[c]) * wcol[c];
                    e1 = (y[size_t(r) * MLP_OUT + c + 1] - tr[c + 1]) * wcol[c + 1];
                    lsum += 0.5f * (e0 * (y[size_t(r) * MLP_OUT + c] - tr[c]) +
                                    e1 * (y[size_t(r) * MLP_OUT + c + 1] - tr[c + 1]));
                }
                d[2 * h] = e0 * inv_n;
                d[2 * h + 1] = e1 * inv_n;
            }
            put_dz(s, warp, lane, c, d[0], d[1], d[2], d[3]);
        }
        bwd_layer<4>(s, warp, lane, x, idx, z, n, tile_row0, grad);
        bwd_layer<3>(s, warp, lane, x, idx, z, n, tile_row0, grad);
        bwd_layer<2>(s, warp, lane, x, idx, z, n, tile_row0, grad);
        bwd_layer<1>(s, warp, lane, x, idx, z, n, tile_row0, grad);
        bwd_layer<0>(s, warp, lane, x, idx, z, n, tile_row0, grad);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
    if (lane == 0 && lsum != 0.f) atomicAdd(loss, lsum * inv_n);
}

// ------------------------------------------------------------------------------------
// backward on tcgen05: one CTA of 8 warps per tile of 128 rows, from the output layer down.
// Per layer l two products into TMEM (one thread issues both, one commit):
//   dW_l | db_l = dZ_l^T [A_{l-1} | 1]   M = 128 (out_l rows, zero-padded), N = in_l + 16,
//                                         K = the tile's 128 rows; column in_l of the
//                                         accumulator is the bias gradient
//   dA_{l-1}    = dZ_l W_l               M = 128 rows, N = in_l, K = out_l   (l >= 1)
// Operands in shared memory in the canonical K-major layout: dZ row-major and transposed,
// [A_{l-1} | 1] transposed (rebuilt from the saved pre-activations), W_l^T (all layers,
// staged once). dZ_{l-1} = dA_{l-1} gelu'(z_{l-1}) stays in the registers of the thread that
// owns the row. The tile's dW, db go to the CTA's own FP32 slice of a partial buffer (no
// atomics: the sum over slices is taken afterwards, in a fixed order).
// ------------------------------------------------------------------------------------
__host__ __device__ constexpr int wtc_off(int l) {  // W_l^T, layers 1..
    return l <= 1 ? 0 : wtc_off(l - 1) + mlp_in(l - 1) * mlp_out(l - 1) * 2;
}
constexpr int WTC_BYTES = wtc_off(MLP_NL);
constexpr int TB_DZ = TC_ROWS * MLP_H * 2;          // dZ, rows x out (K = out)
constexpr int TB_DZT = 128 * TC_ROWS * 2;           // dZ^T, out (padded to 128) x rows
constexpr int TB_AT = (MLP_H + 16) * TC_ROWS * 2;   // [A | 1]^T, (in + 16) x rows
constexpr size_t TCB_SMEM = 1024 + size_t(WTC_BYTES) + TB_DZ + TB_DZT + TB_AT + 64;
static_assert(TCB_SMEM <= 227 * 1024, "shared memory");
constexpr uint32_t TCB_COL_DA = 256;  // TMEM column of the dA accumulator (dW | db at 0)

// bf16 of v at (row r, column k) of a canonical K-major matrix with K columns
__device__ __forceinline__ void put_canon(unsigned char *base, int r, int k, int K, float v) {
    *reinterpret_cast<__nv_bfloat16 *>(base + (r >> 3) * (16 * K) + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2) =
        __float2bfloat16_rn(v);
}

// Transposed writes in pairs: lanes 2m and 2m+1 hold rows r and r+1 (adjacent in the
// transposed matrix's K), so for the columns c, c+1 one shuffle lets the even lane write
// (row c: r, r+1) and the odd lane (row c+1: r, r+1) as one 32-bit word each
__device__ __forceinline__ void put_canon_t2(unsigned char *base, int rl, int c, int K, float vc, float vc1) {
    const bool odd = rl & 1;
    const float recv = __shfl_xor_sync(0xffffffffu, odd ? vc : vc1, 1);
    const int row = odd ? c + 1 : c, k = rl & ~1;
    const uint32_t w = odd ? pack_bf16(recv, vc1) : pack_bf16(vc, recv);
    *reinterpret_cast<uint32_t *>(base + (row >> 3) * (16 * K) + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2) = w;
}

// 16 values (columns c0 .. c0+15 of row rl) as two 16-byte chunks of a canonical K-major
// matrix with C columns
__device__ __forceinline__ void put_row16(unsigned char *base, int rl, int c0, int C, const float *v) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const float *a = v + 8 * h;
        uint4 q;
        q.x = pack_bf16(a[0], a[1]);
        q.y = pack_bf16(a[2], a[3]);
        q.z = pack_bf16(a[4], a[5]);
        q.w = pack_bf16(a[6], a[7]);
        *reinterpret_cast<uint4 *>(base + canon_off(rl, c0 / 8 + h, C)) = q;
    }
}

// [A_{L-1} | 1]^T of the tile: this thread's row (a column of the operand), its half of
// the inputs
template <int L>
__device__ __forceinline__ void tcb_put_at(unsigned char *at, int rl, int half, int row0, int n, const float *x,
                                           const int32_t *idx, const float *z) {
    constexpr int NI = mlp_in(L);
    const int r = row0 + rl;
    const float *src = nullptr;
    if (r < n) src = (L == 0) ? x + size_t(idx ? idx[r] : r) * MLP_IN : z + (size_t(L > 0 ? L - 1 : 0) * n + r) * MLP_H;
    const int c_lo = half * (NI / 2);
#pragma unroll
    for (int c = 0; c < NI / 2; c += 4) {
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (src) {
            v = *reinterpret_cast<const float4 *>(src + c_lo + c);
            if (L > 0) { v.x = gelu(v.x); v.y = gelu(v.y); v.z = gelu(v.z); v.w = gelu(v.w); }
        }
        put_canon_t2(at, rl, c_lo + c + 0, TC_ROWS, v.x, v.y);
        put_canon_t2(at, rl, c_lo + c + 2, TC_ROWS, v.z, v.w);
    }
    if (half) {  // the ones row (bias gradient) and 15 zero rows
#pragma unroll
        for (int j = 0; j < 16; j += 2) put_canon_t2(at, rl, NI + j, TC_ROWS, (j == 0 && r < n) ? 1.f : 0.f, 0.f);
    }
}

template <int L>
__device__ __forceinline__ bool tcb_layer(unsigned char *wtc, unsigned char *dz, unsigned char *dzt,
                                          unsigned char *at, uint32_t tmem, uint32_t mbar, uint32_t &phase, uint32_t wl,
                                          int row0, int n, const float *x, const int32_t *idx, const float *z,
                                          float *part, bool first, float (&d)[64]) {
    constexpr int NO = mlp_out(L), NI = mlp_in(L);
    const int tid = threadIdx.x, warp = tid >> 5, half = warp >> 2;
    const int rl = 32 * (warp & 3) + (tid & 31);
    // operands: dZ_L (from d: this half's 16-column chunks) row-major and transposed
    {
        constexpr int NCH = NO / 16, H0 = (NCH + 1) / 2;
        const int lo = half ? H0 : 0, hi = half ? NCH : H0;
#pragma unroll
        for (int j = 0; j < H0; ++j) {
            if (lo + j < hi) {
                const int c0 = (lo + j) * 16;
                put_row16(dz, rl, c0, NO, d + 16 * j);
#pragma unroll
                for (int c = 0; c < 16; c += 2) put_canon_t2(dzt, rl, c0 + c, TC_ROWS, d[16 * j + c], d[16 * j + c + 1]);
            }
        }
        if (NO < 128 && half)  // zero rows of the padded dZ^T
            for (int o = NO; o < 128; o += 2) put_canon_t2(dzt, rl, o, TC_ROWS, 0.f, 0.f);
    }
    tcb_put_at<L>(at, rl, half, row0, n, x, idx, z);
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    if (tid == 0) {
        tc_fence_after();
        const uint32_t a_dzt = smem_u32(dzt), b_at = smem_u32(at);
        constexpr uint32_t id_w = idesc_bf16(128, NI + 16);
#pragma unroll
        for (int kk = 0; kk < TC_ROWS / 16; ++kk)
            tc_mma(tmem, umma_desc(a_dzt + kk * 256, 128, 16 * TC_ROWS), umma_desc(b_at + kk * 256, 128, 16 * TC_ROWS),
                   id_w, kk > 0 ? 1u : 0u);
        if constexpr (L > 0) {
            const uint32_t a_dz = smem_u32(dz), b_w = smem_u32(wtc + wtc_off(L));
            constexpr uint32_t id_a = idesc_bf16(TC_ROWS, NI);
#pragma unroll
            for (int kk = 0; kk < NO / 16; ++kk)
                tc_mma(tmem + TCB_COL_DA, umma_desc(a_dz + kk * 256, 128, 16 * NO), umma_desc(b_w + kk * 256, 128, 16 * NO),
                       id_a, kk > 0 ? 1u : 0u);
        }
        tc_commit(mbar);
    }
    const bool ok = __syncthreads_and(mbar_wait(mbar, phase, wl)) != 0;
    phase ^= 1u;
    if (!ok) return false;
    tc_fence_after();
    const uint32_t tl = tmem + (uint32_t(32 * (warp & 3)) << 16);
    // dW | db: lane = output unit o, columns = inputs (+ the ones column)
    {
        constexpr int NCH = (NI + 16) / 16, H0 = (NCH + 1) / 2;
        const int lo = half ? H0 : 0, hi = half ? NCH : H0;
        const int o = rl;
#pragma unroll
        for (int j = 0; j < H0; ++j) {
            if (lo + j >= hi) break;
            float v[16];
            tmem_ld16(tl + uint32_t((lo + j) * 16), v);
            tmem_wait_ld();
            if (o < NO) {
                float *pw = part + mlp_woff(L) + size_t(o) * NI;
#pragma unroll
                for (int c = 0; c < 16; ++c) {
                    const int i = (lo + j) * 16 + c;
                    if (i < NI) pw[i] = first ? v[c] : pw[i] + v[c];
                    else if (i == NI) part[mlp_boff(L) + o] = first ? v[c] : part[mlp_boff(L) + o] + v[c];
                }
            }
        }
    }
    if constexpr (L > 0) {
        // dZ_{L-1} = dA gelu'(z_{L-1}): this thread's row, its half of the columns
        const int r = row0 + rl;
        const float *zr = z + (size_t(L - 1) * n + (r < n ? r : 0)) * MLP_H;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int c0 = half * 64 + j * 16;
            float v[16];
            tmem_ld16(tl + TCB_COL_DA + uint32_t(c0), v);
            tmem_wait_ld();
#pragma unroll
            for (int c = 0; c < 16; ++c) d[16 * j + c] = (r < n) ? v[c] * gelu_grad(zr[c0 + c]) : 0.f;
        }
    }
    // every TMEM read and operand read of this layer is done before the next one writes
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    return true;
}

__global__ void __launch_bounds__(TC_THREADS, 1)
    k_mlp_bwd_tc(const uint16_t *wt, const float *x, const float *tg, const float *wcol, const int32_t *idx, int n,
                 const float *y, const float *z, float *partials, float *loss, uint32_t wl) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char *base = smem_raw + ((1024 - (smem_u32(smem_raw) & 1023u)) & 1023u);
    unsigned char *wtc = base;
    unsigned char *dz = wtc + WTC_BYTES;
    unsigned char *dzt = dz + TB_DZ;
    unsigned char *at = dzt + TB_DZT;
    uint64_t *mbar_p = reinterpret_cast<uint64_t *>(at + TB_AT);
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(mbar_p + 1);
    const int tid = threadIdx.x, warp = tid >> 5, half = warp >> 2;
    const int rl = 32 * (warp & 3) + (tid & 31);
    // W_l^T (in_l x out_l, K = out_l) of layers 1..4 into the canonical layout
#pragma unroll
    for (int l = 1; l < MLP_NL; ++l) {
        const int K = mlp_out(l), N = mlp_in(l), chunks = K / 8;
        for (int e = tid; e < N * chunks; e += TC_THREADS) {
            const int r = e / chunks, c8 = e - r * chunks;
            cp_async16(wtc + wtc_off(l) + canon_off(r, c8, K), wt + mlp_woff(l) + size_t(r) * K + c8 * 8);
        }
    }
    float *part = partials + size_t(blockIdx.x) * MLP_NPARAM;
    const uint32_t mbar = smem_u32(mbar_p);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_u32(tmem_slot))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    cp_async_wait_all();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    uint32_t phase = 0;
    bool ok = true;
    const float inv_n = 1.0f / float(n);
    float lsum = 0.f;
    const int tiles = int(ceil_div(n, TC_ROWS));
    for (int tile = blockIdx.x; tile < tiles && ok; tile += gridDim.x) {
        const int row0 = tile * TC_ROWS;
        const int r = row0 + rl;
        const bool first = tile == int(blockIdx.x);
        // dZ_4 = wcol (y - t) / n for this thread's row and half of the 80 outputs
        float d[64];
        {
            constexpr int NCH = MLP_OUT / 16, H0 = (NCH + 1) / 2;
            const int c_lo = half ? H0 * 16 : 0, c_hi = half ? MLP_OUT : H0 * 16;
            const float *tr = (r < n) ? tg + size_t(idx ? idx[r] : r) * MLP_OUT : nullptr;
#pragma unroll
            for (int j = 0; j < H0 * 16; ++j) {
                const int c = c_lo + j;
                float e = 0.f;
                if (tr && c < c_hi) {
                    const float dy = y[size_t(r) * MLP_OUT + c] - tr[c];
                    e = dy * wcol[c];
                    lsum += 0.5f * e * dy;
                }
                d[j] = e * inv_n;
            }
        }
        ok = tcb_layer<4>(wtc, dz, dzt, at, tmem, mbar, phase, wl, row0, n, x, idx, z, part, first, d) &&
             tcb_layer<3>(wtc, dz, dzt, at, tmem, mbar, phase, wl, row0, n, x, idx, z, part, first, d) &&
             tcb_layer<2>(wtc, dz, dzt, at, tmem, mbar, phase, wl, row0, n, x, idx, z, part, first, d) &&
             tcb_layer<1>(wtc, dz, dzt, at, tmem, mbar, phase, wl, row0, n, x, idx, z, part, first, d) &&
             tcb_layer<0>(wtc, dz, dzt, at, tmem, mbar, phase, wl, row0, n, x, idx, z, part, first, d);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
    if ((tid & 31) == 0 && lsum != 0.f) atomicAdd(loss, lsum * inv_n);
    if (!ok && tid == 0) atomicOr(&g_mlp_status, BZ_DEV_LOOKBACK);
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem) : "memory");
}

// grad += sum over the CTAs' slices, in slice order
__global__ void k_mlp_reduce(const float *partials, int slices, float *grad) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < MLP_NPARAM; i += gridDim.x * blockDim.x) {
        float s = 0.f;
        for (int c = 0; c < slices; ++c) s += partials[size_t(c) * MLP_NPARAM + i];
        grad[i] += s;
    }
}

// ------------------------------------------------------------------------------------
// parameters: BF16 copies, Adam, minibatch indices
// ------------------------------------------------------------------------------------
__device__ __forceinline__ void put_bf16_copies(int i, float p, uint16_t *wb, uint16_t *wt) {
    int l = 0;
#pragma unroll
    for (int k = 1; k < MLP_NL; ++k) l += (i >= mlp_woff(k));
    const int e = i - mlp_woff(l);
    const int ni = mlp_in(l), no = mlp_out(l);
    if (e >= ni * no) return;  // a bias
    const int o = e / ni, c = e - o * ni;
    const __nv_bfloat16 b = __float2bfloat16_rn(p);
    const uint16_t u = *reinterpret_cast<const uint16_t *>(&b);
    wb[i] = u;
    wt[mlp_woff(l) + c * no + o] = u;
}

__global__ void k_mlp_sync(const float *prm, uint16_t *wb, uint16_t *wt) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < MLP_NPARAM; i += gridDim.x * blockDim.x)
        put_bf16_copies(i, prm[i], wb, wt);
}

__global__ void k_mlp_adam(float *prm, float *grad, float *m, float *v, uint16_t *wb, uint16_t *wt, float lr_c1,
                           float b1, float b2, float c2, float eps, float lr_wd) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < MLP_NPARAM; i += gridDim.x * blockDim.x) {
        const float gi = grad[i];
        grad[i] = 0.f;
        const float mi = fmaf(b1, m[i], (1.f - b1) * gi);
        const float vi = fmaf(b2, v[i], (1.f - b2) * gi * gi);
        m[i] = mi;
        v[i] = vi;
        int l = 0;
#pragma unroll
        for (int k = 1; k < MLP_NL; ++k) l += (i >= mlp_woff(k));
        const bool is_w = i < mlp_boff(l);
        float p = prm[i];
        if (is_w) p -= lr_wd * p;  // decoupled weight decay (Loshchilov & Hutter 2019)
        p -= lr_c1 * mi / (sqrtf(vi * c2) + eps);
        prm[i] = p;
        put_bf16_copies(i, p, wb, wt);
    }
}

__global__ void k_mlp_batch(int n_rows, int n, Rng g, int32_t *idx) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        const u32x4 q = philox(uint32_t(r), g.s0, g.s1, 0x6d6c7000u, g.k0, g.k1);
        idx[r] = int32_t((uint64_t(q.x) * uint64_t(uint32_t(n_rows))) >> 32);  // Lemire's multiply-shift
    }
}

static int num_sms_mlp() {
    static int n = 0;
    if (n == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

static bool al16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

static int g_mlp_path = 1;  // 0: mma.sync; 1: tcgen05 forward (default); 2: tcgen05 forward and backward

static int mlp_forward(const uint16_t *wb, const float *prm, const float *x, const int32_t *idx, int n, float *y,
                       float *z, cudaStream_t st) {
    if (n == 0) return BZ_OK;
    if (!wb || !prm || !x || !y || n < 0 || !al16(wb) || !al16(x) || !al16(y) || (z && !al16(z))) return BZ_ERR_ARG;
    if (g_mlp_path >= 1) {
        auto run_tc = [&](auto kern) -> int {
            if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(TC_SMEM)) != cudaSuccess)
                return BZ_ERR_UNSUPPORTED;
            const int tiles = int(ceil_div(n, TC_ROWS));
            kern<<<std::min(tiles, num_sms_mlp()), TCF_THREADS, TC_SMEM, st>>>(wb, prm, x, idx, n, y, z,
                                                                       host_wait_limit(TC_WAIT_LIMIT));
            return cudaGetLastError() == cudaSuccess ? int(BZ_OK) : int(BZ_ERR_CUDA);
        };
        return z ? run_tc(k_mlp_fwd_tc<true>) : run_tc(k_mlp_fwd_tc<false>);
    }
    auto run = [&](auto kern) -> int {
        if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(FWD_SMEM)) != cudaSuccess)
            return BZ_ERR_UNSUPPORTED;
        const int tiles = int(ceil_div(n, 16 * MF_WARPS));
        kern<<<std::min(tiles, num_sms_mlp()), 32 * MF_WARPS, FWD_SMEM, st>>>(wb, prm, x, idx, n, y, z);
        return cudaGetLastError() == cudaSuccess ? int(BZ_OK) : int(BZ_ERR_CUDA);
    };
    return z ? run(k_mlp_fwd<true>) : run(k_mlp_fwd<false>);
}

// slices of the tcgen05 backward's partial gradient for n rows
static int mlp_bwd_slices(int n) { return std::max(1, std::min(int(ceil_div(n, TC_ROWS)), num_sms_mlp())); }
static size_t mlp_bwd_ws(int n) { return size_t(mlp_bwd_slices(n)) * MLP_NPARAM * sizeof(float); }

static int mlp_backward(const uint16_t *wt, const float *x, const float *t, const float *wcol, const int32_t *idx,
                        int n, const float *y, const float *z, float *grad, float *loss, void *ws, size_t ws_bytes,
                        cudaStream_t st) {
    if (n == 0) return BZ_OK;
    if (!wt || !x || !t || !wcol || !y || !z || !grad || !loss || n < 0 || !al16(wt) || !al16(y) || !al16(z) ||
        !al16(x))
        return BZ_ERR_ARG;
    if (ws) {  // tcgen05, per-CTA slices summed in a fixed order (deterministic)
        if (!al16(ws)) return BZ_ERR_ARG;
        if (ws_bytes < mlp_bwd_ws(n)) return BZ_ERR_WORKSPACE;
        if (cudaFuncSetAttribute(k_mlp_bwd_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, int(TCB_SMEM)) !=
            cudaSuccess)
            return BZ_ERR_UNSUPPORTED;
        const int slices = mlp_bwd_slices(n);
        float *part = static_cast<float *>(ws);
        k_mlp_bwd_tc<<<slices, TC_THREADS, TCB_SMEM, st>>>(wt, x, t, wcol, idx, n, y, z, part, loss,
                                                            host_wait_limit(TC_WAIT_LIMIT));
        if (cudaGetLastError() != cudaSuccess) return BZ_ERR_CUDA;
        k_mlp_reduce<<<int(ceil_div(MLP_NPARAM, 256)), 256, 0, st>>>(part, slices, grad);
        return cudaGetLastError() == cudaSuccess ? BZ_OK : BZ_ERR_CUDA;
    }
    if (cudaFuncSetAttribute(k_mlp_bwd, cudaFuncAttributeMaxDynamicSharedMemorySize, int(BWD_SMEM)) != cudaSuccess)
        return BZ_ERR_UNSUPPORTED;
    const int tiles = int(ceil_div(n, MB_ROWS));
    k_mlp_bwd<<<std::min(tiles, num_sms_mlp()), 32 * MB_WARPS, BWD_SMEM, st>>>(wt, x, t, wcol, idx, n, y, z, grad,
                                                                                loss);
    return cudaGetLastError() == cudaSuccess ? BZ_OK : BZ_ERR_CUDA;
}

static int mlp_adam(float *prm, float *grad, float *m, float *v, uint16_t *wb, uint16_t *wt, int64_t step, float lr,
                    float b1, float b2, float eps, float wd, cudaStream_t st) {
    if (!prm || !grad || !m || !v || !wb || !wt || step < 1 || !(b1 >= 0.f && b1 < 1.f) || !(b2 >= 0.f && b2 < 1.f))
        return BZ_ERR_ARG;
    const double c1 = 1.0 - std::pow(double(b1), double(step));
    const double c2 = 1.0 - std::pow(double(b2), double(step));
    k_mlp_adam<<<int(ceil_div(MLP_NPARAM, 256)), 256, 0, st>>>(prm, grad, m, v, wb, wt, float(lr / c1), b1, b2,
                                                               float(1.0 / c2), eps, lr * wd);
    return cudaGetLastError() == cudaSuccess ? BZ_OK : BZ_ERR_CUDA;
}

static int mlp_batch(int n_rows, int n, uint64_t seed, uint64_t step, int32_t *idx, cudaStream_t st) {
    if (n == 0) return BZ_OK;
    if (!idx || n < 0 || n_rows < 1) return BZ_ERR_ARG;
    const Rng g{uint32_t(seed), uint32_t(seed >> 32), uint32_t(step), uint32_t(step >> 32)};
    k_mlp_batch<<<int(std::min<int64_t>(ceil_div(n, 256), 1024)), 256, 0, st>>>(n_rows, n, g, idx);
    return cudaGetLastError() == cudaSuccess ? BZ_OK : BZ_ERR_CUDA;
}

// training workspace: idx (n int32, padded to 256 B), y (n x OUT), z ((NL-1) x n x H), and
// the tcgen05 backward's partial gradients
static size_t align256(size_t b) { return (b + 255) & ~size_t(255); }
static size_t mlp_train_ws(int n) {
    return align256(size_t(n) * 4) + align256(size_t(n) * MLP_OUT * 4) +
           align256(size_t(MLP_NL - 1) * n * MLP_H * 4) + align256(mlp_bwd_ws(n));
}

// The tensor-core completion wait on its own, in the network kernels' sequence: TMEM
// allocated, the mbarrier initialised for one arrival, the bounded wait of every thread
// decided together, BZ_DEV_LOOKBACK on a wait that ran out, TMEM freed. When ``arrive`` is
// 0 nothing arrives on the mbarrier (no MMA is issued), so the wait runs out after
// wait_limit polls; when it is 1, thread 0 arrives first and the wait completes.
__global__ void __launch_bounds__(128, 1) k_mlp_wait_selftest(int arrive, uint32_t wl, uint32_t *done) {
    __shared__ __align__(8) uint64_t mbar_s;
    __shared__ uint32_t tmem_slot;
    const int tid = threadIdx.x, warp = tid >> 5;
    const uint32_t mbar = smem_u32(&mbar_s);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 32;" ::"r"(smem_u32(&tmem_slot))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;
    if (arrive && tid == 0) {
        asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(mbar) : "memory");
    }
    const bool ok = __syncthreads_and(mbar_wait(mbar, 0u, wl)) != 0;
    if (!ok && tid == 0) atomicOr(&g_mlp_status, BZ_DEV_LOOKBACK);
    if (tid == 0) *done = ok ? 1u : 2u;
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 32;" ::"r"(tmem) : "memory");
}

}  // namespace bz

using namespace bz;

extern "C" {

int bz_mlp_wait_selftest(int32_t arrive, uint32_t *done, void *stream) {
    if ((arrive != 0 && arrive != 1) || !done) return BZ_ERR_ARG;
    k_mlp_wait_selftest<<<1, 128, 0, as_stream(stream)>>>(arrive, host_wait_limit(TC_WAIT_LIMIT), done);
    return cudaGetLastError() == cudaSuccess ? BZ_OK : BZ_ERR_CUDA;
}

int32_t bz_mlp_param_count(void) { return MLP_NPARAM; }

int bz_mlp_select(int32_t path) {
    if (path < 0 || path > 2) return BZ_ERR_ARG;
    g_mlp_path = path;
    return BZ_OK;
}
int32_t bz_mlp_selected(void) { return g_mlp_path; }

int bz_mlp_status(uint32_t *out) {
    if (!out) return BZ_ERR_ARG;
    uint32_t v = 0, zero = 0;
    if (cudaMemcpyFromSymbol(&v, g_mlp_status, sizeof(v)) != cudaSuccess) return BZ_ERR_CUDA;
    if (v && cudaMemcpyToSymbol(g_mlp_status, &zero, sizeof(zero)) != cudaSuccess) return BZ_ERR_CUDA;
    *out = v;
    return BZ_OK;
}

int bz_mlp_sync(const float *params, uint16_t *wb, uint16_t *wt, void *stream) {
    if (!params || !wb || !wt) return BZ_ERR_ARG;
    k_mlp_sync<<<int(ceil_div(MLP_NPARAM, 256)), 256, 0, as_stream(stream)>>>(params, wb, wt);
    return cudaGetLastError() == cudaSuccess ? BZ_OK : BZ_ERR_CUDA;
}

int bz_mlp_forward(const uint16_t *wb, const float *params, const float *x, const int32_t *idx, int32_t n, float *y,
                   float *z, void *stream) {
    return mlp_forward(wb, params, x, idx, n, y, z, as_stream(stream));
}

size_t bz_mlp_backward_workspace(int32_t n) { return n > 0 ? mlp_bwd_ws(n) : 0; }

int bz_mlp_backward(const uint16_t *wb, const uint16_t *wt, const float *params, const float *x, const float *t,
                    const float *wcol, const int32_t *idx, int32_t n, const float *y, const float *z, float *grad,
                    float *loss, void *workspace, size_t workspace_bytes, void *stream) {
    (void)wb;
    (void)params;  // the output layer's bias and the weights enter through y and z
    return mlp_backward(wt, x, t, wcol, idx, n, y, z, grad, loss, workspace, workspace_bytes, as_stream(stream));
}

int bz_mlp_adam(float *params, float *grad, float *m, float *v, uint16_t *wb, uint16_t *wt, int64_t step, float lr,
                float beta1, float beta2, float eps, float weight_decay, void *stream) {
    return mlp_adam(params, grad, m, v, wb, wt, step, lr, beta1, beta2, eps, weight_decay, as_stream(stream));
}

int bz_mlp_batch(int32_t n_rows, int32_t n, uint64_t seed, uint64_t step, int32_t *idx, void *stream) {
    return mlp_batch(n_rows, n, seed, step, idx, as_stream(stream));
}

size_t bz_mlp_train_workspace(int32_t n) { return n > 0 ? mlp_train_ws(n) : 0; }

int bz_mlp_train_step(float *params, float *grad, float *m, float *v, uint16_t *wb, uint16_t *wt, const float *x,
                      const float *t, const float *wcol, int32_t n_rows, int32_t n, uint64_t seed, int64_t step,
                      float lr, float beta1, float beta2, float eps, float weight_decay, float *loss, void *workspace,
                      size_t workspace_bytes, void *stream) {
    if (n < 1 || n_rows < 1 || !workspace || !al16(workspace)) return BZ_ERR_ARG;
    if (workspace_bytes < mlp_train_ws(n)) return BZ_ERR_WORKSPACE;
    cudaStream_t st = as_stream(stream);
    unsigned char *w = static_cast<unsigned char *>(workspace);
    int32_t *idx = reinterpret_cast<int32_t *>(w);
    float *y = reinterpret_cast<float *>(w + align256(size_t(n) * 4));
    float *z = reinterpret_cast<float *>(w + align256(size_t(n) * 4) + align256(size_t(n) * MLP_OUT * 4));
    void *part = w + align256(size_t(n) * 4) + align256(size_t(n) * MLP_OUT * 4) +
                 align256(size_t(MLP_NL - 1) * n * MLP_H * 4);
    int rc = mlp_batch(n_rows, n, seed, uint64_t(step), idx, st);
    if (rc == BZ_OK) rc = mlp_forward(wb, params, x, idx, n, y, z, st);
    if (rc == BZ_OK)
        rc = mlp_backward(wt, x, t, wcol, idx, n, y, z, grad, loss, g_mlp_path == 2 ? part : nullptr,
                          mlp_bwd_ws(n), st);
    if (rc == BZ_OK) rc = mlp_adam(params, grad, m, v, wb, wt, step, lr, beta1, beta2, eps, weight_decay, st);
    return rc;
}

}  // extern "C"
