// Standalone moment deposit: the (sum w, sum w*ionflag, 0, sum w*energy) per node that
// post_processing forms (post_processing_1D.py:44-57) through the reference's
// reda/redcheck pair (kernels-new.cu:8-73). Node = int(((x+dx/2)/(L+dx))*M)/bnf,
// computed exactly. Per-CTA shared-memory grid, one float64 merge per CTA.
#include "bz_common.cuh"

namespace bz {

constexpr int DT = 256;

template <typename T>
__global__ void __launch_bounds__(DT) k_deposit(bz_params p, NodeMap nm, const T *x, const T *vx, const T *vy, const T *vz,
                                                const T *w, const int32_t *n_ptr, int64_t cap, const uint8_t *flag,
                                                double *moments) {
    extern __shared__ __align__(16) unsigned char smem[];
    T *m = reinterpret_cast<T *>(smem);
    const int nn = p.n_nodes;
    for (int i = threadIdx.x; i < 3 * nn; i += DT) m[i] = T(0);
    __syncthreads();
    const T efac = T(0.5 * m_e() * j_ev());
    const int64_t n = min(int64_t(max(*n_ptr, 0)), cap);
    for (int64_t i = blockIdx.x * DT + threadIdx.x; i < n; i += int64_t(gridDim.x) * DT) {
        T wi = w[i];
        int nd = deposit_node(p.advect, x[i], nm);
        if (nd < 0 || nd >= nn) continue;
        T f = flag ? T(flag[i]) : T(0);
        if (wi > T(0)) {
            T e = efac * (vx[i] * vx[i] + vy[i] * vy[i] + vz[i] * vz[i]);
            atomicAdd(&m[nd], wi);
            if (f != T(0)) atomicAdd(&m[nn + nd], f * wi);
            atomicAdd(&m[2 * nn + nd], e * wi);
        } else if (f != T(0)) {
            atomicAdd(&m[nn + nd], f);  // unweighted flag of a w = 0 particle (post_processing_1D.py:50-55)
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 3 * nn; i += DT) {
        T v = m[i];
        if (v != T(0)) {
            int col = i / nn, nd = i - col * nn;
            atomicAdd(&moments[(col == 2 ? 3 : col) * nn + nd], double(v));
        }
    }
}

template <typename T, typename P>
static int deposit_entry(const bz_params *pp, P s, const int32_t *n, int64_t cap, const uint8_t *flag,
                         double *moments, void *stream) {
    if (!pp || !n || !moments || !s.x || !s.vx || !s.vy || !s.vz || !s.w) return BZ_ERR_ARG;
    const bz_params &p = *pp;
    if (p.n_nodes < 1 || p.bnf < 1 || (p.advect == BZ_ADVECT_1D && (p.dx <= 0 || p.L <= 0))) return BZ_ERR_ARG;
    size_t smem = size_t(3) * p.n_nodes * sizeof(T);
    auto kern = k_deposit<T>;
    if (smem > 48 * 1024 &&
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)) != cudaSuccess)
        return BZ_ERR_UNSUPPORTED;
    int dev = 0, sms = 1, per_sm = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, DT, smem) != cudaSuccess || per_sm < 1)
        return BZ_ERR_UNSUPPORTED;
    kern<<<sms * per_sm, DT, smem, as_stream(stream)>>>(p, make_node_map(p), s.x, s.vx, s.vy, s.vz, s.w, n, cap, flag, moments);
    return cudaGetLastError() == cudaSuccess ? BZ_OK : BZ_ERR_CUDA;
}

}  // namespace bz

extern "C" {
int bz_deposit_f32(const bz_params *p, bz_particles_f32 s, const int32_t *n, int64_t capacity, const uint8_t *ionflag,
                   double *moments, void *stream) {
    return bz::deposit_entry<float>(p, s, n, capacity, ionflag, moments, stream);
}
int bz_deposit_f64(const bz_params *p, bz_particles_f64 s, const int32_t *n, int64_t capacity, const uint8_t *ionflag,
                   double *moments, void *stream) {
    return bz::deposit_entry<double>(p, s, n, capacity, ionflag, moments, stream);
}
}
