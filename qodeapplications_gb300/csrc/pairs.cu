// Two-electron terms through (n-2)-electron intermediates.
//
// <P| c+_p c+_q a_s a_r |Q> = sum_K <P| c+_p c+_q |K> <K| a_s a_r |Q>, and K is unique for
// each (Q, r < s).  A pair list of a determinant space holds, for every determinant X and
// every occupied pair u < v, the position of (K = a_v a_u X, pair) in a class-major array
// [class][state][K][pair]: off = n base_c + k np_c + pair for state 0, stride nK_c np_c per
// state (both per entry), and the sign of
// <K| a_v a_u |X> (parity of the occupied orbitals above u and above v; the convention of
// density_tensors.c).  With it, the monomer two-electron sigma vector and the two-particle
// density of the orbital gradient become
//     D[c][(s, K)][rs] = sign z[Q, s]                     (xrh_pair_scatter)
//     E[c][(s, K)][pq] = sum_rs D[c][(s, K)][rs] W_c[pq, rs] (one GEMM per spin class, W = 4 V)
//     sigma[s, P]      = sum sign E[c][(s, K)][pq]          (xrh_pair_gather over P's entries)
//     Gamma_c[pq, rs]  = sum_(s, K) D_zb[c][(s, K)][pq] D_Y[c][(s, K)][rs]   (a GEMM)
// replacing an enumeration of every double excitation of every determinant.
#include "xrh_common.cuh"

namespace {

__global__ void pair_scatter_kernel(int64_t n_entries, const int32_t* __restrict__ X, const int64_t* __restrict__ off,
                                    const int8_t* __restrict__ sgn, const double* __restrict__ zT, int n,
                                    const int64_t* __restrict__ stride, double* __restrict__ D) {
    const int64_t total = n_entries * n;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = t / n;
        const int s = (int)(t - e * n);
        const double v = __ldg(zT + (int64_t)__ldg(X + e) * n + s);
        D[__ldg(off + e) + (int64_t)s * __ldg(stride + e)] = __ldg(sgn + e) < 0 ? -v : v;
    }
}

__global__ void pair_gather_kernel(int n_X, const int64_t* __restrict__ xptr, const int64_t* __restrict__ off,
                                   const int8_t* __restrict__ sgn, const double* __restrict__ E, int n,
                                   const int64_t* __restrict__ stride, double* __restrict__ sigmaT) {
    const int64_t total = (int64_t)n_X * n;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int s = (int)(t / n_X);
        const int x = (int)(t - (int64_t)s * n_X);
        double acc = 0.0;
        for (int64_t e = __ldg(xptr + x); e < __ldg(xptr + x + 1); ++e) {
            const double v = __ldg(E + __ldg(off + e) + (int64_t)s * __ldg(stride + e));
            acc += __ldg(sgn + e) < 0 ? -v : v;
        }
        sigmaT[(int64_t)s * n_X + x] = acc;
    }
}

// Many scatters / gathers in one launch: blockIdx.y is the task, blocks stride over its entries.
__global__ void pair_scatter_grouped_kernel(const xrh_pair_task* __restrict__ tasks) {
    const xrh_pair_task& T = tasks[blockIdx.y];
    const int n = T.n;
    const int64_t total = T.count * n;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = t / n;
        const int s = (int)(t - e * n);
        const double v = __ldg(T.src + (int64_t)__ldg(T.X + e) * n + s);
        T.dst[__ldg(T.off + e) + (int64_t)s * __ldg(T.stride + e)] = __ldg(T.sign + e) < 0 ? -v : v;
    }
}

__global__ void pair_gather_grouped_kernel(const xrh_pair_task* __restrict__ tasks) {
    const xrh_pair_task& T = tasks[blockIdx.y];
    const int n = T.n;
    const int64_t n_X = T.count;
    const int64_t total = n_X * n;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int s = (int)(t / n_X);
        const int64_t x = t - (int64_t)s * n_X;
        double acc = 0.0;
        for (int64_t e = __ldg(T.xptr + x); e < __ldg(T.xptr + x + 1); ++e) {
            const double v = __ldg(T.src + __ldg(T.off + e) + (int64_t)s * __ldg(T.stride + e));
            acc += __ldg(T.sign + e) < 0 ? -v : v;
        }
        T.dst[(int64_t)s * n_X + x] = acc;
    }
}

unsigned grid_for(int64_t total) {
    const int64_t b = (total + 255) / 256;
    return (unsigned)(b < 152 * 32 ? (b > 0 ? b : 1) : 152 * 32);
}

}  // namespace

extern "C" int xrh_pair_scatter(int64_t n_entries, const int32_t* X_dev, const int64_t* off_dev, const int8_t* sign_dev,
                                const double* zT_dev, int n, const int64_t* stride_dev, double* D_dev, void* stream) {
    if (n_entries < 0 || n <= 0) return XRH_ERR_ARG;
    if (n_entries == 0) return XRH_OK;
    if (!X_dev || !off_dev || !sign_dev || !zT_dev || !stride_dev || !D_dev) return XRH_ERR_ARG;
    pair_scatter_kernel<<<grid_for(n_entries * n), 256, 0, (cudaStream_t)stream>>>(n_entries, X_dev, off_dev, sign_dev,
                                                                                   zT_dev, n, stride_dev, D_dev);
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}

extern "C" int xrh_pair_gather(int n_X, const int64_t* xptr_dev, const int64_t* off_dev, const int8_t* sign_dev,
                               const double* E_dev, int n, const int64_t* stride_dev, double* sigmaT_dev,
                               void* stream) {
    if (n_X < 0 || n <= 0) return XRH_ERR_ARG;
    if (n_X == 0) return XRH_OK;
    if (!xptr_dev || !off_dev || !sign_dev || !E_dev || !stride_dev || !sigmaT_dev) return XRH_ERR_ARG;
    pair_gather_kernel<<<grid_for((int64_t)n_X * n), 256, 0, (cudaStream_t)stream>>>(n_X, xptr_dev, off_dev, sign_dev,
                                                                                    E_dev, n, stride_dev, sigmaT_dev);
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}

extern "C" int xrh_pair_grouped(int gather, const xrh_pair_task* tasks_dev, int n_tasks, int64_t max_total,
                                void* stream) {
    if (n_tasks < 0 || max_total < 0 || n_tasks > 65535) return XRH_ERR_ARG;
    if (n_tasks == 0 || max_total == 0) return XRH_OK;
    if (!tasks_dev) return XRH_ERR_ARG;
    const dim3 grid(grid_for(max_total), (unsigned)n_tasks);
    if (gather)
        pair_gather_grouped_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(tasks_dev);
    else
        pair_scatter_grouped_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(tasks_dev);
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}
