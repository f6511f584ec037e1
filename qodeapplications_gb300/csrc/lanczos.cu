// FP64 building blocks of the Lanczos eigensolver for the lowest eigenpairs of the
// excitonic Hamiltonian (the reference diagonalises the full H with scipy.linalg.eig,
// hermitian-XRCC/mains/workflow.py:229 and StateSpaceOptimizer/state_gradients.py:107; only
// the lowest eigenpair is used, so a Krylov method on the GPU replaces the dense solve).
//
//   xrh_gemv_rows:  y[i] = alpha * sum_j A[i*lda + j] x[j] + beta * y[i]   (warp per row)
//   xrh_gemv_cols:  y[j] += sum_i c[i] * scale * A[i*lda + j]              (thread per column)
//   xrh_lanczos_normalize: beta[k] = ||w||, v = w / beta[k]  (one CTA; the norm stays on the
//       device so the whole Krylov loop can be replayed as one CUDA graph)
// All FP64: the eigensolve is kept in double precision on every precision path.
#include "xrh_common.cuh"

namespace {

__global__ void __launch_bounds__(256) gemv_rows_kernel(int64_t rows, int64_t cols, const double* __restrict__ A,
                                                      int64_t lda, const double* __restrict__ x, double alpha,
                                                      double beta, double* __restrict__ y) {
    const int64_t row = (int64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (row >= rows) return;
    const double* a = A + row * lda;
    double s = 0.0;
    for (int64_t j = lane; j < cols; j += 32) s = fma(a[j], x[j], s);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) y[row] = alpha * s + (beta == 0.0 ? 0.0 : beta * y[row]);
}

__global__ void __launch_bounds__(256) gemv_cols_kernel(int64_t rows, int64_t cols, const double* __restrict__ A,
                                                      int64_t lda, const double* __restrict__ c, double scale,
                                                      double* __restrict__ y) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= cols) return;
    double s = 0.0;
    for (int64_t i = 0; i < rows; ++i) s = fma(c[i], A[i * lda + j], s);
    y[j] += scale * s;
}

__global__ void __launch_bounds__(1024) normalize_kernel(int64_t n, const double* __restrict__ w, double* __restrict__ v,
                                                       double* __restrict__ beta_out) {
    __shared__ double red[32];
    double s = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) s = fma(w[i], w[i], s);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (threadIdx.x == 0) red[0] = s;
    }
    __syncthreads();
    const double b = sqrt(red[0]);
    const double inv = b > 0.0 ? 1.0 / b : 0.0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) v[i] = w[i] * inv;
    if (threadIdx.x == 0) *beta_out = b;
}

// Whole Krylov loop of a small sector in one CTA: m Lanczos steps with two classical
// Gram-Schmidt passes, the same arithmetic as the per-step launches (gemv_rows, two CGS
// passes of gemv_rows + gemv_cols, normalize) without 6 m launches.  H is read from global
// memory (L2-resident for the sizes this serves); w and the CGS coefficients live in shared
// memory.  alpha[j] = sum of both passes' coefficient of V[j]; beta[j] = |w| after them.
__device__ __forceinline__ double block_sum(double s, double* red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    double t = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += red[i];
    return t;
}

__global__ void __launch_bounds__(1024) lanczos_small_kernel(int n, int m, const double* __restrict__ H, int64_t ld,
                                                             const double* __restrict__ v0, double* __restrict__ V,
                                                             double* __restrict__ alpha, double* __restrict__ beta) {
    extern __shared__ double sm[];
    double* w = sm;               // [n]
    double* c = w + n;            // [m + 1]
    __shared__ double red[32];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
    for (int k = tid; k < n; k += blockDim.x) V[k] = v0[k];
    __syncthreads();
    for (int j = 0; j < m; ++j) {
        const double* vj = V + (int64_t)j * n;
        for (int r = warp; r < n; r += nw) {
            const double* h = H + (int64_t)r * ld;
            double s = 0.0;
            for (int k = lane; k < n; k += 32) s = fma(h[k], vj[k], s);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            if (lane == 0) w[r] = s;
        }
        __syncthreads();
        double a = 0.0;
        for (int pass = 0; pass < 2; ++pass) {
            for (int i = warp; i <= j; i += nw) {
                const double* vi = V + (int64_t)i * n;
                double s = 0.0;
                for (int k = lane; k < n; k += 32) s = fma(vi[k], w[k], s);
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
                if (lane == 0) c[i] = s;
            }
            __syncthreads();
            a += c[j];
            for (int k = tid; k < n; k += blockDim.x) {
                double s = 0.0;
                for (int i = 0; i <= j; ++i) s = fma(c[i], V[(int64_t)i * n + k], s);
                w[k] -= s;
            }
            __syncthreads();
        }
        double s = 0.0;
        for (int k = tid; k < n; k += blockDim.x) s = fma(w[k], w[k], s);
        const double b = sqrt(block_sum(s, red));
        const double inv = b > 0.0 ? 1.0 / b : 0.0;
        double* vn = V + (int64_t)(j + 1) * n;
        for (int k = tid; k < n; k += blockDim.x) vn[k] = w[k] * inv;
        if (tid == 0) {
            alpha[j] = a;
            beta[j] = b;
        }
        __syncthreads();
    }
}

}  // namespace

extern "C" int xrh_lanczos_small(int n, int m, const double* H_dev, int64_t ld, const double* v0_dev, double* V_dev,
                                 double* alpha_dev, double* beta_dev, void* stream) {
    if (n <= 0 || m <= 0 || ld < n) return XRH_ERR_ARG;
    if (!H_dev || !v0_dev || !V_dev || !alpha_dev || !beta_dev) return XRH_ERR_ARG;
    const size_t smem = sizeof(double) * ((size_t)n + (size_t)m + 1);
    if (n > 4096 || smem > 48 * 1024) return XRH_ERR_CAPACITY;
    lanczos_small_kernel<<<1, 1024, smem, (cudaStream_t)stream>>>(n, m, H_dev, ld, v0_dev, V_dev, alpha_dev, beta_dev);
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}

extern "C" int xrh_gemv_rows(int64_t rows, int64_t cols, const double* A_dev, int64_t lda, const double* x_dev,
                             double alpha, double beta, double* y_dev, void* stream) {
    if (rows < 0 || cols < 0 || lda < cols) return XRH_ERR_ARG;
    if (rows == 0) return XRH_OK;
    if (!A_dev || !x_dev || !y_dev) return XRH_ERR_ARG;
    if ((rows + 7) / 8 > 0x7fffffffLL) return XRH_ERR_CAPACITY;
    gemv_rows_kernel<<<(unsigned)((rows + 7) / 8), 256, 0, (cudaStream_t)stream>>>(rows, cols, A_dev, lda, x_dev, alpha,
                                                                                  beta, y_dev);
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}

extern "C" int xrh_gemv_cols(int64_t rows, int64_t cols, const double* A_dev, int64_t lda, const double* c_dev,
                             double scale, double* y_dev, void* stream) {
    if (rows < 0 || cols < 0 || lda < cols) return XRH_ERR_ARG;
    if (cols == 0) return XRH_OK;
    if (!A_dev || !c_dev || !y_dev) return XRH_ERR_ARG;
    gemv_cols_kernel<<<(unsigned)((cols + 255) / 256), 256, 0, (cudaStream_t)stream>>>(rows, cols, A_dev, lda, c_dev,
                                                                                      scale, y_dev);
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}

extern "C" int xrh_lanczos_normalize(int64_t n, const double* w_dev, double* v_dev, double* beta_dev, void* stream) {
    if (n <= 0 || !w_dev || !v_dev || !beta_dev) return XRH_ERR_ARG;
    normalize_kernel<<<1, 1024, 0, (cudaStream_t)stream>>>(n, w_dev, v_dev, beta_dev);
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}
