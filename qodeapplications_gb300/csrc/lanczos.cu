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

}  // namespace

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
