// Small dense FP64 matrices of the orbital transformation (n <= 64 spin or spatial orbitals):
//
//   xrh_inverse_small: A^-1 by Gauss-Jordan elimination with partial pivoting, in one CTA with
//       the augmented [A | I] in shared memory.  Replaces the overlap inverse of the
//       biorthogonalisation (hermitian-XRCC/get_ints.py:62-66, direct_Sinv with
//       qode.math.precise_numpy_inverse).  A pivot below 1e-300 in magnitude sets *status = 1.
//   xrh_expm_small: exp(A) by scaling and squaring: A / 2^s with ||A / 2^s||_1 <= 1/4, the
//       Taylor polynomial to degree 16 in Horner form (truncation below 1e-20 relative), then
//       s squarings.  For the rotation R = exp(kappa) of antisymmetric orbital-rotation
//       parameters (StateSpaceOptimizer/orb_grads.py, orbital_solver.py:431 uses the first-
//       order I + s x instead).
// Both run in one CTA: the FP64 work is O(n^3) per product (n <= 64), a few dozen products.
#include "xrh_common.cuh"

namespace {

constexpr int kSmallThreads = 256;
constexpr int kSmallMax = 64;

__global__ void __launch_bounds__(kSmallThreads) inverse_small_kernel(int n, const double* __restrict__ A,
                                                                      int64_t lda, double* __restrict__ Ainv,
                                                                      int64_t ldi, int32_t* status) {
    extern __shared__ double sm[];              // [n][2n]
    __shared__ int piv;
    __shared__ double pmax;
    const int w = 2 * n;
    for (int t = threadIdx.x; t < n * w; t += blockDim.x) {
        const int i = t / w, j = t - i * w;
        sm[t] = j < n ? A[(int64_t)i * lda + j] : (j - n == i ? 1.0 : 0.0);
    }
    __syncthreads();
    for (int k = 0; k < n; ++k) {
        if (threadIdx.x == 0) {
            int best = k;
            double bv = fabs(sm[k * w + k]);
            for (int i = k + 1; i < n; ++i) {
                const double v = fabs(sm[i * w + k]);
                if (v > bv) {
                    bv = v;
                    best = i;
                }
            }
            piv = best;
            pmax = bv;
        }
        __syncthreads();
        if (pmax < 1e-300) {
            if (threadIdx.x == 0 && status) *status = 1;
            return;
        }
        if (piv != k)
            for (int j = threadIdx.x; j < w; j += blockDim.x) {
                const double a = sm[k * w + j];
                sm[k * w + j] = sm[piv * w + j];
                sm[piv * w + j] = a;
            }
        __syncthreads();
        const double inv = 1.0 / sm[k * w + k];
        __syncthreads();
        for (int j = threadIdx.x; j < w; j += blockDim.x) sm[k * w + j] *= inv;
        __syncthreads();
        for (int t = threadIdx.x; t < n * w; t += blockDim.x) {
            const int i = t / w, j = t - i * w;
            if (i == k) continue;
            const double f = sm[i * w + k];
            if (j != k) sm[t] -= f * sm[k * w + j];
        }
        __syncthreads();
        for (int i = threadIdx.x; i < n; i += blockDim.x)
            if (i != k) sm[i * w + k] = 0.0;
        __syncthreads();
    }
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
        const int i = t / n, j = t - i * n;
        Ainv[(int64_t)i * ldi + j] = sm[i * w + n + j];
    }
    if (threadIdx.x == 0 && status) *status = 0;
}

// C = A B for n x n row-major matrices in shared memory (C distinct from A and B)
__device__ void mm_small(int n, const double* A, const double* B, double* C) {
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
        const int i = t / n, j = t - i * n;
        double s = 0.0;
        for (int k = 0; k < n; ++k) s = fma(A[i * n + k], B[k * n + j], s);
        C[t] = s;
    }
    __syncthreads();
}

__global__ void __launch_bounds__(kSmallThreads) expm_small_kernel(int n, const double* __restrict__ A, int64_t lda,
                                                                   double* __restrict__ E, int64_t lde) {
    extern __shared__ double sm[];              // X, P, Q: 3 n^2
    double* X = sm;
    double* P = X + n * n;
    double* Q = P + n * n;
    __shared__ int s_steps;
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) X[t] = A[(int64_t)(t / n) * lda + (t % n)];
    __syncthreads();
    if (threadIdx.x == 0) {
        double mx = 0.0;
        for (int j = 0; j < n; ++j) {
            double c = 0.0;
            for (int i = 0; i < n; ++i) c += fabs(X[i * n + j]);
            mx = c > mx ? c : mx;
        }
        int s = 0;
        while (mx > 0.25 && s < 60) {
            mx *= 0.5;
            ++s;
        }
        s_steps = s;
    }
    __syncthreads();
    const double scale = ldexp(1.0, -s_steps);
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) X[t] *= scale;
    __syncthreads();
    // Horner: P = I + X/1 (I + X/2 (I + ... (I + X/16)))
    constexpr int kDeg = 16;
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) P[t] = ((t / n) == (t % n) ? 1.0 : 0.0) + X[t] / kDeg;
    __syncthreads();
    for (int d = kDeg - 1; d >= 1; --d) {
        mm_small(n, X, P, Q);
        for (int t = threadIdx.x; t < n * n; t += blockDim.x) P[t] = ((t / n) == (t % n) ? 1.0 : 0.0) + Q[t] / d;
        __syncthreads();
    }
    for (int k = 0; k < s_steps; ++k) {
        mm_small(n, P, P, Q);
        for (int t = threadIdx.x; t < n * n; t += blockDim.x) P[t] = Q[t];
        __syncthreads();
    }
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) E[(int64_t)(t / n) * lde + (t % n)] = P[t];
}

}  // namespace

extern "C" int xrh_inverse_small(int n, const double* A_dev, int64_t lda, double* Ainv_dev, int64_t ldi,
                                 int32_t* status_dev, void* stream) {
    if (n <= 0 || !A_dev || !Ainv_dev || lda < n || ldi < n) return XRH_ERR_ARG;
    if (n > kSmallMax) return XRH_ERR_CAPACITY;
    const size_t smem = sizeof(double) * (size_t)n * 2 * n;
    if (smem > 48 * 1024)
        cudaFuncSetAttribute(inverse_small_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    inverse_small_kernel<<<1, kSmallThreads, smem, (cudaStream_t)stream>>>(n, A_dev, lda, Ainv_dev, ldi, status_dev);
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}

extern "C" int xrh_expm_small(int n, const double* A_dev, int64_t lda, double* E_dev, int64_t lde, void* stream) {
    if (n <= 0 || !A_dev || !E_dev || lda < n || lde < n) return XRH_ERR_ARG;
    if (n > kSmallMax) return XRH_ERR_CAPACITY;
    const size_t smem = sizeof(double) * 3 * (size_t)n * n;
    if (smem > 48 * 1024)
        cudaFuncSetAttribute(expm_small_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    expm_small_kernel<<<1, kSmallThreads, smem, (cudaStream_t)stream>>>(n, A_dev, lda, E_dev, lde);
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}

// Spin-orbital form of a spatial matrix: out[a, b] = in[sidx[a], sidx[b]] when spin[a] ==
// spin[b], else 0 (alpha block then beta block inside every fragment).
namespace {
__global__ void spin_block_kernel(int n_so, const int32_t* __restrict__ sidx, const int8_t* __restrict__ spin,
                                  const double* __restrict__ in, int64_t ldin, double* __restrict__ out,
                                  int64_t ldout) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)n_so * n_so) return;
    const int a = (int)(t / n_so), b = (int)(t - (int64_t)a * n_so);
    out[(int64_t)a * ldout + b] = spin[a] == spin[b] ? in[(int64_t)sidx[a] * ldin + sidx[b]] : 0.0;
}
}  // namespace

extern "C" int xrh_spin_block(int n_so, const int32_t* sidx_dev, const int8_t* spin_dev, const double* in_dev,
                              int64_t ldin, double* out_dev, int64_t ldout, void* stream) {
    if (n_so <= 0 || !sidx_dev || !spin_dev || !in_dev || !out_dev || ldout < n_so) return XRH_ERR_ARG;
    const int64_t total = (int64_t)n_so * n_so;
    spin_block_kernel<<<(unsigned)((total + 255) / 256), 256, 0, (cudaStream_t)stream>>>(n_so, sidx_dev, spin_dev,
                                                                                        in_dev, ldin, out_dev, ldout);
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}

// out[i, j] = in[idx[i], idx[j]] for i, j < n (a principal submatrix, e.g. the alpha-alpha
// block of a spin-orbital matrix).
namespace {
__global__ void gather_submatrix_kernel(int n, const int32_t* __restrict__ idx, const double* __restrict__ in,
                                        int64_t ldin, double* __restrict__ out, int64_t ldout) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)n * n) return;
    const int i = (int)(t / n), j = (int)(t - (int64_t)i * n);
    out[(int64_t)i * ldout + j] = in[(int64_t)idx[i] * ldin + idx[j]];
}
}  // namespace

extern "C" int xrh_gather_submatrix(int n, const int32_t* idx_dev, const double* in_dev, int64_t ldin, double* out_dev,
                                    int64_t ldout, void* stream) {
    if (n <= 0 || !idx_dev || !in_dev || !out_dev || ldout < n) return XRH_ERR_ARG;
    const int64_t total = (int64_t)n * n;
    gather_submatrix_kernel<<<(unsigned)((total + 255) / 256), 256, 0, (cudaStream_t)stream>>>(n, idx_dev, in_dev,
                                                                                               ldin, out_dev, ldout);
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}

// ---- small device-side helpers of the optimizer iteration -------------------------------
namespace {
__global__ void index_move_kernel(int64_t n, const int64_t* __restrict__ idx, const double* __restrict__ src,
                                  double* __restrict__ dst, int gather) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (gather == 1) dst[i] = src[idx[i]];
    else if (gather == 2) atomicAdd(dst + idx[i], src[i]);
    else dst[idx[i]] = src[i];
}

__global__ void add_mixed_kernel(int64_t n, double alpha, const double* __restrict__ x64,
                                 const float* __restrict__ x32, double* __restrict__ y) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double v = x64 ? x64[i] : 0.0;
    if (x32) v += (double)x32[i];
    y[i] += alpha * v;
}

__global__ void f64_to_f32_kernel(int64_t n, const double* __restrict__ src, float* __restrict__ dst) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = (float)src[i];
}

__global__ void spin_sum_antisym_kernel(int n_sp, int n_spin, const int32_t* __restrict__ so,
                                        const double* __restrict__ G, int64_t ldg, double* __restrict__ out) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_sp * n_sp) return;
    const int a = t / n_sp, b = t - a * n_sp;
    double s = 0.0;
    for (int k = 0; k < n_spin; ++k) {
        const int64_t pa = so[k * n_sp + a], pb = so[k * n_sp + b];
        s += G[pa * ldg + pb] - G[pb * ldg + pa];
    }
    out[t] = s;
}

// C = alpha A B + beta I for n x n row-major FP64 blocks (n <= 64): CTA per 4 rows of one
// task's C, thread per output; tasks found by binary search on cta_begin.
__global__ void __launch_bounds__(256) small_mm_grouped_kernel(const xrh_small_mm_task* __restrict__ tasks,
                                                               int n_tasks) {
    int lo = 0, hi = n_tasks - 1;
    const int64_t cta = blockIdx.x;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (tasks[mid].cta_begin <= cta) lo = mid; else hi = mid - 1;
    }
    const xrh_small_mm_task& T = tasks[lo];
    const int n = T.n;
    const int row = (int)(cta - T.cta_begin) * 4 + (threadIdx.x >> 6), col = threadIdx.x & 63;
    if (row >= n || col >= n) return;
    const double* a = T.A + (int64_t)row * n;
    double s = 0.0;
    for (int k = 0; k < n; ++k) s = fma(a[k], T.B[(int64_t)k * n + col], s);
    T.C[(int64_t)row * n + col] = T.alpha * s + (row == col ? T.beta : 0.0);
}
}  // namespace

extern "C" int xrh_zero(void* ptr_dev, int64_t bytes, void* stream) {
    if (bytes < 0 || (bytes > 0 && !ptr_dev)) return XRH_ERR_ARG;
    if (bytes == 0) return XRH_OK;
    const cudaError_t e = cudaMemsetAsync(ptr_dev, 0, (size_t)bytes, (cudaStream_t)stream);
    if (e != cudaSuccess) {
        xrh_set_last_cuda_error((int)e);
        return XRH_ERR_CUDA;
    }
    return XRH_OK;
}

extern "C" int xrh_index_move(int64_t n, const int64_t* idx_dev, const double* src_dev, double* dst_dev, int gather,
                              void* stream) {
    if (n < 0 || gather < 0 || gather > 2 || (n > 0 && (!idx_dev || !src_dev || !dst_dev))) return XRH_ERR_ARG;
    if (n == 0) return XRH_OK;
    if ((n + 255) / 256 > 0x7fffffffLL) return XRH_ERR_CAPACITY;
    index_move_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(n, idx_dev, src_dev, dst_dev,
                                                                                   gather);
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}

extern "C" int xrh_add_mixed(int64_t n, double alpha, const double* x64_dev, const float* x32_dev, double* y_dev,
                             void* stream) {
    if (n < 0 || (n > 0 && (!y_dev || (!x64_dev && !x32_dev)))) return XRH_ERR_ARG;
    if (n == 0) return XRH_OK;
    if ((n + 255) / 256 > 0x7fffffffLL) return XRH_ERR_CAPACITY;
    add_mixed_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(n, alpha, x64_dev, x32_dev, y_dev);
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}

extern "C" int xrh_f64_to_f32(int64_t n, const double* src_dev, float* dst_dev, void* stream) {
    if (n < 0 || (n > 0 && (!src_dev || !dst_dev))) return XRH_ERR_ARG;
    if (n == 0) return XRH_OK;
    if ((n + 255) / 256 > 0x7fffffffLL) return XRH_ERR_CAPACITY;
    f64_to_f32_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(n, src_dev, dst_dev);
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}

extern "C" int xrh_spin_sum_antisym(int n_sp, int n_spin, const int32_t* so_dev, const double* G_dev, int64_t ldg,
                                    double* out_dev, void* stream) {
    if (n_sp <= 0 || n_spin <= 0 || !so_dev || !G_dev || !out_dev) return XRH_ERR_ARG;
    const int total = n_sp * n_sp;
    spin_sum_antisym_kernel<<<(total + 255) / 256, 256, 0, (cudaStream_t)stream>>>(n_sp, n_spin, so_dev, G_dev, ldg,
                                                                                  out_dev);
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}

extern "C" int xrh_small_mm_grouped(const xrh_small_mm_task* tasks_dev, int n_tasks, int64_t total_ctas,
                                    void* stream) {
    if (n_tasks < 0 || total_ctas < 0) return XRH_ERR_ARG;
    if (n_tasks == 0 || total_ctas == 0) return XRH_OK;
    if (!tasks_dev) return XRH_ERR_ARG;
    if (total_ctas > 0x7fffffffLL) return XRH_ERR_CAPACITY;
    small_mm_grouped_kernel<<<(unsigned)total_ctas, 256, 0, (cudaStream_t)stream>>>(tasks_dev, n_tasks);
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}
