// The steepest-descent state update of the optimizer, every (fragment, charge) block in one
// launch per stage, and a small-output long-K A B^T for the orbital gradient.
//
// The reference updates states with NumPy per fragment and charge
// (StateSpaceOptimizer/state_solver.py:207-453; the tangent projection and Loewdin
// orthonormalisation of the states between optimizer steps).  For a block with states z
// (n x K, rows orthonormal), gradient g (stored transposed, K x n, as gT [+ gT32]) and step eps:
//   xrh_gram_grouped(which=0):  G += g z^T                    (n x n, K split over CTAs)
//   xrh_tangent_step:           zn = z - eps * t,  t = g - 1/2 (G + G^T) z;  *sq += |t|^2
//   xrh_gram_grouped(which=1):  S += zn zn^T
//   xrh_inv_sqrt_small:         M = S^-1/2                      (coupled Newton-Schulz)
//   xrh_left_multiply:          z = M zn
// n <= 64 (n <= 32 for xrh_inv_sqrt_small).  All arithmetic FP64 (the FP64 rate of the part
// is low, so the K dimension is spread over many CTAs); Gram and norm partials are added with
// FP64 atomics into outputs the caller zeroes.
#include "xrh_common.cuh"

namespace {

constexpr int SS_THREADS = 256;
constexpr int SS_KSLICE = 64;      // K columns per CTA of the state update (xrh_state_ctas)
constexpr int ABT_KSLICE = 256;    // K columns per CTA of the A B^T products (xrh_abt_ctas)
constexpr int GR_KCHUNK = 32;      // columns staged per step in the Gram kernel
constexpr int NS_MAX = 32;

__device__ __forceinline__ int find_task(const xrh_state_task* __restrict__ t, int n_tasks, int64_t cta) {
    int lo = 0, hi = n_tasks - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (t[mid].cta_begin <= cta) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// One CTA: C (m x n) += alpha * A[:, k_begin:k_end] B[:, k_begin:k_end]^T, m, n <= 64.
// A is m x K: A[i][k] = A[i*lda + k], or with at A[k*lda + i] (then plus A_add[k*lda + i] when
// A_add is given); B likewise with bt.  Operands are staged GR_KCHUNK columns at a time with
// loads that run along the contiguous dimension.
// ACC is the type of the per-chunk sums; with FP32 inputs the chunk sums (GR_KCHUNK products)
// are folded into FP32 (hi, lo) pairs by TwoSum, keeping the FP64 pipe out of the loop.
template <typename T>
__device__ __forceinline__ void abt_stage(const T* __restrict__ X, int64_t ld, bool xt, const float* __restrict__ X_add,
                                          int rows, int64_t k0, int64_t k_end, T (*sx)[GR_KCHUNK + 1]) {
    if (!xt) {
        for (int e = threadIdx.x; e < rows * GR_KCHUNK; e += SS_THREADS) {
            const int i = e / GR_KCHUNK, kk = e - i * GR_KCHUNK;
            const int64_t k = k0 + kk;
            sx[i][kk] = k < k_end ? X[(int64_t)i * ld + k] : T(0);
        }
    } else {
        for (int e = threadIdx.x; e < rows * GR_KCHUNK; e += SS_THREADS) {
            const int kk = e / rows, i = e - kk * rows;
            const int64_t k = k0 + kk;
            T v = T(0);
            if (k < k_end) {
                v = X[k * ld + i];
                if (X_add) v += (T)X_add[k * ld + i];
            }
            sx[i][kk] = v;
        }
    }
}

template <typename T, typename ACC>
__device__ __forceinline__ void abt_slice(const T* __restrict__ A, int64_t lda, bool at, const float* __restrict__ A_add,
                                          int m, const T* __restrict__ B, int64_t ldb, bool bt, int n,
                                          int64_t k_begin, int64_t k_end, double alpha, double* __restrict__ C,
                                          T (*sa)[GR_KCHUNK + 1], T (*sb)[GR_KCHUNK + 1]) {
    const int mn = m * n;
    constexpr bool F32 = sizeof(ACC) == 4;
    double acc[16];                    // FP64 sums (FP64 inputs)
    float hi[16], lo[16];              // FP32 (hi, lo) TwoSum pairs (FP32 inputs)
#pragma unroll
    for (int u = 0; u < 16; ++u) {
        acc[u] = 0.0;
        hi[u] = 0.f;
        lo[u] = 0.f;
    }
    for (int64_t k0 = k_begin; k0 < k_end; k0 += GR_KCHUNK) {
        __syncthreads();
        abt_stage<T>(A, lda, at, A_add, m, k0, k_end, sa);
        abt_stage<T>(B, ldb, bt, nullptr, n, k0, k_end, sb);
        __syncthreads();
#pragma unroll
        for (int u = 0; u < 16; ++u) {
            const int o = threadIdx.x + u * SS_THREADS;
            if (o < mn) {
                const int i = o / n, j = o - i * n;
                ACC s = ACC(0);
#pragma unroll 8
                for (int kk = 0; kk < GR_KCHUNK; ++kk) s = fma((ACC)sa[i][kk], (ACC)sb[j][kk], s);
                if constexpr (F32) {
                    float sum, err;
                    xrh_two_sum(hi[u], (float)s, sum, err);
                    hi[u] = sum;
                    lo[u] += err;
                } else {
                    acc[u] += (double)s;
                }
            }
        }
    }
#pragma unroll
    for (int u = 0; u < 16; ++u) {
        const int o = threadIdx.x + u * SS_THREADS;
        if (o >= mn) continue;
        if constexpr (F32) atomicAdd(C + o, alpha * xrh_f32_to_f64(__fadd_rn(hi[u], lo[u])));
        else atomicAdd(C + o, alpha * acc[u]);
    }
}

__global__ void __launch_bounds__(SS_THREADS) gram_kernel(const xrh_state_task* __restrict__ tasks, int n_tasks,
                                                          int which) {
    __shared__ double sa[64][GR_KCHUNK + 1], sb[64][GR_KCHUNK + 1];
    const xrh_state_task& T = tasks[find_task(tasks, n_tasks, blockIdx.x)];
    if (T.n <= 0 || T.n > 64) return;   // the host checks n; nothing is touched otherwise
    const int64_t K = T.K;
    const int64_t k_begin = (blockIdx.x - T.cta_begin) * (int64_t)SS_KSLICE;
    const int64_t k_end = k_begin + SS_KSLICE < K ? k_begin + SS_KSLICE : K;
    if (which == 0)
        abt_slice<double, double>(T.gT, T.n, true, T.gT32, T.n, T.z, K, false, T.n, k_begin, k_end, 1.0, T.G, sa, sb);
    else
        abt_slice<double, double>(T.zn, K, false, nullptr, T.n, T.zn, K, false, T.n, k_begin, k_end, 1.0, T.S, sa, sb);
}

template <typename T, typename ACC>
__global__ void __launch_bounds__(SS_THREADS) abt_kernel(int m, int n, int64_t K, const T* __restrict__ A,
                                                         int64_t lda, const T* __restrict__ B, int64_t ldb,
                                                         double alpha, double* __restrict__ C) {
    __shared__ T sa[64][GR_KCHUNK + 1], sb[64][GR_KCHUNK + 1];
    const int64_t k_begin = (int64_t)blockIdx.x * ABT_KSLICE;
    const int64_t k_end = k_begin + ABT_KSLICE < K ? k_begin + ABT_KSLICE : K;
    abt_slice<T, ACC>(A, lda, false, nullptr, m, B, ldb, false, n, k_begin, k_end, alpha, C, sa, sb);
}

// Many small-output products in one launch: task t owns CTAs [cta_begin, cta_begin +
// ceil(K / SS_KSLICE)) and adds alpha A B^T (m x n, row stride n) into C.
template <typename T, typename ACC>
__global__ void __launch_bounds__(SS_THREADS) abt_grouped_kernel(const xrh_abt_task* __restrict__ tasks, int n_tasks) {
    __shared__ T sa[64][GR_KCHUNK + 1], sb[64][GR_KCHUNK + 1];
    int lo = 0, hi = n_tasks - 1;
    const int64_t cta = blockIdx.x;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (tasks[mid].cta_begin <= cta) lo = mid; else hi = mid - 1;
    }
    const xrh_abt_task& Tk = tasks[lo];
    if (Tk.m <= 0 || Tk.m > 64 || Tk.n <= 0 || Tk.n > 64) return;   // checked by the host
    const int64_t k_begin = (cta - Tk.cta_begin) * (int64_t)ABT_KSLICE;
    const int64_t k_end = k_begin + ABT_KSLICE < Tk.K ? k_begin + ABT_KSLICE : Tk.K;
    abt_slice<T, ACC>(reinterpret_cast<const T*>(Tk.A), Tk.lda, (Tk.flags & 1) != 0, nullptr, (int)Tk.m,
                      reinterpret_cast<const T*>(Tk.B), Tk.ldb, (Tk.flags & 2) != 0, (int)Tk.n, k_begin, k_end,
                      Tk.alpha, Tk.C, sa, sb);
}

// out[i][k] = sum_j W[i][j] X[j][k] over this CTA's K slice: thread per column k (the column
// of X read through L1 n times, W by broadcast from shared memory), n independent FP64 chains.
// mode 0 (tangent): W = sym(G), X = z; t = g - W z; zn = z - eps t; sq += t^2.
// mode 1 (left):    W = M, X = zn; z = W zn.
template <int MODE>
__global__ void __launch_bounds__(SS_THREADS) rowmix_kernel(const xrh_state_task* __restrict__ tasks, int n_tasks,
                                                            double eps, double* __restrict__ sq) {
    __shared__ double w[64 * 64];
    __shared__ double red[SS_THREADS / 32];
    const xrh_state_task& T = tasks[find_task(tasks, n_tasks, blockIdx.x)];
    const int n = T.n;
    if (n <= 0 || n > 64) return;
    const int64_t K = T.K;
    for (int e = threadIdx.x; e < n * n; e += SS_THREADS) {
        const int i = e / n, j = e - i * n;
        w[e] = MODE == 0 ? 0.5 * (T.G[i * n + j] + T.G[j * n + i]) : T.M[e];
    }
    __syncthreads();
    const double* X = MODE == 0 ? T.z : T.zn;
    const int64_t k_begin = (blockIdx.x - T.cta_begin) * (int64_t)SS_KSLICE;
    const int64_t k_end = k_begin + SS_KSLICE < K ? k_begin + SS_KSLICE : K;
    double part = 0.0;
    // SS_THREADS / SS_KSLICE threads per column split the rows
    constexpr int RG = SS_THREADS / SS_KSLICE;
    const int64_t k = k_begin + (threadIdx.x % SS_KSLICE);
    const int r0 = threadIdx.x / SS_KSLICE;
    if (k < k_end) {
        for (int i = r0; i < n; i += RG) {
            double s0 = 0.0, s1 = 0.0;
            int j = 0;
            for (; j + 1 < n; j += 2) {
                s0 = fma(w[i * n + j], X[(int64_t)j * K + k], s0);
                s1 = fma(w[i * n + j + 1], X[(int64_t)(j + 1) * K + k], s1);
            }
            if (j < n) s0 = fma(w[i * n + j], X[(int64_t)j * K + k], s0);
            const double s = s0 + s1;
            if (MODE == 0) {
                double g = T.gT[k * n + i];
                if (T.gT32) g += (double)T.gT32[k * n + i];
                const double t = g - s;
                part = fma(t, t, part);
                T.zn[(int64_t)i * K + k] = X[(int64_t)i * K + k] - eps * t;
            } else {
                T.z[(int64_t)i * K + k] = s;
            }
        }
    }
    if (MODE == 0) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = part;
        __syncthreads();
        if (threadIdx.x == 0) {
            double t = 0.0;
            for (int q = 0; q < SS_THREADS / 32; ++q) t += red[q];
            if (t != 0.0) atomicAdd(sq, t);
        }
    }
}

// out = a b for n x n matrices in shared memory (row stride NS_MAX + 1)
__device__ __forceinline__ void ns_mul(const double (*a)[NS_MAX + 1], const double (*b)[NS_MAX + 1],
                                       double (*out)[NS_MAX + 1], int n) {
    for (int o = threadIdx.x; o < n * n; o += SS_THREADS) {
        const int i = o / n, j = o - i * n;
        double s = 0.0;
        for (int l = 0; l < n; ++l) s = fma(a[i][l], b[l][j], s);
        out[i][j] = s;
    }
}

// One CTA per task: M = S^-1/2 by the coupled Newton-Schulz iteration
//   Y0 = S, Z0 = I;  T = (3I - Z Y)/2;  Y <- Y T;  Z <- T Z   (Z -> S^-1/2 for |I - S| < 1).
__global__ void __launch_bounds__(SS_THREADS) inv_sqrt_kernel(const xrh_state_task* __restrict__ tasks, int iters) {
    __shared__ double buf[4][NS_MAX][NS_MAX + 1];
    const xrh_state_task& T = tasks[blockIdx.x];
    const int n = T.n;
    if (n <= 0 || n > NS_MAX) return;
    int y = 0, z = 1, t = 2, w = 3;
    for (int o = threadIdx.x; o < n * n; o += SS_THREADS) {
        const int i = o / n, j = o - i * n;
        buf[y][i][j] = T.S[o];
        buf[z][i][j] = i == j ? 1.0 : 0.0;
    }
    __syncthreads();
    for (int it = 0; it < iters; ++it) {
        ns_mul(buf[z], buf[y], buf[w], n);
        __syncthreads();
        for (int o = threadIdx.x; o < n * n; o += SS_THREADS) {
            const int i = o / n, j = o - i * n;
            buf[t][i][j] = 0.5 * ((i == j ? 3.0 : 0.0) - buf[w][i][j]);
        }
        __syncthreads();
        ns_mul(buf[y], buf[t], buf[w], n);
        __syncthreads();
        int s = y; y = w; w = s;
        ns_mul(buf[t], buf[z], buf[w], n);
        __syncthreads();
        s = z; z = w; w = s;
    }
    for (int o = threadIdx.x; o < n * n; o += SS_THREADS) T.M[o] = buf[z][o / n][o % n];
}

int check(const xrh_state_task* tasks, int n_tasks, int64_t total_ctas) {
    if (n_tasks < 0 || total_ctas < 0) return XRH_ERR_ARG;
    if (n_tasks > 0 && !tasks) return XRH_ERR_ARG;
    if (total_ctas > 0x7fffffffLL) return XRH_ERR_CAPACITY;
    return XRH_OK;
}

}  // namespace

extern "C" int xrh_state_ctas(int64_t K) { return (int)((K + SS_KSLICE - 1) / SS_KSLICE); }
extern "C" int xrh_abt_ctas(int64_t K) { return (int)((K + ABT_KSLICE - 1) / ABT_KSLICE); }

extern "C" int xrh_gram_grouped(const xrh_state_task* tasks_dev, int n_tasks, int64_t total_ctas, int which,
                                void* stream) {
    const int st = check(tasks_dev, n_tasks, total_ctas);
    if (st != XRH_OK) return st;
    if (which != 0 && which != 1) return XRH_ERR_ARG;
    if (n_tasks == 0 || total_ctas == 0) return XRH_OK;
    gram_kernel<<<(unsigned)total_ctas, SS_THREADS, 0, (cudaStream_t)stream>>>(tasks_dev, n_tasks, which);
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}

extern "C" int xrh_tangent_step(const xrh_state_task* tasks_dev, int n_tasks, int64_t total_ctas, double eps,
                                double* sq_dev, void* stream) {
    const int st = check(tasks_dev, n_tasks, total_ctas);
    if (st != XRH_OK) return st;
    if (!sq_dev) return XRH_ERR_ARG;
    if (n_tasks == 0 || total_ctas == 0) return XRH_OK;
    rowmix_kernel<0><<<(unsigned)total_ctas, SS_THREADS, 0, (cudaStream_t)stream>>>(tasks_dev, n_tasks, eps, sq_dev);
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}

extern "C" int xrh_left_multiply(const xrh_state_task* tasks_dev, int n_tasks, int64_t total_ctas, void* stream) {
    const int st = check(tasks_dev, n_tasks, total_ctas);
    if (st != XRH_OK) return st;
    if (n_tasks == 0 || total_ctas == 0) return XRH_OK;
    rowmix_kernel<1><<<(unsigned)total_ctas, SS_THREADS, 0, (cudaStream_t)stream>>>(tasks_dev, n_tasks, 0.0, nullptr);
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}

extern "C" int xrh_inv_sqrt_small(const xrh_state_task* tasks_dev, int n_tasks, int iters, void* stream) {
    const int st = check(tasks_dev, n_tasks, n_tasks);
    if (st != XRH_OK) return st;
    if (iters < 0) return XRH_ERR_ARG;
    if (n_tasks == 0) return XRH_OK;
    inv_sqrt_kernel<<<(unsigned)n_tasks, SS_THREADS, 0, (cudaStream_t)stream>>>(tasks_dev, iters);
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}

extern "C" int xrh_abt_small(int precision, int m, int n, int64_t K, const void* A_dev, int64_t lda,
                             const void* B_dev, int64_t ldb, double alpha, double* C_dev, void* stream) {
    if (m < 0 || n < 0 || K < 0 || m > 64 || n > 64) return XRH_ERR_ARG;
    if (m == 0 || n == 0 || K == 0) return XRH_OK;
    if (!A_dev || !B_dev || !C_dev || lda < K || ldb < K) return XRH_ERR_ARG;
    const int64_t ctas = (K + ABT_KSLICE - 1) / ABT_KSLICE;
    if (ctas > 0x7fffffffLL) return XRH_ERR_CAPACITY;
    cudaStream_t s = (cudaStream_t)stream;
    if (precision == XRH_FP64)
        abt_kernel<double, double><<<(unsigned)ctas, SS_THREADS, 0, s>>>(m, n, K, (const double*)A_dev, lda,
                                                                        (const double*)B_dev, ldb, alpha, C_dev);
    else if (precision == XRH_FP32)
        abt_kernel<float, float><<<(unsigned)ctas, SS_THREADS, 0, s>>>(m, n, K, (const float*)A_dev, lda,
                                                                      (const float*)B_dev, ldb, alpha, C_dev);
    else
        return XRH_ERR_ARG;
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}

extern "C" int xrh_abt_grouped(int precision, const xrh_abt_task* tasks_dev, int n_tasks, int64_t total_ctas,
                               void* stream) {
    if (n_tasks < 0 || total_ctas < 0) return XRH_ERR_ARG;
    if (n_tasks == 0 || total_ctas == 0) return XRH_OK;
    if (!tasks_dev) return XRH_ERR_ARG;
    if (total_ctas > 0x7fffffffLL) return XRH_ERR_CAPACITY;
    cudaStream_t s = (cudaStream_t)stream;
    if (precision == XRH_FP64)
        abt_grouped_kernel<double, double><<<(unsigned)total_ctas, SS_THREADS, 0, s>>>(tasks_dev, n_tasks);
    else if (precision == XRH_FP32)
        abt_grouped_kernel<float, float><<<(unsigned)total_ctas, SS_THREADS, 0, s>>>(tasks_dev, n_tasks);
    else
        return XRH_ERR_ARG;
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}
