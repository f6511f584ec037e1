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
constexpr int SS_KSLICE = 256;     // K columns per CTA (matches the host's CTA count)
constexpr int GR_KCHUNK = 32;      // columns staged per step in the Gram kernel
constexpr int TS_KCHUNK = 8;       // columns staged per step in the tangent / left kernels
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
// ACC is the type of the per-chunk sums; with FP32 inputs the chunk sums (GR_KCHUNK products)
// are folded into FP32 (hi, lo) pairs by TwoSum, keeping the FP64 pipe out of the loop.
// With AT, A is given transposed (K x m, row stride m) as AT_main + AT_add (AT_add may be null),
// staged with loads that run along the contiguous chunk.
template <typename T, typename ACC, bool AT>
__device__ __forceinline__ void abt_slice(const T* __restrict__ A, int64_t lda, const float* __restrict__ A_add,
                                          int m, const T* __restrict__ B, int64_t ldb, int n, int64_t k_begin,
                                          int64_t k_end, double alpha, double* __restrict__ C,
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
        for (int e = threadIdx.x; e < 64 * GR_KCHUNK; e += SS_THREADS) {
            const int i = e / GR_KCHUNK, kk = e - i * GR_KCHUNK;
            const int64_t k = k0 + kk;
            const bool kin = k < k_end;
            if (!AT && i < m) sa[i][kk] = kin ? A[(int64_t)i * lda + k] : T(0);
            if (i < n) sb[i][kk] = kin ? B[(int64_t)i * ldb + k] : T(0);
        }
        if (AT) {
            for (int e = threadIdx.x; e < m * GR_KCHUNK; e += SS_THREADS) {
                const int kk = e / m, i = e - kk * m;
                const int64_t k = k0 + kk;
                T v = T(0);
                if (k < k_end) {
                    v = A[k * m + i];
                    if (A_add) v += (T)A_add[k * m + i];
                }
                sa[i][kk] = v;
            }
        }
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
        abt_slice<double, double, true>(T.gT, T.n, T.gT32, T.n, T.z, K, T.n, k_begin, k_end, 1.0, T.G, sa, sb);
    else
        abt_slice<double, double, false>(T.zn, K, nullptr, T.n, T.zn, K, T.n, k_begin, k_end, 1.0, T.S, sa, sb);
}

template <typename T, typename ACC>
__global__ void __launch_bounds__(SS_THREADS) abt_kernel(int m, int n, int64_t K, const T* __restrict__ A,
                                                         int64_t lda, const T* __restrict__ B, int64_t ldb,
                                                         double alpha, double* __restrict__ C) {
    __shared__ T sa[64][GR_KCHUNK + 1], sb[64][GR_KCHUNK + 1];
    const int64_t k_begin = (int64_t)blockIdx.x * SS_KSLICE;
    const int64_t k_end = k_begin + SS_KSLICE < K ? k_begin + SS_KSLICE : K;
    abt_slice<T, ACC, false>(A, lda, nullptr, m, B, ldb, n, k_begin, k_end, alpha, C, sa, sb);
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
    const int64_t k_begin = (cta - Tk.cta_begin) * (int64_t)SS_KSLICE;
    const int64_t k_end = k_begin + SS_KSLICE < Tk.K ? k_begin + SS_KSLICE : Tk.K;
    abt_slice<T, ACC, false>(reinterpret_cast<const T*>(Tk.A), Tk.lda, nullptr, (int)Tk.m,
                             reinterpret_cast<const T*>(Tk.B), Tk.ldb, (int)Tk.n, k_begin, k_end, Tk.alpha, Tk.C, sa,
                             sb);
}

// out[i][k] = sum_j W[i][j] X[j][k] over this CTA's K slice, X (and g) staged TS_KCHUNK columns
// at a time; thread (row group, column) = (t / TS_KCHUNK, t % TS_KCHUNK), rows i = row group +
// (SS_THREADS / TS_KCHUNK) r.
// mode 0 (tangent): W = sym(G), X = z; t = g - W z; zn = z - eps t; sq += t^2.
// mode 1 (left):    W = M, X = zn; z = W zn.
template <int MODE>
__global__ void __launch_bounds__(SS_THREADS) rowmix_kernel(const xrh_state_task* __restrict__ tasks, int n_tasks,
                                                            double eps, double* __restrict__ sq) {
    __shared__ double w[64 * 64];
    __shared__ double xs[64][TS_KCHUNK];
    __shared__ double gs[TS_KCHUNK][65];
    const xrh_state_task& T = tasks[find_task(tasks, n_tasks, blockIdx.x)];
    const int n = T.n;
    if (n <= 0 || n > 64) return;
    const int64_t K = T.K;
    for (int e = threadIdx.x; e < n * n; e += SS_THREADS) {
        const int i = e / n, j = e - i * n;
        w[e] = MODE == 0 ? 0.5 * (T.G[i * n + j] + T.G[j * n + i]) : T.M[e];
    }
    const double* X = MODE == 0 ? T.z : T.zn;
    const int64_t k_begin = (blockIdx.x - T.cta_begin) * (int64_t)SS_KSLICE;
    const int64_t k_end = k_begin + SS_KSLICE < K ? k_begin + SS_KSLICE : K;
    const int kk = threadIdx.x & (TS_KCHUNK - 1);
    const int r0 = threadIdx.x / TS_KCHUNK;
    double part = 0.0;
    for (int64_t k0 = k_begin; k0 < k_end; k0 += TS_KCHUNK) {
        __syncthreads();
        for (int e = threadIdx.x; e < n * TS_KCHUNK; e += SS_THREADS) {
            const int j = e / TS_KCHUNK, c = e - j * TS_KCHUNK;
            const int64_t k = k0 + c;
            xs[j][c] = k < k_end ? X[(int64_t)j * K + k] : 0.0;
        }
        if (MODE == 0) {
            for (int e = threadIdx.x; e < n * TS_KCHUNK; e += SS_THREADS) {
                const int c = e / n, i = e - c * n;
                const int64_t k = k0 + c;
                double v = 0.0;
                if (k < k_end) {
                    v = T.gT[k * n + i];
                    if (T.gT32) v += (double)T.gT32[k * n + i];
                }
                gs[c][i] = v;
            }
        }
        __syncthreads();
        const int64_t k = k0 + kk;
        if (k < k_end) {
            for (int i = r0; i < n; i += SS_THREADS / TS_KCHUNK) {
                double s = 0.0;
                for (int j = 0; j < n; ++j) s = fma(w[i * n + j], xs[j][kk], s);
                if (MODE == 0) {
                    const double t = gs[kk][i] - s;
                    part = fma(t, t, part);
                    T.zn[(int64_t)i * K + k] = xs[i][kk] - eps * t;
                } else {
                    T.z[(int64_t)i * K + k] = s;
                }
            }
        }
    }
    if (MODE == 0) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
        if ((threadIdx.x & 31) == 0 && part != 0.0) atomicAdd(sq, part);
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
    const int64_t ctas = (K + SS_KSLICE - 1) / SS_KSLICE;
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
