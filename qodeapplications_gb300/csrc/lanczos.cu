// FP64 building blocks of the Lanczos eigensolver for the lowest eigenpairs of the
// excitonic Hamiltonian (the reference diagonalises the full H with scipy.linalg.eig,
// hermitian-XRCC/mains/workflow.py:229 and StateSpaceOptimizer/state_gradients.py:107; only
// the lowest eigenpair is used, so a Krylov method on the GPU replaces the dense solve).
//
//   xrh_gemv_rows:  y[i] = alpha * sum_j A[i*lda + j] x[j] + beta * y[i]   (warp per row)
//   xrh_gemv_cols:  y[j] += sum_i c[i] * scale * A[i*lda + j]              (thread per column)
//   xrh_lanczos_normalize: beta[k] = ||w||, v = w / beta[k]  (one CTA; the norm stays on the
//       device so the whole Krylov loop can be replayed as one CUDA graph)
//   xrh_gemv_rows_split / xrh_lanczos_normalize_split: the same for long vectors, columns split
//       over CTAs with partials added in a fixed order by a second launch
// All FP64: the eigensolve is kept in double precision on every precision path.
#include <cooperative_groups.h>

#include "xrh_common.cuh"

#include <mutex>

namespace {
// Host-side launch state of the Lanczos loops, one record per device ordinal: function
// attributes (the raised dynamic shared-memory limits, the non-portable cluster size) are
// per device, and so is the cluster shape chosen for a sector.  One mutex guards all records
// (the first eager call of a shape takes it; later calls only read under it).
constexpr int kLzMaxDevices = 64;
struct LzChoice { int n, m, max_ctas, nb, h_smem; size_t smem; bool ok; };
struct LzDeviceState {
    size_t coop_smem_set = 48 * 1024;
    size_t cluster_smem_set = 48 * 1024;
    int nonportable = -1;
    LzChoice cache[32];
    int n_cache = 0;
};
std::mutex g_lz_mutex;
LzDeviceState g_lz_state[kLzMaxDevices];
}  // namespace

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

// Column-split forms for few rows over long vectors (the matrix-free Lanczos of a product space
// of 10^5..10^6 states, where a warp per row leaves most SMs idle).  A CTA takes SPLIT_COLS
// columns: pass 1 writes one partial per (CTA, row), pass 2 sums the partials of a row in CTA
// order, so results do not depend on scheduling.
constexpr int SPLIT_COLS = 2048;

__global__ void __launch_bounds__(256) gemv_rows_partial_kernel(int64_t rows, int64_t cols,
                                                              const double* __restrict__ A, int64_t lda,
                                                              const double* __restrict__ x,
                                                              double* __restrict__ partial) {
    __shared__ double xs[SPLIT_COLS];
    const int64_t c0 = (int64_t)blockIdx.x * SPLIT_COLS;
    const int cn = (int)min((int64_t)SPLIT_COLS, cols - c0);
    for (int j = threadIdx.x; j < cn; j += blockDim.x) xs[j] = x[c0 + j];
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int64_t r = warp; r < rows; r += (blockDim.x >> 5)) {
        const double* a = A + r * lda + c0;
        double s0 = 0.0, s1 = 0.0;
        int j = lane;
        for (; j + 32 < cn; j += 64) {
            s0 = fma(a[j], xs[j], s0);
            s1 = fma(a[j + 32], xs[j + 32], s1);
        }
        if (j < cn) s0 = fma(a[j], xs[j], s0);
        double s = s0 + s1;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) partial[(int64_t)blockIdx.x * rows + r] = s;
    }
}

__global__ void __launch_bounds__(256) gemv_rows_reduce_kernel(int64_t rows, int64_t n_parts,
                                                             const double* __restrict__ partial, double alpha,
                                                             double beta, double* __restrict__ y) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    double s = 0.0;
    for (int64_t b = 0; b < n_parts; ++b) s += partial[b * rows + r];
    y[r] = alpha * s + (beta == 0.0 ? 0.0 : beta * y[r]);
}

__global__ void __launch_bounds__(256) sumsq_partial_kernel(int64_t n, const double* __restrict__ w,
                                                          double* __restrict__ partial) {
    __shared__ double red[8];
    const int64_t c0 = (int64_t)blockIdx.x * SPLIT_COLS;
    const int cn = (int)min((int64_t)SPLIT_COLS, n - c0);
    double s = 0.0;
    for (int j = threadIdx.x; j < cn; j += blockDim.x) s = fma(w[c0 + j], w[c0 + j], s);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += red[i];
        partial[blockIdx.x] = t;
    }
}

// Every CTA sums the partials in the same order (lane-strided, then a fixed shuffle tree), so
// all CTAs scale by the same beta; CTA 0 stores it.
__global__ void __launch_bounds__(256) scale_by_norm_kernel(int64_t n, int64_t n_parts,
                                                          const double* __restrict__ partial,
                                                          const double* __restrict__ w, double* __restrict__ v,
                                                          double* __restrict__ beta_out) {
    __shared__ double bsh;
    if (threadIdx.x < 32) {
        double s = 0.0;
        for (int64_t b = threadIdx.x; b < n_parts; b += 32) s += partial[b];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (threadIdx.x == 0) bsh = sqrt(s);
    }
    __syncthreads();
    const double b = bsh;
    const double inv = b > 0.0 ? 1.0 / b : 0.0;
    const int64_t c0 = (int64_t)blockIdx.x * SPLIT_COLS;
    const int cn = (int)min((int64_t)SPLIT_COLS, n - c0);
    for (int j = threadIdx.x; j < cn; j += blockDim.x) v[c0 + j] = w[c0 + j] * inv;
    if (blockIdx.x == 0 && threadIdx.x == 0) *beta_out = b;
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


// Many row GEMVs in one launch: CTA b (8 warps, a row each) belongs to the task with the last
// row_begin <= 8 b (task row ranges padded to multiples of 8).  With beta == 1 the result is
// added atomically, so tasks may share output rows.
__global__ void __launch_bounds__(256) gemv_rows_grouped_kernel(const xrh_gemv_task* __restrict__ tasks,
                                                              int n_tasks) {
    const int64_t row8 = (int64_t)blockIdx.x * 8;
    int lo = 0, hi = n_tasks - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (tasks[mid].row_begin <= row8) lo = mid; else hi = mid - 1;
    }
    const xrh_gemv_task& T = tasks[lo];
    const int64_t row = row8 - T.row_begin + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (row >= T.rows) return;
    const double* a = T.A + row * T.lda;
    double s = 0.0;
    for (int64_t j = lane; j < T.cols; j += 32) s = fma(a[j], T.x[j], s);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) {
        if (T.beta == 1.0) atomicAdd(T.y + row, T.alpha * s);
        else T.y[row] = T.alpha * s + (T.beta == 0.0 ? 0.0 : T.beta * T.y[row]);
    }
}

// ---- the Krylov loop over many CTAs (cooperative launch) ----------------------------------
// The FP64 rate of one SM bounds the single-CTA loop; here the rows of H, V and w are split
// over the CTAs of one cooperative launch and every step takes three grid barriers:
//   w_R = H_R V[j]; partial dots V[i]_R . w_R (i <= j)                     | barrier
//   c = sum over CTAs; w_R -= c V_R; partial dots again and partial |w_R|^2 | barrier
//   c' = sum; w_R -= c' V_R; beta^2 = |w|^2 - |c'|^2; V[j+1]_R = w_R/beta  | barrier
// (after the first pass w is orthogonal to V[0..j] up to rounding, so the second pass removes
// only |c'| ~ 1e-16 |w| and beta^2 = |w|^2 - |c'|^2 is the norm after it to that accuracy).
// The CTA keeps its own rows of every V[i] in shared memory and stages V[j] whole before the
// product, so the only global traffic per step is H_R, V[j] and the partial sums.  Partial
// sums are reduced by warps in a fixed order, identical in every CTA, so all CTAs hold the same
// coefficients and results do not depend on scheduling.  V is written by every CTA and read
// by all, so its global reads bypass L1 (ld.global.cg).  Barrier k waits until a counter
// reaches (k+1) * gridDim.x; a wait that exceeds wait_limit polls (LC_WAIT_LIMIT unless the
// caller of xrh_lanczos_coop_bounded gives another) sets XRH_ERR_TIMEOUT in *status and the CTA
// returns; every later barrier of the other CTAs then returns too.
constexpr int LC_THREADS = 512;
constexpr int LC_WARPS = LC_THREADS / 32;
constexpr int LC_RPW = 4;                        // rows of H a warp multiplies at once
constexpr int LC_MAX_CTAS = 256;
constexpr int LC_ROWS_PER_CTA = 4;
constexpr long long LC_WAIT_LIMIT = 1LL << 22;   // ~ seconds of polls

__device__ __forceinline__ unsigned int ld_acquire_u32(const unsigned int* p) {
    unsigned int v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Returns false (all threads of the CTA) when the wait gave up or another CTA already failed.
__device__ __forceinline__ bool grid_barrier(unsigned int* count, unsigned int target, int32_t* status,
                                             long long wait_limit) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        __threadfence();
        atomicAdd(count, 1u);
        long long it = 0;
        while (ld_acquire_u32(count) < target) {
            if (++it > wait_limit) { ok = 0; break; }
            __nanosleep(20);
        }
        if (!ok) atomicExch(status, XRH_ERR_TIMEOUT);
        if (ok && *(volatile int32_t*)status != XRH_OK) ok = 0;
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// c[i] = sum_q part[i * nb + q] for i < cnt, warp per i, lanes over q, fixed shuffle tree.
__device__ __forceinline__ void reduce_partials(const double* __restrict__ part, unsigned int nb, int cnt,
                                                double* __restrict__ c) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int i = warp; i < cnt; i += LC_WARPS) {
        double s = 0.0;
        for (unsigned int q = lane; q < nb; q += 32) s += __ldcg(part + (int64_t)i * nb + q);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) c[i] = s;
    }
}

// Dynamic shared memory: Vs [(m + 1) * rows_max] (own rows of V), w [rows_max], c [m + 2],
// then, when stage_v, v [n] (V[j] whole).
__global__ void __launch_bounds__(LC_THREADS) lanczos_coop_kernel(int64_t n, int m, const double* __restrict__ H,
                                                                int64_t ld, const double* __restrict__ v0,
                                                                double* __restrict__ V, double* __restrict__ alpha,
                                                                double* __restrict__ beta, double* __restrict__ part,
                                                                unsigned int* count, int32_t* status, int rows_max,
                                                                int stage_v, long long wait_limit) {
    extern __shared__ double sm[];
    const unsigned int nb = gridDim.x, b = blockIdx.x;
    const int64_t r0 = (int64_t)b * n / nb, r1 = (int64_t)(b + 1) * n / nb;
    const int nr = (int)(r1 - r0);
    const int ms = m + 2;
    double* Vs = sm;                                  // [m + 1][rows_max]
    double* w = Vs + (int64_t)(m + 1) * rows_max;     // [rows_max]
    double* c = w + rows_max;                         // [m + 2]
    double* vst = c + ms;                             // [n] when stage_v
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    double* p1 = part;                                // [m + 2][nb]: pass-1 dots
    double* p2 = part + (int64_t)ms * nb;             // [m + 2][nb]: pass-2 dots, then |w|^2 at row j + 1
    unsigned int bar = 0;
    // 16-byte loads of H rows and of V[j] (V rows start at multiples of n; the staged copy
    // follows c, 16-byte aligned when m is even)
    const bool vec2 = (n % 2 == 0) && (ld % 2 == 0) && (reinterpret_cast<uintptr_t>(H) % 16 == 0) &&
                      (reinterpret_cast<uintptr_t>(V) % 16 == 0) &&
                      (!stage_v || reinterpret_cast<uintptr_t>(vst) % 16 == 0);
    for (int r = tid; r < nr; r += LC_THREADS) {
        const double x = v0[r0 + r];
        V[r0 + r] = x;
        Vs[r] = x;
    }
    if (!grid_barrier(count, ++bar * nb, status, wait_limit)) return;
    for (int j = 0; j < m; ++j) {
        const double* vj = V + (int64_t)j * n;
        if (stage_v) {
            for (int64_t k = tid; k < n; k += LC_THREADS) vst[k] = __ldcg(vj + k);
            __syncthreads();
        }
        // w_R = H_R V[j]: a warp multiplies LC_RPW rows at once, so that one load of V[j] serves
        // them all, with 16-byte loads when the rows allow it: the loop is bound by the bytes in
        // flight per SM, which one 8-byte row stream per warp keeps far below what HBM takes
        for (int rb = warp * LC_RPW; rb < nr; rb += LC_WARPS * LC_RPW) {
            const int nrow = (nr - rb < LC_RPW) ? nr - rb : LC_RPW;
            const double* h[LC_RPW];
#pragma unroll
            for (int q = 0; q < LC_RPW; ++q) h[q] = H + (r0 + rb + (q < nrow ? q : nrow - 1)) * ld;
            double s[LC_RPW][2];
#pragma unroll
            for (int q = 0; q < LC_RPW; ++q) s[q][0] = s[q][1] = 0.0;
            if (vec2) {
                const int64_t n2 = n >> 1;
                const double2* x2 = stage_v ? reinterpret_cast<const double2*>(vst) : reinterpret_cast<const double2*>(vj);
#pragma unroll 2
                for (int64_t k = lane; k < n2; k += 32) {
                    const double2 x = stage_v ? x2[k] : __ldcg(x2 + k);
#pragma unroll
                    for (int q = 0; q < LC_RPW; ++q) {
                        const double2 y = __ldg(reinterpret_cast<const double2*>(h[q]) + k);
                        s[q][0] = fma(y.x, x.x, s[q][0]);
                        s[q][1] = fma(y.y, x.y, s[q][1]);
                    }
                }
            } else {
                for (int64_t k = lane; k < n; k += 32) {
                    const double x = stage_v ? vst[k] : __ldcg(vj + k);
#pragma unroll
                    for (int q = 0; q < LC_RPW; ++q) s[q][0] = fma(__ldg(h[q] + k), x, s[q][0]);
                }
            }
#pragma unroll
            for (int q = 0; q < LC_RPW; ++q) {
                double t = s[q][0] + s[q][1];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
                if (lane == 0 && q < nrow) w[rb + q] = t;
            }
        }
        double a = 0.0;
        double cc2 = 0.0;
        for (int pass = 0; pass < 2; ++pass) {
            double* pp = pass == 0 ? p1 : p2;
            __syncthreads();
            // partial dots of w_R with V[i]_R (i <= j), and after pass 1 also |w_R|^2 (row j + 1)
            const int cnt = j + 1 + pass;
            for (int i = warp; i < cnt; i += LC_WARPS) {
                const double* vi = Vs + (int64_t)i * rows_max;
                double s = 0.0;
                if (i <= j)
                    for (int r = lane; r < nr; r += 32) s = fma(vi[r], w[r], s);
                else
                    for (int r = lane; r < nr; r += 32) s = fma(w[r], w[r], s);
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
                if (lane == 0) pp[(int64_t)i * nb + b] = s;
            }
            if (!grid_barrier(count, ++bar * nb, status, wait_limit)) return;
            reduce_partials(pp, nb, cnt, c);
            __syncthreads();
            a += c[j];
            for (int r = tid; r < nr; r += LC_THREADS) {
                double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
                int i = 0;
                for (; i + 3 <= j; i += 4) {
                    s0 = fma(c[i], Vs[(int64_t)i * rows_max + r], s0);
                    s1 = fma(c[i + 1], Vs[(int64_t)(i + 1) * rows_max + r], s1);
                    s2 = fma(c[i + 2], Vs[(int64_t)(i + 2) * rows_max + r], s2);
                    s3 = fma(c[i + 3], Vs[(int64_t)(i + 3) * rows_max + r], s3);
                }
                for (; i <= j; ++i) s0 = fma(c[i], Vs[(int64_t)i * rows_max + r], s0);
                w[r] -= (s0 + s1) + (s2 + s3);
            }
            if (pass == 1) {
                for (int i = 0; i <= j; ++i) cc2 = fma(c[i], c[i], cc2);
                cc2 = c[j + 1] - cc2;          // |w after pass 2|^2
            }
        }
        const double bj = sqrt(cc2 > 0.0 ? cc2 : 0.0);
        const double inv = bj > 0.0 ? 1.0 / bj : 0.0;
        double* vn = V + (int64_t)(j + 1) * n + r0;
        double* vsn = Vs + (int64_t)(j + 1) * rows_max;
        for (int r = tid; r < nr; r += LC_THREADS) {
            const double x = w[r] * inv;
            vn[r] = x;
            vsn[r] = x;
        }
        if (b == 0 && tid == 0) {
            alpha[j] = a;
            beta[j] = bj;
        }
        if (!grid_barrier(count, ++bar * nb, status, wait_limit)) return;
    }
}


// ---- the Krylov loop in one thread-block cluster ----------------------------------------
// For sectors whose rows of H fit in the shared memory of a cluster (up to 16 CTAs, one per
// SM), the loop runs inside one cluster: CTA b owns rows [r0, r1) of H (kept in its shared
// memory for the whole loop when they fit), of V and of w, and a full copy of V[j].  Partial
// dot products and the slices of V[j+1] are exchanged through distributed shared memory at
// hardware cluster barriers (three per step: after each Gram-Schmidt pass's partial dots and
// after V[j+1]); every CTA sums the partials in the same CTA order, so all hold identical
// coefficients.  Same recurrence as lanczos_coop_kernel (beta^2 = |w|^2 - |c'|^2 after the
// second pass).
namespace cg = cooperative_groups;
constexpr int LK_THREADS = 512;
constexpr int LK_WARPS = LK_THREADS / 32;

__global__ void __launch_bounds__(LK_THREADS, 1) lanczos_cluster_kernel(int n, int m, const double* __restrict__ H,
                                                                   int64_t ld, const double* __restrict__ v0,
                                                                   double* __restrict__ V, double* __restrict__ alpha,
                                                                   double* __restrict__ beta, int rows_max, int h_smem) {
    cg::cluster_group cluster = cg::this_cluster();
    const unsigned int nb = cluster.num_blocks(), b = cluster.block_rank();
    extern __shared__ __align__(16) double lsm[];
    const int r0 = (int)((int64_t)b * n / nb), r1 = (int)((int64_t)(b + 1) * n / nb);
    const int nr = r1 - r0;
    const int ms = m + 2;
    double* vfull = lsm;                              // [n]      V[j] whole
    double* Vs = vfull + n;                           // [m+1][rows_max] own rows of V
    double* w = Vs + (int64_t)(m + 1) * rows_max;     // [rows_max]
    double* vslice = w + rows_max;                    // [rows_max] own rows of V[j+1] for the peers
    double* pa = vslice + rows_max;                   // [ms]     pass-1 partial dots of this CTA
    double* pb = pa + ms;                             // [ms]     pass-2 partial dots (+ |w|^2)
    double* c = pb + ms;                              // [ms]     summed coefficients
    double* Hs = c + ms;                              // [nr][n]  own rows of H (when h_smem)
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (h_smem)
        for (int64_t e = tid; e < (int64_t)nr * n; e += LK_THREADS) {
            const int r = (int)(e / n), k = (int)(e - (int64_t)r * n);
            Hs[e] = H[(int64_t)(r0 + r) * ld + k];
        }
    for (int k = tid; k < n; k += LK_THREADS) vfull[k] = v0[k];
    for (int r = tid; r < nr; r += LK_THREADS) {
        Vs[r] = v0[r0 + r];
        V[r0 + r] = v0[r0 + r];
    }
    __syncthreads();
    for (int j = 0; j < m; ++j) {
        for (int r = warp; r < nr; r += LK_WARPS) {
            const double* h = h_smem ? Hs + (int64_t)r * n : H + (int64_t)(r0 + r) * ld;
            // four independent chains (the FP64 latency, not its rate, bounds this loop)
            double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
            int k = lane;
            for (; k + 96 < n; k += 128) {
                s0 = fma(h[k], vfull[k], s0);
                s1 = fma(h[k + 32], vfull[k + 32], s1);
                s2 = fma(h[k + 64], vfull[k + 64], s2);
                s3 = fma(h[k + 96], vfull[k + 96], s3);
            }
            for (; k < n; k += 32) s0 = fma(h[k], vfull[k], s0);
            double s = (s0 + s1) + (s2 + s3);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            if (lane == 0) w[r] = s;
        }
        double a = 0.0, cc2 = 0.0;
        for (int pass = 0; pass < 2; ++pass) {
            double* pp = pass == 0 ? pa : pb;
            const int cnt = j + 1 + pass;
            __syncthreads();
            for (int i = warp; i < cnt; i += LK_WARPS) {
                double s = 0.0;
                if (i <= j)
                    for (int r = lane; r < nr; r += 32) s = fma(Vs[(int64_t)i * rows_max + r], w[r], s);
                else
                    for (int r = lane; r < nr; r += 32) s = fma(w[r], w[r], s);
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
                if (lane == 0) pp[i] = s;
            }
            cluster.sync();
            // c[i] = sum over the CTAs: warp per i, lane q reads CTA q's partial (one
            // distributed-shared-memory round trip), fixed shuffle tree (same order everywhere)
            for (int i = warp; i < cnt; i += LK_WARPS) {
                double s = lane < (int)nb ? cluster.map_shared_rank(pp, (unsigned int)lane)[i] : 0.0;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
                if (lane == 0) c[i] = s;
            }
            __syncthreads();
            if (pass == 1 && warp == LK_WARPS - 1) {
                // |c'|^2 by one warp (lanes over i, fixed shuffle tree) into c[m + 1], read after
                // the barrier below the pass loop
                double q = 0.0;
                for (int i = lane; i <= j; i += 32) q = fma(c[i], c[i], q);
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) q += __shfl_xor_sync(0xffffffffu, q, o);
                if (lane == 0) c[m + 1] = c[j + 1] - q;
            }
            a += c[j];
            for (int r = tid; r < nr; r += LK_THREADS) {
                double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
                int i = 0;
                for (; i + 3 <= j; i += 4) {
                    s0 = fma(c[i], Vs[(int64_t)i * rows_max + r], s0);
                    s1 = fma(c[i + 1], Vs[(int64_t)(i + 1) * rows_max + r], s1);
                    s2 = fma(c[i + 2], Vs[(int64_t)(i + 2) * rows_max + r], s2);
                    s3 = fma(c[i + 3], Vs[(int64_t)(i + 3) * rows_max + r], s3);
                }
                for (; i <= j; ++i) s0 = fma(c[i], Vs[(int64_t)i * rows_max + r], s0);
                w[r] -= (s0 + s1) + (s2 + s3);
            }
        }
        __syncthreads();
        cc2 = c[m + 1];
        const double bj = sqrt(cc2 > 0.0 ? cc2 : 0.0);
        const double inv = bj > 0.0 ? 1.0 / bj : 0.0;
        for (int r = tid; r < nr; r += LK_THREADS) {
            const double x = w[r] * inv;
            Vs[(int64_t)(j + 1) * rows_max + r] = x;
            vslice[r] = x;
            V[(int64_t)(j + 1) * n + r0 + r] = x;
        }
        if (b == 0 && tid == 0) {
            alpha[j] = a;
            beta[j] = bj;
        }
        cluster.sync();
        for (int k = tid; k < n; k += LK_THREADS) {
            // owner of row k: the largest q with q n / nb <= k
            unsigned int q = (unsigned int)(((int64_t)k * nb) / n);
            while (q + 1 < nb && (int)((int64_t)(q + 1) * n / nb) <= k) ++q;
            while (q > 0 && (int)((int64_t)q * n / nb) > k) --q;
            vfull[k] = cluster.map_shared_rank(vslice, q)[k - (int)((int64_t)q * n / nb)];
        }
        // vslice is rewritten at the end of the next step, two cluster barriers later
        __syncthreads();
    }
    cluster.sync();                                   // peers may still read this CTA's smem
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

extern "C" int xrh_gemv_rows_grouped(const xrh_gemv_task* tasks_dev, int n_tasks, int64_t total_rows8,
                                     void* stream) {
    if (n_tasks < 0 || total_rows8 < 0 || (total_rows8 & 7)) return XRH_ERR_ARG;
    if (n_tasks == 0 || total_rows8 == 0) return XRH_OK;
    if (!tasks_dev) return XRH_ERR_ARG;
    if (total_rows8 / 8 > 0x7fffffffLL) return XRH_ERR_CAPACITY;
    gemv_rows_grouped_kernel<<<(unsigned)(total_rows8 / 8), 256, 0, (cudaStream_t)stream>>>(tasks_dev, n_tasks);
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

extern "C" int64_t xrh_gemv_split_work(int64_t rows, int64_t cols) {
    if (rows < 0 || cols < 0) return -1;
    return ((cols + SPLIT_COLS - 1) / SPLIT_COLS) * (rows > 1 ? rows : 1);
}

extern "C" int xrh_gemv_rows_split(int64_t rows, int64_t cols, const double* A_dev, int64_t lda, const double* x_dev,
                                   double alpha, double beta, double* y_dev, double* work_dev, int64_t work_len,
                                   void* stream) {
    if (rows < 0 || cols < 0 || lda < cols) return XRH_ERR_ARG;
    if (rows == 0) return XRH_OK;
    if (!A_dev || !x_dev || !y_dev || !work_dev) return XRH_ERR_ARG;
    const int64_t parts = (cols + SPLIT_COLS - 1) / SPLIT_COLS;
    if (parts > 0x7fffffffLL || (rows + 255) / 256 > 0x7fffffffLL) return XRH_ERR_CAPACITY;
    if (work_len < parts * rows) return XRH_ERR_CAPACITY;
    if (parts > 0) {
        gemv_rows_partial_kernel<<<(unsigned)parts, 256, 0, (cudaStream_t)stream>>>(rows, cols, A_dev, lda, x_dev,
                                                                                   work_dev);
        XRH_CHECK_LAUNCH();
    }
    gemv_rows_reduce_kernel<<<(unsigned)((rows + 255) / 256), 256, 0, (cudaStream_t)stream>>>(rows, parts, work_dev,
                                                                                             alpha, beta, y_dev);
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}

extern "C" int xrh_lanczos_normalize_split(int64_t n, const double* w_dev, double* v_dev, double* beta_dev,
                                           double* work_dev, int64_t work_len, void* stream) {
    if (n <= 0 || !w_dev || !v_dev || !beta_dev || !work_dev) return XRH_ERR_ARG;
    const int64_t parts = (n + SPLIT_COLS - 1) / SPLIT_COLS;
    if (parts > 0x7fffffffLL) return XRH_ERR_CAPACITY;
    if (work_len < parts) return XRH_ERR_CAPACITY;
    sumsq_partial_kernel<<<(unsigned)parts, 256, 0, (cudaStream_t)stream>>>(n, w_dev, work_dev);
    XRH_CHECK_LAUNCH();
    scale_by_norm_kernel<<<(unsigned)parts, 256, 0, (cudaStream_t)stream>>>(n, parts, work_dev, w_dev, v_dev, beta_dev);
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}

extern "C" int xrh_lanczos_normalize(int64_t n, const double* w_dev, double* v_dev, double* beta_dev, void* stream) {
    if (n <= 0 || !w_dev || !v_dev || !beta_dev) return XRH_ERR_ARG;
    normalize_kernel<<<1, 1024, 0, (cudaStream_t)stream>>>(n, w_dev, v_dev, beta_dev);
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}

// Scratch (in doubles) of xrh_lanczos_coop for m steps: partial sums of up to LC_MAX_CTAS
// CTAs plus the barrier counter.
extern "C" int64_t xrh_lanczos_coop_work(int m) {
    if (m <= 0) return -1;
    return (int64_t)LC_MAX_CTAS * 2 * (int64_t)(m + 2) + 2;
}

static int lanczos_coop_launch(int64_t n, int m, const double* H_dev, int64_t ld, const double* v0_dev,
                               double* V_dev, double* alpha_dev, double* beta_dev, double* work_dev,
                               int64_t work_len, int32_t* status_dev, long long wait_limit, void* stream) {
    if (n <= 0 || m <= 0 || ld < n || wait_limit < 0) return XRH_ERR_ARG;
    if (!H_dev || !v0_dev || !V_dev || !alpha_dev || !beta_dev || !work_dev || !status_dev) return XRH_ERR_ARG;
    if (work_len < xrh_lanczos_coop_work(m)) return XRH_ERR_CAPACITY;
    int dev = 0, sms = 0, per_sm = 0, smem_optin = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return XRH_ERR_CUDA;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return XRH_ERR_CUDA;
    if (cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
        return XRH_ERR_CUDA;
    int64_t nb = (n + LC_ROWS_PER_CTA - 1) / LC_ROWS_PER_CTA;
    if (nb > sms) nb = sms;
    if (nb > LC_MAX_CTAS) nb = LC_MAX_CTAS;
    const int64_t rows_max = (n + nb - 1) / nb;
    const size_t base = sizeof(double) * ((size_t)(m + 1) * rows_max + rows_max + (size_t)m + 2);
    if (base > (size_t)smem_optin) return XRH_ERR_CAPACITY;
    const int stage_v = base + sizeof(double) * (size_t)n <= (size_t)smem_optin ? 1 : 0;
    const size_t smem = base + (stage_v ? sizeof(double) * (size_t)n : 0);
    // raise the kernel's dynamic shared-memory limit on this device once per larger size (set
    // before any capture by the first, eager call)
    if (dev < 0 || dev >= kLzMaxDevices) return XRH_ERR_CAPACITY;
    {
        std::lock_guard<std::mutex> lock(g_lz_mutex);
        size_t& smem_set = g_lz_state[dev].coop_smem_set;
        if (smem > smem_set) {
            if (cudaFuncSetAttribute(lanczos_coop_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
                cudaSuccess)
                return XRH_ERR_CUDA;
            smem_set = smem;
        }
    }
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, lanczos_coop_kernel, LC_THREADS, smem) != cudaSuccess)
        return XRH_ERR_CUDA;
    if ((int64_t)per_sm * sms < nb) return XRH_ERR_CAPACITY;
    cudaStream_t s = (cudaStream_t)stream;
    double* part = work_dev;
    unsigned int* count = reinterpret_cast<unsigned int*>(work_dev + (int64_t)LC_MAX_CTAS * 2 * (int64_t)(m + 2));
    if (cudaMemsetAsync(count, 0, sizeof(unsigned int), s) != cudaSuccess) return XRH_ERR_CUDA;
    int64_t n_arg = n, ld_arg = ld;
    int m_arg = m, rows_arg = (int)rows_max, stage_arg = stage_v;
    long long limit_arg = wait_limit;
    void* args[] = {&n_arg,         &m_arg,       (void*)&H_dev, &ld_arg,           (void*)&v0_dev,
                    (void*)&V_dev,  (void*)&alpha_dev, (void*)&beta_dev, (void*)&part, (void*)&count,
                    (void*)&status_dev, &rows_arg, &stage_arg,  &limit_arg};
    const cudaError_t e = cudaLaunchCooperativeKernel((const void*)lanczos_coop_kernel, dim3((unsigned)nb),
                                                      dim3(LC_THREADS), args, smem, s);
    if (e != cudaSuccess) {
        xrh_set_last_cuda_error((int)e);
        return XRH_ERR_CUDA;
    }
    return XRH_OK;
}

extern "C" int xrh_lanczos_coop(int64_t n, int m, const double* H_dev, int64_t ld, const double* v0_dev,
                                double* V_dev, double* alpha_dev, double* beta_dev, double* work_dev,
                                int64_t work_len, int32_t* status_dev, void* stream) {
    return lanczos_coop_launch(n, m, H_dev, ld, v0_dev, V_dev, alpha_dev, beta_dev, work_dev, work_len, status_dev,
                               LC_WAIT_LIMIT, stream);
}

extern "C" int xrh_lanczos_coop_bounded(int64_t n, int m, const double* H_dev, int64_t ld, const double* v0_dev,
                                        double* V_dev, double* alpha_dev, double* beta_dev, double* work_dev,
                                        int64_t work_len, int32_t* status_dev, int64_t max_polls, void* stream) {
    return lanczos_coop_launch(n, m, H_dev, ld, v0_dev, V_dev, alpha_dev, beta_dev, work_dev, work_len, status_dev,
                               (long long)max_polls, stream);
}

// Shared memory (bytes) of the cluster loop for a given split; 0 when it does not fit.
static size_t lanczos_cluster_smem(int n, int m, int nb, int h_smem, int smem_optin) {
    const int rows_max = (n + nb - 1) / nb;
    size_t d = (size_t)n + (size_t)(m + 1) * rows_max + 2 * (size_t)rows_max + 3 * (size_t)(m + 2);
    if (h_smem) d += (size_t)rows_max * n;
    const size_t bytes = d * sizeof(double);
    return bytes <= (size_t)smem_optin ? bytes : 0;
}

// Cluster size (16 CTAs when the part schedules such clusters with the needed shared memory,
// else 8), H in shared memory or not, and the shared memory per CTA for an n x n sector and m
// steps on the current device.  Decided once per (device, shape) on the first, eager call and
// cached, so no occupancy query runs inside a stream capture.  Returns false when no cluster
// takes the sector.
static bool lanczos_cluster_choice(int n, int m, int max_ctas, int& nb, int& h_smem, size_t& smem) {
    int dev = 0, smem_optin = 0;
    nb = 0;
    h_smem = 0;
    smem = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kLzMaxDevices) return false;
    std::lock_guard<std::mutex> lock(g_lz_mutex);
    LzDeviceState& st = g_lz_state[dev];
    for (int i = 0; i < st.n_cache; ++i)
        if (st.cache[i].n == n && st.cache[i].m == m && st.cache[i].max_ctas == max_ctas) {
            nb = st.cache[i].nb;
            h_smem = st.cache[i].h_smem;
            smem = st.cache[i].smem;
            return st.cache[i].ok;
        }
    bool ok = false;
    if (cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) == cudaSuccess) {
        if (st.nonportable < 0)
            st.nonportable = cudaFuncSetAttribute(lanczos_cluster_kernel,
                                                  cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess
                                 ? 1
                                 : 0;
        const int nonportable = st.nonportable;
        const int top = (nonportable ? 16 : 8) < max_ctas || max_ctas <= 0 ? (nonportable ? 16 : 8) : max_ctas;
        for (int want = top; !ok && want >= 1; want = want > 8 ? 8 : want / 2) {
            nb = want < n ? want : n;
            h_smem = 1;
            smem = lanczos_cluster_smem(n, m, nb, 1, smem_optin);
            if (!smem) {
                h_smem = 0;
                smem = lanczos_cluster_smem(n, m, nb, 0, smem_optin);
            }
            if (!smem) continue;
            if (smem > st.cluster_smem_set) {
                if (cudaFuncSetAttribute(lanczos_cluster_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem) != cudaSuccess)
                    continue;
                st.cluster_smem_set = smem;
            }
            cudaLaunchConfig_t cfg = {};
            cudaLaunchAttribute attr[1];
            attr[0].id = cudaLaunchAttributeClusterDimension;
            attr[0].val.clusterDim.x = (unsigned)nb;
            attr[0].val.clusterDim.y = 1;
            attr[0].val.clusterDim.z = 1;
            cfg.gridDim = dim3((unsigned)nb);
            cfg.blockDim = dim3(LK_THREADS);
            cfg.dynamicSmemBytes = smem;
            cfg.attrs = attr;
            cfg.numAttrs = 1;
            int clusters = 0;
            ok = cudaOccupancyMaxActiveClusters(&clusters, lanczos_cluster_kernel, &cfg) == cudaSuccess && clusters > 0;
        }
        cudaGetLastError();
    }
    if (st.n_cache < 32) st.cache[st.n_cache++] = LzChoice{n, m, max_ctas, nb, h_smem, smem, ok};
    return ok;
}

extern "C" int xrh_lanczos_cluster_fits(int n, int m, int max_ctas) {
    if (n <= 0 || m <= 0) return 0;
    int nb, h_smem;
    size_t smem;
    return lanczos_cluster_choice(n, m, max_ctas, nb, h_smem, smem) ? 1 : 0;
}

extern "C" int xrh_lanczos_cluster(int n, int m, const double* H_dev, int64_t ld, const double* v0_dev, double* V_dev,
                                   double* alpha_dev, double* beta_dev, int max_ctas, void* stream) {
    if (n <= 0 || m <= 0 || ld < n) return XRH_ERR_ARG;
    if (!H_dev || !v0_dev || !V_dev || !alpha_dev || !beta_dev) return XRH_ERR_ARG;
    int nb = 0, h_smem = 0;
    size_t smem = 0;
    if (!lanczos_cluster_choice(n, m, max_ctas, nb, h_smem, smem)) return XRH_ERR_CAPACITY;
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)nb;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3((unsigned)nb);
    cfg.blockDim = dim3(LK_THREADS);
    cfg.dynamicSmemBytes = smem;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cfg.stream = (cudaStream_t)stream;
    const int rows_max = (n + nb - 1) / nb;
    const cudaError_t e = cudaLaunchKernelEx(&cfg, lanczos_cluster_kernel, n, m, H_dev, ld, v0_dev, V_dev, alpha_dev,
                                             beta_dev, rows_max, h_smem);
    if (e != cudaSuccess) {
        xrh_set_last_cuda_error((int)e);
        return XRH_ERR_CUDA;
    }
    return XRH_OK;
}
