// Transition densities and the fused monomer two-electron term.
//
//   xrh_density_accumulate: rho[idx, I, J] = sum_c s_c zb[I,P_c] zk[J,Q_c]  (z_contract,
//       general-XRCC/density_tensors.c:142-154), gathered per operator index from the
//       resident coupling lists: one CTA per idx, the coupling columns of zb and zk staged
//       in shared memory, every (I,J) output owned by one thread (no atomics, deterministic).
//   xrh_sigma2e: sigma[P, J] = sum_Q <P|V|Q> zk[J,Q] (direct-CI sigma vector of the
//       fragment's two-electron operator), which together with one GEMM replaces building
//       the N^4 ccaa density and contracting it with V (general-XRCC/
//       build_density_tensors.py:122-133, H_contractions.c:61-78).
#include "xrh_common.cuh"

namespace {

constexpr int kAccThreads = 256;
constexpr int kAccPerThread = 16;                 // outputs per thread per pass
constexpr int kAccPass = kAccThreads * kAccPerThread;

template <typename T>
__global__ void __launch_bounds__(kAccThreads) density_acc_kernel(
    const int64_t* __restrict__ idx_ptr, const int32_t* __restrict__ P, const int32_t* __restrict__ Q,
    const int8_t* __restrict__ sgn, const double* __restrict__ zbT, int nb, const double* __restrict__ zkT,
    int nk, double* __restrict__ rhoT, int chunk) {
    extern __shared__ unsigned char smem_raw[];
    T* sb = reinterpret_cast<T*>(smem_raw);           // [chunk][nb]
    T* sk = sb + (size_t)chunk * nb;                  // [chunk][nk]
    const int64_t idx = blockIdx.x;
    const int64_t c_begin = idx_ptr[idx], c_end = idx_ptr[idx + 1];
    const int n_out = nb * nk;
    double* out = rhoT + idx * (int64_t)n_out;
    for (int pass0 = 0; pass0 < n_out; pass0 += kAccPass) {
        double acc[kAccPerThread];
#pragma unroll
        for (int r = 0; r < kAccPerThread; ++r) acc[r] = 0.0;
        for (int64_t c0 = c_begin; c0 < c_end; c0 += chunk) {
            const int64_t rem_c = c_end - c0;
            const int nc = rem_c < chunk ? (int)rem_c : chunk;
            __syncthreads();
            for (int t = threadIdx.x; t < nc * nb; t += blockDim.x) {
                const int c = t / nb, i = t - c * nb;
                const double s = sgn[c0 + c] < 0 ? -1.0 : 1.0;
                sb[c * nb + i] = (T)(s * zbT[(int64_t)P[c0 + c] * nb + i]);
            }
            for (int t = threadIdx.x; t < nc * nk; t += blockDim.x) {
                const int c = t / nk, j = t - c * nk;
                sk[c * nk + j] = (T)zkT[(int64_t)Q[c0 + c] * nk + j];
            }
            __syncthreads();
#pragma unroll
            for (int r = 0; r < kAccPerThread; ++r) {
                const int o = pass0 + threadIdx.x + r * kAccThreads;
                if (o < n_out) {
                    const int i = o / nk, j = o - i * nk;
                    T a = 0;
                    for (int c = 0; c < nc; ++c) a = fma(sb[c * nb + i], sk[c * nk + j], a);
                    acc[r] += (double)a;     // FP32 variant: FP32 partial sums per chunk, FP64 total
                }
            }
        }
#pragma unroll
        for (int r = 0; r < kAccPerThread; ++r) {
            const int o = pass0 + threadIdx.x + r * kAccThreads;
            if (o < n_out) out[o] = acc[r];
        }
    }
}

__global__ void transpose_kernel(const double* __restrict__ in, int64_t rows, int64_t cols, double* __restrict__ out) {
    __shared__ double tile[32][33];
    const int64_t c0 = (int64_t)blockIdx.x * 32, r0 = (int64_t)blockIdx.y * 32;
    for (int dy = threadIdx.y; dy < 32; dy += blockDim.y) {
        const int64_t r = r0 + dy, c = c0 + threadIdx.x;
        if (r < rows && c < cols) tile[dy][threadIdx.x] = in[r * cols + c];
    }
    __syncthreads();
    for (int dy = threadIdx.y; dy < 32; dy += blockDim.y) {
        const int64_t c = c0 + dy, r = r0 + threadIdx.x;
        if (r < rows && c < cols) out[c * rows + r] = tile[threadIdx.x][dy];
    }
}

// ---- sigma vector of the two-electron operator ------------------------------------------
constexpr int kSigThreads = 128;
constexpr int kSigMaxNk = 256;

template <typename T>
__global__ void __launch_bounds__(kSigThreads) sigma2e_kernel(
    int N, const double* __restrict__ V, const uint64_t* __restrict__ bra, int n_bra,
    const uint64_t* __restrict__ ket_sorted, const int32_t* __restrict__ ket_pos, int n_ket,
    const double* __restrict__ zkT, int nk, double* __restrict__ sigmaT) {
    // smem: entry list (Q position, coefficient) for one (p,q) pair: at most C(N,2) entries
    extern __shared__ unsigned char smem_raw[];
    int* eq = reinterpret_cast<int*>(smem_raw);
    double* ev = reinterpret_cast<double*>(smem_raw + sizeof(int) * 2048);
    __shared__ int s_count;
    __shared__ int s_occ[64];
    __shared__ int s_free[64];
    __shared__ int s_nfree;
    __shared__ int s_ne;
    const int Pb = blockIdx.x;
    const uint64_t m = bra[Pb];
    if (threadIdx.x == 0) {
        int n = 0;
        for (int o = 0; o < N; ++o)
            if ((m >> o) & 1ull) s_occ[n++] = o;
        s_ne = n;
    }
    __syncthreads();
    const int ne = s_ne;
    constexpr int JR = kSigMaxNk / kSigThreads;
    double acc[JR];
#pragma unroll
    for (int r = 0; r < JR; ++r) acc[r] = 0.0;
    for (int a = 0; a < ne; ++a) {
        for (int b = a + 1; b < ne; ++b) {
            const int p = s_occ[a], q = s_occ[b];
            // <P| c+_p c+_q a_s a_r |Q> = <Q| c+_r c+_s a_q a_p |P>: act on P with a_p, a_q, c+_s, c+_r
            uint64_t m1 = m;
            int s1 = 0;
            xrh_apply(0, p, m1, s1);
            xrh_apply(0, q, m1, s1);
            __syncthreads();
            if (threadIdx.x == 0) {
                int n = 0;
                for (int o = 0; o < N; ++o)
                    if (!((m1 >> o) & 1ull)) s_free[n++] = o;
                s_nfree = n;
                s_count = 0;
            }
            __syncthreads();
            const int nf = s_nfree;
            const int n_rs = nf * (nf - 1) / 2;
            const double* Vpq = V + ((int64_t)p * N + q) * N * N;
            for (int e = threadIdx.x; e < n_rs; e += blockDim.x) {
                // unrank e -> (i < j) over the free list
                int i = 0, rem = e;
                while (rem >= nf - 1 - i) { rem -= nf - 1 - i; ++i; }
                const int j = i + 1 + rem;
                const int r = s_free[i], s = s_free[j];
                const double v = __ldg(Vpq + (int64_t)r * N + s);
                if (v == 0.0) continue;
                uint64_t m2 = m1;
                int s2 = s1;
                xrh_apply(1, s, m2, s2);
                xrh_apply(1, r, m2, s2);
                const int hit = xrh_lookup(ket_sorted, n_ket, m2);
                if (hit < 0) continue;
                const int slot = atomicAdd(&s_count, 1);
                eq[slot] = __ldg(ket_pos + hit);
                ev[slot] = (s2 ? -4.0 : 4.0) * v;
            }
            __syncthreads();
            const int ne2 = s_count;
#pragma unroll
            for (int rr = 0; rr < JR; ++rr) {
                const int J = threadIdx.x + rr * kSigThreads;
                if (J < nk) {
                    T part = 0;
                    for (int t = 0; t < ne2; ++t) part = fma((T)ev[t], (T)zkT[(int64_t)eq[t] * nk + J], part);
                    acc[rr] += (double)part;
                }
            }
        }
    }
#pragma unroll
    for (int rr = 0; rr < JR; ++rr) {
        const int J = threadIdx.x + rr * kSigThreads;
        if (J < nk) sigmaT[(int64_t)J * n_bra + Pb] = acc[rr];
    }
}

}  // namespace

extern "C" int xrh_density_accumulate(int precision, int64_t K, const int64_t* idx_ptr_dev, const int32_t* P_dev,
                                      const int32_t* Q_dev, const int8_t* sign_dev, const double* zbT_dev, int n_b,
                                      const double* zkT_dev, int n_k, double* rhoT_dev, void* stream) {
    if (K <= 0 || n_b <= 0 || n_k <= 0 || !idx_ptr_dev || !rhoT_dev || !zbT_dev || !zkT_dev) return XRH_ERR_ARG;
    if (K > 0x7fffffffLL) return XRH_ERR_CAPACITY;
    const size_t esz = (precision == XRH_FP32) ? sizeof(float) : sizeof(double);
    int chunk = (int)((40 * 1024) / (esz * (size_t)(n_b + n_k)));
    if (chunk < 1) return XRH_ERR_CAPACITY;
    if (chunk > 64) chunk = 64;
    const size_t smem = esz * (size_t)chunk * (n_b + n_k);
    if (precision == XRH_FP64) {
        density_acc_kernel<double><<<(unsigned)K, kAccThreads, smem, (cudaStream_t)stream>>>(
            idx_ptr_dev, P_dev, Q_dev, sign_dev, zbT_dev, n_b, zkT_dev, n_k, rhoT_dev, chunk);
    } else if (precision == XRH_FP32) {
        density_acc_kernel<float><<<(unsigned)K, kAccThreads, smem, (cudaStream_t)stream>>>(
            idx_ptr_dev, P_dev, Q_dev, sign_dev, zbT_dev, n_b, zkT_dev, n_k, rhoT_dev, chunk);
    } else {
        return XRH_ERR_UNSUPPORTED;
    }
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}

extern "C" int xrh_transpose(const double* in_dev, int64_t rows, int64_t cols, double* out_dev, void* stream) {
    if (rows < 0 || cols < 0 || (!in_dev && rows * cols) || (!out_dev && rows * cols)) return XRH_ERR_ARG;
    if (rows == 0 || cols == 0) return XRH_OK;
    if ((cols + 31) / 32 > 0x7fffffffLL || (rows + 31) / 32 > 65535) return XRH_ERR_CAPACITY;
    dim3 grid((unsigned)((cols + 31) / 32), (unsigned)((rows + 31) / 32));
    transpose_kernel<<<grid, dim3(32, 8), 0, (cudaStream_t)stream>>>(in_dev, rows, cols, out_dev);
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}

extern "C" int xrh_sigma2e(int precision, int n_orbs, const double* V_dev, const uint64_t* bra_masks_dev,
                           int n_bra_conf, const uint64_t* ket_sorted_masks_dev, const int32_t* ket_sorted_pos_dev,
                           int n_ket_conf, const double* zkT_dev, int n_k, double* sigmaT_dev, void* stream) {
    const int N = 2 * n_orbs;
    if (n_orbs < 1 || N > 64 || n_k < 1 || n_k > kSigMaxNk || n_bra_conf < 0 || n_ket_conf < 0) return XRH_ERR_ARG;
    if (n_bra_conf == 0) return XRH_OK;
    if (!V_dev || !bra_masks_dev || !zkT_dev || !sigmaT_dev) return XRH_ERR_ARG;
    // entry list capacity: C(64,2) = 2016 <= 2048
    const size_t smem = 2048 * (sizeof(int) + sizeof(double));
    if (precision == XRH_FP64) {
        cudaFuncSetAttribute(sigma2e_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        sigma2e_kernel<double><<<n_bra_conf, kSigThreads, smem, (cudaStream_t)stream>>>(
            N, V_dev, bra_masks_dev, n_bra_conf, ket_sorted_masks_dev, ket_sorted_pos_dev, n_ket_conf, zkT_dev, n_k,
            sigmaT_dev);
    } else if (precision == XRH_FP32) {
        cudaFuncSetAttribute(sigma2e_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        sigma2e_kernel<float><<<n_bra_conf, kSigThreads, smem, (cudaStream_t)stream>>>(
            N, V_dev, bra_masks_dev, n_bra_conf, ket_sorted_masks_dev, ket_sorted_pos_dev, n_ket_conf, zkT_dev, n_k,
            sigmaT_dev);
    } else {
        return XRH_ERR_UNSUPPORTED;
    }
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}

// ---- allocation-free density build ------------------------------------------------------
// For callers that cannot allocate device memory: the scratch that xrh_density_accumulate's
// callers provide (the [K, n_b, n_k] buffer before the transpose) is a fixed-size array in
// the module's own global memory.  Every GPU that loads libxrh.so holds it until exit.
namespace {
constexpr int64_t kNoAllocScratchDoubles = 1LL << 20;          // 8 MiB of FP64
__device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchDoubles];
double* g_noalloc_scratch_addr[256] = {};                      // device address per device ordinal
}  // namespace

extern "C" int xrh_density_build_noalloc(int precision, int64_t K, const int64_t* idx_ptr_dev, const int32_t* P_dev,
                                         const int32_t* Q_dev, const int8_t* sign_dev, const double* zbT_dev, int n_b,
                                         const double* zkT_dev, int n_k, double* rho_dev, void* stream) {
    if (K <= 0 || n_b <= 0 || n_k <= 0 || !idx_ptr_dev || !zbT_dev || !zkT_dev || !rho_dev) return XRH_ERR_ARG;
    if (precision != XRH_FP64 && precision != XRH_FP32) return XRH_ERR_UNSUPPORTED;
    if (K * (int64_t)n_b * (int64_t)n_k > kNoAllocScratchDoubles) return XRH_ERR_CAPACITY;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        xrh_set_last_cuda_error((int)e);
        return XRH_ERR_CUDA;
    }
    if (dev < 0 || dev >= 256) return XRH_ERR_CAPACITY;
    double* scratch = g_noalloc_scratch_addr[dev];
    if (!scratch) {
        // once per device, with that device current: the host-side name of the array is not a
        // device address, so ask the runtime for this device's address of it
        e = cudaGetSymbolAddress(reinterpret_cast<void**>(&scratch), g_noalloc_scratch);
        if (e != cudaSuccess || !scratch) {
            xrh_set_last_cuda_error((int)e);
            return XRH_ERR_CUDA;
        }
        g_noalloc_scratch_addr[dev] = scratch;
    }
    // the accumulate kernel overwrites every scratch element it uses: nothing to clear
    int st = xrh_density_accumulate(precision, K, idx_ptr_dev, P_dev, Q_dev, sign_dev, zbT_dev, n_b, zkT_dev, n_k,
                                    scratch, stream);
    if (st != XRH_OK) return st;
    return xrh_transpose(scratch, K, (int64_t)n_b * n_k, rho_dev, stream);
}
