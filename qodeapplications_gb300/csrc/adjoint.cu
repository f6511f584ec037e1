// Adjoint kernels of the density build (energy gradients).
//
// The reference obtains state gradients by rebuilding densities between determinants and
// states and re-running the whole H build (StateSpaceOptimizer/state_gradients.py:164-185),
// and orbital gradients from XR 1- and 2-particle densities (orb_grads.py:867-1000).  Here
// both come from one reverse pass over the same resident coupling lists:
//
//   xrh_density_adjoint:  given G = dE/drho (layout [K, n_b, n_k]),
//       gzb[P, I] += sum_{c: P_c = P} s_c sum_J G[idx_c, I, J] zk[J, Q_c]
//       gzk[Q, J] += sum_{c: Q_c = Q} s_c sum_I G[idx_c, I, J] zb[I, P_c]
//     One CTA per operator index: G[idx] is staged in shared memory once and reused by every
//     coupling of that index; results go out with FP64 atomics (bra and ket may alias).
//   xrh_ccaa_weighted: Gamma[p,q,r,s] += sum_{P,Q} W[P,Q] <P|c+_p c+_q a_s a_r|Q>  for p<q, r<s,
//     with W[P,Q] = sum_I zb[I,P] Y[I,Q] (Y = G zk): the two-particle density of a weighted
//     ensemble, i.e. dE/dV of the monomer term sum V rho^ccaa, without the N^4 density.
#include "xrh_common.cuh"

namespace {

constexpr int kAdjThreads = 256;
constexpr int kAdjChunk = 64;

// One CTA per operator index.  G[idx] (n_b x n_k) is staged in shared memory once; the
// couplings of the index are processed in chunks of kAdjChunk: their z columns are staged,
// then every (coupling, output) pair of the chunk is one work item for the whole CTA
// (n_k ket outputs + n_b bra outputs per coupling), reduced with FP64 atomics.
template <typename T>
__global__ void __launch_bounds__(kAdjThreads) density_adjoint_kernel(
    const int64_t* __restrict__ idx_ptr, const int32_t* __restrict__ P, const int32_t* __restrict__ Q,
    const int8_t* __restrict__ sgn, const double* __restrict__ zbT, int nb, const double* __restrict__ zkT, int nk,
    const double* __restrict__ gT, double* __restrict__ gzbT, double* __restrict__ gzkT) {
    extern __shared__ unsigned char smem_raw[];
    T* g = reinterpret_cast<T*>(smem_raw);                 // [nb][nk]
    T* zb = g + nb * nk;                                    // [chunk][nb] (sign folded in)
    T* zk = zb + kAdjChunk * nb;                            // [chunk][nk]
    __shared__ int sP[kAdjChunk], sQ[kAdjChunk];
    const int64_t idx = blockIdx.x;
    const int64_t c_begin = idx_ptr[idx], c_end = idx_ptr[idx + 1];
    if (c_begin == c_end) return;
    const double* gi = gT + idx * (int64_t)nb * nk;
    for (int t = threadIdx.x; t < nb * nk; t += blockDim.x) g[t] = (T)gi[t];
    const int per = nk + nb;
    for (int64_t c0 = c_begin; c0 < c_end; c0 += kAdjChunk) {
        const int64_t rem = c_end - c0;
        const int nc = rem < kAdjChunk ? (int)rem : kAdjChunk;
        __syncthreads();
        for (int t = threadIdx.x; t < nc; t += blockDim.x) {
            sP[t] = P[c0 + t];
            sQ[t] = Q[c0 + t];
        }
        __syncthreads();
        for (int t = threadIdx.x; t < nc * nb; t += blockDim.x) {
            const int c = t / nb, i = t - c * nb;
            const double s = sgn[c0 + c] < 0 ? -1.0 : 1.0;
            zb[c * nb + i] = (T)(s * zbT[(int64_t)sP[c] * nb + i]);
        }
        for (int t = threadIdx.x; t < nc * nk; t += blockDim.x) {
            const int c = t / nk, j = t - c * nk;
            zk[c * nk + j] = (T)zkT[(int64_t)sQ[c] * nk + j];
        }
        __syncthreads();
        for (int w = threadIdx.x; w < nc * per; w += blockDim.x) {
            const int c = w / per, o = w - c * per;
            T a = 0;
            if (o < nk) {             // ket: gzk[Q, J] += sum_I g[I, J] (s zb[I])
                const int J = o;
                for (int I = 0; I < nb; ++I) a = fma(g[I * nk + J], zb[c * nb + I], a);
                atomicAdd(gzkT + (int64_t)sQ[c] * nk + J, (double)a);
            } else {                  // bra: gzb[P, I] += sum_J g[I, J] zk[J] (times s)
                const int I = o - nk;
                for (int J = 0; J < nk; ++J) a = fma(g[I * nk + J], zk[c * nk + J], a);
                const double s = sgn[c0 + c] < 0 ? -1.0 : 1.0;
                atomicAdd(gzbT + (int64_t)sP[c] * nb + I, s * (double)a);
            }
        }
    }
}

constexpr int kWThreads = 128;

__global__ void __launch_bounds__(kWThreads) ccaa_weighted_kernel(
    int N, const uint64_t* __restrict__ bra, int n_bra, const uint64_t* __restrict__ ket_sorted,
    const int32_t* __restrict__ ket_pos, int n_ket, const double* __restrict__ zbT, const double* __restrict__ YT,
    int n, double* __restrict__ Gamma) {
    __shared__ int s_occ[64];
    __shared__ int s_free[64];
    __shared__ int s_ne, s_nfree;
    __shared__ double s_zb[256];
    const int Pb = blockIdx.x;
    const uint64_t m = bra[Pb];
    if (threadIdx.x == 0) {
        int k = 0;
        for (int o = 0; o < N; ++o)
            if ((m >> o) & 1ull) s_occ[k++] = o;
        s_ne = k;
    }
    for (int t = threadIdx.x; t < n; t += blockDim.x) s_zb[t] = zbT[(int64_t)Pb * n + t];
    __syncthreads();
    const int ne = s_ne;
    for (int a = 0; a < ne; ++a) {
        for (int b = a + 1; b < ne; ++b) {
            const int p = s_occ[a], q = s_occ[b];
            uint64_t m1 = m;
            int s1 = 0;
            xrh_apply(0, p, m1, s1);
            xrh_apply(0, q, m1, s1);
            __syncthreads();
            if (threadIdx.x == 0) {
                int k = 0;
                for (int o = 0; o < N; ++o)
                    if (!((m1 >> o) & 1ull)) s_free[k++] = o;
                s_nfree = k;
            }
            __syncthreads();
            const int nf = s_nfree;
            const int n_rs = nf * (nf - 1) / 2;
            for (int e = threadIdx.x; e < n_rs; e += blockDim.x) {
                int i = 0, rem = e;
                while (rem >= nf - 1 - i) { rem -= nf - 1 - i; ++i; }
                const int j = i + 1 + rem;
                const int r = s_free[i], s = s_free[j];
                uint64_t m2 = m1;
                int s2 = s1;
                xrh_apply(1, s, m2, s2);
                xrh_apply(1, r, m2, s2);
                const int hit = xrh_lookup(ket_sorted, n_ket, m2);
                if (hit < 0) continue;
                const int Qp = __ldg(ket_pos + hit);
                double w = 0.0;
                for (int I = 0; I < n; ++I) w = fma(s_zb[I], YT[(int64_t)Qp * n + I], w);
                if (w == 0.0) continue;
                // <P| c+_p c+_q a_s a_r |Q>  (p<q, r<s) = sign of <Q| c+_r c+_s a_q a_p |P>
                atomicAdd(Gamma + (((int64_t)p * N + q) * N + r) * N + s, s2 ? -w : w);
            }
        }
    }
}

}  // namespace

extern "C" int xrh_density_adjoint(int precision, int64_t K, const int64_t* idx_ptr_dev, const int32_t* P_dev,
                                   const int32_t* Q_dev, const int8_t* sign_dev, const double* zbT_dev, int n_b,
                                   const double* zkT_dev, int n_k, const double* gT_dev, double* gzbT_dev,
                                   double* gzkT_dev, void* stream) {
    if (K <= 0 || n_b <= 0 || n_k <= 0 || !idx_ptr_dev || !zbT_dev || !zkT_dev || !gT_dev || !gzbT_dev || !gzkT_dev)
        return XRH_ERR_ARG;
    if (K > 0x7fffffffLL) return XRH_ERR_CAPACITY;
    const size_t esz = (precision == XRH_FP32) ? sizeof(float) : sizeof(double);
    const size_t smem = esz * ((size_t)n_b * n_k + (size_t)kAdjChunk * (n_b + n_k));
    if (smem > 200 * 1024) return XRH_ERR_CAPACITY;
    if (precision == XRH_FP64) {
        cudaFuncSetAttribute(density_adjoint_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        density_adjoint_kernel<double><<<(unsigned)K, kAdjThreads, smem, (cudaStream_t)stream>>>(
            idx_ptr_dev, P_dev, Q_dev, sign_dev, zbT_dev, n_b, zkT_dev, n_k, gT_dev, gzbT_dev, gzkT_dev);
    } else if (precision == XRH_FP32) {
        cudaFuncSetAttribute(density_adjoint_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        density_adjoint_kernel<float><<<(unsigned)K, kAdjThreads, smem, (cudaStream_t)stream>>>(
            idx_ptr_dev, P_dev, Q_dev, sign_dev, zbT_dev, n_b, zkT_dev, n_k, gT_dev, gzbT_dev, gzkT_dev);
    } else {
        return XRH_ERR_UNSUPPORTED;
    }
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}

extern "C" int xrh_ccaa_weighted(int n_orbs, const uint64_t* bra_masks_dev, int n_bra_conf,
                                 const uint64_t* ket_sorted_masks_dev, const int32_t* ket_sorted_pos_dev,
                                 int n_ket_conf, const double* zbT_dev, const double* YT_dev, int n,
                                 double* Gamma_dev, void* stream) {
    const int N = 2 * n_orbs;
    if (n_orbs < 1 || N > 64 || n < 1 || n > 256 || n_bra_conf < 0 || n_ket_conf < 0) return XRH_ERR_ARG;
    if (n_bra_conf == 0) return XRH_OK;
    if (!bra_masks_dev || !zbT_dev || !YT_dev || !Gamma_dev) return XRH_ERR_ARG;
    ccaa_weighted_kernel<<<n_bra_conf, kWThreads, 0, (cudaStream_t)stream>>>(
        N, bra_masks_dev, n_bra_conf, ket_sorted_masks_dev, ket_sorted_pos_dev, n_ket_conf, zbT_dev, YT_dev, n,
        Gamma_dev);
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}
