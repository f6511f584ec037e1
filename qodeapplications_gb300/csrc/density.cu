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

#include <atomic>

namespace {

constexpr int kAccThreads = 256;
constexpr int kAccChunk = 64;

template <typename T> struct Vec4;
template <> struct Vec4<float> { using type = float4; };
template <> struct Vec4<double> { using type = double4; };

// One CTA per operator index.  Each thread owns a 4 x 4 block of (I, J) outputs; the
// couplings of the index are staged 64 at a time in shared memory (bra columns with the
// sign folded in, ket columns), rows padded to a multiple of 4 so that one coupling costs
// two 4-wide shared loads per 16 FMAs.  Partial sums of a chunk are in T, the running sum in
// FP64 (the FP32 variant therefore rounds only within a chunk).
template <typename T>
__global__ void __launch_bounds__(kAccThreads) density_acc_kernel(
    const int64_t* __restrict__ idx_ptr, const int32_t* __restrict__ P, const int32_t* __restrict__ Q,
    const int8_t* __restrict__ sgn, const double* __restrict__ zbT, int nb, const double* __restrict__ zkT,
    int nk, double* __restrict__ rhoT) {
    using V4 = typename Vec4<T>::type;
    extern __shared__ __align__(32) unsigned char smem_raw[];
    const int nbp = (nb + 3) & ~3, nkp = (nk + 3) & ~3;
    T* sb = reinterpret_cast<T*>(smem_raw);            // [chunk][nbp]
    T* sk = sb + (size_t)kAccChunk * nbp;              // [chunk][nkp]
    const int64_t idx = blockIdx.x;
    const int64_t c_begin = idx_ptr[idx], c_end = idx_ptr[idx + 1];
    double* out = rhoT + idx * (int64_t)nb * nk;
    const int tiles_j = nkp / 4, n_tiles = (nbp / 4) * tiles_j;
    for (int t0 = 0; t0 < n_tiles; t0 += kAccThreads) {
        const int t = t0 + threadIdx.x;
        const bool active = t < n_tiles;
        const int i0 = active ? (t / tiles_j) * 4 : 0, j0 = active ? (t % tiles_j) * 4 : 0;
        double acc[4][4];
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int b = 0; b < 4; ++b) acc[a][b] = 0.0;
        for (int64_t c0 = c_begin; c0 < c_end; c0 += kAccChunk) {
            const int64_t rem = c_end - c0;
            const int nc = rem < kAccChunk ? (int)rem : kAccChunk;
            __syncthreads();
            for (int x = threadIdx.x; x < nc * nbp; x += blockDim.x) {
                const int c = x / nbp, i = x - c * nbp;
                const double s = sgn[c0 + c] < 0 ? -1.0 : 1.0;
                sb[x] = i < nb ? (T)(s * zbT[(int64_t)P[c0 + c] * nb + i]) : (T)0;
            }
            for (int x = threadIdx.x; x < nc * nkp; x += blockDim.x) {
                const int c = x / nkp, j = x - c * nkp;
                sk[x] = j < nk ? (T)zkT[(int64_t)Q[c0 + c] * nk + j] : (T)0;
            }
            __syncthreads();
            if (active) {
                T part[4][4];
#pragma unroll
                for (int a = 0; a < 4; ++a)
#pragma unroll
                    for (int b = 0; b < 4; ++b) part[a][b] = 0;
                for (int c = 0; c < nc; ++c) {
                    const V4 va = *reinterpret_cast<const V4*>(sb + c * nbp + i0);
                    const V4 vb = *reinterpret_cast<const V4*>(sk + c * nkp + j0);
                    const T av[4] = {va.x, va.y, va.z, va.w};
                    const T bv[4] = {vb.x, vb.y, vb.z, vb.w};
#pragma unroll
                    for (int a = 0; a < 4; ++a)
#pragma unroll
                        for (int b = 0; b < 4; ++b) part[a][b] = fma(av[a], bv[b], part[a][b]);
                }
#pragma unroll
                for (int a = 0; a < 4; ++a)
#pragma unroll
                    for (int b = 0; b < 4; ++b) acc[a][b] += (double)part[a][b];
            }
        }
        if (active) {
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int b = 0; b < 4; ++b)
                    if (i0 + a < nb && j0 + b < nk) out[(int64_t)(i0 + a) * nk + j0 + b] = acc[a][b];
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

// Many transposes in one launch: 32 x 32 tiles, CTA -> task by binary search on tile_begin.
__global__ void transpose_grouped_kernel(const xrh_transpose_task* __restrict__ tasks, int n_tasks) {
    __shared__ double tile[32][33];
    const int64_t bt = blockIdx.x;
    int lo = 0, hi = n_tasks - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (tasks[mid].tile_begin <= bt) lo = mid; else hi = mid - 1;
    }
    const xrh_transpose_task& T = tasks[lo];
    const int64_t local = bt - T.tile_begin;
    const int64_t tiles_c = (T.cols + 31) / 32;
    const int64_t c0 = (local % tiles_c) * 32, r0 = (local / tiles_c) * 32;
    for (int dy = threadIdx.y; dy < 32; dy += blockDim.y) {
        const int64_t r = r0 + dy, c = c0 + threadIdx.x;
        if (r < T.rows && c < T.cols) tile[dy][threadIdx.x] = T.in[r * T.cols + c];
    }
    __syncthreads();
    for (int dy = threadIdx.y; dy < 32; dy += blockDim.y) {
        const int64_t c = c0 + dy, r = r0 + threadIdx.x;
        if (r < T.rows && c < T.cols) T.out[c * T.rows + r] = tile[threadIdx.x][dy];
    }
}

// ---- sigma vector of the two-electron operator ------------------------------------------
constexpr int kSigThreads = 128;
constexpr int kSigMaxNk = 256;

template <typename T>
__global__ void __launch_bounds__(kSigThreads) sigma2e_kernel(
    int N, const double* __restrict__ V, const uint64_t* __restrict__ bra, int n_bra,
    const uint64_t* __restrict__ ket_sorted, const int32_t* __restrict__ ket_pos, int n_ket,
    const int32_t* __restrict__ rank_table, int64_t table_size, const int64_t* __restrict__ binom,
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
                int qpos;
                if (rank_table) {
                    qpos = xrh_rank_lookup(rank_table, table_size, binom, m2);
                } else {
                    const int hit = xrh_lookup(ket_sorted, n_ket, m2);
                    qpos = hit < 0 ? -1 : __ldg(ket_pos + hit);
                }
                if (qpos < 0) continue;
                const int slot = atomicAdd(&s_count, 1);
                eq[slot] = qpos;
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
    const size_t smem = esz * (size_t)kAccChunk * (size_t)(((n_b + 3) & ~3) + ((n_k + 3) & ~3));
    if (smem > 200 * 1024) return XRH_ERR_CAPACITY;
    if (precision == XRH_FP64) {
        if (smem > 48 * 1024)
            cudaFuncSetAttribute(density_acc_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        density_acc_kernel<double><<<(unsigned)K, kAccThreads, smem, (cudaStream_t)stream>>>(
            idx_ptr_dev, P_dev, Q_dev, sign_dev, zbT_dev, n_b, zkT_dev, n_k, rhoT_dev);
    } else if (precision == XRH_FP32) {
        if (smem > 48 * 1024)
            cudaFuncSetAttribute(density_acc_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        density_acc_kernel<float><<<(unsigned)K, kAccThreads, smem, (cudaStream_t)stream>>>(
            idx_ptr_dev, P_dev, Q_dev, sign_dev, zbT_dev, n_b, zkT_dev, n_k, rhoT_dev);
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
                           int n_ket_conf, const int32_t* rank_table_dev, int64_t table_size,
                           const int64_t* binom_dev, const double* zkT_dev, int n_k, double* sigmaT_dev,
                           void* stream) {
    const int N = 2 * n_orbs;
    if (n_orbs < 1 || N > 64 || n_k < 1 || n_k > kSigMaxNk || n_bra_conf < 0 || n_ket_conf < 0) return XRH_ERR_ARG;
    if (n_bra_conf == 0) return XRH_OK;
    if (!V_dev || !bra_masks_dev || !zkT_dev || !sigmaT_dev) return XRH_ERR_ARG;
    if (rank_table_dev && !binom_dev) return XRH_ERR_ARG;
    // entry list capacity: C(64,2) = 2016 <= 2048
    const size_t smem = 2048 * (sizeof(int) + sizeof(double));
    if (precision == XRH_FP64) {
        cudaFuncSetAttribute(sigma2e_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        sigma2e_kernel<double><<<n_bra_conf, kSigThreads, smem, (cudaStream_t)stream>>>(
            N, V_dev, bra_masks_dev, n_bra_conf, ket_sorted_masks_dev, ket_sorted_pos_dev, n_ket_conf, rank_table_dev,
            table_size, binom_dev, zkT_dev, n_k, sigmaT_dev);
    } else if (precision == XRH_FP32) {
        cudaFuncSetAttribute(sigma2e_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        sigma2e_kernel<float><<<n_bra_conf, kSigThreads, smem, (cudaStream_t)stream>>>(
            N, V_dev, bra_masks_dev, n_bra_conf, ket_sorted_masks_dev, ket_sorted_pos_dev, n_ket_conf, rank_table_dev,
            table_size, binom_dev, zkT_dev, n_k, sigmaT_dev);
    } else {
        return XRH_ERR_UNSUPPORTED;
    }
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}

// ---- mirrored blocks -----------------------------------------------------------------------
// <P| c+_p c+_q a_r |Q> = <Q| c+_r a_q a_p |P> for real states, so rho^cca(b, k)[I, J, p, q, r]
// = rho^caa(k, b)[J, I, r, q, p]; likewise cc / aa and c / a: the creation-side blocks are the
// annihilation-side ones with bra and ket swapped and the operator indices reversed.
//   dst[a][b][f] = (accumulate ? dst : 0) + src[b][a][reverse(f)],  f over N^L
// One CTA per (a, b[, q]) plane: reversing (p, q, r) -> (r, q, p) transposes the (p, r) plane at
// fixed q, reversing (p, q) -> (q, p) transposes the plane; both go through shared memory so
// that loads and stores stay coalesced (N <= 64).
// Many mirrors in one launch: CTA -> task by binary search on cta_begin; the tasks' dst
// blocks are distinct (the host checks), so accumulating tasks do not race.  For L = 3 a CTA
// takes mirror_planes(N) consecutive q planes of one (a, b) (about 4096 elements), so that each
// thread keeps several loads in flight; L = 1, 2: one CTA per (a, b).
__host__ __device__ __forceinline__ int mirror_planes(int N) {
    const int q = 4096 / (N * N);
    return q < 1 ? 1 : (q > N ? N : q);
}
__host__ __device__ __forceinline__ int64_t mirror_ctas_per_pair(int N, int L) {
    return L == 3 ? (N + mirror_planes(N) - 1) / mirror_planes(N) : 1;
}
constexpr int kMirrorTile = 4352;      // max over N <= 64 of planes * N * (N + 1) doubles

__device__ __forceinline__ void mirror_plane(int na, int nb, int N, int L, const double* __restrict__ src,
                                             double* __restrict__ dst, int accumulate, int64_t blk,
                                             double* __restrict__ tile) {
    int64_t F = 1;
    for (int l = 0; l < L; ++l) F *= N;
    const int64_t per = mirror_ctas_per_pair(N, L);
    const int64_t ab = blk / per;
    const int qb = (int)(blk - ab * per);
    const int a = (int)(ab / nb), b = (int)(ab - (int64_t)(ab / nb) * nb);
    const double* sp = src + ((int64_t)b * na + a) * F;
    double* dp = dst + ((int64_t)a * nb + b) * F;
    if (L == 1) {
        for (int p = threadIdx.x; p < N; p += blockDim.x) dp[p] = (accumulate ? dp[p] : 0.0) + sp[p];
        return;
    }
    const int NN = N * N, W = N + 1;
    const int QB = (L == 3) ? mirror_planes(N) : 1;
    const int q0 = qb * QB;
    const int nq = (L == 3) ? (N - q0 < QB ? N - q0 : QB) : 1;
    // load: consecutive threads along r (contiguous in src), store: along p (contiguous in dst)
    for (int e = threadIdx.x; e < nq * NN; e += blockDim.x) {
        const int qq = e / NN, rem = e - qq * NN, p = rem / N, r = rem - p * N;
        tile[(qq * N + p) * W + r] = sp[L == 2 ? rem : ((int64_t)p * N + q0 + qq) * N + r];
    }
    __syncthreads();
    for (int e = threadIdx.x; e < nq * NN; e += blockDim.x) {
        const int qq = e / NN, rem = e - qq * NN, r = rem / N, p = rem - r * N;
        const int64_t pos = L == 2 ? rem : ((int64_t)r * N + q0 + qq) * N + p;
        const double v = tile[(qq * N + p) * W + r];
        dp[pos] = accumulate ? dp[pos] + v : v;
    }
}

__global__ void __launch_bounds__(256) mirror_grouped_kernel(const xrh_mirror_task* __restrict__ tasks, int n_tasks) {
    __shared__ double tile[kMirrorTile];
    const int64_t cta = blockIdx.x;
    int lo = 0, hi = n_tasks - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (tasks[mid].cta_begin <= cta) lo = mid; else hi = mid - 1;
    }
    const xrh_mirror_task& T = tasks[lo];
    if (T.N <= 0 || T.N > 64 || T.L < 1 || T.L > 3) return;   // checked by the host
    mirror_plane(T.na, T.nb, T.N, T.L, T.src, T.dst, T.accumulate, cta - T.cta_begin, tile);
}

__global__ void __launch_bounds__(256) mirror_kernel(int na, int nb, int N, int L, const double* __restrict__ src,
                                                     double* __restrict__ dst, int accumulate) {
    __shared__ double tile[kMirrorTile];
    mirror_plane(na, nb, N, L, src, dst, accumulate, blockIdx.x, tile);
}

// ---- antisymmetric operator pairs -------------------------------------------------------
// Two adjacent operators of one kind anticommute (a_q a_r = -a_r a_q, c+_p c+_q = -c+_q c+_p), so
// rho[.. o_u, o_u+1 ..] = -rho[.. o_u+1, o_u ..]: the density and adjoint kernels may run over the
// canonical index tuples (o_u < o_u+1) only, and one pass over the rows of the [K][R] layout
// (idx row-major over the L operator indices, R = n_b n_k) completes the rest:
//   mode 0 (fill): row[idx] = -row[swap(idx)] for o_u > o_u+1 (rows with o_u = o_u+1 stay as the
//                  kernels wrote them: zero, they have no couplings);
//   mode 1 (fold): row[idx] -= row[swap(idx)] for o_u < o_u+1 (dE/drho of a canonical tuple from
//                  the full gradient).
// A creation-annihilation pair between the same states (rho^ca of a diagonal charge block, real
// states) is Hermitian instead: rho[i, j, p, q] = rho[j, i, q, p], the row of (q, p) the row of
// (p, q) transposed as an n x n matrix (n = nrow):
//   mode 2 (fill):  row[idx][i n + j] = row[swap(idx)][j n + i] for o_u > o_u+1;
//   mode 3 (fold):  row[idx][i n + j] += row[swap(idx)][j n + i] for o_u < o_u+1.
// One CTA per operator index of a task (non-target indices return at once).
__global__ void __launch_bounds__(256) antisym_rows_kernel(const xrh_antisym_task* __restrict__ tasks, int n_tasks) {
    const int64_t cta = blockIdx.x;
    int lo = 0, hi = n_tasks - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (tasks[mid].cta_begin <= cta) lo = mid; else hi = mid - 1;
    }
    const xrh_antisym_task& T = tasks[lo];
    const int64_t idx = cta - T.cta_begin;
    int64_t w_lo = 1;                                   // N^(L-2-u): weight of digit u+1
    for (int t = T.u + 2; t < T.L; ++t) w_lo *= T.N;
    const int64_t w_hi = w_lo * T.N;                    // weight of digit u
    const int a = (int)((idx / w_hi) % T.N), b = (int)((idx / w_lo) % T.N);
    const bool target = (T.mode == 0 || T.mode == 2) ? a > b : a < b;
    if (!target) return;
    const int64_t partner = idx + (int64_t)(b - a) * w_hi + (int64_t)(a - b) * w_lo;
    double* dst = T.rows + idx * T.R;
    const double* src = T.rows + partner * T.R;
    if (T.mode == 0) {
        for (int64_t e = threadIdx.x; e < T.R; e += blockDim.x) dst[e] = -src[e];
    } else if (T.mode == 1) {
        for (int64_t e = threadIdx.x; e < T.R; e += blockDim.x) dst[e] -= src[e];
    } else {
        const int n = T.nrow;
        for (int64_t e = threadIdx.x; e < T.R; e += blockDim.x) {
            const int i = (int)(e / n), j = (int)(e - (int64_t)i * n);
            const double v = src[(int64_t)j * n + i];
            dst[e] = T.mode == 2 ? v : dst[e] + v;
        }
    }
}

extern "C" int xrh_antisym_rows(const xrh_antisym_task* tasks_dev, int n_tasks, int64_t total_ctas, void* stream) {
    if (n_tasks < 0 || total_ctas < 0) return XRH_ERR_ARG;
    if (n_tasks == 0 || total_ctas == 0) return XRH_OK;
    if (!tasks_dev) return XRH_ERR_ARG;
    if (total_ctas > 0x7fffffffLL) return XRH_ERR_CAPACITY;
    antisym_rows_kernel<<<(unsigned)total_ctas, 256, 0, (cudaStream_t)stream>>>(tasks_dev, n_tasks);
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}

extern "C" int64_t xrh_mirror_ctas(int N, int L) {
    if (N <= 0 || N > 64 || L < 1 || L > 3) return 0;
    return mirror_ctas_per_pair(N, L);
}

extern "C" int xrh_mirror_density(int na, int nb, int N, int L, const double* src_dev, double* dst_dev, int accumulate,
                                  void* stream) {
    if (na <= 0 || nb <= 0 || N <= 0 || L < 1 || L > 3 || !src_dev || !dst_dev || src_dev == dst_dev)
        return XRH_ERR_ARG;
    if (N > 64) return XRH_ERR_CAPACITY;
    const int64_t blocks = (int64_t)na * nb * mirror_ctas_per_pair(N, L);
    if (blocks > 0x7fffffffLL) return XRH_ERR_CAPACITY;
    mirror_kernel<<<(unsigned)blocks, L == 1 ? 64 : 256, 0, (cudaStream_t)stream>>>(na, nb, N, L, src_dev, dst_dev,
                                                                                      accumulate);
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
// device address of the array per device ordinal; a first call from two host threads at once
// looks the address up twice and stores the same value, so relaxed atomics suffice
std::atomic<double*> g_noalloc_scratch_addr[256] = {};
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
    double* scratch = g_noalloc_scratch_addr[dev].load(std::memory_order_relaxed);
    if (!scratch) {
        // once per device, with that device current: the host-side name of the array is not a
        // device address, so ask the runtime for this device's address of it
        e = cudaGetSymbolAddress(reinterpret_cast<void**>(&scratch), g_noalloc_scratch);
        if (e != cudaSuccess || !scratch) {
            xrh_set_last_cuda_error((int)e);
            return XRH_ERR_CUDA;
        }
        g_noalloc_scratch_addr[dev].store(scratch, std::memory_order_relaxed);
    }
    // the accumulate kernel overwrites every scratch element it uses: nothing to clear
    int st = xrh_density_accumulate(precision, K, idx_ptr_dev, P_dev, Q_dev, sign_dev, zbT_dev, n_b, zkT_dev, n_k,
                                    scratch, stream);
    if (st != XRH_OK) return st;
    return xrh_transpose(scratch, K, (int64_t)n_b * n_k, rho_dev, stream);
}

// ---- FP32 density build with asynchronous gathers ----------------------------------------
// Same product as density_acc_kernel<float>, for the split-precision paths.  The state
// coefficients come pre-converted to FP32 with rows padded to a multiple of 4 (16-byte
// aligned), so the z columns of a chunk of couplings are gathered with cp.async 16-byte
// copies into a double-buffered shared-memory ring: the gathers of chunk k+1 are in flight
// while chunk k is multiplied.  blockIdx.y splits the couplings of one operator index over
// several CTAs (for the operator strings with few indices, e.g. K = N); with splits > 1
// the partial sums are added atomically to rhoT, which the caller zeroes first.
namespace {


constexpr int kF32StageFloats = 8192;            // one stage of gathered rows: at most 32 KB

// Thread groups of the FP32 forward: a block of n_b x n_k has T = (n_b/4)(n_k/4) register
// tiles; when T < kAccThreads, G = kAccThreads / T groups of T threads share a stage, each
// group taking every G-th coupling, and their sums are combined at the end.
__host__ __device__ __forceinline__ int f32_groups(int nbp, int nkp) {
    const int T = (nbp >> 2) * (nkp >> 2);
    return T >= kAccThreads ? 1 : kAccThreads / T;
}
// Couplings per stage: 64 per group, as many as fit kF32StageFloats.
__host__ __device__ __forceinline__ int f32_chunk(int nbp, int nkp) {
    int c = 64 * f32_groups(nbp, nkp);
    const int cap = kF32StageFloats / (nbp + nkp);
    return c < cap ? c : (cap < 4 ? 4 : cap);
}

// One operator index (and one split of its couplings) per CTA: 4 x 4 register tiles of the
// n_b x n_k block over a double-buffered ring of gathered FP32 coefficient rows, ONE barrier
// per stage (the rows of stage k+1 are gathered with cp.async while stage k is multiplied).
// The coupling list of an index is ordered positive signs first (FragmentSpace), so the
// stages cover the positive range, then the negative one, and a stage multiplies with a
// uniform sign (the FFMA negates its operand for free).  FP32 stage sums are folded into
// FP32 (hi, lo) pairs by TwoSum and fl32(hi + lo) is written: the FP64 pipe, a small
// fraction of the FP32 rate on this part, stays idle.
__device__ __forceinline__ void density_f32_body(int64_t idx, int split, const int64_t* __restrict__ idx_ptr,
                                                 const int32_t* __restrict__ P, const int32_t* __restrict__ Q,
                                                 const int8_t* __restrict__ sgn, const float* __restrict__ zb32, int nb,
                                                 const float* __restrict__ zk32, int nk, double* __restrict__ rhoT,
                                                 int splits, unsigned char* smem_raw) {
    const int nbp = (nb + 3) & ~3, nkp = (nk + 3) & ~3;
    const int G = f32_groups(nbp, nkp), C = f32_chunk(nbp, nkp);
    float* zb_s = reinterpret_cast<float*>(smem_raw);               // [2][C][nbp]
    float* zk_s = zb_s + 2 * C * nbp;                                // [2][C][nkp]
    __shared__ int64_t s_split;
    const int64_t cb0 = idx_ptr[idx], ce0 = idx_ptr[idx + 1];
    const int64_t len = ce0 - cb0;
    const int64_t per = (len + splits - 1) / splits;
    const int64_t c_begin = cb0 + split * per;
    const int64_t c_end = (c_begin + per < ce0) ? c_begin + per : ce0;
    double* out = rhoT + idx * (int64_t)nb * nk;
    const int tiles_j = nkp / 4, n_tiles = (nbp / 4) * tiles_j;
    if (c_begin >= c_end) {
        if (splits == 1)
            for (int o = threadIdx.x; o < nb * nk; o += blockDim.x) out[o] = 0.0;
        return;
    }
    if (threadIdx.x == 0) {                       // first negative coupling (signs sorted + then -)
        int64_t lo = c_begin, hi = c_end;
        while (lo < hi) {
            const int64_t mid = (lo + hi) >> 1;
            if (__ldg(sgn + mid) < 0) hi = mid; else lo = mid + 1;
        }
        s_split = lo;
    }
    __syncthreads();
    const int64_t c_split = s_split;
    const int n_pos = (int)((c_split - c_begin + C - 1) / C);
    const int n_chunks = n_pos + (int)((c_end - c_split + C - 1) / C);
    const int gb = nbp / 4, gk = nkp / 4;
    auto range = [&](int k, int64_t& c0, int64_t& ce) {
        if (k < n_pos) {
            c0 = c_begin + (int64_t)k * C;
            ce = c_split;
        } else {
            c0 = c_split + (int64_t)(k - n_pos) * C;
            ce = c_end;
        }
    };
    auto stage = [&](int k, int buf) {
        int64_t c0, ce;
        range(k, c0, ce);
        float* zbb = zb_s + buf * C * nbp;
        float* zkb = zk_s + buf * C * nkp;
        for (int x = threadIdx.x; x < C * gb; x += blockDim.x) {
            const int c = x / gb, part = x - c * gb;
            const int64_t cc = c0 + c;
            if (cc < ce) cp_async16(zbb + c * nbp + part * 4, zb32 + (int64_t)__ldg(P + cc) * nbp + part * 4);
            else *reinterpret_cast<float4*>(zbb + c * nbp + part * 4) = make_float4(0.f, 0.f, 0.f, 0.f);
        }
        for (int x = threadIdx.x; x < C * gk; x += blockDim.x) {
            const int c = x / gk, part = x - c * gk;
            const int64_t cc = c0 + c;
            if (cc < ce) cp_async16(zkb + c * nkp + part * 4, zk32 + (int64_t)__ldg(Q + cc) * nkp + part * 4);
            else *reinterpret_cast<float4*>(zkb + c * nkp + part * 4) = make_float4(0.f, 0.f, 0.f, 0.f);
        }
        cp_async_commit();
    };

    const int active_threads = G * (n_tiles < kAccThreads ? n_tiles : kAccThreads);
    for (int t0 = 0; t0 < n_tiles; t0 += kAccThreads) {
        const bool grouped = G > 1;
        const int t = grouped ? (int)threadIdx.x % n_tiles : t0 + (int)threadIdx.x;
        const int grp = grouped ? (int)threadIdx.x / n_tiles : 0;
        const bool active = (int)threadIdx.x < active_threads && t < n_tiles;
        const int i0 = active ? (t / tiles_j) * 4 : 0, j0 = active ? (t % tiles_j) * 4 : 0;
        float acc[4][4], acc_lo[4][4];          // running sums as FP32 (hi, lo) pairs (TwoSum)
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                acc[a][b] = 0.f;
                acc_lo[a][b] = 0.f;
            }
        __syncthreads();                             // the ring is free (previous round done)
        stage(0, 0);
        for (int k = 0; k < n_chunks; ++k) {
            const int buf = k & 1;
            cp_async_wait<0>();
            __syncthreads();                         // stage k visible, stage k-1 consumed
            if (k + 1 < n_chunks) stage(k + 1, buf ^ 1);
            if (active) {
                const float* zbb = zb_s + buf * C * nbp;
                const float* zkb = zk_s + buf * C * nkp;
                float part[4][4] = {};
                if (k < n_pos) {
#pragma unroll 4
                    for (int c = grp; c < C; c += G) {
                        const float4 va = *reinterpret_cast<const float4*>(zbb + c * nbp + i0);
                        const float4 vb = *reinterpret_cast<const float4*>(zkb + c * nkp + j0);
                        const float av[4] = {va.x, va.y, va.z, va.w};
                        const float bv[4] = {vb.x, vb.y, vb.z, vb.w};
#pragma unroll
                        for (int a = 0; a < 4; ++a)
#pragma unroll
                            for (int b = 0; b < 4; ++b) part[a][b] = fmaf(av[a], bv[b], part[a][b]);
                    }
                } else {
#pragma unroll 4
                    for (int c = grp; c < C; c += G) {
                        const float4 va = *reinterpret_cast<const float4*>(zbb + c * nbp + i0);
                        const float4 vb = *reinterpret_cast<const float4*>(zkb + c * nkp + j0);
                        const float av[4] = {va.x, va.y, va.z, va.w};
                        const float bv[4] = {vb.x, vb.y, vb.z, vb.w};
#pragma unroll
                        for (int a = 0; a < 4; ++a)
#pragma unroll
                            for (int b = 0; b < 4; ++b) part[a][b] = fmaf(-av[a], bv[b], part[a][b]);
                    }
                }
#pragma unroll
                for (int a = 0; a < 4; ++a)
#pragma unroll
                    for (int b = 0; b < 4; ++b) {
                        float sum, err;
                        xrh_two_sum(acc[a][b], part[a][b], sum, err);
                        acc[a][b] = sum;
                        acc_lo[a][b] += err;
                    }
            }
        }
        if (grouped) {
            // combine the groups' (hi, lo) sums through the (now idle) ring, in group order
            __syncthreads();
            float* red = zb_s;                       // [G][n_tiles][32]: hi 16, lo 16
            if (active) {
                float* r = red + ((int64_t)grp * n_tiles + t) * 32;
#pragma unroll
                for (int a = 0; a < 4; ++a)
#pragma unroll
                    for (int b = 0; b < 4; ++b) {
                        r[a * 4 + b] = acc[a][b];
                        r[16 + a * 4 + b] = acc_lo[a][b];
                    }
            }
            __syncthreads();
            if (active && grp == 0) {
                for (int q = 1; q < G; ++q) {
                    const float* r = red + ((int64_t)q * n_tiles + t) * 32;
#pragma unroll
                    for (int a = 0; a < 4; ++a)
#pragma unroll
                        for (int b = 0; b < 4; ++b) {
                            float sum, err;
                            xrh_two_sum(acc[a][b], r[a * 4 + b], sum, err);
                            acc[a][b] = sum;
                            acc_lo[a][b] += err + r[16 + a * 4 + b];
                        }
                }
            }
        }
        if (active && grp == 0) {
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int b = 0; b < 4; ++b) {
                    if (i0 + a >= nb || j0 + b >= nk) continue;
                    double* o = out + (int64_t)(i0 + a) * nk + j0 + b;
                    const double v = xrh_f32_to_f64(__fadd_rn(acc[a][b], acc_lo[a][b]));
                    if (splits == 1) *o = v;
                    else atomicAdd(o, v);
                }
        }
        if (grouped) break;                          // every tile was covered by the groups
    }
}

// Shared memory (bytes) of the FP32 forward for the largest n_b, n_k of a launch: two stages
// of gathered rows, and the group reduction that reuses them.
static size_t f32_smem(int max_nb, int max_nk) {
    const int nbp = (max_nb + 3) & ~3, nkp = (max_nk + 3) & ~3;
    size_t need = 0;
    for (int b = 4; b <= nbp; b += 4)
        for (int k = 4; k <= nkp; k += 4) {
            const size_t ring = 2 * (size_t)f32_chunk(b, k) * (b + k);
            const int T = (b / 4) * (k / 4);
            const size_t red = T < kAccThreads ? (size_t)f32_groups(b, k) * T * 32 : 0;
            const size_t v = ring > red ? ring : red;
            need = v > need ? v : need;
        }
    return sizeof(float) * need;
}

__global__ void __launch_bounds__(kAccThreads, 3) density_acc_f32_kernel(
    const int64_t* __restrict__ idx_ptr, const int32_t* __restrict__ P, const int32_t* __restrict__ Q,
    const int8_t* __restrict__ sgn, const float* __restrict__ zb32, int nb, const float* __restrict__ zk32, int nk,
    double* __restrict__ rhoT, int splits) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    density_f32_body(blockIdx.x, blockIdx.y, idx_ptr, P, Q, sgn, zb32, nb, zk32, nk, rhoT, splits, smem_raw);
}

// Every block of a task table in one launch: CTA -> task by binary search on cta_begin.
__global__ void __launch_bounds__(kAccThreads, 3) density_acc_f32_grouped_kernel(const xrh_dens_task* __restrict__ tasks,
                                                                              int n_tasks) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    int lo = 0, hi = n_tasks - 1;
    const int64_t cta = blockIdx.x;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (tasks[mid].cta_begin <= cta) lo = mid; else hi = mid - 1;
    }
    const xrh_dens_task& T = tasks[lo];
    const int64_t local = cta - T.cta_begin;
    density_f32_body(local / T.splits, (int)(local % T.splits), T.idx_ptr, T.P, T.Q, T.sign, T.zb32, T.nb, T.zk32,
                     T.nk, T.rhoT, T.splits, smem_raw);
}


// Coefficient staging for the builds: for every task (one charge sector), zT[k][i] = src[i][k]
// (FP64, K x n) and zT32[k][i] = fl32(src[i][k]) (FP32, K x npad, columns n.. npad left as
// they are: zero from allocation).  Thread per row k of the launch (rows of a task start at
// row_begin; CTAs of 256 rows find their task by binary search).
__global__ void __launch_bounds__(256) coeff_stage_kernel(const xrh_coeff_task* __restrict__ tasks, int n_tasks,
                                                          int64_t total_rows) {
    const int64_t row = (int64_t)blockIdx.x * 256 + threadIdx.x;
    const int64_t row0 = (int64_t)blockIdx.x * 256;
    int lo = 0, hi = n_tasks - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (tasks[mid].row_begin <= row0) lo = mid; else hi = mid - 1;
    }
    // a CTA's rows may run into the next task: step forward per thread
    int t = lo;
    while (t + 1 < n_tasks && tasks[t + 1].row_begin <= row) ++t;
    if (row >= total_rows) return;
    const xrh_coeff_task& T = tasks[t];
    const int64_t k = row - T.row_begin;
    if (k >= T.K) return;
    for (int i = 0; i < T.n; ++i) {
        const double x = T.src[(int64_t)i * T.K + k];
        if (T.zT) T.zT[k * T.n + i] = x;
        if (T.zT32) T.zT32[k * T.npad + i] = xrh_f64_to_f32(x);
    }
}

// ---- small blocks: one warp per coupling range ----------------------------------------------
// For blocks of at most 16 states per side a CTA per operator index leaves most threads idle
// and pays three barriers per chunk.  Here a warp owns one unit (an operator index, or a range
// of at most a few hundred of its couplings) and walks its couplings 32 at a time:
//   * staging: lane l copies the padded FP32 rows zb[P_c] and zk[Q_c] of coupling c = c0 + l
//     into the warp's shared-memory buffer with cp.async (one instruction gathers 32 rows),
//     one chunk ahead of the compute, double buffered;
//   * compute: lane l holds the output quads (I, 4 jq .. 4 jq + 3), I * ceil(n_k/4) + jq =
//     l + 32 r (r < R); per staged coupling it reads zb[I] and the float4 zk[4 jq..] from
//     shared memory and the sign by shuffle, and does four FMAs.
// Accumulation stays off the FP64 pipe (a small fraction of the FP32 rate on this part): FP32
// partial sums per chunk are folded into FP32 (hi, lo) pairs by TwoSum and fl32(hi + lo) is
// written to the FP64 rhoT.  Units covering a whole index store rhoT[idx]; units of a split
// index add atomically (rhoT zeroed by the caller).
// Staged row: [zb (nbp floats) | zk (nkp floats)], stride = an odd number of float4s.
constexpr int UNIT_WARPS = 4;

__host__ __device__ __forceinline__ int unit_stride(int nbp, int nkp) {
    const int q = (nbp + nkp) / 4;
    return 4 * (q | 1);
}

template <int R>
__global__ void __launch_bounds__(UNIT_WARPS * 32) density_f32_units_kernel(const xrh_dens_task* __restrict__ tasks,
                                                                           const xrh_dens_unit* __restrict__ units,
                                                                           int64_t n_units, int max_stride) {
    extern __shared__ __align__(16) float usm[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t u = (int64_t)blockIdx.x * UNIT_WARPS + warp;
    if (u >= n_units) return;
    const xrh_dens_unit U = units[u];
    const xrh_dens_task& T = tasks[U.task];
    const int nb = T.nb, nk = T.nk;
    const int nbp = (nb + 3) & ~3, nkp = (nk + 3) & ~3, nbq = nbp >> 2, nkq = nkp >> 2;
    const int stride = unit_stride(nbp, nkp);
    const int pairs = nb * nkq;
    if (pairs > 32 * R || stride > max_stride) return;      // the host never builds such a unit
    float* buf0 = usm + (int64_t)warp * 2 * 32 * max_stride;
    const int64_t base = T.idx_ptr[U.idx];
    const int64_t len = T.idx_ptr[U.idx + 1] - base;
    const int64_t c_lo = base + U.c_lo, c_hi = base + U.c_hi;
    const bool whole = U.c_lo == 0 && (int64_t)U.c_hi == len;
    int Iu[R], jq[R];
    bool act[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int pr = lane + 32 * r;
        act[r] = pr < pairs;
        Iu[r] = act[r] ? pr / nkq : 0;
        jq[r] = act[r] ? pr - (pr / nkq) * nkq : 0;
    }
    float hi[R][4], lo[R][4];
#pragma unroll
    for (int r = 0; r < R; ++r)
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            hi[r][k] = 0.f;
            lo[r][k] = 0.f;
        }
    const float* __restrict__ zb = T.zb32;
    const float* __restrict__ zk = T.zk32;
    // stage the chunk starting at c0 into buffer b; returns this lane's sign (0 beyond c_hi)
    auto stage = [&](int64_t c0, int b) -> float {
        const int64_t c = c0 + lane;
        float sg = 0.f;
        if (c < c_hi) {
            const int p = T.P[c], q = T.Q[c];
            sg = T.sign[c] < 0 ? -1.f : 1.f;
            float* row = buf0 + (b * 32 + lane) * max_stride;
            const float* zbr = zb + (int64_t)p * nbp;
            const float* zkr = zk + (int64_t)q * nkp;
            for (int x = 0; x < nbq; ++x) cp_async16_ca(row + 4 * x, zbr + 4 * x);
            for (int x = 0; x < nkq; ++x) cp_async16_ca(row + nbp + 4 * x, zkr + 4 * x);
        }
        cp_async_commit();
        return sg;
    };
    float s_cur = stage(c_lo, 0);
    int b = 0;
    for (int64_t c0 = c_lo; c0 < c_hi; c0 += 32) {
        float s_next = 0.f;
        if (c0 + 32 < c_hi) {
            s_next = stage(c0 + 32, b ^ 1);
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncwarp();
        const float* rows = buf0 + b * 32 * max_stride;
        const int cnt = (int)((c_hi - c0) < 32 ? (c_hi - c0) : 32);
        float part[R][4];
#pragma unroll
        for (int r = 0; r < R; ++r)
#pragma unroll
            for (int k = 0; k < 4; ++k) part[r][k] = 0.f;
#pragma unroll 4
        for (int t = 0; t < cnt; ++t) {
            const float st = __shfl_sync(0xffffffffu, s_cur, t);
            const float* row = rows + t * max_stride;
#pragma unroll
            for (int r = 0; r < R; ++r) {
                if (act[r]) {
                    const float a = st * row[Iu[r]];
                    const float4 b4 = *reinterpret_cast<const float4*>(row + nbp + 4 * jq[r]);
                    part[r][0] = fmaf(a, b4.x, part[r][0]);
                    part[r][1] = fmaf(a, b4.y, part[r][1]);
                    part[r][2] = fmaf(a, b4.z, part[r][2]);
                    part[r][3] = fmaf(a, b4.w, part[r][3]);
                }
            }
        }
#pragma unroll
        for (int r = 0; r < R; ++r)
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                float sum, err;
                xrh_two_sum(hi[r][k], part[r][k], sum, err);
                hi[r][k] = sum;
                lo[r][k] += err;
            }
        __syncwarp();                                  // buffer b is restaged two chunks on
        s_cur = s_next;
        b ^= 1;
    }
    double* out = T.rhoT + (int64_t)U.idx * nb * nk;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        if (!act[r]) continue;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int J = 4 * jq[r] + k;
            if (J >= nk) continue;
            const double v = xrh_f32_to_f64(__fadd_rn(hi[r][k], lo[r][k]));
            double* o = out + (int64_t)Iu[r] * nk + J;
            if (whole) *o = v;
            else atomicAdd(o, v);
        }
    }
}

}  // namespace

extern "C" int xrh_density_accumulate_f32_grouped(const xrh_dens_task* tasks_dev, int n_tasks, int64_t total_ctas,
                                                  int max_nb, int max_nk, void* stream) {
    if (n_tasks < 0 || total_ctas < 0 || max_nb <= 0 || max_nk <= 0) return XRH_ERR_ARG;
    if (n_tasks == 0 || total_ctas == 0) return XRH_OK;
    if (!tasks_dev) return XRH_ERR_ARG;
    if (total_ctas > 0x7fffffffLL) return XRH_ERR_CAPACITY;
    if (max_nb > 1024 || max_nk > 1024) return XRH_ERR_CAPACITY;
    const size_t smem = f32_smem(max_nb, max_nk);
    if (smem > 200 * 1024) return XRH_ERR_CAPACITY;
    if (smem > 48 * 1024)
        cudaFuncSetAttribute(density_acc_f32_grouped_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    density_acc_f32_grouped_kernel<<<(unsigned)total_ctas, kAccThreads, smem, (cudaStream_t)stream>>>(tasks_dev,
                                                                                                     n_tasks);
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}

extern "C" int xrh_density_accumulate_f32(int64_t K, int splits, const int64_t* idx_ptr_dev, const int32_t* P_dev,
                                          const int32_t* Q_dev, const int8_t* sign_dev, const float* zb32_dev, int n_b,
                                          const float* zk32_dev, int n_k, double* rhoT_dev, void* stream) {
    if (K <= 0 || n_b <= 0 || n_k <= 0 || splits < 1 || splits > 65535 || !idx_ptr_dev || !zb32_dev || !zk32_dev ||
        !rhoT_dev)
        return XRH_ERR_ARG;
    if (K > 0x7fffffffLL) return XRH_ERR_CAPACITY;
    if ((reinterpret_cast<uintptr_t>(zb32_dev) & 15) || (reinterpret_cast<uintptr_t>(zk32_dev) & 15)) return XRH_ERR_ARG;
    if (n_b > 1024 || n_k > 1024) return XRH_ERR_CAPACITY;
    const size_t smem = f32_smem(n_b, n_k);
    if (smem > 200 * 1024) return XRH_ERR_CAPACITY;
    if (smem > 48 * 1024)
        cudaFuncSetAttribute(density_acc_f32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    dim3 grid((unsigned)K, (unsigned)splits);
    density_acc_f32_kernel<<<grid, kAccThreads, smem, (cudaStream_t)stream>>>(idx_ptr_dev, P_dev, Q_dev, sign_dev,
                                                                             zb32_dev, n_b, zk32_dev, n_k, rhoT_dev,
                                                                             splits);
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}

extern "C" int xrh_density_accumulate_f32_units(const xrh_dens_task* tasks_dev, int n_tasks,
                                                const xrh_dens_unit* units_dev, int64_t n_units, int max_n,
                                                void* stream) {
    if (n_tasks < 0 || n_units < 0 || max_n <= 0) return XRH_ERR_ARG;
    if (max_n > 16) return XRH_ERR_CAPACITY;
    if (n_tasks == 0 || n_units == 0) return XRH_OK;
    if (!tasks_dev || !units_dev) return XRH_ERR_ARG;
    const int64_t ctas = (n_units + UNIT_WARPS - 1) / UNIT_WARPS;
    if (ctas > 0x7fffffffLL) return XRH_ERR_CAPACITY;
    const int np = (max_n + 3) & ~3;
    const int max_stride = unit_stride(np, np);     // 4 (q | 1) grows with q: the largest stride
    const size_t smem = sizeof(float) * (size_t)UNIT_WARPS * 2 * 32 * (size_t)max_stride;
    cudaStream_t s = (cudaStream_t)stream;
    // output quads per warp: max_n * ceil(max_n / 4) <= 64
    if (max_n * ((max_n + 3) / 4) <= 32)
        density_f32_units_kernel<1><<<(unsigned)ctas, UNIT_WARPS * 32, smem, s>>>(tasks_dev, units_dev, n_units,
                                                                                  max_stride);
    else
        density_f32_units_kernel<2><<<(unsigned)ctas, UNIT_WARPS * 32, smem, s>>>(tasks_dev, units_dev, n_units,
                                                                                  max_stride);
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}

extern "C" int xrh_coeff_stage(const xrh_coeff_task* tasks_dev, int n_tasks, int64_t total_rows, void* stream) {
    if (n_tasks < 0 || total_rows < 0) return XRH_ERR_ARG;
    if (n_tasks == 0 || total_rows == 0) return XRH_OK;
    if (!tasks_dev) return XRH_ERR_ARG;
    const int64_t ctas = (total_rows + 255) / 256;
    if (ctas > 0x7fffffffLL) return XRH_ERR_CAPACITY;
    coeff_stage_kernel<<<(unsigned)ctas, 256, 0, (cudaStream_t)stream>>>(tasks_dev, n_tasks, total_rows);
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}

extern "C" int xrh_transpose_grouped(const xrh_transpose_task* tasks_dev, int n_tasks, int64_t total_tiles,
                                     void* stream) {
    if (n_tasks < 0 || total_tiles < 0) return XRH_ERR_ARG;
    if (n_tasks == 0 || total_tiles == 0) return XRH_OK;
    if (!tasks_dev) return XRH_ERR_ARG;
    if (total_tiles > 0x7fffffffLL) return XRH_ERR_CAPACITY;
    transpose_grouped_kernel<<<(unsigned)total_tiles, dim3(32, 8), 0, (cudaStream_t)stream>>>(tasks_dev, n_tasks);
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}

extern "C" int xrh_mirror_grouped(const xrh_mirror_task* tasks_dev, int n_tasks, int64_t total_ctas, void* stream) {
    if (n_tasks < 0 || total_ctas < 0) return XRH_ERR_ARG;
    if (n_tasks == 0 || total_ctas == 0) return XRH_OK;
    if (!tasks_dev) return XRH_ERR_ARG;
    if (total_ctas > 0x7fffffffLL) return XRH_ERR_CAPACITY;
    mirror_grouped_kernel<<<(unsigned)total_ctas, 256, 0, (cudaStream_t)stream>>>(tasks_dev, n_tasks);
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}
