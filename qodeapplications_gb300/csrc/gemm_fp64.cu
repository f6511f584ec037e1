// Plain FP64 grouped GEMM with K-concatenated segments and the XR-H epilogue.
//
// This is the drop-in FP64 path.  Every density x integral contraction of the H build
// (precontractions of hermitian-XRCC/precontract.py:32-80, final diagram contractions of
// diagrams/S*_2mer_0.py, element formulas of general-XRCC/H_contractions.c) is one
// segment; all segments that land in the same charge block of H are summed in one task,
// so each H element is produced once and stored once (mode 2), with the delta-function
// terms (u100, monomer H1 x 1) added in the epilogue.  One launch covers every task: a
// flat tile index is mapped to (task, tile) by binary search over the tasks' tile_begin.
//
// GB300 FP64 throughput is low (about 2 DFMA/clk/SM), so this kernel is DFMA-bound at any
// reasonable tiling: 64x64 tiles, 256 threads, 4x4 outputs per thread, K staged in 16s.
#include "xrh_common.cuh"

namespace {

constexpr int BM = 64, BN = 64, BK = 16, NT = 256;

__device__ __forceinline__ int find_task(const xrh_gemm_task* __restrict__ tasks, int n_tasks, int64_t tile) {
    int lo = 0, hi = n_tasks - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (tasks[mid].tile_begin <= tile) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// T = double: the plain FP64 path.  T = float (the adjoint on the split-precision paths):
// operands rounded to FP32 (by integer operations) into shared memory, products and partial
// sums of each 32 K in FP32, running sums as FP32 (hi, lo) pairs by TwoSum, results written
// as fl32(hi + lo).  Nothing of the float variant runs on the FP64 pipe, a small fraction of
// the FP32 rate on this part.
template <typename T_>
__global__ void __launch_bounds__(NT) gemm_fp64_kernel(const xrh_gemm_task* __restrict__ tasks, int n_tasks,
                                                      const xrh_gemm_segment* __restrict__ segs) {
    __shared__ T_ As[BK][BM + 1];
    __shared__ T_ Bs[BK][BN + 1];
    const int64_t tile = blockIdx.x;
    const int t_id = find_task(tasks, n_tasks, tile);
    const xrh_gemm_task& Tk = tasks[t_id];
    const int64_t tiles_m = (Tk.M + BM - 1) / BM, tiles_n = (Tk.N + BN - 1) / BN;
    int64_t local = tile - Tk.tile_begin;
    const int64_t per_batch = tiles_m * tiles_n * Tk.splitk;
    const int64_t bidx = local / per_batch;
    local -= bidx * per_batch;
    const int64_t split = local / (tiles_m * tiles_n);
    local -= split * tiles_m * tiles_n;
    const int64_t m0 = (local / tiles_n) * BM, n0 = (local % tiles_n) * BN;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    constexpr bool F32 = sizeof(T_) == 4;
    double acc[4][4];                  // FP64 variant
    float hi[4][4], lo[4][4];          // FP32 variant
    T_ part[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            acc[i][j] = 0.0;
            hi[i][j] = 0.f;
            lo[i][j] = 0.f;
            part[i][j] = (T_)0;
        }
    int pending = 0;                   // K steps summed in part since the last fold

    for (int64_t s = Tk.seg_begin; s < Tk.seg_begin + Tk.seg_count; ++s) {
        const xrh_gemm_segment S = segs[s];
        const double* __restrict__ Ap = S.A + bidx * S.sA;
        const double* __restrict__ Bp = S.B + bidx * S.sB;
        const bool at = (S.flags & 1) != 0, bt = (S.flags & 2) != 0;
        const float alpha32 = F32 ? xrh_f64_to_f32(S.alpha) : 0.f;
        int64_t kb = 0, ke = S.K;
        if (Tk.splitk > 1) {
            const int64_t per = (S.K + Tk.splitk - 1) / Tk.splitk;
            kb = split * per;
            ke = (kb + per < S.K) ? kb + per : S.K;
        }
        for (int64_t k0 = kb; k0 < ke; k0 += BK) {
            __syncthreads();
#pragma unroll
            for (int e = 0; e < (BM * BK) / NT; ++e) {
                const int l = threadIdx.x + e * NT;
                // K-contiguous operands: consecutive threads walk k; otherwise they walk m / n
                const int r = l / BK, c = l % BK;
                const int r2 = l % BM, c2 = l / BM;
                {
                    const int rr = at ? r2 : r, cc = at ? c2 : c;
                    const int64_t gm = m0 + rr, gk = k0 + cc;
                    const double x = (gm < Tk.M && gk < ke) ? (at ? Ap[gk * S.lda + gm] : Ap[gm * S.lda + gk]) : 0.0;
                    if constexpr (F32) As[cc][rr] = alpha32 * xrh_f64_to_f32(x);
                    else As[cc][rr] = S.alpha * x;
                }
                {
                    const int rr = bt ? r2 : r, cc = bt ? c2 : c;
                    const int64_t gn = n0 + rr, gk = k0 + cc;
                    const double x = (gn < Tk.N && gk < ke) ? (bt ? Bp[gk * S.ldb + gn] : Bp[gn * S.ldb + gk]) : 0.0;
                    if constexpr (F32) Bs[cc][rr] = xrh_f64_to_f32(x);
                    else Bs[cc][rr] = x;
                }
            }
            __syncthreads();
#pragma unroll
            for (int kk = 0; kk < BK; ++kk) {
                T_ a[4], b[4];
#pragma unroll
                for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
                for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
                for (int i = 0; i < 4; ++i)
#pragma unroll
                    for (int j = 0; j < 4; ++j) part[i][j] = fma(a[i], b[j], part[i][j]);
            }
            if constexpr (F32) {
                if (++pending == 2) {          // fold every 32 products
#pragma unroll
                    for (int i = 0; i < 4; ++i)
#pragma unroll
                        for (int j = 0; j < 4; ++j) {
                            float sum, err;
                            xrh_two_sum(hi[i][j], (float)part[i][j], sum, err);
                            hi[i][j] = sum;
                            lo[i][j] += err;
                            part[i][j] = (T_)0;
                        }
                    pending = 0;
                }
            } else {
#pragma unroll
                for (int i = 0; i < 4; ++i)
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        acc[i][j] += (double)part[i][j];
                        part[i][j] = (T_)0;
                    }
            }
        }
    }
    if constexpr (F32) {
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                float sum, err;
                xrh_two_sum(hi[i][j], (float)part[i][j], sum, err);
                acc[i][j] = xrh_f32_to_f64(__fadd_rn(sum, lo[i][j] + err));
            }
    }

#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int64_t m = m0 + ty + 16 * i;
        if (m >= Tk.M) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int64_t n = n0 + tx + 16 * j;
            if (n >= Tk.N) continue;
            double v = acc[i][j];
            double* Cb = Tk.C + bidx * Tk.sC;
            if (Tk.mode == 0) {
                Cb[m * Tk.ldc + n] = v;
            } else if (Tk.mode == 1) {
                atomicAdd(Cb + m * Tk.ldc + n, v);
            } else {
                if (Tk.DA && Tk.diagB[n]) v += Tk.DA[m];
                if (Tk.DB && Tk.diagA[m]) v += Tk.DB[n];
                Cb[((int64_t)Tk.rowA[m] + Tk.rowB[n]) * Tk.ldc + Tk.colA[m] + Tk.colB[n]] = v;
            }
        }
    }
}

}  // namespace

extern "C" int xrh_gemm_simt_grouped(int precision, const xrh_gemm_task* tasks_dev, int n_tasks, int64_t total_tiles,
                                     const xrh_gemm_segment* segs_dev, void* stream) {
    if (n_tasks < 0 || total_tiles < 0) return XRH_ERR_ARG;
    if (n_tasks == 0 || total_tiles == 0) return XRH_OK;
    if (!tasks_dev || !segs_dev) return XRH_ERR_ARG;
    if (total_tiles > 0x7fffffffLL) return XRH_ERR_CAPACITY;
    if (precision == XRH_FP64)
        gemm_fp64_kernel<double><<<(unsigned)total_tiles, NT, 0, (cudaStream_t)stream>>>(tasks_dev, n_tasks, segs_dev);
    else if (precision == XRH_FP32)
        gemm_fp64_kernel<float><<<(unsigned)total_tiles, NT, 0, (cudaStream_t)stream>>>(tasks_dev, n_tasks, segs_dev);
    else
        return XRH_ERR_UNSUPPORTED;
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}

extern "C" int xrh_gemm_fp64_grouped(const xrh_gemm_task* tasks_dev, int n_tasks, int64_t total_tiles,
                                     const xrh_gemm_segment* segs_dev, void* stream) {
    return xrh_gemm_simt_grouped(XRH_FP64, tasks_dev, n_tasks, total_tiles, segs_dev, stream);
}
