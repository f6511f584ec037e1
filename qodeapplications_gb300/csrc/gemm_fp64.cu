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

__global__ void __launch_bounds__(NT) gemm_fp64_kernel(const xrh_gemm_task* __restrict__ tasks, int n_tasks,
                                                      const xrh_gemm_segment* __restrict__ segs) {
    __shared__ double As[BK][BM + 1];
    __shared__ double Bs[BK][BN + 1];
    const int64_t tile = blockIdx.x;
    const int t_id = find_task(tasks, n_tasks, tile);
    const xrh_gemm_task& T = tasks[t_id];
    const int64_t tiles_m = (T.M + BM - 1) / BM, tiles_n = (T.N + BN - 1) / BN;
    int64_t local = tile - T.tile_begin;
    const int64_t per_batch = tiles_m * tiles_n * T.splitk;
    const int64_t bidx = local / per_batch;
    local -= bidx * per_batch;
    const int64_t split = local / (tiles_m * tiles_n);
    local -= split * tiles_m * tiles_n;
    const int64_t m0 = (local / tiles_n) * BM, n0 = (local % tiles_n) * BN;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    double acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;

    for (int64_t s = T.seg_begin; s < T.seg_begin + T.seg_count; ++s) {
        const xrh_gemm_segment S = segs[s];
        const double* __restrict__ Ap = S.A + bidx * S.sA;
        const double* __restrict__ Bp = S.B + bidx * S.sB;
        const bool at = (S.flags & 1) != 0, bt = (S.flags & 2) != 0;
        int64_t kb = 0, ke = S.K;
        if (T.splitk > 1) {
            const int64_t per = (S.K + T.splitk - 1) / T.splitk;
            kb = split * per;
            ke = (kb + per < S.K) ? kb + per : S.K;
        }
        double sacc[4][4];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) sacc[i][j] = 0.0;
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
                    As[cc][rr] = (gm < T.M && gk < ke) ? (at ? Ap[gk * S.lda + gm] : Ap[gm * S.lda + gk]) : 0.0;
                }
                {
                    const int rr = bt ? r2 : r, cc = bt ? c2 : c;
                    const int64_t gn = n0 + rr, gk = k0 + cc;
                    Bs[cc][rr] = (gn < T.N && gk < ke) ? (bt ? Bp[gk * S.ldb + gn] : Bp[gn * S.ldb + gk]) : 0.0;
                }
            }
            __syncthreads();
#pragma unroll
            for (int kk = 0; kk < BK; ++kk) {
                double a[4], b[4];
#pragma unroll
                for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
                for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
                for (int i = 0; i < 4; ++i)
#pragma unroll
                    for (int j = 0; j < 4; ++j) sacc[i][j] = fma(a[i], b[j], sacc[i][j]);
            }
        }
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) acc[i][j] = fma(S.alpha, sacc[i][j], acc[i][j]);
    }

#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int64_t m = m0 + ty + 16 * i;
        if (m >= T.M) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int64_t n = n0 + tx + 16 * j;
            if (n >= T.N) continue;
            double v = acc[i][j];
            double* Cb = T.C + bidx * T.sC;
            if (T.mode == 0) {
                Cb[m * T.ldc + n] = v;
            } else if (T.mode == 1) {
                atomicAdd(Cb + m * T.ldc + n, v);
            } else {
                if (T.DA && T.diagB[n]) v += T.DA[m];
                if (T.DB && T.diagA[m]) v += T.DB[n];
                Cb[((int64_t)T.rowA[m] + T.rowB[n]) * T.ldc + T.colA[m] + T.colB[n]] = v;
            }
        }
    }
}

}  // namespace

extern "C" int xrh_gemm_fp64_grouped(const xrh_gemm_task* tasks_dev, int n_tasks, int64_t total_tiles,
                                     const xrh_gemm_segment* segs_dev, void* stream) {
    if (n_tasks < 0 || total_tiles < 0) return XRH_ERR_ARG;
    if (n_tasks == 0 || total_tiles == 0) return XRH_OK;
    if (!tasks_dev || !segs_dev) return XRH_ERR_ARG;
    if (total_tiles > 0x7fffffffLL) return XRH_ERR_CAPACITY;
    gemm_fp64_kernel<<<(unsigned)total_tiles, NT, 0, (cudaStream_t)stream>>>(tasks_dev, n_tasks, segs_dev);
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}
