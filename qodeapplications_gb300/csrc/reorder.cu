// Reordering of the three-fragment vectors (matrix-free H x v of general-XRCC's three-fragment
// Hamiltonian, general-XRCC/hamiltonian.py:18-80 assembled from build_H.py:38-188):
//
//   xrh_permute_grouped: dst = scale * permute(src) for up to 6-index row-major blocks, every
//       block of a task table in one launch (element per thread, tasks found by binary search
//       on elem_begin);
//   xrh_gather_sum: dst[j] (+)= sum_t src_t[idx_t[j]] for up to 8 (src, idx) pairs, added in
//       pair order -- the return of several permuted accumulators into one vector without
//       atomics (idx_t the inverse of the permutation that made src_t).
// Both are HBM-bound copies: 8 bytes read and 8 written per element and term.
#include "xrh_common.cuh"

namespace {

__global__ void __launch_bounds__(256) permute_grouped_kernel(const xrh_permute_task* __restrict__ tasks, int n_tasks,
                                                              int64_t total) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= total) return;
    int lo = 0, hi = n_tasks - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (tasks[mid].elem_begin <= e) lo = mid; else hi = mid - 1;
    }
    const xrh_permute_task& T = tasks[lo];
    int64_t r = e - T.elem_begin;
    if (r >= T.n_elems) return;
    // dst is row-major over dst_shape; walk its indices from the last one
    int64_t off = 0;
    for (int k = T.ndim - 1; k >= 0; --k) {
        const int64_t d = T.dst_shape[k];
        const int64_t i = r % d;
        r /= d;
        off += i * T.src_stride[k];
    }
    T.dst[e - T.elem_begin] = T.scale * T.src[off];
}

__global__ void __launch_bounds__(256) gather_sum_kernel(int64_t n, xrh_gather_terms terms, double* __restrict__ dst,
                                                         int accumulate) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    double s = accumulate ? dst[j] : 0.0;
    for (int t = 0; t < terms.n_terms; ++t) s += terms.src[t][terms.idx[t][j]];
    dst[j] = s;
}

}  // namespace

extern "C" int xrh_permute_grouped(const xrh_permute_task* tasks_dev, int n_tasks, int64_t total_elems,
                                   void* stream) {
    if (n_tasks < 0 || total_elems < 0) return XRH_ERR_ARG;
    if (n_tasks == 0 || total_elems == 0) return XRH_OK;
    if (!tasks_dev) return XRH_ERR_ARG;
    if ((total_elems + 255) / 256 > 0x7fffffffLL) return XRH_ERR_CAPACITY;
    permute_grouped_kernel<<<(unsigned)((total_elems + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
        tasks_dev, n_tasks, total_elems);
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}

extern "C" int xrh_gather_sum(int64_t n, const xrh_gather_terms* terms, double* dst_dev, int accumulate,
                              void* stream) {
    if (n < 0 || !terms || terms->n_terms < 0 || terms->n_terms > 8) return XRH_ERR_ARG;
    if (n == 0) return XRH_OK;
    if (!dst_dev) return XRH_ERR_ARG;
    for (int t = 0; t < terms->n_terms; ++t)
        if (!terms->src[t] || !terms->idx[t]) return XRH_ERR_ARG;
    if ((n + 255) / 256 > 0x7fffffffLL) return XRH_ERR_CAPACITY;
    gather_sum_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(n, *terms, dst_dev, accumulate);
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}
