// Shared definitions for the XR-H CUDA library (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/xrh.h"

extern "C" void xrh_set_last_cuda_error(int e);

#define XRH_CHECK_LAUNCH()                                   \
    do {                                                     \
        cudaError_t e_ = cudaGetLastError();                 \
        if (e_ != cudaSuccess) {                             \
            xrh_set_last_cuda_error((int)e_);                \
            return XRH_ERR_CUDA;                             \
        }                                                    \
    } while (0)

// Parity of moving a field operator on spin orbital o to the end of an ascending
// occupation list: (-1)^(number of occupied orbitals above o).  Same rule as the
// reference's annihilate/create (general-XRCC/density_tensors.c:80-113).
__device__ __forceinline__ int xrh_above_parity(uint64_t mask, int o) {
    return (o >= 63) ? 0 : (__popcll(mask >> (o + 1)) & 1);
}

// Apply c+_o (is_c = 1) or a_o (is_c = 0).  Returns false on a Pauli violation.
__device__ __forceinline__ bool xrh_apply(int is_c, int o, uint64_t& m, int& sgn) {
    const uint64_t bit = 1ull << o;
    const int occ = (m & bit) ? 1 : 0;
    if (occ == is_c) return false;
    sgn ^= xrh_above_parity(m, o);
    m ^= bit;
    return true;
}

// Position of mask in an ascending-sorted mask array, or -1.
__device__ __forceinline__ int xrh_lookup(const uint64_t* __restrict__ sorted, int n, uint64_t key) {
    int lo = 0, hi = n - 1;
    while (lo <= hi) {
        int mid = (lo + hi) >> 1;
        uint64_t v = __ldg(sorted + mid);
        if (v == key) return mid;
        if (v < key) lo = mid + 1; else hi = mid - 1;
    }
    return -1;
}
