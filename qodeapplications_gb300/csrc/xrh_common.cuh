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

// Position of a determinant through its colexicographic rank: rank = sum_i C(o_i, i+1) over
// the occupied orbitals o_0 < o_1 < ... (binom[n*17 + k] = C(n, k), n <= 64, k <= 16), then
// pos_table[rank] (-1 where the determinant is not in the list).  n_e fast steps and one
// table load instead of a binary search over the sorted list.
__device__ __forceinline__ int xrh_rank_lookup(const int32_t* __restrict__ pos_table, int64_t table_size,
                                               const int64_t* __restrict__ binom, uint64_t mask) {
    int64_t r = 0;
    int i = 1;
    while (mask) {
        const int o = __ffsll((long long)mask) - 1;
        if (i > 16) return -1;
        r += __ldg(binom + o * 17 + i);
        mask &= mask - 1;
        ++i;
    }
    return (r < table_size) ? __ldg(pos_table + r) : -1;
}

// 16-byte asynchronous global -> shared copies (both addresses 16-byte aligned)
__device__ __forceinline__ void cp_async16(void* smem_dst, const void* gmem_src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(smem_dst)),
                 "l"(gmem_src)
                 : "memory");
}
// Error-free FP32 sum (Knuth's TwoSum): s + e == a + b exactly, s = fl(a + b).
__device__ __forceinline__ void xrh_two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// Exact FP32 -> FP64 by integer operations (keeps conversions off the FP64 pipe, which is a
// small fraction of the FP32 rate on this part).  Zero, subnormal, infinite and NaN inputs
// take the hardware conversion.
__device__ __forceinline__ double xrh_f32_to_f64(float f) {
    const uint32_t u = __float_as_uint(f);
    const uint32_t e = (u >> 23) & 0xffu;
    if (e == 0u || e == 0xffu) return (double)f;
    const uint64_t bits = ((uint64_t)(u >> 31) << 63) | ((uint64_t)(e + 896u) << 52) | ((uint64_t)(u & 0x7fffffu) << 29);
    return __longlong_as_double((long long)bits);
}

// FP64 -> FP32 round-to-nearest-even by integer operations (same result as __double2float_rn;
// zero takes a shortcut, values outside the normal FP32 range the hardware conversion).
__device__ __forceinline__ float xrh_f64_to_f32(double x) {
    const uint64_t b = (uint64_t)__double_as_longlong(x);
    if ((b << 1) == 0) return __uint_as_float((uint32_t)(b >> 32) & 0x80000000u);
    const uint32_t e = (uint32_t)(b >> 52) & 0x7ffu;
    if (e < 897u || e > 1150u) return __double2float_rn(x);
    uint32_t m = (uint32_t)(b >> 29) & 0x7fffffu;
    const uint32_t rem = (uint32_t)b & 0x1fffffffu;
    uint32_t fe = e - 896u;
    if (rem > 0x10000000u || (rem == 0x10000000u && (m & 1u))) {
        m += 1u;
        if (m == 0x800000u) {
            m = 0u;
            fe += 1u;
        }
    }
    if (fe >= 255u) return __double2float_rn(x);
    return __uint_as_float(((uint32_t)(b >> 63) << 31) | (fe << 23) | m);
}

// Fire-and-forget vector additions to global memory (red: no value comes back, so nothing
// waits on the L2 round trip; the vector atomicAdd overloads return the old value).
// Addresses 16- (v4) or 8-byte (v2) aligned.
__device__ __forceinline__ void xrh_red_add_v4(float* addr, float a, float b, float c, float d) {
    asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(addr), "f"(a), "f"(b), "f"(c), "f"(d)
                 : "memory");
}
__device__ __forceinline__ void xrh_red_add_v2(float* addr, float a, float b) {
    asm volatile("red.global.add.v2.f32 [%0], {%1, %2};" ::"l"(addr), "f"(a), "f"(b) : "memory");
}
__device__ __forceinline__ void xrh_red_add(float* addr, float a) {
    asm volatile("red.global.add.f32 [%0], %1;" ::"l"(addr), "f"(a) : "memory");
}

// Same through L1 (gathers with reuse across warps of an SM).
__device__ __forceinline__ void cp_async16_ca(void* smem_dst, const void* gmem_src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(smem_dst)),
                 "l"(gmem_src)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }
