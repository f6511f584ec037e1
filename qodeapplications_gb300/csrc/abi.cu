// Status helpers of the C ABI (include/xrh.h).
#include "xrh_common.cuh"

static int g_last_cuda_error = 0;

extern "C" void xrh_set_last_cuda_error(int e) { g_last_cuda_error = e; }

extern "C" int xrh_abi_version(void) { return 1; }

extern "C" const char* xrh_status_string(int status) {
    switch (status) {
        case XRH_OK: return "ok";
        case XRH_ERR_ARG: return "invalid argument";
        case XRH_ERR_CUDA: return "CUDA error";
        case XRH_ERR_UNSUPPORTED: return "unsupported precision or feature";
        case XRH_ERR_TIMEOUT: return "bounded device wait timed out";
        case XRH_ERR_CAPACITY: return "size exceeds a documented limit";
        default: return "unknown status";
    }
}

extern "C" int xrh_last_cuda_error(void) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) g_last_cuda_error = (int)e;
    return g_last_cuda_error;
}

static_assert(sizeof(xrh_gemm_segment) == 72, "xrh_gemm_segment layout is part of the ABI");
static_assert(sizeof(xrh_gemm_task) == 152, "xrh_gemm_task layout is part of the ABI");
static_assert(sizeof(xrh_tc_segment) == 32, "xrh_tc_segment layout is part of the ABI");
static_assert(sizeof(xrh_dens_task) == 88, "xrh_dens_task layout is part of the ABI");
static_assert(sizeof(xrh_dens_adj_task) == 96, "xrh_dens_adj_task layout is part of the ABI");
static_assert(sizeof(xrh_dens_adj_tc_task) == 112, "xrh_dens_adj_tc_task layout is part of the ABI");
static_assert(sizeof(xrh_pair_task) == 72, "xrh_pair_task layout is part of the ABI");
static_assert(sizeof(xrh_orbital_inputs) == 128, "xrh_orbital_inputs layout is part of the ABI");
static_assert(sizeof(xrh_mirror_task) == 48, "xrh_mirror_task layout is part of the ABI");
static_assert(sizeof(xrh_antisym_task) == 48, "xrh_antisym_task layout is part of the ABI");
static_assert(sizeof(xrh_transpose_task) == 40, "xrh_transpose_task layout is part of the ABI");
static_assert(sizeof(xrh_coeff_task) == 56, "xrh_coeff_task layout is part of the ABI");
static_assert(sizeof(xrh_abt_task) == 88, "xrh_abt_task layout is part of the ABI");
static_assert(sizeof(xrh_gemv_task) == 72, "xrh_gemv_task layout is part of the ABI");
static_assert(sizeof(xrh_split_task) == 64, "xrh_split_task layout is part of the ABI");
static_assert(sizeof(xrh_dens_unit) == 16, "xrh_dens_unit layout is part of the ABI");
static_assert(sizeof(xrh_state_task) == 80, "xrh_state_task layout is part of the ABI");
static_assert(sizeof(xrh_tc_task) == 144, "xrh_tc_task layout is part of the ABI");
static_assert(sizeof(xrh_small_mm_task) == 56, "xrh_small_mm_task layout is part of the ABI");
static_assert(sizeof(xrh_permute_task) == 144, "xrh_permute_task layout is part of the ABI");
static_assert(sizeof(xrh_gather_terms) == 136, "xrh_gather_terms layout is part of the ABI");
