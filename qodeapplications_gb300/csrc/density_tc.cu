// Adjoint of the transition densities on the tensor cores (3 x TF32 split, tcgen05).
//
// For one operator index idx with density gradient G = dE/drho[idx] (n_b x n_k) and the
// couplings (P_c, Q_c, s_c) of idx, the coefficient gradients are
//     dE/dzk[Q_c, J] += s_c sum_I zb[P_c, I] G[I, J]     (ket direction)
//     dE/dzb[P_c, I] += s_c sum_J zk[Q_c, J] G[I, J]     (bra direction)
// i.e. two small GEMMs per tile of 128 couplings with gathered coefficient rows as the
// K-major A operand (M = couplings, K = states) and G (or G^T) as the K-major B operand
// (N = states).  Per CTA (one operator index, 4 warps):
//   * G is loaded once, split into TF32 hi/lo and written in both orientations into
//     128-byte-swizzled shared-memory tiles (rows padded with zeros to 64);
//   * per tile of 128 couplings: the pre-split coefficient rows (64 TF32 per row, zero
//     padded) are gathered with 16-byte cp.async copies into the same swizzle, thread 0
//     issues A_hi.B_hi + A_hi.B_lo + A_lo.B_hi for K = 64 (24 MMAs of 128 x 64 x 8 per
//     direction) into TMEM, and the 4 warps read their 32 rows back (tcgen05.ld), scale
//     by s_c and add them to the FP32 gradient rows with 16-byte vector atomics.
// K = 64 is 8 MMA steps per product: no accumulator needs draining.  Every mbarrier wait
// is bounded (status XRH_ERR_TIMEOUT, then the CTA frees its TMEM and returns).
#include "tc_common.cuh"
#include "xrh_common.cuh"

namespace {
using namespace xrh_tc;

constexpr int DT_THREADS = 128;
constexpr int DT_M = 128;                       // couplings per tile (TMEM lanes)
constexpr int DT_N = 64;                        // states, padded
constexpr uint32_t DT_A_TILE = DT_M * 128;      // one K-chunk (32 TF32) of 128 rows: 16 KB
constexpr uint32_t DT_B_TILE = DT_N * 128;      // one K-chunk of 64 rows: 8 KB
// [Bw: G^T, rows J][Bu: G, rows I] x [chunk 0, 1] x [hi, lo], then A [chunk] x [hi, lo]
constexpr uint32_t DT_OFF_BW = 0;
constexpr uint32_t DT_OFF_BU = 4 * DT_B_TILE;
constexpr uint32_t DT_OFF_A = 8 * DT_B_TILE;
constexpr uint32_t DT_SMEM = 8 * DT_B_TILE + 4 * DT_A_TILE;   // 128 KB

// byte offset of TF32 element (row, k), k < 32, in a 128-byte-swizzled K-chunk tile
__device__ __forceinline__ uint32_t sw_off(int row, int k) {
    return (uint32_t)(row * 128 + ((((k >> 2) ^ (row & 7)) << 4) | ((k & 3) << 2)));
}

__device__ __forceinline__ void split_tf32(double x, uint32_t& h, uint32_t& l) {
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"((float)x));
    const double rem = x - (double)__uint_as_float(h);
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(l) : "f"((float)rem));
}

__device__ __forceinline__ void atomic_row4(float* dst, const float* v, float s, int n) {
    for (int j = 0; j < n; j += 4) {
        const int valid = n - j < 4 ? n - j : 4;
        if (valid == 4 && (reinterpret_cast<uintptr_t>(dst + j) & 15) == 0) {
            xrh_red_add_v4(dst + j, s * v[j], s * v[j + 1], s * v[j + 2], s * v[j + 3]);
        } else {
            for (int t = 0; t < valid; ++t) xrh_red_add(dst + j + t, s * v[j + t]);
        }
    }
}

__global__ void __launch_bounds__(DT_THREADS, 1)
    density_adjoint_tc_kernel(const xrh_dens_adj_tc_task* __restrict__ tasks, int n_tasks, int32_t* status) {
    extern __shared__ unsigned char smem_raw[];
    uint8_t* sm = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    __shared__ __align__(8) uint64_t mma_bar;
    __shared__ uint32_t tmem_base_sh;
    __shared__ int sP[DT_M], sQ[DT_M];
    __shared__ float sS[DT_M];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    int lo = 0, hi = n_tasks - 1;
    const int64_t cta = blockIdx.x;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (tasks[mid].cta_begin <= cta) lo = mid; else hi = mid - 1;
    }
    const xrh_dens_adj_tc_task& T = tasks[lo];
    const int64_t idx = cta - T.cta_begin;
    const int64_t cb = T.idx_ptr[idx], ce = T.idx_ptr[idx + 1];
    if (cb >= ce) return;                       // uniform: nothing allocated yet
    const int nb = T.nb, nk = T.nk;

    if (tid == 0) {
        mbar_init(smem_u32(&mma_bar), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base_sh)),
                     "r"(128u)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    // zero the G tiles (padding rows and columns stay zero), then write G split in both layouts
    for (uint32_t o = tid * 16; o < 8 * DT_B_TILE; o += DT_THREADS * 16)
        *reinterpret_cast<uint4*>(sm + o) = make_uint4(0u, 0u, 0u, 0u);
    __syncthreads();
    const double* gi = T.gT + idx * (int64_t)nb * nk;
    for (int e = tid; e < nb * nk; e += DT_THREADS) {
        const int I = e / nk, J = e - I * nk;
        uint32_t h, l;
        split_tf32(gi[e], h, l);
        // Bu: rows I, K = J       Bw: rows J, K = I
        uint8_t* bu = sm + DT_OFF_BU + (uint32_t)(J >> 5) * 2 * DT_B_TILE;
        uint8_t* bw = sm + DT_OFF_BW + (uint32_t)(I >> 5) * 2 * DT_B_TILE;
        *reinterpret_cast<uint32_t*>(bu + sw_off(I, J & 31)) = h;
        *reinterpret_cast<uint32_t*>(bu + DT_B_TILE + sw_off(I, J & 31)) = l;
        *reinterpret_cast<uint32_t*>(bw + sw_off(J, I & 31)) = h;
        *reinterpret_cast<uint32_t*>(bw + DT_B_TILE + sw_off(J, I & 31)) = l;
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base_sh;
    const uint32_t idesc = make_idesc(2u, DT_M, DT_N, false);
    uint32_t phase = 0;
    bool failed = false;

    for (int64_t c0 = cb; c0 < ce && !failed; c0 += DT_M) {
        {
            const int64_t c = c0 + tid;
            const bool ok = c < ce;
            sP[tid] = ok ? T.P[c] : -1;
            sQ[tid] = ok ? T.Q[c] : -1;
            sS[tid] = ok ? (T.sign[c] < 0 ? -1.f : 1.f) : 0.f;
        }
        __syncthreads();
        for (int dir = 0; dir < 2; ++dir) {
            // dir 0 (ket direction): A = zb rows of P_c, B = G^T;  dir 1: A = zk rows of Q_c, B = G
            const int src = dir == 0 ? sP[tid] : sQ[tid];
            const uint32_t* rh = dir == 0 ? T.zbh : T.zkh;
            const uint32_t* rl = dir == 0 ? T.zbl : T.zkl;
            const int r = tid;
#pragma unroll
            for (int part = 0; part < 2; ++part) {
                const uint32_t* row = (part == 0 ? rh : rl) + (int64_t)(src < 0 ? 0 : src) * DT_N;
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    uint8_t* dst = sm + DT_OFF_A + (uint32_t)((j >> 3) * 2 + part) * DT_A_TILE + (uint32_t)r * 128 +
                                   (uint32_t)(((j & 7) ^ (r & 7)) << 4);
                    if (src >= 0) cp_async16(dst, row + j * 4);
                    else *reinterpret_cast<uint4*>(dst) = make_uint4(0u, 0u, 0u, 0u);
                }
            }
            cp_async_commit();
            cp_async_wait<0>();
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            tc_fence_before();
            __syncthreads();
            tc_fence_after();
            if (tid == 0) {
                const uint32_t d = tmem + (uint32_t)dir * 64u;
                const uint32_t Bb = smem_u32(sm + (dir == 0 ? DT_OFF_BW : DT_OFF_BU));
                const uint32_t Ab = smem_u32(sm + DT_OFF_A);
#pragma unroll
                for (int kc = 0; kc < 2; ++kc) {
                    const uint64_t a_hi = umma_desc_sw128(Ab + (uint32_t)(kc * 2) * DT_A_TILE);
                    const uint64_t a_lo = umma_desc_sw128(Ab + (uint32_t)(kc * 2 + 1) * DT_A_TILE);
                    const uint64_t b_hi = umma_desc_sw128(Bb + (uint32_t)(kc * 2) * DT_B_TILE);
                    const uint64_t b_lo = umma_desc_sw128(Bb + (uint32_t)(kc * 2 + 1) * DT_B_TILE);
                    const uint64_t pa[3] = {a_hi, a_hi, a_lo};
                    const uint64_t pb[3] = {b_hi, b_lo, b_hi};
#pragma unroll
                    for (int p = 0; p < 3; ++p)
#pragma unroll
                        for (int st = 0; st < 4; ++st)   // 4 MMA K-steps of 8 TF32 (32 bytes) per chunk
                            umma<1>(d, pa[p] + 2 * st, pb[p] + 2 * st, idesc, (kc | p | st) ? 1u : 0u);
                }
                umma_commit(smem_u32(&mma_bar));
            }
            // MMAs done: the A tiles may be overwritten and TMEM read
            const bool got = mbar_wait(smem_u32(&mma_bar), phase & 1u, nullptr);
            ++phase;
            if (__syncthreads_or(!got)) {
                failed = true;
                if (tid == 0) atomicExch(status, XRH_ERR_TIMEOUT);
                break;
            }
            tc_fence_after();
        }
        if (failed) break;
        // epilogue: warp w reads TMEM lanes 32w.. (rows = couplings of this tile)
        const int r = warp * 32 + lane;
        const float s = sS[r];
#pragma unroll
        for (int dir = 0; dir < 2; ++dir) {
            float va[32], vb[32];
            const uint32_t ta = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)dir * 64u;
            tmem_ld_pair(ta, ta + 32u, va, vb);
            if (s != 0.f) {
                float v[64];
#pragma unroll
                for (int j = 0; j < 32; ++j) {
                    v[j] = va[j];
                    v[32 + j] = vb[j];
                }
                if (dir == 0) atomic_row4(T.gzk + (int64_t)sQ[r] * nk, v, s, nk);
                else atomic_row4(T.gzb + (int64_t)sP[r] * nb, v, s, nb);
            }
        }
        tc_fence_before();
        __syncthreads();                        // TMEM read and indices used before the next tile
        tc_fence_after();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(128u) : "memory");
    }
}

}  // namespace

extern "C" int xrh_density_adjoint_tc_grouped(const xrh_dens_adj_tc_task* tasks_dev, int n_tasks, int64_t total_ctas,
                                              int32_t* status_dev, void* stream) {
    if (n_tasks < 0 || total_ctas < 0) return XRH_ERR_ARG;
    if (n_tasks == 0 || total_ctas == 0) return XRH_OK;
    if (!tasks_dev || !status_dev) return XRH_ERR_ARG;
    if (total_ctas > 0x7fffffffLL) return XRH_ERR_CAPACITY;
    const size_t smem = DT_SMEM + 1024;
    cudaFuncSetAttribute(density_adjoint_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    density_adjoint_tc_kernel<<<(unsigned)total_ctas, DT_THREADS, smem, (cudaStream_t)stream>>>(tasks_dev, n_tasks,
                                                                                              status_dev);
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}
