// Split-precision grouped GEMM on the 5th-generation tensor cores (tcgen05, sm_103a).
//
// Same task model as the FP64 path (gemm_fp64.cu): every output block of the XR-H build is
// one task whose K-concatenated segments are the density x integral contractions that land
// in it.  Each FP64 operand X is split once per build into hi = round(X) and
// lo = round(X - hi) in BF16 (XRH_BF16X3) or TF32 (XRH_TF32X3); a segment contributes
//     A_hi B_hi^T + A_hi B_lo^T + A_lo B_hi^T.
//
// Accuracy: the tensor core's FP32 accumulation is not round-to-nearest, and its error grows
// with the number of MMA steps summed into one accumulator.  So no accumulator outlives a K
// chunk (128 bytes of K: 64 BF16 / 32 TF32 elements): every chunk writes a fresh main slot
// (hi*hi, 4 MMA steps) and a fresh correction slot (hi*lo + lo*hi, 8 steps, 2^-8 smaller),
// and the epilogue warps drain both into FP32 registers with ordinary round-to-nearest adds
// while the tensor core works on the next chunk.  The tile is converted to FP64 once, where
// the segment-independent delta terms are added and the result is scattered like the FP64
// path.
//
// Per CTA (persistent over 128 x BN output tiles, one CTA per SM), 9 warps:
//   * warp 8, one thread: TMA loads (cp.async.bulk.tensor, 128B swizzle) of the four operand
//     tiles of a chunk into a 3-stage shared-memory ring, prefetched across tile boundaries,
//     and the 12 tcgen05.mma of each chunk into one of two TMEM chunk buffers (main +
//     correction slot, 128 columns each: 512 columns); tcgen05.commit releases the ring stage
//     (empty) and hands the buffer to the epilogue (ready);
//   * warps 0-7: per chunk, tcgen05.ld of both slots (warp w reads TMEM lanes 32(w%4).. =
//     rows, 32-column groups alternate between w<4 and w>=4), add into registers, release the
//     buffer (drained); at the end of the tile, the FP64 epilogue.
// Every mbarrier wait is bounded; on timeout the kernel records XRH_ERR_TIMEOUT in *status,
// every warp leaves its loop (the epilogue warps decide together through bar.red.or once per
// tile), the producer waits (bounded) for its copies and MMAs in flight, TMEM is freed and the
// kernel returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include "tc_common.cuh"
#include "xrh_common.cuh"

namespace {
using namespace xrh_tc;

constexpr int TC_BM = 128;
constexpr int TC_STAGES = 3;
constexpr int TC_EPI_WARPS = 8;
constexpr int TC_EPI_THREADS = TC_EPI_WARPS * 32;
constexpr int TC_THREADS = TC_EPI_THREADS + 32;    // + the producer / MMA warp
constexpr uint32_t TC_TMEM_COLS = 512;             // 2 chunk buffers x (main, correction) x 128
constexpr uint32_t TC_A_BYTES = TC_BM * 128;       // 128 rows x 128 B (one swizzle width of K)
constexpr uint32_t TC_B_MAX_BYTES = 128 * 128;
constexpr uint32_t TC_STAGE_BYTES = 2 * TC_A_BYTES + 2 * TC_B_MAX_BYTES;
constexpr long long TC_IDLE_LIMIT = 1LL << 26;     // producer polls without progress before giving up

// Named barrier 1 over the epilogue warps, returning the OR of a predicate over them.
__device__ __forceinline__ int epi_bar_or(int pred) {
    int r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\tsetp.ne.b32 p, %1, 0;\n\t"
        "bar.red.or.pred q, 1, %2, p;\n\tselp.b32 %0, 1, 0, q;\n\t}\n"
        : "=r"(r)
        : "r"(pred), "n"(TC_EPI_THREADS)
        : "memory");
    return r;
}
__device__ __forceinline__ void epi_bar() { asm volatile("bar.sync 1, %0;" ::"n"(TC_EPI_THREADS) : "memory"); }

__device__ __forceinline__ int find_task(const xrh_tc_task* __restrict__ tasks, int n_tasks, int64_t tile) {
    int lo = 0, hi = n_tasks - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (tasks[mid].tile_begin <= tile) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Where a persistent CTA's tile lies: its task, output corner, N tile and K-chunk range.
struct TileInfo {
    int task, m0, n0, BN, nk;
    int64_t cb;
};

__device__ __forceinline__ TileInfo tile_info(const xrh_tc_task* __restrict__ tasks, int n_tasks,
                                              const xrh_tc_segment* __restrict__ segs, int64_t tile) {
    TileInfo r;
    r.task = find_task(tasks, n_tasks, tile);
    const xrh_tc_task& T = tasks[r.task];
    r.BN = (int)T.bn;
    const int64_t tiles_m = (T.M + TC_BM - 1) / TC_BM, tiles_n = (T.N + r.BN - 1) / r.BN;
    int64_t local = tile - T.tile_begin;
    const int64_t split = local / (tiles_m * tiles_n);
    local -= split * tiles_m * tiles_n;
    // the CTAs running at once take consecutive tiles: they walk the M tiles of one N tile when
    // M < N, so the smaller operand (A, M x K) is the one every CTA re-reads (from L2) and each
    // tile of the larger one comes from HBM once; else the N tiles of one M tile
    if (T.M < T.N) {
        r.m0 = (int)((local % tiles_m) * TC_BM);
        r.n0 = (int)((local / tiles_m) * r.BN);
    } else {
        r.m0 = (int)((local / tiles_n) * TC_BM);
        r.n0 = (int)((local % tiles_n) * r.BN);
    }
    int64_t kc_total = 0;
    for (int64_t s = 0; s < T.seg_count; ++s) kc_total += segs[T.seg_begin + s].kchunks;
    const int64_t per = (kc_total + T.splitk - 1) / T.splitk;
    r.cb = split * per;
    const int64_t ce = (r.cb + per < kc_total) ? r.cb + per : kc_total;
    r.nk = (int)(ce > r.cb ? ce - r.cb : 0);
    return r;
}

template <int KIND>
__global__ void __launch_bounds__(TC_THREADS, 1)
    gemm_tc_kernel(const xrh_tc_task* __restrict__ tasks, int n_tasks, int64_t total_tiles,
                   const xrh_tc_segment* __restrict__ segs, const CUtensorMap* __restrict__ maps, int32_t* status) {
    extern __shared__ unsigned char smem_raw[];
    uint8_t* stages = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    __shared__ __align__(8) uint64_t full_bar[TC_STAGES];
    __shared__ __align__(8) uint64_t empty_bar[TC_STAGES];
    __shared__ __align__(8) uint64_t ready_bar[2];
    __shared__ __align__(8) uint64_t drained_bar[2];
    __shared__ __align__(8) uint64_t done_bar;
    __shared__ uint32_t tmem_base_sh;
    __shared__ volatile int abort_sh;
    __shared__ int s_rowB[128], s_colB[128];
    __shared__ double s_DB[128];
    // per-row metadata of the tile and the 32-column staging slice of the epilogue
    __shared__ int64_t s_rbase[128], s_cbase[128];
    __shared__ double s_DA[128];
    __shared__ unsigned char s_diagA[128];
    __shared__ float s_stage[128][33];
    __shared__ unsigned char s_diagB[128];
    constexpr int KCH = (KIND == 0) ? 64 : 32;          // elements of K per 128-byte chunk
    constexpr uint32_t FMT = (KIND == 0) ? 1u : 2u;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    if (tid == 0) {
        for (int s = 0; s < TC_STAGES; ++s) {
            mbar_init(smem_u32(&full_bar[s]), 1);
            mbar_init(smem_u32(&empty_bar[s]), 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(smem_u32(&ready_bar[b]), 1);
            mbar_init(smem_u32(&drained_bar[b]), TC_EPI_WARPS);
        }
        mbar_init(smem_u32(&done_bar), 1);
        abort_sh = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncwarp();
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base_sh)),
                     "r"(TC_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base_sh;

    if (warp == TC_EPI_WARPS) {
        // ------------------------------------------------------------ producer + MMA --
        if (lane == 0) {
            uint64_t gl = 0, gm = 0;           // chunks loaded / consumed by MMAs (global order)
            int64_t tl = blockIdx.x, tm = blockIdx.x;
            int ql = 0, qm = 0;
            TileInfo L{}, Mi{};
            bool l_ok = false, m_ok = false;
            // next tile with at least one chunk, from tile t on
            auto seek = [&](int64_t& t, TileInfo& I) -> bool {
                for (; t < total_tiles; t += gridDim.x) {
                    I = tile_info(tasks, n_tasks, segs, t);
                    if (I.nk > 0) return true;
                }
                return false;
            };
            // running (segment, chunk-in-segment) cursors of the loads and the MMAs: a tile's
            // start is located once (its split-K offset), then each chunk advances the cursor
            // instead of walking the task's segment list from its first segment again
            int64_t l_si = 0, l_c = 0, m_si = 0, m_c = 0;
            l_ok = seek(tl, L);
            m_ok = seek(tm, Mi);
            if (l_ok) { l_si = tasks[L.task].seg_begin; l_c = L.cb; }
            if (m_ok) { m_si = tasks[Mi.task].seg_begin; m_c = Mi.cb; }
            bool ok = true;
            // one thread drives both queues without blocking on either: a load is issued as soon
            // as its ring stage is free, the MMAs of a chunk as soon as its operands have landed
            // and its TMEM buffer is drained, so that the next chunk's MMAs queue behind the
            // running ones; a stretch of TC_IDLE_LIMIT polls without progress gives up
            long long idle = 0;
            while (m_ok && ok) {
                bool progress = false;
                while (l_ok && gl < gm + TC_STAGES) {
                    const int s = (int)(gl % TC_STAGES);
                    if (gl >= TC_STAGES && !mbar_test(smem_u32(&empty_bar[s]), (uint32_t)((gl / TC_STAGES) - 1) & 1u))
                        break;
                    while (l_c >= segs[l_si].kchunks) { l_c -= segs[l_si].kchunks; ++l_si; }
                    const xrh_tc_segment& S = segs[l_si];
                    const int kcoord = (int)(l_c * KCH);
                    ++l_c;
                    const uint32_t b_bytes = (uint32_t)L.BN * 128u;
                    uint8_t* st = stages + (size_t)s * TC_STAGE_BYTES;
                    const uint32_t bar = smem_u32(&full_bar[s]);
                    mbar_expect_tx(bar, 2u * TC_A_BYTES + 2u * b_bytes);
                    tma_load_2d(smem_u32(st), maps + S.tmA, bar, kcoord, L.m0);
                    tma_load_2d(smem_u32(st + TC_A_BYTES), maps + S.tmA + 1, bar, kcoord, L.m0);
                    tma_load_2d(smem_u32(st + 2 * TC_A_BYTES), maps + S.tmB, bar, kcoord, L.n0);
                    tma_load_2d(smem_u32(st + 2 * TC_A_BYTES + b_bytes), maps + S.tmB + 1, bar, kcoord, L.n0);
                    ++gl;
                    progress = true;
                    if (++ql == L.nk) {
                        ql = 0;
                        tl += gridDim.x;
                        l_ok = seek(tl, L);
                        if (l_ok) { l_si = tasks[L.task].seg_begin; l_c = L.cb; }
                    }
                }
                // the MMAs of chunk gm into chunk buffer gm & 1
                const int s = (int)(gm % TC_STAGES);
                const uint32_t b = (uint32_t)(gm & 1);
                if (gm < gl && mbar_test(smem_u32(&full_bar[s]), (uint32_t)(gm / TC_STAGES) & 1u) &&
                    (gm < 2 || mbar_test(smem_u32(&drained_bar[b]), (uint32_t)((gm >> 1) - 1) & 1u))) {
                    tc_fence_after();
                    while (m_c >= segs[m_si].kchunks) { m_c -= segs[m_si].kchunks; ++m_si; }
                    const uint32_t idesc = make_idesc(FMT, TC_BM, (uint32_t)Mi.BN, segs[m_si].negate != 0);
                    ++m_c;
                    const uint32_t b_bytes = (uint32_t)Mi.BN * 128u;
                    const uint32_t st = smem_u32(stages + (size_t)s * TC_STAGE_BYTES);
                    const uint64_t da_hi = umma_desc_sw128(st), da_lo = umma_desc_sw128(st + TC_A_BYTES);
                    const uint64_t db_hi = umma_desc_sw128(st + 2 * TC_A_BYTES);
                    const uint64_t db_lo = umma_desc_sw128(st + 2 * TC_A_BYTES + b_bytes);
                    const uint32_t t_main = tmem + b * 256u, t_corr = t_main + 128u;
#pragma unroll
                    for (int j = 0; j < 4; ++j)              // 4 MMA K-steps of 32 bytes inside the chunk
                        umma<KIND>(t_main, da_hi + 2 * j, db_hi + 2 * j, idesc, j > 0 ? 1u : 0u);
#pragma unroll
                    for (int j = 0; j < 4; ++j) umma<KIND>(t_corr, da_hi + 2 * j, db_lo + 2 * j, idesc, j > 0 ? 1u : 0u);
#pragma unroll
                    for (int j = 0; j < 4; ++j) umma<KIND>(t_corr, da_lo + 2 * j, db_hi + 2 * j, idesc, 1u);
                    umma_commit(smem_u32(&empty_bar[s]));
                    umma_commit(smem_u32(&ready_bar[b]));
                    ++gm;
                    progress = true;
                    if (++qm == Mi.nk) {
                        qm = 0;
                        tm += gridDim.x;
                        m_ok = seek(tm, Mi);
                        if (m_ok) { m_si = tasks[Mi.task].seg_begin; m_c = Mi.cb; }
                    }
                }
                if (progress) {
                    idle = 0;
                } else if (++idle > TC_IDLE_LIMIT || abort_sh) {
                    ok = false;
                }
            }
            if (!ok) {
                abort_sh = 1;
                atomicExch(status, XRH_ERR_TIMEOUT);
            }
            // before TMEM and shared memory go away: every MMA issued has completed, and every
            // copy issued has landed (bounded waits)
            if (gm > 0) {
                umma_commit(smem_u32(&done_bar));
                mbar_wait(smem_u32(&done_bar), 0u, nullptr);
            }
            for (uint64_t g = gm; g < gl; ++g)
                mbar_wait(smem_u32(&full_bar[g % TC_STAGES]), (uint32_t)(g / TC_STAGES) & 1u, nullptr);
        }
    } else {
        // ------------------------------------------------------------------ epilogue --
        const int quarter = warp & 3, half = warp >> 2;      // TMEM lanes 32*quarter.., column half
        uint64_t ge = 0;
        bool aborted = false;
        for (int64_t tile = blockIdx.x; tile < total_tiles && !aborted; tile += gridDim.x) {
            const TileInfo I = tile_info(tasks, n_tasks, segs, tile);
            if (I.nk == 0) continue;
            const xrh_tc_task& T = tasks[I.task];
            const int BN = I.BN, m0 = I.m0, n0 = I.n0;
            if (T.mode == 2) {
                for (int j = tid; j < BN; j += TC_EPI_THREADS) {
                    const int n = n0 + j;
                    const bool ok = n < T.N;
                    s_rowB[j] = ok ? T.rowB[n] : 0;
                    s_colB[j] = ok ? T.colB[n] : 0;
                    s_diagB[j] = ok ? T.diagB[n] : 0;
                    s_DB[j] = (ok && T.DB) ? T.DB[n] : 0.0;
                }
            }
            float acc[2][32];
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
                for (int j = 0; j < 32; ++j) acc[i][j] = 0.f;
            // the warps drain their chunks independently; a wait that gives up raises abort_sh,
            // so the others' waits give up too, and all decide together once per tile below
            bool failed = false;
            for (int q = 0; q < I.nk; ++q, ++ge) {
                const uint32_t b = (uint32_t)(ge & 1);
                if (!mbar_wait(smem_u32(&ready_bar[b]), (uint32_t)(ge >> 1) & 1u, &abort_sh)) {
                    failed = true;
                    abort_sh = 1;
                    break;
                }
                tc_fence_after();
                const uint32_t lane_base = (uint32_t)(quarter * 32) << 16;
#pragma unroll
                for (int i = 0; i < 2; ++i) {
                    const int cc = half * 32 + 64 * i;
                    if (cc < BN) {
                        float vm[32], vc[32];
                        tmem_ld_pair(tmem + lane_base + b * 256u + (uint32_t)cc,
                                     tmem + lane_base + b * 256u + 128u + (uint32_t)cc, vm, vc);
#pragma unroll
                        for (int j = 0; j < 32; ++j) acc[i][j] += vm[j] + vc[j];
                    }
                }
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(smem_u32(&drained_bar[b]));
            }
            // one collective decision per tile (also the barrier after the column metadata)
            if (epi_bar_or(failed)) aborted = true;
            if (aborted) {
                abort_sh = 1;
                if (tid == 0) atomicExch(status, XRH_ERR_TIMEOUT);
                break;
            }
            // FP64 epilogue, one 32-column slice at a time: the 4 warps that hold the slice put it
            // into shared memory (a row per lane), then every warp writes 16 rows with its lanes
            // on consecutive columns, so that stores (and atomics) of a warp touch few cache
            // lines.  Column metadata came before the decision barrier; row metadata first:
            for (int rr = tid; rr < TC_BM; rr += TC_EPI_THREADS) {
                const int m = m0 + rr;
                int64_t rb = 0, cb2 = 0;
                unsigned char dgA = 0;
                double dam = 0.0;
                if (m < T.M) {
                    if (T.mode == 2) {
                        rb = T.rowA[m];
                        cb2 = T.colA[m];
                        dgA = T.diagA[m];
                        dam = T.DA ? T.DA[m] : 0.0;
                    } else {
                        rb = (int64_t)m * T.ldc;
                    }
                }
                s_rbase[rr] = rb;
                s_cbase[rr] = cb2;
                s_diagA[rr] = dgA;
                s_DA[rr] = dam;
            }
            double* C = T.C;
#pragma unroll
            for (int p = 0; p < 4; ++p) {
                const int c0 = 32 * p;
                if (c0 >= BN) break;                                   // uniform
                if (half == (p & 1)) {
#pragma unroll
                    for (int j = 0; j < 32; ++j) s_stage[quarter * 32 + lane][j] = acc[p >> 1][j];
                }
                epi_bar();
                const int jj = c0 + lane;
                const bool col_ok = n0 + jj < T.N;
                for (int rr = warp * 16; rr < warp * 16 + 16; ++rr) {
                    if (m0 + rr >= T.M) break;                         // uniform within the warp
                    if (!col_ok) continue;
                    double x = (double)s_stage[rr][lane];
                    if (T.mode == 2) {
                        if (s_diagB[jj]) x += s_DA[rr];
                        if (s_diagA[rr]) x += s_DB[jj];
                        C[(s_rbase[rr] + s_rowB[jj]) * T.ldc + s_cbase[rr] + s_colB[jj]] = x;
                    } else if (T.mode == 0) {
                        C[s_rbase[rr] + n0 + jj] = x;
                    } else {
                        atomicAdd(C + s_rbase[rr] + n0 + jj, x);
                    }
                }
                epi_bar();                                             // slice consumed
            }
            epi_bar();          // metadata reads done before the next tile overwrites it
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_TMEM_COLS) : "memory");
    }
}

// ---- operand split --------------------------------------------------------------------
// One thread per group of 4 consecutive K elements of a row (one division per group), one
// 8- or 16-byte store per group and part.
template <int KIND>
__device__ __forceinline__ void split_group(const double* __restrict__ src, int64_t K, int64_t ld, int64_t Kp,
                                            void* __restrict__ hi, void* __restrict__ lo, int64_t t) {
    const int64_t groups = Kp >> 2;
    const int64_t r = t / groups;
    const int64_t k0 = (t - r * groups) * 4;
    const double* srow = src + r * ld;
    // x rounded to FP32 by integer operations; hi from it and lo = x32 - hi, exact in FP32 (it
    // keeps the low mantissa bits of x32); the part of x below FP32 (2^-24 |x|) lies under
    // lo's own resolution.  No FP64 arithmetic: the FP64 pipe is slow on this part.
    float x[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) x[e] = (k0 + e < K) ? xrh_f64_to_f32(__ldg(srow + k0 + e)) : 0.f;
    const int64_t o = r * Kp + k0;
    if constexpr (KIND == 0) {
        __nv_bfloat16 h[4], l[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            h[e] = __float2bfloat16_rn(x[e]);
            l[e] = __float2bfloat16_rn(__fsub_rn(x[e], __bfloat162float(h[e])));
        }
        *reinterpret_cast<uint2*>(reinterpret_cast<__nv_bfloat16*>(hi) + o) = *reinterpret_cast<uint2*>(h);
        *reinterpret_cast<uint2*>(reinterpret_cast<__nv_bfloat16*>(lo) + o) = *reinterpret_cast<uint2*>(l);
    } else {
        uint32_t h[4], l[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h[e]) : "f"(x[e]));
            const float rem = __fsub_rn(x[e], __uint_as_float(h[e]));
            asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(l[e]) : "f"(rem));
        }
        *reinterpret_cast<uint4*>(reinterpret_cast<uint32_t*>(hi) + o) = make_uint4(h[0], h[1], h[2], h[3]);
        *reinterpret_cast<uint4*>(reinterpret_cast<uint32_t*>(lo) + o) = make_uint4(l[0], l[1], l[2], l[3]);
    }
}

template <int KIND>
__global__ void split_kernel(const double* __restrict__ src, int64_t rows, int64_t K, int64_t ld, int64_t Kp,
                             void* __restrict__ hi, void* __restrict__ lo) {
    const int64_t total = rows * (Kp >> 2);
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x)
        split_group<KIND>(src, K, ld, Kp, hi, lo, t);
}

// Every operand of a task table in one launch: global 4-element group g belongs to the task
// with the last group_begin <= g (binary search over the group_begin values staged in shared
// memory, SPLIT_SMEM_TASKS of them at most; larger tables search global memory).
constexpr int SPLIT_SMEM_TASKS = 512;

template <int KIND>
__global__ void __launch_bounds__(256) split_grouped_kernel(const xrh_split_task* __restrict__ tasks, int n_tasks,
                                                            int64_t total) {
    __shared__ int64_t s_begin[SPLIT_SMEM_TASKS];
    const bool in_smem = n_tasks <= SPLIT_SMEM_TASKS;
    if (in_smem)
        for (int i = threadIdx.x; i < n_tasks; i += blockDim.x) s_begin[i] = tasks[i].group_begin;
    __syncthreads();
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        int lo = 0, hi = n_tasks - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            const int64_t b = in_smem ? s_begin[mid] : tasks[mid].group_begin;
            if (b <= t) lo = mid; else hi = mid - 1;
        }
        const xrh_split_task& T = tasks[lo];
        split_group<KIND>(T.src, T.K, T.ld, T.Kp, T.hi, T.lo, t - T.group_begin);
    }
}

PFN_cuTensorMapEncodeTiled_v12000 get_encode() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        cudaDriverEntryPointQueryResult q;
        void* p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

}  // namespace

extern "C" int xrh_tc_chunk_elems(int precision) {
    return precision == XRH_BF16X3 ? 64 : (precision == XRH_TF32X3 ? 32 : 0);
}

extern "C" int xrh_split_operand(int precision, const double* src_dev, int64_t rows, int64_t K, int64_t ld,
                                 int64_t Kp, void* hi_dev, void* lo_dev, void* stream) {
    const int kch = xrh_tc_chunk_elems(precision);
    if (!kch) return XRH_ERR_UNSUPPORTED;
    if (rows < 0 || K < 0 || ld < K || Kp < K || Kp % kch) return XRH_ERR_ARG;
    if (rows == 0 || Kp == 0) return XRH_OK;
    if (!src_dev || !hi_dev || !lo_dev) return XRH_ERR_ARG;
    // the hi / lo arrays are [rows, Kp] with Kp a multiple of 32 elements: 16-byte row starts
    if ((reinterpret_cast<uintptr_t>(hi_dev) & 15) || (reinterpret_cast<uintptr_t>(lo_dev) & 15)) return XRH_ERR_ARG;
    const int64_t total = rows * (Kp / 4);
    const int64_t blocks64 = (total + 255) / 256;
    const unsigned blocks = (unsigned)(blocks64 < 152 * 64 ? blocks64 : 152 * 64);
    if (precision == XRH_BF16X3)
        split_kernel<0><<<blocks, 256, 0, (cudaStream_t)stream>>>(src_dev, rows, K, ld, Kp, hi_dev, lo_dev);
    else
        split_kernel<1><<<blocks, 256, 0, (cudaStream_t)stream>>>(src_dev, rows, K, ld, Kp, hi_dev, lo_dev);
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}

extern "C" int xrh_split_grouped(int precision, const xrh_split_task* tasks_dev, int n_tasks, int64_t total_groups,
                                 void* stream) {
    if (!xrh_tc_chunk_elems(precision)) return XRH_ERR_UNSUPPORTED;
    if (n_tasks < 0 || total_groups < 0) return XRH_ERR_ARG;
    if (n_tasks == 0 || total_groups == 0) return XRH_OK;
    if (!tasks_dev) return XRH_ERR_ARG;
    const int64_t blocks64 = (total_groups + 255) / 256;
    const unsigned blocks = (unsigned)(blocks64 < 152 * 32 ? blocks64 : 152 * 32);
    if (precision == XRH_BF16X3)
        split_grouped_kernel<0><<<blocks, 256, 0, (cudaStream_t)stream>>>(tasks_dev, n_tasks, total_groups);
    else
        split_grouped_kernel<1><<<blocks, 256, 0, (cudaStream_t)stream>>>(tasks_dev, n_tasks, total_groups);
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}

extern "C" int xrh_tc_encode_map(int precision, const void* base_dev, int64_t rows, int64_t Kp, int box_rows,
                                 void* map_out_host) {
    const int kch = xrh_tc_chunk_elems(precision);
    if (!kch) return XRH_ERR_UNSUPPORTED;
    if (!base_dev || !map_out_host || rows <= 0 || Kp <= 0 || Kp % kch) return XRH_ERR_ARG;
    if (box_rows != 32 && box_rows != 64 && box_rows != 128) return XRH_ERR_ARG;
    if ((reinterpret_cast<uintptr_t>(base_dev) & 15) != 0) return XRH_ERR_ARG;
    PFN_cuTensorMapEncodeTiled_v12000 enc = get_encode();
    if (!enc) return XRH_ERR_UNSUPPORTED;
    const int esz = precision == XRH_BF16X3 ? 2 : 4;
    const cuuint64_t dims[2] = {(cuuint64_t)Kp, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)Kp * esz};
    const cuuint32_t box[2] = {(cuuint32_t)kch, (cuuint32_t)box_rows};
    const cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(reinterpret_cast<CUtensorMap*>(map_out_host),
                     precision == XRH_BF16X3 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2,
                     const_cast<void*>(base_dev), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                     CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? XRH_OK : XRH_ERR_ARG;
}

extern "C" int xrh_gemm_tc_grouped(int precision, const xrh_tc_task* tasks_dev, int n_tasks, int64_t total_tiles,
                                   const xrh_tc_segment* segs_dev, const void* maps_dev, int32_t* status_dev,
                                   void* stream) {
    if (!xrh_tc_chunk_elems(precision)) return XRH_ERR_UNSUPPORTED;
    if (n_tasks < 0 || total_tiles < 0) return XRH_ERR_ARG;
    if (n_tasks == 0 || total_tiles == 0) return XRH_OK;
    if (!tasks_dev || !segs_dev || !maps_dev || !status_dev) return XRH_ERR_ARG;
    if ((reinterpret_cast<uintptr_t>(maps_dev) & 63) != 0) return XRH_ERR_ARG;
    int dev = 0, n_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
    const size_t smem = (size_t)TC_STAGES * TC_STAGE_BYTES + 1024;
    const int64_t grid64 = total_tiles < n_sm ? total_tiles : n_sm;
    const unsigned grid = (unsigned)(grid64 > 0 ? grid64 : 1);
    if (precision == XRH_BF16X3) {
        cudaFuncSetAttribute(gemm_tc_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        gemm_tc_kernel<0><<<grid, TC_THREADS, smem, (cudaStream_t)stream>>>(
            tasks_dev, n_tasks, total_tiles, segs_dev, reinterpret_cast<const CUtensorMap*>(maps_dev), status_dev);
    } else {
        cudaFuncSetAttribute(gemm_tc_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        gemm_tc_kernel<1><<<grid, TC_THREADS, smem, (cudaStream_t)stream>>>(
            tasks_dev, n_tasks, total_tiles, segs_dev, reinterpret_cast<const CUtensorMap*>(maps_dev), status_dev);
    }
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}
