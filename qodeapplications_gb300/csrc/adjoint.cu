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

// FP32 variant for the split-precision paths.  Per chunk of 64 couplings of one operator
// index, the ket and bra results are two small GEMMs against G[idx]:
//   U[c, J] = sum_I (s_c zb[I, P_c]) G[I, J],   W[c, I] = s_c sum_J G[I, J] zk[J, Q_c]
// computed in 4 couplings x 4 outputs register tiles from shared memory laid out so that every
// load is a 16-byte vector (G in both orientations, staged z columns transposed), and reduced
// into FP32 gradient rows with 16-byte vector atomics.
__device__ __forceinline__ void atomic_add4(float* dst, const float (&v)[4], int valid) {
    if (valid == 4 && (reinterpret_cast<uintptr_t>(dst) & 15) == 0) {
        xrh_red_add_v4(dst, v[0], v[1], v[2], v[3]);
    } else {
        for (int k = 0; k < valid; ++k) xrh_red_add(dst + k, v[k]);
    }
}

// Couplings per stage of the FP32 adjoint: the work items of a stage, (C/4) x (n_k/4 + n_b/4)
// register tiles, about one per thread (C a multiple of 4, 4..128), so a stage keeps every
// thread busy for any state count, and the staging buffers hold about 4 x 256 x 4 floats.
__host__ __device__ __forceinline__ int adj_chunk(int nbp, int nkp) {
    int c = 4 * (kAdjThreads / ((nbp >> 2) + (nkp >> 2)));
    return c < 4 ? 4 : (c > 128 ? 128 : c);
}

// Shared memory (bytes) of the FP32 adjoint for the largest n_b, n_k of a launch: G in both
// orientations plus two stages of gathered rows (at most 2 x 4096 floats, see adj_chunk).
static size_t adj_f32_smem(int max_nb, int max_nk) {
    const int nbp = (max_nb + 3) & ~3, nkp = (max_nk + 3) & ~3;
    size_t stage = 0;
    for (int b = 4; b <= nbp; b += 4)           // the largest C (nbp' + nkp' + 3) over the smaller tasks
        for (int k = 4; k <= nkp; k += 4) {
            const size_t v = (size_t)adj_chunk(b, k) * (b + k + 3);
            stage = v > stage ? v : stage;
        }
    return sizeof(float) * (2 * (size_t)nbp * nkp + 2 * stage);
}

// One CTA per operator index.  G[idx] is staged in shared memory in both orientations; the
// couplings are streamed in stages of C (adj_chunk): the coefficient rows of stage k+1 are
// gathered with cp.async while stage k is multiplied, with ONE barrier per stage (the buffer a
// gather overwrites was read in the stage before that barrier).  The stage's P, Q and signs are
// written to shared memory beside its rows (same double buffer), for the atomics that send a
// work item's results out.
__device__ __forceinline__ void density_adjoint_f32_body(
    int64_t idx, const int64_t* __restrict__ idx_ptr, const int32_t* __restrict__ P, const int32_t* __restrict__ Q,
    const int8_t* __restrict__ sgn, const float* __restrict__ zb32, int nb, const float* __restrict__ zk32, int nk,
    const double* __restrict__ gT, float* __restrict__ gzbT, float* __restrict__ gzkT, unsigned char* smem_raw) {
    const int nbp = (nb + 3) & ~3, nkp = (nk + 3) & ~3;
    const int C = adj_chunk(nbp, nkp);
    float* g = reinterpret_cast<float*>(smem_raw);          // [nbp][nkp]
    float* gt = g + nbp * nkp;                              // [nkp][nbp]
    float* zb_s = gt + nkp * nbp;                           // [2][C][nbp]
    float* zk_s = zb_s + 2 * C * nbp;                       // [2][C][nkp]
    int* sPQ = reinterpret_cast<int*>(zk_s + 2 * C * nkp);  // [2][C][2]: P, Q (-1 past the end)
    float* sS = reinterpret_cast<float*>(sPQ + 4 * C);      // [2][C]: signs
    const int64_t c_begin = idx_ptr[idx], c_end = idx_ptr[idx + 1];
    if (c_begin == c_end) return;
    const double* gi = gT + idx * (int64_t)nb * nk;
    for (int t = threadIdx.x; t < nbp * nkp; t += blockDim.x) {
        const int i = t / nkp, j = t - i * nkp;
        const float v = (i < nb && j < nk) ? (float)gi[i * nk + j] : 0.f;
        g[t] = v;
        gt[j * nbp + i] = v;
    }
    const int n_chunks = (int)((c_end - c_begin + C - 1) / C);
    const int gb = nbp / 4, gk = nkp / 4;
    auto stage = [&](int k, int buf) {
        const int64_t c0 = c_begin + (int64_t)k * C;
        float* zbb = zb_s + buf * C * nbp;
        float* zkb = zk_s + buf * C * nkp;
        for (int c = threadIdx.x; c < C; c += blockDim.x) {    // indices of the stage, for its atomics
            const int64_t cc = c0 + c;
            const bool in = cc < c_end;
            sPQ[(buf * C + c) * 2] = in ? __ldg(P + cc) : -1;
            sPQ[(buf * C + c) * 2 + 1] = in ? __ldg(Q + cc) : -1;
            sS[buf * C + c] = in ? (__ldg(sgn + cc) < 0 ? -1.f : 1.f) : 0.f;
        }
        for (int x = threadIdx.x; x < C * gb; x += blockDim.x) {
            const int c = x / gb, part = x - c * gb;
            const int64_t cc = c0 + c;
            if (cc < c_end) cp_async16(zbb + c * nbp + part * 4, zb32 + (int64_t)__ldg(P + cc) * nbp + part * 4);
            else *reinterpret_cast<float4*>(zbb + c * nbp + part * 4) = make_float4(0.f, 0.f, 0.f, 0.f);
        }
        for (int x = threadIdx.x; x < C * gk; x += blockDim.x) {
            const int c = x / gk, part = x - c * gk;
            const int64_t cc = c0 + c;
            if (cc < c_end) cp_async16(zkb + c * nkp + part * 4, zk32 + (int64_t)__ldg(Q + cc) * nkp + part * 4);
            else *reinterpret_cast<float4*>(zkb + c * nkp + part * 4) = make_float4(0.f, 0.f, 0.f, 0.f);
        }
        cp_async_commit();
    };
    const int tj = nkp / 4, ti = nbp / 4;
    const int ket_tiles = (C / 4) * tj, bra_tiles = (C / 4) * ti;
    stage(0, 0);
    for (int k = 0; k < n_chunks; ++k) {
        const int buf = k & 1;
        cp_async_wait<0>();                          // this thread's gathers of stage k landed
        __syncthreads();                             // everyone's landed; stage k-1 fully consumed
        if (k + 1 < n_chunks) stage(k + 1, buf ^ 1); // in flight while stage k is multiplied
        const float* zbb = zb_s + buf * C * nbp;
        const float* zkb = zk_s + buf * C * nkp;
        for (int w = threadIdx.x; w < ket_tiles + bra_tiles; w += blockDim.x) {
            float acc[4][4] = {};
            const bool ket = w < ket_tiles;
            const int wl = ket ? w : w - ket_tiles;
            const int tw = ket ? tj : ti;
            const int c4 = (wl / tw) * 4, o4 = (wl % tw) * 4;
            // ket: U[c, J] = sum_I zb[c, I] G[I, J]   bra: W[c, I] = sum_J zk[c, J] G^T[J, I]
            const float* A = ket ? zbb : zkb;
            const float* B = ket ? g : gt;
            const int la = ket ? nbp : nkp, lb = ket ? nkp : nbp;
            for (int K0 = 0; K0 < la; K0 += 4) {
                float4 a[4], b[4];
#pragma unroll
                for (int x = 0; x < 4; ++x) a[x] = *reinterpret_cast<const float4*>(A + (c4 + x) * la + K0);
#pragma unroll
                for (int i = 0; i < 4; ++i) b[i] = *reinterpret_cast<const float4*>(B + (K0 + i) * lb + o4);
#pragma unroll
                for (int x = 0; x < 4; ++x) {
                    const float av[4] = {a[x].x, a[x].y, a[x].z, a[x].w};
#pragma unroll
                    for (int i = 0; i < 4; ++i) {
                        acc[x][0] = fmaf(av[i], b[i].x, acc[x][0]);
                        acc[x][1] = fmaf(av[i], b[i].y, acc[x][1]);
                        acc[x][2] = fmaf(av[i], b[i].z, acc[x][2]);
                        acc[x][3] = fmaf(av[i], b[i].w, acc[x][3]);
                    }
                }
            }
            const int n_out = ket ? nk : nb;
            const int valid = n_out - o4 < 4 ? n_out - o4 : 4;
            for (int x = 0; x < 4; ++x) {
                const int row = sPQ[(buf * C + c4 + x) * 2 + (ket ? 1 : 0)];
                if (row < 0) break;
                const float sc = sS[buf * C + c4 + x];
#pragma unroll
                for (int y = 0; y < 4; ++y) acc[x][y] *= sc;
                float* dst = ket ? gzkT + (int64_t)row * nk + o4 : gzbT + (int64_t)row * nb + o4;
                atomic_add4(dst, acc[x], valid);
            }
        }
    }
}

__global__ void __launch_bounds__(kAdjThreads, 3) density_adjoint_f32_kernel(
    const int64_t* __restrict__ idx_ptr, const int32_t* __restrict__ P, const int32_t* __restrict__ Q,
    const int8_t* __restrict__ sgn, const float* __restrict__ zb32, int nb, const float* __restrict__ zk32, int nk,
    const double* __restrict__ gT, float* __restrict__ gzbT, float* __restrict__ gzkT) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    density_adjoint_f32_body(blockIdx.x, idx_ptr, P, Q, sgn, zb32, nb, zk32, nk, gT, gzbT, gzkT, smem_raw);
}

// Every block of a task table in one launch (one CTA per operator index).
__global__ void __launch_bounds__(kAdjThreads, 3) density_adjoint_f32_grouped_kernel(
    const xrh_dens_adj_task* __restrict__ tasks, int n_tasks) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    int lo = 0, hi = n_tasks - 1;
    const int64_t cta = blockIdx.x;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (tasks[mid].cta_begin <= cta) lo = mid; else hi = mid - 1;
    }
    const xrh_dens_adj_task& T = tasks[lo];
    density_adjoint_f32_body(cta - T.cta_begin, T.idx_ptr, T.P, T.Q, T.sign, T.zb32, T.nb, T.zk32, T.nk, T.gT, T.gzb,
                             T.gzk, smem_raw);
}

constexpr int kWThreads = 128;

template <typename T>
__global__ void __launch_bounds__(kWThreads) ccaa_weighted_kernel(
    int N, const uint64_t* __restrict__ bra, int n_bra, const uint64_t* __restrict__ ket_sorted,
    const int32_t* __restrict__ ket_pos, int n_ket, const int32_t* __restrict__ rank_table, int64_t table_size,
    const int64_t* __restrict__ binom, const double* __restrict__ zbT, const double* __restrict__ YT,
    int n, T* __restrict__ Gamma) {
    __shared__ int s_occ[64];
    __shared__ int s_free[64];
    __shared__ int s_ne, s_nfree;
    __shared__ T s_zb[256];
    const int Pb = blockIdx.x;
    const uint64_t m = bra[Pb];
    if (threadIdx.x == 0) {
        int k = 0;
        for (int o = 0; o < N; ++o)
            if ((m >> o) & 1ull) s_occ[k++] = o;
        s_ne = k;
    }
    for (int t = threadIdx.x; t < n; t += blockDim.x) s_zb[t] = (T)zbT[(int64_t)Pb * n + t];
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
                int Qp;
                if (rank_table) {
                    Qp = xrh_rank_lookup(rank_table, table_size, binom, m2);
                } else {
                    const int hit = xrh_lookup(ket_sorted, n_ket, m2);
                    Qp = hit < 0 ? -1 : __ldg(ket_pos + hit);
                }
                if (Qp < 0) continue;
                T w = 0;
                for (int I = 0; I < n; ++I) w = fma(s_zb[I], (T)YT[(int64_t)Qp * n + I], w);
                if (w == (T)0) continue;
                // <P| c+_p c+_q a_s a_r |Q>  (p<q, r<s) = sign of <Q| c+_r c+_s a_q a_p |P>
                atomicAdd(Gamma + (((int64_t)p * N + q) * N + r) * N + s, s2 ? -w : w);
            }
        }
    }
}


// ---- small blocks: lane per coupling ------------------------------------------------------
// For blocks of few states (n_b, n_k <= 4 * MAXQ) a warp owns one unit (an operator index, or a
// range of its couplings, as in the forward units kernel) and stages G = dE/drho[idx]
// (n_b x n_k, FP32, rows padded with zeros to 4 * MAXQ) in its shared memory; lane l takes
// couplings c = c_lo + l, c_lo + l + 32, ...: it gathers the padded FP32 rows zb[P_c] and
// zk[Q_c] (padding entries are zero), reads G by broadcast, forms
//   U[J] = s_c sum_I zb[P_c, I] G[I, J]   and   W[I] = s_c sum_J G[I, J] zk[Q_c, J]
// and adds them to gzk[Q_c] and gzb[P_c] with vector atomics (float4 when 16-byte aligned,
// else float2 when 8-byte aligned, else scalar).
template <int MP>
__device__ __forceinline__ void atomic_add_row(float* dst, const float (&v)[MP], int n) {
    const uintptr_t a = reinterpret_cast<uintptr_t>(dst);
    const bool a16 = (a & 15) == 0, a8 = (a & 7) == 0;
#pragma unroll
    for (int k = 0; k < MP; k += 4) {
        if (k >= n) break;
        if (a16 && k + 3 < n) {
            xrh_red_add_v4(dst + k, v[k], v[k + 1], v[k + 2], v[k + 3]);
            continue;
        }
#pragma unroll
        for (int h = 0; h < 4; h += 2) {
            const int kk = k + h;
            if (kk >= n) break;
            if (kk + 1 < n && a8) {
                xrh_red_add_v2(dst + kk, v[kk], v[kk + 1]);
            } else {
                xrh_red_add(dst + kk, v[kk]);
                if (kk + 1 < n) xrh_red_add(dst + kk + 1, v[kk + 1]);
            }
        }
    }
}

template <int MAXQ>
__global__ void __launch_bounds__(256) density_adjoint_units_kernel(const xrh_dens_adj_task* __restrict__ tasks,
                                                                   const xrh_dens_unit* __restrict__ units,
                                                                   int64_t n_units, int g_layout) {
    constexpr int MP = 4 * MAXQ;
    __shared__ __align__(16) float gsm[8][MP][MP];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t u = (int64_t)blockIdx.x * 8 + warp;
    if (u >= n_units) return;
    const xrh_dens_unit U = units[u];
    const xrh_dens_adj_task& T = tasks[U.task];
    const int nb = T.nb, nk = T.nk;
    if (nb > MP || nk > MP) return;                  // the host never builds such a unit
    const int nbp = (nb + 3) & ~3, nkp = (nk + 3) & ~3;
    float (*g)[MP] = gsm[warp];
    for (int e = lane; e < MP * MP; e += 32) {
        const int I = e / MP, J = e - I * MP;
        float v = 0.f;
        if (I < nb && J < nk)
            v = xrh_f64_to_f32(g_layout == 0 ? T.gT[((int64_t)U.idx * nb + I) * nk + J]
                                             : T.gT[((int64_t)I * nk + J) * T.K + U.idx]);
        g[I][J] = v;
    }
    __syncwarp();
    const int64_t base = T.idx_ptr[U.idx];
    const int64_t c_lo = base + U.c_lo, c_hi = base + U.c_hi;
    for (int64_t c = c_lo + lane; c < c_hi; c += 32) {
        const int p = T.P[c], q = T.Q[c];
        const float s = T.sign[c] < 0 ? -1.f : 1.f;
        float zb[MP], zk[MP];
        const float4* zbr = reinterpret_cast<const float4*>(T.zb32 + (int64_t)p * nbp);
        const float4* zkr = reinterpret_cast<const float4*>(T.zk32 + (int64_t)q * nkp);
#pragma unroll
        for (int x = 0; x < MAXQ; ++x) {
            const float4 a = 4 * x < nbp ? __ldg(zbr + x) : make_float4(0.f, 0.f, 0.f, 0.f);
            const float4 b = 4 * x < nkp ? __ldg(zkr + x) : make_float4(0.f, 0.f, 0.f, 0.f);
            zb[4 * x] = a.x; zb[4 * x + 1] = a.y; zb[4 * x + 2] = a.z; zb[4 * x + 3] = a.w;
            zk[4 * x] = b.x; zk[4 * x + 1] = b.y; zk[4 * x + 2] = b.z; zk[4 * x + 3] = b.w;
        }
        float Uj[MP], Wi[MP];
#pragma unroll
        for (int k = 0; k < MP; ++k) { Uj[k] = 0.f; Wi[k] = 0.f; }
#pragma unroll
        for (int I = 0; I < MP; ++I) {
            if (I >= nbp) break;
#pragma unroll
            for (int x = 0; x < MAXQ; ++x) {
                if (4 * x >= nkp) break;
                const float4 gv = *reinterpret_cast<const float4*>(&g[I][4 * x]);
                Uj[4 * x] = fmaf(zb[I], gv.x, Uj[4 * x]);
                Uj[4 * x + 1] = fmaf(zb[I], gv.y, Uj[4 * x + 1]);
                Uj[4 * x + 2] = fmaf(zb[I], gv.z, Uj[4 * x + 2]);
                Uj[4 * x + 3] = fmaf(zb[I], gv.w, Uj[4 * x + 3]);
                float w = Wi[I];
                w = fmaf(gv.x, zk[4 * x], w);
                w = fmaf(gv.y, zk[4 * x + 1], w);
                w = fmaf(gv.z, zk[4 * x + 2], w);
                w = fmaf(gv.w, zk[4 * x + 3], w);
                Wi[I] = w;
            }
        }
#pragma unroll
        for (int k = 0; k < MP; ++k) { Uj[k] *= s; Wi[k] *= s; }
        atomic_add_row(T.gzk + (int64_t)q * nk, Uj, nk);
        atomic_add_row(T.gzb + (int64_t)p * nb, Wi, nb);
    }
}
}  // namespace

extern "C" int xrh_density_adjoint_f32_grouped(const xrh_dens_adj_task* tasks_dev, int n_tasks, int64_t total_ctas,
                                               int max_nb, int max_nk, void* stream) {
    if (n_tasks < 0 || total_ctas < 0 || max_nb <= 0 || max_nk <= 0) return XRH_ERR_ARG;
    if (n_tasks == 0 || total_ctas == 0) return XRH_OK;
    if (!tasks_dev) return XRH_ERR_ARG;
    if (total_ctas > 0x7fffffffLL) return XRH_ERR_CAPACITY;
    if (max_nb > 1024 || max_nk > 1024) return XRH_ERR_CAPACITY;
    const size_t smem = adj_f32_smem(max_nb, max_nk);
    if (smem > 200 * 1024) return XRH_ERR_CAPACITY;
    if (smem > 48 * 1024)
        cudaFuncSetAttribute(density_adjoint_f32_grouped_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
    density_adjoint_f32_grouped_kernel<<<(unsigned)total_ctas, kAdjThreads, smem, (cudaStream_t)stream>>>(tasks_dev,
                                                                                                         n_tasks);
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}

extern "C" int xrh_density_adjoint_f32_units(const xrh_dens_adj_task* tasks_dev, int n_tasks,
                                             const xrh_dens_unit* units_dev, int64_t n_units, int max_n,
                                             int g_layout, void* stream) {
    if (n_tasks < 0 || n_units < 0 || max_n <= 0 || (g_layout != 0 && g_layout != 1)) return XRH_ERR_ARG;
    if (n_tasks == 0 || n_units == 0) return XRH_OK;
    if (!tasks_dev || !units_dev) return XRH_ERR_ARG;
    const int64_t ctas = (n_units + 7) / 8;
    if (ctas > 0x7fffffffLL) return XRH_ERR_CAPACITY;
    cudaStream_t s = (cudaStream_t)stream;
    if (max_n <= 8)
        density_adjoint_units_kernel<2><<<(unsigned)ctas, 256, 0, s>>>(tasks_dev, units_dev, n_units, g_layout);
    else if (max_n <= 12)
        density_adjoint_units_kernel<3><<<(unsigned)ctas, 256, 0, s>>>(tasks_dev, units_dev, n_units, g_layout);
    else if (max_n <= 16)
        density_adjoint_units_kernel<4><<<(unsigned)ctas, 256, 0, s>>>(tasks_dev, units_dev, n_units, g_layout);
    else
        return XRH_ERR_CAPACITY;
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}

extern "C" int xrh_density_adjoint(int precision, int64_t K, const int64_t* idx_ptr_dev, const int32_t* P_dev,
                                   const int32_t* Q_dev, const int8_t* sign_dev, const void* zbT_dev, int n_b,
                                   const void* zkT_dev, int n_k, const double* gT_dev, void* gzbT_dev,
                                   void* gzkT_dev, void* stream) {
    if (K <= 0 || n_b <= 0 || n_k <= 0 || !idx_ptr_dev || !zbT_dev || !zkT_dev || !gT_dev || !gzbT_dev || !gzkT_dev)
        return XRH_ERR_ARG;
    if (K > 0x7fffffffLL) return XRH_ERR_CAPACITY;
    const size_t esz = (precision == XRH_FP32) ? sizeof(float) : sizeof(double);
    const size_t smem = esz * ((size_t)n_b * n_k + (size_t)kAdjChunk * (n_b + n_k));
    if (smem > 200 * 1024) return XRH_ERR_CAPACITY;
    if (precision == XRH_FP64) {
        cudaFuncSetAttribute(density_adjoint_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        density_adjoint_kernel<double><<<(unsigned)K, kAdjThreads, smem, (cudaStream_t)stream>>>(
            idx_ptr_dev, P_dev, Q_dev, sign_dev, reinterpret_cast<const double*>(zbT_dev), n_b,
            reinterpret_cast<const double*>(zkT_dev), n_k, gT_dev, reinterpret_cast<double*>(gzbT_dev),
            reinterpret_cast<double*>(gzkT_dev));
    } else if (precision == XRH_FP32) {
        if (n_b > 1024 || n_k > 1024) return XRH_ERR_CAPACITY;
        const size_t smem32 = adj_f32_smem(n_b, n_k);
        if (smem32 > 200 * 1024) return XRH_ERR_CAPACITY;
        cudaFuncSetAttribute(density_adjoint_f32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem32);
        if ((reinterpret_cast<uintptr_t>(zbT_dev) & 15) || (reinterpret_cast<uintptr_t>(zkT_dev) & 15)) return XRH_ERR_ARG;
        density_adjoint_f32_kernel<<<(unsigned)K, kAdjThreads, smem32, (cudaStream_t)stream>>>(
            idx_ptr_dev, P_dev, Q_dev, sign_dev, reinterpret_cast<const float*>(zbT_dev), n_b,
            reinterpret_cast<const float*>(zkT_dev), n_k, gT_dev, reinterpret_cast<float*>(gzbT_dev),
            reinterpret_cast<float*>(gzkT_dev));
    } else {
        return XRH_ERR_UNSUPPORTED;
    }
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}

extern "C" int xrh_ccaa_weighted(int precision, int n_orbs, const uint64_t* bra_masks_dev, int n_bra_conf,
                                 const uint64_t* ket_sorted_masks_dev, const int32_t* ket_sorted_pos_dev,
                                 int n_ket_conf, const int32_t* rank_table_dev, int64_t table_size,
                                 const int64_t* binom_dev, const double* zbT_dev, const double* YT_dev, int n,
                                 void* Gamma_dev, void* stream) {
    const int N = 2 * n_orbs;
    if (n_orbs < 1 || N > 64 || n < 1 || n > 256 || n_bra_conf < 0 || n_ket_conf < 0) return XRH_ERR_ARG;
    if (n_bra_conf == 0) return XRH_OK;
    if (!bra_masks_dev || !zbT_dev || !YT_dev || !Gamma_dev) return XRH_ERR_ARG;
    if (rank_table_dev && !binom_dev) return XRH_ERR_ARG;
    if (precision == XRH_FP64)
        ccaa_weighted_kernel<double><<<n_bra_conf, kWThreads, 0, (cudaStream_t)stream>>>(
            N, bra_masks_dev, n_bra_conf, ket_sorted_masks_dev, ket_sorted_pos_dev, n_ket_conf, rank_table_dev,
            table_size, binom_dev, zbT_dev, YT_dev, n, reinterpret_cast<double*>(Gamma_dev));
    else if (precision == XRH_FP32)
        ccaa_weighted_kernel<float><<<n_bra_conf, kWThreads, 0, (cudaStream_t)stream>>>(
            N, bra_masks_dev, n_bra_conf, ket_sorted_masks_dev, ket_sorted_pos_dev, n_ket_conf, rank_table_dev,
            table_size, binom_dev, zbT_dev, YT_dev, n, reinterpret_cast<float*>(Gamma_dev));
    else
        return XRH_ERR_UNSUPPORTED;
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}
