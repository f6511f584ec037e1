// Coupling lists <P| op_idx |Q> = +-1 between determinant lists (integer work).
//
// GB300 form of the operator loops of general-XRCC/density_tensors.c:162-556: the reference
// walks every ket configuration and every operator index tuple inside each density kernel,
// re-deriving the same couplings for every op string and every call.  Here the couplings
// of one (op string, bra list, ket list) are enumerated once on the device (one thread per
// ket determinant, depth-first over the operator positions with Pauli pruning) and kept
// resident; every later density build, adjoint and gradient reuses them.
#include "xrh_common.cuh"

namespace {

template <bool FILL>
__global__ void __launch_bounds__(128) couplings_kernel(
    int k, int cbits, int N, uint64_t core, const uint64_t* __restrict__ ket, int n_ket,
    const uint64_t* __restrict__ bra_sorted, const int32_t* __restrict__ bra_pos, int n_bra,
    int64_t* __restrict__ counts, const int64_t* __restrict__ offsets, int32_t* __restrict__ idx_out,
    int32_t* __restrict__ P_out, int32_t* __restrict__ Q_out, int8_t* __restrict__ s_out) {
    const int Q = blockIdx.x * blockDim.x + threadIdx.x;
    if (Q >= n_ket) return;
    uint64_t ms[5];
    int ss[5];
    int o[4];
    int pw[4];
    {
        int p = 1;
        for (int pos = k - 1; pos >= 0; --pos) { pw[pos] = p; p *= N; }
    }
    ms[k] = __ldg(ket + Q);
    ss[k] = 0;
    int64_t cnt = 0;
    int64_t w = FILL ? offsets[Q] : 0;
    int L = k;          // level: positions L-1 .. 0 still to apply
    o[k - 1] = -1;
    while (true) {
        const int pos = L - 1;
        o[pos]++;
        if (o[pos] >= N) {
            L++;
            if (L > k) break;
            continue;
        }
        uint64_t m = ms[L];
        int s = ss[L];
        if (!xrh_apply((cbits >> pos) & 1, o[pos], m, s)) continue;
        if (pos == 0) {
            if ((m & core) != core) continue;
            const int hit = xrh_lookup(bra_sorted, n_bra, m);
            if (hit < 0) continue;
            if (FILL) {
                int id = 0;
                for (int t = 0; t < k; ++t) id += o[t] * pw[t];
                idx_out[w] = id;
                P_out[w] = __ldg(bra_pos + hit);
                Q_out[w] = Q;
                s_out[w] = s ? -1 : 1;
                ++w;
            } else {
                ++cnt;
            }
        } else {
            ms[L - 1] = m;
            ss[L - 1] = s;
            L--;
            o[L - 1] = -1;
        }
    }
    if (!FILL) counts[Q] = cnt;
}

uint64_t core_mask(int n_orbs, int n_core) {
    uint64_t m = 0;
    for (int i = 0; i < n_core; ++i) m |= (1ull << i) | (1ull << (n_orbs + i));
    return m;
}

int check_args(int op_code, int n_orbs, int n_core, int n_ket, int n_bra) {
    const int k = op_code & 15;
    if (k < 1 || k > 4) return XRH_ERR_ARG;
    if (n_orbs < 1 || 2 * n_orbs > 64 || n_core < 0 || n_core > n_orbs) return XRH_ERR_ARG;
    if (n_ket < 0 || n_bra < 0) return XRH_ERR_ARG;
    return XRH_OK;
}

}  // namespace

extern "C" int xrh_couplings_count(int op_code, int n_orbs, int n_core, const uint64_t* ket_masks_dev,
                                   int n_ket, const uint64_t* bra_sorted_masks_dev,
                                   const int32_t* bra_sorted_pos_dev, int n_bra, int64_t* counts_dev,
                                   void* stream) {
    int st = check_args(op_code, n_orbs, n_core, n_ket, n_bra);
    if (st) return st;
    if (n_ket == 0) return XRH_OK;
    if (!ket_masks_dev || !counts_dev || (n_bra && (!bra_sorted_masks_dev || !bra_sorted_pos_dev))) return XRH_ERR_ARG;
    const int k = op_code & 15, cbits = op_code >> 4;
    couplings_kernel<false><<<(n_ket + 127) / 128, 128, 0, (cudaStream_t)stream>>>(
        k, cbits, 2 * n_orbs, core_mask(n_orbs, n_core), ket_masks_dev, n_ket, bra_sorted_masks_dev,
        bra_sorted_pos_dev, n_bra, counts_dev, nullptr, nullptr, nullptr, nullptr, nullptr);
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}

extern "C" int xrh_couplings_fill(int op_code, int n_orbs, int n_core, const uint64_t* ket_masks_dev, int n_ket,
                                  const uint64_t* bra_sorted_masks_dev, const int32_t* bra_sorted_pos_dev,
                                  int n_bra, const int64_t* offsets_dev, int32_t* idx_dev, int32_t* P_dev,
                                  int32_t* Q_dev, int8_t* sign_dev, void* stream) {
    int st = check_args(op_code, n_orbs, n_core, n_ket, n_bra);
    if (st) return st;
    if (n_ket == 0) return XRH_OK;
    if (!ket_masks_dev || !offsets_dev || !idx_dev || !P_dev || !Q_dev || !sign_dev) return XRH_ERR_ARG;
    const int k = op_code & 15, cbits = op_code >> 4;
    couplings_kernel<true><<<(n_ket + 127) / 128, 128, 0, (cudaStream_t)stream>>>(
        k, cbits, 2 * n_orbs, core_mask(n_orbs, n_core), ket_masks_dev, n_ket, bra_sorted_masks_dev,
        bra_sorted_pos_dev, n_bra, nullptr, offsets_dev, idx_dev, P_dev, Q_dev, sign_dev);
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}
