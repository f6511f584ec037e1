// Transition densities through intermediate determinants: the index kernels around the
// tensor-core GEMM  X[(I, ci), (J, ai)] = sum_K Ct[(I, ci), K] At[(J, ai), K].
//
//   xrh_im_scatter   Ct / At (and the [K][(s, idx)] copies the adjoint GEMMs read) from the
//                    state coefficients: one entry per (determinant, index) with its K and sign
//   xrh_im_expand    rho[I][J][f] = sign_f X[(I, ci_f), (J, ai_f)]   (f = full operator index)
//   xrh_im_fold      dX[(I, ci), (J, ai)] = sum over the (at most two) f of (ci, ai) of sign_f drho[I][J][f]
//   xrh_im_gather    dz[x][s] += sum over x's entries of sign dCt[(s, idx), K]   (no atomics)
//
// All of it is index work on FP64 arrays; the entry lists and maps are built once per
// determinant space (qodeapplications_gb300/intermediates.py).
#include "xrh_common.cuh"

namespace {

unsigned grid_for(int64_t total) {
    const int64_t b = (total + 255) / 256;
    return (unsigned)(b < 152 * 32 ? (b > 0 ? b : 1) : 152 * 32);
}

__global__ void im_scatter_kernel(int64_t n_entries, const int32_t* __restrict__ x, const int32_t* __restrict__ idx,
                                  const int32_t* __restrict__ k, const int8_t* __restrict__ sgn,
                                  const double* __restrict__ zT, int n, int64_t nK, int nidx, double* __restrict__ Dt,
                                  double* __restrict__ D) {
    const int64_t total = n_entries * n;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = t / n;
        const int s = (int)(t - e * n);
        double v = __ldg(zT + (int64_t)__ldg(x + e) * n + s);
        if (__ldg(sgn + e) < 0) v = -v;
        const int64_t i = __ldg(idx + e), kk = __ldg(k + e);
        Dt[((int64_t)s * nidx + i) * nK + kk] = v;
        if (D) D[kk * ((int64_t)n * nidx) + (int64_t)s * nidx + i] = v;
    }
}

__global__ void im_expand_kernel(int nb, int nk, int64_t F, const int32_t* __restrict__ ci,
                                 const int32_t* __restrict__ ai, const int8_t* __restrict__ sgn, int ncre, int nann,
                                 const double* __restrict__ X, double* __restrict__ rho) {
    const int64_t total = (int64_t)nb * nk * F;
    const int64_t ldx = (int64_t)nk * nann;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t ij = t / F;
        const int64_t f = t - ij * F;
        const int I = (int)(ij / nk), J = (int)(ij - (int64_t)I * nk);
        const int s = __ldg(sgn + f);
        double v = 0.0;
        if (s) {
            v = __ldg(X + ((int64_t)I * ncre + __ldg(ci + f)) * ldx + (int64_t)J * nann + __ldg(ai + f));
            if (s < 0) v = -v;
        }
        rho[t] = v;
    }
}

__global__ void im_fold_kernel(int nb, int nk, int64_t F, int ncre, int nann, const int32_t* __restrict__ src,
                               const int8_t* __restrict__ sgn, const double* __restrict__ grho,
                               double* __restrict__ gX) {
    // gX[(I, c), (J, a)]: thread order (I, c, J, a) with a fastest
    const int64_t total = (int64_t)nb * ncre * nk * nann;
    const int64_t nca = (int64_t)ncre * nann;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        int64_t r = t;
        const int a = (int)(r % nann); r /= nann;
        const int J = (int)(r % nk); r /= nk;
        const int c = (int)(r % ncre);
        const int I = (int)(r / ncre);
        const int64_t ca = (int64_t)c * nann + a;
        const double* g = grho + ((int64_t)I * nk + J) * F;
        double v = 0.0;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int64_t q = 2 * ca + h;
            const int s = __ldg(sgn + q);
            if (s) v += s > 0 ? g[__ldg(src + q)] : -g[__ldg(src + q)];
        }
        gX[t] = v;
        (void)nca;
    }
}

__global__ void im_gather_kernel(int n_x, const int64_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                                 const int32_t* __restrict__ k, const int8_t* __restrict__ sgn, int n, int64_t nK,
                                 int nidx, const double* __restrict__ gDt, double* __restrict__ gzT) {
    const int64_t total = (int64_t)n_x * n;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int x = (int)(t / n);
        const int s = (int)(t - (int64_t)x * n);
        double acc = 0.0;
        for (int64_t e = __ldg(ptr + x); e < __ldg(ptr + x + 1); ++e) {
            const double v = __ldg(gDt + ((int64_t)s * nidx + __ldg(idx + e)) * nK + __ldg(k + e));
            acc += __ldg(sgn + e) < 0 ? -v : v;
        }
        gzT[t] += acc;
    }
}

}  // namespace

extern "C" int xrh_im_scatter(int64_t n_entries, const int32_t* x_dev, const int32_t* idx_dev, const int32_t* k_dev,
                              const int8_t* sign_dev, const double* zT_dev, int n, int64_t nK, int nidx,
                              double* Dt_dev, double* D_dev, void* stream) {
    if (n_entries < 0 || n <= 0 || nK <= 0 || nidx <= 0) return XRH_ERR_ARG;
    if (n_entries == 0) return XRH_OK;
    if (!x_dev || !idx_dev || !k_dev || !sign_dev || !zT_dev || !Dt_dev) return XRH_ERR_ARG;
    im_scatter_kernel<<<grid_for(n_entries * n), 256, 0, (cudaStream_t)stream>>>(n_entries, x_dev, idx_dev, k_dev,
                                                                                 sign_dev, zT_dev, n, nK, nidx, Dt_dev,
                                                                                 D_dev);
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}

extern "C" int xrh_im_expand(int nb, int nk, int64_t F, const int32_t* ci_dev, const int32_t* ai_dev,
                             const int8_t* sign_dev, int ncre, int nann, const double* X_dev, double* rho_dev,
                             void* stream) {
    if (nb <= 0 || nk <= 0 || F <= 0 || ncre <= 0 || nann <= 0) return XRH_ERR_ARG;
    if (!ci_dev || !ai_dev || !sign_dev || !X_dev || !rho_dev) return XRH_ERR_ARG;
    im_expand_kernel<<<grid_for((int64_t)nb * nk * F), 256, 0, (cudaStream_t)stream>>>(nb, nk, F, ci_dev, ai_dev,
                                                                                        sign_dev, ncre, nann, X_dev,
                                                                                        rho_dev);
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}

extern "C" int xrh_im_fold(int nb, int nk, int64_t F, int ncre, int nann, const int32_t* src_dev,
                           const int8_t* sign_dev, const double* grho_dev, double* gX_dev, void* stream) {
    if (nb <= 0 || nk <= 0 || F <= 0 || ncre <= 0 || nann <= 0) return XRH_ERR_ARG;
    if (!src_dev || !sign_dev || !grho_dev || !gX_dev) return XRH_ERR_ARG;
    im_fold_kernel<<<grid_for((int64_t)nb * ncre * nk * nann), 256, 0, (cudaStream_t)stream>>>(
        nb, nk, F, ncre, nann, src_dev, sign_dev, grho_dev, gX_dev);
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}

extern "C" int xrh_im_gather(int n_x, const int64_t* ptr_dev, const int32_t* idx_dev, const int32_t* k_dev,
                             const int8_t* sign_dev, int n, int64_t nK, int nidx, const double* gDt_dev,
                             double* gzT_dev, void* stream) {
    if (n_x < 0 || n <= 0 || nK <= 0 || nidx <= 0) return XRH_ERR_ARG;
    if (n_x == 0) return XRH_OK;
    if (!ptr_dev || !idx_dev || !k_dev || !sign_dev || !gDt_dev || !gzT_dev) return XRH_ERR_ARG;
    im_gather_kernel<<<grid_for((int64_t)n_x * n), 256, 0, (cudaStream_t)stream>>>(n_x, ptr_dev, idx_dev, k_dev,
                                                                                   sign_dev, n, nK, nidx, gDt_dev,
                                                                                   gzT_dev);
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}
