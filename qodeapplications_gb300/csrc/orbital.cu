// Integral derivatives of the orbital gradient, assembled element-wise from the adjoint's
// pieces without forming dE/dV (the reference differentiates the energy w.r.t. the integrals in
// StateSpaceOptimizer/orb_grads.py and rotates them; here the derivative tensors feed the
// contraction dE/dkappa = 4 V_(1) Gbar_(1)^T + one-body terms).
//
// dE/dV of the dimer is a sum of blocks of the supersystem spin-orbital tensor, each a fixed
// permutation of one piece of the reverse pass (fragment 0 owns spin orbitals [0, N0),
// fragment 1 [N0, N0 + N1); m is a fragment, o the other, local indices a b c d):
//   (0,1,0,1):  4 gw[b, d, a, c]                gw: (N1, N1, N0, N0)
//   (m,m,m,o): -2 cca_m[d, a, b, c]             cca_m: (No, Nm, Nm, Nm)
//   (m,o,m,m):  2 caa_m[b, a, d, c]             caa_m: (No, Nm, Nm, Nm)
//   (m,m,o,o):    cc_m[d, c, a, b]              cc_m: (No, No, Nm, Nm)
//   (m,m,m,m):    Gamma_m antisymmetrised in (a,b) and (c,d)   Gamma_m: (Nm^4), FP64 + FP32 part
// and every (p,q,r,s) lies in at most one block.  xrh_orbital_terms writes
//   B[p,q,r,s] = Ga[p,q,r,s] + Ga[r,s,p,q],  Ga = dV - dV^(qprs) - dV^(pqsr) + dV^(qpsr)
// (8 Gbar of the symmetric part of dV) and dT (t x t):  dT[a in m, b in o] = h1_m[b, a]
// (h1_m: (No, Nm)), dT[a in m, b in m] = mono1_m[a, b].  The one-body derivative of every
// fragment potential U_k equals dT.
#include "xrh_common.cuh"

namespace {

template <typename T>
__device__ __forceinline__ T ld_as(const double* p) {
    if constexpr (sizeof(T) == 4) return xrh_f64_to_f32(*p);
    else return *p;
}

// fragment m's piece of a two-entry pointer array (selects, no dynamic indexing of the
// kernel parameter)
template <typename P>
__device__ __forceinline__ P pick(const P (&arr)[2], int m) {
    return m ? arr[1] : arr[0];
}

template <typename T>
__device__ __forceinline__ T gamma_at(const xrh_orbital_inputs& in, int m, int Nm, int a, int b, int c, int d) {
    const int64_t i = (((int64_t)a * Nm + b) * Nm + c) * Nm + d;
    T v = ld_as<T>(pick(in.gamma64, m) + i);
    const float* g32 = pick(in.gamma32, m);
    if (g32) v += (T)g32[i];
    return v;
}

template <typename T>
__device__ T dv_at(const xrh_orbital_inputs& in, int p, int q, int r, int s) {
    const int N0 = in.N0, N1 = in.N1;
    const int fp = p >= N0, fq = q >= N0, fr = r >= N0, fs = s >= N0;
    const int a = p - (fp ? N0 : 0), b = q - (fq ? N0 : 0), c = r - (fr ? N0 : 0), d = s - (fs ? N0 : 0);
    if (fp == 0 && fq == 1 && fr == 0 && fs == 1)
        return (T)4 * ld_as<T>(in.gw + (((int64_t)b * N1 + d) * N0 + a) * N0 + c);
    const int m = fp, o = 1 - fp;
    const int Nm = m ? N1 : N0, No = m ? N0 : N1;
    if (fq == m && fr == m && fs == o)
        return (T)(-2) * ld_as<T>(pick(in.cca, m) + (((int64_t)d * Nm + a) * Nm + b) * Nm + c);
    if (fq == o && fr == m && fs == m)
        return (T)2 * ld_as<T>(pick(in.caa, m) + (((int64_t)b * Nm + a) * Nm + d) * Nm + c);
    if (fq == m && fr == o && fs == o)
        return ld_as<T>(pick(in.cc, m) + (((int64_t)d * No + c) * Nm + a) * Nm + b);
    if (fq == m && fr == m && fs == m)
        return gamma_at<T>(in, m, Nm, a, b, c, d) - gamma_at<T>(in, m, Nm, b, a, c, d) -
               gamma_at<T>(in, m, Nm, a, b, d, c) + gamma_at<T>(in, m, Nm, b, a, d, c);
    return (T)0;
}

template <typename T>
__device__ __forceinline__ T ga_at(const xrh_orbital_inputs& in, int p, int q, int r, int s) {
    return dv_at<T>(in, p, q, r, s) - dv_at<T>(in, q, p, r, s) - dv_at<T>(in, p, q, s, r) + dv_at<T>(in, q, p, s, r);
}

// (i, j) with i <= j from a triangular index k = j (j + 1) / 2 + i (float estimate, fixed up)
__device__ __forceinline__ void tri_decode(int64_t k, int64_t& i, int64_t& j) {
    j = (int64_t)((sqrt(8.0 * (double)k + 1.0) - 1.0) * 0.5);
    while (j * (j + 1) / 2 > k) --j;
    while ((j + 1) * (j + 2) / 2 <= k) ++j;
    i = k - j * (j + 1) / 2;
}

// B has the symmetry B[pqrs] = -B[qprs] = -B[pqsr] = B[rspq] (and B = 0 for p = q or r = s, set
// by the caller's zero fill): one thread per canonical element p < q, r < s, (pq) <= (rs)
// evaluates it once and writes its up to eight images.
template <typename T>
__global__ void __launch_bounds__(256) orbital_B_kernel(xrh_orbital_inputs in, T* __restrict__ B) {
    const int t = in.N0 + in.N1;
    const int64_t np = (int64_t)t * (t - 1) / 2;                 // pairs p < q
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= np * (np + 1) / 2) return;
    int64_t P, R;
    tri_decode(k, P, R);                                          // pair indices P <= R
    int64_t p, q, r, s;
    tri_decode(P, p, q);                                          // p <= q - 1 of pair P
    tri_decode(R, r, s);
    q += 1;                                                       // pair P = (p, q) with p < q
    s += 1;
    const T v = ga_at<T>(in, (int)p, (int)q, (int)r, (int)s) + ga_at<T>(in, (int)r, (int)s, (int)p, (int)q);
    const int64_t t2 = (int64_t)t * t;
    const int64_t pq = p * t + q, qp = q * t + p, rs = r * t + s, sr = s * t + r;
    B[pq * t2 + rs] = v;
    B[qp * t2 + rs] = -v;
    B[pq * t2 + sr] = -v;
    B[qp * t2 + sr] = v;
    if (P != R) {
        B[rs * t2 + pq] = v;
        B[sr * t2 + pq] = -v;
        B[rs * t2 + qp] = -v;
        B[sr * t2 + qp] = v;
    }
}

__global__ void __launch_bounds__(256) orbital_dT_kernel(xrh_orbital_inputs in, double* __restrict__ dT) {
    const int N0 = in.N0, N1 = in.N1, t = N0 + N1;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= t * t) return;
    const int p = e / t, q = e - (e / t) * t;
    const int fp = p >= N0, fq = q >= N0;
    const int a = p - (fp ? N0 : 0), b = q - (fq ? N0 : 0);
    const int Nm = fp ? N1 : N0;
    dT[e] = fp == fq ? pick(in.mono1, fp)[(int64_t)a * Nm + b] : pick(in.h1, fp)[(int64_t)b * Nm + a];
}

}  // namespace

extern "C" int xrh_orbital_terms(const xrh_orbital_inputs* in_host, double* dT_dev, void* B_dev, int precision,
                                 void* stream) {
    if (!in_host || !dT_dev || !B_dev) return XRH_ERR_ARG;
    const xrh_orbital_inputs& in = *in_host;
    if (in.N0 <= 0 || in.N1 <= 0 || in.N0 + in.N1 > 64) return XRH_ERR_ARG;
    if (!in.gw) return XRH_ERR_ARG;
    for (int m = 0; m < 2; ++m)
        if (!in.h1[m] || !in.cca[m] || !in.caa[m] || !in.cc[m] || !in.mono1[m] || !in.gamma64[m]) return XRH_ERR_ARG;
    const int t = in.N0 + in.N1;
    const int64_t t4 = (int64_t)t * t * t * t;
    cudaStream_t s = (cudaStream_t)stream;
    orbital_dT_kernel<<<(unsigned)((t * t + 255) / 256), 256, 0, s>>>(in, dT_dev);
    XRH_CHECK_LAUNCH();
    const int64_t np = (int64_t)t * (t - 1) / 2;
    const unsigned blocks = (unsigned)((np * (np + 1) / 2 + 255) / 256);
    if (precision == XRH_FP32) {
        if (cudaMemsetAsync(B_dev, 0, sizeof(float) * (size_t)t4, s) != cudaSuccess) return XRH_ERR_CUDA;
        orbital_B_kernel<float><<<blocks, 256, 0, s>>>(in, reinterpret_cast<float*>(B_dev));
    } else if (precision == XRH_FP64) {
        if (cudaMemsetAsync(B_dev, 0, sizeof(double) * (size_t)t4, s) != cudaSuccess) return XRH_ERR_CUDA;
        orbital_B_kernel<double><<<blocks, 256, 0, s>>>(in, reinterpret_cast<double*>(B_dev));
    } else {
        return XRH_ERR_ARG;
    }
    XRH_CHECK_LAUNCH();
    return XRH_OK;
}
