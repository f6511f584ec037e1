/* xrh.h - C ABI of the GB300 (sm_103a) excitonic-Hamiltonian build library, libxrh.so.
 *
 * Plain C types only (pointers, sizes, status codes).  Every pointer named *_dev is a
 * device pointer (CUDA global memory) owned by the caller; the library allocates nothing
 * on these paths.  `stream` is a cudaStream_t passed as void*.  Every call is stream
 * ordered, does not synchronise the host, and returns XRH_OK or an error status.
 *
 * The entry points replace the reference's native kernels and their Python drivers:
 *   general-XRCC/density_tensors.c   (density builder)            -> xrh_couplings_*,
 *                                                                    xrh_density_accumulate
 *   general-XRCC/build_density_tensors.py:122-133 (ccaa folded    -> xrh_sigma2e
 *        with V into one number per state pair)
 *   general-XRCC/H_contractions.c + hermitian-XRCC precontract.py  -> xrh_gemm_grouped
 *        + diagrams/* (all density x integral contractions, batched as grouped GEMMs)
 * The reference binds its C kernels one matrix element at a time through Qode's PyC
 * (general-XRCC/build_H.py:20-29, build_density_tensors.py:23-26); here each call covers
 * whole blocks of elements.  The ctypes binding is qodeapplications_gb300/_lib.py.
 */
#ifndef XRH_H
#define XRH_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define XRH_OK 0
#define XRH_ERR_ARG 1          /* bad size, null pointer or unsupported combination */
#define XRH_ERR_CUDA 2         /* a CUDA launch or API call failed (see xrh_last_cuda_error) */
#define XRH_ERR_UNSUPPORTED 3  /* precision / feature not built for this device */
#define XRH_ERR_TIMEOUT 4      /* a bounded device-side wait gave up (kernel returned early) */
#define XRH_ERR_CAPACITY 5     /* a size exceeds a documented limit */

/* arithmetic of a contraction */
#define XRH_FP64 0       /* IEEE FP64 on CUDA cores (the plain drop-in path) */
#define XRH_FP32 1       /* FP32 products, FP32 partial sums, FP64 final sums */
#define XRH_BF16X3 2     /* tcgen05 kind::f16, operands split hi+lo in BF16, 3 products, FP32 accum */
#define XRH_TF32X3 3     /* tcgen05 kind::tf32, operands split hi+lo in TF32, 3 products, FP32 accum */

int xrh_abi_version(void);
const char* xrh_status_string(int status);
int xrh_last_cuda_error(void);

/* Field-operator strings ("a", "c", "ca", "aa", "cc", "caa", "cca", "ccaa") are encoded
 * as  len | (c_bits << 4)  where bit i of c_bits is set when letter i is 'c'.  Operators
 * act right to left; operator indices are flattened row-major in string order, the
 * layout of general-XRCC/density_tensors.c:272,319,420,480,543. */

/* Coupling lists <P| op_idx |Q> = +-1 between determinant lists (uint64 occupation masks,
 * spin orbital i<n_orbs alpha, n_orbs+i beta; N = 2*n_orbs <= 64).  Results that empty
 * the frozen core (n_core lowest orbitals of each spin) or are not in the bra list are
 * dropped (density_tensors.c:125-134, :49-62).  The bra list is given sorted
 * (bra_sorted_masks) with the original position of each entry (bra_sorted_pos).
 * count: counts_dev[Q] = number of couplings of ket Q.
 * fill:  writes them at offsets_dev[Q] (exclusive scan of the counts), in ascending
 *        idx order per Q: idx (flat operator index), P (bra position), Q, sign (+1/-1). */
int xrh_couplings_count(int op_code, int n_orbs, int n_core,
                        const uint64_t* ket_masks_dev, int n_ket,
                        const uint64_t* bra_sorted_masks_dev, const int32_t* bra_sorted_pos_dev, int n_bra,
                        int64_t* counts_dev, void* stream);
int xrh_couplings_fill(int op_code, int n_orbs, int n_core,
                       const uint64_t* ket_masks_dev, int n_ket,
                       const uint64_t* bra_sorted_masks_dev, const int32_t* bra_sorted_pos_dev, int n_bra,
                       const int64_t* offsets_dev, int32_t* idx_dev, int32_t* P_dev, int32_t* Q_dev,
                       int8_t* sign_dev, void* stream);

/* Transition densities from coupling lists sorted by idx (CSR, idx_ptr_dev has K+1 entries):
 *   rhoT[idx, I, J] = sum_c sign_c * zb[I, P_c] * zk[J, Q_c]
 * (z_contract, density_tensors.c:142-154).  zbT_dev is [n_bra_conf, n_b] (coefficients
 * transposed, one row per determinant), zkT_dev is [n_ket_conf, n_k].  precision is
 * XRH_FP64 or XRH_FP32.  Output rhoT_dev [K, n_b, n_k] is fully overwritten. */
int xrh_density_accumulate(int precision, int64_t K, const int64_t* idx_ptr_dev,
                           const int32_t* P_dev, const int32_t* Q_dev, const int8_t* sign_dev,
                           const double* zbT_dev, int n_b, const double* zkT_dev, int n_k,
                           double* rhoT_dev, void* stream);

/* FP32 variant of xrh_density_accumulate for the split-precision paths: coefficients given
 * pre-converted to FP32 as zb32 [n_bra_conf, round_up(n_b,4)] and zk32 [n_ket_conf,
 * round_up(n_k,4)] (rows padded with zeros, 16-byte aligned); FP32 products and stage sums,
 * running sums as FP32 (hi, lo) pairs.  The couplings of every operator index must come
 * positive signs first (the order FragmentSpace builds): the kernel multiplies each sign range
 * with a uniform sign.  splits > 1 divides the couplings of every operator index over that
 * many CTAs and ADDS to rhoT_dev, which must then be zeroed by the caller.  n_b, n_k <= 1024. */
int xrh_density_accumulate_f32(int64_t K, int splits, const int64_t* idx_ptr_dev, const int32_t* P_dev,
                               const int32_t* Q_dev, const int8_t* sign_dev, const float* zb32_dev, int n_b,
                               const float* zk32_dev, int n_k, double* rhoT_dev, void* stream);

/* Every density block of a fragment in one launch (same product as
 * xrh_density_accumulate_f32 per block).  tasks_dev: n_tasks entries sorted by cta_begin,
 * task t owning CTAs [cta_begin, cta_begin + K * splits); total_ctas = sum of K * splits;
 * max_nb / max_nk bound the tasks' state counts (shared-memory size).  rhoT of a task with
 * splits > 1 must be zeroed by the caller. */
typedef struct {
    const int64_t* idx_ptr;
    const int32_t* P;
    const int32_t* Q;
    const int8_t* sign;
    const float* zb32;
    const float* zk32;
    double* rhoT;
    int64_t K;
    int32_t nb, nk;
    int32_t splits, reserved;
    int64_t cta_begin;
} xrh_dens_task;   /* 88 bytes */
int xrh_density_accumulate_f32_grouped(const xrh_dens_task* tasks_dev, int n_tasks, int64_t total_ctas,
                                       int max_nb, int max_nk, void* stream);

/* Same product for blocks of at most max_n <= 16 states per side, one warp per unit: unit u
 * covers couplings [idx_ptr[idx] + c_lo, idx_ptr[idx] + c_hi) of operator index idx of task
 * `task` (cta_begin and splits of the tasks are not used).  A unit with c_lo = 0 and c_hi =
 * the index's coupling count stores rhoT[idx] (an index with no couplings needs such a unit,
 * it writes zeros); the units of an index split into several ranges ADD atomically, so the
 * rhoT of their tasks must be zeroed by the caller.  zb32 / zk32 rows as for
 * xrh_density_accumulate_f32 (16-byte aligned, padded with zeros). */
typedef struct {
    int32_t task;
    int32_t idx;
    int32_t c_lo, c_hi;
} xrh_dens_unit;   /* 16 bytes */
int xrh_density_accumulate_f32_units(const xrh_dens_task* tasks_dev, int n_tasks,
                                     const xrh_dens_unit* units_dev, int64_t n_units, int max_n,
                                     void* stream);

/* Coefficient staging of the builds in one launch: task t (a charge sector) writes
 * zT[k*n + i] = src[i*K + k] (FP64; skipped when zT is NULL) and zT32[k*npad + i] =
 * fl32(src[i*K + k]) (FP32 round to nearest; skipped when zT32 is NULL; columns n..npad
 * untouched) for k < K, i < n; its rows are [row_begin, row_begin + K) of the launch (tasks
 * sorted by row_begin, total_rows = the last row_begin + K). */
typedef struct {
    const double* src;
    double* zT;
    float* zT32;
    int64_t n, K, npad;
    int64_t row_begin;
} xrh_coeff_task;   /* 56 bytes */
int xrh_coeff_stage(const xrh_coeff_task* tasks_dev, int n_tasks, int64_t total_rows, void* stream);

/* Allocation-free transition densities (this entry point has no counterpart in the
 * reference).  For callers that cannot allocate device memory -- for example code running
 * inside another application's CUDA context whose allocator owns all device memory, or a
 * host program without a device allocator of its own -- this variant needs no scratch from
 * the caller: it uses a fixed 8 MiB array in the library's own device memory
 * (K * n_b * n_k <= 1048576 doubles, else XRH_ERR_CAPACITY) and writes rho_dev directly in
 * the (n_b, n_k, K) layout.  Arguments are those of xrh_density_accumulate.  It calls no
 * cudaMalloc/cudaFree.  The first call on a device looks up that device's address of the
 * array (cudaGetSymbolAddress) and must therefore happen before any stream capture; first
 * calls from several host threads at once are safe (each stores the same address).  All
 * calls share the array: calls that overlap on the GPU (other streams, other host threads)
 * race and must be serialised by the caller.  Every GPU that loads the library keeps the
 * 8 MiB until the process exits. */
int xrh_density_build_noalloc(int precision, int64_t K, const int64_t* idx_ptr_dev,
                              const int32_t* P_dev, const int32_t* Q_dev, const int8_t* sign_dev,
                              const double* zbT_dev, int n_b, const double* zkT_dev, int n_k,
                              double* rho_dev, void* stream);

/* out[c, r] = in[r, c] for a row-major [rows, cols] FP64 matrix. */
int xrh_transpose(const double* in_dev, int64_t rows, int64_t cols, double* out_dev, void* stream);
/* Many transposes in one launch: task t transposes in [rows, cols] into out [cols, rows] and
 * owns the launch's 32 x 32 tiles [tile_begin, tile_begin + ceil(rows/32) * ceil(cols/32))
 * (tasks sorted by tile_begin, total_tiles the sum). */
typedef struct {
    const double* in;
    double* out;
    int64_t rows, cols;
    int64_t tile_begin;
} xrh_transpose_task;   /* 40 bytes */
int xrh_transpose_grouped(const xrh_transpose_task* tasks_dev, int n_tasks, int64_t total_tiles, void* stream);

/* Mirrored density blocks (no reference counterpart: the reference builds every block):
 * rho^cca(b, k)[I, J, p, q, r] = rho^caa(k, b)[J, I, r, q, p], and likewise cc / aa, c / a.
 *   dst[a][b][f] = (accumulate ? dst[a][b][f] : 0) + src[b][a][reverse(f)]
 * for a < na, b < nb and f over N^L (L <= 3 operator indices, N <= 64, reverse = digits in
 * reverse order).  The adjoint uses the same map with accumulate = 1. */
int xrh_mirror_density(int na, int nb, int N, int L, const double* src_dev, double* dst_dev,
                       int accumulate, void* stream);
/* Many mirrors in one launch: task t is one xrh_mirror_density call and owns the launch's CTAs
 * [cta_begin, cta_begin + na * nb * xrh_mirror_ctas(N, L)) (tasks sorted by cta_begin,
 * total_ctas the sum).  The tasks' dst blocks must not overlap.  xrh_mirror_ctas: CTAs per
 * (a, b) pair (1 for L < 3; for L = 3 one CTA per group of about 4096 / N^2 q planes), 0 for
 * unsupported N or L. */
int64_t xrh_mirror_ctas(int N, int L);

/* Antisymmetric operator pairs (no reference counterpart: the reference's density loops visit
 * every ordered index tuple, density_tensors.c:283-556).  Two adjacent operators of one kind
 * anticommute, so rho[.. o_u, o_u+1 ..] = -rho[.. o_u+1, o_u ..] and the density kernels need
 * the canonical tuples (o_u < o_u+1) only.  Task t covers one block in the transposed layout
 * rows[idx * R + e] (idx row-major over L indices of N values, R = n_b n_k elements per row)
 * and owns the launch's CTAs [cta_begin, cta_begin + N^L) (sorted, total_ctas the sum):
 *   mode 0: rows[idx] = -rows[swap_u(idx)] for every idx with o_u > o_u+1 (fill);
 *   mode 1: rows[idx] -= rows[swap_u(idx)] for every idx with o_u < o_u+1 (fold, the gradient
 *           of the canonical rows from the full gradient);
 * and for a Hermitian pair (rho^ca between the same real states, R = nrow^2, rows read as
 * nrow x nrow matrices M):
 *   mode 2: M[idx] = M[swap_u(idx)]^T for o_u > o_u+1;   mode 3: M[idx] += M[swap_u(idx)]^T
 *           for o_u < o_u+1. */
typedef struct {
    double* rows;
    int64_t R;
    int32_t N, L, u, mode;
    int32_t nrow, reserved;
    int64_t cta_begin;
} xrh_antisym_task;   /* 48 bytes */
int xrh_antisym_rows(const xrh_antisym_task* tasks_dev, int n_tasks, int64_t total_ctas, void* stream);
typedef struct {
    const double* src;
    double* dst;
    int32_t na, nb, N, L;
    int32_t accumulate, reserved;
    int64_t cta_begin;
} xrh_mirror_task;   /* 48 bytes */
int xrh_mirror_grouped(const xrh_mirror_task* tasks_dev, int n_tasks, int64_t total_ctas, void* stream);

/* Monomer two-electron term without the N^4 density (replaces building rho^ccaa and
 * contracting it, general-XRCC/build_density_tensors.py:122-133 + H_contractions.c:61-78):
 *   sigmaT[J, P] = sum_Q <P| sum_pqrs V_pqrs c+_p c+_q a_s a_r |Q> zk[J, Q]
 * for every bra determinant P; V_dev is the fragment's antisymmetric N^4 block.  The
 * caller finishes with E2 = Zb . sigma (one GEMM).  precision XRH_FP64 or XRH_FP32. */
int xrh_sigma2e(int precision, int n_orbs, const double* V_dev,
                const uint64_t* bra_masks_dev, int n_bra_conf,
                const uint64_t* ket_sorted_masks_dev, const int32_t* ket_sorted_pos_dev, int n_ket_conf,
                const int32_t* rank_table_dev, int64_t table_size, const int64_t* binom_dev,
                const double* zkT_dev, int n_k, double* sigmaT_dev, void* stream);
/* Determinant lookup in xrh_sigma2e and xrh_ccaa_weighted: with rank_table_dev == NULL, a
 * binary search of the sorted ket list; otherwise rank_table_dev[colex_rank(mask)] (size
 * table_size = C(N, n_e), -1 for determinants not in the list) with
 * colex_rank = sum_i C(o_i, i+1) over the occupied spin orbitals o_0 < o_1 < ..., and
 * binom_dev[n*17 + k] = C(n, k) for n <= 64, k <= 16. */

/* Grouped GEMM with K-concatenated segments and an FP64 epilogue.
 * For each task t and each (m, n) in [0,M) x [0,N):
 *   acc = sum over the task's segments s of alpha_s * sum_k A_s[m, k] * B_s[n, k]
 * (A_s, B_s row-major with K contiguous, row strides lda/ldb in elements).  Then
 *   mode 0: C[m*ldc + n]  = acc
 *   mode 1: C[m*ldc + n] += acc   (atomic; the task may be split splitk ways along K)
 *   mode 2: H[(rowA[m]+rowB[n])*ldc + colA[m]+colB[n]] =
 *              acc + (diagB[n] ? DA[m] : 0) + (diagA[m] ? DB[n] : 0)
 *           (charge-block to product-state scatter with the delta-function terms,
 *            hermitian-XRCC/XR_term.py:36-94, get_xr_result.py:300-353)
 * Operand storage per segment (flags): bit 0 clear: A[m,k] = A[m*lda + k]; set: A[k*lda + m].
 * bit 1 clear: B[n,k] = B[n*ldb + k]; set: B[k*ldb + n].  A task covers `batch`
 * independent problems: problem b uses A + b*sA, B + b*sB (per segment) and C + b*sC.
 * tasks_dev / segs_dev are device arrays of the structs below; tile_begin of every task
 * and total_tiles come from the host (64x64 tiles for XRH_FP64, times splitk, times batch). */
typedef struct {
    const double* A;
    const double* B;
    int64_t lda, ldb;
    int64_t K;
    double alpha;
    int64_t flags;
    int64_t sA, sB;
} xrh_gemm_segment;

typedef struct {
    int64_t M, N;
    int64_t seg_begin, seg_count;
    int64_t mode;
    int64_t splitk;
    int64_t tile_begin;
    double* C;
    int64_t ldc;
    const int32_t* rowA;
    const int32_t* colA;
    const int32_t* rowB;
    const int32_t* colB;
    const double* DA;
    const double* DB;
    const uint8_t* diagA;
    const uint8_t* diagB;
    int64_t batch;
    int64_t sC;
} xrh_gemm_task;

int xrh_gemm_fp64_grouped(const xrh_gemm_task* tasks_dev, int n_tasks, int64_t total_tiles,
                          const xrh_gemm_segment* segs_dev, void* stream);
/* Same tasks with a choice of arithmetic on CUDA cores: XRH_FP64 (identical to
 * xrh_gemm_fp64_grouped) or XRH_FP32 (operands rounded to FP32, products and the partial
 * sum of each 16-wide K step in FP32, running sums and epilogue in FP64). */
int xrh_gemm_simt_grouped(int precision, const xrh_gemm_task* tasks_dev, int n_tasks, int64_t total_tiles,
                          const xrh_gemm_segment* segs_dev, void* stream);

/* FP64 Lanczos building blocks for the lowest eigenpairs of H (replaces the dense
 * scipy.linalg.eig of hermitian-XRCC/mains/workflow.py:229 and
 * StateSpaceOptimizer/state_gradients.py:107 for the eigenpairs the optimizer uses):
 *   xrh_gemv_rows: y[i] = alpha * sum_j A[i*lda+j] x[j] + beta * y[i],  i < rows
 *   xrh_gemv_cols: y[j] += scale * sum_i c[i] A[i*lda+j],                j < cols
 *   xrh_lanczos_normalize: *beta = ||w||_2, v = w / *beta (v = 0 when w = 0). */
int xrh_gemv_rows(int64_t rows, int64_t cols, const double* A_dev, int64_t lda, const double* x_dev,
                  double alpha, double beta, double* y_dev, void* stream);
int xrh_gemv_cols(int64_t rows, int64_t cols, const double* A_dev, int64_t lda, const double* c_dev,
                  double scale, double* y_dev, void* stream);
int xrh_lanczos_normalize(int64_t n, const double* w_dev, double* v_dev, double* beta_dev, void* stream);
/* The same products for few rows over long vectors (the matrix-free Lanczos of a product space,
 * n ~ 10^5..10^6; replaces the same dense eigensolve as above): the columns are split over CTAs
 * of 2048 columns, each writing one partial per row into work_dev, and a second launch adds the
 * partials of a row in CTA order (deterministic).  work_len >= xrh_gemv_split_work(rows, cols)
 * doubles for xrh_gemv_rows_split and >= xrh_gemv_split_work(1, n) for
 * xrh_lanczos_normalize_split; XRH_ERR_CAPACITY when smaller. */
int64_t xrh_gemv_split_work(int64_t rows, int64_t cols);
int xrh_gemv_rows_split(int64_t rows, int64_t cols, const double* A_dev, int64_t lda, const double* x_dev,
                        double alpha, double beta, double* y_dev, double* work_dev, int64_t work_len, void* stream);
int xrh_lanczos_normalize_split(int64_t n, const double* w_dev, double* v_dev, double* beta_dev, double* work_dev,
                                int64_t work_len, void* stream);
/* xrh_gemv_rows for a table of GEMVs in one launch: task t computes rows [0, rows) of
 * y = alpha A x + beta y and owns the launch's rows [row_begin, row_begin + round_up(rows, 8));
 * tasks sorted by row_begin, total_rows8 = the sum of the rounded row counts.  With beta == 1
 * the products are added with FP64 atomics (tasks may then share rows of y). */
typedef struct {
    const double* A;
    const double* x;
    double* y;
    int64_t rows, cols, lda;
    double alpha, beta;
    int64_t row_begin;
} xrh_gemv_task;   /* 72 bytes */
int xrh_gemv_rows_grouped(const xrh_gemv_task* tasks_dev, int n_tasks, int64_t total_rows8, void* stream);
/* The whole Krylov loop of a small sector (n <= 4096) in one launch (one CTA): V[0] = v0,
 * then for j < m: w = H V[j]; two classical Gram-Schmidt passes against V[0..j];
 * alpha[j] = the two passes' coefficients of V[j] summed; beta[j] = |w|;
 * V[j+1] = w / beta[j] (0 when beta[j] = 0).  V is (m+1) x n.  Same arithmetic as
 * xrh_gemv_rows / xrh_gemv_cols / xrh_lanczos_normalize step by step. */
int xrh_lanczos_small(int n, int m, const double* H_dev, int64_t ld, const double* v0_dev,
                      double* V_dev, double* alpha_dev, double* beta_dev, void* stream);

/* The same Krylov loop for any n as ONE cooperative launch (cudaLaunchCooperativeKernel):
 * the CTAs (about 4 rows of H each, at most one per SM) split the rows of H, V and w and meet
 * at four grid barriers per step; cross-CTA sums run in a fixed CTA order, so results do not
 * depend on scheduling.  work_dev holds xrh_lanczos_coop_work(m) doubles of scratch (partial
 * sums and the barrier words, reset by this call).  A barrier wait that exceeds its poll
 * limit sets *status_dev = XRH_ERR_TIMEOUT and the kernel returns early; *status_dev must be
 * XRH_OK on entry. */
/* The same loop inside one thread-block cluster (up to 16 CTAs, one per SM; at most max_ctas
 * when max_ctas > 0; hardware cluster barriers, partial sums and V[j+1] exchanged through
 * distributed shared memory, H rows kept in shared memory when they fit).  XRH_ERR_CAPACITY
 * when the sector does not fit the cluster's shared memory (then use xrh_lanczos_coop). */
int xrh_lanczos_cluster(int n, int m, const double* H_dev, int64_t ld, const double* v0_dev, double* V_dev,
                        double* alpha_dev, double* beta_dev, int max_ctas, void* stream);
/* 1 when xrh_lanczos_cluster can take an n x n sector and m steps (same max_ctas) on the
 * current device. */
int xrh_lanczos_cluster_fits(int n, int m, int max_ctas);
int64_t xrh_lanczos_coop_work(int m);
int xrh_lanczos_coop(int64_t n, int m, const double* H_dev, int64_t ld, const double* v0_dev,
                     double* V_dev, double* alpha_dev, double* beta_dev, double* work_dev,
                     int64_t work_len, int32_t* status_dev, void* stream);
/* xrh_lanczos_coop with the grid barriers' wait bound given by the caller: a CTA that has
 * polled max_polls times without the others arriving writes XRH_ERR_TIMEOUT to *status_dev
 * and returns, and the other CTAs return at their next barrier (max_polls = 0: a CTA gives
 * up unless every other CTA has already arrived, so any launch of two or more CTAs reports
 * XRH_ERR_TIMEOUT; for tests of the failure path).  No reference counterpart. */
int xrh_lanczos_coop_bounded(int64_t n, int m, const double* H_dev, int64_t ld, const double* v0_dev,
                             double* V_dev, double* alpha_dev, double* beta_dev, double* work_dev,
                             int64_t work_len, int32_t* status_dev, int64_t max_polls, void* stream);

/* The optimizer's state update for every (fragment, charge) block at once; replaces the
 * per-fragment NumPy step of StateSpaceOptimizer/state_solver.py:207-453 (tangent
 * projection, steepest-descent step, Loewdin orthonormalisation).  A block holds n <= 64
 * row-orthonormal states z (n x K row-major), their gradient g = gT^T (+ gT32^T when gT32 is
 * not NULL; gT, gT32 are K x n), a scratch zn (n x K) and three n x n matrices G, S, M.  Task t owns CTAs [cta_begin, cta_begin +
 * xrh_state_ctas(K)).  In FP64 throughout:
 *   xrh_gram_grouped(which=0): G += g z^T;   (which=1): S += zn zn^T   (G, S zeroed by the caller)
 *   xrh_tangent_step:  zn = z - eps (g - 1/2 (G + G^T) z);  *sq_dev += |g - 1/2 (G + G^T) z|^2
 *   xrh_inv_sqrt_small: M = S^-1/2 by `iters` coupled Newton-Schulz steps (n <= 32; one CTA
 *                       per task, the tasks array indexed directly)
 *   xrh_left_multiply:  z = M zn */
typedef struct {
    const double* gT;
    const float* gT32;
    double* z;
    double* zn;
    double* G;
    double* S;
    double* M;
    int64_t K;
    int32_t n;
    int32_t reserved;
    int64_t cta_begin;
} xrh_state_task;

int xrh_state_ctas(int64_t K);
int xrh_gram_grouped(const xrh_state_task* tasks_dev, int n_tasks, int64_t total_ctas, int which,
                     void* stream);
int xrh_tangent_step(const xrh_state_task* tasks_dev, int n_tasks, int64_t total_ctas, double eps,
                     double* sq_dev, void* stream);
int xrh_inv_sqrt_small(const xrh_state_task* tasks_dev, int n_tasks, int iters, void* stream);
int xrh_left_multiply(const xrh_state_task* tasks_dev, int n_tasks, int64_t total_ctas, void* stream);

/* Integral derivatives for the orbital gradient from the reverse pass's pieces (replaces the
 * integral-derivative assembly feeding StateSpaceOptimizer/orb_grads.py): pointers to the
 * contiguous FP64 pieces of a dimer (fragment 0 = spin orbitals [0, N0), fragment 1 = [N0,
 * N0 + N1), N0 + N1 <= 64; gw (N1, N1, N0, N0); per fragment m with o the other: h1 (No, Nm),
 * cca and caa (No, Nm, Nm, Nm), cc (No, No, Nm, Nm), mono1 (Nm, Nm), gamma64 (Nm^4) plus an
 * optional FP32 part gamma32).  xrh_orbital_terms writes dT (t x t, t = N0 + N1; also the
 * derivative of every fragment potential) and B[p,q,r,s] = Ga[pqrs] + Ga[rspq] with Ga the
 * (pq)- and (rs)-antisymmetrised dE/dV (t^4; FP32 with FP32 arithmetic for XRH_FP32, FP64 for
 * XRH_FP64).  dE/dkappa's two-electron part is then 1/2 V_(1) B_(1)^T (xrh_abt_small).
 * in_host is a host pointer; two kernel launches. */
typedef struct {
    const double* gw;
    const double* h1[2];
    const double* cca[2];
    const double* caa[2];
    const double* cc[2];
    const double* mono1[2];
    const double* gamma64[2];
    const float* gamma32[2];
    int32_t N0, N1;
} xrh_orbital_inputs;   /* 128 bytes */
int xrh_orbital_terms(const xrh_orbital_inputs* in_host, double* dT_dev, void* B_dev, int precision, void* stream);

/* C (m x n, FP64, row-major, ld n) += alpha * A B^T for m, n <= 64 and long K: A (m x K, ld
 * lda) and B (n x K, ld ldb) are double (XRH_FP64) or float (XRH_FP32: FP32 products summed in
 * FP32 over 32 columns, then in FP64).  K is split over CTAs with FP64 atomic adds into C.
 * The orbital-gradient contraction 4 V_(1) Gbar_(1)^T of the integral derivative
 * (StateSpaceOptimizer/orb_grads.py, the two-electron term) is its main use. */
int xrh_abt_small(int precision, int m, int n, int64_t K, const void* A_dev, int64_t lda,
                  const void* B_dev, int64_t ldb, double alpha, double* C_dev, void* stream);
/* A table of such products in one launch: task t owns CTAs [cta_begin, cta_begin +
 * xrh_abt_ctas(K)) (tasks sorted by cta_begin, total_ctas the sum), m, n <= 64, C row
 * stride n.  Used for E2 = Zb sigma^T, the monomer two-electron blocks
 * (general-XRCC/build_density_tensors.py:122-133 folds them into ccaa numbers). */
typedef struct {
    const void* A;
    const void* B;
    double* C;
    int64_t m, n, K, lda, ldb;
    double alpha;
    int64_t cta_begin;
    int64_t flags;    /* bit 0: A stored K-major (A[i][k] = A[k*lda + i]); bit 1: B likewise */
} xrh_abt_task;   /* 88 bytes */
int xrh_abt_ctas(int64_t K);
int xrh_abt_grouped(int precision, const xrh_abt_task* tasks_dev, int n_tasks, int64_t total_ctas,
                    void* stream);

/* Adjoint of the density build (dE/dz from dE/drho), the reverse of xrh_density_accumulate
 * over the same coupling lists; replaces the determinant-bra density rebuild plus second H
 * build of StateSpaceOptimizer/state_gradients.py:164-185.  gT_dev is dE/drho in
 * [K, n_b, n_k] layout; results are ADDED (atomically) to gzbT_dev [n_bra_conf, n_b] and
 * gzkT_dev [n_ket_conf, n_k], which may be the same buffer: double arrays for XRH_FP64,
 * float arrays for XRH_FP32 (FP32 products and sums, 16-byte vector atomics).  For XRH_FP32
 * the coefficients zbT_dev/zkT_dev are the padded FP32 copies of xrh_density_accumulate_f32
 * (rows of round_up(n,4) floats); for XRH_FP64 the double [n_conf, n] arrays. */
int xrh_density_adjoint(int precision, int64_t K, const int64_t* idx_ptr_dev,
                        const int32_t* P_dev, const int32_t* Q_dev, const int8_t* sign_dev,
                        const void* zbT_dev, int n_b, const void* zkT_dev, int n_k,
                        const double* gT_dev, void* gzbT_dev, void* gzkT_dev, void* stream);

/* xrh_density_adjoint (XRH_FP32) for every density block of a fragment in one launch:
 * task t owns CTAs [cta_begin, cta_begin + K) (one per operator index), gT its transposed
 * density gradient [K, nb, nk], gzb / gzk the FP32 gradient rows of its bra / ket charge
 * (several tasks may share them: vector atomics). */
typedef struct {
    const int64_t* idx_ptr;
    const int32_t* P;
    const int32_t* Q;
    const int8_t* sign;
    const float* zb32;
    const float* zk32;
    const double* gT;
    float* gzb;
    float* gzk;
    int64_t K;
    int32_t nb, nk;
    int64_t cta_begin;
} xrh_dens_adj_task;   /* 96 bytes */
int xrh_density_adjoint_f32_grouped(const xrh_dens_adj_task* tasks_dev, int n_tasks, int64_t total_ctas,
                                    int max_nb, int max_nk, void* stream);
/* The same adjoint for blocks with n_b, n_k <= max_n <= 16 over a unit table (one warp per
 * unit, one lane per coupling; xrh_dens_unit as for xrh_density_accumulate_f32_units, every
 * unit adds atomically so split indices need nothing extra; cta_begin is not used).
 * g_layout 0: gT is dE/drho in [K, n_b, n_k] layout (as above); 1: in the density's own
 * [n_b, n_k, K] layout (no transposed copy needed). */
int xrh_density_adjoint_f32_units(const xrh_dens_adj_task* tasks_dev, int n_tasks,
                                  const xrh_dens_unit* units_dev, int64_t n_units, int max_n,
                                  int g_layout, void* stream);

/* The same reverse pass on the tensor cores (3 x TF32 split, tcgen05), for blocks with
 * n_b, n_k <= 64: per operator index, tiles of 128 couplings times G (both orientations)
 * as two 128 x 64 x 64 GEMMs with gathered coefficient rows.  zbh/zbl, zkh/zkl: the bra /
 * ket coefficients split into TF32 hi and lo (xrh_split_operand, rows of 64 values, zero
 * padded).  gzb / gzk receive FP32 vector atomics; *status_dev = XRH_ERR_TIMEOUT when a
 * bounded wait expired. */
typedef struct {
    const int64_t* idx_ptr;
    const int32_t* P;
    const int32_t* Q;
    const int8_t* sign;
    const uint32_t* zbh;
    const uint32_t* zbl;
    const uint32_t* zkh;
    const uint32_t* zkl;
    const double* gT;
    float* gzb;
    float* gzk;
    int64_t K;
    int32_t nb, nk;
    int64_t cta_begin;
} xrh_dens_adj_tc_task;   /* 112 bytes */
int xrh_density_adjoint_tc_grouped(const xrh_dens_adj_tc_task* tasks_dev, int n_tasks, int64_t total_ctas,
                                   int32_t* status_dev, void* stream);

/* Two-electron terms through (n-2)-electron intermediates K (no reference counterpart: the
 * reference builds rho^ccaa element by element, density_tensors.c:493-556, and contracts it,
 * H_contractions.c:61-78).  A pair list holds, for every determinant X of a space and every
 * occupied pair u < v, the sign of <K| a_v a_u |X> and the position of (K, pair) in a
 * class-major array [spin class][state][K][pair]: off_e for state 0 and stride_e per state.
 *   xrh_pair_scatter:  D[off_e + s * stride_e] = sign_e * zT[X_e * n + s]  for s < n
 *   xrh_pair_gather:   sigmaT[s * n_X + x] = sum over x's entries e (xptr[x] .. xptr[x+1])
 *                      of sign_e * E[off_e + s * stride_e]
 * With E = D . W^T per class (W[pq, rs] = 4 V_pqrs), gather gives xrh_sigma2e's sigmaT, and
 * D_zb^T D_Y per class gives xrh_ccaa_weighted's Gamma for p<q, r<s.  Positions of D never
 * written stay as the caller initialised them (zero). */
int xrh_pair_scatter(int64_t n_entries, const int32_t* X_dev, const int64_t* off_dev,
                     const int8_t* sign_dev, const double* zT_dev, int n, const int64_t* stride_dev,
                     double* D_dev, void* stream);
int xrh_pair_gather(int n_X, const int64_t* xptr_dev, const int64_t* off_dev,
                    const int8_t* sign_dev, const double* E_dev, int n, const int64_t* stride_dev,
                    double* sigmaT_dev, void* stream);
/* Many xrh_pair_scatter (gather = 0) or xrh_pair_gather (gather = 1) calls in one launch.
 * Scatter task: dst = D, src = zT, count = n_entries (X, off, sign, stride per entry).
 * Gather task: dst = sigmaT, src = E, count = n_X (xptr, off, sign, stride per entry).
 * max_total = the largest count * n over the tasks (it sizes the grid). */
typedef struct {
    const int32_t* X;
    const int64_t* xptr;
    const int64_t* off;
    const int8_t* sign;
    const int64_t* stride;
    const double* src;
    double* dst;
    int64_t count;
    int64_t n;
} xrh_pair_task;   /* 72 bytes */
int xrh_pair_grouped(int gather, const xrh_pair_task* tasks_dev, int n_tasks, int64_t max_total, void* stream);

/* Transition densities through intermediate determinants K (no reference counterpart; they
 * replace the per-coupling outer products of density_tensors.c:142-556 on the split-precision
 * paths).  rho^op[I, J, cre, ann] = sum_K C[K, cre, I] A[K, ann, J] with C, A index scatters
 * of the coefficients; X[(I, ci), (J, ai)] = sum_K Ct[(I, ci), K] At[(J, ai), K] is a GEMM.
 *   xrh_im_scatter: for entries e (determinant x_e, index idx_e < nidx, intermediate k_e < nK,
 *       sign_e) and states s < n:  v = sign_e zT[x_e * n + s];
 *       Dt[(s * nidx + idx_e) * nK + k_e] = v  and, when D_dev is not NULL,
 *       D[k_e * (n * nidx) + s * nidx + idx_e] = v.  Unwritten positions keep their value.
 *   xrh_im_expand:  rho[(I * nk + J) * F + f] = sign_f X[(I * ncre + ci_f) * (nk * nann)
 *       + J * nann + ai_f]  (0 where sign_f = 0).
 *   xrh_im_fold:    gX[((I * ncre + c) * nk + J) * nann + a] = sum_{h < 2} sign[2 q + h]
 *       grho[(I * nk + J) * F + src[2 q + h]],  q = c * nann + a  (sign 0: no source).
 *   xrh_im_gather:  gzT[x * n + s] += sum_{e = ptr[x]}^{ptr[x+1]-1} sign_e
 *       gDt[(s * nidx + idx_e) * nK + k_e]. */
int xrh_im_scatter(int64_t n_entries, const int32_t* x_dev, const int32_t* idx_dev, const int32_t* k_dev,
                   const int8_t* sign_dev, const double* zT_dev, int n, int64_t nK, int nidx,
                   double* Dt_dev, double* D_dev, void* stream);
int xrh_im_expand(int nb, int nk, int64_t F, const int32_t* ci_dev, const int32_t* ai_dev,
                  const int8_t* sign_dev, int ncre, int nann, const double* X_dev, double* rho_dev,
                  void* stream);
int xrh_im_fold(int nb, int nk, int64_t F, int ncre, int nann, const int32_t* src_dev,
                const int8_t* sign_dev, const double* grho_dev, double* gX_dev, void* stream);
int xrh_im_gather(int n_x, const int64_t* ptr_dev, const int32_t* idx_dev, const int32_t* k_dev,
                  const int8_t* sign_dev, int n, int64_t nK, int nidx, const double* gDt_dev,
                  double* gzT_dev, void* stream);

/* Two-particle density of a weighted ensemble for the monomer two-electron term:
 *   Gamma[p,q,r,s] += sum_{P,Q} W[P,Q] <P| c+_p c+_q a_s a_r |Q>,  p<q and r<s only,
 *   W[P,Q] = sum_I zbT[P, I] YT[Q, I]   (Y = G . z for weights G over state pairs)
 * i.e. dE/dV for E = sum_IJ G_IJ sum_pqrs V_pqrs rho^ccaa_IJ[p,q,s,r] (orb_grads.py:921
 * two_p_dens for the intra-fragment term) without the N^4 density.  Gamma_dev is N^4
 * (N = 2 n_orbs) doubles (XRH_FP64) or floats (XRH_FP32), accumulated atomically; the
 * caller fills the other index orders by antisymmetry.  n <= 256 states. */
int xrh_ccaa_weighted(int precision, int n_orbs, const uint64_t* bra_masks_dev, int n_bra_conf,
                      const uint64_t* ket_sorted_masks_dev, const int32_t* ket_sorted_pos_dev, int n_ket_conf,
                      const int32_t* rank_table_dev, int64_t table_size, const int64_t* binom_dev,
                      const double* zbT_dev, const double* YT_dev, int n, void* Gamma_dev, void* stream);

/* ---- split-precision tensor-core path (tcgen05, sm_103a) -------------------------------
 * Same task model as xrh_gemm_fp64_grouped for the forward build.  Every FP64 operand is
 * first split by xrh_split_operand into hi = round(x), lo = round(x - hi) in BF16
 * (XRH_BF16X3) or TF32 stored as 32-bit words (XRH_TF32X3), row-major [rows, Kp] with
 * Kp a multiple of xrh_tc_chunk_elems(precision) (64 or 32; the padding is zero).
 * xrh_tc_encode_map writes (on the host) the 128-byte TMA descriptor of one such array with
 * a box of xrh_tc_chunk_elems x box_rows and 128-byte swizzle; an operand is described by
 * two consecutive maps (hi, lo) in a device array of maps (64-byte aligned).
 * A segment contributes A_hi B_hi^T + A_hi B_lo^T + A_lo B_hi^T with FP32 accumulation
 * (negate != 0 flips its sign; other scale factors must be folded into the operands).
 * Tiles are 128 x bn (bn = 32, 64 or 128, the box rows of the B maps), times splitk.
 * Modes and the epilogue are those of xrh_gemm_fp64_grouped (FP64 output).  A bounded
 * wait that expires sets *status_dev = XRH_ERR_TIMEOUT (status_dev must start at 0). */
typedef struct {
    int64_t tmA;       /* index of A's hi map (lo map at tmA + 1) */
    int64_t tmB;       /* index of B's hi map (lo map at tmB + 1) */
    int64_t kchunks;   /* K chunks of this segment (Kp / xrh_tc_chunk_elems) */
    int64_t negate;
} xrh_tc_segment;

typedef struct {
    int64_t M, N;
    int64_t seg_begin, seg_count;
    int64_t mode;
    int64_t splitk;
    int64_t tile_begin;
    int64_t bn;
    double* C;
    int64_t ldc;
    const int32_t* rowA;
    const int32_t* colA;
    const int32_t* rowB;
    const int32_t* colB;
    const double* DA;
    const double* DB;
    const uint8_t* diagA;
    const uint8_t* diagB;
} xrh_tc_task;

int xrh_tc_chunk_elems(int precision);
int xrh_split_operand(int precision, const double* src_dev, int64_t rows, int64_t K, int64_t ld,
                      int64_t Kp, void* hi_dev, void* lo_dev, void* stream);
/* xrh_split_operand for every operand of a task table in one launch.  Task t splits rows x Kp
 * (src rows of ld doubles, K of them used, the rest of each row written as zeros) into hi/lo
 * (16-byte aligned, Kp a multiple of xrh_tc_chunk_elems); its 4-element groups are
 * [group_begin, group_begin + rows * Kp / 4) of the launch, tasks sorted by group_begin and
 * total_groups the sum. */
typedef struct {
    const double* src;
    void* hi;
    void* lo;
    int64_t rows, K, ld, Kp;
    int64_t group_begin;
} xrh_split_task;   /* 64 bytes */
int xrh_split_grouped(int precision, const xrh_split_task* tasks_dev, int n_tasks, int64_t total_groups,
                      void* stream);
int xrh_tc_encode_map(int precision, const void* base_dev, int64_t rows, int64_t Kp, int box_rows,
                      void* map_out_host);
int xrh_gemm_tc_grouped(int precision, const xrh_tc_task* tasks_dev, int n_tasks, int64_t total_tiles,
                        const xrh_tc_segment* segs_dev, const void* maps_dev, int32_t* status_dev,
                        void* stream);

/* Small dense FP64 matrices of the orbital transformation (n <= 64, row-major, one CTA each;
 * XRH_ERR_CAPACITY above):
 *   xrh_inverse_small: Ainv = A^-1 by Gauss-Jordan with partial pivoting; *status_dev = 0, or 1
 *       for a pivot below 1e-300 (Ainv then undefined).  Replaces the overlap inverse of the
 *       biorthogonalisation, direct_Sinv (hermitian-XRCC/get_ints.py:62-66).
 *   xrh_expm_small: E = exp(A) by scaling and squaring with a degree-16 Taylor polynomial: the
 *       orbital rotation R = exp(kappa) (no reference counterpart: the reference's orbital
 *       solver rotates with the first-order I + s x, StateSpaceOptimizer/orbital_solver.py:431).
 *   xrh_spin_block: out[a, b] = in[sidx[a], sidx[b]] if spin[a] == spin[b] else 0, the
 *       spin-orbital form of a spatial matrix (no reference counterpart: qode's
 *       spin_orb_integrals, hermitian-XRCC/get_ints.py:134-135, does this on the host). */
int xrh_inverse_small(int n, const double* A_dev, int64_t lda, double* Ainv_dev, int64_t ldi,
                      int32_t* status_dev, void* stream);
int xrh_expm_small(int n, const double* A_dev, int64_t lda, double* E_dev, int64_t lde, void* stream);
int xrh_spin_block(int n_so, const int32_t* sidx_dev, const int8_t* spin_dev, const double* in_dev, int64_t ldin,
                   double* out_dev, int64_t ldout, void* stream);
/* out[i, j] = in[idx[i], idx[j]], i, j < n: a principal submatrix (the alpha-alpha block of
 * a spin-orbital overlap before its inverse; no reference counterpart). */
int xrh_gather_submatrix(int n, const int32_t* idx_dev, const double* in_dev, int64_t ldin, double* out_dev,
                         int64_t ldout, void* stream);

/* Helpers of the device-resident optimizer iteration (no reference counterpart; they keep
 * PyTorch and library kernels out of the captured iteration):
 *   xrh_zero: cudaMemsetAsync of bytes at ptr_dev;
 *   xrh_index_move: dst[idx[i]] = src[i] (gather = 0, indices distinct), dst[i] = src[idx[i]]
 *       (gather = 1) or dst[idx[i]] += src[i] (gather = 2, FP64 atomic adds: repeated indices
 *       allowed), i < n;
 *   xrh_f64_to_f32: dst[i] = (float)src[i], i < n (round to nearest);
 *   xrh_add_mixed: y[i] += alpha * (x64[i] + x32[i]) with either input NULL for zero (the two
 *       precision parts of a state gradient summed into an FP64 total);
 *   xrh_spin_sum_antisym: out[a, b] = sum_k (G[s_k(a), s_k(b)] - G[s_k(b), s_k(a)]) with
 *       s_k(a) = so[k * n_sp + a] the spin orbital of spatial orbital a in spin block k: the
 *       antisymmetric spatial orbital gradient from the spin-orbital one;
 *   xrh_small_mm_grouped: C = alpha A B + beta I for n x n row-major FP64 blocks, n <= 64, task
 *       t owning CTAs [cta_begin, cta_begin + ceil(n / 4)) (sorted, total_ctas the sum) -- the
 *       Newton-Schulz steps of the Loewdin orthonormalisation of every state block at once. */
typedef struct {
    const double* A;
    const double* B;
    double* C;
    int32_t n, reserved;
    double alpha, beta;
    int64_t cta_begin;
} xrh_small_mm_task;   /* 56 bytes */
int xrh_zero(void* ptr_dev, int64_t bytes, void* stream);
int xrh_index_move(int64_t n, const int64_t* idx_dev, const double* src_dev, double* dst_dev, int gather,
                   void* stream);
int xrh_f64_to_f32(int64_t n, const double* src_dev, float* dst_dev, void* stream);
int xrh_add_mixed(int64_t n, double alpha, const double* x64_dev, const float* x32_dev, double* y_dev, void* stream);
int xrh_spin_sum_antisym(int n_sp, int n_spin, const int32_t* so_dev, const double* G_dev, int64_t ldg,
                         double* out_dev, void* stream);
int xrh_small_mm_grouped(const xrh_small_mm_task* tasks_dev, int n_tasks, int64_t total_ctas, void* stream);

/* Reordering of the three-fragment vectors of the matrix-free H x v (no reference
 * counterpart: the reference forms the dense product-basis H, general-XRCC/hamiltonian.py:18-80):
 *   xrh_permute_grouped: task t writes dst[e] = scale * src[sum_k i_k src_stride[k]] for the
 *       row-major multi-index (i_0 .. i_{ndim-1}) of element e over dst_shape (ndim <= 6),
 *       e < n_elems; its elements are [elem_begin, elem_begin + n_elems) of the launch (tasks
 *       sorted by elem_begin, total_elems the sum);
 *   xrh_gather_sum: dst[j] = (accumulate ? dst[j] : 0) + sum_t src_t[idx_t[j]], t < n_terms <= 8,
 *       j < n, added in term order (deterministic; no atomics). */
typedef struct {
    const double* src;
    double* dst;
    int64_t dst_shape[6];
    int64_t src_stride[6];
    int32_t ndim, reserved;
    double scale;
    int64_t elem_begin, n_elems;
} xrh_permute_task;   /* 144 bytes */
int xrh_permute_grouped(const xrh_permute_task* tasks_dev, int n_tasks, int64_t total_elems, void* stream);
typedef struct {
    const double* src[8];
    const int64_t* idx[8];
    int32_t n_terms, reserved;
} xrh_gather_terms;   /* 136 bytes, passed by host pointer (the kernel receives a copy) */
int xrh_gather_sum(int64_t n, const xrh_gather_terms* terms, double* dst_dev, int accumulate, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* XRH_H */
