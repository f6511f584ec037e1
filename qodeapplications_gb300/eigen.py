"""Lowest eigenpairs of the symmetric excitonic Hamiltonian by FP64 Lanczos on the GPU.

Replaces the dense scipy.linalg.eig of the reference (hermitian-XRCC/mains/workflow.py:229,
StateSpaceOptimizer/state_gradients.py:107) for the quantities the optimizer uses: the
lowest eigenvalues and the ground-state eigenvector.  The Krylov loop (H x v, two passes of
classical Gram-Schmidt against all previous vectors, normalisation) runs entirely on the
device with fixed shapes, so it can be captured in a CUDA graph; only the small tridiagonal
eigenproblem (m x m) is solved on the host.

The default loop is "cluster" (one thread-block cluster of 8-16 CTAs, hardware cluster
barriers, distributed shared memory; for sectors whose rows fit the cluster's shared memory)
or else "coop" (one cooperative launch whose CTAs split the rows of H and meet at three grid
barriers per step): the FP64 rate of one SM would otherwise bound the loop.  "small" is the
one-CTA loop and "steps" six launches per step, kept as cross-checks.
"""
import numpy as np
import torch

from . import _lib
from ._lib import call, ptr, stream_ptr

SMALL_SECTOR = 2048
MODES = ("auto", "cluster", "coop", "small", "steps")
CLUSTER_MAX_CTAS = 0     # CTAs of the cluster loop at most (0: the largest cluster the part runs)
CLUSTER_MAX_N = 512      # "auto" takes the cluster loop up to this sector size, the cooperative one above


class Lanczos:
    def __init__(self, n, m=96, device="cuda", seed=7, mode="auto", cluster_ctas=None):
        self.n = int(n)
        self.m = int(min(m, n))
        dev = torch.device(device)
        f64 = dict(dtype=torch.float64, device=dev)
        g = torch.Generator().manual_seed(seed)
        v0 = torch.randn(self.n, generator=g, dtype=torch.float64)
        self.v0 = (v0 / v0.norm()).to(dev)
        self.V = torch.zeros((self.m + 1, self.n), **f64)
        self.w = torch.empty(self.n, **f64)
        self.CC = torch.zeros((self.m, self.m + 1), **f64)
        self.CC2 = torch.zeros((self.m, self.m + 1), **f64)
        self.beta = torch.zeros(self.m, **f64)
        self.y = torch.zeros(self.m + 1, **f64)
        self.vec = torch.zeros(self.n, **f64)
        self.ab = torch.zeros(2 * self.m, **f64)          # alpha_j, beta_j
        self._host = torch.empty(3 * self.m, dtype=torch.float64).pin_memory() if torch.cuda.is_available() else None
        if mode not in MODES:
            raise ValueError(f"mode must be one of {MODES}")
        if mode == "small" and self.n > SMALL_SECTOR:
            mode = "steps"
        self.cluster_ctas = CLUSTER_MAX_CTAS if cluster_ctas is None else int(cluster_ctas)
        if mode in ("auto", "cluster"):
            from ._lib import lib
            fits = bool(lib().xrh_lanczos_cluster_fits(self.n, self.m, self.cluster_ctas))
            if mode == "auto" and self.n > CLUSTER_MAX_N:
                fits = False
            if mode == "cluster" and not fits:
                raise ValueError("sector too large for the cluster Lanczos loop")
            mode = "cluster" if fits else "coop"
        self.mode = mode
        self.small = mode != "steps"      # alpha/beta written straight into self.ab
        if mode == "coop":
            from ._lib import lib
            self.work = torch.zeros(int(lib().xrh_lanczos_coop_work(self.m)), **f64)
            self.status = torch.zeros(1, dtype=torch.int32, device=dev)
            self._host_status = torch.zeros(1, dtype=torch.int32).pin_memory() if torch.cuda.is_available() else None

    def krylov(self, H, ld=None):
        """Device-only part: m Lanczos steps on H (n x n, row stride ld)."""
        s = stream_ptr()
        n, m = self.n, self.m
        ld = n if ld is None else ld
        if self.mode == "cluster":
            call("xrh_lanczos_cluster", n, m, ptr(H), ld, ptr(self.v0), ptr(self.V), ptr(self.ab), ptr(self.ab[m:]),
                 self.cluster_ctas, s)
            return
        if self.mode == "coop":
            call("xrh_lanczos_coop", n, m, ptr(H), ld, ptr(self.v0), ptr(self.V), ptr(self.ab), ptr(self.ab[m:]),
                 ptr(self.work), self.work.numel(), ptr(self.status), s)
            return
        if self.mode == "small":
            call("xrh_lanczos_small", n, m, ptr(H), ld, ptr(self.v0), ptr(self.V), ptr(self.ab),
                 ptr(self.ab[m:]), s)
            return
        self.V[0].copy_(self.v0)
        for j in range(m):
            call("xrh_gemv_rows", n, n, ptr(H), ld, ptr(self.V[j]), 1.0, 0.0, ptr(self.w), s)
            for C in (self.CC, self.CC2):
                call("xrh_gemv_rows", j + 1, n, ptr(self.V), n, ptr(self.w), 1.0, 0.0, ptr(C[j]), s)
                call("xrh_gemv_cols", j + 1, n, ptr(self.V), n, ptr(C[j]), -1.0, ptr(self.w), s)
            call("xrh_lanczos_normalize", n, ptr(self.w), ptr(self.V[j + 1]), ptr(self.beta[j:j + 1]), s)

    def krylov_operator(self, apply):
        """The same m steps on a matrix-free operator (mode "steps" only): apply(x, y) writes
        y = H x for device vectors of length n, enqueued on the current stream."""
        if self.small:
            raise ValueError("krylov_operator needs mode='steps'")
        from ._lib import lib
        s = stream_ptr()
        n, m = self.n, self.m
        if getattr(self, "_split_work", None) is None:
            self._split_work = torch.zeros(int(lib().xrh_gemv_split_work(m + 1, n)), dtype=torch.float64,
                                           device=self.V.device)
        wk, nwk = self._split_work, self._split_work.numel()
        self.V[0].copy_(self.v0)
        for j in range(m):
            apply(self.V[j], self.w)
            for C in (self.CC, self.CC2):
                call("xrh_gemv_rows_split", j + 1, n, ptr(self.V), n, ptr(self.w), 1.0, 0.0, ptr(C[j]), ptr(wk), nwk, s)
                call("xrh_gemv_cols", j + 1, n, ptr(self.V), n, ptr(C[j]), -1.0, ptr(self.w), s)
            call("xrh_lanczos_normalize_split", n, ptr(self.w), ptr(self.V[j + 1]), ptr(self.beta[j:j + 1]),
                 ptr(wk), nwk, s)

    def stage_to_host(self):
        """Queue the copy of the tridiagonal coefficients (alpha_j, beta_j) to pinned memory."""
        m = self.m
        if not self.small:
            idx = torch.arange(m, device=self.CC.device)
            self.ab[:m].copy_(self.CC[idx, idx] + self.CC2[idx, idx])
            self.ab[m:].copy_(self.beta)
        self._host[:2 * m].copy_(self.ab, non_blocking=True)
        if self.mode == "coop":
            self._host_status.copy_(self.status, non_blocking=True)

    def solve(self, k=5):
        """Host part (after a sync): eigenpairs of the m x m tridiagonal matrix.
        Returns (lowest k Ritz values, residual norm estimate of the lowest)."""
        from scipy.linalg import eigh_tridiagonal
        m = self.m
        if self.mode == "coop" and int(self._host_status[0]) != 0:
            from ._lib import lib
            code = int(self._host_status[0])
            raise RuntimeError(f"xrh_lanczos_coop: {lib().xrh_status_string(code).decode()}")
        a = self._host[:m].numpy().copy()
        b = self._host[m:2 * m].numpy().copy()
        # stop at an invariant subspace (tiny beta): the rest of the basis is meaningless
        scale = max(np.abs(a).max(), np.abs(b).max(), 1e-300)
        cut = m
        for j in range(m - 1):
            if b[j] <= 1e-12 * scale:
                cut = j + 1
                break
        w, Y = eigh_tridiagonal(a[:cut], b[:cut - 1])
        self._ritz = Y[:, 0]
        self._cut = cut
        resid = abs(b[cut - 1] * Y[cut - 1, 0]) if cut == m else 0.0
        return w[:k], resid

    def ritz(self, k=5):
        """Host part (after a sync): the lowest k Ritz values, their tridiagonal eigenvectors
        (cut x k) and the residual norm estimate of each."""
        from scipy.linalg import eigh_tridiagonal
        self.solve(1)
        m, cut = self.m, self._cut
        a = self._host[:m].numpy()[:cut].copy()
        b = self._host[m:2 * m].numpy()[:cut].copy()
        w, Y = eigh_tridiagonal(a, b[:cut - 1])
        k = min(k, cut)
        resid = np.abs(b[cut - 1] * Y[cut - 1, :k]) if cut == m else np.zeros(k)
        return w[:k], Y[:, :k], resid

    def ritz_vector(self, y, out):
        """out = V^T y for a tridiagonal eigenvector y (length <= m), on the device."""
        yy = np.zeros(self.m + 1)
        yy[:len(y)] = y
        self.y.copy_(torch.from_numpy(yy))
        _lib.zero_(out)
        call("xrh_gemv_cols", self.m, self.n, ptr(self.V), self.n, ptr(self.y), 1.0, ptr(out), stream_ptr())
        return out

    def ground_vector(self):
        """Ritz vector of the lowest eigenvalue (device, normalised)."""
        y = np.zeros(self.m + 1)
        y[:self._cut] = self._ritz
        self.y.copy_(torch.from_numpy(y))
        _lib.zero_(self.vec)
        call("xrh_gemv_cols", self.m, self.n, ptr(self.V), self.n, ptr(self.y), 1.0, ptr(self.vec), stream_ptr())
        return self.vec


def lowest_eigenpairs_lanczos(H, k=5, m=96):
    """Convenience wrapper: (lowest k eigenvalues as numpy, ground-state vector on device)."""
    lz = Lanczos(H.shape[0], m=m, device=H.device)
    lz.krylov(H.contiguous())
    lz.stage_to_host()
    torch.cuda.current_stream().synchronize()
    w, resid = lz.solve(k)
    return w, lz.ground_vector(), resid


def lowest_eigenpairs(H, k=5, tol=1e-10, m=None):
    """Lowest k eigenvalues (numpy) and eigenvectors (device, n x k) of a symmetric FP64
    matrix on the device by this library's Lanczos loop: the Krylov depth doubles until every
    one of the k Ritz pairs has a residual below tol (relative to max(1, |w|)) or the depth
    reaches n, where the Krylov space is the whole space."""
    n = int(H.shape[0])
    H = H.contiguous()
    m = min(n, max(120, 8 * k) if m is None else int(m))
    while True:
        lz = Lanczos(n, m=m, device=H.device)
        lz.krylov(H)
        lz.stage_to_host()
        torch.cuda.current_stream().synchronize()
        w, Y, resid = lz.ritz(k)
        if m >= n or np.all(resid <= tol * np.maximum(1.0, np.abs(w))):
            break
        m = min(n, 2 * m)
    vecs = torch.zeros((n, len(w)), dtype=torch.float64, device=H.device)
    tmp = torch.zeros(n, dtype=torch.float64, device=H.device)
    for i in range(len(w)):
        vecs[:, i].copy_(lz.ritz_vector(Y[:, i], tmp))
    return w, vecs
