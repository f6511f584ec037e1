"""Lowest eigenpairs of the symmetric excitonic Hamiltonian by FP64 Lanczos on the GPU.

Replaces the dense scipy.linalg.eig of the reference (hermitian-XRCC/mains/workflow.py:229,
StateSpaceOptimizer/state_gradients.py:107) for the quantities the optimizer uses: the
lowest eigenvalues and the ground-state eigenvector.  The Krylov loop (H x v, two passes of
classical Gram-Schmidt against all previous vectors, normalisation) runs entirely on the
device with fixed shapes, so it can be captured in a CUDA graph; only the small tridiagonal
eigenproblem (m x m) is solved on the host.
"""
import numpy as np
import torch

from ._lib import call, ptr, stream_ptr

SMALL_SECTOR = 2048


class Lanczos:
    def __init__(self, n, m=96, device="cuda", seed=7):
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
        # sectors up to this size run the whole Krylov loop in one launch
        self.small = self.n <= SMALL_SECTOR

    def krylov(self, H, ld=None):
        """Device-only part: m Lanczos steps on H (n x n, row stride ld)."""
        s = stream_ptr()
        n, m = self.n, self.m
        ld = n if ld is None else ld
        if self.small:
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

    def stage_to_host(self):
        """Queue the copy of the tridiagonal coefficients (alpha_j, beta_j) to pinned memory."""
        m = self.m
        if not self.small:
            idx = torch.arange(m, device=self.CC.device)
            self.ab[:m].copy_(self.CC[idx, idx] + self.CC2[idx, idx])
            self.ab[m:].copy_(self.beta)
        self._host[:2 * m].copy_(self.ab, non_blocking=True)

    def solve(self, k=5):
        """Host part (after a sync): eigenpairs of the m x m tridiagonal matrix.
        Returns (lowest k Ritz values, residual norm estimate of the lowest)."""
        from scipy.linalg import eigh_tridiagonal
        m = self.m
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

    def ground_vector(self):
        """Ritz vector of the lowest eigenvalue (device, normalised)."""
        y = np.zeros(self.m + 1)
        y[:self._cut] = self._ritz
        self.y.copy_(torch.from_numpy(y))
        self.vec.zero_()
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
