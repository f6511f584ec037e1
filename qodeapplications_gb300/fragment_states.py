"""Fragment-state production on the device: determinant-space H Psi and FCI states.

Replaces the fragment-state machinery of general-XRCC/atomic_states:

* compute_HPsi (LMO_frozen_Hamiltonian.c:358): H Psi for a block of CI vectors over the
  determinants of one fragment and one electron count (frozen core allowed);
* generic_fci (generic_hamiltonian.c:167): the dense FCI matrix over a determinant list;
* the lowest FCI states of a charge sector, which the reference takes from a dense
  diagonalisation of that matrix, here from this library's FP64 Lanczos loop on H Psi.

H = sum h_pq c+_p a_q + sum V_pqrs c+_p c+_q a_s a_r (V antisymmetric in (p, q) and (r, s)).
On n-electron determinants the one-body part equals a two-body operator,
sum_pq h_pq c+_p a_q = 1/(n-1) sum_pqr h_pq c+_p c+_r a_r a_q, so H Psi is one two-electron
sigma vector with V' = V + antisym(h x 1)/(n-1): the (n-2)-electron pair intermediates of
SigmaTwoElectron (one pair scatter, one grouped GEMM per spin class, one pair gather) --
the same kernels as the monomer two-electron term of the XR-H build.  Needs n >= 2.
"""
import numpy as np
import torch

from ._lib import call, ptr, stream_ptr
from .densities import FragmentSpace
from .eigen import Lanczos
from .hamiltonian import SigmaTwoElectron


def folded_two_body(h, V, n_elec):
    """V' with V'_pqrs c+_p c+_q a_s a_r = V + h_pr c+_p (N - 1)^-1 ... antisymmetrised:
    W[p, r, q, r] += h_pq / (n - 1), V' = V + (W - W^(qp) - W^(sr) + W^(qp,sr)) / 4."""
    if n_elec < 2:
        raise ValueError("the folded one-body term needs at least two electrons")
    N = h.shape[0]
    W = torch.zeros_like(V)
    eye = torch.eye(N, dtype=h.dtype, device=h.device)
    # W[p, q', r', s'] = h[p, r'] delta(q', s') / (n - 1)  (c+_p c+_q' a_s' a_r' with q' = s')
    W += (h[:, None, :, None] * eye[None, :, None, :]) / (n_elec - 1)
    Wa = 0.25 * (W - W.permute(1, 0, 2, 3) - W.permute(0, 1, 3, 2) + W.permute(1, 0, 3, 2))
    return (V + Wa).contiguous()


class FragmentHamiltonian:
    """H of one fragment on the determinants of one charge sector.

    masks:    determinants (uint64 occupation masks, alpha spin orbitals 0..n_orbs-1, beta
              n_orbs..2 n_orbs-1), all with the same electron count
    h, V:     the fragment's one- and two-electron integrals (spin orbitals, FP64, device or host)
    n_vec:    columns per apply() (the block size of compute_HPsi)."""

    def __init__(self, masks, n_orbs, n_core, h, V, n_vec=1, device="cuda"):
        dev = torch.device(device)
        masks = np.asarray(masks, dtype=np.uint64)
        n_e = {bin(int(m)).count("1") for m in masks}
        if len(n_e) != 1:
            raise ValueError("determinants with different electron counts")
        self.n_elec = n_e.pop()
        self.space = FragmentSpace({0: masks}, n_orbs, n_core, self.n_elec, device=dev, ops=())
        self.n_conf = len(masks)
        self.n_vec = int(n_vec)
        h = torch.as_tensor(h, dtype=torch.float64, device=dev)
        V = torch.as_tensor(V, dtype=torch.float64, device=dev)
        self.sigma = SigmaTwoElectron(self.space, 0, self.n_vec, folded_two_body(h, V, self.n_elec))
        self.zT = torch.zeros((self.n_conf, self.n_vec), dtype=torch.float64, device=dev)

    def apply(self, Psi, out=None):
        """H Psi for Psi (n_vec, n_conf) (rows = CI vectors); returns (n_vec, n_conf)."""
        s = stream_ptr()
        Psi = Psi.contiguous()             # kept alive until the launch is enqueued
        call("xrh_transpose", ptr(Psi), self.n_vec, self.n_conf, ptr(self.zT), s)
        self.sigma.run_sigma(self.zT)
        if out is None:
            return self.sigma.sigmaT
        out.copy_(self.sigma.sigmaT)
        return out

    def matrix(self):
        """The dense FCI matrix (generic_fci): H applied to the unit vectors, n_vec at a time."""
        n = self.n_conf
        H = torch.empty((n, n), dtype=torch.float64, device=self.zT.device)
        E = torch.zeros((self.n_vec, n), dtype=torch.float64, device=self.zT.device)
        for c0 in range(0, n, self.n_vec):
            k = min(self.n_vec, n - c0)
            E.zero_()
            E[torch.arange(k), torch.arange(c0, c0 + k)] = 1.0
            HE = self.apply(E)
            H[c0:c0 + k].copy_(HE[:k])
        return H

    def lowest(self, k=1, m=None, tol=1e-10, max_restarts=50):
        """Lowest k eigenvalues (numpy) and eigenvectors (device, (k, n_conf)) by restarted
        FP64 Lanczos on H Psi (n_vec must be 1): the Krylov depth m (default max(60, 8k),
        at most n_conf) restarts from the lowest Ritz vectors' sum until every one of the k
        Ritz pairs has a residual below tol."""
        if self.n_vec != 1:
            raise ValueError("lowest() applies H to one vector at a time (n_vec = 1)")
        n = self.n_conf
        m = min(n, m or max(60, 8 * k))
        lz = Lanczos(n, m=m, device=self.zT.device, mode="steps")

        def apply(x, y):
            self.sigma.run_sigma(x.view(n, 1))
            y.copy_(self.sigma.sigmaT.view(-1))

        vecs = torch.zeros((k, n), dtype=torch.float64, device=self.zT.device)
        for _ in range(max_restarts):
            lz.krylov_operator(apply)
            lz.stage_to_host()
            torch.cuda.current_stream().synchronize()
            w, Y, resid = lz.ritz(k)
            for i in range(len(w)):
                lz.ritz_vector(Y[:, i], vecs[i])
            if m >= n or np.all(resid <= tol * np.maximum(1.0, np.abs(w))):
                break
            v0 = vecs[:len(w)].sum(0)
            lz.v0.copy_(v0 / v0.norm())
        return w, vecs[:len(w)]


def fci_states(masks, n_orbs, n_core, h, V, n_states, tol=1e-10, device="cuda"):
    """(energies, CI vectors (n_states, n_conf)) of the lowest FCI states of one sector."""
    return FragmentHamiltonian(masks, n_orbs, n_core, h, V, device=device).lowest(n_states, tol=tol)
