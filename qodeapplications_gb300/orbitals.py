"""Orbital transformations of the fragment-blocked integrals on the device.

Replaces the integral re-transformation of the reference's orbital optimizer and its
biorthogonalisation:

* StateSpaceOptimizer/orbital_solver.py:323-413 (transform_ints): the symmetric integrals in
  the new orbitals, every index transformed by the orbital transformation U
  (ket_transformed then bra_transformed with U^T as qode's fragments module applies them),
  then the biorthogonal integrals, the bra indices transformed by S^-1 of the new overlap;
* hermitian-XRCC/get_ints.py:62-66 (direct_Sinv) and :142-143 (bra_transformed(Sinv, ...)).

Here the integrals are supersystem spin-orbital arrays (alpha block then beta block inside
every fragment): S, T (n x n), U (n_frag x n x n), V (n^4), on the device in FP64.  Every index
transformation is one pass of this library's FP64 grouped GEMM kernel:

    pass(X, M):   Y[rest, p] = sum_a X[a, rest] M[a, p]

which transforms the leading index and moves it to the back, so k passes over a k-index
array transform every index once and end in the original index order.  The small matrices
(S^-1, exp(kappa), spin blocking) are one-CTA kernels (csrc/smallmat.cu).

Conventions: X'[p, q, ...] = sum_{a, b, ...} M[a, p] M[b, q] ... X[a, b, ...] for the symmetric
transformation (M = U); the biorthogonal integrals contract S^-1 into the bra indices --
T_b[p, q] = sum_a Sinv[p, a] T[a, q], V_b[p, q, r, s] = sum_ab Sinv[p, a] Sinv[q, b] V[a, b, r, s]
(the first two indices of V_pqrs are the creators, H = sum V_pqrs c+_p c+_q a_s a_r) -- so that
the biorthogonal overlap Sinv S is the identity.
"""
import numpy as np
import torch

from . import _lib
from ._lib import call, ptr, stream_ptr
from .gemm import GroupedGemm
from .synthetic import spin_orbital_spatial_index


def _spin_of(frag_sizes):
    return np.concatenate([np.repeat([0, 1], nf) for nf in frag_sizes]).astype(np.int8)


def _spin_index_tensors(frag_sizes, device):
    """(spatial index int32, spin int8) device arrays of the spin orbitals.  The caller keeps
    both alive until the launch that reads them is enqueued: a temporary freed before the
    call returns its block to the caching allocator, and the next allocation may take it."""
    sidx = spin_orbital_spatial_index(frag_sizes)
    return (torch.as_tensor(np.array(sidx, dtype=np.int32), device=device),
            torch.as_tensor(_spin_of(frag_sizes), device=device))


def _spin_block(src, ld_src, frag_sizes, out):
    """out = spin-orbital form of the spatial matrix src (xrh_spin_block)."""
    sidx_t, spin_t = _spin_index_tensors(frag_sizes, src.device)
    call("xrh_spin_block", sidx_t.numel(), ptr(sidx_t), ptr(spin_t), ptr(src), ld_src, ptr(out), out.shape[1],
         stream_ptr())
    return out


def _pass(X, n, M, out):
    """out[rest, p] = sum_a X[a, rest] M[a, p] with X of n * rest elements (one GEMM)."""
    rest = X.numel() // n
    g = GroupedGemm(X.device)
    # A = X stored [k = a][m = rest] (flag bit 0), B = M stored [k = a][n = p] (flag bit 1)
    g.add(rest, n, [(X, rest, M, n, n, 1.0, 3, 0, 0)], out, n, mode=0)
    g.finalize().run()
    return out


def transform_indices(X, mats):
    """Every index of the n^k array X transformed by its matrix (mats[i] for index i, None
    for the identity): X'[p, q, ...] = sum M0[a, p] M1[b, q] ... X[a, b, ...]."""
    n = X.shape[0]
    dev = X.device
    eye = None
    cur = X.contiguous()
    for M in mats:
        if M is None:
            if eye is None:
                eye = torch.eye(n, dtype=torch.float64, device=dev)
            M = eye
        nxt = torch.empty_like(cur)
        _pass(cur, n, M.contiguous(), nxt)
        cur = nxt.view(cur.shape)
    return cur


def transform_integrals(M, ints):
    """The integrals {S, T, U, V} (any subset) in the orbitals transformed by M (n x n):
    every index transformed (the symmetric integrals of orbital_solver.transform_ints)."""
    out = {}
    for key, X in ints.items():
        if X is None:
            out[key] = None
        elif key == "U":
            out[key] = torch.stack([transform_indices(X[k], [M, M]) for k in range(X.shape[0])])
        else:
            out[key] = transform_indices(X, [M] * X.dim())
    return out


def inverse_spin_free(S, frag_sizes):
    """S^-1 of a spin-free spin-orbital overlap (alpha and beta blocks equal, no alpha-beta
    coupling): the inverse of its alpha-alpha block (spatial, <= 64 orbitals), spin-blocked."""
    dev = S.device
    sidx = spin_orbital_spatial_index(frag_sizes)
    spin = _spin_of(frag_sizes)
    n_sp = sum(frag_sizes)
    alpha = torch.as_tensor(np.array([a for a in range(len(sidx)) if spin[a] == 0], dtype=np.int32), device=dev)
    # order the alpha spin orbitals by their spatial index
    order = np.argsort([sidx[a] for a in alpha.cpu().numpy()])
    alpha = alpha[torch.as_tensor(order, device=dev)].contiguous()
    s_sp = torch.empty((n_sp, n_sp), dtype=torch.float64, device=dev)
    inv_sp = torch.empty_like(s_sp)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    s = stream_ptr()
    call("xrh_gather_submatrix", n_sp, ptr(alpha), ptr(S), S.shape[1], ptr(s_sp), n_sp, s)
    call("xrh_inverse_small", n_sp, ptr(s_sp), n_sp, ptr(inv_sp), n_sp, ptr(status), s)
    out = _spin_block(inv_sp, n_sp, frag_sizes, torch.empty_like(S))
    if int(status.item()) != 0:
        raise _lib.XRHError("overlap matrix is singular")
    return out


def biorthogonal_integrals(symm, frag_sizes):
    """The biorthogonal integrals from the symmetric ones (get_ints.py:62-66,142-143): S^-1
    of symm['S'] contracted into the bra indices of T, U and V.  Returns a dict with S (the
    biorthogonal overlap, the identity up to rounding), T, U, V and Sinv."""
    Sinv = inverse_spin_free(symm["S"], frag_sizes)
    SinvT = Sinv.t().contiguous()        # pass matrix: M[a, p] = Sinv[p, a]
    out = {"Sinv": Sinv}
    out["S"] = transform_indices(symm["S"], [SinvT, None])
    out["T"] = transform_indices(symm["T"], [SinvT, None])
    if symm.get("U") is not None:
        out["U"] = torch.stack([transform_indices(symm["U"][k], [SinvT, None]) for k in range(symm["U"].shape[0])])
    out["V"] = transform_indices(symm["V"], [SinvT, SinvT, None, None])
    return out


def rotation_matrix(kappa, frag_sizes):
    """Spin-orbital R = exp(kappa) for antisymmetric spatial kappa (the same rotation for both
    spins), computed by xrh_expm_small and spin-blocked by xrh_spin_block."""
    kappa = kappa.contiguous()
    dev = kappa.device
    n_sp = kappa.shape[0]
    R_sp = torch.empty_like(kappa)
    s = stream_ptr()
    call("xrh_expm_small", n_sp, ptr(kappa), n_sp, ptr(R_sp), n_sp, s)
    n_so = 2 * sum(frag_sizes)
    return _spin_block(R_sp, n_sp, frag_sizes, torch.empty((n_so, n_so), dtype=torch.float64, device=dev))


def transform_ints(U_sp, ints, frag_sizes):
    """orbital_solver.transform_ints (StateSpaceOptimizer/orbital_solver.py:323-413) for
    supersystem arrays: U_sp is the spatial orbital transformation (n_sp x n_sp, e.g. the
    first-order I + s x of :431 or exp(kappa)), ints a dict {S, T, U, V} of spin-orbital
    arrays.  Returns (symmetric, biorthogonal) integral dicts."""
    dev = ints["T"].device
    n_so = 2 * sum(frag_sizes)
    Usp = torch.as_tensor(U_sp, dtype=torch.float64, device=dev).contiguous()
    M = _spin_block(Usp, Usp.shape[0], frag_sizes, torch.empty((n_so, n_so), dtype=torch.float64, device=dev))
    symm = transform_integrals(M, ints)
    bior = biorthogonal_integrals(symm, frag_sizes)
    return symm, bior
