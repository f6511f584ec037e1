"""Order-0 diagram catalogs with the reference's catalog interface, evaluated on the device.

The reference keeps one catalog module per integral family (hermitian-XRCC/diagrams/
ST_diagrams.py:28-64, SU_diagrams.py:28-94, SV_diagrams.py:28-103):

    catalog[frag_order][label] = build_diagram(body, Dchgs=..., permutations=[(phase, perm), ...])

and diagrammatic_expansion.blocks looks labels up there.  The objects ST_diagrams,
SU_diagrams and SV_diagrams below have the same .catalog[frag_order][label] structure for the
order-0 labels of get_xr_result.py:86-132 (monomers t00, u000, v0000; dimers t01, u100, u001,
u101, v0101, v0001, v0100, v0011), with the reference's charge changes (Dchgs), permutations
and phases.  Each body is the reference's two-step contraction (precontraction with the
integral block, precontract.py:75, then the contraction with the second fragment's density)
run by this library's FP64 grouped GEMM kernel; the prefactors and parities are those of
SV_2mer_0.py:25-67, ST_2mer_0.py:25-34, SU_2mer_0.py:37-118 and the monomer bodies
(ST_1mer_0.py:24, SU_1mer_0.py:24, SV_1mer_0.py:24).  The S-dressed labels of XR orders 1
and 2 (s01..., S_diagrams.py) are not in these catalogs: looking them up raises
NotImplementedError as the reference does for a label it lacks.
"""
import torch

from .gemm import GroupedGemm


def _gemm(A, W, M, x, K, alpha=1.0):
    """C[M, x] = alpha * A[M, K] W[x, K]^T on the device (one FP64 grouped-GEMM task)."""
    C = torch.zeros((M, x), dtype=torch.float64, device=A.device)
    g = GroupedGemm(A.device)
    g.add(M, x, [(A.contiguous(), K, W.contiguous(), K, K, float(alpha))], C, x, mode=0)
    g.finalize().run()
    return C


class Term:
    """One evaluated permutation: body(X) with the fragments and charges of the permutation."""

    def __init__(self, body, X):
        self.body, self.X = body, X

    def __call__(self, contract_last=False, special_processing=None):
        if contract_last or special_processing is not None:
            raise NotImplementedError("bra_det / ket_det evaluations (contract_last) are not provided")
        return self.body(self.X)


class Resolved:
    """What a body needs of one permutation (the role of frag_resolve, build_diagram.py:81-134):
    the densities and integrals of fragments A = '0', B = '1', their charge pairs, the state
    counts and the ket parity n_j0 of the unpermuted first fragment (:88-92)."""

    def __init__(self, info, frags, charges, n_j0):
        self.rho, self.ints = info["rho"], info["integrals"]
        self.frags, self.charges, self.n_j0 = frags, charges, n_j0
        self.N = [info["N"][f] for f in frags]

    def dens(self, k, op):
        return self.rho[self.frags[k]][op].get(tuple(self.charges[k]))

    def n(self, k):
        bc, kc = self.charges[k]
        rho = self.rho[self.frags[k]]
        return rho["ns"][bc], rho["ns"][kc]


def _blk(arr):
    return torch.as_tensor(arr, dtype=torch.float64)


def _int_block(X, kind, *idx):
    f = X.frags
    src = getattr(X.ints, kind)
    t = src[tuple(f[i] for i in idx)]
    return (t if isinstance(t, torch.Tensor) else _blk(t)).to(X.rho_device)


# ------------------------------------------------------------------------------ monomers --
def _monomer(op, kind, idx, weight_perm=None):
    def body(X):
        r = X.dens(0, op)
        if r is None:
            return None
        ni, nj = X.n(0)
        N = X.N[0]
        w = _int_block(X, kind, *idx)
        if weight_perm is not None:
            w = w.permute(*weight_perm)
        k = N ** len(op)
        return _gemm(r.reshape(ni * nj, k), w.reshape(1, k), ni * nj, 1, k).view(ni, nj)
    return body


# -------------------------------------------------------------------------------- dimers --
def _dimer(op0, op1, kind, idx, weight_perm, ext0, ext1, prefactor):
    """out[i0, i1, j0, j1] = prefactor(n_j0) sum P[(i0 j0), y] rho1[(i1 j1), y],
    P[(i0 j0), y] = sum_x rho0[(i0 j0), x] W[y, x],  W = integral.permute(weight_perm)."""
    def body(X):
        r0, r1 = X.dens(0, op0), X.dens(1, op1)
        if r0 is None or r1 is None:
            return None
        ni0, nj0 = X.n(0)
        ni1, nj1 = X.n(1)
        k0, k1 = X.N[0] ** ext0, X.N[1] ** ext1
        W = _int_block(X, kind, *idx).permute(*weight_perm).reshape(k1, k0)
        P = _gemm(r0.reshape(ni0 * nj0, k0), W, ni0 * nj0, k1, k0)
        out = _gemm(P, r1.reshape(ni1 * nj1, k1), ni0 * nj0, ni1 * nj1, k1, prefactor(X.n_j0))
        return out.view(ni0, nj0, ni1, nj1).permute(0, 2, 1, 3)
    return body


def _u100(X):
    """delta(i1, j1) ca0pq_U1pq(i0, j0) (SU_2mer_0.py:37)."""
    r0 = X.dens(0, "ca")
    if r0 is None:
        return None
    ni0, nj0 = X.n(0)
    ni1, nj1 = X.n(1)
    N = X.N[0]
    w = _int_block(X, "U", 1, 0, 0).reshape(1, N * N)
    P = _gemm(r0.reshape(ni0 * nj0, N * N), w, ni0 * nj0, 1, N * N).view(ni0, nj0)
    out = torch.zeros((ni0, ni1, nj0, nj1), dtype=torch.float64, device=P.device)
    for i in range(min(ni1, nj1)):
        out[:, i, :, i] = P
    return out


class build_diagram:
    """catalog entry: body, the charge changes it applies to and its (phase, permutation)s."""

    def __init__(self, body, Dchgs, permutations):
        self.body, self.Dchgs, self.permutations = body, tuple(Dchgs), list(permutations)

    def __call__(self, info, subsys_charges):
        frags = tuple(f for f, _ in subsys_charges)
        chgs = tuple(tuple(c) for _, c in subsys_charges)
        n_j0 = info["rho"][frags[0]]["n_elec"][chgs[0][1]] % 2
        terms = []
        for phase, perm in self.permutations:
            pf = tuple(frags[k] for k in perm)
            pc = tuple(chgs[k] for k in perm)
            if not all(pc[k][0] - pc[k][1] == self.Dchgs[k] for k in range(len(perm))):
                terms.append(None)
                continue
            X = Resolved(info, pf, pc, n_j0)
            X.rho_device = info["device"]
            terms.append((_Phased(Term(self.body, X), phase), perm))
        return terms


class _Phased:
    def __init__(self, term, phase):
        self.term, self.phase = term, phase

    def __call__(self, **kw):
        r = self.term(**kw)
        return None if r is None else self.phase * r


def _sgn(p):
    return lambda n_j0: float((-1) ** ((n_j0 + p) % 2))


class _Catalog:
    def __init__(self, catalog):
        self.catalog = catalog


ST_diagrams = _Catalog({
    1: {"t00": build_diagram(_monomer("ca", "T", (0, 0)), (0,), [(+1, (0,))])},
    2: {"t01": build_diagram(_dimer("c", "a", "T", (0, 1), (1, 0), 1, 1, _sgn(0)), (-1, +1),
                             [(+1, (0, 1)), (-1, (1, 0))])},
})
SU_diagrams = _Catalog({
    1: {"u000": build_diagram(_monomer("ca", "U", (0, 0, 0)), (0,), [(+1, (0,))])},
    2: {"u100": build_diagram(_u100, (0, 0), [(+1, (0, 1)), (+1, (1, 0))]),
        "u001": build_diagram(_dimer("c", "a", "U", (0, 0, 1), (1, 0), 1, 1, _sgn(0)), (-1, +1),
                              [(+1, (0, 1)), (-1, (1, 0))]),
        "u101": build_diagram(_dimer("c", "a", "U", (1, 0, 1), (1, 0), 1, 1, _sgn(0)), (-1, +1),
                              [(+1, (0, 1)), (-1, (1, 0))])},
})
SV_diagrams = _Catalog({
    1: {"v0000": build_diagram(_monomer("ccaa", "V", (0, 0, 0, 0), weight_perm=(0, 1, 3, 2)), (0,), [(+1, (0,))])},
    2: {"v0101": build_diagram(_dimer("ca", "ca", "V", (0, 1, 0, 1), (1, 3, 0, 2), 2, 2, lambda n: 4.0), (0, 0),
                               [(+1, (0, 1))]),
        "v0001": build_diagram(_dimer("cca", "a", "V", (0, 0, 0, 1), (3, 0, 1, 2), 3, 1,
                                      lambda n: 2.0 * (-1) ** ((n + 1) % 2)), (-1, +1), [(+1, (0, 1)), (-1, (1, 0))]),
        "v0100": build_diagram(_dimer("caa", "c", "V", (0, 1, 0, 0), (1, 0, 3, 2), 3, 1,
                                      lambda n: 2.0 * (-1) ** (n % 2)), (+1, -1), [(+1, (0, 1)), (-1, (1, 0))]),
        "v0011": build_diagram(_dimer("cc", "aa", "V", (0, 0, 1, 1), (3, 2, 0, 1), 2, 2, lambda n: 1.0), (-2, +2),
                               [(+1, (0, 1)), (+1, (1, 0))])},
})
