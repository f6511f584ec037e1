"""FP64 NumPy oracle for the excitonic-Hamiltonian (XR-H) build.

TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
leg import this module, and only as the checker (or the timed CPU reference).  The product
path (qodeapplications_gb300) never imports it.

It restates, in plain NumPy and in the reference's own contraction order, the algorithms of:

* general-XRCC/density_tensors.c (fragment transition densities from CI vectors):
  operator application with fermionic parity  (annihilate :80-95, create :97-113),
  frozen-core filter (all_core_occupied :125-134), configuration lookup
  (find_config_index :49-62), accumulation  rho_IJ[idx] += sign z_I[P] z_J[Q]
  (z_contract :142-154) and the operator loops a/c/ca/aa/cc/caa/cca/ccaa (:162-556).
* general-XRCC/build_density_tensors.py:57-160 (which op string for which charge change,
  ccaa folded into a scalar with V, :129-133).
* general-XRCC/H_contractions.c + build_H.py:37-188 (element formulas, charge cases, signs).
* hermitian-XRCC order-0 diagrams: monomer t00/u000/v0000 (diagrams/ST_1mer_0.py:24,
  SU_1mer_0.py:24, SV_1mer_0.py:24), dimer t01 (ST_2mer_0.py:25), u100/u001/u101
  (SU_2mer_0.py:37-118), v0101/v0001/v0100/v0011 (SV_2mer_0.py:25-67); catalog phases and
  permutations (ST_diagrams.py:33-35, SU_diagrams.py:33-37, SV_diagrams.py:33-38); the ket
  parity n_j0 of the UNPERMUTED first fragment (diagrams/build_diagram.py:88-92);
  precontraction label grammar (precontract.py:32-80); block assembly and transposition
  (diagrammatic_expansion.py:27-59, XR_term.py:22-165); charge-blocked -> product-state
  permutation (get_xr_result.py:300-353); full H and eigensolve (mains/workflow.py:214-230).
* A brute-force supersystem FCI in the same sign convention (known-answer test: with
  complete fragment state sets the order-0 XR Hamiltonian equals the FCI Hamiltonian).

Parity anchors: the compiled reference C kernels (oracle/_ref, via oracle/ref_ctypes.py)
pin the density builder and the element formulas; the FCI identity pins the hermitian
diagram signs (the hermitian-XRCC Python path itself needs the absent Qode library).
"""
import itertools
import math

import numpy as np
import scipy.sparse as sp

# ----------------------------------------------------------------------------------------
# bit utilities
# ----------------------------------------------------------------------------------------

if hasattr(np, "bitwise_count"):
    def popcount(x):
        return np.bitwise_count(np.asarray(x, dtype=np.uint64)).astype(np.int64)
else:  # pragma: no cover - numpy < 2.0
    _PC8 = np.array([bin(i).count("1") for i in range(256)], dtype=np.int64)

    def popcount(x):
        x = np.asarray(x, dtype=np.uint64)
        return _PC8[x.view(np.uint8).reshape(x.shape + (8,))].sum(-1)


OP_DCHG = {"a": +1, "c": -1, "ca": 0, "aa": +2, "cc": -2, "caa": +1, "cca": -1, "ccaa": 0}
# op strings per (bra_chg - ket_chg), general-XRCC/build_density_tensors.py:90-157
OPS_FOR_DCHG = {+2: ("aa",), +1: ("a", "caa"), 0: ("ca", "ccaa"), -1: ("c", "cca"), -2: ("cc",)}


def valence_orbitals(n_orbs, n_core):
    """Spin-orbital indices of the valence space (alpha block then beta block)."""
    return [o for o in range(2 * n_orbs) if not (o < n_core or n_orbs <= o < n_orbs + n_core)]


def core_mask(n_orbs, n_core):
    m = 0
    for i in range(n_core):
        m |= (1 << i) | (1 << (n_orbs + i))
    return m


def all_configs(n_orbs, n_core, n_elec, sz2=None):
    """All determinants with n_elec electrons and a filled frozen core, in the lexicographic
    valence order that find_valence_config_index (density_tensors.c:29-47) ranks by.
    sz2: optional filter on 2*Sz = n_alpha - n_beta.  Returns uint64 masks."""
    val = valence_orbitals(n_orbs, n_core)
    cm = core_mask(n_orbs, n_core)
    k = n_elec - 2 * n_core
    out = []
    for comb in itertools.combinations(range(len(val)), k):
        m = cm
        for v in comb:
            m |= 1 << val[v]
        if sz2 is not None:
            na = bin(m & ((1 << n_orbs) - 1)).count("1")
            nb = bin(m >> n_orbs).count("1")
            if na - nb != sz2:
                continue
        out.append(m)
    return np.array(out, dtype=np.uint64)


def masks_to_occ(masks, N):
    masks = [int(m) for m in masks]
    n_e = bin(masks[0]).count("1") if masks else 0
    occ = np.zeros((len(masks), n_e), dtype=np.int64)
    for i, m in enumerate(masks):
        occ[i] = [o for o in range(N) if (m >> o) & 1]
    return occ


# ----------------------------------------------------------------------------------------
# density builder (density_tensors.c restated with bit masks)
# ----------------------------------------------------------------------------------------

def coupling_list(op, ket_masks, bra_masks, N, n_orbs, n_core):
    """Nonzero couplings <P| op_{idx} |Q> = sign for one op string.

    Operators are applied right to left (the last letter acts first), each with parity
    (-1)^(number of occupied spin orbitals above it) as in annihilate/create
    (density_tensors.c:80-113); the result must keep the frozen core filled
    (:125-134) and be one of the bra configurations.  idx is the row-major flat index of the
    operator indices in op-string order (density_tensors.c:272,319,420,480,543).
    Returns int64 arrays idx, P, Q and sign."""
    ket_masks = np.asarray(ket_masks, dtype=np.uint64)
    k = len(op)
    masks = ket_masks.copy()
    Q = np.arange(len(ket_masks), dtype=np.int64)
    idx = np.zeros(len(ket_masks), dtype=np.int64)
    sign = np.ones(len(ket_masks), dtype=np.int64)
    orbs = np.arange(N, dtype=np.uint64)
    for pos in range(k - 1, -1, -1):
        kind = op[pos]
        bit = (np.uint64(1) << orbs)[None, :]
        occ = (masks[:, None] & bit) != 0
        valid = occ if kind == "a" else ~occ
        r, o = np.nonzero(valid)
        m = masks[r]
        above = popcount(m >> (orbs[o] + np.uint64(1)))
        sign = sign[r] * np.where(above % 2 == 1, -1, 1)
        masks = m ^ (np.uint64(1) << orbs[o])
        Q = Q[r]
        idx = idx[r] + o.astype(np.int64) * N ** (k - 1 - pos)
    cm = np.uint64(core_mask(n_orbs, n_core))
    keep = (masks & cm) == cm
    masks, Q, idx, sign = masks[keep], Q[keep], idx[keep], sign[keep]
    bra_masks = np.asarray(bra_masks, dtype=np.uint64)
    order = np.argsort(bra_masks, kind="stable")
    sorted_b = bra_masks[order]
    pos = np.searchsorted(sorted_b, masks)
    pos_c = np.minimum(pos, max(len(sorted_b) - 1, 0))
    found = (len(sorted_b) > 0) & (sorted_b[pos_c] == masks) if len(sorted_b) else np.zeros(len(masks), bool)
    P = order[pos_c[found]] if len(sorted_b) else np.zeros(0, np.int64)
    return idx[found], P.astype(np.int64), Q[found], sign[found]


def transition_density(op, zb, bra_masks, zk, ket_masks, N, n_orbs, n_core, chunk=200000):
    """rho[I,J,idx] = sum_couplings sign z_I[P] z_J[Q] (z_contract, density_tensors.c:142-154).
    Returns ndarray (n_bra, n_ket, N, ..., N)."""
    zb = np.asarray(zb, dtype=np.float64)
    zk = np.asarray(zk, dtype=np.float64)
    k = len(op)
    nb, nk = zb.shape[0], zk.shape[0]
    idx, P, Q, s = coupling_list(op, ket_masks, bra_masks, N, n_orbs, n_core)
    out = np.zeros((N ** k, nb * nk))
    for c0 in range(0, len(idx), chunk):
        sl = slice(c0, c0 + chunk)
        n = len(idx[sl])
        K = (zb[:, P[sl]].T * s[sl][:, None])[:, :, None] * zk[:, Q[sl]].T[:, None, :]
        S = sp.csr_matrix((np.ones(n), (idx[sl], np.arange(n))), shape=(N ** k, n))
        out += S @ K.reshape(n, nb * nk)
    return out.T.reshape((nb, nk) + (N,) * k)


class Sector:
    """States of one fragment in one charge sector: coeffs (n_states, n_conf), masks (n_conf,)."""

    def __init__(self, coeffs, masks):
        self.coeffs = np.asarray(coeffs, dtype=np.float64)
        self.masks = np.asarray(masks, dtype=np.uint64)
        self.n_elec = bin(int(self.masks[0])).count("1") if len(self.masks) else 0


def build_densities(sectors, n_orbs, n_core, n_elec_ref, bra_coeffs=None, ops=None):
    """Per-fragment density dictionary in the layout of the hermitian-XRCC path
    (Be-states/densities.py:167-231): rho[op][(bra_chg, ket_chg)] -> (n_bra, n_ket, N...),
    plus 'n_elec', 'n_states', 'n_states_bra'.  bra_coeffs optionally replaces the bra
    coefficient sets per charge (e.g. identity for the determinant-bra densities that
    state_gradients.py:170 requests with 'bra_det')."""
    N = 2 * n_orbs
    dens = {op: {} for op in OP_DCHG}
    for bc, bsec in sectors.items():
        zb = bsec.coeffs if bra_coeffs is None else bra_coeffs[bc]
        for kc, ksec in sectors.items():
            d = bc - kc
            for op in OPS_FOR_DCHG.get(d, ()):
                if ops is not None and op not in ops:
                    continue
                dens[op][(bc, kc)] = transition_density(op, zb, bsec.masks, ksec.coeffs, ksec.masks,
                                                        N, n_orbs, n_core)
    dens["n_elec"] = {c: n_elec_ref - c for c in sectors}
    dens["n_states"] = {c: s.coeffs.shape[0] for c, s in sectors.items()}
    dens["n_states_bra"] = ({c: bra_coeffs[c].shape[0] for c in sectors} if bra_coeffs is not None
                            else dict(dens["n_states"]))
    return dens


# ----------------------------------------------------------------------------------------
# fragment-blocked integrals
# ----------------------------------------------------------------------------------------

class FragInts:
    """Supersystem spin-orbital integrals, indexable by fragment tuples like qode's
    fragment-blocked integrals (hermitian-XRCC/get_ints.py:116-155):
    T[m,n] (N_m x N_n), U[k,m,n] (nuclei of fragment k), V[m,n,o,p], S[m,n].
    H = sum h_pq c+_p a_q + sum V_pqrs c+_p c+_q a_s a_r,  h = T + sum_k U_k."""

    def __init__(self, h, V, Ns, U=None):
        self.h = np.asarray(h, dtype=np.float64)
        self.Vfull = np.asarray(V, dtype=np.float64)
        self.Ns = list(Ns)
        self.off = np.concatenate([[0], np.cumsum(self.Ns)]).astype(int)
        n_f = len(self.Ns)
        tot = self.off[-1]
        self.Ufull = np.zeros((n_f, tot, tot)) if U is None else np.asarray(U, dtype=np.float64)
        outer = self

        class _Blk:
            def __init__(self, arr, lead=0):
                self.arr, self.lead = arr, lead

            def __getitem__(self, key):
                key = key if isinstance(key, tuple) else (key,)
                lead = key[:self.lead]
                sl = tuple(slice(outer.off[m], outer.off[m + 1]) for m in key[self.lead:])
                return self.arr[lead + sl]

        self.T = _Blk(self.h - self.Ufull.sum(0))
        self.U = _Blk(self.Ufull, lead=1)
        self.V = _Blk(self.Vfull)
        self.S = _Blk(np.eye(tot))

    def h_total(self):
        return self.h


# ----------------------------------------------------------------------------------------
# hermitian-XRCC order-0 diagrams
# ----------------------------------------------------------------------------------------

def monomer_block(dens_m, ints, m, ci, cj):
    """t00 + u000 + v0000 for one charge block (ci == cj only; Dchgs=(0,)).
    t00: sum_pq rho^ca[i,j,p,q] T[m,m][p,q]          (ST_1mer_0.py:24, label ca0pq_Tpq)
    u000: sum_pq rho^ca[i,j,p,q] U[m,m,m][p,q]       (SU_1mer_0.py:24, label ca0pq_U0pq)
    v0000: sum_pqrs rho^ccaa[i,j,p,q,s,r] V_mmmm[pqrs] (SV_1mer_0.py:24, label ccaa0pqsr_Vpqrs)"""
    if ci != cj:
        return None
    ca = dens_m["ca"][(ci, cj)]
    ccaa = dens_m["ccaa"][(ci, cj)]
    out = np.einsum("ijpq,pq->ij", ca, ints.T[m, m])
    out += np.einsum("ijpq,pq->ij", ca, ints.U[m, m, m])
    out += np.einsum("ijpqsr,pqrs->ij", ccaa, ints.V[m, m, m, m])
    return out


def monomer_matrix(dens_m, ints, m, charges):
    """XR_term.monomer_matrix (XR_term.py:96-115) for t00+u000+v0000."""
    nb = [dens_m["n_states_bra"][c] for c in charges]
    nk = [dens_m["n_states"][c] for c in charges]
    H = np.zeros((sum(nb), sum(nk)))
    ib = 0
    for a, ci in enumerate(charges):
        jb = 0
        for b, cj in enumerate(charges):
            blk = monomer_block(dens_m, ints, m, ci, cj)
            if blk is not None:
                H[ib:ib + nb[a], jb:jb + nk[b]] += blk
            jb += nk[b]
        ib += nb[a]
    return H


# (label, Dchgs, [(phase, permutation)]) for the order-0 dimer catalogs
DIMER_CATALOG_0 = [
    ("t01", (-1, +1), [(+1, (0, 1)), (-1, (1, 0))]),
    ("u100", (0, 0), [(+1, (0, 1)), (+1, (1, 0))]),
    ("u001", (-1, +1), [(+1, (0, 1)), (-1, (1, 0))]),
    ("u101", (-1, +1), [(+1, (0, 1)), (-1, (1, 0))]),
    ("v0101", (0, 0), [(+1, (0, 1))]),
    ("v0001", (-1, +1), [(+1, (0, 1)), (-1, (1, 0))]),
    ("v0100", (+1, -1), [(+1, (0, 1)), (-1, (1, 0))]),
    ("v0011", (-2, +2), [(+1, (0, 1)), (+1, (1, 0))]),
]
DIMER_ORDER0_LISTS = {"T": ["t01"], "U": ["u100", "u001", "u101"], "V": ["v0101", "v0001", "v0100", "v0011"]}


def dimer_diagram(label, dens, ints, frags, chgs, n_j0):
    """One order-0 dimer diagram body in the relative frame: fragment 'A' = frags[0]
    plays the reference's '0', 'B' = frags[1] plays '1'.  chgs = ((ciA,cjA),(ciB,cjB)).
    Returns (iA, iB, jA, jB) or None.  Each term follows the reference's two-step order:
    precontraction with the integral (precontract.py:75) then the final contraction."""
    A, B = frags
    (ciA, cjA), (ciB, cjB) = chgs
    dA, dB = dens[A], dens[B]

    def rho(dd, op, key):
        return dd[op].get(key)

    kA, kB = (ciA, cjA), (ciB, cjB)
    if label == "t01":      # (-1)^{n_j0} c0p_Tp1(i0,j0,q) a1(i1,j1,q)
        c0, a1 = rho(dA, "c", kA), rho(dB, "a", kB)
        P = np.einsum("ijp,pq->ijq", c0, ints.T[A, B])
        return (-1) ** n_j0 * np.einsum("ikq,jlq->ijkl", P, a1)
    if label == "u001":     # (-1)^{n_j0} c0p_U0p1(i0,j0,q) a1(i1,j1,q)
        c0, a1 = rho(dA, "c", kA), rho(dB, "a", kB)
        P = np.einsum("ijp,pq->ijq", c0, ints.U[A, A, B])
        return (-1) ** n_j0 * np.einsum("ikq,jlq->ijkl", P, a1)
    if label == "u101":     # (-1)^{n_j0} c0p_U1p1(i0,j0,q) a1(i1,j1,q)
        c0, a1 = rho(dA, "c", kA), rho(dB, "a", kB)
        P = np.einsum("ijp,pq->ijq", c0, ints.U[B, A, B])
        return (-1) ** n_j0 * np.einsum("ikq,jlq->ijkl", P, a1)
    if label == "u100":     # delta(i1,j1) ca0pq_U1pq(i0,j0)
        ca0 = rho(dA, "ca", kA)
        P = np.einsum("ijpq,pq->ij", ca0, ints.U[B, A, A])
        n1i = dB["n_states_bra"][ciB]
        n1j = dB["n_states"][cjB]
        out = np.zeros((P.shape[0], n1i, P.shape[1], n1j))
        for i1 in range(min(n1i, n1j)):
            out[:, i1, :, i1] = P
        return out
    if label == "v0101":    # 4 ca0pr_Vp1r1(i0,j0,q,s) ca1(i1,j1,q,s)
        ca0, ca1 = rho(dA, "ca", kA), rho(dB, "ca", kB)
        P = np.einsum("ijpr,pqrs->ijqs", ca0, ints.V[A, B, A, B])
        return 4 * np.einsum("ikqs,jlqs->ijkl", P, ca1)
    if label == "v0001":    # 2 (-1)^{n_j0+1} cca0pqr_Vpqr1(i0,j0,s) a1(i1,j1,s)
        cca0, a1 = rho(dA, "cca", kA), rho(dB, "a", kB)
        P = np.einsum("ijpqr,pqrs->ijs", cca0, ints.V[A, A, A, B])
        return 2 * (-1) ** (n_j0 + 1) * np.einsum("iks,jls->ijkl", P, a1)
    if label == "v0100":    # 2 (-1)^{n_j0} caa0psr_Vp1rs(i0,j0,q) c1(i1,j1,q)
        caa0, c1 = rho(dA, "caa", kA), rho(dB, "c", kB)
        P = np.einsum("ijpsr,pqrs->ijq", caa0, ints.V[A, B, A, A])
        return 2 * (-1) ** n_j0 * np.einsum("ikq,jlq->ijkl", P, c1)
    if label == "v0011":    # cc0pq_Vpq11(i0,j0,r,s) aa1(i1,j1,s,r)
        cc0, aa1 = rho(dA, "cc", kA), rho(dB, "aa", kB)
        P = np.einsum("ijpq,pqrs->ijrs", cc0, ints.V[A, A, B, B])
        return np.einsum("ikrs,jlsr->ijkl", P, aa1)
    raise NotImplementedError(f"diagram '{label}' not implemented for 2 bodies")


def dimer_charge_block(dens, ints, frags, chg_pairs, labels):
    """Sum of the listed diagrams for one dimer charge block, all permutations, transposed to
    (i0,i1,j0,j1) (diagrammatic_expansion.py:27-59,76-93).  chg_pairs = ((ci0,cj0),(ci1,cj1))
    for the fragments frags (ascending).  Returns ndarray or None."""
    n_j0 = dens[frags[0]]["n_elec"][chg_pairs[0][1]] % 2      # unpermuted first fragment
    total = None
    cat = {lab: (dch, perms) for lab, dch, perms in DIMER_CATALOG_0}
    for lab in labels:
        dchgs, perms = cat[lab]
        for phase, perm in perms:
            pf = tuple(frags[k] for k in perm)
            pc = tuple(chg_pairs[k] for k in perm)
            if not all(pc[k][0] - pc[k][1] == dchgs[k] for k in range(2)):
                continue
            blk = dimer_diagram(lab, dens, ints, pf, pc, n_j0)
            if blk is None:
                continue
            reorder = list(perm) + [2 + p for p in perm]
            blk = phase * blk.transpose(reorder)
            total = blk if total is None else total + blk
    return total


def dimer_matrix(dens, ints, frags, charge_blocks, labels):
    """XR_term.dimer_matrix (XR_term.py:117-165) in charge-blocked order."""
    d0, d1 = dens[frags[0]], dens[frags[1]]
    nb = [d0["n_states_bra"][c0] * d1["n_states_bra"][c1] for c0, c1 in charge_blocks]
    nk = [d0["n_states"][c0] * d1["n_states"][c1] for c0, c1 in charge_blocks]
    M = np.zeros((sum(nb), sum(nk)))
    ib = 0
    for a, (ci0, ci1) in enumerate(charge_blocks):
        jb = 0
        for b, (cj0, cj1) in enumerate(charge_blocks):
            if ci0 + ci1 == cj0 + cj1:
                blk = dimer_charge_block(dens, ints, frags, ((ci0, cj0), (ci1, cj1)), labels)
                if blk is not None:
                    M[ib:ib + nb[a], jb:jb + nk[b]] += blk.reshape(nb[a], nk[b])
            jb += nk[b]
        ib += nb[a]
    return M


def product_order_map(n0_list, n1_list):
    """mapping[product index] = charge-blocked index (get_xr_result.py:300-340)."""
    tot0, tot1 = sum(n0_list), sum(n1_list)
    m2 = np.zeros((tot0, tot1), dtype=np.int64)
    idx, b0 = 0, 0
    for d0 in n0_list:
        b1 = 0
        for d1 in n1_list:
            for m in range(d0):
                for n in range(d1):
                    m2[b0 + m, b1 + n] = idx
                    idx += 1
            b1 += d1
        b0 += d0
    return m2.reshape(-1)


def get_xr_H0(ints, dens, monomer_charges):
    """Order-0 get_xr_H (get_xr_result.py:86-132 + :300-355) with S = 1 integrals
    (symmetric == biorthogonal).  Returns (H1 list, H2 in product-state order)."""
    H1 = [monomer_matrix(dens[m], ints, m, monomer_charges[m]) for m in (0, 1)]
    charge_blocks = [(c0, c1) for c0 in monomer_charges[0] for c1 in monomer_charges[1]]
    labels = DIMER_ORDER0_LISTS["T"] + DIMER_ORDER0_LISTS["U"] + DIMER_ORDER0_LISTS["V"]
    H2b = dimer_matrix(dens, ints, (0, 1), charge_blocks, labels)
    mb = product_order_map([dens[0]["n_states_bra"][c] for c in monomer_charges[0]],
                           [dens[1]["n_states_bra"][c] for c in monomer_charges[1]])
    mk = product_order_map([dens[0]["n_states"][c] for c in monomer_charges[0]],
                           [dens[1]["n_states"][c] for c in monomer_charges[1]])
    return H1, H2b[np.ix_(mb, mk)]


def full_H(H1, H2):
    """full = H2 + H1[0] x 1 + 1 x H1[1] (mains/workflow.py:216-230; H1 is charge-block
    diagonal, so adding the Kronecker products on every block is the same thing)."""
    n0, n1 = H1[0].shape[0], H1[1].shape[0]
    return H2 + np.kron(H1[0], np.eye(n1)) + np.kron(np.eye(n0), H1[1])


def lowest_eigs(H, k=5):
    """Lowest k eigenvalues (and eigenvectors) of the symmetric excitonic H."""
    w, v = np.linalg.eigh(0.5 * (H + H.T))
    return w[:k], v[:, :k]


# ----------------------------------------------------------------------------------------
# general-XRCC element formulas (H_contractions.c + build_H.py), vectorised over (I,J)
# ----------------------------------------------------------------------------------------

def gen_monomer_2e(ccaa, V):
    """monomer_2e (H_contractions.c:61-78): sum V[p,q,r,s] R[p,q,s,r]; over all (I,J)."""
    return np.einsum("pqrs,ijpqsr->ij", V, ccaa)


def gen_dimer_block(rho, T, U, V, n_elec, nuc, m1, m2, ci1, cj1, ci2, cj2):
    """build_matrix_elements.dimer (build_H.py:56-102) for all (I1,I2),(J1,J2) of one charge
    block; returns (nI1, nI2, nJ1, nJ2) or None."""
    if not (ci1 + ci2 == cj1 + cj2 and cj1 - 2 <= ci1 <= cj1 + 2):
        return None
    sign2 = (-1) ** ((n_elec[m2] - ci2) % 2)
    k1, k2 = (ci1, cj1), (ci2, cj2)
    if ci1 == cj1 - 2:   # dimer_2min2pls(Rcc1, Raa2, V[m1,m1,m2,m2]) :95
        return np.einsum("pqrs,ikpq,jlsr->ijkl", V[m1, m1, m2, m2], rho[m1]["cc"][k1], rho[m2]["aa"][k2])
    if ci1 == cj1 - 1:
        h = T[m1, m2] + U[m1, m1, m2] + U[m2, m1, m2]
        c1, cca1, a2, caa2 = rho[m1]["c"][k1], rho[m1]["cca"][k1], rho[m2]["a"][k2], rho[m2]["caa"][k2]
        t = np.einsum("pq,ikp,jlq->ijkl", h, c1, a2)                                   # :116-127
        t2 = np.einsum("pqrs,ikqpr,jls->ijkl", V[m1, m1, m1, m2], cca1, a2)               # :132-144
        t2 += np.einsum("pqrs,ikp,jlqsr->ijkl", V[m1, m2, m2, m2], c1, caa2)              # :145-157
        return sign2 * (t + 2 * t2)
    if ci1 == cj1:
        ca1, ca2 = rho[m1]["ca"][k1], rho[m2]["ca"][k2]
        out = 4 * np.einsum("pqrs,ikpr,jlqs->ijkl", V[m1, m2, m1, m2], ca1, ca2)         # :163-180
        e2 = np.einsum("pq,jlpq->jl", U[m1, m2, m2], ca2)                                # extPot :80
        e1 = np.einsum("pq,ikpq->ik", U[m2, m1, m1], ca1)
        n1, n2 = ca1.shape[0], ca2.shape[0]
        out += np.einsum("ik,jl->ijkl", np.eye(n1), e2)
        out += np.einsum("ik,jl->ijkl", e1, np.eye(n2))
        out += nuc[m1][m2] * np.einsum("ik,jl->ijkl", np.eye(n1), np.eye(n2))
        return out
    if ci1 == cj1 + 1:
        h = T[m2, m1] + U[m1, m2, m1] + U[m2, m2, m1]
        a1, caa1, c2, cca2 = rho[m1]["a"][k1], rho[m1]["caa"][k1], rho[m2]["c"][k2], rho[m2]["cca"][k2]
        t = np.einsum("pq,jlp,ikq->ijkl", h, c2, a1)
        t2 = np.einsum("pqrs,jlqpr,iks->ijkl", V[m2, m2, m2, m1], cca2, a1)
        t2 += np.einsum("pqrs,jlp,ikqsr->ijkl", V[m2, m1, m1, m1], c2, caa1)
        return -sign2 * (t + 2 * t2)
    if ci1 == cj1 + 2:   # dimer_2min2pls(Rcc2, Raa1, V[m2,m2,m1,m1])
        return np.einsum("pqrs,jlpq,iksr->ijkl", V[m2, m2, m1, m1], rho[m2]["cc"][k2], rho[m1]["aa"][k1])
    return None


def gen_trimer_block(rho, T, U, V, n_elec, m, chg_i, chg_j):
    """build_matrix_elements.trimer (build_H.py:103-188) for all (I1,I2,I3),(J1,J2,J3) of one
    charge block; returns (nI1,nI2,nI3,nJ1,nJ2,nJ3) or None."""
    m1, m2, m3 = m
    (ci1, ci2, ci3), (cj1, cj2, cj3) = chg_i, chg_j
    d = sorted([ci1 - cj1, ci2 - cj2, ci3 - cj3])
    if d not in ([-2, 1, 1], [-1, 0, 1], [-1, -1, 2]):
        return None
    s2 = (-1) ** ((n_elec[m2] - ci2) % 2)
    s3 = (-1) ** ((n_elec[m3] - ci3) % 2)
    k1, k2, k3 = (ci1, cj1), (ci2, cj2), (ci3, cj3)

    def r(mm, op, kk):
        return rho[mm][op][kk]

    # 2min1pls1pls: 2 sum V[p1 q1 r2 s3] Rcc1[q1,p1] Ra2[r2] Ra3[s3]  (H_contractions.c:184-204)
    def t2m(Rcc, Ra, Rb, Vb):
        return 2 * np.einsum("pqrs,xaqp,ybr,zcs->xyzabc", Vb, Rcc, Ra, Rb, optimize=True)

    # 2pls1min1min: 2 sum V[r2 s3 p1 q1] Raa1[q1,p1] Rc2[r2] Rc3[s3]  (:208-228)
    def t2p(Raa, Rc, Rd, Vb):
        return 2 * np.einsum("rspq,xaqp,ybr,zcs->xyzabc", Vb, Raa, Rc, Rd, optimize=True)

    # Ex1min1pls: 4 sum V[p1 r2 q1 s3] Rca1[p1,q1] Rc2[r2] Ra3[s3]  (:232-252)
    def tex(Rca, Rc, Ra, Vb):
        return 4 * np.einsum("prqs,xapq,ybr,zcs->xyzabc", Vb, Rca, Rc, Ra, optimize=True)

    def ext(Rc, Ra, Ub, nI):   # dimer_1min1pls_1e(Rc, Ra, U) times delta on the Ex fragment
        return np.einsum("pq,ybp,zcq,xa->xyzabc", Ub, Rc, Ra, np.eye(nI), optimize=True)

    def perm(x, order):
        # x indexed (f_order[0], f_order[1], f_order[2]) for bra then ket -> absolute (1,2,3)
        inv = [order.index(k) for k in range(3)]
        return x.transpose(inv + [3 + v for v in inv])

    if ci1 == cj1 - 2:
        return s3 * perm(t2m(r(m1, "cc", k1), r(m2, "a", k2), r(m3, "a", k3), V[m1, m1, m2, m3]), [0, 1, 2])
    if ci2 == cj2 - 2:
        return s2 * s3 * perm(t2m(r(m2, "cc", k2), r(m1, "a", k1), r(m3, "a", k3), V[m2, m2, m1, m3]), [1, 0, 2])
    if ci3 == cj3 - 2:
        return s2 * perm(t2m(r(m3, "cc", k3), r(m1, "a", k1), r(m2, "a", k2), V[m3, m3, m1, m2]), [2, 0, 1])
    if ci1 == cj1 + 2:
        return s3 * perm(t2p(r(m1, "aa", k1), r(m2, "c", k2), r(m3, "c", k3), V[m2, m3, m1, m1]), [0, 1, 2])
    if ci2 == cj2 + 2:
        return s2 * s3 * perm(t2p(r(m2, "aa", k2), r(m1, "c", k1), r(m3, "c", k3), V[m1, m3, m2, m2]), [1, 0, 2])
    if ci3 == cj3 + 2:
        return s2 * perm(t2p(r(m3, "aa", k3), r(m1, "c", k1), r(m2, "c", k2), V[m1, m2, m3, m3]), [2, 0, 1])
    if ci1 == cj1:
        Rca1 = r(m1, "ca", k1)
        n1 = Rca1.shape[0]
        if ci2 == cj2 - 1:
            t = tex(Rca1, r(m2, "c", k2), r(m3, "a", k3), V[m1, m2, m1, m3]) + ext(r(m2, "c", k2), r(m3, "a", k3), U[m1, m2, m3], n1)
            return s3 * perm(t, [0, 1, 2])
        if ci3 == cj3 - 1:
            t = tex(Rca1, r(m3, "c", k3), r(m2, "a", k2), V[m1, m3, m1, m2]) + ext(r(m3, "c", k3), r(m2, "a", k2), U[m1, m3, m2], n1)
            return -s3 * perm(t, [0, 2, 1])
    if ci2 == cj2:
        Rca2 = r(m2, "ca", k2)
        n2 = Rca2.shape[0]
        if ci1 == cj1 - 1:
            t = tex(Rca2, r(m1, "c", k1), r(m3, "a", k3), V[m2, m1, m2, m3]) + ext(r(m1, "c", k1), r(m3, "a", k3), U[m2, m1, m3], n2)
            return s2 * s3 * perm(t, [1, 0, 2])
        if ci3 == cj3 - 1:
            t = tex(Rca2, r(m3, "c", k3), r(m1, "a", k1), V[m2, m3, m2, m1]) + ext(r(m3, "c", k3), r(m1, "a", k1), U[m2, m3, m1], n2)
            return -s2 * s3 * perm(t, [1, 2, 0])
    if ci3 == cj3:
        Rca3 = r(m3, "ca", k3)
        n3 = Rca3.shape[0]
        if ci1 == cj1 - 1:
            t = tex(Rca3, r(m1, "c", k1), r(m2, "a", k2), V[m3, m1, m3, m2]) + ext(r(m1, "c", k1), r(m2, "a", k2), U[m3, m1, m2], n3)
            return s2 * perm(t, [2, 0, 1])
        if ci2 == cj2 - 1:
            t = tex(Rca3, r(m2, "c", k2), r(m1, "a", k1), V[m3, m2, m3, m1]) + ext(r(m2, "c", k2), r(m1, "a", k1), U[m3, m2, m1], n3)
            return -s2 * perm(t, [2, 1, 0])
    return None


# ----------------------------------------------------------------------------------------
# supersystem FCI in the product-determinant basis (known-answer test)
# ----------------------------------------------------------------------------------------

def general_xr_H_full(dens, ints, n_ref, charges, n_frag):
    """Order-0 general-XRCC Hamiltonian of n_frag fragments (2 or 3) in the full product
    basis |I_0 I_1 ... > = C_0 C_1 ... |0> (fragment-major, charge blocks in `charges` order):
    monomer terms (build_H.py:38-47), pair blocks (build_H.py:48-102) and triple blocks
    (build_H.py:103-188), each embedded with identity on the other fragments.

    The embedding carries the fermionic phase of spectator fragments that the reference's
    own embedding (general-XRCC/hamiltonian.py:18-80) leaves out: moving the operators of a
    term past the creation string C_O of a spectator O costs (-1)^(n_O * p), p = parity of
    the number of the term's operators on fragments after O.  With it, complete fragment
    bases reproduce the supersystem FCI spectrum (exact for 3 fragments; without it, odd
    charge transfers between fragments 0 and 2 take the wrong sign).  Small systems only."""
    ns = [dens[0]["n_states"][c] for c in charges]          # identical state counts on every fragment
    tot = sum(ns)
    off = np.concatenate([[0], np.cumsum(ns)]).astype(int)
    chg_of = np.concatenate([[c] * n for c, n in zip(charges, ns)])
    par_n = ((n_ref - chg_of) % 2).astype(int)              # electron-count parity of each state
    T, U, V = ints.T, ints.U, ints.V
    nel = [n_ref] * n_frag
    nuc = np.zeros((n_frag, n_frag))
    eye = np.eye(tot)
    dim = tot ** n_frag
    H = np.zeros((tot,) * (2 * n_frag))
    letters = "abcdefghijkl"

    dq = (np.abs(chg_of[:, None] - chg_of[None, :]) % 2).astype(int)   # charge-change parity (bra, ket)

    def axes_shape(pairs):
        shape = [1] * (2 * n_frag)
        for ax in pairs:
            shape[ax] = tot
        return shape

    def embed(block, frags):
        """block indexed (bra of frags..., ket of frags...) -> full product space."""
        others = [o for o in range(n_frag) if o not in frags]
        bra = [letters[f] for f in range(n_frag)]
        ket = [letters[n_frag + f] for f in range(n_frag)]
        spec = "".join(bra[f] for f in frags) + "".join(ket[f] for f in frags)
        terms = [spec] + [bra[o] + ket[o] for o in others]
        out = np.einsum(",".join(terms) + "->" + "".join(bra + ket), block, *[eye] * len(others))
        for o in others:
            p = 0
            for f in frags:
                if f > o:
                    p = p + dq.reshape(axes_shape([f, n_frag + f]))
            if np.ndim(p) == 0:
                continue
            n_o = par_n.reshape(axes_shape([o]))
            out = out * (1.0 - 2.0 * ((p * n_o) % 2))
        return out

    for m in range(n_frag):
        h1 = np.zeros((tot, tot))
        for a_, ch in enumerate(charges):
            sl = slice(off[a_], off[a_ + 1])
            h1[sl, sl] = (np.einsum("pq,ijpq->ij", T[m, m] + U[m, m, m], dens[m]["ca"][(ch, ch)]) +
                          gen_monomer_2e(dens[m]["ccaa"][(ch, ch)], V[m, m, m, m]))
        H += embed(h1, [m])
    for m1 in range(n_frag):
        for m2 in range(m1 + 1, n_frag):
            blk = np.zeros((tot,) * 4)
            for a_, ci1 in enumerate(charges):
                for b_, ci2 in enumerate(charges):
                    for c_, cj1 in enumerate(charges):
                        for d_, cj2 in enumerate(charges):
                            x = gen_dimer_block(dens, T, U, V, nel, nuc, m1, m2, ci1, cj1, ci2, cj2)
                            if x is not None:
                                blk[off[a_]:off[a_ + 1], off[b_]:off[b_ + 1], off[c_]:off[c_ + 1],
                                    off[d_]:off[d_ + 1]] += x
            H += embed(blk, [m1, m2])
    if n_frag == 3:
        blk = np.zeros((tot,) * 6)
        for ci in np.ndindex(*(len(charges),) * 3):
            for cj in np.ndindex(*(len(charges),) * 3):
                x = gen_trimer_block(dens, T, U, V, nel, (0, 1, 2), tuple(charges[i] for i in ci),
                                     tuple(charges[j] for j in cj))
                if x is not None:
                    sl = tuple(slice(off[i], off[i + 1]) for i in ci) + tuple(slice(off[j], off[j + 1]) for j in cj)
                    blk[sl] += x
        H += blk          # all three fragments take part: no spectator
    return H.reshape(dim, dim)


def fci_hamiltonian(h, V, masks):
    """<P|H|Q> for H = sum h_pq c+_p a_q + sum V_pqrs c+_p c+_q a_s a_r over global
    determinants (uint64 masks), parity = (-1)^(occupied orbitals above), the convention of
    density_tensors.c applied to the whole supersystem."""
    NN = h.shape[0]
    n = len(masks)
    H = np.zeros((n, n))
    idx, P, Q, s = coupling_list("ca", masks, masks, NN, NN, 0)
    p, q = idx // NN, idx % NN
    np.add.at(H, (P, Q), s * h[p, q])
    idx, P, Q, s = coupling_list("ccaa", masks, masks, NN, NN, 0)
    p, q, x, y = idx // NN ** 3, (idx // NN ** 2) % NN, (idx // NN) % NN, idx % NN
    np.add.at(H, (P, Q), s * V[p, q, y, x])     # c+_p c+_q a_x a_y  <->  V_pq,r=y,s=x
    return H


# ----------------------------------------------------------------------------------------
# scalar element formulas (one (I,J) pair), H_contractions.c restated with einsum
# ----------------------------------------------------------------------------------------

def h_element(name, *args):
    """NumPy restatement of one H_contractions.c function (same argument order: the integer
    orbital counts first, then the flattened arrays)."""
    if name in ("monomer_1e", "monomer_extPot"):          # :48-59, :80-91
        n, R, h = args
        return float(np.dot(h.reshape(-1), R.reshape(-1)))
    if name == "monomer_2e":                              # :61-78
        n, R, V = args
        return float(np.einsum("pqrs,pqsr->", V.reshape((n,) * 4), R.reshape((n,) * 4)))
    if name == "dimer_2min2pls":                          # :95-112
        n1, n2, Rcc1, Raa2, V = args
        return float(np.einsum("pqrs,pq,sr->", V.reshape(n1, n1, n2, n2), Rcc1.reshape(n1, n1),
                               Raa2.reshape(n2, n2)))
    if name == "dimer_1min1pls_1e":                       # :116-127
        n1, n2, Rc1, Ra2, h = args
        return float(np.einsum("pq,p,q->", h.reshape(n1, n2), Rc1, Ra2))
    if name == "dimer_1min1pls_2e":                       # :129-159
        n1, n2, Rc1, Rcca1, Ra2, Rcaa2, V1112, V1222 = args
        t = np.einsum("pqrs,qpr,s->", V1112.reshape(n1, n1, n1, n2), Rcca1.reshape(n1, n1, n1), Ra2)
        t += np.einsum("pqrs,p,qsr->", V1222.reshape(n1, n2, n2, n2), Rc1, Rcaa2.reshape(n2, n2, n2))
        return float(2 * t)
    if name == "dimer_ExEx":                              # :163-180
        n1, n2, Rca1, Rca2, V = args
        return float(4 * np.einsum("pqrs,pr,qs->", V.reshape(n1, n2, n1, n2), Rca1.reshape(n1, n1),
                                   Rca2.reshape(n2, n2)))
    if name == "trimer_2min1pls1pls":                     # :184-204
        n1, n2, n3, Rcc1, Ra2, Ra3, V = args
        return float(2 * np.einsum("pqrs,qp,r,s->", V.reshape(n1, n1, n2, n3), Rcc1.reshape(n1, n1), Ra2, Ra3))
    if name == "trimer_2pls1min1min":                     # :208-228
        n1, n2, n3, Raa1, Rc2, Rc3, V = args
        return float(2 * np.einsum("rspq,qp,r,s->", V.reshape(n2, n3, n1, n1), Raa1.reshape(n1, n1), Rc2, Rc3))
    if name == "trimer_Ex1min1pls":                       # :232-252
        n1, n2, n3, Rca1, Rc2, Ra3, V = args
        return float(4 * np.einsum("prqs,pq,r,s->", V.reshape(n1, n2, n1, n3), Rca1.reshape(n1, n1), Rc2, Ra3))
    raise NotImplementedError(name)


# ----------------------------------------------------------------------------------------
# energies and the reference's state-gradient formula (checkers for the adjoint)
# ----------------------------------------------------------------------------------------

def xr_energy(h, V, Ns, n_orb, n_core, n_elec_ref, states, charges):
    """Lowest eigenvalue and eigenvector of the full order-0 XR H for fragment states
    states[m][chg] = (coeffs, masks) (coefficients need not be orthonormal)."""
    ints = FragInts(h, V, Ns)
    dens = [build_densities({c: Sector(*states[m][c]) for c in charges}, n_orb, n_core, n_elec_ref)
            for m in range(2)]
    H1, H2 = get_xr_H0(ints, dens, [list(charges), list(charges)])
    H = full_H(H1, H2)
    w, v = np.linalg.eigh(0.5 * (H + H.T))
    return w[0], v[:, 0], H1, H2


def reference_state_gradient_herm(h, V, Ns, n_orb, n_core, n_elec_ref, states, charges, frag=0):
    """The 'herm' state gradient of StateSpaceOptimizer/state_gradients.py:121-244 restated
    by brute force: for fragment A = frag, G[k, P] = sum_l d[k,l] <P (x) l| H - E |Psi>,
    where P runs over A's determinants and l over the other fragment's states
    (state_gradients.py:205-216: monomer H term with determinant bras, E term with the
    adapted overlaps, dimer term with bra_det densities, other fragment's H1 term).
    The bra-determinant Hamiltonian is built with complete determinant bases on A (the
    'bra_det' densities of Be-states/densities.py:107-113) and contracted with the states
    on the ket side.  Returns {chg: (n_states, n_conf)}."""
    E, d, _, _ = xr_energy(h, V, Ns, n_orb, n_core, n_elec_ref, states, charges)
    A, B = frag, 1 - frag
    det_states = [dict(s) for s in states]
    det_states[A] = {c: (np.eye(len(states[A][c][1])), states[A][c][1]) for c in charges}
    ints = FragInts(h, V, Ns)
    dens = [build_densities({c: Sector(*det_states[m][c]) for c in charges}, n_orb, n_core, n_elec_ref)
            for m in range(2)]
    H1, H2 = get_xr_H0(ints, dens, [list(charges), list(charges)])
    Hdet = full_H(H1, H2)
    nA_det = [len(states[A][c][1]) for c in charges]
    nA = [states[A][c][0].shape[0] for c in charges]
    nB = sum(states[B][c][0].shape[0] for c in charges)
    Zt = np.zeros((sum(nA_det), sum(nA)))      # det x state, block diagonal by charge
    r0 = c0 = 0
    for c, nd, ns_ in zip(charges, nA_det, nA):
        Zt[r0:r0 + nd, c0:c0 + ns_] = states[A][c][0].T
        r0 += nd
        c0 += ns_
    if A == 0:
        Smix = np.kron(Zt, np.eye(nB))
        Dm = d.reshape(sum(nA), nB)
    else:
        Smix = np.kron(np.eye(nB), Zt)
        Dm = d.reshape(nB, sum(nA)).T
    Hmix = Hdet @ Smix
    r = (Hmix - E * Smix) @ d
    R = r.reshape(sum(nA_det), nB) if A == 0 else r.reshape(nB, sum(nA_det)).T   # [P, l]
    Gfull = Dm @ R.T                                                                # [k, P]
    out = {}
    r0 = c0 = 0
    for c, nd, ns_ in zip(charges, nA_det, nA):
        out[c] = Gfull[c0:c0 + ns_, r0:r0 + nd]
        r0 += nd
        c0 += ns_
    return out, E
