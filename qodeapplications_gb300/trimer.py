"""Trimer blocks of the general-XRCC excitonic Hamiltonian on the device.

The reference evaluates one matrix element at a time: general-XRCC/build_H.py:103-188
(build_matrix_elements.trimer) picks, from the charge changes of the three fragments, one of
H_contractions.c:184-252

    trimer_2min1pls1pls  2 sum V[p1 q1 r2 s3] Rcc1[q1,p1] Ra2[r2] Ra3[s3]
    trimer_2pls1min1min  2 sum V[r2 s3 p1 q1] Raa1[q1,p1] Rc2[r2] Rc3[s3]
    trimer_Ex1min1pls    4 sum V[p1 r2 q1 s3] Rca1[p1,q1] Rc2[r2] Ra3[s3]
                         (+ dimer_1min1pls_1e(Rc2, Ra3, U[1,2,3]) when I1 = J1)

with the phases sign2 = (-1)^(n_elec2 - i2_chg), sign3 = (-1)^(n_elec3 - i3_chg).  Here a
whole charge block (every state triple of bra and ket) is three GEMM stages, and every block
of a plan shares one grouped launch per stage:

  1. P[(x x'), (r s)]  = sum_(k k') R1[(x x'), (k k')] W[(r s), (k k')]   (+ delta(x,x') U[r,s]/4)
  2. Q[(x x'), s, (y y')] = sum_r P[(x x'), r, s] R2[(y y'), r]          (batched over x x')
  3. B[(x x'), (y y'), (z z')] = a sum_s Q[(x x'), s, (y y')] R3[(z z'), s]  (batched)

(x, y, z) is the fragment order of the case (the fragment carrying the two-index density
first), W the V block with the indices of R1 contracted, a = 2 or 4 times the phase.  The
delta U term of trimer_Ex1min1pls folds into stage 1, since 4 * (U/4) contracted with Rc and
Ra is the one-electron term.  block() returns the reference's index order
(I1, I2, I3, J1, J2, J3).
"""
import numpy as np
import torch

from . import _lib
from .gemm import GroupedGemm


def _case(ci, cj):
    """(kind, fragment order, the three density op strings, V block fragments, phase key) for
    one charge block, or None: the dispatch of build_H.py:108-187."""
    d = sorted(a - b for a, b in zip(ci, cj))
    if d not in ([-2, 1, 1], [-1, 0, 1], [-1, -1, 2]):
        return None
    for f in range(3):
        o = [g for g in range(3) if g != f]
        if ci[f] == cj[f] - 2:          # cc on f, a on the others: V[f, f, o0, o1]
            return ("t2m", (f, o[0], o[1]), ("cc", "a", "a"), (f, f, o[0], o[1]))
        if ci[f] == cj[f] + 2:          # aa on f, c on the others: V[o0, o1, f, f]
            return ("t2p", (f, o[0], o[1]), ("aa", "c", "c"), (o[0], o[1], f, f))
    ex = [f for f in range(3) if ci[f] == cj[f]][0]
    cr = [f for f in range(3) if ci[f] == cj[f] - 1][0]
    an = [f for f in range(3) if ci[f] == cj[f] + 1][0]
    return ("tex", (ex, cr, an), ("ca", "c", "a"), (ex, cr, ex, an))


def _phase(kind, order, s2, s3):
    """build_H.py's sign of each case (:119-187), for fragments (0, 1, 2) = (m1, m2, m3)."""
    if kind in ("t2m", "t2p"):
        return {0: s3, 1: s2 * s3, 2: s2}[order[0]]
    return {(0, 1, 2): s3, (0, 2, 1): -s3, (1, 0, 2): s2 * s3, (1, 2, 0): -s2 * s3,
            (2, 0, 1): s2, (2, 1, 0): -s2}[tuple(order)]


class XRTrimerPlan:
    """All trimer charge blocks of fragments (m1, m2, m3) in three grouped launches.

    rho:      three {op: {(bra_chg, ket_chg): CUDA float64 (n_b, n_k, N, ...)}} (DensityBuilder.rho)
    ints:     DeviceIntegrals over the three fragments (T, U, V block accessors)
    n_elec:   reference electron counts of the three fragments
    charges:  three charge lists;  n_states: three {charge: n}
    The density tensors are read in place: rebuild them, then launch() again."""

    def __init__(self, rho, ints, n_elec, charges, n_states, frags=(0, 1, 2), device="cuda"):
        dev = torch.device(device)
        self.device = dev
        f64 = dict(dtype=torch.float64, device=dev)
        m = list(frags)
        self.charges = [list(c) for c in charges]
        self.n_states = [dict(n) for n in n_states]
        N = [int(ints.T(mm, mm).shape[0]) for mm in m]
        self.N = N
        st1, st2, st3 = GroupedGemm(dev), GroupedGemm(dev), GroupedGemm(dev)
        self.blocks_out = {}
        self._keep = []
        Wcache = {}
        ones_cache = {}
        for ci in np.ndindex(*[len(c) for c in self.charges]):
            for cj in np.ndindex(*[len(c) for c in self.charges]):
                chg_i = tuple(self.charges[f][ci[f]] for f in range(3))
                chg_j = tuple(self.charges[f][cj[f]] for f in range(3))
                case = _case(chg_i, chg_j)
                if case is None:
                    continue
                kind, order, ops, vfr = case
                try:
                    R = [rho[order[k]][ops[k]][(chg_i[order[k]], chg_j[order[k]])] for k in range(3)]
                except KeyError:
                    continue                     # a density of this charge pair is absent
                x, y, z = order
                Nx, Ny, Nz = N[x], N[y], N[z]
                s2 = -1.0 if (n_elec[1] - chg_i[1]) % 2 else 1.0
                s3 = -1.0 if (n_elec[2] - chg_i[2]) % 2 else 1.0
                alpha = (4.0 if kind == "tex" else 2.0) * _phase(kind, order, s2, s3)
                wkey = (kind, order)
                if wkey not in Wcache:
                    Vb = ints.V(*[m[f] for f in vfr])
                    if kind == "t2m":            # V[p,q,r,s], R1 indexed (q, p)
                        W = Vb.permute(2, 3, 1, 0)
                    elif kind == "t2p":          # V[r,s,p,q], R1 indexed (q, p)
                        W = Vb.permute(0, 1, 3, 2)
                    else:                        # V[p,r,q,s], R1 indexed (p, q)
                        W = Vb.permute(1, 3, 0, 2)
                    Wcache[wkey] = W.reshape(Ny * Nz, Nx * Nx).contiguous()
                W = Wcache[wkey]
                nxa = R[0].shape[0] * R[0].shape[1]
                nyb = R[1].shape[0] * R[1].shape[1]
                nzc = R[2].shape[0] * R[2].shape[1]
                P = torch.zeros((nxa, Ny * Nz), **f64)
                Q = torch.zeros((nxa, Nz, nyb), **f64)
                B = torch.zeros((nxa, nyb, nzc), **f64)
                R1 = R[0].reshape(nxa, Nx * Nx)
                R2 = R[1].reshape(nyb, Ny)
                R3 = R[2].reshape(nzc, Nz)
                segs = [(R1, Nx * Nx, W, Nx * Nx, Nx * Nx, 1.0)]
                if kind == "tex":
                    # delta(x, x') U[ex, cr, an] / 4 as a K = 1 segment
                    nx = R[0].shape[0]
                    if nx not in ones_cache:
                        ones_cache[nx] = torch.eye(nx, **f64).reshape(nx * nx, 1).contiguous()
                    Ukey = ("U", order)
                    if Ukey not in Wcache:
                        Wcache[Ukey] = (0.25 * ints.U(m[x], m[y], m[z])).reshape(Ny * Nz, 1).contiguous()
                    segs.append((ones_cache[nx], 1, Wcache[Ukey], 1, 1, 1.0))
                st1.add(nxa, Ny * Nz, segs, P, Ny * Nz, mode=0)
                # Q[xa][s][yb] = sum_r P[xa][r][s] R2[yb][r]: A = P_xa stored [k = r][m = s]
                st2.add(Nz, nyb, [(P, Nz, R2, Ny, Ny, 1.0, 1, Ny * Nz, 0)], Q, nyb, mode=0, batch=nxa,
                        sC=Nz * nyb)
                # B[xa][yb][zc] = alpha sum_s Q[xa][s][yb] R3[zc][s]: A = Q_xa stored [k = s][m = yb]
                st3.add(nyb, nzc, [(Q, nyb, R3, Nz, Nz, alpha, 1, Nz * nyb, 0)], B, nzc, mode=0, batch=nxa,
                        sC=nyb * nzc)
                shape = (R[0].shape[0], R[0].shape[1], R[1].shape[0], R[1].shape[1], R[2].shape[0], R[2].shape[1])
                # axes of B (x, x', y, y', z, z') -> (I1, I2, I3, J1, J2, J3)
                perm = [2 * order.index(f) for f in range(3)] + [2 * order.index(f) + 1 for f in range(3)]
                self.blocks_out[(chg_i, chg_j)] = (B, shape, perm)
                self._keep += [P, Q, R1, R2, R3]
        self.stages = [st1.finalize(), st2.finalize(), st3.finalize()]
        self.flops = sum(s.flops for s in self.stages)

    def launch(self, stream=None):
        """Enqueue the three grouped stages (no host synchronisation)."""
        for st in self.stages:
            st.run(stream)

    def block(self, chg_i, chg_j):
        """(n_I1, n_I2, n_I3, n_J1, n_J2, n_J3) view of one charge block, or None."""
        if (tuple(chg_i), tuple(chg_j)) not in self.blocks_out:
            return None
        B, shape, perm = self.blocks_out[(tuple(chg_i), tuple(chg_j))]
        return B.view(shape).permute(perm)

    def keys(self):
        return list(self.blocks_out)
