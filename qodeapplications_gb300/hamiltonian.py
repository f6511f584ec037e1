"""Excitonic-Hamiltonian (XR-H) build on the GPU for a fragment dimer (order 0, S = 1).

This is the GB300 form of hermitian-XRCC get_xr_H at xr_order 0
(get_xr_result.py:86-132, :300-355) and of general-XRCC build_matrix_elements.dimer /
.monomer (build_H.py:42-102).  The reference evaluates every (diagram, charge block,
permutation) lazily in Python and calls BLAS per term; here the whole build is planned
once into two grouped launches:

1. precontractions (precontract.py:32-80): rho x integral GEMMs, one task per
   (fragment, charge pair, family), plus the monomer one-electron GEMVs and the
   delta-function u100 terms;
2. final contractions: ONE task per output charge block (ci0,ci1 | cj0,cj1), whose
   K-concatenated segments are all order-0 diagrams that land in that block
   (t01, u001, u101, v0001, v0100, v0011, v0101 with their catalog phases and
   n_j0 parities, diagrams/S*_diagrams.py), and whose FP64 epilogue adds u100 and
   H1 x 1 + 1 x H1 and scatters from charge-blocked to product-state order.

The monomer two-electron energy (v0000, SV_1mer_0.py:24) never materialises the N^4
ccaa density: a sigma-vector kernel plus one GEMM compute sum V rho^ccaa directly.
"""
import numpy as np
import torch

from . import _lib
from ._lib import call, ptr, stream_ptr
from .densities import DensityBuilder, FragmentSpace
from .gemm import GroupedGemm, SplitRegistry, TCGroupedGemm


class DeviceIntegrals:
    """Fragment-blocked spin-orbital integrals on the device.

    source: any object with block accessors T[m,n], U[k,m,n], V[m,n,o,p] returning arrays
    (the interface of the reference's integral structs, hermitian-XRCC/get_ints.py), or
    the supersystem arrays h (with U folded in) and V plus the spin orbitals per fragment."""

    def __init__(self, h=None, V=None, Ns=None, U=None, source=None, device="cuda"):
        self.device = torch.device(device)
        self._cache = {}
        if source is not None:
            self._src = source
            return
        self.Ns = list(Ns)
        off = np.concatenate([[0], np.cumsum(self.Ns)]).astype(int)
        self.off = off
        n_f = len(self.Ns)
        tot = off[-1]
        U = np.zeros((n_f, tot, tot)) if U is None else np.asarray(U, dtype=np.float64)
        self._h = torch.as_tensor(np.asarray(h, dtype=np.float64), device=self.device)
        self._U = torch.as_tensor(U, device=self.device)
        self._Tfull = self._h - self._U.sum(0)
        self._V = torch.as_tensor(np.asarray(V, dtype=np.float64), device=self.device)
        self._src = None

    @classmethod
    def from_tensors(cls, h, V, Ns, U=None):
        """Device tensors in (no host round trip): h (tot x tot, U folded in when U is None),
        V (tot^4), U (n_frag x tot x tot) or None."""
        self = cls.__new__(cls)
        self.device = h.device
        self._cache = {}
        self.Ns = list(Ns)
        self.off = np.concatenate([[0], np.cumsum(self.Ns)]).astype(int)
        tot = int(self.off[-1])
        self._h = h
        self._U = torch.zeros((len(self.Ns), tot, tot), dtype=h.dtype, device=h.device) if U is None else U
        self._Tfull = h - self._U.sum(0)
        self._V = V
        self._src = None
        return self

    def _sl(self, m):
        return slice(int(self.off[m]), int(self.off[m + 1]))

    def T(self, m, n):
        if self._src is not None:
            return self._get(("T", m, n), lambda: self._src.T[m, n])
        return self._Tfull[self._sl(m), self._sl(n)]

    def U(self, k, m, n):
        if self._src is not None:
            return self._get(("U", k, m, n), lambda: self._src.U[k, m, n])
        return self._U[k][self._sl(m), self._sl(n)]

    def V(self, m, n, o, p):
        if self._src is not None:
            return self._get(("V", m, n, o, p), lambda: self._src.V[m, n, o, p])
        return self._V[self._sl(m), self._sl(n), self._sl(o), self._sl(p)]

    def _get(self, key, fn):
        if key not in self._cache:
            self._cache[key] = torch.as_tensor(np.asarray(fn(), dtype=np.float64), device=self.device)
        return self._cache[key]


class SigmaTwoElectron:
    """E2[I,J] = sum_PQ zb[I,P] <P|V|Q> zk[J,Q] for one fragment and charge (v0000).

    run_sigma(zT) fills sigmaT[J, P] = sum_Q <P| sum V_pqrs c+_p c+_q a_s a_r |Q> zk[J, Q].
    With a spin-conserving V the space goes through (n-2)-electron intermediates (its pair list):
    D = pair scatter of zk, E = D . W^T per spin class (one grouped GEMM, W = 4 V over pairs),
    sigma = pair gather of E; D is kept for the two-particle density of the adjoint.  Otherwise
    xrh_sigma2e (every double excitation of every determinant).  The adjoint's two-particle
    density then holds the same-class blocks only: the entries between pairs of different
    spin classes multiply integrals that vanish by spin symmetry."""

    def __init__(self, space, charge, n_states, V_block, precision=_lib.FP64, own_gemm=True):
        self.space, self.c, self.n = space, charge, n_states
        self.V = V_block.contiguous()
        self.precision = precision if precision in (_lib.FP64, _lib.FP32) else _lib.FP32
        dev = space.device
        nconf = space.n_conf[charge]
        self.sigmaT = torch.empty((n_states, nconf), dtype=torch.float64, device=dev)
        self.pl = space.pair_list(charge)
        if self.pl is not None and not self._spin_conserving(space):
            self.pl = None
        self.tc = False
        if self.pl is not None:
            from .densities import pair_offsets
            pl = self.pl
            n = n_states
            off, stride = pair_offsets(pl, n)
            self.off_dev = torch.from_numpy(off).to(dev)
            self.stride_dev = torch.from_numpy(stride).to(dev)
            f64 = dict(dtype=torch.float64, device=dev)
            # class-major [class][state][K][pair]; positions never written stay zero
            self.D = torch.zeros(n * pl["L"], **f64)
            self.E = torch.zeros(n * pl["L"], **f64)
            self.W, self._uv, self.Dc, self.Ec = [], [], [], []
            # split-precision plans: 3 x TF32 on the tensor cores (sigma feeds the monomer
            # energies, the largest entries of H); FP64 plans: the FP64 grouped GEMM
            self.tc = self.precision == _lib.FP32
            self.reg, self.gemm, g = None, None, None
            if own_gemm and self.tc:
                self.reg = SplitRegistry("tf32x3", dev)
                g = TCGroupedGemm(self.reg)
            elif own_gemm:
                g = GroupedGemm(dev, precision="fp64")
            for cl in pl["classes"]:
                u = torch.as_tensor(cl["u"], device=dev)
                v = torch.as_tensor(cl["v"], device=dev)
                self._uv.append((u, v))
                W = (4.0 * self.V[u[:, None], v[:, None], u[None, :], v[None, :]]).contiguous()
                self.W.append(W)
                b, nK, npr = n * cl["base"], cl["n_K"], cl["n_p"]
                Dc = self.D[b:b + n * nK * npr].view(n * nK, npr)
                Ec = self.E[b:b + n * nK * npr].view(n * nK, npr)
                self.Dc.append(Dc)
                self.Ec.append(Ec)
                if g is not None:
                    self.add_gemm_tasks(g, len(self.Dc) - 1)
            if g is not None and self.tc:
                self.reg.upload()
                self.reg.split("sigW")
                self.gemm = g.finalize().autotune()
            elif g is not None:
                self.gemm = g.finalize()

    def add_gemm_tasks(self, g, k):
        """E[c][(s, K)][pq] = sum_rs D[c][(s, K)][rs] W_c[pq, rs] for spin class k into grouped
        GEMM g (tensor cores, 3 x TF32, when self.tc)."""
        cl = self.pl["classes"][k]
        rows, npr = self.n * cl["n_K"], cl["n_p"]
        if self.tc:
            g.add(rows, npr, [(self.Dc[k], npr, self.W[k], npr, npr, 1.0)], self.Ec[k], npr, mode=0,
                  groups=[("sig", "sigW")])
        else:
            g.add(rows, npr, [(self.Dc[k], npr, self.W[k], npr, npr, 1.0)], self.Ec[k], npr, mode=0)

    def set_V(self, V_block):
        """New integrals in place (the launch tables keep their pointers)."""
        self.V.copy_(V_block)
        if self.pl is not None:
            for W, (u, v) in zip(self.W, self._uv):
                W.copy_(4.0 * self.V[u[:, None], v[:, None], u[None, :], v[None, :]])
            if self.reg is not None:
                self.reg.split("sigW")

    def _spin_conserving(self, space):
        """V couples only pairs with the same number of beta orbitals (checked once)."""
        N, no = space.N, space.n_orbs
        nb = (torch.arange(N, device=self.V.device) >= no).to(torch.int64)
        cls = nb[:, None] + nb[None, :]
        cross = cls[:, :, None, None] != cls[None, None, :, :]
        return float(self.V.abs().masked_fill(~cross, 0.0).max()) == 0.0

    def scatter(self, zT, D):
        pl = self.pl
        call("xrh_pair_scatter", len(pl["X"]), ptr(pl["X_dev"]), ptr(self.off_dev), ptr(pl["sign_dev"]), ptr(zT),
             self.n, ptr(self.stride_dev), ptr(D), stream_ptr())

    def run_sigma(self, zT):
        sp = self.space
        c = self.c
        if self.pl is None:
            call("xrh_sigma2e", self.precision, sp.n_orbs, ptr(self.V), ptr(sp.masks[c]), sp.n_conf[c],
                 ptr(sp.sorted_masks[c]), ptr(sp.sorted_pos[c]), sp.n_conf[c], ptr(sp.rank_table[c]),
                 sp.table_size[c], ptr(sp.binom), ptr(zT), self.n, ptr(self.sigmaT), stream_ptr())
            return
        if self.gemm is None:
            raise RuntimeError("this sigma runs inside a SigmaBatch")
        pl = self.pl
        self.scatter(zT, self.D)
        if self.tc:
            self.reg.split("sig")
        self.gemm.run()
        call("xrh_pair_gather", sp.n_conf[c], ptr(pl["xptr_dev"]), ptr(self.off_dev), ptr(pl["sign_dev"]),
             ptr(self.E), self.n, ptr(self.stride_dev), ptr(self.sigmaT), stream_ptr())


class SigmaBatch:
    """Every pair-list sigma of a plan in four launches: one grouped pair scatter, one operand
    split (tensor-core plans), one grouped GEMM over all spin classes, fragments and charges,
    one grouped pair gather.  items: [(SigmaTwoElectron built with own_gemm=False, its zT)]."""

    def __init__(self, items, device):
        self.items = items
        self.tc = bool(items) and items[0][0].tc
        if not items:
            self.reg = None
            return
        self.scatter = _lib.PairLaunch([(sg.pl, sg.off_dev, sg.stride_dev, zT, sg.D, sg.n) for sg, zT in items],
                                       False, device)
        self.gather = _lib.PairLaunch([(sg.pl, sg.off_dev, sg.stride_dev, sg.E, sg.sigmaT, sg.n)
                                       for sg, zT in items], True, device)
        self.reg = SplitRegistry("tf32x3", device) if self.tc else None
        g = TCGroupedGemm(self.reg) if self.tc else GroupedGemm(device, precision="fp64")
        for sg, _zT in items:
            for k in range(len(sg.Dc)):
                sg.add_gemm_tasks(g, k)
        if self.tc:
            self.reg.upload()
            self.reg.split("sigW")
            self.gemm = g.finalize().autotune()
        else:
            self.gemm = g.finalize()

    def run(self):
        if not self.items:
            return
        self.scatter.run()
        if self.tc:
            self.reg.split("sig")
        self.gemm.run()
        self.gather.run()

    def refresh_W(self):
        """Re-split W after the sigmas' set_V (tensor-core plans)."""
        if self.tc:
            self.reg.split("sigW")

    def check(self):
        if self.tc and self.items:
            self.gemm.check()


def monomer_two_electron(space, coeffs, V_block, c):
    """sum_pqrs V_pqrs rho^ccaa_IJ[p,q,s,r] for all state pairs of charge c (FP64)."""
    z = coeffs[c].contiguous()
    n = z.shape[0]
    zT = z.t().contiguous()
    s2 = SigmaTwoElectron(space, c, n, V_block)
    s2.run_sigma(zT)
    out = torch.zeros((n, n), dtype=torch.float64, device=space.device)
    g = GroupedGemm(space.device)
    nconf = space.n_conf[c]
    splitk = max(1, min(64, nconf // 512))
    g.add(n, n, [(z, nconf, s2.sigmaT, nconf, nconf, 1.0)], out, n, mode=1, splitk=splitk)
    g.finalize().run()
    return out


def _product_offsets(n_states, charges):
    off, acc = {}, 0
    for c in charges:
        off[c] = acc
        acc += n_states[c]
    return off, acc


class _Arena:
    """One device buffer carved into the accumulation targets of a build, so that a single
    memset clears every split-K / atomic output before the launches."""

    def __init__(self, device):
        self.device, self.sizes, self.views, self.buf = device, [], [], None

    def request(self, shape):
        n = int(np.prod(shape))
        self.sizes.append((n, tuple(shape)))
        return len(self.sizes) - 1

    def allocate(self):
        total = sum(n for n, _ in self.sizes)
        self.buf = torch.zeros(max(total, 1), dtype=torch.float64, device=self.device)
        off = 0
        for n, shape in self.sizes:
            self.views.append(self.buf[off:off + n].view(shape))
            off += n
        return self.views


def _splitk(K_total, target=384, cap=32):
    return int(max(1, min(cap, K_total // target)))



def _abt_table(entries, device):
    """Task table of xrh_abt_grouped (FP64) for [(m, n, (A, lda, B, ldb, K, alpha), C)], C with
    row stride n; None when empty."""
    if not entries:
        return None
    tab = np.zeros(len(entries), dtype=_lib.ABT_TASK_DTYPE)
    cta = 0
    for i, (m, n, (A, lda, B, ldb, K, alpha), C) in enumerate(entries):
        t = tab[i]
        t["A"], t["B"], t["C"] = A.data_ptr(), B.data_ptr(), C.data_ptr()
        t["m"], t["n"], t["K"], t["lda"], t["ldb"], t["alpha"], t["cta_begin"] = m, n, K, lda, ldb, alpha, cta
        cta += int(_lib.lib().xrh_abt_ctas(K))
    return torch.from_numpy(tab.view(np.uint8).copy()).to(device), len(entries), cta


class XRDimerPlan:
    """Planned order-0 XR-H build of a dimer (fragments 0 and 1, S = 1 integrals).

    spaces:   two FragmentSpace objects (resident coupling lists)
    n_states: two {charge: number of states}
    charges:  two charge lists (also the state order of each fragment's H1 and of the
              product basis, as monomer_charges in get_xr_result.py:76-79)
    ints:     DeviceIntegrals
    output:   'split' -> (H1 list, H2) as get_xr_H returns them;
              'full'  -> H = H2 + H1 x 1 + 1 x H1 (mains/workflow.py:216-230)
    autotune: time the tile policies of the tensor-core launches on the device once per
              problem shape and keep the fastest (TCGroupedGemm.autotune).
    convention: 'hermitian' (diagram phases of hermitian-XRCC) or 'general' (the sign
              convention of general-XRCC/build_H.py:68, charge-transfer blocks differ by
              the gauge (-1)^(n_i1 + n_j0)).
    builders: two DensityBuilder objects shared with other plans (built by their owner;
              launch(build_densities=False)), or None for the plan's own.
    monomer_2e: how the monomer two-electron term v0000 is formed: 'sigma' (the default:
              sigma vectors through (n-2)-electron pair intermediates, rho^ccaa never
              stored), 'ccaa' (a stored rho^ccaa block per charge, contracted with V as
              SV_1mer_0.py:24 does; for densities handed in by a caller) or 'none'.
    total_charges: with layout='sector', the total charges whose sectors are built (None: all);
              H conserves the total charge, so the other sectors are never needed when the
              eigenvector is sought in one of these (the pairs of a neutral ring).
    registry: a SplitRegistry shared with other plans over the same density builders (split
              precision): each builder's densities are split copies held once, in the split
              group named by the builder (builder.split_group); precontraction outputs and
              integral matrices stay in groups of this plan.

    The inputs are the persistent coefficient buffers self.coeffs[m][charge]
    (n_states x n_conf); launch() enqueues the whole build on the current stream without
    host synchronisation or allocation, so it can be captured in a CUDA graph.
    """

    def __init__(self, spaces, n_states, charges, ints, output="full", precision="fp64",
                 convention="hermitian", layout="product", dens_precision=None, sigma_precision=None,
                 autotune=True, builders=None, monomer_2e="sigma", total_charges=None, registry=None):
        if monomer_2e not in ("sigma", "ccaa", "none"):
            raise ValueError("monomer_2e must be 'sigma', 'ccaa' or 'none'")
        if total_charges is not None and layout == "product":
            raise ValueError("total_charges needs the sector layout")
        self.total_charges = None if total_charges is None else set(total_charges)
        self.monomer_2e = monomer_2e
        self.spaces, self.charges = spaces, [list(c) for c in charges]
        self.n_states = [dict(n) for n in n_states]
        self.ints = ints
        self.output, self.convention = output, convention
        self.precision = _lib.PRECISIONS[precision]
        self.device = spaces[0].device
        dev = self.device
        f64 = dict(dtype=torch.float64, device=dev)
        self.coeffs = [{c: torch.zeros((self.n_states[m][c], spaces[m].n_conf[c]), **f64) for c in self.charges[m]}
                       for m in (0, 1)]
        # densities and sigma vectors: FP64 on the fp64 path; FP32 products with FP64 sums on the
        # split-precision paths unless requested otherwise
        tc_mode = self.precision in (_lib.BF16X3, _lib.TF32X3)
        # densities: coupling-list kernels with FP32 products on the split-precision paths;
        # "im" builds them through intermediate determinants on the tensor cores instead (dense
        # over the intermediates: at 2 x 14 orbitals / 60 states its GEMMs, scatters and operand
        # splits cost about what the coupling lists do, so it is not the default)
        self.dens_precision = dens_precision or ("fp32" if tc_mode else "fp64")
        self.sigma_precision = sigma_precision or ("fp32" if tc_mode else "fp64")
        if self.dens_precision == "im":
            assert tc_mode, "the intermediate-determinant densities run on the split-precision paths"
            from .intermediates import IntermediateDensityBuilder
            # the density GEMMs multiply state coefficients: 3 x TF32 (22-bit products) keeps them
            # near FP32 accuracy; 3 x BF16 (16-bit) would cost about 1e-5 relative per element
            self.builders = [IntermediateDensityBuilder(spaces[m], self.n_states[m], precision="tf32x3",
                                                        autotune=autotune) for m in (0, 1)]
        elif builders is not None:
            # density builders shared with other plans (the pairs of a larger system): the
            # owner builds them once per iteration and calls launch(build_densities=False)
            self.builders = list(builders)
        else:
            self.builders = [DensityBuilder(spaces[m], self.n_states[m], precision=self.dens_precision)
                             for m in (0, 1)]
        N = [spaces[0].N, spaces[1].N]
        self.N = N
        rho = [b.rho for b in self.builders]
        chg, ns = self.charges, self.n_states

        # ---- integral matrices in B-role layout [x, y] (y contracted, contiguous) ----
        W = self._integral_matrices(ints)
        self.W = W

        # ---- accumulation targets (one arena, cleared by one memset per build) ----
        arena = _Arena(dev)
        req = {}
        for c in chg[0]:
            if ("ca", c, c) in spaces[0].couplings:
                req[("v0101", c)] = arena.request((ns[0][c] ** 2, N[1] ** 2))
        for m, o in ((0, 1), (1, 0)):
            for (op, bc, kc) in spaces[m].couplings:
                nbk = ns[m][bc] * ns[m][kc]
                if op == "c":
                    req[("p1", m, bc, kc)] = arena.request((nbk, N[o]))
                elif op == "caa":
                    req[("pcaa", m, bc, kc)] = arena.request((nbk, N[o]))
                elif op == "cc":
                    req[("pcc", m, bc, kc)] = arena.request((nbk, N[o] ** 2))
            for c in chg[m]:
                if ("ca", c, c) in spaces[m].couplings:
                    n = ns[m][c]
                    for kind in ("h1", "du", "fd"):
                        req[(kind, m, c)] = arena.request((n * n, 1))
        views = arena.allocate()
        self.arena = arena
        self.P = {k: views[i] for k, i in req.items() if k[0] in ("v0101", "p1", "pcaa", "pcc")}
        self.H1blk = [{c: views[req[("h1", m, c)]] for c in chg[m] if ("h1", m, c) in req} for m in (0, 1)]
        self.DU = [{c: views[req[("du", m, c)]] for c in chg[m] if ("du", m, c) in req} for m in (0, 1)]
        self.FULLD = [{c: views[req[("fd", m, c)]] for c in chg[m] if ("fd", m, c) in req} for m in (0, 1)]

        # ---- precontraction tasks (split-K, atomic accumulation into the arena) ----
        pre = GroupedGemm(dev)
        self.pre_specs = []       # (output P, [(rho, integral-matrix key)]) for the adjoint

        def add_pre(M, Ncols, segs, out, ldc, wkeys=None):
            pre.add(M, Ncols, segs, out, ldc, mode=1, splitk=_splitk(sum(sg[4] for sg in segs)))
            if wkeys is not None:
                self.pre_specs.append((out, [(sg[0], wk) for sg, wk in zip(segs, wkeys)]))

        for c in chg[0]:
            if ("v0101", c) in self.P:
                n2 = ns[0][c] ** 2
                add_pre(n2, N[1] ** 2, [(rho[0]["ca"][(c, c)], N[0] ** 2, W["v0101"], N[0] ** 2, N[0] ** 2, 1.0)],
                        self.P[("v0101", c)], N[1] ** 2, wkeys=["v0101"])
        for m, o in ((0, 1), (1, 0)):
            for (op, bc, kc) in spaces[m].couplings:
                nbk = ns[m][bc] * ns[m][kc]
                if op == "c":        # bra - ket = -1: P1 = rho^c h + rho^cca (-2V)
                    segs = [(rho[m]["c"][(bc, kc)], N[m], W[("h1", m)], N[m], N[m], 1.0)]
                    wk = [("h1", m)]
                    if ("cca", bc, kc) in spaces[m].couplings:
                        segs.append((rho[m]["cca"][(bc, kc)], N[m] ** 3, W[("cca", m)], N[m] ** 3, N[m] ** 3, 1.0))
                        wk.append(("cca", m))
                    add_pre(nbk, N[o], segs, self.P[("p1", m, bc, kc)], N[o], wkeys=wk)
                elif op == "caa":
                    add_pre(nbk, N[o], [(rho[m]["caa"][(bc, kc)], N[m] ** 3, W[("caa", m)], N[m] ** 3, N[m] ** 3, 1.0)],
                            self.P[("pcaa", m, bc, kc)], N[o], wkeys=[("caa", m)])
                elif op == "cc":
                    add_pre(nbk, N[o] ** 2, [(rho[m]["cc"][(bc, kc)], N[m] ** 2, W[("cc", m)], N[m] ** 2, N[m] ** 2, 1.0)],
                            self.P[("pcc", m, bc, kc)], N[o] ** 2, wkeys=[("cc", m)])
        # monomer pieces: H1 (e1 + e2), u100 (du), and their sum (fd) for the full H
        self.sigma = [{}, {}]
        mono = []
        for m, o in ((0, 1), (1, 0)):
            for c in chg[m]:
                if c not in self.H1blk[m]:
                    continue
                n = ns[m][c]
                ca = rho[m]["ca"][(c, c)]
                if monomer_2e == "sigma":
                    sg = SigmaTwoElectron(spaces[m], c, n, ints.V(m, m, m, m),
                                          precision=_lib.PRECISIONS[self.sigma_precision], own_gemm=False)
                    self.sigma[m][c] = sg
                    nconf = spaces[m].n_conf[c]
                    zrow = self.coeffs[m][c]
                targets_h1 = [self.H1blk[m][c]] + ([self.FULLD[m][c]] if output == "full" else [])
                targets_du = [self.DU[m][c]] + ([self.FULLD[m][c]] if output == "full" else [])
                for tgt in targets_h1:
                    mono.append((n * n, 1, [(ca, N[m] ** 2, W[("hmm", m)], N[m] ** 2, N[m] ** 2, 1.0)], tgt, 1,
                                 _splitk(N[m] ** 2)))
                    if monomer_2e == "sigma":
                        mono.append((n, n, [(zrow, nconf, sg.sigmaT, nconf, nconf, 1.0)], tgt, n,
                                     _splitk(nconf, target=128, cap=512)))
                    elif monomer_2e == "ccaa":
                        mono.append((n * n, 1, [(rho[m]["ccaa"][(c, c)], N[m] ** 4, W[("vmmmm", m)], N[m] ** 4,
                                                 N[m] ** 4, 1.0)], tgt, 1, _splitk(N[m] ** 4)))
                for tgt in targets_du:
                    mono.append((n * n, 1, [(ca, N[m] ** 2, W[("u100", m)], N[m] ** 2, N[m] ** 2, 1.0)], tgt, 1,
                                 _splitk(N[m] ** 2)))
        self.sigma_batch = SigmaBatch([(sg, self.builders[m].zT[c]) for m in (0, 1)
                                       for c, sg in self.sigma[m].items() if sg.pl is not None], dev)
        # one-column terms (rho^ca . h) are row GEMVs: a 64 x 64 FP64 tile would spend 64x the
        # FMAs of the result on them, and an FP64 tile is slow on this part
        self.mono_gemv = [(sg_[0][0], sg_[0][2], out_, M_, sg_[0][4]) for (M_, N_, sg_, out_, _l, _s) in mono if N_ == 1]
        mono = [t for t in mono if t[1] != 1]
        self.mono_flops = sum(2.0 * M_ * K_ for (_a, _w, _o, M_, K_) in self.mono_gemv)
        self.mono_gemv_tasks = None
        if self.mono_gemv:
            gt = np.zeros(len(self.mono_gemv), dtype=_lib.GEMV_TASK_DTYPE)
            rb = 0
            for i, (A_, w_, out_, M_, K_) in enumerate(self.mono_gemv):
                t = gt[i]
                t["A"], t["x"], t["y"] = A_.data_ptr(), w_.data_ptr(), out_.data_ptr()
                t["rows"], t["cols"], t["lda"], t["alpha"], t["beta"], t["row_begin"] = M_, K_, K_, 1.0, 1.0, rb
                rb += (M_ + 7) // 8 * 8
            self.mono_gemv_tasks = (torch.from_numpy(gt.view(np.uint8).copy()).to(self.device), len(gt), rb)
        # small outputs over long K (E2 = Zb sigma^T, n x n over the determinants): split-K
        # products in one launch instead of 64 x 64 tiles
        abt = [t for t in mono if len(t[2]) == 1 and t[0] <= 64 and t[1] <= 64 and t[4] == t[1]]
        mono = [t for t in mono if not any(t is a for a in abt)]
        self.mono_abt = _abt_table([(M_, N_, segs_[0], out_) for (M_, N_, segs_, out_, _l, _s) in abt], dev)
        self.mono_flops += sum(2.0 * M_ * N_ * segs_[0][4] for (M_, N_, segs_, _o, _l, _s) in abt)
        for (M_, N_, segs_, out_, ldc_, sk_) in mono:
            pre.add(M_, N_, segs_, out_, ldc_, mode=1, splitk=sk_)
        self.pre = pre.finalize()

        # ---- final tasks: one per output charge block ----
        nb = [ns[m] for m in (0, 1)]
        off0, tot0 = _product_offsets(nb[0], chg[0])
        off1, tot1 = _product_offsets(nb[1], chg[1])
        self.offsets = (off0, off1)
        self.dim = (tot0 * tot1, tot0 * tot1)
        self.tot = (tot0, tot1)
        self.layout = layout
        if layout == "product":
            self.H = torch.zeros(self.dim, **f64)
        else:
            # H is block diagonal in the total charge: one dense matrix per sector t, rows
            # ordered block-major over (c0, c1 = t - c0) and row-major (i0, i1) inside a block
            self.sectors = {}
            for c0 in chg[0]:
                for c1 in chg[1]:
                    t = c0 + c1
                    if self.total_charges is not None and t not in self.total_charges:
                        continue
                    sec = self.sectors.setdefault(t, dict(base={}, dim=0, rows=[]))
                    sec["base"][c0] = sec["dim"]
                    i0 = np.repeat(np.arange(nb[0][c0]), nb[1][c1])
                    i1 = np.tile(np.arange(nb[1][c1]), nb[0][c0])
                    sec["rows"].append((off0[c0] + i0) * tot1 + off1[c1] + i1)
                    sec["dim"] += nb[0][c0] * nb[1][c1]
            for t, sec in self.sectors.items():
                sec["rows"] = torch.as_tensor(np.concatenate(sec["rows"]), dtype=torch.int64, device=dev)
                sec["H"] = torch.zeros((sec["dim"], sec["dim"]), **f64)
            self.H = None
        fin = GroupedGemm(dev)
        i32 = dict(dtype=torch.int32, device=dev)
        n_ref0 = spaces[0].n_elec_ref
        n_ref1 = spaces[1].n_elec_ref
        self.block_keys = []
        self.final_tasks = []
        for ci0 in chg[0]:
            for ci1 in chg[1]:
                for cj0 in chg[0]:
                    for cj1 in chg[1]:
                        if ci0 + ci1 != cj0 + cj1:
                            continue
                        if self.total_charges is not None and ci0 + ci1 not in self.total_charges:
                            continue
                        d0 = ci0 - cj0
                        if abs(d0) > 2:
                            continue
                        sgn = -1.0 if ((n_ref0 - cj0) % 2) else 1.0
                        if convention == "general" and abs(d0) == 1:
                            sign2 = -1.0 if ((n_ref1 - ci1) % 2) else 1.0
                            gauge = sign2 * sgn
                        else:
                            gauge = 1.0
                        k0, k1 = (ci0, cj0), (ci1, cj1)
                        segs = []
                        try:
                            if d0 == 0:
                                segs.append((self.P[("v0101", ci0)], N[1] ** 2, rho[1]["ca"][k1], N[1] ** 2, N[1] ** 2, 1.0))
                            elif d0 == -1:
                                segs.append((self.P[("p1", 0, ci0, cj0)], N[1], rho[1]["a"][k1], N[1], N[1], sgn))
                                segs.append((rho[0]["c"][k0], N[0], self.P[("pcaa", 1, ci1, cj1)], N[0], N[0], -sgn))
                            elif d0 == 1:
                                segs.append((rho[0]["a"][k0], N[0], self.P[("p1", 1, ci1, cj1)], N[0], N[0], -sgn))
                                segs.append((self.P[("pcaa", 0, ci0, cj0)], N[1], rho[1]["c"][k1], N[1], N[1], sgn))
                            elif d0 == -2:
                                segs.append((self.P[("pcc", 0, ci0, cj0)], N[1] ** 2, rho[1]["aa"][k1], N[1] ** 2, N[1] ** 2, 1.0))
                            elif d0 == 2:
                                segs.append((rho[0]["aa"][k0], N[0] ** 2, self.P[("pcc", 1, ci1, cj1)], N[0] ** 2, N[0] ** 2, 1.0))
                        except KeyError:
                            continue     # a density is absent (charge not present): block is zero
                        segs = [(A, lda, B, ldb, K, a * gauge) for (A, lda, B, ldb, K, a) in segs]
                        ni0, nj0, ni1, nj1 = nb[0][ci0], nb[0][cj0], nb[1][ci1], nb[1][cj1]
                        M, Nn = ni0 * nj0, ni1 * nj1
                        i0 = np.repeat(np.arange(ni0), nj0)
                        j0 = np.tile(np.arange(nj0), ni0)
                        i1 = np.repeat(np.arange(ni1), nj1)
                        j1 = np.tile(np.arange(nj1), ni1)
                        if layout == "product":
                            Cbuf, ldc = self.H, self.dim[1]
                            rowA = torch.as_tensor((off0[ci0] + i0) * tot1, **i32)
                            colA = torch.as_tensor((off0[cj0] + j0) * tot1, **i32)
                            rowB = torch.as_tensor(off1[ci1] + i1, **i32)
                            colB = torch.as_tensor(off1[cj1] + j1, **i32)
                        else:
                            sec = self.sectors[ci0 + ci1]
                            Cbuf, ldc = sec["H"], sec["dim"]
                            rowA = torch.as_tensor(sec["base"][ci0] + i0 * ni1, **i32)
                            colA = torch.as_tensor(sec["base"][cj0] + j0 * nj1, **i32)
                            rowB = torch.as_tensor(i1, **i32)
                            colB = torch.as_tensor(j1, **i32)
                        diagA = torch.as_tensor(((ci0 == cj0) & (i0 == j0)).astype(np.uint8), device=dev)
                        diagB = torch.as_tensor(((ci1 == cj1) & (i1 == j1)).astype(np.uint8), device=dev)
                        DA = DB = None
                        if d0 == 0:
                            src = self.FULLD if output == "full" else self.DU
                            DA = src[0].get(ci0)
                            DB = src[1].get(ci1)
                        fin.add(M, Nn, segs, Cbuf, ldc, mode=2,
                                maps=(rowA, colA, rowB, colB, diagA, diagB), DA=DA, DB=DB)
                        self.block_keys.append((ci0, ci1, cj0, cj1))
                        self.final_tasks.append(dict(key=(ci0, ci1, cj0, cj1), segs=segs, M=M, N=Nn, C=Cbuf, ldc=ldc,
                                                     dims=(ni0, nj0, ni1, nj1),
                                                     maps=(rowA, colA, rowB, colB, diagA, diagB), DA=DA, DB=DB))
        self.fin = fin.finalize()

        # ---- split-precision tensor-core variant of both launches ----
        self.tc = self.precision in (_lib.BF16X3, _lib.TF32X3)
        if self.tc:
            reg = registry if registry is not None else SplitRegistry(precision, dev)
            tag = "%x" % id(self)
            self._grp_P, self._grp_W = "P" + tag, "W" + tag
            p_ptrs = {t.data_ptr() for t in self.P.values()}
            w_ptrs = {t.data_ptr() for t in W.values()}
            # every density builder's blocks form one split group, shared by the plans that hold it
            b_of = {}
            for b in self.builders:
                if getattr(b, "split_group", None) is None:
                    b.split_group = "in%x" % id(b)
                for blocks in b.rho.values():
                    for t_ in blocks.values():
                        b_of[t_.data_ptr()] = b.split_group
            self._grp_in = set()

            def grp(t):
                p_ = t.data_ptr()
                if p_ in p_ptrs:
                    return self._grp_P
                if p_ in w_ptrs:
                    return self._grp_W
                g_ = b_of.get(p_, "in" + tag)
                self._grp_in.add(g_)
                return g_

            pre_tc = TCGroupedGemm(reg)
            for out, segs_ in self.pre_specs:
                M_, X_ = out.shape
                tsegs = [(r_, r_.numel() // M_, W[wk], W[wk].shape[1], W[wk].shape[1], 1.0) for r_, wk in segs_]
                pre_tc.add(M_, X_, tsegs, out, X_, mode=1,
                           groups=[(grp(a[0]), grp(a[2])) for a in tsegs])
            pre64 = GroupedGemm(dev)
            for (M_, N_, segs_, out_, ldc_, sk_) in mono:
                pre64.add(M_, N_, segs_, out_, ldc_, mode=1, splitk=sk_)
            fin_tc = TCGroupedGemm(reg)
            for t in self.final_tasks:
                fin_tc.add(t["M"], t["N"], t["segs"], t["C"], t["ldc"], mode=2, maps=t["maps"], DA=t["DA"],
                           DB=t["DB"], groups=[(grp(a[0]), grp(a[2])) for a in t["segs"]])
            reg.upload()
            reg.split(self._grp_W)
            self._grp_in = sorted(self._grp_in)
            self.reg, self.pre_tc, self.pre64, self.fin_tc = reg, pre_tc.finalize(), pre64.finalize(), fin_tc.finalize()
            if autotune:
                self.pre_tc.autotune()
                self.fin_tc.autotune()

    # ------------------------------------------------------------------------------------
    def _integral_matrices(self, ints):
        """Integral blocks with the diagram prefactors folded in, in B-role layout [x, y]
        (y contracted, contiguous): v0101 (4 V_0101, hermitian-XRCC/diagrams/SV_2mer_0.py:28),
        h1 (T + U of t01/u001-type transfers, ST_2mer_0.py:28, SU_2mer_0.py:37-118), cca and
        caa (2 V of v0001/v0100 with their phases, SV_2mer_0.py:39,50), cc (v0011,
        SV_2mer_0.py:61), hmm and u100 (the monomer and u100 terms)."""
        N = self.N
        W = {}
        W["v0101"] = (4.0 * ints.V(0, 1, 0, 1).permute(1, 3, 0, 2).reshape(N[1] ** 2, N[0] ** 2)).contiguous()
        for m, o in ((0, 1), (1, 0)):
            h_mo = ints.T(m, o) + ints.U(m, m, o) + ints.U(o, m, o)
            W[("h1", m)] = h_mo.t().contiguous()                                                   # [q, p]
            W[("cca", m)] = (-2.0 * ints.V(m, m, m, o).permute(3, 0, 1, 2).reshape(N[o], N[m] ** 3)).contiguous()
            W[("caa", m)] = (2.0 * ints.V(m, o, m, m).permute(1, 0, 3, 2).reshape(N[o], N[m] ** 3)).contiguous()
            W[("cc", m)] = ints.V(m, m, o, o).permute(3, 2, 0, 1).reshape(N[o] ** 2, N[m] ** 2).contiguous()
            W[("hmm", m)] = (ints.T(m, m) + ints.U(m, m, m)).reshape(1, N[m] ** 2).contiguous()
            W[("u100", m)] = ints.U(o, m, m).reshape(1, N[m] ** 2).contiguous()
            if getattr(self, "monomer_2e", "sigma") == "ccaa":
                # v0000 on a stored rho^ccaa[i, j, p, q, s, r]: the weights V_pqrs in (p, q, s, r) order
                W[("vmmmm", m)] = ints.V(m, m, m, m).permute(0, 1, 3, 2).reshape(1, N[m] ** 4).contiguous()
        return W

    def set_integrals(self, ints):
        """Replace the integrals in place: every launch table keeps its pointers, so a captured
        CUDA graph stays valid.  Enqueued on the current stream (no host synchronisation)."""
        for k, w in self._integral_matrices(ints).items():
            self.W[k].copy_(w)
        for m in (0, 1):
            for c, sg in self.sigma[m].items():
                sg.set_V(ints.V(m, m, m, m))
        self.sigma_batch.refresh_W()
        if self.tc:
            self.reg.split(self._grp_W)
        self.ints = ints

    def integral_set(self, ints):
        """Device copies of everything set_integrals writes for these integrals (the integral
        matrices and each monomer sigma's V and pair-class W), for load_integral_set: one plan
        then serves many fragment pairs of a larger system, each with its own prepared set."""
        S = {("W", k): w.contiguous() for k, w in self._integral_matrices(ints).items()}
        for m in (0, 1):
            Vm = ints.V(m, m, m, m).contiguous()
            S[("sV", m)] = Vm.clone()            # never an alias of a cached block
            for c, sg in self.sigma[m].items():
                if sg.pl is not None:
                    for k, (u, v) in enumerate(sg._uv):
                        S[("sW", m, c, k)] = (4.0 * Vm[u[:, None], v[:, None], u[None, :], v[None, :]]).contiguous()
        return S

    def load_integral_set(self, S):
        """set_integrals from a prepared integral_set: device-to-device copies and the operand
        splits of the split-precision paths, nothing else, on the current stream."""
        for k, w in self.W.items():
            w.copy_(S[("W", k)])
        for m in (0, 1):
            for c, sg in self.sigma[m].items():
                sg.V.copy_(S[("sV", m)])
                if sg.pl is not None:
                    for k, W in enumerate(sg.W):
                        W.copy_(S[("sW", m, c, k)])
                    if sg.reg is not None:
                        sg.reg.split("sigW")
        self.sigma_batch.refresh_W()
        if self.tc:
            self.reg.split(self._grp_W)

    def set_coeffs(self, coeffs):
        """Copy new state coefficients {charge: (n_states, n_conf)} per fragment into the plan."""
        for m in (0, 1):
            for c in self.charges[m]:
                self.coeffs[m][c].copy_(coeffs[m][c], non_blocking=True)

    def launch(self, build_densities=True, split_inputs=True):
        """Enqueue the whole build (densities, sigma, precontractions, final blocks); with
        build_densities=False the density builders are taken as already built, with
        split_inputs=False (split precision) their split copies too."""
        for m in (0, 1):
            if build_densities:
                self.builders[m].build(self.coeffs[m])
        self.sigma_batch.run()
        for m in (0, 1):
            for c, sg in self.sigma[m].items():
                if sg.pl is None:
                    sg.run_sigma(self.builders[m].zT[c])
        _lib.zero_(self.arena.buf)
        s = stream_ptr()
        if self.mono_gemv_tasks is not None:
            gtd, n_g, rows8 = self.mono_gemv_tasks
            call("xrh_gemv_rows_grouped", ptr(gtd), n_g, rows8, s)
        if self.mono_abt is not None:
            atd, n_a, ctas = self.mono_abt
            call("xrh_abt_grouped", _lib.FP64, ptr(atd), n_a, ctas, s)
        if self.tc:
            if split_inputs:
                for g in self._grp_in:
                    self.reg.split(g)
            self.pre_tc.run()
            self.pre64.run()
            self.reg.split(self._grp_P)
            self.fin_tc.run()
        else:
            self.pre.run()
            self.fin.run()

    def build(self, coeffs=None):
        """coeffs: two {charge: CUDA float64 (n_states, n_conf)} dicts -> fills self.H."""
        if coeffs is not None:
            self.set_coeffs(coeffs)
        self.launch()
        return self.H

    def H1(self):
        out = []
        for m in (0, 1):
            tot = self.tot[m]
            h = torch.zeros((tot, tot), dtype=torch.float64, device=self.device)
            acc = 0
            for c in self.charges[m]:
                n = self.n_states[m][c]
                if c in self.H1blk[m]:
                    h[acc:acc + n, acc:acc + n] = self.H1blk[m][c].view(n, n)
                acc += n
            out.append(h)
        return out

    @property
    def flops(self):
        return self.pre.flops + self.fin.flops + self.mono_flops

    def check_status(self):
        """Raise if a bounded device wait of the tensor-core kernels timed out (syncs)."""
        if self.tc:
            self.pre_tc.check()
            self.fin_tc.check()
        for b in self.builders:
            if hasattr(b, "check"):
                b.check()
        self.sigma_batch.check()


def lowest_eigenpairs(H, k=5, tol=1e-10):
    """Lowest k eigenvalues (numpy) and eigenvectors (device) of the symmetric excitonic H
    in FP64 on the GPU, by this library's Lanczos loop (eigen.lowest_eigenpairs)."""
    from .eigen import lowest_eigenpairs as _lanczos_pairs
    return _lanczos_pairs(H, k=k, tol=tol)
