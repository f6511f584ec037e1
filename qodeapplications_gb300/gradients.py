"""Adjoint of the XR-H build: energy gradients w.r.t. fragment-state coefficients and
orbital rotations, on the GPU.

What the reference computes (StateSpaceOptimizer/state_gradients.py:121-244 for the states,
orb_grads.py:976-1000 for the orbitals) is re-derived as one reverse pass of the planned
build.  With d the normalised ground-state eigenvector of the symmetric excitonic H and
E = d^T H d (Hellmann-Feynman), every planned contraction is differentiated in reverse:

  final blocks    C = sum_s alpha_s A_s B_s^T scattered to H  ->  dE/dA_s, dE/dB_s
                  (two small GEMMs each with the ground-state coefficient matrix D)
  delta terms     u100, H1 x 1, 1 x H1                        ->  G_m = D D^T / D^T D blocks
  precontractions P = rho W^T                                 ->  dE/drho, dE/dW
  densities       rho = zb O zk^T (coupling lists)            ->  dE/dz (xrh_density_adjoint)
  monomer 2e      zb M2 zk^T (sigma vectors)                  ->  dE/dz, dE/dV_mmmm (xrh_ccaa_weighted)

dE/dW, dE/dT, dE/dU, dE/dV then give the orbital-rotation gradient by the chain rule of
X' = R^T X R (R = exp(kappa), at kappa = 0 on the current orbitals).  All FP64.
"""
import numpy as np
import torch

from . import _lib
from ._lib import call, ptr, stream_ptr
from .gemm import GroupedGemm, SplitRegistry, TCGroupedGemm
from .hamiltonian import _Arena, _splitk


ADJ_UNIT_MAX = 16     # blocks with at most this many states per side use the lane-per-coupling adjoint
ORBITAL_FUSED = True  # integral derivatives of the orbital gradient by xrh_orbital_terms
GAMMA_TC_MIN = 0      # Gamma pair blocks with n * n_K >= this go to the tensor cores (3 x TF32)

class XRDimerAdjoint:
    def __init__(self, plan, density_adjoint="simt", monomer_terms=False, scratch=None):
        """density_adjoint: 'simt' (the grouped CUDA-core kernel) or 'tc' (tensor cores, split-
        precision plans with at most 64 states per side; exact to the same tolerance but slower
        at 2 x 9 / 10 and 2 x 14 / 60 states: one CTA per SM runs its gather, MMA and atomic
        phases in sequence).
        monomer_terms: every monomer block's G gets -dmono[m][c] dmono[m][c]^T added (the
        vectors self.dmono, zero unless the caller writes them before launch): the reverse pass
        of E - sum_m u_m^T H1_m u_m with dmono = u_m, so a larger system folds its monomer
        energy terms (weighted ground vectors of H1_m) into the pair reverse passes.
        scratch: FP64 device tensors whose memory the transposed density gradients may take
        (they are written and read inside launch() only): working buffers of another
        computation that never runs between the launches of one reverse pass, on the same
        stream; what does not fit is allocated."""
        assert plan.output == "full", "the adjoint differentiates the full H (H2 + H1 x 1 + 1 x H1)"
        self.plan = plan
        self._spatial_cache = {}
        dev = plan.device
        f64 = dict(dtype=torch.float64, device=dev)
        tot0, tot1 = plan.tot
        self.d = torch.zeros(tot0 * tot1, **f64)
        Dflat = self.d
        off0, off1 = plan.offsets
        ns, chg, N = plan.n_states, plan.charges, plan.N

        arena = _Arena(dev)
        req = {}

        def want(key, shape):
            if key not in req:
                req[key] = arena.request(shape)

        # gradients of every operand that appears in the plan
        operands = {}
        for t in plan.final_tasks:
            for (A, lda, B, ldb, K, a) in t["segs"]:
                operands[A.data_ptr()] = A
                operands[B.data_ptr()] = B
        for out, segs in plan.pre_specs:
            operands[out.data_ptr()] = out
            for rho_t, _wk in segs:
                operands[rho_t.data_ptr()] = rho_t
        for m in (0, 1):
            for c in plan.H1blk[m]:
                operands[plan.builders[m].rho["ca"][(c, c)].data_ptr()] = plan.builders[m].rho["ca"][(c, c)]
        for p_, t_ in operands.items():
            want(("g", p_), tuple(t_.shape))
        for wk, Wt in plan.W.items():
            want(("gW", wk), tuple(Wt.shape))
        gp_total = [0, 0]
        for m in (0, 1):
            want(("gmono1", m), (1, N[m] ** 2))
            want(("Gamma", m), (N[m] ** 4,))
            for c in plan.charges[m]:
                want(("gzT", m, c), (plan.spaces[m].n_conf[c], ns[m][c]))
                if c in plan.H1blk[m]:
                    want(("gblk", m, c), (ns[m][c], ns[m][c]))
                    want(("YT", m, c), (plan.spaces[m].n_conf[c], ns[m][c]))
                    sg = plan.sigma[m][c]
                    if sg.pl is not None:
                        for k, cl in enumerate(sg.pl["classes"]):
                            gp_total[m] += cl["n_p"] ** 2
        for m in (0, 1):
            if gp_total[m]:
                want(("Gpairs", m), (gp_total[m],))      # the pair blocks of Gamma, one buffer per fragment
        for i, t in enumerate(plan.final_tasks):
            ni0, nj0, ni1, nj1 = t["dims"]
            for s, (A, lda, B, ldb, K, a) in enumerate(t["segs"]):
                want(("Y", i, s), (ni0, nj1 * K))
                want(("Z", i, s), (ni1, nj0 * K))
        views = arena.allocate()
        self.arena = arena
        G = {k: views[v] for k, v in req.items()}
        self.G = G
        grad_of = {p_: G[("g", p_)] for p_ in operands}
        self.grad_of = grad_of

        # the adjoint contractions run in FP32 (FP64 sums) on the split-precision paths
        gprec = "fp64" if plan.dens_precision == "fp64" else "fp32"
        self.dmono = None
        if monomer_terms:
            self.dmono = [{c: torch.zeros(ns[m][c], **f64) for c in plan.H1blk[m]} for m in (0, 1)]
        # ---- launch 1: G blocks, Y and Z per final segment ----
        L1 = GroupedGemm(dev, gprec)
        for m in (0, 1):
            for c in plan.H1blk[m]:
                n = ns[m][c]
                gb = G[("gblk", m, c)]
                # - u u^T of a folded monomer term (one K = 1 segment of the same task)
                extra = [(self.dmono[m][c], 1, self.dmono[m][c], 1, 1, -1.0)] if monomer_terms else []
                if m == 0:      # G0[i,j] = sum_b D[off+i, b] D[off+j, b]
                    Dsub = Dflat[off0[c] * tot1:]
                    L1.add(n, n, [(Dsub, tot1, Dsub, tot1, tot1, 1.0)] + extra, gb, n)
                else:           # G1[i,j] = sum_a D[a, off+i] D[a, off+j]
                    Dsub = Dflat[off1[c]:]
                    L1.add(n, n, [(Dsub, tot1, Dsub, tot1, tot0, 1.0, 3, 0, 0)] + extra, gb, n)
        self.final_adj = []
        for i, t in enumerate(plan.final_tasks):
            ci0, ci1, cj0, cj1 = t["key"]
            ni0, nj0, ni1, nj1 = t["dims"]
            Di = Dflat[off0[ci0] * tot1 + off1[ci1]:]     # rows i0, cols i1
            Dj = Dflat[off0[cj0] * tot1 + off1[cj1]:]     # rows j0, cols j1
            for s, (A, lda, B, ldb, K, a) in enumerate(t["segs"]):
                Y, Z = G[("Y", i, s)], G[("Z", i, s)]
                # Y[i0, (j1,x)] = a sum_i1 D[i0,i1] B[(i1,j1),x]
                L1.add(ni0, nj1 * K, [(Di, tot1, B, nj1 * K, ni1, a, 2, 0, 0)], Y, nj1 * K)
                # Z[i1, (j0,x)] = a sum_i0 D[i0,i1] A[(i0,j0),x]
                L1.add(ni1, nj0 * K, [(Di, tot1, A, nj0 * K, ni0, a, 3, 0, 0)], Z, nj0 * K)
                self.final_adj.append((A, B, K, Y, Z, Dj, (ni0, nj0, ni1, nj1)))
        self.L1 = L1.finalize()

        # ---- launch 2: dA, dB (batched), monomer pieces ----
        L2 = GroupedGemm(dev, gprec)
        for (A, B, K, Y, Z, Dj, (ni0, nj0, ni1, nj1)) in self.final_adj:
            gA, gB = grad_of[A.data_ptr()], grad_of[B.data_ptr()]
            # dA[(i0,j0),x] += sum_j1 D[j0,j1] Y[i0,(j1,x)]          (batch over i0)
            L2.add(nj0, K, [(Dj, tot1, Y, K, nj1, 1.0, 2, 0, nj1 * K)], gA, K, mode=1, batch=ni0, sC=nj0 * K)
            # dB[(i1,j1),x] += sum_j0 D[j0,j1] Z[i1,(j0,x)]          (batch over i1)
            L2.add(nj1, K, [(Dj, tot1, Z, K, nj0, 1.0, 3, 0, nj0 * K)], gB, K, mode=1, batch=ni1, sC=nj1 * K)
        for m in (0, 1):
            for c in plan.H1blk[m]:
                n = ns[m][c]
                gb = G[("gblk", m, c)]
                ca = plan.builders[m].rho["ca"][(c, c)]
                gca = grad_of[ca.data_ptr()]
                N2 = N[m] ** 2
                # d rho^ca += g (x) (h_mm + U_omm)  (rank one, K = 1)
                L2.add(n * n, N2, [(gb, 1, plan.W[("hmm", m)], N2, 1, 1.0, 2, 0, 0),
                                   (gb, 1, plan.W[("u100", m)], N2, 1, 1.0, 2, 0, 0)], gca, N2, mode=1)
                # d(h_mm) = d(U_omm) += sum_ij g[i,j] rho^ca[i,j,:]
                L2.add(1, N2, [(gb, n * n, ca, N2, n * n, 1.0, 2, 0, 0)], G[("gmono1", m)], N2, mode=1,
                       splitk=_splitk(n * n, 256, 16))
                # e2 = z M2 z^T: dz^T[P, I] += 2 sum_J sigma^T[J, P] g[I, J]
                sg = plan.sigma[m][c]
                nconf = plan.spaces[m].n_conf[c]
                L2.add(nconf, n, [(sg.sigmaT, nconf, gb, n, n, 2.0, 1, 0, 0)], G[("gzT", m, c)], n, mode=1)
                # Y^T = z^T g^T for the two-particle density of the weighted ensemble
                L2.add(nconf, n, [(plan.builders[m].zT[c], n, gb, n, n, 1.0)], G[("YT", m, c)], n)
        self.L2 = L2.finalize()

        # ---- launch 3: precontraction adjoint ----
        # every gradient buffer's writers: outputs written by this launch alone take plain stores
        writers = {}
        for (A, B, K, Y, Z, Dj, _dims) in self.final_adj:
            for t_ in (A, B):
                writers[t_.data_ptr()] = writers.get(t_.data_ptr(), 0) + 1
        for m in (0, 1):
            for c in plan.H1blk[m]:
                p_ = plan.builders[m].rho["ca"][(c, c)].data_ptr()
                writers[p_] = writers.get(p_, 0) + 1
        for out, segs in plan.pre_specs:
            for rho_t, wk in segs:
                writers[rho_t.data_ptr()] = writers.get(rho_t.data_ptr(), 0) + 1
        self.l3_tc = plan.tc
        self.l3_T = []
        self._l3_tr = None
        self._mirror_adj_launch = None
        self._gamma_scatter = None
        self._gam_tr = None
        if plan.tc:
            # tensor cores (split precision, FP32 chunk sums): d rho = dP W on K-major W^T; dW = dP^T rho
            # on rho^T, which the density build leaves in its pre-transpose buffer
            rhoT_of = {}
            for m in (0, 1):
                b = plan.builders[m]
                for (op, bc, kc), tmp in b._tmp.items():
                    rt = b.rho[op][(bc, kc)]
                    rhoT_of[rt.data_ptr()] = tmp.view(plan.spaces[m].couplings[(op, bc, kc)].K, -1)
            pname = {v: k for k, v in _lib.PRECISIONS.items()}[plan.precision]
            self.reg3 = SplitRegistry(pname, dev)
            L3 = TCGroupedGemm(self.reg3)
            WT, gPT = {}, {}
            for out, segs in plan.pre_specs:
                gP = grad_of[out.data_ptr()]
                M, X = out.shape
                if gP.data_ptr() not in gPT:
                    gPT[gP.data_ptr()] = torch.empty((X, M), **f64)
                    self.l3_T.append((gP, gPT[gP.data_ptr()]))
                gpt = gPT[gP.data_ptr()]
                for rho_t, wk in segs:
                    Wt = plan.W[wk]
                    Yk = Wt.shape[1]
                    if wk not in WT:
                        WT[wk] = torch.empty((Yk, X), **f64)
                        self.l3_T.append((Wt, WT[wk]))
                    grho = grad_of[rho_t.data_ptr()]
                    mode = 0 if writers[rho_t.data_ptr()] == 1 else 1
                    L3.add(M, Yk, [(gP, X, WT[wk], X, X, 1.0)], grho, Yk, mode=mode, groups=[("g", "g")])
                    L3.add(X, Yk, [(gpt, M, rhoT_of[rho_t.data_ptr()], M, M, 1.0)], G[("gW", wk)], Yk, mode=1,
                           groups=[("g", "rhoT")])
            self.reg3.upload()
            self.L3 = L3.finalize().autotune()
        else:
            L3 = GroupedGemm(dev, gprec)
            for out, segs in plan.pre_specs:
                gP = grad_of[out.data_ptr()]
                M, X = out.shape
                for rho_t, wk in segs:
                    Wt = plan.W[wk]
                    Yk = Wt.shape[1]
                    grho = grad_of[rho_t.data_ptr()]
                    # d rho[m, y] += sum_x dP[m, x] W[x, y]
                    mode = 0 if writers[rho_t.data_ptr()] == 1 else 1
                    L3.add(M, Yk, [(gP, X, Wt, Yk, X, 1.0, 2, 0, 0)], grho, Yk, mode=mode)
                    # dW[x, y] += sum_m dP[m, x] rho[m, y]
                    L3.add(X, Yk, [(gP, X, rho_t, Yk, M, 1.0, 3, 0, 0)], G[("gW", wk)], Yk, mode=1,
                           splitk=_splitk(M, 256, 32))
            self.L3 = L3.finalize()

        # ---- launch 4 inputs: transposed density gradients for the coupling-list adjoint ----
        # (FP32 accumulation buffers on the split-precision paths)
        self.prec32 = plan.dens_precision == "fp32"
        self.gz32, self.Gamma32 = None, None
        if self.prec32:
            self.gz32 = [{c: torch.zeros((plan.spaces[m].n_conf[c], ns[m][c]), dtype=torch.float32, device=dev)
                          for c in plan.charges[m]} for m in (0, 1)]
            self.Gamma32 = [torch.zeros(N[m] ** 4, dtype=torch.float32, device=dev) for m in (0, 1)]
        # ---- two-particle density of the monomer two-electron term through (n-2)-electron
        # intermediates: Gamma[pq, rs] = sum_(I, K) D_zb[I, (K, pq)] D_Y[I, (K, rs)] per spin
        # class (D_zb is the forward pass's pair scatter of the same coefficients) ----
        self.gamma_ri, self.gamma_old = [], []
        Lg = GroupedGemm(dev, gprec)
        self.gam_reg = SplitRegistry("tf32x3", dev)
        Lgt = TCGroupedGemm(self.gam_reg)
        self.gam_T = []
        self.gam_scatter = []
        for m in (0, 1):
            off = 0
            flat_all = []
            for c in plan.H1blk[m]:
                sg = plan.sigma[m][c]
                if sg.pl is None:
                    self.gamma_old.append((m, c))
                    continue
                Dy = torch.zeros_like(sg.D)
                n = plan.n_states[m][c]
                Nm = N[m]
                for k, cl in enumerate(sg.pl["classes"]):
                    nK, npr = cl["n_K"], cl["n_p"]
                    b = n * cl["base"]
                    Dyc = Dy[b:b + n * nK * npr].view(n * nK, npr)
                    Gp = self.G[("Gpairs", m)][off:off + npr * npr].view(npr, npr)
                    off += npr * npr
                    if sg.tc and n * nK >= GAMMA_TC_MIN:
                        # Gamma_c = D^T Dy on the tensor cores (3 x TF32), from K-major transposed
                        # copies; n states x n_K intermediates is a long K: split-K, FP64 atomics
                        DT = torch.empty((npr, n * nK), **f64)
                        DyT = torch.empty((npr, n * nK), **f64)
                        self.gam_T += [(sg.Dc[k], DT), (Dyc, DyT)]
                        Lgt.add(npr, npr, [(DT, n * nK, DyT, n * nK, n * nK, 1.0)], Gp, npr, mode=1,
                                groups=[("gam", "gam")])
                    else:                 # short K: the SIMT GEMM reads both operands transposed
                        Lg.add(npr, npr, [(sg.Dc[k], npr, Dyc, npr, n * nK, 1.0, 3, 0, 0)], Gp, npr, mode=1,
                               splitk=_splitk(n * nK, 256, 64))
                    pq = cl["u"] * Nm + cl["v"]
                    flat_all.append((pq[:, None] * Nm * Nm + pq[None, :]).reshape(-1))
                self.gamma_ri.append((m, c, sg, Dy))
            if flat_all:
                idx = torch.as_tensor(np.concatenate(flat_all), dtype=torch.int64, device=dev)
                self.gam_scatter.append((m, idx, self.G[("Gpairs", m)][:off]))
        self.Lgamma = Lg.finalize()
        self.gam_reg.upload()
        self.Lgamma_tc = Lgt.finalize().autotune()

        pool = [t.reshape(-1) for t in (scratch or ())]
        pool_off = [0] * len(pool)

        def take(n):
            """n FP64 elements from the scratch tensors (256-byte aligned pieces), else new."""
            n_al = (n + 31) // 32 * 32
            for i, t_ in enumerate(pool):
                if t_.dtype == torch.float64 and t_.data_ptr() % 256 == 0 and pool_off[i] + n_al <= t_.numel():
                    v = t_[pool_off[i]:pool_off[i] + n]
                    pool_off[i] += n_al
                    return v
            return torch.empty(n, **f64)

        self.dens_adj = []
        self.mirror_adj = []      # (d rho of a mirrored block, d rho of its partner, partner dims, N, L)
        self.im_adj = []          # intermediate-determinant builders: (builder, density gradients, gzT)
        for m in (0, 1):
            b = plan.builders[m]
            if plan.dens_precision == "im":
                grads = {}
                for op, blocks in b.rho.items():
                    for key, rt in blocks.items():
                        if rt.data_ptr() in grad_of:
                            grads[(op,) + key] = grad_of[rt.data_ptr()]
                b.setup_adjoint()
                self.im_adj.append((b, grads, {c: G[("gzT", m, c)] for c in plan.charges[m]}))
                continue
            for (op, bc, kc), cp in plan.spaces[m].couplings.items():
                rt = b.rho[op][(bc, kc)]
                if rt.data_ptr() not in grad_of:
                    continue
                mir = getattr(b, "mirror", {}).get((op, bc, kc))
                if mir is not None and b.rho[mir[0]][mir[1:]].data_ptr() in grad_of:
                    # a mirrored block: its gradient folds into the partner's before the adjoint
                    self.mirror_adj.append((grad_of[rt.data_ptr()], grad_of[b.rho[mir[0]][mir[1:]].data_ptr()],
                                            rt.shape[1], rt.shape[0], plan.N[m], len(op)))
                    continue
                gT = take(cp.K * rt.shape[0] * rt.shape[1])
                self.dens_adj.append((m, op, bc, kc, cp, rt, grad_of[rt.data_ptr()], gT))
        self.dens_adj_all = list(self.dens_adj)
        self._fold = None
        # FP32 path: every block of a fragment in one grouped launch, on the tensor cores when
        # every block has at most 64 states per side (else the CUDA-core kernel)
        self.dens_adj_groups = []
        self.dens_adj_tc = []
        self.tc_status = torch.zeros(1, dtype=torch.int32, device=dev)
        use_tc = (density_adjoint == "tc" and self.prec32 and plan.tc and
                  all(e[5].shape[0] <= 64 and e[5].shape[1] <= 64 for e in self.dens_adj))
        if density_adjoint == "tc" and not use_tc:
            raise ValueError("the tensor-core density adjoint needs a split-precision plan and <= 64 states")
        if use_tc:
            self._canonicalize()
            self.z_split = []
            for m in (0, 1):
                bld = plan.builders[m]
                zs = {c: (torch.zeros((plan.spaces[m].n_conf[c], 64), dtype=torch.int32, device=dev),
                          torch.zeros((plan.spaces[m].n_conf[c], 64), dtype=torch.int32, device=dev))
                      for c in plan.charges[m]}
                self.z_split.append((bld, zs))
                entries = [e for e in self.dens_adj if e[0] == m]
                if not entries:
                    continue
                tasks = np.zeros(len(entries), dtype=_lib.DENS_ADJ_TC_TASK_DTYPE)
                begin = 0
                for i, (_m, op, bc, kc, cp, rt, grho, gT) in enumerate(entries):
                    t = tasks[i]
                    t["idx_ptr"], t["P"], t["Q"], t["sign"] = (cp.idx_ptr.data_ptr(), cp.P.data_ptr(),
                                                               cp.Q.data_ptr(), cp.sign.data_ptr())
                    t["zbh"], t["zbl"] = zs[bc][0].data_ptr(), zs[bc][1].data_ptr()
                    t["zkh"], t["zkl"] = zs[kc][0].data_ptr(), zs[kc][1].data_ptr()
                    t["gT"] = gT.data_ptr()
                    t["gzb"], t["gzk"] = self.gz32[m][bc].data_ptr(), self.gz32[m][kc].data_ptr()
                    t["K"], t["nb"], t["nk"], t["cta_begin"] = cp.K, rt.shape[0], rt.shape[1], begin
                    begin += cp.K
                self.dens_adj_tc.append((torch.from_numpy(tasks.view(np.uint8).copy()).to(dev), len(entries), begin))
        elif self.prec32:
            from .densities import _coupling_units
            self.dens_adj_units = []
            for m in (0, 1):
                bld = plan.builders[m]
                # blocks of at most 16 states per side: lane per coupling, dE/drho read in place
                small = [e for e in self.dens_adj
                         if e[0] == m and e[5].shape[0] <= ADJ_UNIT_MAX and e[5].shape[1] <= ADJ_UNIT_MAX]
                if small:
                    tasks = np.zeros(len(small), dtype=_lib.DENS_ADJ_TASK_DTYPE)
                    ulist = []
                    for i, (_m, op, bc, kc, cp, rt, grho, gT) in enumerate(small):
                        t = tasks[i]
                        t["idx_ptr"], t["P"], t["Q"], t["sign"] = (cp.idx_ptr.data_ptr(), cp.P.data_ptr(),
                                                                   cp.Q.data_ptr(), cp.sign.data_ptr())
                        t["zb32"], t["zk32"] = bld.zbT32[bc].data_ptr(), bld.zT32[kc].data_ptr()
                        t["gT"] = grho.data_ptr()
                        t["gzb"], t["gzk"] = self.gz32[m][bc].data_ptr(), self.gz32[m][kc].data_ptr()
                        t["K"], t["nb"], t["nk"] = cp.K, rt.shape[0], rt.shape[1]
                        un = _coupling_units(cp)[0]
                        un["task"] = i
                        ulist.append(un)
                    units = np.concatenate(ulist)
                    self.dens_adj_units.append((torch.from_numpy(tasks.view(np.uint8).copy()).to(dev), len(small),
                                                torch.from_numpy(units.view(np.uint8).copy()).to(dev), len(units),
                                                max(max(e[5].shape[0], e[5].shape[1]) for e in small)))
                    self.dens_adj = [e for e in self.dens_adj if not any(e is x for x in small)]
                self._canonicalize(m)
                entries = [e for e in self.dens_adj if e[0] == m]
                if not entries:
                    continue
                tasks = np.zeros(len(entries), dtype=_lib.DENS_ADJ_TASK_DTYPE)
                begin = 0
                for i, (_m, op, bc, kc, cp, rt, grho, gT) in enumerate(entries):
                    t = tasks[i]
                    t["idx_ptr"], t["P"], t["Q"], t["sign"] = (cp.idx_ptr.data_ptr(), cp.P.data_ptr(),
                                                               cp.Q.data_ptr(), cp.sign.data_ptr())
                    t["zb32"], t["zk32"] = bld.zbT32[bc].data_ptr(), bld.zT32[kc].data_ptr()
                    t["gT"] = gT.data_ptr()
                    t["gzb"], t["gzk"] = self.gz32[m][bc].data_ptr(), self.gz32[m][kc].data_ptr()
                    t["K"], t["nb"], t["nk"], t["cta_begin"] = cp.K, rt.shape[0], rt.shape[1], begin
                    begin += cp.K
                dev_tasks = torch.from_numpy(tasks.view(np.uint8).copy()).to(dev)
                self.dens_adj_groups.append((dev_tasks, len(entries), begin,
                                             max(e[5].shape[0] for e in entries), max(e[5].shape[1] for e in entries)))
        else:
            self._canonicalize()         # the FP64 per-block adjoint

    def _canonicalize(self, m=None):
        """Entries of self.dens_adj (of fragment m, or all) whose op string has an anticommuting
        pair run over the canonical tuples: their coupling list becomes the canonical one and
        their transposed gradient is folded first (dE/drho_canonical = g - g_swapped)."""
        from .densities import HERMITIAN_PAIR, canonical_couplings, pair_position
        plan = self.plan
        out, fold = [], list(self._fold.keep) if self._fold is not None else []
        for e in self.dens_adj:
            (m_, op, bc, kc, cp, rt, grho, gT) = e
            pp = pair_position(op)
            hermitian_ok = op not in HERMITIAN_PAIR or (bc == kc and getattr(plan.builders[m_], "same_bra_states", False))
            if (m is None or m_ == m) and pp is not None and hermitian_ok and getattr(self, "_antisym", True):
                cc = canonical_couplings(plan.spaces[m_], (op, bc, kc))
                if cc is not None and cc is not cp:
                    e = (m_, op, bc, kc, cc, rt, grho, gT)
                    fold.append((gT, rt.shape[0] * rt.shape[1], plan.N[m_], len(op), pp[0], pp[2]))
            out.append(e)
        self.dens_adj = out
        if fold:
            self._fold = _lib.AntisymRows(fold, plan.device)
        # the work actually done per launch: the canonical lists where they are used
        ids = {(e[0],) + e[1:4]: e for e in out}
        self.dens_adj_all = [ids.get((e[0],) + e[1:4], e) for e in self.dens_adj_all]

    # ------------------------------------------------------------------------------------
    def launch_L3(self):
        """The precontraction adjoint (after launches 1 and 2)."""
        if self.l3_tc:
            if self._l3_tr is None:
                flat = [(a, b) for a, b in self.l3_T if a.is_contiguous() and a.dtype == torch.float64]
                self._l3_tr = _lib.Transposes([(a, b, a.shape[0], a.shape[1]) for a, b in flat], self.plan.device)
                self._l3_rest = [(a, b) for a, b in self.l3_T if not any(a is x for x, _ in flat)]
            self._l3_tr.run()
            for src, dst in self._l3_rest:
                dst.copy_(src.t())
            self.reg3.split("g")
            self.reg3.split("rhoT")
        self.L3.run()

    def launch_density_adjoint(self):
        """dE/dz from the density gradients (after launch 3)."""
        plan = self.plan
        s = stream_ptr()
        for (b, grads, gz) in self.im_adj:
            b.adjoint(grads, gz)
        if self.mirror_adj:
            if self._mirror_adj_launch is None:
                self._mirror_adj_launch = _lib.Mirrors(
                    [(gsrc, gdst, na, nb, Nm, L, 1) for (gsrc, gdst, na, nb, Nm, L) in self.mirror_adj],
                    self.plan.device)
            self._mirror_adj_launch.run()
        for (m, op, bc, kc, cp, rt, grho, gT) in self.dens_adj:
            nb, nk = rt.shape[0], rt.shape[1]
            call("xrh_transpose", ptr(grho), nb * nk, cp.K, ptr(gT), s)
        if self._fold is not None:
            self._fold.run()
        for (m, op, bc, kc, cp, rt, grho, gT) in self.dens_adj:
            if self.prec32:
                break
            nb, nk = rt.shape[0], rt.shape[1]
            bld = plan.builders[m]
            call("xrh_density_adjoint", _lib.PRECISIONS[plan.dens_precision], cp.K, ptr(cp.idx_ptr), ptr(cp.P),
                 ptr(cp.Q), ptr(cp.sign), ptr(bld.zbT[bc]), nb, ptr(bld.zT[kc]), nk, ptr(gT),
                 ptr(self.G[("gzT", m, bc)]), ptr(self.G[("gzT", m, kc)]), s)
        for (tasks, n_t, ctas, mnb, mnk) in self.dens_adj_groups:
            call("xrh_density_adjoint_f32_grouped", ptr(tasks), n_t, ctas, mnb, mnk, s)
        for (tasks, n_t, units, n_u, mx) in getattr(self, "dens_adj_units", ()):
            call("xrh_density_adjoint_f32_units", ptr(tasks), n_t, ptr(units), n_u, mx, 1, s)
        if self.dens_adj_tc:
            for (bld, zs) in self.z_split:
                for c, (zh, zl) in zs.items():
                    n = bld.zT[c].shape[1]
                    call("xrh_split_operand", _lib.TF32X3, ptr(bld.zT[c]), zh.shape[0], n, n, 64, ptr(zh), ptr(zl), s)
            for (tasks, n_t, ctas) in self.dens_adj_tc:
                call("xrh_density_adjoint_tc_grouped", ptr(tasks), n_t, ctas, ptr(self.tc_status), s)

    def launch_gamma(self):
        """Two-particle densities of the monomer two-electron terms (after launch 2)."""
        plan = self.plan
        s = stream_ptr()
        if self.gamma_ri:
            if self._gamma_scatter is None:
                self._gamma_scatter = _lib.PairLaunch(
                    [(sg.pl, sg.off_dev, sg.stride_dev, self.G[("YT", m, c)], Dy, sg.n) for (m, c, sg, Dy) in self.gamma_ri],
                    False, self.plan.device)
            self._gamma_scatter.run()
        if self.gam_T:
            if self._gam_tr is None:
                self._gam_tr = _lib.Transposes([(a, b, a.shape[0], a.shape[1]) for a, b in self.gam_T], self.plan.device)
            self._gam_tr.run()
            self.gam_reg.split("gam")
        self.Lgamma.run()
        self.Lgamma_tc.run()
        for (m, idx, vals) in self.gam_scatter:
            # every pair block of the fragment (all charges) into the N^4 Gamma in one atomic
            # scatter-add
            call("xrh_index_move", idx.numel(), ptr(idx), ptr(vals), ptr(self.G[("Gamma", m)]), 2, s)
        for (m, c) in self.gamma_old:
            sp = plan.spaces[m]
            call("xrh_ccaa_weighted", _lib.FP32 if self.prec32 else _lib.FP64, sp.n_orbs, ptr(sp.masks[c]),
                 sp.n_conf[c], ptr(sp.sorted_masks[c]), ptr(sp.sorted_pos[c]), sp.n_conf[c],
                 ptr(sp.rank_table[c]), sp.table_size[c], ptr(sp.binom),
                 ptr(plan.builders[m].zbT[c]), ptr(self.G[("YT", m, c)]), plan.n_states[m][c],
                 ptr(self.Gamma32[m] if self.prec32 else self.G[("Gamma", m)]), s)

    def check_status(self):
        """Raise if a bounded device wait of the tensor-core launch timed out (syncs)."""
        if self.l3_tc:
            self.L3.check()
        self.Lgamma_tc.check()
        st = int(self.tc_status.item())
        if st != 0:
            raise _lib.XRHError(f"tensor-core density adjoint reported status {st}")

    def launch(self, d):
        """Enqueue the reverse pass for ground-state vector d (device, product order)."""
        plan = self.plan
        s = stream_ptr()
        if d is not None:
            self.d.copy_(d)
        _lib.zero_(self.arena.buf)
        if self.prec32:
            for m in (0, 1):
                for t in self.gz32[m].values():
                    _lib.zero_(t)
                _lib.zero_(self.Gamma32[m])
        self.L1.run()
        self.L2.run()
        self.launch_L3()
        self.launch_density_adjoint()
        self.launch_gamma()


    # ---------------------------------------------------------------------- results ---
    def state_gradient(self):
        """dE/dz[m][charge] (n_states x n_conf), the unconstrained derivative of the lowest
        eigenvalue w.r.t. the CI coefficients (bra and ket occurrences)."""
        if self.prec32:
            return [{c: self.G[("gzT", m, c)].t() + self.gz32[m][c].t().to(torch.float64)
                     for c in self.plan.charges[m]} for m in (0, 1)]
        return [{c: self.G[("gzT", m, c)].t() for c in self.plan.charges[m]} for m in (0, 1)]

    def state_gradient_parts(self):
        """The persistent buffers the state gradient is summed from: [(m, charge, gT, gT32)]
        with gT (n_conf x n, FP64) and gT32 (n_conf x n, FP32, or None): dE/dz = (gT + gT32)^T."""
        out = []
        for m in (0, 1):
            for c in self.plan.charges[m]:
                out.append((m, c, self.G[("gzT", m, c)], self.gz32[m][c] if self.prec32 else None))
        return out

    def integral_gradients(self):
        """dE/dT, dE/dU, dE/dV as supersystem spin-orbital tensors (device, new tensors)."""
        tot = sum(self.plan.N)
        dev = self.plan.device
        dT = torch.zeros((tot, tot), dtype=torch.float64, device=dev)
        dU = torch.zeros((2, tot, tot), dtype=torch.float64, device=dev)
        dV = torch.zeros((tot,) * 4, dtype=torch.float64, device=dev)
        return self._integral_gradients_into(dT, dU, dV)

    def _integral_gradients_into(self, dT, dU, dV):
        """Add dE/dT, dE/dU, dE/dV into zeroed (tot, tot), (2, tot, tot), (tot,)*4 tensors."""
        plan = self.plan
        Ns = plan.N
        off = [0, Ns[0], Ns[0] + Ns[1]]
        sl = [slice(off[m], off[m + 1]) for m in (0, 1)]
        G = self.G
        gw = G[("gW", "v0101")].view(Ns[1], Ns[1], Ns[0], Ns[0])
        dV[sl[0], sl[1], sl[0], sl[1]] += 4.0 * gw.permute(2, 0, 3, 1)
        for m, o in ((0, 1), (1, 0)):
            dh = G[("gW", ("h1", m))].t()
            dT[sl[m], sl[o]] += dh
            dU[m][sl[m], sl[o]] += dh
            dU[o][sl[m], sl[o]] += dh
            dV[sl[m], sl[m], sl[m], sl[o]] += -2.0 * G[("gW", ("cca", m))].view(Ns[o], Ns[m], Ns[m], Ns[m]).permute(1, 2, 3, 0)
            dV[sl[m], sl[o], sl[m], sl[m]] += 2.0 * G[("gW", ("caa", m))].view(Ns[o], Ns[m], Ns[m], Ns[m]).permute(1, 0, 3, 2)
            dV[sl[m], sl[m], sl[o], sl[o]] += G[("gW", ("cc", m))].view(Ns[o], Ns[o], Ns[m], Ns[m]).permute(2, 3, 1, 0)
            g1 = G[("gmono1", m)].view(Ns[m], Ns[m])
            dT[sl[m], sl[m]] += g1
            dU[m][sl[m], sl[m]] += g1
            dU[o][sl[m], sl[m]] += g1
            Gm = G[("Gamma", m)] + self.Gamma32[m].to(torch.float64) if self.prec32 else G[("Gamma", m)]
            Gm = Gm.view(Ns[m], Ns[m], Ns[m], Ns[m])
            Gf = Gm - Gm.permute(1, 0, 2, 3) - Gm.permute(0, 1, 3, 2) + Gm.permute(1, 0, 3, 2)
            dV[sl[m], sl[m], sl[m], sl[m]] += Gf
        return dT, dU, dV

    def _orbital_buffers(self, T, U, V):
        """Persistent buffers and the one-body task table of orbital_gradient for these
        integral tensors (None when t > 64 or the tensors are not contiguous FP64)."""
        t = V.shape[0]
        ok = (t <= 64 and all(x.dtype == torch.float64 and x.is_contiguous() for x in (T, U, V)) and
              tuple(T.shape) == (t, t) and tuple(U.shape[1:]) == (t, t))
        if not ok:
            return None
        key = (T.data_ptr(), U.data_ptr(), V.data_ptr(), t, U.shape[0])
        b = getattr(self, "_orb", None)
        if b is not None and b["key"] == key:
            return b
        dev = V.device
        f64 = dict(dtype=torch.float64, device=dev)
        b = dict(key=key, keep=(T, U, V))
        b["dT"] = torch.zeros((t, t), **f64)
        b["dU"] = torch.zeros((U.shape[0], t, t), **f64)
        b["dV"] = torch.zeros((t,) * 4, **f64)
        b["Gso"] = torch.zeros((t, t), **f64)
        if self.prec32:
            b["A"] = torch.empty((t,) * 4, dtype=torch.float32, device=dev)
            b["B"] = torch.empty((t,) * 4, dtype=torch.float32, device=dev)
        else:
            b["A"] = V
            b["B"] = torch.empty((t,) * 4, **f64)
        # the derivative of every fragment potential U_k equals dT (both receive the same
        # one-electron pieces)
        pairs = [(T, b["dT"], b["Gso"])] + [(U[k], b["dT"], b["Gso"]) for k in range(U.shape[0])]
        b["one_body"] = _one_body_table(pairs, dev)
        b["inputs"] = self._orbital_inputs()
        self._orb = b
        return b

    def _orbital_inputs(self):
        """Host struct of xrh_orbital_terms: the reverse pass's pieces of dE/dT and dE/dV."""
        plan, G = self.plan, self.G
        inp = np.zeros(1, dtype=_lib.ORBITAL_INPUTS_DTYPE)

        def ptr_of(x):
            if not x.is_contiguous() or x.dtype != torch.float64:
                raise ValueError("orbital-gradient pieces must be contiguous FP64 tensors")
            return x.data_ptr()

        inp["gw"] = ptr_of(G[("gW", "v0101")])
        for m in (0, 1):
            inp["h1"][0, m] = ptr_of(G[("gW", ("h1", m))])
            inp["cca"][0, m] = ptr_of(G[("gW", ("cca", m))])
            inp["caa"][0, m] = ptr_of(G[("gW", ("caa", m))])
            inp["cc"][0, m] = ptr_of(G[("gW", ("cc", m))])
            inp["mono1"][0, m] = ptr_of(G[("gmono1", m)])
            inp["gamma64"][0, m] = ptr_of(G[("Gamma", m)])
            inp["gamma32"][0, m] = self.Gamma32[m].data_ptr() if self.prec32 else 0
        inp["N0"], inp["N1"] = plan.N[0], plan.N[1]
        return inp

    def orbital_gradient(self, T, U, V, spatial_index):
        """dE/dkappa (antisymmetric, spatial orbitals) for X' = R^T X R with R = exp(kappa)
        applied to every integral at kappa = 0.  T (tot x tot), U (n_frag x tot x tot),
        V (tot^4) are the current spin-orbital integrals on the device; spatial_index[i]
        is the spatial orbital of spin orbital i."""
        t = V.shape[0]
        b = self._orbital_buffers(T, U, V)
        if b is None:
            dT, dU, dV = self.integral_gradients()
            Gso = T @ dT.t() + T.t() @ dT
            for k in range(U.shape[0]):
                Gso += U[k] @ dU[k].t() + U[k].t() @ dU[k]
        else:
            dT, Gso = b["dT"], b["Gso"]
            prec = _lib.FP32 if self.prec32 else _lib.FP64
            s = stream_ptr()
            if ORBITAL_FUSED:
                # dT and B = Ga + Ga^(rs,pq) element-wise from the reverse pass's pieces
                call("xrh_orbital_terms", b["inputs"].ctypes.data, ptr(dT), ptr(b["B"]), prec, s)
            else:
                dU, dV = b["dU"], b["dV"]
                dT.zero_()
                dU.zero_()
                dV.zero_()
                self._integral_gradients_into(dT, dU, dV)
                Ga = dV - dV.permute(1, 0, 2, 3) - dV.permute(0, 1, 3, 2) + dV.permute(1, 0, 3, 2)
                torch.add(Ga, Ga.permute(2, 3, 0, 1), out=b["B"])
            _lib.zero_(Gso)
            # the one-body terms T dT^T + T^T dT + sum_k U_k dU_k^T + U_k^T dU_k (dU_k = dT) in
            # one launch
            tab, n_tab, ctas = b["one_body"]
            call("xrh_abt_grouped", _lib.FP64, ptr(tab), n_tab, ctas, s)
            # E sees V only through its symmetric part (V_pqrs = -V_qprs = -V_pqsr = V_rspq for
            # real orbitals), so dE/dV may be replaced by its projection on that symmetry; then
            # the four index positions of V' = R^T..R contribute equally: dE/dR = 4 V_(1) Gbar_(1)^T
            # with Gbar = B / 8: a t x t result over t^3 terms, split over CTAs by xrh_abt_small
            # (FP32 products on the split-precision paths)
            if self.prec32:
                call("xrh_f64_to_f32", V.numel(), ptr(V), ptr(b["A"]), s)
            K3 = t ** 3
            call("xrh_abt_small", prec, t, t, K3, ptr(b["A"]), K3, ptr(b["B"]), K3, 0.5, ptr(Gso), s)
        if b is None:
            Ga = dV - dV.permute(1, 0, 2, 3) - dV.permute(0, 1, 3, 2) + dV.permute(1, 0, 3, 2)
            Gbar = 0.125 * (Ga + Ga.permute(2, 3, 0, 1))
            Gso += 4.0 * (V.reshape(t, -1) @ Gbar.reshape(t, -1).t())
        key = (tuple(spatial_index), T.device)
        if key not in self._spatial_cache:     # built on first use, outside any graph capture
            self._spatial_cache[key] = _spin_blocks(spatial_index, T.device)
        so, n_sp, n_spin, out = self._spatial_cache[key]
        # a spatial rotation acts on both spins alike: sum the same-spin spin-orbital pairs of
        # every spatial pair, antisymmetrised (xrh_spin_sum_antisym)
        call("xrh_spin_sum_antisym", n_sp, n_spin, ptr(so), ptr(Gso), Gso.shape[1], ptr(out), stream_ptr())
        return out


def _one_body_table(pairs, device):
    """xrh_abt_grouped (FP64) tasks C += X dX^T and C += X^T dX for each (X, dX, C), all t x t
    row-major."""
    tab = np.zeros(2 * len(pairs), dtype=_lib.ABT_TASK_DTYPE)
    cta = 0
    for i, (X, dX, C) in enumerate(pairs):
        t = X.shape[0]
        for h, flags in enumerate((0, 3)):
            e = tab[2 * i + h]
            e["A"], e["B"], e["C"] = X.data_ptr(), dX.data_ptr(), C.data_ptr()
            e["m"], e["n"], e["K"], e["lda"], e["ldb"], e["alpha"] = t, t, t, t, t, 1.0
            e["cta_begin"], e["flags"] = cta, flags
            cta += int(_lib.lib().xrh_abt_ctas(t))
    return torch.from_numpy(tab.view(np.uint8).copy()).to(device), len(tab), cta


def _spin_blocks(spatial_index, device):
    """so[k, a] = the spin orbital of spatial orbital a in spin block k (alpha, beta), with the
    output buffer of the spatial gradient."""
    n_sp = int(max(spatial_index)) + 1
    so = np.full((2, n_sp), -1, dtype=np.int32)
    seen = {}
    for i, sp in enumerate(spatial_index):
        k = seen.get(sp, 0)
        so[k, sp] = i
        seen[sp] = k + 1
    if (so < 0).any():
        raise ValueError("every spatial orbital needs an alpha and a beta spin orbital")
    out = torch.zeros((n_sp, n_sp), dtype=torch.float64, device=device)
    return torch.from_numpy(so.reshape(-1).copy()).to(device), n_sp, 2, out


def _same_spin(t, spatial_index, device):
    """Mask of spin-orbital pairs with the same spin (alpha block then beta block per fragment)."""
    spins = np.zeros(t, dtype=np.int64)
    seen = {}
    for i, sp in enumerate(spatial_index):
        spins[i] = seen.get(sp, 0)
        seen[sp] = seen.get(sp, 0) + 1
    s = torch.as_tensor(spins, device=device)
    return (s[:, None] == s[None, :]).to(torch.float64)


def tangent_project(g, z):
    """Project dE/dz onto the tangent space of row-orthonormal z (Stiefel manifold)."""
    return g - 0.5 * (g @ z.t() + z @ g.t()) @ z
