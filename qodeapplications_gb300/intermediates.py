"""Transition densities through intermediate determinants (host-side planning).

Every density operator string of the build splits into a creation part and an annihilation
part (the annihilation part acts first):

    rho^op[I, J, cre, ann] = sum_P,Q zb[P, I] <P| cre ann |Q> zk[Q, J]
                           = sum_K C[K, cre, I] A[K, ann, J]
    C[K, cre, I] = sum_P <K| cre^+ |P> zb[P, I],     A[K, ann, J] = sum_Q <K| ann |Q> zk[Q, J]

with K the unique determinant ann|Q> = cre^+|P>.  C and A are index scatters of the state
coefficients (one annihilation, a pair of annihilations, or none: then K is the bra or ket
determinant itself), and the sum over K is a dense GEMM that runs on the tensor cores:

    X[(I, ci), (J, ai)] = sum_K Ct[(I, ci), K] At[(J, ai), K]

rho itself follows by a signed gather of X (the two orders of a pair are one entry of X).
The adjoint is the same three steps reversed: a signed fold of d rho into dX, two GEMMs
(dCt = dX A, dAt = dX^T C) and a gather per determinant (each determinant's entries are its
own, so no atomics).  This replaces the per-coupling outer products of
general-XRCC/density_tensors.c:142-556 (z_contract) on the split-precision paths.

Conventions (those of density_tensors.c, parity = occupied orbitals above):
  single p:      value <K| a_p |X>
  pair u < v:    value <K| a_v a_u |X>   (a_u applied first), pair index v (v - 1) / 2 + u
  rho^aa[p, q] = <P| a_p a_q |Q>:  +pair(q, p) for p > q, -pair(p, q) for p < q
  rho^cc[p, q] = <P| c+_p c+_q |Q> = <Q| a_q a_p |P>:  +pair(p, q) for p < q, -pair(q, p) for p > q
"""
import numpy as np

from .densities import _popcount64

# (creation count, annihilation count) of each density operator string
OP_SPLIT = {"a": (0, 1), "c": (1, 0), "ca": (1, 1), "aa": (0, 2), "cc": (2, 0), "caa": (1, 2), "cca": (2, 1)}


def n_index(k, N):
    return 1 if k == 0 else (N if k == 1 else N * (N - 1) // 2)


def pair_index(u, v):
    """Index of the pair u < v (colexicographic)."""
    return v * (v - 1) // 2 + u


def annihilation_entries(masks, k, N):
    """For every determinant x and every k occupied orbitals (k = 0: the determinant itself;
    1: orbital p; 2: pair u < v): (x, K mask, index, sign of <K| a.. |X>)."""
    masks = np.asarray(masks, dtype=np.uint64)
    n = len(masks)
    if k == 0:
        return (np.arange(n, dtype=np.int64), masks.copy(), np.zeros(n, dtype=np.int64), np.ones(n, dtype=np.int8))
    bits = ((masks[:, None] >> np.arange(N, dtype=np.uint64)[None, :]) & np.uint64(1)).astype(bool)
    x_all, o_all = np.nonzero(bits)                      # occupied orbitals, row-major (sorted per det)
    if k == 1:
        x, p = x_all, o_all
        above = _popcount64(masks[x] >> (p + 1).astype(np.uint64)) & 1
        K = masks[x] & ~(np.uint64(1) << p.astype(np.uint64))
        return x.astype(np.int64), K, p.astype(np.int64), np.where(above == 1, -1, 1).astype(np.int8)
    ne = int(_popcount64(masks[:1])[0]) if n else 0
    if n == 0 or ne < 2:
        z = np.zeros(0, dtype=np.int64)
        return z, np.zeros(0, dtype=np.uint64), z, np.zeros(0, dtype=np.int8)
    assert (_popcount64(masks) == ne).all(), "determinants of one list share the electron count"
    occ = o_all.reshape(n, ne)
    iu, iv = np.triu_indices(ne, 1)
    u, v = occ[:, iu].ravel(), occ[:, iv].ravel()
    x = np.repeat(np.arange(n, dtype=np.int64), len(iu))
    mx = masks[x]
    K = mx & ~(np.uint64(1) << u.astype(np.uint64)) & ~(np.uint64(1) << v.astype(np.uint64))
    par = (_popcount64(mx >> (u + 1).astype(np.uint64)) + _popcount64(mx >> (v + 1).astype(np.uint64))) & 1
    return x, K, pair_index(u, v).astype(np.int64), np.where(par == 1, -1, 1).astype(np.int8)


def expand_maps(op, N):
    """For every full index (p, q, ...) of rho^op (row-major over N^len(op)): the creation
    index, the annihilation index and the sign that pick it out of X (sign 0: rho = 0)."""
    kc, ka = OP_SPLIT[op]
    L = len(op)
    idx = np.indices((N,) * L).reshape(L, -1)
    sign = np.ones(idx.shape[1], dtype=np.int8)

    def part(cols, k, kind):
        nonlocal sign
        if k == 0:
            return np.zeros(idx.shape[1], dtype=np.int64)
        if k == 1:
            return idx[cols[0]].astype(np.int64)
        p, q = idx[cols[0]], idx[cols[1]]
        lo, hi = np.minimum(p, q), np.maximum(p, q)
        if kind == "cre":        # <P| c+_p c+_q |K> = <K| a_q a_p |P>: + for p < q
            s = np.where(p < q, 1, -1)
        else:                    # <K| a_p a_q |Q>: + for p > q
            s = np.where(p > q, 1, -1)
        sign = (sign * np.where(p == q, 0, s)).astype(np.int8)
        return np.where(p == q, 0, pair_index(lo, hi)).astype(np.int64)      # p == q: sign 0

    ci = part(list(range(kc)), kc, "cre")
    ai = part(list(range(kc, L)), ka, "ann")
    return ci, ai, sign


def plan_block(op, bra_masks, ket_masks, N):
    """Index plan of one (op, bra list, ket list) density block (see the module docstring).

    Returns a dict with the intermediate count nK, the index counts ncre / nann, the bra-side
    entries (x = bra determinant, ci, k, sign) and ket-side entries (x = ket determinant, ai,
    k, sign), each sorted by determinant with a CSR pointer, and the expansion maps; or None
    when no coupling exists."""
    kc, ka = OP_SPLIT[op]
    xb, Kb, cb, sb = annihilation_entries(bra_masks, kc, N)
    xk, Kk, ck, sk = annihilation_entries(ket_masks, ka, N)
    Ks = np.intersect1d(np.unique(Kb), np.unique(Kk))
    if len(Ks) == 0:
        return None
    out = dict(op=op, N=N, nK=len(Ks), ncre=n_index(kc, N), nann=n_index(ka, N))
    for side, (x, K, c, s, n_x) in (("bra", (xb, Kb, cb, sb, len(bra_masks))),
                                    ("ket", (xk, Kk, ck, sk, len(ket_masks)))):
        pos = np.searchsorted(Ks, K)
        pos_c = np.minimum(pos, len(Ks) - 1)
        keep = Ks[pos_c] == K
        x, c, s, k = x[keep], c[keep], s[keep], pos_c[keep]
        order = np.argsort(x, kind="stable")
        x, c, s, k = x[order], c[order], s[order], k[order]
        ptr = np.zeros(n_x + 1, dtype=np.int64)
        np.add.at(ptr, x + 1, 1)
        out[side] = dict(x=x.astype(np.int32), idx=c, k=k.astype(np.int64), sign=s, ptr=np.cumsum(ptr))
    out["ci"], out["ai"], out["sign"] = expand_maps(op, N)
    return out


def numpy_density(plan, zb, zk):
    """rho^op (n_b, n_k, N, ...) of one block by the intermediate route, in NumPy (a check of
    the plan; the device path runs the same three steps)."""
    nK, ncre, nann, N = plan["nK"], plan["ncre"], plan["nann"], plan["N"]
    nb, nk = zb.shape[1], zk.shape[1]
    Ct = np.zeros((nb, ncre, nK))
    b = plan["bra"]
    np.add.at(Ct, (slice(None), b["idx"], b["k"]), (b["sign"][:, None] * zb[b["x"]]).T)
    At = np.zeros((nk, nann, nK))
    a = plan["ket"]
    np.add.at(At, (slice(None), a["idx"], a["k"]), (a["sign"][:, None] * zk[a["x"]]).T)
    X = Ct.reshape(nb * ncre, nK) @ At.reshape(nk * nann, nK).T
    X = X.reshape(nb, ncre, nk, nann)
    rho = plan["sign"][None, None, :] * np.moveaxis(X[:, plan["ci"], :, plan["ai"]], 0, -1)
    return rho.reshape((nb, nk) + (N,) * len(plan["op"]))


def fold_maps(plan):
    """For every X entry q = ci * nann + ai, the (at most two) full indices f with their signs
    (src -1 / sign 0 where absent): the reverse of the expansion, for the adjoint."""
    ncre, nann = plan["ncre"], plan["nann"]
    src = np.full((ncre * nann, 2), 0, dtype=np.int32)
    sgn = np.zeros((ncre * nann, 2), dtype=np.int8)
    f = np.nonzero(plan["sign"])[0]
    q = plan["ci"][f] * nann + plan["ai"][f]
    order = np.argsort(q, kind="stable")
    f, q = f[order], q[order]
    first = np.ones(len(q), dtype=bool)
    first[1:] = q[1:] != q[:-1]
    slot = np.where(first, 0, 1)
    assert (np.bincount(q, minlength=ncre * nann) <= 2).all()
    src[q, slot] = f
    sgn[q, slot] = plan["sign"][f]
    return src.reshape(-1), sgn.reshape(-1)


class IntermediateDensityBuilder:
    """Drop-in for densities.DensityBuilder on the split-precision paths: the same rho, zT,
    zbT and _tmp (rho transposed, [index][state pair]) buffers, built through intermediate
    determinants with one grouped tensor-core launch (see the module docstring); adjoint()
    adds dE/dz of given density gradients into FP64 [n_conf, n] buffers.

    precision: 'bf16x3' or 'tf32x3' (the split of the GEMM operands)."""

    def __init__(self, space, n_states, precision="bf16x3", n_states_bra=None, autotune=True):
        import torch
        from ._lib import call, ptr, stream_ptr  # noqa: F401
        from .gemm import SplitRegistry, TCGroupedGemm
        self.torch = torch
        self.space = space
        self.precision = precision
        self.n_states = dict(n_states)
        self.n_states_bra = dict(n_states_bra or n_states)
        dev = space.device
        self.device = dev
        f64 = dict(dtype=torch.float64, device=dev)
        N = space.N
        self.rho, self._tmp, self.blocks = {}, {}, []
        self.zT = {c: torch.empty((space.n_conf[c], self.n_states[c]), **f64) for c in space.charges}
        self.zbT = {c: torch.empty((space.n_conf[c], self.n_states_bra[c]), **f64) for c in space.charges}
        self.reg = SplitRegistry(precision, dev)
        fwd = TCGroupedGemm(self.reg)

        def dev_i32(a):
            return torch.from_numpy(np.ascontiguousarray(a, dtype=np.int32)).to(dev)

        for (op, bc, kc) in space.couplings:
            if op not in OP_SPLIT:
                continue
            nb, nk = self.n_states_bra[bc], self.n_states[kc]
            F = N ** len(op)
            rho = torch.zeros((nb, nk) + (N,) * len(op), **f64)
            self.rho.setdefault(op, {})[(bc, kc)] = rho
            self._tmp[(op, bc, kc)] = torch.zeros(F * nb * nk, **f64)
            pl = plan_block(op, space.masks_np[bc], space.masks_np[kc], N)
            if pl is None:
                continue
            nK, ncre, nann = pl["nK"], pl["ncre"], pl["nann"]
            blk = dict(key=(op, bc, kc), nb=nb, nk=nk, F=F, nK=nK, ncre=ncre, nann=nann, rho=rho,
                       tmp=self._tmp[(op, bc, kc)],
                       Ct=torch.zeros((nb * ncre, nK), **f64), At=torch.zeros((nk * nann, nK), **f64),
                       Db=torch.zeros((nK, nb * ncre), **f64), Dk=torch.zeros((nK, nk * nann), **f64),
                       X=torch.zeros((nb * ncre, nk * nann), **f64),
                       ci=dev_i32(pl["ci"]), ai=dev_i32(pl["ai"]),
                       sign=torch.from_numpy(pl["sign"].astype(np.int8)).to(dev))
            for side in ("bra", "ket"):
                e = pl[side]
                blk[side] = dict(x=dev_i32(e["x"]), idx=dev_i32(e["idx"]), k=dev_i32(e["k"]),
                                 sign=torch.from_numpy(e["sign"].astype(np.int8)).to(dev),
                                 ptr=torch.from_numpy(e["ptr"]).to(dev), n=len(e["x"]))
            src, fsg = fold_maps(pl)
            blk["fsrc"], blk["fsign"] = dev_i32(src), torch.from_numpy(fsg).to(dev)
            fwd.add(nb * ncre, nk * nann, [(blk["Ct"], nK, blk["At"], nK, nK, 1.0)], blk["X"], nk * nann, mode=0,
                    groups=[("dens", "dens")])
            # the [K][(state, index)] copies feed the adjoint GEMMs: registered now, so that every
            # build splits them whether or not the adjoint exists yet
            self.reg.operand(blk["Db"], nK, nb * ncre, nb * ncre, "dens")
            self.reg.operand(blk["Dk"], nK, nk * nann, nk * nann, "dens")
            self.blocks.append(blk)
        self.reg.upload()
        self.fwd = fwd.finalize()
        if autotune and self.blocks:
            self.fwd.autotune()
        self.bwd = None

    # ------------------------------------------------------------------------------------
    def _scatter(self, blk, s):
        from ._lib import call, ptr
        for side, zT, n, nidx, Dt, D in (("bra", self.zbT[blk["key"][1]], blk["nb"], blk["ncre"], blk["Ct"], blk["Db"]),
                                         ("ket", self.zT[blk["key"][2]], blk["nk"], blk["nann"], blk["At"], blk["Dk"])):
            e = blk[side]
            call("xrh_im_scatter", e["n"], ptr(e["x"]), ptr(e["idx"]), ptr(e["k"]), ptr(e["sign"]), ptr(zT), n,
                 blk["nK"], nidx, ptr(Dt), ptr(D), s)

    def build(self, coeffs, bra_coeffs=None):
        """coeffs: {charge: CUDA float64 (n_states, n_conf)} -> self.rho (and self._tmp)."""
        from ._lib import call, ptr, stream_ptr
        s = stream_ptr()
        for c in self.space.charges:
            self.zT[c].copy_(coeffs[c].t())
            self.zbT[c].copy_((coeffs if bra_coeffs is None else bra_coeffs)[c].t())
        for blk in self.blocks:
            self._scatter(blk, s)
        self.reg.split("dens")
        self.fwd.run()
        for blk in self.blocks:
            call("xrh_im_expand", blk["nb"], blk["nk"], blk["F"], ptr(blk["ci"]), ptr(blk["ai"]), ptr(blk["sign"]),
                 blk["ncre"], blk["nann"], ptr(blk["X"]), ptr(blk["rho"]), s)
            call("xrh_transpose", ptr(blk["rho"]), blk["nb"] * blk["nk"], blk["F"], ptr(blk["tmp"]), s)
        return self.rho

    def check(self):
        self.fwd.check()
        if self.bwd is not None:
            self.bwd.check()

    # ------------------------------------------------------------------------------------
    def setup_adjoint(self, autotune=True):
        """Buffers and the grouped launch of the reverse pass (once)."""
        from .gemm import TCGroupedGemm
        torch = self.torch
        f64 = dict(dtype=torch.float64, device=self.device)
        bwd = TCGroupedGemm(self.reg)
        for blk in self.blocks:
            nb, nk, ncre, nann, nK = blk["nb"], blk["nk"], blk["ncre"], blk["nann"], blk["nK"]
            blk["gX"] = torch.zeros((nb * ncre, nk * nann), **f64)
            blk["gXT"] = torch.zeros((nk * nann, nb * ncre), **f64)
            blk["gCt"] = torch.zeros((nb * ncre, nK), **f64)
            blk["gAt"] = torch.zeros((nk * nann, nK), **f64)
            # dCt[(I, ci), K] = sum_(J, ai) dX[(I, ci), (J, ai)] A[K, (J, ai)]
            bwd.add(nb * ncre, nK, [(blk["gX"], nk * nann, blk["Dk"], nk * nann, nk * nann, 1.0)], blk["gCt"], nK,
                    mode=0, groups=[("dg", "dens")])
            # dAt[(J, ai), K] = sum_(I, ci) dX[(I, ci), (J, ai)] C[K, (I, ci)]
            bwd.add(nk * nann, nK, [(blk["gXT"], nb * ncre, blk["Db"], nb * ncre, nb * ncre, 1.0)], blk["gAt"], nK,
                    mode=0, groups=[("dg", "dens")])
        self.reg.upload()
        self.bwd = bwd.finalize()
        if autotune and self.blocks:
            self.bwd.autotune()

    def adjoint(self, grad_rho, gzT):
        """grad_rho: {(op, bra_chg, ket_chg): dE/drho like self.rho}; gzT: {charge: FP64
        [n_conf, n_states]} += dE/dz from both the bra and the ket occurrences."""
        from ._lib import call, ptr, stream_ptr
        if self.bwd is None:
            self.setup_adjoint()
        s = stream_ptr()
        live = [blk for blk in self.blocks if blk["key"] in grad_rho]
        for blk in live:
            call("xrh_im_fold", blk["nb"], blk["nk"], blk["F"], blk["ncre"], blk["nann"], ptr(blk["fsrc"]),
                 ptr(blk["fsign"]), ptr(grad_rho[blk["key"]]), ptr(blk["gX"]), s)
            call("xrh_transpose", ptr(blk["gX"]), blk["nb"] * blk["ncre"], blk["nk"] * blk["nann"], ptr(blk["gXT"]), s)
        self.reg.split("dg")          # blocks without a gradient keep gX = 0 from setup
        self.bwd.run()
        for blk in live:
            op, bc, kc = blk["key"]
            for side, n, nidx, g, c in (("bra", blk["nb"], blk["ncre"], blk["gCt"], bc),
                                        ("ket", blk["nk"], blk["nann"], blk["gAt"], kc)):
                e = blk[side]
                call("xrh_im_gather", self.space.n_conf[c], ptr(e["ptr"]), ptr(e["idx"]), ptr(e["k"]), ptr(e["sign"]),
                     n, blk["nK"], nidx, ptr(g), ptr(gzT[c]), s)
