"""Fragment transition densities on the GPU.

Mirrors the reference's density builders:
  general-XRCC/build_density_tensors.py:57-160  build_density_tensors(z_lists, n_orbs, Vints, n_core)
  Be-states/densities.py:236                    build_tensors(states, n_orbs, n_elec_0, ...)
and the C kernels they drive (general-XRCC/density_tensors.c).

GB300 design: the determinant lists of a fragment never change during an optimisation, so
the integer coupling lists <P|op_idx|Q> = +-1 are built once on the device
(FragmentSpace) and stay resident in HBM.  Each density build (DensityBuilder.build)
is then only the floating-point gather-accumulate rho[I,J,idx] = sum s z_I[P] z_J[Q]
plus a transpose into the reference's (n_bra, n_ket, N, ..., N) layout.
"""
import math

import numpy as np
import torch

from . import _lib
from ._lib import call, ptr, stream_ptr

# op strings per (bra_chg - ket_chg) (general-XRCC/build_density_tensors.py:90-157); the
# four-operator ccaa density is never stored: its only use (monomer two-electron energy)
# goes through the sigma-vector kernel instead.
OPS_FOR_DCHG = {+2: ("aa",), +1: ("a", "caa"), 0: ("ca",), -1: ("c", "cca"), -2: ("cc",)}


class Couplings:
    """Resident coupling list of one (op, bra charge, ket charge), CSR by operator index."""

    def __init__(self, op, K, idx_ptr, P, Q, sign):
        self.op, self.K = op, K
        self.idx_ptr, self.P, self.Q, self.sign = idx_ptr, P, Q, sign

    @property
    def count(self):
        return int(self.P.numel())


# op strings with two adjacent operators of one kind: position u of the anticommuting pair
# (o_u, o_u+1).  rho[.. o_u, o_u+1 ..] = -rho[.. o_u+1, o_u ..], so the kernels need the
# canonical tuples (o_u < o_u+1) only and xrh_antisym_rows completes the rest.
ANTISYM_PAIR = {"aa": 0, "cc": 0, "caa": 1, "cca": 0}
# rho^ca between the same real states is Hermitian: rho[i, j, p, q] = rho[j, i, q, p], so the
# tuples p <= q suffice there (the (q, p) row is the (p, q) row transposed)
HERMITIAN_PAIR = {"ca": 0}


def pair_position(op):
    """(u, mode_fill, mode_fold) of op's operator pair for xrh_antisym_rows, or None."""
    if op in ANTISYM_PAIR:
        return ANTISYM_PAIR[op], 0, 1
    if op in HERMITIAN_PAIR:
        return HERMITIAN_PAIR[op], 2, 3
    return None


def canonical_couplings(space, key):
    """The couplings of key = (op, bra charge, ket charge) restricted to the canonical index
    tuples of op's operator pair (o_u < o_u+1 for an anticommuting pair, o_u <= o_u+1 for the
    Hermitian ca pair; about half of them; same order, same CSR over all K indices, empty rows
    elsewhere), cached on the space; None for other op strings.  The Hermitian form holds for
    a block between the same states only: the caller decides."""
    op = key[0]
    if pair_position(op) is None or key not in space.couplings:
        return None
    cache = space.__dict__.setdefault("_canonical", {})
    if key not in cache:
        cp = space.couplings[key]
        u, L, N = pair_position(op)[0], len(op), space.N
        dev = cp.idx_ptr.device
        counts = cp.idx_ptr[1:] - cp.idx_ptr[:-1]
        idx_all = torch.arange(cp.K, dtype=torch.int64, device=dev)
        a = (idx_all // N ** (L - 1 - u)) % N
        b = (idx_all // N ** (L - 2 - u)) % N
        keep = a < b if op in ANTISYM_PAIR else a <= b
        per = torch.repeat_interleave(keep, counts)
        counts_c = torch.where(keep, counts, torch.zeros_like(counts))
        idx_ptr = torch.zeros(cp.K + 1, dtype=torch.int64, device=dev)
        idx_ptr[1:] = torch.cumsum(counts_c, 0)
        cache[key] = Couplings(op, cp.K, idx_ptr, cp.P[per].contiguous(), cp.Q[per].contiguous(),
                               cp.sign[per].contiguous())
    return cache[key]


def _sort_masks(masks_np):
    order = np.argsort(masks_np, kind="stable")
    return masks_np[order], order.astype(np.int32)


_BINOM = np.zeros((65, 17), dtype=np.int64)
for _n in range(65):
    for _k in range(17):
        _BINOM[_n, _k] = math.comb(_n, _k)
RANK_TABLE_LIMIT = 1 << 26        # positions stored (int32) per charge sector at most


def colex_rank(masks_np, N):
    """sum_i C(o_i, i+1) over the occupied orbitals o_0 < o_1 < ... (a bijection between the
    n_e-electron determinants over N spin orbitals and [0, C(N, n_e)))."""
    m = np.asarray(masks_np, dtype=np.uint64)
    rank = np.zeros(len(m), dtype=np.int64)
    cnt = np.zeros(len(m), dtype=np.int64)
    for o in range(N):
        bit = ((m >> np.uint64(o)) & np.uint64(1)).astype(np.int64)
        rank += bit * _BINOM[o, np.minimum(cnt + 1, 16)]
        cnt += bit
    return rank


class FragmentSpace:
    """Determinant lists of one fragment (per charge) and their coupling lists on the GPU.

    sectors: {charge: uint64 numpy array of occupation masks}; spin orbital i < n_orbs is
    alpha i, n_orbs + i is beta i (general-XRCC/density_tensors.c:58-59 ordering)."""

    def __init__(self, sectors, n_orbs, n_core, n_elec_ref, device="cuda", ops=None):
        self.n_orbs, self.n_core, self.n_elec_ref = n_orbs, n_core, n_elec_ref
        self.N = 2 * n_orbs
        self.device = torch.device(device)
        self.charges = list(sectors.keys())
        self.masks_np = {c: np.ascontiguousarray(np.asarray(m, dtype=np.uint64)) for c, m in sectors.items()}
        self.n_conf = {c: len(m) for c, m in self.masks_np.items()}
        self.n_elec = {c: n_elec_ref - c for c in self.charges}
        self.masks = {}
        self.sorted_masks = {}
        self.sorted_pos = {}
        self.rank_table, self.table_size = {}, {}
        self.binom = torch.from_numpy(_BINOM.reshape(-1).copy()).to(self.device)
        for c, m in self.masks_np.items():
            sm, order = _sort_masks(m)
            self.masks[c] = torch.from_numpy(m.view(np.int64).copy()).to(self.device)
            self.sorted_masks[c] = torch.from_numpy(sm.view(np.int64).copy()).to(self.device)
            self.sorted_pos[c] = torch.from_numpy(order).to(self.device)
            ne = bin(int(m[0])).count("1") if len(m) else 0
            size = math.comb(self.N, ne) if ne <= 16 else RANK_TABLE_LIMIT + 1
            if len(m) and size <= RANK_TABLE_LIMIT:
                table = np.full(size, -1, dtype=np.int32)
                table[colex_rank(m, self.N)] = np.arange(len(m), dtype=np.int32)
                self.rank_table[c] = torch.from_numpy(table).to(self.device)
                self.table_size[c] = size
            else:
                self.rank_table[c], self.table_size[c] = None, 0
        self.couplings = {}
        for bc in self.charges:
            for kc in self.charges:
                for op in OPS_FOR_DCHG.get(bc - kc, ()):
                    if ops is not None and op not in ops:
                        continue
                    self.couplings[(op, bc, kc)] = self._build(op, bc, kc)

    def pair_list(self, c):
        """Device copy of build_pair_list for charge c (cached), or None."""
        if not hasattr(self, "_pairs"):
            self._pairs = {}
        if c not in self._pairs:
            pl = build_pair_list(self.masks_np[c], self.n_orbs)
            if pl is not None:
                for k in ("X", "sign", "xptr"):
                    pl[k + "_dev"] = torch.from_numpy(pl[k]).to(self.device)
            self._pairs[c] = pl
        return self._pairs[c]

    def _build(self, op, bc, kc):
        n_ket, n_bra = self.n_conf[kc], self.n_conf[bc]
        K = self.N ** len(op)
        s = stream_ptr()
        counts = torch.zeros(max(n_ket, 1), dtype=torch.int64, device=self.device)
        call("xrh_couplings_count", _lib.op_code(op), self.n_orbs, self.n_core, ptr(self.masks[kc]), n_ket,
             ptr(self.sorted_masks[bc]), ptr(self.sorted_pos[bc]), n_bra, ptr(counts), s)
        offsets = torch.zeros_like(counts)
        if n_ket > 1:
            offsets[1:] = torch.cumsum(counts, 0)[:-1]
        total = int(counts.sum().item())
        idx = torch.empty(max(total, 1), dtype=torch.int32, device=self.device)
        P = torch.empty_like(idx)
        Q = torch.empty_like(idx)
        sign = torch.empty(max(total, 1), dtype=torch.int8, device=self.device)
        if total:
            call("xrh_couplings_fill", _lib.op_code(op), self.n_orbs, self.n_core, ptr(self.masks[kc]), n_ket,
                 ptr(self.sorted_masks[bc]), ptr(self.sorted_pos[bc]), n_bra, ptr(offsets), ptr(idx), ptr(P),
                 ptr(Q), ptr(sign), s)
        idx, P, Q, sign = idx[:total], P[:total], Q[:total], sign[:total]
        # sort by operator index, inside an index positive signs first (the FP32 density kernel
        # multiplies each sign range with a uniform sign), then by Q: deterministic sums
        nk = max(n_ket, 1)
        order = torch.argsort((idx.to(torch.int64) * 2 + (sign < 0).to(torch.int64)) * nk + Q.to(torch.int64))
        idx, P, Q, sign = idx[order].contiguous(), P[order].contiguous(), Q[order].contiguous(), sign[order].contiguous()
        idx_ptr = torch.zeros(K + 1, dtype=torch.int64, device=self.device)
        if total:
            idx_ptr[1:] = torch.cumsum(torch.bincount(idx.to(torch.int64), minlength=K), 0)
        return Couplings(op, K, idx_ptr, P, Q, sign)


def _popcount64(x):
    x = x.astype(np.uint64)
    out = np.zeros(x.shape, dtype=np.int64)
    for sh in range(0, 64, 8):
        out += _POP8[((x >> np.uint64(sh)) & np.uint64(0xFF)).astype(np.int64)]
    return out


_POP8 = np.array([bin(i).count("1") for i in range(256)], dtype=np.int64)


def build_pair_list(masks, n_orbs):
    """Pair list of one determinant space for the two-electron terms through (n-2)-electron
    intermediates (the layout of include/xrh.h, xrh_pair_scatter / xrh_pair_gather).

    For every determinant X (uint64 masks over N = 2 n_orbs spin orbitals, alpha block then
    beta block) and occupied pair u < v: K = X - u - v, sign of <K| a_v a_u |X> (parity of
    the occupied orbitals above u plus those above v), spin class c = number of beta
    orbitals in (u, v).  Pairs and intermediates are numbered inside their class; a class
    block holds nK_c x np_c positions, blocks concatenated: off = base_c + k * np_c + pair.
    A spin-conserving two-electron operator only couples pairs of the same class, so the
    classes need not be tied to one Sz: the space may mix Sz values.  Returns None for
    fewer than two electrons or mixed electron counts."""
    masks = np.asarray(masks, dtype=np.uint64)
    n_conf = len(masks)
    if n_conf == 0:
        return None
    ne = int(_popcount64(masks[:1])[0])
    if ne < 2 or (_popcount64(masks) != ne).any():
        return None
    N = 2 * n_orbs
    occ = np.zeros((n_conf, ne), dtype=np.int64)
    for j, row in enumerate(((masks[:, None] >> np.arange(N, dtype=np.uint64)[None, :]) & np.uint64(1)).astype(bool)):
        occ[j] = np.nonzero(row)[0]
    iu, iv = np.triu_indices(ne, 1)
    u, v = occ[:, iu].ravel(), occ[:, iv].ravel()
    X = np.repeat(np.arange(n_conf, dtype=np.int64), len(iu))
    mX = masks[X]
    K = mX & ~(np.uint64(1) << u.astype(np.uint64)) & ~(np.uint64(1) << v.astype(np.uint64))
    par = (_popcount64(mX >> (u + 1).astype(np.uint64)) + _popcount64(mX >> (v + 1).astype(np.uint64))) & 1
    cls = (u >= n_orbs).astype(np.int64) + (v >= n_orbs).astype(np.int64)
    off = np.zeros(len(X), dtype=np.int64)
    ent_cls, ent_k, ent_p = np.zeros(len(X), dtype=np.int64), np.zeros(len(X), dtype=np.int64), np.zeros(len(X), dtype=np.int64)
    classes = []
    base = 0
    for c in range(3):
        sel = np.nonzero(cls == c)[0]
        if len(sel) == 0:
            continue
        pair_key = u[sel] * N + v[sel]
        pairs, pidx = np.unique(pair_key, return_inverse=True)
        Ks, kidx = np.unique(K[sel], return_inverse=True)
        n_p, n_k = len(pairs), len(Ks)
        off[sel] = base + kidx * n_p + pidx
        ent_cls[sel], ent_k[sel], ent_p[sel] = len(classes), kidx, pidx
        classes.append(dict(base=base, n_K=n_k, n_p=n_p, u=pairs // N, v=pairs % N))
        base += n_k * n_p
    return dict(X=X.astype(np.int32), off=off, sign=np.where(par == 1, -1, 1).astype(np.int8),
                xptr=np.arange(n_conf + 1, dtype=np.int64) * len(iu), L=base, classes=classes, n_conf=n_conf,
                cls=ent_cls, k=ent_k, p=ent_p)


def pair_offsets(pl, n):
    """Per-entry position (state 0) and state stride of a pair list in the class-major array
    [class][state][K][pair] for n states."""
    base = np.array([n * cl["base"] for cl in pl["classes"]], dtype=np.int64)
    n_p = np.array([cl["n_p"] for cl in pl["classes"]], dtype=np.int64)
    stride = np.array([cl["n_K"] * cl["n_p"] for cl in pl["classes"]], dtype=np.int64)
    c = pl["cls"]
    return base[c] + pl["k"] * n_p[c] + pl["p"], stride[c]


# creation-side operator string -> its annihilation-side partner (bra and ket swapped,
# operator indices reversed: rho^cca(b, k)[I, J, p, q, r] = rho^caa(k, b)[J, I, r, q, p])
MIRROR_OF = {"c": "a", "cc": "aa", "cca": "caa"}


def mirror_pairs(space):
    """{derived block key: partner block key} for the blocks of a space that follow from
    their partner by xrh_mirror_density."""
    out = {}
    for (op, bc, kc) in space.couplings:
        if op in MIRROR_OF and (MIRROR_OF[op], kc, bc) in space.couplings:
            out[(op, bc, kc)] = (MIRROR_OF[op], kc, bc)
    return out


UNIT_MAX_STATES = 16     # blocks with at most this many states per side take the warp-per-unit kernel
UNIT_COUPLINGS = 256     # couplings per unit at most


def _coupling_units(cp):
    """Unit table of one coupling list for xrh_density_accumulate_f32_units: every operator
    index as one unit, or as ranges of at most UNIT_COUPLINGS couplings.  Returns (units,
    any index split)."""
    ip = cp.idx_ptr.cpu().numpy().astype(np.int64)
    lens = np.diff(ip)
    nu = np.maximum(1, (lens + UNIT_COUPLINGS - 1) // UNIT_COUPLINGS)
    total = int(nu.sum())
    units = np.zeros(total, dtype=_lib.DENS_UNIT_DTYPE)
    idx = np.repeat(np.arange(len(lens), dtype=np.int64), nu)
    first = np.repeat(np.cumsum(nu) - nu, nu)
    part = np.arange(total, dtype=np.int64) - first
    units["idx"] = idx
    units["c_lo"] = part * UNIT_COUPLINGS
    units["c_hi"] = np.minimum((part + 1) * UNIT_COUPLINGS, lens[idx])
    return units, bool((nu > 1).any())


class DensityBuilder:
    """Preallocated, reusable density build for one fragment and fixed state counts.

    build(coeffs, bra_coeffs=None) fills self.rho[op][(bra_chg, ket_chg)], each a CUDA
    float64 tensor of shape (n_bra, n_ket, N, ..., N) (the reference's layout,
    Be-states/densities.py:167-208).  Buffers are reused by every call (CUDA-graph safe).
    With the same states on both sides (mirror=True, no bra_coeffs) the c, cc and cca
    blocks are mirrored from their a, aa and caa partners instead of accumulated."""

    def __init__(self, space, n_states, precision="fp64", n_states_bra=None, mirror=True, antisym=True):
        self.space = space
        self.precision = _lib.PRECISIONS[precision]
        if self.precision not in (_lib.FP64, _lib.FP32):
            self.precision = _lib.FP32       # tensor-core variants build densities with FP32 products
        self.n_states = dict(n_states)
        self.n_states_bra = dict(n_states_bra or n_states)
        self.mirror = mirror_pairs(space) if (mirror and self.n_states_bra == self.n_states) else {}
        # bra states are the ket states (no separate bra coefficients can come in)
        self.same_bra_states = bool(mirror) and self.n_states_bra == self.n_states
        dev = space.device
        self.rho = {}
        self._tmp = {}
        # FP32 path: blocks with few states (<= UNIT_MAX_STATES per side) go to the warp-per-unit
        # kernel; units of split operator indices add atomically into a zeroed arena
        self.f32 = self.precision == _lib.FP32
        self._unit_keys = set()
        if self.f32:
            self._unit_keys = {key for key in space.couplings if key not in self.mirror and
                               max(self.n_states_bra[key[1]], self.n_states[key[2]]) <= UNIT_MAX_STATES}
        unit_units, split_keys = {}, []
        for key in sorted(self._unit_keys, key=str):
            cp = space.couplings[key]
            unit_units[key] = _coupling_units(cp)
            if unit_units[key][1]:
                split_keys.append(key)
        arena_n = sum(space.couplings[k].K * self.n_states_bra[k[1]] * self.n_states[k[2]] for k in split_keys)
        self._unit_zero = torch.zeros(arena_n, dtype=torch.float64, device=dev) if arena_n else None
        arena_off = 0
        for (op, bc, kc), cp in space.couplings.items():
            nb, nk = self.n_states_bra[bc], self.n_states[kc]
            shape = (nb, nk) + (space.N,) * len(op)
            self.rho.setdefault(op, {})[(bc, kc)] = torch.empty(shape, dtype=torch.float64, device=dev)
            if (op, bc, kc) in split_keys:
                self._tmp[(op, bc, kc)] = self._unit_zero[arena_off:arena_off + cp.K * nb * nk]
                arena_off += cp.K * nb * nk
            else:
                self._tmp[(op, bc, kc)] = torch.empty(cp.K * nb * nk, dtype=torch.float64, device=dev)
        # canonical lists for the accumulated blocks of op strings with an anticommuting pair (not
        # the warp-per-unit blocks, whose unit tables index the full lists)
        self._canon = {}
        if antisym:
            for key in space.couplings:
                if key in self.mirror or key in self._unit_keys:
                    continue
                if key[0] in HERMITIAN_PAIR and not (self.same_bra_states and key[1] == key[2]):
                    continue             # Hermitian only between the same states
                cc = canonical_couplings(space, key)
                if cc is not None:
                    self._canon[key] = cc
        self._fill = None
        self.zT = {c: torch.empty((space.n_conf[c], self.n_states[c]), dtype=torch.float64, device=dev)
                   for c in space.charges}
        # the bra side is the ket side unless separate bra states are built (mirror off)
        self.same_bra = bool(mirror) and self.n_states_bra == self.n_states
        self.zbT = self.zT if self.same_bra else {
            c: torch.empty((space.n_conf[c], self.n_states_bra[c]), dtype=torch.float64, device=dev)
            for c in space.charges}
        self._stage = None
        self._tr_direct = self._tr_derived = None
        self._mirrors = None
        # FP32 path: coefficients converted once per build, rows padded to 16 bytes
        if self.f32:
            pad = lambda n: (n + 3) // 4 * 4
            self.zT32 = {c: torch.zeros((space.n_conf[c], pad(self.n_states[c])), dtype=torch.float32, device=dev)
                         for c in space.charges}
            self.zbT32 = self.zT32 if self.same_bra else {
                c: torch.zeros((space.n_conf[c], pad(self.n_states_bra[c])), dtype=torch.float32, device=dev)
                for c in space.charges}
            # operator strings with few indices (K < 1024, e.g. K = N for a/c) spread the couplings
            # of every index over several CTAs, about 256 couplings each
            self.splits = {}
            for key, cp in ((k_, self._canon.get(k_, c_)) for k_, c_ in space.couplings.items()):
                if cp.K >= 1024:
                    self.splits[key] = 1
                else:
                    self.splits[key] = int(min(64, max(1, round(cp.count / max(cp.K, 1) / 256))))
            # every accumulated block of the fragment in one grouped launch (CTA per operator index);
            # op strings with an anticommuting pair run over their canonical tuples and are
            # completed by one xrh_antisym_rows pass
            direct = [(key, self._canon.get(key, cp)) for key, cp in space.couplings.items()
                      if key not in self.mirror and key not in self._unit_keys]
            tasks = np.zeros(len(direct), dtype=_lib.DENS_TASK_DTYPE)
            begin = 0
            self._zero_first = []
            for i, ((op, bc, kc), cp) in enumerate(direct):
                t = tasks[i]
                t["idx_ptr"], t["P"], t["Q"], t["sign"] = (cp.idx_ptr.data_ptr(), cp.P.data_ptr(), cp.Q.data_ptr(),
                                                           cp.sign.data_ptr())
                t["zb32"], t["zk32"] = self.zbT32[bc].data_ptr(), self.zT32[kc].data_ptr()
                t["rhoT"] = self._tmp[(op, bc, kc)].data_ptr()
                t["K"], t["nb"], t["nk"] = cp.K, self.n_states_bra[bc], self.n_states[kc]
                t["splits"], t["cta_begin"] = self.splits[(op, bc, kc)], begin
                begin += cp.K * self.splits[(op, bc, kc)]
                if self.splits[(op, bc, kc)] > 1:
                    self._zero_first.append(self._tmp[(op, bc, kc)])
            self._dens_tasks = torch.from_numpy(tasks.view(np.uint8).copy()).to(dev)
            self._n_dens_tasks, self._dens_ctas = len(tasks), begin
            # the warp-per-unit blocks: tasks (cta_begin unused) and their unit table
            ukeys = sorted(self._unit_keys, key=str)
            utasks = np.zeros(len(ukeys), dtype=_lib.DENS_TASK_DTYPE)
            ulist, self._max_n = [], 1
            for i, (op, bc, kc) in enumerate(ukeys):
                cp = space.couplings[(op, bc, kc)]
                t = utasks[i]
                t["idx_ptr"], t["P"], t["Q"], t["sign"] = (cp.idx_ptr.data_ptr(), cp.P.data_ptr(), cp.Q.data_ptr(),
                                                           cp.sign.data_ptr())
                t["zb32"], t["zk32"] = self.zbT32[bc].data_ptr(), self.zT32[kc].data_ptr()
                t["rhoT"] = self._tmp[(op, bc, kc)].data_ptr()
                nb, nk = self.n_states_bra[bc], self.n_states[kc]
                t["K"], t["nb"], t["nk"], t["splits"] = cp.K, nb, nk, 1
                self._max_n = max(self._max_n, nb, nk)
                un = unit_units[(op, bc, kc)][0].copy()
                un["task"] = i
                ulist.append(un)
            self._n_unit_tasks = len(ukeys)
            self._unit_tasks = torch.from_numpy(utasks.view(np.uint8).copy()).to(dev) if ukeys else None
            units = np.concatenate(ulist) if ulist else np.zeros(0, dtype=_lib.DENS_UNIT_DTYPE)
            self._n_units = len(units)
            self._units = torch.from_numpy(units.view(np.uint8).copy()).to(dev) if len(units) else None
            self._max_nb = max(self.n_states_bra.values()) if self.n_states_bra else 1
            self._max_nk = max(self.n_states.values()) if self.n_states else 1

    def _stage_coefficients(self, coeffs, bra_coeffs, s):
        """zT (and zbT) = coefficients transposed, plus their padded FP32 copies on the FP32
        path, in one launch (task table rebuilt when other coefficient tensors come in)."""
        sides = [(coeffs, self.zT, self.zT32 if self.f32 else None, self.n_states)]
        if not self.same_bra:
            sides.append((coeffs if bra_coeffs is None else bra_coeffs, self.zbT,
                          self.zbT32 if self.f32 else None, self.n_states_bra))
        key = tuple(src[c].data_ptr() for src, _, _, _ in sides for c in self.space.charges)
        if self._stage is None or self._stage[0] != key:
            tab = np.zeros(len(sides) * len(self.space.charges), dtype=_lib.COEFF_TASK_DTYPE)
            row, i = 0, 0
            for src, zt, z32, ns in sides:
                for c in self.space.charges:
                    x = src[c]
                    if x.dtype != torch.float64 or not x.is_contiguous() or x.shape != (ns[c], self.space.n_conf[c]):
                        raise ValueError("coefficients must be contiguous FP64 (n_states, n_conf) tensors")
                    t = tab[i]
                    t["src"], t["zT"] = x.data_ptr(), zt[c].data_ptr()
                    t["zT32"] = z32[c].data_ptr() if z32 is not None else 0
                    t["n"], t["K"], t["row_begin"] = ns[c], self.space.n_conf[c], row
                    t["npad"] = z32[c].shape[1] if z32 is not None else ns[c]
                    row += self.space.n_conf[c]
                    i += 1
            self._stage = (key, torch.from_numpy(tab.view(np.uint8).copy()).to(self.space.device), len(tab), row,
                           [src for src, _, _, _ in sides])
        _, tab_dev, n_t, rows, _keep = self._stage
        call("xrh_coeff_stage", ptr(tab_dev), n_t, rows, s)

    def build(self, coeffs, bra_coeffs=None):
        """coeffs: {charge: CUDA float64 tensor (n_states, n_conf)}."""
        s = stream_ptr()
        if bra_coeffs is not None and (self.mirror or self.same_bra):
            raise ValueError("separate bra coefficients need DensityBuilder(..., mirror=False)")
        self._stage_coefficients(coeffs, bra_coeffs, s)
        if self.f32:
            for t in self._zero_first:
                _lib.zero_(t)
            if self._n_dens_tasks:
                call("xrh_density_accumulate_f32_grouped", ptr(self._dens_tasks), self._n_dens_tasks,
                     self._dens_ctas, self._max_nb, self._max_nk, s)
            if self._n_units:
                if self._unit_zero is not None:
                    _lib.zero_(self._unit_zero)
                call("xrh_density_accumulate_f32_units", ptr(self._unit_tasks), self._n_unit_tasks, ptr(self._units),
                     self._n_units, self._max_n, s)
        if not self.f32:
            for (op, bc, kc), cp in self.space.couplings.items():
                if (op, bc, kc) in self.mirror:
                    continue
                cp = self._canon.get((op, bc, kc), cp)
                nb, nk = self.n_states_bra[bc], self.n_states[kc]
                call("xrh_density_accumulate", self.precision, cp.K, ptr(cp.idx_ptr), ptr(cp.P), ptr(cp.Q),
                     ptr(cp.sign), ptr(self.zbT[bc]), nb, ptr(self.zT[kc]), nk, ptr(self._tmp[(op, bc, kc)]), s)
        if self._canon:
            if self._fill is None:
                self._fill = _lib.AntisymRows(
                    [(self._tmp[key], self.n_states_bra[key[1]] * self.n_states[key[2]], self.space.N, len(key[0]),
                      pair_position(key[0])[0], pair_position(key[0])[1]) for key in self._canon], self.space.device)
            self._fill.run()
        if self._tr_direct is None:
            # rho^T [K, nb nk] -> rho [nb nk, K] for the accumulated blocks; the mirrored blocks go
            # the other way after the mirror kernels (their rho^T feeds the reverse pass)
            direct, derived = [], []
            for (op, bc, kc), cp in self.space.couplings.items():
                nbnk = self.n_states_bra[bc] * self.n_states[kc]
                tmp, rho = self._tmp[(op, bc, kc)], self.rho[op][(bc, kc)]
                if (op, bc, kc) in self.mirror:
                    derived.append((rho, tmp, nbnk, cp.K))
                else:
                    direct.append((tmp, rho, cp.K, nbnk))
            self._tr_direct = _lib.Transposes(direct, self.space.device)
            self._tr_derived = _lib.Transposes(derived, self.space.device)
        self._tr_direct.run()
        if self._mirrors is None:
            self._mirrors = _lib.Mirrors(
                [(self.rho[pop][(pbc, pkc)], self.rho[op][(bc, kc)], self.n_states_bra[bc], self.n_states[kc],
                  self.space.N, len(op), 0) for (op, bc, kc), (pop, pbc, pkc) in self.mirror.items()],
                self.space.device)
        self._mirrors.run()
        self._tr_derived.run()
        return self.rho


def as_device_sectors(states, device="cuda"):
    """{chg: (coeffs (n_states, n_conf), masks)} -> device coefficient tensors."""
    return {c: torch.as_tensor(np.asarray(co), dtype=torch.float64, device=device) for c, (co, _m) in states.items()}


def build_density_tensors(z_lists, n_orbs, Vints, n_core, n_threads=1):
    """Drop-in for general-XRCC/build_density_tensors.py:57 (same arguments and result
    layout): z_lists[chg].configs is (n_conf, n_e) occupied spin-orbital lists,
    z_lists[chg].coeffs (n_states, n_conf).  Returns (densities, total_size) with
    densities[op][(bra_chg, ket_chg)][I][J] an ndarray and densities['ccaa'][..][I][J] the
    scalar sum V_pqrs rho^ccaa_IJ[p,q,s,r] (build_density_tensors.py:129-133).
    n_threads is accepted for signature compatibility (the reference ignores it too)."""
    from .hamiltonian import monomer_two_electron
    sectors, coeffs = {}, {}
    for chg, st in z_lists.items():
        occ = np.asarray(st.configs, dtype=np.int64)
        masks = np.zeros(occ.shape[0], dtype=np.uint64)
        for col in range(occ.shape[1]):
            masks |= np.uint64(1) << occ[:, col].astype(np.uint64)
        sectors[chg] = masks
        coeffs[chg] = np.asarray(list(st.coeffs), dtype=np.float64)
    space = FragmentSpace(sectors, n_orbs, n_core, n_elec_ref=0)
    builder = DensityBuilder(space, {c: coeffs[c].shape[0] for c in sectors})
    rho = builder.build({c: torch.as_tensor(coeffs[c], device=space.device) for c in sectors})
    out = {op: {} for op in ("aa", "a", "caa", "ca", "ccaa", "c", "cca", "cc")}
    total = 0
    for op, blocks in rho.items():
        for key, t in blocks.items():
            a = t.cpu().numpy()
            out[op][key] = [[a[i, j] for j in range(a.shape[1])] for i in range(a.shape[0])]
            total += a.size
    V = torch.as_tensor(np.asarray(Vints, dtype=np.float64), device=space.device)
    for c in sectors:
        e2 = monomer_two_electron(space, {c: torch.as_tensor(coeffs[c], device=space.device)}, V, c).cpu().numpy()
        out["ccaa"][(c, c)] = [[float(e2[i, j]) for j in range(e2.shape[1])] for i in range(e2.shape[0])]
        total += e2.size
    return out, total
