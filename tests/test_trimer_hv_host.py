"""The three-fragment H x v plan (qodeapplications_gb300.trimer_hv.TrimerHvPlan) on the CPU.

The plan is host data: GEMM records in the xrh_gemm_task / xrh_gemm_segment contract over
named flat buffers.  Here a NumPy interpreter of that contract executes the plan with the
oracle's densities, monomer blocks and pair blocks (general-XRCC/build_H.py:38-102 as
restated in oracle/xr_oracle.py), and the product must equal the oracle's dense three-fragment
Hamiltonian (general_xr_H_full: monomers, pairs with spectator phases, trimer blocks of
build_H.py:103-188) times the same vector, to 1e-12.  The interpreter also checks that every
index of every record stays inside its buffer, which is the bounds check of the tables the
device launches read."""
import numpy as np
import pytest

import xr_oracle as O
from qodeapplications_gb300 import synthetic as S

pytest.importorskip("torch")

from qodeapplications_gb300.trimer_hv import PAIRS, TrimerHvPlan, trimer_integral_matrices  # noqa: E402


def _gather(buf, idx):
    assert idx.min() >= 0 and idx.max() < buf.size, "record reads outside its buffer"
    return buf[idx]


def _run_task(resolve, t):
    C, c0 = resolve(t["C"])
    M, N = t["M"], t["N"]
    m, n = np.arange(M)[:, None], np.arange(N)[None, :]
    for b in range(t["batch"]):
        acc = np.zeros((M, N))
        for s in t["segs"]:
            A, a0 = resolve(s["A"])
            B, b0 = resolve(s["B"])
            k = np.arange(s["K"])[None, :]
            ia = a0 + b * s["sA"] + (k * s["lda"] + m if s["flags"] & 1 else m * s["lda"] + k)
            ib = b0 + b * s["sB"] + (k * s["ldb"] + np.arange(N)[:, None] if s["flags"] & 2
                                     else np.arange(N)[:, None] * s["ldb"] + k)
            acc += s["alpha"] * _gather(A, ia) @ _gather(B, ib).T
        if t["mode"] == 2:         # scatter: C[(rowA[m] + rowB[n]) ldc + colA[m] + colB[n]] = acc
            rowA, colA, rowB, colB = (np.asarray(a, dtype=np.int64) for a in t["maps"])
            ic = c0 + (rowA[:, None] + rowB[None, :]) * t["ldc"] + colA[:, None] + colB[None, :]
        else:
            ic = c0 + b * t["sC"] + m * t["ldc"] + n
        assert ic.min() >= 0 and ic.max() < C.size, "record writes outside its buffer"
        if t["mode"] in (0, 2):
            C[ic] = acc
        else:
            C[ic] += acc


class _Interpreter:
    """Runs a TrimerHvPlan with oracle inputs (NumPy, FP64)."""

    def __init__(self, plan, dens, ints):
        self.plan = plan
        nel = plan.n_elec
        nuc = np.zeros((3, 3))
        ext = {}
        for f in range(3):
            for op, blocks in dens[f].items():
                if op in O.OP_DCHG:
                    for (bc, kc), r in blocks.items():
                        ext[("rho", f, op, bc, kc)] = np.ascontiguousarray(r).ravel()
            for c in plan.charges[f]:
                if (c, c) in dens[f]["ca"]:
                    h1 = (np.einsum("pq,ijpq->ij", ints.T[f, f] + ints.U[f, f, f], dens[f]["ca"][(c, c)]) +
                          O.gen_monomer_2e(dens[f]["ccaa"][(c, c)], ints.V[f, f, f, f]))
                    ext[("H1", f, c)] = h1.ravel()
        for p, (a, b) in enumerate(PAIRS):
            for t, (base, dimt) in plan.pair_layout[p].items():
                H = np.zeros((dimt, dimt))
                for ca in plan.charges[a]:
                    for ca2 in plan.charges[a]:
                        cb, cb2 = t - ca, t - ca2
                        if cb not in plan.charges[b] or cb2 not in plan.charges[b]:
                            continue
                        blk = O.gen_dimer_block(dens, ints.T, ints.U, ints.V, nel, nuc, a, b, ca, ca2, cb, cb2)
                        if blk is None:
                            continue
                        ni, nj = blk.shape[0] * blk.shape[1], blk.shape[2] * blk.shape[3]
                        H[base[ca]:base[ca] + ni, base[ca2]:base[ca2] + nj] = blk.reshape(ni, nj)
                ext[("H2", p, t)] = H.ravel()
        W, Uq = trimer_integral_matrices(lambda *k: ints.V[k], lambda *k: ints.U[k], plan.integral_keys, plan.Ns)
        for k, w in W.items():
            ext[("W",) + k] = np.ascontiguousarray(w).ravel()
        for k, u in Uq.items():
            ext[("Uq", k)] = np.ascontiguousarray(u).ravel()
        self.ext = ext
        self.bufs = {k: np.zeros(max(n, 1)) for k, n in plan.sizes.items()}
        for t in plan.build_tasks:
            _run_task(self._resolve, t)
        for src, shape, ax, dst in plan.permutes:
            self._permute(src, shape, ax, dst, 1.0)
        self.gather = {o: plan.permutation(o) for o in plan.orders_v if o != (0, 1, 2)}
        self.scatter = {o: plan.permutation(o) for o in plan.orders_w if o != (0, 1, 2)}

    def _permute(self, src, shape, ax, dst, scale):
        s_arr, s0 = self._resolve(src)
        d_arr, d0 = self._resolve(dst)
        n = int(np.prod(shape))
        assert s0 + n <= s_arr.size and d0 + n <= d_arr.size
        d_arr[d0:d0 + n] = scale * s_arr[s0:s0 + n].reshape(shape).transpose(ax).ravel()

    def _resolve(self, ref):
        key, off = ref
        if isinstance(key, str):
            return self.bufs[key], off
        if key[0] == "eye":
            return np.eye(key[1]).ravel(), off
        return self.ext[key], off

    def apply(self, v):
        b = self.bufs
        b["v"][:] = v
        for k in b:
            if k.startswith("w"):
                b[k][:] = 0.0
        for o, idx in self.gather.items():
            b["v%d%d%d" % o][:] = v[idx]
        for k, L in enumerate(self.plan.launches):
            if k == 2:
                for src, shape, ax, dst, scale in self.plan.mid_permutes:
                    self._permute(src, shape, ax, dst, scale)
            for t in L:
                _run_task(self._resolve, t)
        w = b["w"].copy()
        for o, idx in self.scatter.items():
            w[idx] += b["w%d%d%d" % o]
        return w


def _complete_basis(seed=3, n_orb=2, n_ref=2):
    rng = np.random.default_rng(seed)
    N, nsp = 2 * n_orb, 3 * n_orb
    a = rng.normal(0, 0.3, (nsp, nsp))
    L = rng.normal(0, 0.2, (5, nsp, nsp))
    L = L + L.transpose(0, 2, 1)
    h, V = S.spin_orbital_integrals(a + a.T, np.einsum("kpq,krs->pqrs", L, L), [n_orb] * 3)
    U = np.zeros((3, 3 * N, 3 * N))
    for k in range(3):
        b = rng.normal(0, 0.2, (nsp, nsp))
        U[k], _ = S.spin_orbital_integrals(b + b.T, np.zeros((nsp,) * 4), [n_orb] * 3)
    ints = O.FragInts(h + U.sum(0), V, [N] * 3, U=U)
    charges = [2, 1, 0, -1, -2]
    dens = []
    for _m in range(3):
        sec = {c: O.Sector(np.eye(len(O.all_configs(n_orb, 0, n_ref - c))), O.all_configs(n_orb, 0, n_ref - c))
               for c in charges}
        dens.append(O.build_densities(sec, n_orb, 0, n_ref))
    return ints, dens, charges, n_ref


def _random_states(seed=21, n_orb=3, n_states=2, n_ref=4):
    charges = (+1, 0, -1)
    sysd = S.make_system(n_frag=3, n_orb=n_orb, n_states=n_states, charges=charges, n_elec_ref=n_ref, seed=seed)
    rng = np.random.default_rng(seed + 1)
    nsp = 3 * n_orb
    U = np.array([S.spin_orbital_integrals(b + b.T, np.zeros((nsp,) * 4), [n_orb] * 3)[0]
                  for b in rng.normal(0, 0.1, (3, nsp, nsp))])
    ints = O.FragInts(sysd["h"] + U.sum(0), sysd["V"], sysd["Ns"], U=U)
    dens = [O.build_densities({c: O.Sector(*sysd["states"][m][c]) for c in charges}, n_orb, 0, n_ref)
            for m in range(3)]
    return ints, dens, list(charges), n_ref


@pytest.mark.parametrize("system", ["complete", "random"])
@pytest.mark.parametrize("total_charge", [None, 0, 1])
def test_plan_matches_dense_three_fragment_H(system, total_charge):
    ints, dens, charges, n_ref = _complete_basis() if system == "complete" else _random_states()
    ns = [{c: dens[f]["n_states"][c] for c in charges} for f in range(3)]

    def avail(f, op, bc, kc):
        return (bc, kc) in dens[f].get(op, {})

    plan = TrimerHvPlan([charges] * 3, ns, [n_ref] * 3, ints.Ns, avail, total_charge)
    assert plan.n_trimer_blocks > 0
    Hfull = O.general_xr_H_full(dens, ints, n_ref, charges, 3)
    idx, D = plan.product_index()
    assert D == Hfull.shape[0] and len(np.unique(idx)) == plan.dim
    it = _Interpreter(plan, dens, ints)
    rng = np.random.default_rng(5)
    for _ in range(2):
        v = rng.normal(size=plan.dim)
        vp = np.zeros(D)
        vp[idx] = v
        ref = (Hfull @ vp)[idx]
        got = it.apply(v)
        assert np.abs(got - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max())


def test_plan_sector_ground_state_is_fci():
    """Known answer: with complete fragment bases the lowest eigenvalue of the planned
    operator in the 6-electron sector is the supersystem FCI ground state."""
    ints, dens, charges, n_ref = _complete_basis()
    ns = [{c: dens[f]["n_states"][c] for c in charges} for f in range(3)]
    plan = TrimerHvPlan([charges] * 3, ns, [n_ref] * 3, ints.Ns, lambda f, op, bc, kc: (bc, kc) in dens[f].get(op, {}),
                        total_charge=0)
    assert plan.dim == 924
    it = _Interpreter(plan, dens, ints)
    H = np.stack([it.apply(e) for e in np.eye(plan.dim)], axis=1)
    assert np.abs(H - H.T).max() < 1e-12
    # supersystem FCI over the 6-electron determinants of 3 x 4 spin orbitals
    masks = [np.concatenate([O.all_configs(2, 0, n_ref - c) for c in charges]) for _ in range(3)]
    G = masks[0]
    for m in (1, 2):
        G = (G[:, None] | (masks[m][None, :] << np.uint64(4 * m))).reshape(-1)
    G = G[O.popcount(G) == 6]
    E_fci = np.linalg.eigvalsh(O.fci_hamiltonian(ints.h, ints.Vfull, G))
    np.testing.assert_allclose(np.linalg.eigvalsh(H)[:5], E_fci[:5], atol=1e-11)


def test_plan_uneven_state_counts_and_charge_order():
    """Charge blocks of different sizes (3, 2 and 1 states for charges 0, +1, -1, in the
    general-XRCC order with the reference charge first) on all three fragments."""
    charges = (0, +1, -1)
    counts = {0: 3, +1: 2, -1: 1}
    sysd = S.make_system(n_frag=3, n_orb=3, n_states=3, charges=charges, n_elec_ref=4, seed=77)
    ints = O.FragInts(sysd["h"], sysd["V"], sysd["Ns"])
    dens = []
    for m in range(3):
        secs = {c: O.Sector(sysd["states"][m][c][0][:counts[c]], sysd["states"][m][c][1]) for c in charges}
        dens.append(O.build_densities(secs, 3, 0, 4))
    ns = [dict(counts)] * 3
    for tc in (None, 0):
        plan = TrimerHvPlan([list(charges)] * 3, ns, [4] * 3, ints.Ns,
                            lambda f, op, bc, kc: (bc, kc) in dens[f].get(op, {}), tc)
        Hfull = O.general_xr_H_full(dens, ints, 4, list(charges), 3)
        idx, D = plan.product_index()
        it = _Interpreter(plan, dens, ints)
        v = np.random.default_rng(9).normal(size=plan.dim)
        vp = np.zeros(D)
        vp[idx] = v
        ref = (Hfull @ vp)[idx]
        assert np.abs(it.apply(v) - ref).max() <= 1e-12 * np.abs(ref).max()


def test_plan_empty_sector_has_no_work():
    """A total charge that no charge triple reaches gives an empty plan (the device class
    then refuses it with ValueError before any product)."""
    plan = TrimerHvPlan([[1, 0, -1]] * 3, [{1: 2, 0: 2, -1: 2}] * 3, [4] * 3, [6] * 3,
                        lambda f, op, bc, kc: True, total_charge=5)
    assert plan.dim == 0 and plan.triples == [] and all(not L for L in plan.launches)
    assert plan.flops_apply == 0.0 and not plan.build_tasks


def test_permute_task_records_match_numpy_transpose():
    """The xrh_permute_grouped records (dst shape, source strides) reproduce
    numpy.transpose when the kernel's index walk is replayed on the host."""
    from qodeapplications_gb300.trimer_hv import permute_tasks
    rng = np.random.default_rng(2)
    cases = [((3, 4, 5), (2, 0, 1), 1.0), ((2, 3, 4, 5), (1, 3, 0, 2), -0.5), ((6, 7), (1, 0), 2.0),
             ((2, 2, 3, 2, 3, 2), (5, 4, 3, 2, 1, 0), 1.0)]
    srcs = [rng.standard_normal(int(np.prod(sh))) for sh, _, _ in cases]
    tab, total = permute_tasks([(i, sh, ax, i, sc) for i, (sh, ax, sc) in enumerate(cases)])
    assert total == sum(int(np.prod(sh)) for sh, _, _ in cases)
    for rec, (sh, ax, sc), src in zip(tab, cases, srcs):
        out = np.empty(int(rec["n_elems"]))
        for e in range(int(rec["n_elems"])):
            r, off = e, 0
            for k in range(int(rec["ndim"]) - 1, -1, -1):
                d = int(rec["dst_shape"][k])
                off += (r % d) * int(rec["src_stride"][k])
                r //= d
            out[e] = rec["scale"] * src[off]
        np.testing.assert_array_equal(out, sc * src.reshape(sh).transpose(ax).ravel())
