"""A ring of fragments: the order-0 XR energy by the many-body expansion over all fragment
pairs and the nearest-neighbour triples, with the state gradient, on one GPU.

The reference forms the Hamiltonian of N fragments in the full product basis
(general-XRCC/hamiltonian.py:18-80: the monomer, dimer and trimer blocks of
build_H.py:38-188 embedded with identity on the spectators) and diagonalises it.  For a ring
of 8 fragments with 300 states each (100 per charge +1, 0, -1) that basis holds 300^8 states,
and one pair Hamiltonian alone holds 15 GB in FP64 (7.2 GB in its neutral sector), so the
ring's energy is assembled from the lowest eigenvalues of its sub-clusters, each the
reference's own Hamiltonian of those fragments in their neutral total-charge sector:

    E_I    the monomer block H1_I of charge 0
    E_IJ   the pair Hamiltonian H1 x 1 + 1 x H1 + H2 (hamiltonian.XRDimerPlan)
    E_IJK  the three-fragment Hamiltonian (trimer_hv.XRTrimerHamiltonian, matrix-free)

    E2 = sum_I E_I + sum_{I<J} (E_IJ - E_I - E_J)                      (every pair)
    E3 = E2 + sum_{NN triples} (E_IJK - E_IJ - E_JK - E_IK + E_I + E_J + E_K)

The state gradient is that of E2 (dE2/dz, z the fragment-state coefficients, unconstrained):
by Hellmann-Feynman every pair contributes the reverse pass of its build with its ground
vector (gradients.XRDimerAdjoint), and every monomer term -(n - 2) E_I rides on one pair's
reverse pass as a weighted ground vector of H1_I (XRDimerAdjoint monomer_terms).  The
triple increments enter the energy only.

Layout on the device: one pair plan with its reverse pass and one three-fragment Hamiltonian
(whose first two density builders the pair plan shares) hold every buffer, and each pair and
triple passes through them in turn: its fragments' coefficients and its prepared integral
set are copied in (device to device), its densities are rebuilt, its Hamiltonian built and
its ground state found by restarted FP64 Lanczos, started from the lower orders of the same
iteration (a pair from the product of its monomer ground states, a triple from the product
of one of its pairs' ground state and the third monomer's).  The densities
of one fragment at 14 spatial orbitals and 100 states take 7.2 GB in FP64 (14.4 GB with
their transposed copies), so the eight fragments' densities are recomputed per sub-cluster
rather than all held at once.
"""
import math

import numpy as np
import torch

from . import _lib
from ._lib import call, ptr, stream_ptr
from .densities import DensityBuilder, FragmentSpace
from .eigen import Lanczos
from .gemm import GroupedGemm
from .gradients import XRDimerAdjoint
from .hamiltonian import DeviceIntegrals, XRDimerPlan
from .synthetic import ChainIntegralSource
from .trimer_hv import PAIRS, XRTrimerHamiltonian, _PairIntegrals


SEED_MIX = 0.3       # weight of the fixed random vector in every Lanczos start vector


def _unit_random(n, seed, device):
    g = torch.Generator().manual_seed(seed)
    v = torch.randn(n, generator=g, dtype=torch.float64)
    return (v / v.norm()).to(device)


def ring_pairs(n_frag):
    """Every fragment pair (I < J)."""
    return [(i, j) for i in range(n_frag) for j in range(i + 1, n_frag)]


def ring_triples(n_frag):
    """The nearest-neighbour triples (I, I+1, I+2) around the ring, each cluster once."""
    if n_frag < 3:
        return []
    out, seen = [], set()
    for i in range(n_frag):
        t = (i, (i + 1) % n_frag, (i + 2) % n_frag)
        if frozenset(t) not in seen:
            seen.add(frozenset(t))
            out.append(t)
    return out


def mbe_energies(E_mono, E_pair, E_triple, n_frag):
    """(E2, E3) of the many-body expansion from the sub-cluster energies: E_mono {I: E},
    E_pair {(I, J) with I < J: E}, E_triple {(I, J, K): E}."""
    E2 = sum(E_pair.values()) - (n_frag - 2) * sum(E_mono.values())
    E3 = E2
    for T, Et in E_triple.items():
        inc = Et + sum(E_mono[f] for f in T)
        for a, b in ((0, 1), (1, 2), (0, 2)):
            inc -= E_pair[tuple(sorted((T[a], T[b])))]
        E3 += inc
    return E2, E3


class XRRing:
    """Order-0 XR energy (E2, E3) and the state gradient of E2 for a ring of fragments.

    n_frag, n_orb, n_states, charges, n_elec_ref: the ring (every fragment with the same
        determinant spaces; n_states per charge); integrals and states are those of
        synthetic.ChainIntegralSource(n_frag, n_orb, seed) (U = 0)
    precision: 'fp64', 'bf16x3' or 'tf32x3' (pair builds); hv_precision: the triples' H x v
        (default: tf32x3 on the split paths, else fp64)
    triples: include the nearest-neighbour triples (E3); without them only E2 is formed
    tol: Lanczos residual bound (relative to max(1, |E|)) of every pair and triple ground state
    """

    def __init__(self, n_frag=8, n_orb=14, n_states=100, charges=(+1, 0, -1), n_elec_ref=4, precision="tf32x3",
                 hv_precision=None, triples=True, seed=1234, pair_m=90, triple_m=100, tol=1e-6, max_restarts=60,
                 graph=True, autotune=True, device="cuda"):
        dev = torch.device(device)
        self.device = dev
        self.n_frag = int(n_frag)
        self.charges = list(charges)
        self.n_states = int(n_states)
        self.tol, self.max_restarts, self.graph = float(tol), int(max_restarts), bool(graph)
        self.triple_m = int(triple_m)
        self.src = ChainIntegralSource(self.n_frag, n_orb, seed=seed)
        states = self.src.make_states(self.charges, n_states, n_elec_ref=n_elec_ref)
        masks = {c: states[0][c][1] for c in self.charges}
        for f in range(1, self.n_frag):
            for c in self.charges:
                if not np.array_equal(states[f][c][1], masks[c]):
                    raise ValueError("ring fragments must share their determinant spaces")
        self.masks = masks
        self.n_orb, self.n_elec_ref = int(n_orb), int(n_elec_ref)
        self.space = FragmentSpace(masks, n_orb, 0, n_elec_ref, device=dev)
        ns = {c: self.n_states for c in self.charges}
        f64 = dict(dtype=torch.float64, device=dev)
        self.coeffs = [{c: torch.as_tensor(np.ascontiguousarray(states[f][c][0]), **f64) for c in self.charges}
                       for f in range(self.n_frag)]
        self.ints = DeviceIntegrals(source=self.src, device=dev)
        self.pairs = ring_pairs(self.n_frag)
        self.triples = ring_triples(self.n_frag) if triples else []
        split = precision in ("bf16x3", "tf32x3")
        hv = hv_precision or ("tf32x3" if split else "fp64")
        if self.triples:
            self.slot = XRTrimerHamiltonian([self.space] * 3, [ns] * 3, [self.charges] * 3,
                                            _PairIntegrals(self.ints, self.triples[0]), precision=precision,
                                            hv_precision=hv, total_charge=0, autotune=autotune, pair_output="full")
            builders = self.slot.builders[:2]
            registry = self.slot.pair_registry
        else:
            self.slot = None
            builders = [DensityBuilder(self.space, ns, precision="fp32" if split else "fp64") for _ in range(2)]
            registry = None
        # the pair plan shares the triple's first two density builders and their split copies
        self.plan = XRDimerPlan([self.space] * 2, [ns] * 2, [self.charges] * 2, _PairIntegrals(self.ints, (0, 1)),
                                output="full", precision=precision, convention="general", layout="sector",
                                autotune=autotune, builders=builders, total_charges=[0], registry=registry)
        # the reverse pass's transposed density gradients live in the triple's H x v
        # intermediates: the two never run inside one another
        scratch = [self.slot.bufs[k] for k in ("T2p", "T1") if k in self.slot.bufs] if self.triples else None
        self.adj = XRDimerAdjoint(self.plan, monomer_terms=True, scratch=scratch)
        # integral sets, prepared once: every pair (I < J) and the ordered pairs of the triples
        need = set(self.pairs)
        for T in self.triples:
            need.update((T[a], T[b]) for a, b in PAIRS)
        self.pair_sets = {p: self.plan.integral_set(_PairIntegrals(self.ints, p)) for p in sorted(need)}
        self.triple_sets = {T: self.slot.trimer_integral_set(_PairIntegrals(self.ints, T)) for T in self.triples}
        self.ints._cache.clear()           # the blocks live on in the sets
        # the monomer term -(n - 2) E_F rides on pair (F, F+1) (the last fragment: (0, F))
        self.mono_pair = {F: (F, F + 1) if F + 1 < self.n_frag else (0, F) for F in range(self.n_frag)}
        self.mono_scale = math.sqrt(max(self.n_frag - 2, 0))
        sec = self.plan.sectors[0]
        self.rows = sec["rows"]
        self.lz_pair = Lanczos(sec["dim"], m=pair_m, device=dev)
        self.lz_mono = Lanczos(self.n_states, m=self.n_states, device=dev)
        self.v_mono = self.lz_mono.v0.clone()
        # start vectors from the lower orders of the same iteration: a pair from the product of
        # its monomer ground states (charge block (0, 0)), a triple from the product of one of
        # its pairs' ground state and the third fragment's monomer ground state
        # (a product of lower-order ground states has one value of every symmetry the
        # Hamiltonian conserves, e.g. total S_z, and its Krylov space never leaves that sector:
        # each start vector is the product plus SEED_MIX times a fixed random unit vector, normalised)
        n = self.n_states
        self.u = [torch.zeros(n, **f64) for _ in range(self.n_frag)]     # monomer ground vectors
        self.u_a, self.u_b = torch.zeros(n, **f64), torch.zeros(n, **f64)
        self.r_pair = _unit_random(sec["dim"], 13, dev)
        self.seed_pair = torch.zeros(sec["dim"], **f64)
        self.v_pair = torch.zeros(sec["dim"], **f64)
        self.seed_norm = torch.zeros(1, **f64)
        g0 = GroupedGemm(dev)
        g0.add(n, n, [(self.u_a, 1, self.u_b, 1, 1, 1.0)], self.seed_pair[sec["base"][0]:], n)
        self._pair_seed = g0.finalize()
        self.d_seed = torch.zeros(sec["dim"], **f64)
        self.d_pair = {}                  # pair ground vectors (sector layout) that seed a triple
        self.triple_seed = {}
        if self.triples:
            tp = self.slot.plan
            self.r_triple = _unit_random(tp.dim, 11, dev)
            self.seed_triple = [torch.zeros(tp.dim, **f64) for _ in range(2)]
            self.v_triple = torch.zeros(tp.dim, **f64)
            self.norm_work = torch.zeros(int(_lib.lib().xrh_gemv_split_work(1, tp.dim)), **f64)
            seeds = []
            for lay in range(2):
                g = GroupedGemm(dev)
                for t in tp.triples:
                    n0, n1, n2 = tp.shape[t]
                    C = self.seed_triple[lay][tp.off[t]:]
                    if lay == 0 and t[2] == 0:       # d_(T0 T1) x u_T2 in blocks (c0, -c0, 0)
                        g.add(n0 * n1, n2, [(self.d_seed[sec["base"][t[0]]:], 1, self.u_a, 1, 1, 1.0)], C, n2)
                    elif lay == 1 and t[0] == 0:     # u_T0 x d_(T1 T2) in blocks (0, c1, -c1)
                        g.add(n0, n1 * n2, [(self.u_a, 1, self.d_seed[sec["base"][t[1]]:], 1, 1, 1.0)], C, n1 * n2)
                seeds.append(g.finalize())
            self._triple_seed = seeds
            for T in self.triples:
                if T[0] < T[1]:
                    self.triple_seed[T] = (0, (T[0], T[1]), T[2])
                elif T[1] < T[2]:
                    self.triple_seed[T] = (1, (T[1], T[2]), T[0])
                else:
                    raise ValueError(f"no ordered pair seeds triple {T}")
                self.d_pair[self.triple_seed[T][1]] = torch.zeros(sec["dim"], **f64)
        self.grad = [{c: torch.zeros((self.space.n_conf[c], self.n_states), **f64) for c in self.charges}
                     for _ in range(self.n_frag)]
        self.E_mono, self.E_pair, self.E_triple = {}, {}, {}
        self.resid = {}
        self.products = {}                # H x v products of each triple's last ground state
        self.phase_ms = {}

    # ------------------------------------------------------------------------------------
    def _lowest(self, lz, v0, H):
        """Restarted FP64 Lanczos on a dense symmetric H from v0: (E0, residual, ground vector)."""
        lz.v0.copy_(v0)
        w = resid = None
        self.cycles = 0
        for _ in range(self.max_restarts):
            self.cycles += 1
            lz.krylov(H)
            lz.stage_to_host()
            torch.cuda.current_stream().synchronize()
            w, resid = lz.solve(1)
            if lz.m >= lz.n or resid <= self.tol * max(1.0, abs(float(w[0]))):
                break
            lz.v0.copy_(lz.ground_vector())
        return float(w[0]), float(resid), lz.ground_vector()

    def run_pair(self, I, J):
        """Build pair (I, J), its ground state and its reverse pass (added into self.grad);
        the ground states of its monomers the first time they are met in an iteration."""
        pl, adj, s = self.plan, self.adj, stream_ptr()
        n = self.n_states
        for m, F in ((0, I), (1, J)):
            for c in self.charges:
                pl.coeffs[m][c].copy_(self.coeffs[F][c])
        pl.load_integral_set(self.pair_sets[(I, J)])
        pl.launch()
        for m, F in ((0, I), (1, J)):
            if F not in self.E_mono:
                E, resid, d = self._lowest(self.lz_mono, self.v_mono, pl.H1blk[m][0].view(n, n))
                self.E_mono[F] = E
                self.resid[F] = resid
                self.u[F].copy_(d)
            dm = adj.dmono[m][0]
            _lib.zero_(dm)
            if self.mono_pair[F] == (I, J):
                # G -= (n - 2) u u^T: the monomer term of E2 in this pair's reverse pass
                call("xrh_add_mixed", n, self.mono_scale, ptr(self.u[F]), None, ptr(dm), s)
        self.u_a.copy_(self.u[I])
        self.u_b.copy_(self.u[J])
        _lib.zero_(self.seed_pair)
        self._pair_seed.run()
        call("xrh_add_mixed", self.seed_pair.numel(), SEED_MIX, ptr(self.r_pair), None, ptr(self.seed_pair), s)
        call("xrh_lanczos_normalize", self.seed_pair.numel(), ptr(self.seed_pair), ptr(self.v_pair),
             ptr(self.seed_norm), s)
        E, resid, d = self._lowest(self.lz_pair, self.v_pair, pl.sectors[0]["H"])
        self.E_pair[(I, J)] = E
        self.resid[(I, J)] = resid
        if (I, J) in self.d_pair:
            self.d_pair[(I, J)].copy_(d)
        _lib.zero_(adj.d)
        call("xrh_index_move", self.rows.numel(), ptr(self.rows), ptr(d), ptr(adj.d), 0, s)
        adj.launch(None)
        for m, c, gT, gT32 in adj.state_gradient_parts():
            F = (I, J)[m]
            call("xrh_add_mixed", gT.numel(), 1.0, ptr(gT), ptr(gT32) if gT32 is not None else None,
                 ptr(self.grad[F][c]), s)
        return E

    def run_triple(self, T):
        """Build triple T and its ground state (energy only)."""
        S = self.slot
        S.set_coeffs([self.coeffs[f] for f in T])
        S.load_integral_sets([self.pair_sets[(T[a], T[b])] for a, b in PAIRS], self.triple_sets[T])
        S.build()
        lay, P, F = self.triple_seed[T]
        s = stream_ptr()
        self.d_seed.copy_(self.d_pair[P])
        self.u_a.copy_(self.u[F])
        seed = self.seed_triple[lay]
        _lib.zero_(seed)
        self._triple_seed[lay].run()
        call("xrh_add_mixed", seed.numel(), SEED_MIX, ptr(self.r_triple), None, ptr(seed), s)
        call("xrh_lanczos_normalize_split", seed.numel(), ptr(seed), ptr(self.v_triple), ptr(self.seed_norm),
             ptr(self.norm_work), self.norm_work.numel(), s)
        w, resid = S.lowest(k=1, m=self.triple_m, tol=self.tol, max_restarts=self.max_restarts, graph=self.graph,
                            v0=self.v_triple)
        self.E_triple[T] = float(w[0])
        self.resid[T] = float(resid)
        self.products[T] = S.lanczos_cycles * S.lanczos.m
        return float(w[0])

    def iterate(self, with_triples=True):
        """One ring iteration: every pair (build, ground state, reverse pass), the monomer
        terms, every nearest-neighbour triple (build, ground state; skipped with
        with_triples=False).  Returns {'E2', 'E3'}; the gradient of E2 is in
        self.grad[fragment][charge] (n_conf x n_states, dE2/dz^T)."""
        for g in self.grad:
            for t in g.values():
                _lib.zero_(t)
        self.E_mono, self.E_pair, self.E_triple = {}, {}, {}
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        ev[0].record()
        for I, J in self.pairs:
            self.run_pair(I, J)
        ev[1].record()
        for T in (self.triples if with_triples else ()):
            self.run_triple(T)
        ev[2].record()
        torch.cuda.current_stream().synchronize()
        self.phase_ms = {"pairs": ev[0].elapsed_time(ev[1]), "triples": ev[1].elapsed_time(ev[2])}
        E2, E3 = mbe_energies(self.E_mono, self.E_pair, self.E_triple, self.n_frag)
        self.E2, self.E3 = E2, (E3 if self.triples and with_triples else None)
        return {"E2": E2, "E3": self.E3}

    def check_status(self):
        """Raise if a bounded device wait of a tensor-core launch timed out (syncs)."""
        self.plan.check_status()
        self.adj.check_status()
        if self.slot is not None:
            self.slot.check_status()

    def state_gradient(self):
        """dE2/dz per fragment: [{charge: (n_states, n_conf) device tensor}] (new tensors)."""
        return [{c: g[c].t().contiguous() for c in self.charges} for g in self.grad]
