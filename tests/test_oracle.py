"""The FP64 oracle pinned against the reference itself (CPU only).

* densities and H_contractions.c element formulas against golden fixtures produced by the
  reference's compiled C kernels (tests/golden/make_golden.py);
* the order-0 hermitian diagrams against a supersystem FCI (known answer: with complete
  fragment state sets, H_XR equals H_FCI element by element up to the product-state
  sign convention);
* the general-XRCC element formulas against the same FCI spectrum.
"""
import os

import numpy as np
import pytest

import ref_ctypes as R
import xr_oracle as O
from qodeapplications_gb300 import synthetic as S

N_ORBS, N_CORE, N_REF = 9, 1, 4
CHARGES = (+1, 0, -1)


def _be(golden_dir):
    g = np.load(os.path.join(golden_dir, "be_densities.npz"))
    sectors = {c: O.Sector(g[f"coeffs_{c}"], g[f"masks_{c}"]) for c in CHARGES}
    return g, sectors


def test_densities_match_reference_kernels(golden_dir):
    g, sectors = _be(golden_dir)
    N = 2 * N_ORBS
    checked = 0
    for bc in CHARGES:
        for kc in CHARGES:
            for op in O.OPS_FOR_DCHG.get(bc - kc, ()):
                rho = O.transition_density(op, sectors[bc].coeffs, sectors[bc].masks,
                                           sectors[kc].coeffs, sectors[kc].masks, N, N_ORBS, N_CORE)
                flat = rho.reshape(rho.shape[0], rho.shape[1], -1)
                w = np.cos(0.37 * np.arange(flat.shape[2]) + 0.1)
                np.testing.assert_allclose(flat @ w, g[f"probe_{op}_{bc}_{kc}"], rtol=0, atol=1e-12)
                np.testing.assert_allclose((flat ** 2).sum(-1), g[f"norm2_{op}_{bc}_{kc}"], rtol=1e-12, atol=1e-12)
                if len(op) <= 2:
                    np.testing.assert_allclose(rho, g[f"full_{op}_{bc}_{kc}"], rtol=0, atol=1e-13)
                checked += 1
    assert checked == 16


def test_density_sum_rules(golden_dir):
    """Tr rho^ca_II = N_e and rho^ca = contraction of rho^ccaa / (N_e - 1)."""
    _, sectors = _be(golden_dir)
    N = 2 * N_ORBS
    sec = sectors[0]
    ca = O.transition_density("ca", sec.coeffs, sec.masks, sec.coeffs, sec.masks, N, N_ORBS, N_CORE)
    ccaa = O.transition_density("ccaa", sec.coeffs, sec.masks, sec.coeffs, sec.masks, N, N_ORBS, N_CORE)
    ne = sec.n_elec
    np.testing.assert_allclose(np.einsum("iipp->i", ca), ne, atol=1e-12)
    # sum_q <c+_p c+_q a_q a_r> = (N_e - 1) <c+_p a_r>
    np.testing.assert_allclose(np.einsum("ijpqqr->ijpr", ccaa), (ne - 1) * ca, atol=1e-12)


def test_h_element_formulas_match_reference(golden_dir):
    g = np.load(os.path.join(golden_dir, "h_elements.npz"))
    names = sorted({k.split("__")[0] for k in g.files})
    assert len(names) == 10
    for name in names:
        ints = [int(x) for x in g[f"{name}__ints"]]
        arrs = []
        i = 0
        while f"{name}__arg{i}" in g.files:
            arrs.append(g[f"{name}__arg{i}"])
            i += 1
        got = O.h_element(name, *ints, *arrs)
        assert abs(got - float(g[f"{name}__out"])) <= 1e-12 * max(1.0, abs(float(g[f"{name}__out"]))), name


def _be_dimer_from_golden(golden_dir):
    g, sectors = _be(golden_dir)
    e = np.load(os.path.join(golden_dir, "be_dimer_elements.npz"))
    h, V = S.spin_orbital_integrals(e["h_sp"], np.einsum("kpq,krs->pqrs", e["L"], e["L"]), [N_ORBS, N_ORBS])
    N = 2 * N_ORBS
    ints = O.FragInts(h, V, [N, N])
    dens = O.build_densities(sectors, N_ORBS, N_CORE, N_REF)
    return e, ints, dens


def test_general_dimer_elements_match_reference(golden_dir):
    e, ints, dens = _be_dimer_from_golden(golden_dir)
    rho = [dens, dens]
    cache = {}
    for ci1, ci2, cj1, cj2, i1, i2, j1, j2, v in e["elements"]:
        key = tuple(int(x) for x in (ci1, ci2, cj1, cj2))
        if key not in cache:
            cache[key] = O.gen_dimer_block(rho, ints.T, ints.U, ints.V, [N_REF, N_REF], [[0, 0], [0, 0]],
                                           0, 1, key[0], key[2], key[1], key[3])
        got = cache[key][int(i1), int(i2), int(j1), int(j2)]
        assert abs(got - v) <= 1e-12 * max(1, abs(v))
    for c, i, j, v in e["monomer"]:
        c, i, j = int(c), int(i), int(j)
        got = (np.einsum("pq,pq->", ints.T[0, 0], dens["ca"][(c, c)][i, j]) +
               O.gen_monomer_2e(dens["ccaa"][(c, c)][i:i + 1, j:j + 1], ints.V[0, 0, 0, 0])[0, 0])
        assert abs(got - v) <= 1e-12 * max(1, abs(v))


def _tiny_complete_dimer(seed=7):
    rng = np.random.default_rng(seed)
    n_orb, n_ref = 3, 2
    N = 2 * n_orb
    nsp = 2 * n_orb
    a = rng.normal(0, 0.3, (nsp, nsp))
    L = rng.normal(0, 0.2, (5, nsp, nsp))
    L = L + L.transpose(0, 2, 1)
    h, V = S.spin_orbital_integrals(a + a.T, np.einsum("kpq,krs->pqrs", L, L), [n_orb, n_orb])
    U = np.zeros((2, 2 * N, 2 * N))
    for k in range(2):
        b = rng.normal(0, 0.2, (nsp, nsp))
        U[k], _ = S.spin_orbital_integrals(b + b.T, np.zeros((nsp,) * 4), [n_orb, n_orb])
    htot = h + U.sum(0)
    ints = O.FragInts(htot, V, [N, N], U=U)
    charges = [2, 1, 0, -1, -2]
    sectors, dens = [], []
    for _m in range(2):
        secs = {c: O.Sector(np.eye(len(O.all_configs(n_orb, 0, n_ref - c))), O.all_configs(n_orb, 0, n_ref - c))
                for c in charges}
        sectors.append(secs)
        dens.append(O.build_densities(secs, n_orb, 0, n_ref))
    m0 = np.concatenate([sectors[0][c].masks for c in charges])
    m1 = np.concatenate([sectors[1][c].masks for c in charges])
    G = (m0[:, None] | (m1[None, :] << np.uint64(N))).reshape(-1)
    n0, n1 = O.popcount(m0), O.popcount(m1)
    gauge = ((-1.0) ** (n0[:, None] * n1[None, :])).reshape(-1)
    Hf = gauge[:, None] * O.fci_hamiltonian(htot, V, G) * gauge[None, :]
    sel = np.nonzero((n0[:, None] + n1[None, :]).reshape(-1) == 2 * n_ref)[0]
    return ints, dens, charges, Hf, sel, n_ref


def test_order0_xr_equals_fci_known_answer():
    ints, dens, charges, Hf, sel, _ = _tiny_complete_dimer()
    H1, H2 = O.get_xr_H0(ints, dens, [charges, charges])
    Hx = O.full_H(H1, H2)
    assert len(sel) == 495
    np.testing.assert_allclose(Hx[np.ix_(sel, sel)], Hf[np.ix_(sel, sel)], rtol=0, atol=1e-12)


def test_general_xrcc_reproduces_fci_spectrum():
    ints, dens, charges, Hf, sel, n_ref = _tiny_complete_dimer(seed=11)
    ns = [dens[0]["n_states"][c] for c in charges]
    off = np.concatenate([[0], np.cumsum(ns)])
    tot = off[-1]
    H = np.zeros((tot,) * 4)
    for a, ci1 in enumerate(charges):
        for b, ci2 in enumerate(charges):
            for c, cj1 in enumerate(charges):
                for d, cj2 in enumerate(charges):
                    blk = O.gen_dimer_block(dens, ints.T, ints.U, ints.V, [n_ref, n_ref], [[0, 0], [0, 0]],
                                            0, 1, ci1, cj1, ci2, cj2)
                    if blk is not None:
                        H[off[a]:off[a + 1], off[b]:off[b + 1], off[c]:off[c + 1], off[d]:off[d + 1]] += blk
    H1 = []
    for m in range(2):
        h1 = np.zeros((tot, tot))
        for a, ch in enumerate(charges):
            sl = slice(off[a], off[a + 1])
            h1[sl, sl] = (np.einsum("pq,ijpq->ij", ints.T[m, m] + ints.U[m, m, m], dens[m]["ca"][(ch, ch)]) +
                          O.gen_monomer_2e(dens[m]["ccaa"][(ch, ch)], ints.V[m, m, m, m]))
        H1.append(h1)
    Hg = H.reshape(tot * tot, -1) + np.kron(H1[0], np.eye(tot)) + np.kron(np.eye(tot), H1[1])
    Hs = Hg[np.ix_(sel, sel)]
    np.testing.assert_allclose(np.abs(Hs), np.abs(Hf[np.ix_(sel, sel)]), atol=1e-12)
    np.testing.assert_allclose(np.linalg.eigvalsh(Hs), np.linalg.eigvalsh(Hf[np.ix_(sel, sel)]), atol=1e-11)


@pytest.mark.skipif(not R.available(), reason="oracle/_ref not built (needs the reference tree)")
def test_reference_kernels_direct_on_synthetic():
    """Where the compiled reference is present: oracle == reference kernels on a synthetic
    Sz-definite system embedded in the complete lexicographic configuration lists."""
    sysd = S.make_system(n_frag=1, n_orb=5, n_states=3, seed=3)
    n_orb, N = 5, 10
    chgs = list(sysd["charges"])
    secs, osecs = [], {}
    for c in chgs:
        coeffs, masks = sysd["states"][0][c]
        full = O.all_configs(n_orb, 0, 4 - c)
        pos = {int(m): i for i, m in enumerate(full)}
        z = np.zeros((coeffs.shape[0], len(full)))
        z[:, [pos[int(m)] for m in masks]] = coeffs
        secs.append((z, O.masks_to_occ(full, N)))
        osecs[c] = O.Sector(coeffs, masks)
    for bi, bc in enumerate(chgs):
        for ki, kc in enumerate(chgs):
            for op in O.OPS_FOR_DCHG.get(bc - kc, ()):
                ref = R.ref_density(op, secs, bi, ki, n_orb, 0)
                got = O.transition_density(op, osecs[bc].coeffs, osecs[bc].masks, osecs[kc].coeffs,
                                           osecs[kc].masks, N, n_orb, 0)
                np.testing.assert_allclose(got, ref, rtol=0, atol=1e-13)


def test_trimer_elements_match_reference(golden_dir):
    """Oracle trimer blocks (general-XRCC/build_H.py:103-188) against elements the compiled
    reference kernels (H_contractions.c:184-252) produced for a Be3 system with nuclear
    potentials, dispatched as build_H.py does."""
    g, sectors = _be(golden_dir)
    e = np.load(os.path.join(golden_dir, "be_trimer_elements.npz"))
    N = 2 * N_ORBS
    U = np.array([S.spin_orbital_integrals(u, np.zeros((3 * N_ORBS,) * 4), [N_ORBS] * 3)[0] for u in e["u_sp"]])
    h, V = S.spin_orbital_integrals(e["h_sp"], np.einsum("kpq,krs->pqrs", e["L"], e["L"]), [N_ORBS] * 3)
    ints = O.FragInts(h + U.sum(0), V, [N, N, N], U=U)
    dens = O.build_densities(sectors, N_ORBS, N_CORE, N_REF, ops=("a", "c", "ca", "aa", "cc"))
    rho = [dens, dens, dens]
    cache = {}
    for row in e["elements"]:
        ci, cj = tuple(int(x) for x in row[0:3]), tuple(int(x) for x in row[3:6])
        I, J = [int(x) for x in row[6:9]], [int(x) for x in row[9:12]]
        v = row[12]
        if (ci, cj) not in cache:
            cache[(ci, cj)] = O.gen_trimer_block(rho, ints.T, ints.U, ints.V, [N_REF] * 3, (0, 1, 2), ci, cj)
        got = cache[(ci, cj)][I[0], I[1], I[2], J[0], J[1], J[2]]
        assert abs(got - v) <= 1e-12 * max(1.0, abs(v)), (ci, cj, got, v)


def _complete_basis_system(n_frag, seed=3, n_orb=2, n_ref=2):
    rng = np.random.default_rng(seed)
    N = 2 * n_orb
    nsp = n_frag * n_orb
    a = rng.normal(0, 0.3, (nsp, nsp))
    L = rng.normal(0, 0.2, (5, nsp, nsp))
    L = L + L.transpose(0, 2, 1)
    h, V = S.spin_orbital_integrals(a + a.T, np.einsum("kpq,krs->pqrs", L, L), [n_orb] * n_frag)
    U = np.zeros((n_frag, n_frag * N, n_frag * N))
    for k in range(n_frag):
        b = rng.normal(0, 0.2, (nsp, nsp))
        U[k], _ = S.spin_orbital_integrals(b + b.T, np.zeros((nsp,) * 4), [n_orb] * n_frag)
    htot = h + U.sum(0)
    ints = O.FragInts(htot, V, [N] * n_frag, U=U)
    charges = [2, 1, 0, -1, -2]
    secs, dens = [], []
    for _m in range(n_frag):
        sec = {c: O.Sector(np.eye(len(O.all_configs(n_orb, 0, n_ref - c))), O.all_configs(n_orb, 0, n_ref - c))
               for c in charges}
        secs.append(sec)
        dens.append(O.build_densities(sec, n_orb, 0, n_ref))
    masks = [np.concatenate([secs[m][c].masks for c in charges]) for m in range(n_frag)]
    G, ntot = masks[0], O.popcount(masks[0])
    for m in range(1, n_frag):
        G = (G[:, None] | (masks[m][None, :] << np.uint64(m * N))).reshape(-1)
        ntot = (ntot[:, None] + O.popcount(masks[m])[None, :]).reshape(-1)
    sel = np.nonzero(ntot == n_frag * n_ref)[0]
    return ints, dens, charges, O.fci_hamiltonian(htot, V, G), sel, n_ref


def test_three_fragment_complete_basis_reproduces_fci():
    """Known answer for the trimer terms: with complete fragment bases the order-0
    general-XRCC Hamiltonian of three fragments (monomers, the three pairs and the triple,
    build_H.py:38-188) is the supersystem Hamiltonian in another basis phase convention."""
    ints, dens, charges, Hf, sel, n_ref = _complete_basis_system(3)
    Hx = O.general_xr_H_full(dens, ints, n_ref, charges, 3)
    assert len(sel) == 924
    Hs, Fs = Hx[np.ix_(sel, sel)], Hf[np.ix_(sel, sel)]
    np.testing.assert_allclose(np.abs(Hs), np.abs(Fs), atol=1e-12)
    np.testing.assert_allclose(np.linalg.eigvalsh(Hs), np.linalg.eigvalsh(Fs), atol=1e-11)
