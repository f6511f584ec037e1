"""The reference-signature drop-ins, through the device path.

* get_xr_result.get_xr_H(ints, dens, xr_order, monomer_charges) with the reference's density
  dictionaries (oracle-built, U != 0) against the oracle's (H1, H2) at 1e-12 (FP64) and
  1e-6 relative to the largest element (3 x TF32); its NotImplementedError cases.
* diagrammatic_expansion.blocks(...)[subsystem][charges][label] for every order-0 label and
  charge combination against the oracle's label blocks (1e-12).
* build_H.build_matrix_elements(...).monomer / dimer / trimer on the reference's Be fixture
  states (densities from the build_density_tensors drop-in, general-XRCC format) against the
  elements the compiled reference kernels produced (be_dimer_elements.npz,
  be_trimer_elements.npz), 1e-12 relative.
"""
import os
import types

import numpy as np
import pytest

import xr_oracle as O
from qodeapplications_gb300 import synthetic as S

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

CHG = [+1, 0, -1]


def _system(seed=21, n_orb=5, n_states=4):
    sysd = S.make_system(n_frag=2, n_orb=n_orb, n_states=n_states, charges=CHG, seed=seed)
    U = S.make_nuclear_potentials(2, n_orb, scale=0.08, seed=seed + 1)
    oi = O.FragInts(sysd["h"], sysd["V"], sysd["Ns"], U=U)
    dens = [O.build_densities({c: O.Sector(*sysd["states"][m][c]) for c in CHG}, n_orb, 0, 4) for m in range(2)]
    return sysd, oi, dens


@pytest.mark.parametrize("charges", [CHG, [0, +1, -1]])
def test_get_xr_H_matches_oracle(charges):
    from qodeapplications_gb300.get_xr_result import get_xr_H
    _, oi, dens = _system()
    H1, H2 = get_xr_H((oi, oi, np.zeros((2, 2))), dens, 0, [charges, charges])
    H1r, H2r = O.get_xr_H0(oi, dens, [charges, charges])
    assert isinstance(H2, np.ndarray) and H2.shape == H2r.shape
    np.testing.assert_allclose(H2, H2r, rtol=0, atol=1e-12)
    for a, b in zip(H1, H1r):
        np.testing.assert_allclose(a, b, rtol=0, atol=1e-12)


def test_get_xr_H_split_precision_close():
    from qodeapplications_gb300.get_xr_result import get_xr_H
    _, oi, dens = _system(seed=23)
    H1, H2 = get_xr_H((oi, oi, None), dens, 0, [CHG, CHG], precision="tf32x3")
    H1r, H2r = O.get_xr_H0(oi, dens, [CHG, CHG])
    assert np.abs(H2 - H2r).max() <= 1e-6 * np.abs(H2r).max()
    for a, b in zip(H1, H1r):
        assert np.abs(a - b).max() <= 1e-6 * np.abs(b).max()


def test_get_xr_H_errors_mirror_the_reference():
    from qodeapplications_gb300.get_xr_result import get_xr_H
    _, oi, dens = _system()
    with pytest.raises(NotImplementedError):
        get_xr_H((oi, oi, None), dens, 1, [CHG, CHG])
    with pytest.raises(NotImplementedError):
        get_xr_H((oi, oi, None), dens, 0, [CHG, CHG], bra_det=True)
    bad = dict(dens[1])
    bad["ca"] = dict(bad["ca"])
    bad["ca"][(0, 0)] = bad["ca"][(0, 0)][:, :, :3]
    with pytest.raises(ValueError):
        get_xr_H((oi, oi, None), [dens[0], bad], 0, [CHG, CHG])


def test_blocks_every_order0_label_matches_oracle():
    from qodeapplications_gb300 import diagrams as D
    from qodeapplications_gb300.diagrammatic_expansion import blocks
    _, oi, dens = _system(seed=25)
    fam = {"T": D.ST_diagrams, "U": D.SU_diagrams, "V": D.SV_diagrams}
    n_checked = 0
    for kind, cat in fam.items():
        ints = types.SimpleNamespace(S=oi.S, **{kind: getattr(oi, kind)})
        b = blocks(dens, ints, cat, None, None, None)
        for label in O.DIMER_ORDER0_LISTS[kind]:
            for ci0 in CHG:
                for ci1 in CHG:
                    for cj0 in CHG:
                        for cj1 in CHG:
                            if ci0 + ci1 != cj0 + cj1:
                                continue
                            key = ((ci0, cj0), (ci1, cj1))
                            got = b[(0, 1)][key][label]
                            ref = O.dimer_charge_block(dens, oi, (0, 1), key, [label])
                            if ref is None:
                                assert got is None, (label, key)
                                continue
                            np.testing.assert_allclose(got, ref, rtol=0, atol=1e-12, err_msg=f"{label} {key}")
                            n_checked += 1
        for label in cat.catalog[1]:
            for m in (0, 1):
                for c in CHG:
                    got = b[(m,)][((c, c),)][label]
                    if label == "t00":
                        ref = np.einsum("ijpq,pq->ij", dens[m]["ca"][(c, c)], oi.T[m, m])
                    elif label == "u000":
                        ref = np.einsum("ijpq,pq->ij", dens[m]["ca"][(c, c)], oi.U[m, m, m])
                    else:
                        ref = O.gen_monomer_2e(dens[m]["ccaa"][(c, c)], oi.V[m, m, m, m])
                    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-12)
                    n_checked += 1
    assert n_checked > 60
    with pytest.raises(NotImplementedError):
        blocks(dens, types.SimpleNamespace(S=oi.S, V=oi.V), D.SV_diagrams, None, None, None)[(0, 1)][
            ((0, 0), (0, 0))]["s01v0100"]


N_ORBS, N_CORE, N_REF = 9, 1, 4


def _be_fragment(golden_dir, Vints):
    """A general-XRCC fragment on the reference's Be fixture states: .rho from the
    build_density_tensors drop-in (general-XRCC format), .n_elec_ref."""
    from qodeapplications_gb300.densities import build_density_tensors
    g = np.load(os.path.join(golden_dir, "be_densities.npz"))
    N = 2 * N_ORBS
    z_lists = {}
    for c in (+1, 0, -1):
        occ = np.array([[o for o in range(N) if (int(mk) >> o) & 1] for mk in g[f"masks_{c}"]], dtype=np.int64)
        z_lists[c] = types.SimpleNamespace(configs=occ, coeffs=g[f"coeffs_{c}"])
    rho, _ = build_density_tensors(z_lists, N_ORBS, Vints, N_CORE)
    return types.SimpleNamespace(rho=rho, n_elec_ref=N_REF)


def test_build_matrix_elements_dimer_matches_reference_kernels(golden_dir):
    from qodeapplications_gb300.build_H import build_matrix_elements
    e = np.load(os.path.join(golden_dir, "be_dimer_elements.npz"))
    h, V = S.spin_orbital_integrals(e["h_sp"], np.einsum("kpq,krs->pqrs", e["L"], e["L"]), [N_ORBS, N_ORBS])
    N = 2 * N_ORBS
    oi = O.FragInts(h, V, [N, N])
    frag = _be_fragment(golden_dir, oi.V[0, 0, 0, 0])
    H = build_matrix_elements([frag, frag], oi, np.zeros((2, 2)))
    n = 0
    for ci1, ci2, cj1, cj2, i1, i2, j1, j2, v in e["elements"]:
        I = ((int(ci1), int(i1)), (int(ci2), int(i2)))
        J = ((int(cj1), int(j1)), (int(cj2), int(j2)))
        got = H.dimer((0, 1), I, J)
        assert abs(got - v) <= 1e-12 * max(1, abs(v)), (I, J, got, v)
        n += 1
    for c, i, j, v in e["monomer"]:
        got = H.monomer(0, (int(c), int(i)), (int(c), int(j)))
        assert abs(got - v) <= 1e-12 * max(1, abs(v))
        n += 1
    assert n >= 400
    # charge changes the reference rejects give 0, and nuclear repulsion enters as build_H.py does
    assert H.dimer((0, 1), ((1, 0), (1, 0)), ((-1, 0), (-1, 0))) == 0
    Hn = build_matrix_elements([frag, frag], oi, np.array([[0.5, 0.25], [0.25, 0.5]]))
    I = ((0, 1), (0, 2))
    assert abs(Hn.dimer((0, 1), I, I) - H.dimer((0, 1), I, I) - 0.25) < 1e-12
    assert abs(Hn.monomer(0, (0, 1), (0, 1)) - H.monomer(0, (0, 1), (0, 1)) - 0.5) < 1e-12


def test_build_matrix_elements_trimer_matches_reference_kernels(golden_dir):
    from qodeapplications_gb300.build_H import build_matrix_elements
    e = np.load(os.path.join(golden_dir, "be_trimer_elements.npz"))
    N = 2 * N_ORBS
    U = np.array([S.spin_orbital_integrals(u, np.zeros((3 * N_ORBS,) * 4), [N_ORBS] * 3)[0] for u in e["u_sp"]])
    h, V = S.spin_orbital_integrals(e["h_sp"], np.einsum("kpq,krs->pqrs", e["L"], e["L"]), [N_ORBS] * 3)
    oi = O.FragInts(h + U.sum(0), V, [N, N, N], U=U)
    frag = _be_fragment(golden_dir, oi.V[0, 0, 0, 0])
    H = build_matrix_elements([frag, frag, frag], oi, np.zeros((3, 3)))
    n = 0
    for row in e["elements"]:
        ci, cj = [int(x) for x in row[0:3]], [int(x) for x in row[3:6]]
        Ii, Jj = [int(x) for x in row[6:9]], [int(x) for x in row[9:12]]
        got = H.trimer((0, 1, 2), tuple(zip(ci, Ii)), tuple(zip(cj, Jj)))
        assert abs(got - row[12]) <= 1e-12 * max(1.0, abs(row[12])), (ci, cj, Ii, Jj, got, row[12])
        n += 1
    assert n >= 300
