"""Host logic of the two-electron terms through (n-2)-electron intermediates (no GPU):
the pair list of a determinant space, contracted as the device does it, reproduces the
two-electron operator matrix <P| sum V_pqrs c+_p c+_q a_s a_r |Q> of the oracle."""
import numpy as np
import pytest

import xr_oracle as O
from qodeapplications_gb300 import synthetic as S
from qodeapplications_gb300.densities import build_pair_list


@pytest.mark.parametrize("n_orb,n_elec,sz2", [(4, 3, [1]), (5, 4, [0]), (4, 5, [-1]), (6, 2, [0]),
                                               (4, 3, [1, -1]), (4, 4, [2, 0, -2])])
def test_pair_list_reproduces_two_electron_operator(n_orb, n_elec, sz2):
    rng = np.random.default_rng(n_orb * 10 + n_elec)
    L = rng.normal(0, 0.1, (6, n_orb, n_orb))
    L = L + L.transpose(0, 2, 1)
    _, V = S.spin_orbital_integrals(np.zeros((n_orb, n_orb)), np.einsum("kpq,krs->pqrs", L, L), [n_orb])
    masks = S.sector_configs(n_orb, 0, n_elec, sz2)         # one or several Sz values
    pl = build_pair_list(masks, n_orb)
    assert pl is not None
    n = len(masks)
    from qodeapplications_gb300.densities import pair_offsets
    off, stride = pair_offsets(pl, 1)                   # one state: the class-major offsets
    np.testing.assert_array_equal(off, pl["off"])
    D = np.zeros((n, pl["L"]))
    D[pl["X"], off] = pl["sign"]
    assert len(np.unique(pl["off"] + pl["X"].astype(np.int64) * pl["L"])) == len(pl["off"])   # no collisions
    M2 = np.zeros((n, n))
    for cl in pl["classes"]:
        Dc = D[:, cl["base"]:cl["base"] + cl["n_K"] * cl["n_p"]].reshape(n, cl["n_K"], cl["n_p"])
        W = 4.0 * V[cl["u"][:, None], cl["v"][:, None], cl["u"][None, :], cl["v"][None, :]]
        M2 += np.einsum("xkp,pr,ykr->xy", Dc, W, Dc)
    ref = O.fci_hamiltonian(np.zeros((2 * n_orb, 2 * n_orb)), V, masks)
    np.testing.assert_allclose(M2, ref, atol=1e-12)


def test_pair_list_rejects_mixed_electron_counts():
    masks = np.concatenate([S.sector_configs(4, 0, 3, [1]), S.sector_configs(4, 0, 4, [0])])
    assert build_pair_list(masks, 4) is None
