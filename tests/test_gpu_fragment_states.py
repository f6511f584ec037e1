"""Fragment-state production on the device (qodeapplications_gb300.fragment_states) against
the oracle's determinant-space Hamiltonian (xr_oracle.fci_hamiltonian, the same sign
convention as the density builder): H Psi for a block of vectors and the dense FCI matrix at
1e-12, the lowest FCI eigenvalues (Lanczos on H Psi) at 1e-9 with eigenvector residuals below
1e-6, for several electron counts, with and without a frozen core."""
import numpy as np
import pytest

import xr_oracle as O
from qodeapplications_gb300 import synthetic as S

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n_orb,n_core,n_elec,sz2", [(5, 0, 4, 0), (5, 0, 3, 1), (6, 1, 5, None)])
def test_hpsi_and_fci_match_oracle(n_orb, n_core, n_elec, sz2):
    from qodeapplications_gb300.fragment_states import FragmentHamiltonian
    sysd = S.make_system(n_frag=1, n_orb=n_orb, n_states=1, seed=13 + n_elec)
    h, V = sysd["h"], sysd["V"]
    masks = O.all_configs(n_orb, n_core, n_elec, sz2=sz2)
    Href = O.fci_hamiltonian(h, V, masks)
    Hf = FragmentHamiltonian(masks, n_orb, n_core, h, V, n_vec=4)
    rng = np.random.default_rng(3)
    Psi = rng.standard_normal((4, len(masks)))
    got = Hf.apply(torch.as_tensor(Psi, device="cuda")).cpu().numpy()
    np.testing.assert_allclose(got, Psi @ Href.T, rtol=0, atol=1e-12 * max(1.0, np.abs(Href).max()) * 10)
    np.testing.assert_allclose(Hf.matrix().cpu().numpy(), Href, rtol=0, atol=1e-12)
    k = 3
    H1 = FragmentHamiltonian(masks, n_orb, n_core, h, V, n_vec=1)
    w, vecs = H1.lowest(k, tol=1e-10)
    wref = np.linalg.eigvalsh(Href)[:k]
    np.testing.assert_allclose(w, wref, rtol=0, atol=1e-9)
    v = vecs.cpu().numpy()
    for i in range(k):
        r = Href @ v[i] - w[i] * v[i]
        assert np.linalg.norm(r) < 1e-6, (i, np.linalg.norm(r))


def test_fci_states_feed_the_density_builder():
    """FCI states from the device feed a density build (orthonormal: rho^ca traces = N_e)."""
    from qodeapplications_gb300.densities import DensityBuilder, FragmentSpace
    from qodeapplications_gb300.fragment_states import fci_states
    sysd = S.make_system(n_frag=1, n_orb=5, n_states=1, seed=29)
    masks = O.all_configs(5, 0, 4, sz2=0)
    w, Z = fci_states(masks, 5, 0, sysd["h"], sysd["V"], 3)
    G = (Z @ Z.t()).cpu().numpy()
    np.testing.assert_allclose(G, np.eye(3), rtol=0, atol=1e-8)
    space = FragmentSpace({0: masks}, 5, 0, 4)
    rho = DensityBuilder(space, {0: 3}).build({0: Z.contiguous()})
    tr = torch.einsum("iipp->i", rho["ca"][(0, 0)]).cpu().numpy()
    np.testing.assert_allclose(tr, 4.0, atol=1e-8)
