"""Matrix-free three-fragment H x v on the GPU (qodeapplications_gb300.trimer_hv) against the
oracle's dense order-0 general-XRCC Hamiltonian of three fragments (general_xr_H_full:
build_H.py:38-188 restated and pinned by test_oracle.py to the compiled reference kernels and
to the three-fragment FCI identity).  Tolerances: FP64 1e-12 relative to the largest element
of the product; FP32 products (FP64 sums), 3xTF32 pair builds and the 3xTF32 tensor-core
stage 1e-6 relative; Lanczos
ground state within 1e-9 Eh (plus its residual estimate) of the FCI ground state."""
import numpy as np
import pytest

import xr_oracle as O
from qodeapplications_gb300 import synthetic as S

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _random_system(seed=21, n_orb=3, n_states=2, n_ref=4):
    charges = [+1, 0, -1]
    sysd = S.make_system(n_frag=3, n_orb=n_orb, n_states=n_states, charges=charges, n_elec_ref=n_ref, seed=seed)
    rng = np.random.default_rng(seed + 1)
    nsp = 3 * n_orb
    U = np.array([S.spin_orbital_integrals(b + b.T, np.zeros((nsp,) * 4), [n_orb] * 3)[0]
                  for b in rng.normal(0, 0.1, (3, nsp, nsp))])
    states = [{c: sysd["states"][m][c] for c in charges} for m in range(3)]
    return sysd["h"] + U.sum(0), sysd["V"], U, states, charges, n_orb, n_ref


def _complete_system(seed=3, n_orb=2, n_ref=2):
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
    charges = [2, 1, 0, -1, -2]
    states = []
    for _m in range(3):
        states.append({c: (np.eye(len(O.all_configs(n_orb, 0, n_ref - c))), O.all_configs(n_orb, 0, n_ref - c))
                       for c in charges})
    return h + U.sum(0), V, U, states, charges, n_orb, n_ref


def _device(system, total_charge=None, precision="fp64", hv_precision="fp64"):
    from qodeapplications_gb300.densities import FragmentSpace
    from qodeapplications_gb300.hamiltonian import DeviceIntegrals
    from qodeapplications_gb300.trimer_hv import XRTrimerHamiltonian
    h, V, U, states, charges, n_orb, n_ref = system
    spaces = [FragmentSpace({c: states[m][c][1] for c in charges}, n_orb, 0, n_ref) for m in range(3)]
    ns = [{c: states[m][c][0].shape[0] for c in charges} for m in range(3)]
    ints = DeviceIntegrals(h=h, V=V, Ns=[2 * n_orb] * 3, U=U)
    ham = XRTrimerHamiltonian(spaces, ns, [charges] * 3, ints, precision=precision, hv_precision=hv_precision,
                              total_charge=total_charge)
    ham.build([{c: torch.as_tensor(states[m][c][0], device="cuda") for c in charges} for m in range(3)])
    return ham


def _oracle(system):
    h, V, U, states, charges, n_orb, n_ref = system
    ints = O.FragInts(h, V, [2 * n_orb] * 3, U=U)
    dens = [O.build_densities({c: O.Sector(*states[m][c]) for c in charges}, n_orb, 0, n_ref) for m in range(3)]
    return O.general_xr_H_full(dens, ints, n_ref, charges, 3)


def _check_products(ham, Hfull, tol, n_vec=2):
    idx, D = ham.product_index()
    idx = idx.cpu().numpy()
    assert D == Hfull.shape[0]
    rng = np.random.default_rng(3)
    for _ in range(n_vec):
        v = rng.normal(size=ham.dim)
        vp = np.zeros(D)
        vp[idx] = v
        ref = (Hfull @ vp)[idx]
        got = ham.apply(torch.as_tensor(v, device="cuda")).cpu().numpy()
        err = np.abs(got - ref).max()
        assert err <= tol * np.abs(ref).max(), err


@pytest.mark.parametrize("total_charge", [None, 0, -1])
def test_trimer_hv_matches_oracle(total_charge):
    system = _random_system()
    _check_products(_device(system, total_charge), _oracle(system), 1e-12)


def test_trimer_hv_complete_basis_matches_oracle():
    system = _complete_system()
    _check_products(_device(system, None), _oracle(system), 1e-12)


def test_trimer_hv_lanczos_is_fci_ground_state():
    """Known answer: complete fragment bases, the 6-electron sector (924 product states):
    the matrix-free Lanczos ground state is the supersystem FCI ground state."""
    system = _complete_system()
    h, V = system[0], system[1]
    ham = _device(system, total_charge=0)
    assert ham.dim == 924
    w, resid = ham.lowest(k=1, m=120)
    masks = [np.concatenate([O.all_configs(2, 0, 2 - c) for c in system[4]]) for _ in range(3)]
    G = masks[0]
    for m in (1, 2):
        G = (G[:, None] | (masks[m][None, :] << np.uint64(4 * m))).reshape(-1)
    G = G[O.popcount(G) == 6]
    E_fci = np.linalg.eigvalsh(O.fci_hamiltonian(h, V, G))[0]
    assert abs(w[0] - E_fci) <= 1e-9 + resid, (w[0], E_fci, resid)


@pytest.mark.parametrize("precision,hv_precision", [("fp64", "fp32"), ("tf32x3", "fp64"), ("fp64", "tf32x3"),
                                                    ("tf32x3", "tf32x3")])
def test_trimer_hv_reduced_precision_close(precision, hv_precision):
    system = _random_system(seed=31, n_orb=3, n_states=3)
    ham = _device(system, 0, precision, hv_precision)
    _check_products(ham, _oracle(system), 1e-6)
    ham.check_status()


def test_trimer_hv_rebuild_tracks_new_states():
    """Buffers are reused: a second build with other states gives the new product."""
    sys_a = _random_system(seed=41)
    sys_b = _random_system(seed=42)
    sys_b = sys_a[:3] + (sys_b[3],) + sys_a[4:]
    ham = _device(sys_a, 0)
    charges = sys_b[4]
    ham.build([{c: torch.as_tensor(sys_b[3][m][c][0], device="cuda") for c in charges} for m in range(3)])
    _check_products(ham, _oracle(sys_b), 1e-12, n_vec=1)
