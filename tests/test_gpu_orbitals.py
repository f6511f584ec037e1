"""Orbital transformations on the device (qodeapplications_gb300.orbitals) against NumPy/SciPy
FP64 on the same inputs: exp(kappa) (1e-13), the overlap inverse (1e-12 relative), the
four-index transformation (1e-12 relative to the largest element), the biorthogonal
integrals (S_b = identity to 1e-12, T_b / V_b against the einsum definitions) and
transform_ints with the reference's first-order orbital update I + s x
(StateSpaceOptimizer/orbital_solver.py:431)."""
import numpy as np
import pytest

from qodeapplications_gb300 import synthetic as S

torch = pytest.importorskip("torch")
scipy_linalg = pytest.importorskip("scipy.linalg")
pytestmark = pytest.mark.gpu


def _ints(n_orb=5, seed=3):
    sysd = S.make_system(n_frag=2, n_orb=n_orb, n_states=2, seed=seed)
    U = S.make_nuclear_potentials(2, n_orb, seed=seed + 1)
    n = sysd["h"].shape[0]
    return sysd, dict(S=np.eye(n), T=sysd["h"] - U.sum(0), U=U, V=sysd["V"])


def _dev(d):
    return {k: torch.as_tensor(v, device="cuda") for k, v in d.items()}


@pytest.mark.parametrize("scale", [1e-3, 0.7, 3.0])
def test_expm_matches_scipy(scale):
    from qodeapplications_gb300.orbitals import rotation_matrix
    rng = np.random.default_rng(1)
    n_sp = 12
    a = rng.standard_normal((n_sp, n_sp)) * scale
    k = a - a.T
    R = rotation_matrix(torch.as_tensor(k, device="cuda"), [6, 6]).cpu().numpy()
    Rsp = scipy_linalg.expm(k)
    sidx = S.spin_orbital_spatial_index([6, 6])
    spin = np.concatenate([np.repeat([0, 1], 6)] * 2)
    ref = Rsp[np.ix_(sidx, sidx)] * (spin[:, None] == spin[None, :])
    np.testing.assert_allclose(R, ref, rtol=0, atol=1e-13 * max(1.0, np.abs(ref).max()))
    np.testing.assert_allclose(R @ R.T, np.eye(R.shape[0]), rtol=0, atol=1e-12)


def test_inverse_matches_numpy():
    from qodeapplications_gb300 import _lib
    rng = np.random.default_rng(2)
    for n in (7, 42, 64):
        A = np.eye(n) + 0.3 * rng.standard_normal((n, n))
        Ad = torch.as_tensor(A, device="cuda")
        out = torch.empty_like(Ad)
        st = torch.ones(1, dtype=torch.int32, device="cuda")
        _lib.call("xrh_inverse_small", n, _lib.ptr(Ad), n, _lib.ptr(out), n, _lib.ptr(st), _lib.stream_ptr())
        assert int(st.item()) == 0
        ref = np.linalg.inv(A)
        np.testing.assert_allclose(out.cpu().numpy(), ref, rtol=0, atol=1e-12 * np.abs(ref).max())
    Z = torch.zeros((5, 5), dtype=torch.float64, device="cuda")
    _lib.call("xrh_inverse_small", 5, _lib.ptr(Z), 5, _lib.ptr(out), 5, _lib.ptr(st), _lib.stream_ptr())
    assert int(st.item()) == 1           # singular: reported, no result
    with pytest.raises(_lib.XRHError):
        _lib.call("xrh_inverse_small", 65, _lib.ptr(out), 65, _lib.ptr(out), 65, _lib.ptr(st), _lib.stream_ptr())


def test_transform_integrals_matches_einsum():
    from qodeapplications_gb300.orbitals import transform_integrals
    _, ints = _ints()
    n = ints["T"].shape[0]
    rng = np.random.default_rng(4)
    M = np.eye(n) + 0.2 * rng.standard_normal((n, n))
    got = transform_integrals(torch.as_tensor(M, device="cuda"), _dev(ints))
    ref = {"S": M.T @ ints["S"] @ M, "T": M.T @ ints["T"] @ M,
           "U": np.einsum("ap,kab,bq->kpq", M, ints["U"], M),
           "V": np.einsum("ap,bq,cr,ds,abcd->pqrs", M, M, M, M, ints["V"], optimize=True)}
    for k, r in ref.items():
        np.testing.assert_allclose(got[k].cpu().numpy(), r, rtol=0, atol=1e-12 * max(1.0, np.abs(r).max()), err_msg=k)


def test_rotated_integrals_match_host_rotation():
    """exp(kappa) on the device and the four-index transformation against the host rotation
    the energy tests use (synthetic.rotate_integrals, SciPy expm + einsum)."""
    from qodeapplications_gb300.orbitals import rotation_matrix, transform_integrals
    sysd, ints = _ints(n_orb=4, seed=9)
    rng = np.random.default_rng(5)
    a = rng.normal(0, 0.05, (8, 8))
    k = a - a.T
    R = rotation_matrix(torch.as_tensor(k, device="cuda"), [4, 4])
    got = transform_integrals(R, _dev({"T": sysd["h"], "V": sysd["V"]}))
    h2, V2 = S.rotate_integrals(sysd["h"], sysd["V"], k, [4, 4])
    np.testing.assert_allclose(got["T"].cpu().numpy(), h2, rtol=0, atol=1e-12)
    np.testing.assert_allclose(got["V"].cpu().numpy(), V2, rtol=0, atol=1e-12)


def test_transform_ints_biorthogonal():
    from qodeapplications_gb300.orbitals import transform_ints
    _, ints = _ints(n_orb=5, seed=11)
    rng = np.random.default_rng(6)
    n_sp = 10
    x = rng.normal(0, 0.05, (n_sp, n_sp))
    U_sp = np.eye(n_sp) + 0.5 * (x - x.T)          # first-order update: not orthogonal, S != 1
    symm, bior = transform_ints(U_sp, _dev(ints), [5, 5])
    sidx = S.spin_orbital_spatial_index([5, 5])
    spin = np.concatenate([np.repeat([0, 1], 5)] * 2)
    M = U_sp[np.ix_(sidx, sidx)] * (spin[:, None] == spin[None, :])
    Sn = M.T @ M
    np.testing.assert_allclose(symm["S"].cpu().numpy(), Sn, rtol=0, atol=1e-13)
    assert np.abs(Sn - np.eye(len(sidx))).max() > 1e-3
    Sinv = np.linalg.inv(Sn)
    np.testing.assert_allclose(bior["Sinv"].cpu().numpy(), Sinv, rtol=0, atol=1e-12)
    np.testing.assert_allclose(bior["S"].cpu().numpy(), np.eye(len(sidx)), rtol=0, atol=1e-12)
    Tn = M.T @ ints["T"] @ M
    np.testing.assert_allclose(bior["T"].cpu().numpy(), Sinv @ Tn, rtol=0, atol=1e-12)
    Vn = np.einsum("ap,bq,cr,ds,abcd->pqrs", M, M, M, M, ints["V"], optimize=True)
    Vb = np.einsum("pa,qb,abrs->pqrs", Sinv, Sinv, Vn, optimize=True)
    np.testing.assert_allclose(bior["V"].cpu().numpy(), Vb, rtol=0, atol=1e-12 * np.abs(Vb).max())
    Ub = np.einsum("pa,kaq->kpq", Sinv, np.einsum("ap,kab,bq->kpq", M, ints["U"], M))
    np.testing.assert_allclose(bior["U"].cpu().numpy(), Ub, rtol=0, atol=1e-12)
