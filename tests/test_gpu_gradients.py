"""GPU adjoint (state and orbital gradients) and the Lanczos eigensolver against the oracle.

Tolerances: gradients vs central finite differences of the FP64 oracle energy with step
1e-5 (FD truncation error ~ 1e-10 relative for these smooth functions): relative 1e-6;
vs the restated reference gradient formula (exact identity): absolute 1e-10."""
import numpy as np
import pytest

import xr_oracle as O
from qodeapplications_gb300 import synthetic as S

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

CHG = (+1, 0, -1)


def _setup(seed=31, n_orb=4, n_states=3):
    from qodeapplications_gb300.densities import FragmentSpace
    from qodeapplications_gb300.gradients import XRDimerAdjoint
    from qodeapplications_gb300.hamiltonian import DeviceIntegrals, XRDimerPlan
    sysd = S.make_system(n_frag=2, n_orb=n_orb, n_states=n_states, charges=CHG, seed=seed)
    spaces = [FragmentSpace({c: sysd["states"][m][c][1] for c in CHG}, n_orb, 0, 4) for m in range(2)]
    ns = [{c: n_states for c in CHG}] * 2
    plan = XRDimerPlan(spaces, ns, [list(CHG)] * 2, DeviceIntegrals(h=sysd["h"], V=sysd["V"], Ns=sysd["Ns"]))
    adj = XRDimerAdjoint(plan)
    coeffs = [{c: torch.as_tensor(sysd["states"][m][c][0], device="cuda") for c in CHG} for m in range(2)]
    return sysd, plan, adj, coeffs


def _gpu_energy_and_grad(plan, adj, coeffs):
    from qodeapplications_gb300.eigen import Lanczos
    H = plan.build(coeffs)
    lz = Lanczos(H.shape[0], m=min(120, H.shape[0]))
    lz.krylov(H)
    lz.stage_to_host()
    torch.cuda.synchronize()
    w, resid = lz.solve(1)
    d = lz.ground_vector()
    adj.launch(d)
    torch.cuda.synchronize()
    return float(w[0]), d, resid


def test_lanczos_matches_dense_eigh():
    sysd, plan, adj, coeffs = _setup()
    E, d, resid = _gpu_energy_and_grad(plan, adj, coeffs)
    Eref, vref, _, _ = O.xr_energy(sysd["h"], sysd["V"], sysd["Ns"], 4, 0, 4, sysd["states"], CHG)
    assert abs(E - Eref) < 1e-10
    assert abs(abs(float(torch.dot(d, torch.as_tensor(vref, device="cuda")))) - 1.0) < 1e-8
    assert resid < 1e-7


def test_state_gradient_matches_finite_differences():
    sysd, plan, adj, coeffs = _setup()
    E, d, _ = _gpu_energy_and_grad(plan, adj, coeffs)
    g = adj.state_gradient()
    rng = np.random.default_rng(4)
    for trial in range(3):
        dirs = [{c: rng.standard_normal(sysd["states"][m][c][0].shape) for c in CHG} for m in range(2)]
        pred = sum(float((g[m][c].cpu().numpy() * dirs[m][c]).sum()) for m in range(2) for c in CHG)
        eps = 1e-5
        vals = []
        for sgn in (+1, -1):
            st = [{c: (sysd["states"][m][c][0] + sgn * eps * dirs[m][c], sysd["states"][m][c][1]) for c in CHG}
                  for m in range(2)]
            vals.append(O.xr_energy(sysd["h"], sysd["V"], sysd["Ns"], 4, 0, 4, st, CHG)[0])
        fd = (vals[0] - vals[1]) / (2 * eps)
        assert abs(fd - pred) <= 1e-6 * max(1.0, abs(fd)), (trial, fd, pred)


@pytest.mark.parametrize("frag", [0, 1])
def test_state_gradient_matches_reference_formula(frag):
    """The reference's 'herm' gradient (state_gradients.py:205-216, restated brute force with
    determinant bras) uses state overlaps where the XR H has Kronecker deltas, and adds the
    E * overlap term; both differences are (symmetric matrix) x z and vanish on the tangent
    space of the orthonormal states.  So tangent(1/2 dE/dz) == tangent(reference)."""
    from qodeapplications_gb300.gradients import tangent_project
    sysd, plan, adj, coeffs = _setup(seed=33)
    E, d, _ = _gpu_energy_and_grad(plan, adj, coeffs)
    g = adj.state_gradient()
    ref, Eref = O.reference_state_gradient_herm(sysd["h"], sysd["V"], sysd["Ns"], 4, 0, 4, sysd["states"], CHG, frag)
    assert abs(E - Eref) < 1e-10
    for c in CHG:
        z = torch.as_tensor(sysd["states"][frag][c][0], device="cuda")
        mine = tangent_project(0.5 * g[frag][c], z).cpu().numpy()
        theirs = tangent_project(torch.as_tensor(ref[c], device="cuda"), z).cpu().numpy()
        np.testing.assert_allclose(mine, theirs, rtol=0, atol=1e-10)


def test_orbital_gradient_matches_finite_differences():
    sysd, plan, adj, coeffs = _setup(seed=35)
    E, d, _ = _gpu_energy_and_grad(plan, adj, coeffs)
    dev = "cuda"
    T = torch.as_tensor(sysd["h"], device=dev)
    U = torch.zeros((2,) + T.shape, dtype=torch.float64, device=dev)
    V = torch.as_tensor(sysd["V"], device=dev)
    sidx = S.spin_orbital_spatial_index([4, 4])
    Kg = adj.orbital_gradient(T, U, V, sidx).cpu().numpy()
    assert np.abs(Kg + Kg.T).max() < 1e-12
    rng = np.random.default_rng(8)
    for trial in range(3):
        Dk = rng.standard_normal((8, 8))
        Dk = Dk - Dk.T
        pred = 0.5 * float((Kg * Dk).sum())
        eps = 1e-5
        vals = []
        for sgn in (+1, -1):
            h2, V2 = S.rotate_integrals(sysd["h"], sysd["V"], sgn * eps * Dk, [4, 4])
            vals.append(O.xr_energy(h2, V2, sysd["Ns"], 4, 0, 4, sysd["states"], CHG)[0])
        fd = (vals[0] - vals[1]) / (2 * eps)
        assert abs(fd - pred) <= 1e-6 * max(1.0, abs(fd)), (trial, fd, pred)


@pytest.mark.parametrize("prec,dens", [("bf16x3", "fp32"), ("tf32x3", "fp32"), ("bf16x3", "im")])
def test_split_precision_gradients_close_to_fp64(prec, dens):
    """The split-precision adjoint (FP32 density adjoint, tensor-core build) against the FP64
    adjoint: relative error of the tangent state gradient and of dE/dkappa below 1e-5."""
    from qodeapplications_gb300.densities import FragmentSpace
    from qodeapplications_gb300.gradients import XRDimerAdjoint, tangent_project
    from qodeapplications_gb300.hamiltonian import DeviceIntegrals, XRDimerPlan
    sysd = S.make_system(n_frag=2, n_orb=4, n_states=3, charges=CHG, seed=31)
    spaces = [FragmentSpace({c: sysd["states"][m][c][1] for c in CHG}, 4, 0, 4) for m in range(2)]
    ns = [{c: 3 for c in CHG}] * 2
    coeffs = [{c: torch.as_tensor(sysd["states"][m][c][0], device="cuda") for c in CHG} for m in range(2)]
    out = {}
    for p in ("fp64", prec):
        plan = XRDimerPlan(spaces, ns, [list(CHG)] * 2, DeviceIntegrals(h=sysd["h"], V=sysd["V"], Ns=sysd["Ns"]),
                           precision=p, dens_precision=None if p == "fp64" else dens)
        adj = XRDimerAdjoint(plan)
        E, d, _ = _gpu_energy_and_grad(plan, adj, coeffs)
        plan.check_status()
        adj.check_status()
        g = adj.state_gradient()
        gt = torch.cat([tangent_project(g[m][c], coeffs[m][c]).reshape(-1) for m in range(2) for c in CHG])
        T = torch.as_tensor(sysd["h"], device="cuda")
        kg = adj.orbital_gradient(T, torch.zeros((2,) + T.shape, dtype=torch.float64, device="cuda"),
                                  torch.as_tensor(sysd["V"], device="cuda"), S.spin_orbital_spatial_index([4, 4]))
        out[p] = (gt, kg)
    for a, b in zip(out[prec], out["fp64"]):
        assert float((a - b).norm() / b.norm()) < 1e-5


def test_adjoint_built_after_the_build_matches_adjoint_built_before():
    """The reverse pass may be set up after a build (the intermediate-determinant density
    route splits its adjoint GEMM operands in every build from the plan's construction on):
    same gradient either way."""
    from qodeapplications_gb300.densities import FragmentSpace
    from qodeapplications_gb300.gradients import XRDimerAdjoint
    from qodeapplications_gb300.hamiltonian import DeviceIntegrals, XRDimerPlan
    from qodeapplications_gb300.eigen import Lanczos
    sysd = S.make_system(n_frag=2, n_orb=4, n_states=3, charges=CHG, seed=33)
    spaces = [FragmentSpace({c: sysd["states"][m][c][1] for c in CHG}, 4, 0, 4) for m in range(2)]
    ns = [{c: 3 for c in CHG}] * 2
    coeffs = [{c: torch.as_tensor(sysd["states"][m][c][0], device="cuda") for c in CHG} for m in range(2)]
    out = []
    for adj_first in (True, False):
        plan = XRDimerPlan(spaces, ns, [list(CHG)] * 2, DeviceIntegrals(h=sysd["h"], V=sysd["V"], Ns=sysd["Ns"]),
                           precision="bf16x3", dens_precision="im")
        adj = XRDimerAdjoint(plan) if adj_first else None
        H = plan.build(coeffs)
        lz = Lanczos(H.shape[0], m=min(120, H.shape[0]))
        lz.krylov(H)
        lz.stage_to_host()
        torch.cuda.synchronize()
        lz.solve(1)
        d = lz.ground_vector().clone()
        adj = adj or XRDimerAdjoint(plan)
        adj.launch(d)
        g = adj.state_gradient()
        out.append(torch.cat([g[m][c].reshape(-1) for m in range(2) for c in CHG]).clone())
    assert float((out[0] - out[1]).abs().max()) <= 1e-12 * float(out[0].abs().max())


def test_tensor_core_density_adjoint_matches_fp64_over_many_coupling_tiles():
    """The tensor-core density adjoint (3 x TF32, tiles of 128 couplings) against the FP64
    adjoint on a system whose operator indices have several hundred couplings each:
    tangent state gradient within 1e-5 relative."""
    from qodeapplications_gb300.densities import FragmentSpace
    from qodeapplications_gb300.gradients import XRDimerAdjoint, tangent_project
    from qodeapplications_gb300.hamiltonian import DeviceIntegrals, XRDimerPlan
    n_orb, n_st = 6, 8
    sysd = S.make_system(n_frag=2, n_orb=n_orb, n_states=n_st, charges=CHG, seed=41)
    spaces = [FragmentSpace({c: sysd["states"][m][c][1] for c in CHG}, n_orb, 0, 4) for m in range(2)]
    assert max(cp.count / cp.K for cp in spaces[0].couplings.values()) > 128
    ns = [{c: n_st for c in CHG}] * 2
    coeffs = [{c: torch.as_tensor(sysd["states"][m][c][0], device="cuda") for c in CHG} for m in range(2)]
    out = {}
    for p in ("fp64", "tf32x3"):
        plan = XRDimerPlan(spaces, ns, [list(CHG)] * 2, DeviceIntegrals(h=sysd["h"], V=sysd["V"], Ns=sysd["Ns"]),
                           precision=p)
        adj = XRDimerAdjoint(plan, density_adjoint="tc" if p == "tf32x3" else "simt")
        if p == "tf32x3":
            assert adj.dens_adj_tc
        E, d, _ = _gpu_energy_and_grad(plan, adj, coeffs)
        torch.cuda.synchronize()
        plan.check_status()
        adj.check_status()
        g = adj.state_gradient()
        out[p] = torch.cat([tangent_project(g[m][c], coeffs[m][c]).reshape(-1) for m in range(2) for c in CHG])
    rel = float((out["tf32x3"] - out["fp64"]).norm() / out["fp64"].norm())
    assert rel < 1e-5, rel


@pytest.mark.parametrize("path", ["units", "cta"])
def test_fp32_density_adjoint_paths_match_fp64(path, monkeypatch):
    """The FP32 density adjoint, lane per coupling on unit tables (dE/drho read in place) or
    one CTA per operator index (transposed dE/drho), against the FP64 adjoint on a system with
    hundreds of couplings per operator index: tangent state gradient within 1e-5 relative."""
    from qodeapplications_gb300 import densities as D
    from qodeapplications_gb300 import gradients as Gm
    from qodeapplications_gb300.hamiltonian import DeviceIntegrals, XRDimerPlan
    if path == "cta":
        monkeypatch.setattr(Gm, "ADJ_UNIT_MAX", 0)
        monkeypatch.setattr(D, "UNIT_MAX_STATES", 0)
    n_orb, n_st = 6, 8
    sysd = S.make_system(n_frag=2, n_orb=n_orb, n_states=n_st, charges=CHG, seed=43)
    spaces = [D.FragmentSpace({c: sysd["states"][m][c][1] for c in CHG}, n_orb, 0, 4) for m in range(2)]
    ns = [{c: n_st for c in CHG}] * 2
    coeffs = [{c: torch.as_tensor(sysd["states"][m][c][0], device="cuda") for c in CHG} for m in range(2)]
    out = {}
    for p in ("fp64", "tf32x3"):
        plan = XRDimerPlan(spaces, ns, [list(CHG)] * 2, DeviceIntegrals(h=sysd["h"], V=sysd["V"], Ns=sysd["Ns"]),
                           precision=p)
        adj = Gm.XRDimerAdjoint(plan)
        if p == "tf32x3":
            assert bool(adj.dens_adj_units) == (path == "units")
        E, d, _ = _gpu_energy_and_grad(plan, adj, coeffs)
        torch.cuda.synchronize()
        plan.check_status()
        adj.check_status()
        g = adj.state_gradient()
        out[p] = torch.cat([Gm.tangent_project(g[m][c], coeffs[m][c]).reshape(-1) for m in range(2) for c in CHG])
    rel = float((out["tf32x3"] - out["fp64"]).norm() / out["fp64"].norm())
    assert rel < 1e-5, rel


@pytest.mark.parametrize("prec", ["fp64", "tf32x3"])
def test_orbital_gradient_fused_terms_match_torch_assembly(prec, monkeypatch):
    """dE/dkappa with the integral derivatives assembled element-wise by xrh_orbital_terms
    against the same contraction with dE/dT, dE/dV formed by PyTorch block operations:
    relative 1e-12 in FP64, 1e-5 with the FP32 B of the split-precision paths."""
    from qodeapplications_gb300 import gradients as Gm
    sysd, plan, adj, coeffs = _setup() if prec == "fp64" else (None, None, None, None)
    if prec != "fp64":
        from qodeapplications_gb300.densities import FragmentSpace
        from qodeapplications_gb300.hamiltonian import DeviceIntegrals, XRDimerPlan
        sysd = S.make_system(n_frag=2, n_orb=4, n_states=3, charges=CHG, seed=31)
        spaces = [FragmentSpace({c: sysd["states"][m][c][1] for c in CHG}, 4, 0, 4) for m in range(2)]
        plan = XRDimerPlan(spaces, [{c: 3 for c in CHG}] * 2, [list(CHG)] * 2,
                           DeviceIntegrals(h=sysd["h"], V=sysd["V"], Ns=sysd["Ns"]), precision=prec)
        adj = Gm.XRDimerAdjoint(plan)
        coeffs = [{c: torch.as_tensor(sysd["states"][m][c][0], device="cuda") for c in CHG} for m in range(2)]
    _gpu_energy_and_grad(plan, adj, coeffs)
    T = torch.as_tensor(sysd["h"], device="cuda").contiguous()
    U = torch.zeros((2,) + T.shape, dtype=torch.float64, device="cuda")
    U[0] = 0.01 * T                    # nonzero fragment potentials exercise the U terms
    V = torch.as_tensor(sysd["V"], device="cuda").contiguous()
    sidx = S.spin_orbital_spatial_index([4, 4])
    out = {}
    for fused in (True, False):
        monkeypatch.setattr(Gm, "ORBITAL_FUSED", fused)
        out[fused] = adj.orbital_gradient(T, U, V, sidx).clone()
    torch.cuda.synchronize()
    tol = 1e-12 if prec == "fp64" else 1e-5
    assert float((out[True] - out[False]).norm() / out[False].norm()) < tol
