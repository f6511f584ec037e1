"""GPU parity at the benchmark workloads, against the FP64 oracle.

* dimer 2 x 9 spatial orbitals, 10 states per charge sector (+1, 0, -1), H 900 x 900, the
  seeded system of the benchmark with fragment nuclear potentials U != 0 (T = h - sum U), so
  the u-diagrams (SU_1mer_0.py:24, SU_2mer_0.py:37-118) and the extPot terms of the
  general-XRCC convention (build_H.py:72, :84-87) are exercised:
    - FP64: max |dH| <= 1e-12 against the oracle's product-order H, lowest five eigenvalues
      (this library's Lanczos) within 1e-10 of the oracle's dense eigensolve, in both sign
      conventions;
    - 3 x BF16 and 3 x TF32 (tcgen05): lowest eigenvalue within 1e-6 Eh of the oracle,
      per-charge-block max |dH| reported and bounded by 1e-4;
* dimer 2 x 14 spatial orbitals, 60 states per charge sector: dE/dz and dE/dkappa of the
  lowest eigenvalue (adjoint kernels, FP64) against central finite differences of the FP64
  GPU energy (step 1e-5) along 20 directions at kappa ~ N(0, 1e-3): relative error <= 1e-5;
* the build_density_tensors drop-in (general-XRCC/build_density_tensors.py:57) on the
  reference's Be fixture states against the reference kernels' golden probes.
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
SEED = 1234          # the benchmark's seed


@pytest.fixture(scope="module")
def cfg0():
    sysd = S.make_system(n_frag=2, n_orb=9, n_states=10, charges=CHG, seed=SEED)
    U = S.make_nuclear_potentials(2, 9)
    ints = O.FragInts(sysd["h"], sysd["V"], sysd["Ns"], U=U)
    dens = [O.build_densities({c: O.Sector(*sysd["states"][m][c]) for c in CHG}, 9, 0, 4) for m in range(2)]
    H1, H2 = O.get_xr_H0(ints, dens, [CHG, CHG])
    Href = O.full_H(H1, H2)
    w_ref = np.linalg.eigvalsh(Href)[:5]
    return dict(sysd=sysd, U=U, ints=ints, dens=dens, H1=H1, H2=H2, Href=Href, w_ref=w_ref)


def _plan(cfg, precision="fp64", output="full", convention="hermitian", charges=CHG):
    from qodeapplications_gb300.densities import FragmentSpace
    from qodeapplications_gb300.hamiltonian import DeviceIntegrals, XRDimerPlan
    sysd = cfg["sysd"]
    spaces = [FragmentSpace({c: sysd["states"][m][c][1] for c in charges}, 9, 0, 4) for m in range(2)]
    ns = [{c: 10 for c in charges}] * 2
    ints = DeviceIntegrals(h=sysd["h"], V=sysd["V"], Ns=sysd["Ns"], U=cfg["U"])
    plan = XRDimerPlan(spaces, ns, [list(charges)] * 2, ints, output=output, precision=precision,
                       convention=convention)
    coeffs = [{c: torch.as_tensor(sysd["states"][m][c][0], device="cuda") for c in charges} for m in range(2)]
    return plan, coeffs


def _blocks_max_err(H, Href, n=10, charges=CHG):
    """max |dH| per (i0, i1 | j0, j1) charge block of the product-order matrix."""
    nc = len(charges)
    out = {}
    A = np.abs(H - Href).reshape(nc, n, nc, n, nc, n, nc, n)
    for a in range(nc):
        for b in range(nc):
            for c in range(nc):
                for d in range(nc):
                    err = float(A[a, :, b, :, c, :, d, :].max())
                    if err > 0:
                        out[(charges[a], charges[b], charges[c], charges[d])] = err
    return out


def test_cfg0_fp64_matches_oracle(cfg0):
    from qodeapplications_gb300.eigen import lowest_eigenpairs
    plan, coeffs = _plan(cfg0)
    H = plan.build(coeffs)
    w, vecs = lowest_eigenpairs(H, 5, tol=1e-11)
    torch.cuda.synchronize()
    err = float(np.abs(H.cpu().numpy() - cfg0["Href"]).max())
    assert err <= 1e-12, err
    np.testing.assert_allclose(w, cfg0["w_ref"], rtol=0, atol=1e-10)
    # the ground vector is an eigenvector of the oracle H
    v = vecs[:, 0].cpu().numpy()
    assert np.abs(cfg0["Href"] @ v - w[0] * v).max() < 1e-8


def test_cfg0_fp64_split_output_matches_oracle(cfg0):
    """output='split' = get_xr_H's (H1, H2) (get_xr_result.py:45,355) with U != 0."""
    plan, coeffs = _plan(cfg0, output="split")
    H2 = plan.build(coeffs).cpu().numpy()
    np.testing.assert_allclose(H2, cfg0["H2"], rtol=0, atol=1e-12)
    for m, h1 in enumerate(plan.H1()):
        np.testing.assert_allclose(h1.cpu().numpy(), cfg0["H1"][m], rtol=0, atol=1e-12)


@pytest.mark.parametrize("precision", ["bf16x3", "tf32x3"])
def test_cfg0_split_precision_energy_within_1e6(cfg0, precision):
    from qodeapplications_gb300.eigen import lowest_eigenpairs
    plan, coeffs = _plan(cfg0, precision=precision)
    H = plan.build(coeffs)
    w, _ = lowest_eigenpairs(H, 5, tol=1e-10)
    torch.cuda.synchronize()
    plan.check_status()
    blocks = _blocks_max_err(H.cpu().numpy(), cfg0["Href"])
    worst = max(blocks.values())
    dE = np.abs(w - cfg0["w_ref"])
    print(f"{precision}: |dE0| = {dE[0]:.3e}, lowest five max {dE.max():.3e}, "
          f"max |dH| over {len(blocks)} charge blocks = {worst:.3e}")
    assert dE[0] <= 1e-6, dE
    assert dE.max() <= 1e-6, dE
    assert worst <= 1e-4, worst


def test_cfg0_general_convention_matches_element_formulas(cfg0):
    """The general-XRCC sign convention (build_H.py:56-102) at the 2 x 9 / 10-state size with
    U != 0, block by block against the oracle's element formulas (gen_dimer_block), and the
    same spectrum as the hermitian convention (the two differ by a diagonal gauge)."""
    from qodeapplications_gb300.eigen import lowest_eigenpairs
    charges = [0, +1, -1]       # general-XRCC order: reference charge first (Be631g.py:77-81)
    oi, dens = cfg0["ints"], cfg0["dens"]
    plan, coeffs = _plan(cfg0, output="split", convention="general", charges=charges)
    H = plan.build(coeffs).cpu().numpy()
    off = np.array([0, 10, 20, 30])
    ref = np.zeros((30,) * 4)
    for a, ci1 in enumerate(charges):
        for b, ci2 in enumerate(charges):
            for c, cj1 in enumerate(charges):
                for d, cj2 in enumerate(charges):
                    blk = O.gen_dimer_block(dens, oi.T, oi.U, oi.V, [4, 4], [[0, 0], [0, 0]], 0, 1, ci1, cj1, ci2, cj2)
                    if blk is not None:
                        ref[off[a]:off[a + 1], off[b]:off[b + 1], off[c]:off[c + 1], off[d]:off[d + 1]] += blk
    np.testing.assert_allclose(H, ref.reshape(900, 900), rtol=0, atol=1e-12)
    full, coeffs = _plan(cfg0, output="full", convention="general", charges=charges)
    w, _ = lowest_eigenpairs(full.build(coeffs), 5, tol=1e-11)
    np.testing.assert_allclose(w, cfg0["w_ref"], rtol=0, atol=1e-10)


# --------------------------------------------------------------------------------------------
# finite differences at 2 x 14 spatial orbitals / 60 states per charge sector
# --------------------------------------------------------------------------------------------

def test_cfg3_gradients_match_finite_differences():
    from qodeapplications_gb300.autograd import XRDimerEnergy, rotate_integrals
    sysd = S.make_system(n_frag=2, n_orb=14, n_states=60, charges=CHG, seed=SEED)
    dev = "cuda"
    eng = XRDimerEnergy.from_system(sysd, precision="fp64", tol=1e-10, lanczos_m=64)
    h0 = torch.as_tensor(sysd["h"], device=dev)
    V0 = torch.as_tensor(sysd["V"], device=dev)
    rng = np.random.default_rng(17)
    n_sp = 28
    k0 = rng.normal(0.0, 1e-3, (n_sp, n_sp))
    kappa0 = torch.as_tensor(k0 - k0.T, device=dev)
    z0 = [{c: torch.as_tensor(sysd["states"][m][c][0], device=dev) for c in CHG} for m in range(2)]

    def energy(kappa, zs):
        h, V = rotate_integrals(h0, V0, kappa, [14, 14])
        return float(eng(h, V, zs))

    # the adjoint: dE/dz and dE/dkappa at (kappa0, z0)
    kap = kappa0.clone().requires_grad_(True)
    zr = [{c: z.clone().requires_grad_(True) for c, z in d.items()} for d in z0]
    h, V = rotate_integrals(h0, V0, kap, [14, 14])
    E = eng(h, V, zr)
    E.backward()
    gk = kap.grad.clone()
    gz = [{c: zr[m][c].grad.clone() for c in CHG} for m in range(2)]
    assert eng.residual < 1e-9

    eps = 1e-5
    checks = []
    # 10 unit state-coefficient directions: 5 dense ones (the normalised gradient plus a
    # random unit vector, so that the directional derivative is not lost in the 10^7
    # dimensions), 5 single coefficients among the 200 largest |dE/dz|
    flat = torch.cat([gz[m][c].reshape(-1) for m in range(2) for c in CHG]).abs().cpu().numpy()
    top = np.argsort(flat)[-200:]
    sizes = [gz[m][c].numel() for m in range(2) for c in CHG]
    offs = np.concatenate([[0], np.cumsum(sizes)])
    gnorm = float(np.sqrt(sum(float((gz[m][c] ** 2).sum()) for m in range(2) for c in CHG)))
    for i in range(10):
        if i < 5:
            R = [{c: torch.as_tensor(rng.standard_normal(z0[m][c].shape), device=dev) for c in CHG} for m in range(2)]
            rnorm = float(np.sqrt(sum(float((R[m][c] ** 2).sum()) for m in range(2) for c in CHG)))
            D = [{c: gz[m][c] / gnorm + R[m][c] / rnorm for c in CHG} for m in range(2)]
            dnorm = float(np.sqrt(sum(float((D[m][c] ** 2).sum()) for m in range(2) for c in CHG)))
            D = [{c: D[m][c] / dnorm for c in CHG} for m in range(2)]
        else:
            pos = int(rng.choice(top))
            D = [{c: torch.zeros_like(z0[m][c]) for c in CHG} for m in range(2)]
            blk = int(np.searchsorted(offs, pos, side="right") - 1)
            m, c = divmod(blk, 3)
            D[m][CHG[c]].view(-1)[pos - offs[blk]] = 1.0
        pred = sum(float((gz[m][c] * D[m][c]).sum()) for m in range(2) for c in CHG)
        ep = energy(kappa0, [{c: z0[m][c] + eps * D[m][c] for c in CHG} for m in range(2)])
        em = energy(kappa0, [{c: z0[m][c] - eps * D[m][c] for c in CHG} for m in range(2)])
        checks.append(("z", i, (ep - em) / (2 * eps), pred))
    # 10 orbital-rotation directions: 5 dense antisymmetric, 5 single pairs among the 50
    # largest |dE/dkappa_pq|
    gkn = gk.cpu().numpy()
    iu = np.triu_indices(n_sp, 1)
    order = np.argsort(np.abs(gkn[iu]))[-50:]
    for i in range(10):
        if i < 5:
            a = rng.standard_normal((n_sp, n_sp))
            Dk = a - a.T
            Dk = Dk / np.linalg.norm(Dk) + gkn / np.linalg.norm(gkn)
            Dk = Dk / np.linalg.norm(Dk)
        else:
            j = int(rng.choice(order))
            p, q = iu[0][j], iu[1][j]
            Dk = np.zeros((n_sp, n_sp))
            Dk[p, q], Dk[q, p] = 1.0, -1.0
        Dk = torch.as_tensor(Dk, device=dev)
        pred = float((gk * Dk).sum())
        ep = energy(kappa0 + eps * Dk, z0)
        em = energy(kappa0 - eps * Dk, z0)
        checks.append(("kappa", i, (ep - em) / (2 * eps), pred))
    worst = 0.0
    for kind, i, fd, pred in checks:
        rel = abs(fd - pred) / max(abs(fd), 1e-12)
        worst = max(worst, rel)
        assert rel <= 1e-5, (kind, i, fd, pred, rel)
    print(f"2x14/60 states: {len(checks)} FD directions, worst relative error {worst:.2e}")


# --------------------------------------------------------------------------------------------
# build_density_tensors drop-in on the reference's Be fixture states
# --------------------------------------------------------------------------------------------

def test_build_density_tensors_dropin_matches_reference_kernels(golden_dir):
    from qodeapplications_gb300.densities import build_density_tensors
    g = np.load(os.path.join(golden_dir, "be_densities.npz"))
    n_orbs, n_core, N = 9, 1, 18
    z_lists = {}
    for c in (+1, 0, -1):
        masks = g[f"masks_{c}"]
        occ = np.array([[o for o in range(N) if (int(mk) >> o) & 1] for mk in masks], dtype=np.int64)
        z_lists[c] = types.SimpleNamespace(configs=occ, coeffs=g[f"coeffs_{c}"])
    rng = np.random.default_rng(3)
    L = rng.normal(0, 0.05, (10, n_orbs, n_orbs))
    L = L + L.transpose(0, 2, 1)
    _, Vints = S.spin_orbital_integrals(np.zeros((n_orbs, n_orbs)), np.einsum("kpq,krs->pqrs", L, L), [n_orbs])
    dens, total = build_density_tensors(z_lists, n_orbs, Vints, n_core)
    checked, size = 0, 0
    for bc in (+1, 0, -1):
        for kc in (+1, 0, -1):
            for op in O.OPS_FOR_DCHG.get(bc - kc, ()):
                blk = dens[op][(bc, kc)]
                nb, nk = len(blk), len(blk[0])
                if op == "ccaa":
                    got = np.array([[blk[i][j] for j in range(nk)] for i in range(nb)])
                    sec = O.Sector(g[f"coeffs_{bc}"], g[f"masks_{bc}"])
                    ccaa = O.transition_density("ccaa", sec.coeffs, sec.masks, sec.coeffs, sec.masks, N, n_orbs, n_core)
                    np.testing.assert_allclose(got, O.gen_monomer_2e(ccaa, Vints), rtol=0, atol=1e-12)
                    size += nb * nk
                else:
                    rho = np.array([[blk[i][j] for j in range(nk)] for i in range(nb)])
                    assert rho.shape == (nb, nk) + (N,) * len(op)
                    flat = rho.reshape(nb, nk, -1)
                    w = np.cos(0.37 * np.arange(flat.shape[2]) + 0.1)
                    np.testing.assert_allclose(flat @ w, g[f"probe_{op}_{bc}_{kc}"], rtol=0, atol=1e-12)
                    np.testing.assert_allclose((flat ** 2).sum(-1), g[f"norm2_{op}_{bc}_{kc}"], rtol=1e-12, atol=1e-12)
                    if len(op) <= 2:
                        np.testing.assert_allclose(rho, g[f"full_{op}_{bc}_{kc}"], rtol=0, atol=1e-13)
                    size += rho.size
                checked += 1
    assert checked == 16
    assert total == size
