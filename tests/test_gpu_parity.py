"""GPU parity: the CUDA path (libxrh.so through its C ABI) against the FP64 oracle."""
import numpy as np
import pytest

import xr_oracle as O
from qodeapplications_gb300 import synthetic as S

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _system(n_orb=5, n_states=4, seed=21, charges=(+1, 0, -1)):
    return S.make_system(n_frag=2, n_orb=n_orb, n_states=n_states, charges=charges, seed=seed)


def _oracle_H(sysd, charges):
    N = 2 * sysd["n_orb"]
    ints = O.FragInts(sysd["h"], sysd["V"], sysd["Ns"])
    dens = []
    for m in range(2):
        secs = {c: O.Sector(*sysd["states"][m][c]) for c in charges}
        dens.append(O.build_densities(secs, sysd["n_orb"], sysd["n_core"], sysd["n_elec_ref"]))
    H1, H2 = O.get_xr_H0(ints, dens, [list(charges), list(charges)])
    return ints, dens, H1, H2, N


def _plan(sysd, charges, output="full", precision="fp64", convention="hermitian"):
    from qodeapplications_gb300.densities import FragmentSpace
    from qodeapplications_gb300.hamiltonian import DeviceIntegrals, XRDimerPlan
    spaces = [FragmentSpace({c: sysd["states"][m][c][1] for c in charges}, sysd["n_orb"], sysd["n_core"],
                            sysd["n_elec_ref"]) for m in range(2)]
    ns = [{c: sysd["states"][m][c][0].shape[0] for c in charges} for m in range(2)]
    ints = DeviceIntegrals(h=sysd["h"], V=sysd["V"], Ns=sysd["Ns"])
    plan = XRDimerPlan(spaces, ns, [list(charges)] * 2, ints, output=output, precision=precision,
                       convention=convention)
    coeffs = [{c: torch.as_tensor(sysd["states"][m][c][0], device="cuda") for c in charges} for m in range(2)]
    return plan, coeffs


def test_densities_match_oracle():
    from qodeapplications_gb300.densities import DensityBuilder, FragmentSpace
    sysd = _system()
    charges = (+1, 0, -1)
    st = sysd["states"][0]
    space = FragmentSpace({c: st[c][1] for c in charges}, sysd["n_orb"], 0, 4)
    b = DensityBuilder(space, {c: st[c][0].shape[0] for c in charges})
    rho = b.build({c: torch.as_tensor(st[c][0], device="cuda") for c in charges})
    N = 2 * sysd["n_orb"]
    n = 0
    for op, blocks in rho.items():
        for (bc, kc), t in blocks.items():
            ref = O.transition_density(op, st[bc][0], st[bc][1], st[kc][0], st[kc][1], N, sysd["n_orb"], 0)
            np.testing.assert_allclose(t.cpu().numpy(), ref, rtol=0, atol=1e-13)
            n += 1
    assert n == 13        # 16 blocks of the reference minus the 3 ccaa blocks (never stored)


def test_density_fp32_variant_close():
    from qodeapplications_gb300.densities import DensityBuilder, FragmentSpace
    sysd = _system()
    st = sysd["states"][1]
    charges = (+1, 0, -1)
    space = FragmentSpace({c: st[c][1] for c in charges}, sysd["n_orb"], 0, 4)
    b = DensityBuilder(space, {c: st[c][0].shape[0] for c in charges}, precision="fp32")
    rho = b.build({c: torch.as_tensor(st[c][0], device="cuda") for c in charges})
    N = 2 * sysd["n_orb"]
    ref = O.transition_density("caa", st[0][0], st[0][1], st[-1][0], st[-1][1], N, sysd["n_orb"], 0)
    np.testing.assert_allclose(rho["caa"][(0, -1)].cpu().numpy(), ref, rtol=0, atol=2e-6)


@pytest.mark.parametrize("path", ["units", "cta"])
@pytest.mark.parametrize("n_states", [10, 7, 40])
def test_density_fp32_paths_match_fp64(path, n_states, monkeypatch):
    """Every FP32 block (warp-per-unit kernel, including operator indices split over several
    units, or the CTA-per-index kernel) against the FP64 build, to FP32 accuracy: 2e-6 of
    the block's largest element (64 couplings or fewer per FP32 partial sum)."""
    from qodeapplications_gb300 import densities as D
    if path == "cta":
        monkeypatch.setattr(D, "UNIT_MAX_STATES", 0)
    sysd = S.make_system(n_frag=2, n_orb=9, n_states=n_states, charges=(+1, 0, -1), seed=5)
    st = sysd["states"][0]
    charges = (+1, 0, -1)
    space = D.FragmentSpace({c: st[c][1] for c in charges}, sysd["n_orb"], sysd["n_core"], sysd["n_elec_ref"])
    ns = {c: st[c][0].shape[0] for c in charges}
    co = {c: torch.as_tensor(st[c][0], device="cuda") for c in charges}
    b32 = D.DensityBuilder(space, ns, precision="fp32")
    if path == "units" and n_states <= 20:
        assert b32._n_units > 0
        assert b32._unit_zero is not None          # some index has more than one unit
    r32 = {op: {k: t.clone() for k, t in blocks.items()} for op, blocks in b32.build(co).items()}
    r64 = D.DensityBuilder(space, ns, precision="fp64").build(co)
    for op, blocks in r64.items():
        for key, t in blocks.items():
            scale = max(t.abs().max().item(), 1e-30)
            assert (r32[op][key] - t).abs().max().item() <= 2e-6 * scale, (op, key)
    # a second build with the same buffers gives the same result (the split arena is re-zeroed)
    again = b32.build(co)
    for op, blocks in again.items():
        for key, t in blocks.items():
            assert torch.equal(t, r32[op][key]) or (t - r32[op][key]).abs().max().item() < 1e-12


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_densities_with_separate_bra_states_match_oracle(precision):
    """Transition densities between different bra and ket state sets (the determinant-bra
    densities of the reference's state gradient) through DensityBuilder(mirror=False)."""
    from qodeapplications_gb300.densities import DensityBuilder, FragmentSpace
    sysd = _system(n_states=3)
    charges = (+1, 0, -1)
    st = sysd["states"][0]
    rng = np.random.default_rng(8)
    bra = {c: rng.standard_normal((5, st[c][0].shape[1])) for c in charges}
    space = FragmentSpace({c: st[c][1] for c in charges}, sysd["n_orb"], 0, 4)
    b = DensityBuilder(space, {c: 3 for c in charges}, precision=precision, n_states_bra={c: 5 for c in charges},
                       mirror=False)
    rho = b.build({c: torch.as_tensor(st[c][0], device="cuda") for c in charges},
                  bra_coeffs={c: torch.as_tensor(bra[c], device="cuda") for c in charges})
    N = 2 * sysd["n_orb"]
    tol = 1e-13 if precision == "fp64" else 2e-6
    for op, blocks in rho.items():
        for (bc, kc), t in blocks.items():
            ref = O.transition_density(op, bra[bc], st[bc][1], st[kc][0], st[kc][1], N, sysd["n_orb"], 0)
            np.testing.assert_allclose(t.cpu().numpy(), ref, rtol=0, atol=tol * max(1.0, np.abs(ref).max()))


def test_monomer_two_electron_matches_oracle():
    from qodeapplications_gb300.densities import FragmentSpace
    from qodeapplications_gb300.hamiltonian import DeviceIntegrals, monomer_two_electron
    sysd = _system()
    st = sysd["states"][0]
    space = FragmentSpace({c: st[c][1] for c in (0, -1)}, sysd["n_orb"], 0, 4)
    ints = DeviceIntegrals(h=sysd["h"], V=sysd["V"], Ns=sysd["Ns"])
    oi = O.FragInts(sysd["h"], sysd["V"], sysd["Ns"])
    N = 2 * sysd["n_orb"]
    for c in (0, -1):
        got = monomer_two_electron(space, {c: torch.as_tensor(st[c][0], device="cuda")}, ints.V(0, 0, 0, 0), c)
        ccaa = O.transition_density("ccaa", st[c][0], st[c][1], st[c][0], st[c][1], N, sysd["n_orb"], 0)
        ref = O.gen_monomer_2e(ccaa, oi.V[0, 0, 0, 0])
        np.testing.assert_allclose(got.cpu().numpy(), ref, rtol=0, atol=1e-12)


@pytest.mark.parametrize("output", ["split", "full"])
def test_dimer_H_matches_oracle(output):
    sysd = _system()
    charges = (+1, 0, -1)
    _, _, H1, H2, _ = _oracle_H(sysd, charges)
    plan, coeffs = _plan(sysd, charges, output=output)
    H = plan.build(coeffs).cpu().numpy()
    if output == "split":
        np.testing.assert_allclose(H, H2, rtol=0, atol=1e-12)
        for m, h1 in enumerate(plan.H1()):
            np.testing.assert_allclose(h1.cpu().numpy(), H1[m], rtol=0, atol=1e-12)
    else:
        np.testing.assert_allclose(H, O.full_H(H1, H2), rtol=0, atol=1e-12)


def test_dimer_H_known_answer_fci_complete_basis():
    """Complete fragment bases over charges -2..+2: GPU H equals the supersystem FCI."""
    rng = np.random.default_rng(7)
    n_orb, n_ref = 3, 2
    N = 2 * n_orb
    nsp = 2 * n_orb
    a = rng.normal(0, 0.3, (nsp, nsp))
    L = rng.normal(0, 0.2, (5, nsp, nsp))
    L = L + L.transpose(0, 2, 1)
    h, V = S.spin_orbital_integrals(a + a.T, np.einsum("kpq,krs->pqrs", L, L), [n_orb, n_orb])
    charges = [2, 1, 0, -1, -2]
    states = []
    for _m in range(2):
        states.append({c: (np.eye(len(O.all_configs(n_orb, 0, n_ref - c))), O.all_configs(n_orb, 0, n_ref - c))
                       for c in charges})
    sysd = dict(n_orb=n_orb, n_core=0, n_elec_ref=n_ref, h=h, V=V, Ns=[N, N], states=states)
    plan, coeffs = _plan(sysd, charges, output="full")
    Hx = plan.build(coeffs).cpu().numpy()
    m0 = np.concatenate([states[0][c][1] for c in charges])
    m1 = np.concatenate([states[1][c][1] for c in charges])
    G = (m0[:, None] | (m1[None, :] << np.uint64(N))).reshape(-1)
    n0, n1 = O.popcount(m0), O.popcount(m1)
    gauge = ((-1.0) ** (n0[:, None] * n1[None, :])).reshape(-1)
    Hf = gauge[:, None] * O.fci_hamiltonian(h, V, G) * gauge[None, :]
    sel = np.nonzero((n0[:, None] + n1[None, :]).reshape(-1) == 2 * n_ref)[0]
    np.testing.assert_allclose(Hx[np.ix_(sel, sel)], Hf[np.ix_(sel, sel)], rtol=0, atol=1e-12)


def test_general_convention_matches_element_formulas():
    sysd = _system(seed=5)
    charges = (0, +1, -1)       # general-XRCC order: reference charge first (Be631g.py:77-81)
    oi = O.FragInts(sysd["h"], sysd["V"], sysd["Ns"])
    dens = []
    for m in range(2):
        secs = {c: O.Sector(*sysd["states"][m][c]) for c in charges}
        dens.append(O.build_densities(secs, sysd["n_orb"], 0, 4))
    plan, coeffs = _plan(sysd, charges, output="split", convention="general")
    H = plan.build(coeffs).cpu().numpy()
    ns = [dens[0]["n_states"][c] for c in charges]
    off = np.concatenate([[0], np.cumsum(ns)])
    tot = off[-1]
    ref = np.zeros((tot,) * 4)
    for a, ci1 in enumerate(charges):
        for b, ci2 in enumerate(charges):
            for c, cj1 in enumerate(charges):
                for d, cj2 in enumerate(charges):
                    blk = O.gen_dimer_block(dens, oi.T, oi.U, oi.V, [4, 4], [[0, 0], [0, 0]], 0, 1, ci1, cj1, ci2, cj2)
                    if blk is not None:
                        ref[off[a]:off[a + 1], off[b]:off[b + 1], off[c]:off[c + 1], off[d]:off[d + 1]] += blk
    np.testing.assert_allclose(H, ref.reshape(tot * tot, -1), rtol=0, atol=1e-12)


def test_build_is_repeatable_and_tracks_new_states():
    """Buffers are reused: a second build with new coefficients gives the new answer."""
    sysd = _system(seed=9)
    charges = (+1, 0, -1)
    plan, coeffs = _plan(sysd, charges)
    H_a = plan.build(coeffs).cpu().numpy().copy()
    sysd2 = _system(seed=10)
    for m in range(2):
        for c in charges:
            sysd["states"][m][c] = (sysd2["states"][m][c][0], sysd["states"][m][c][1])
    _, _, H1, H2, _ = _oracle_H(sysd, charges)
    coeffs2 = [{c: torch.as_tensor(sysd["states"][m][c][0], device="cuda") for c in charges} for m in range(2)]
    H_b = plan.build(coeffs2).cpu().numpy()
    np.testing.assert_allclose(H_b, O.full_H(H1, H2), rtol=0, atol=1e-12)
    assert np.abs(H_a - H_b).max() > 1e-3


@pytest.mark.parametrize("prec", ["bf16x3", "tf32x3"])
def test_intermediate_densities_match_coupling_lists(prec):
    """Densities through intermediate determinants on the tensor cores (split precision)
    against the FP64 coupling-list build, every operator string and charge pair, frozen core
    included.  Tolerance of the largest element: 2e-6 for 3 x TF32 (22-bit split products,
    FP32 chunk sums; the route the plans use), 5e-5 for 3 x BF16 (16-bit split products)."""
    from qodeapplications_gb300.densities import DensityBuilder, FragmentSpace
    from qodeapplications_gb300.intermediates import IntermediateDensityBuilder
    chg = (+1, 0, -1)
    sysd = S.make_system(n_frag=1, n_orb=5, n_states=4, charges=chg, n_core=1, seed=17)
    st = sysd["states"][0]
    sp = FragmentSpace({c: st[c][1] for c in chg}, 5, 1, 4)
    ns = {c: 4 for c in chg}
    coeffs = {c: torch.as_tensor(st[c][0], device="cuda") for c in chg}
    ref = DensityBuilder(sp, ns).build(coeffs)
    im = IntermediateDensityBuilder(sp, ns, precision=prec)
    got = im.build(coeffs)
    torch.cuda.synchronize()
    im.check()
    n = 0
    for op, blocks in ref.items():
        for key, r in blocks.items():
            g = got[op][key]
            scale = max(float(r.abs().max()), 1e-30)
            tol = 2e-6 if prec == "tf32x3" else 5e-5
            assert float((g - r).abs().max()) <= tol * scale, (op, key, float((g - r).abs().max()) / scale)
            n += 1
    assert n == 13          # 3 ca, 4 a/caa, 4 c/cca, 1 aa, 1 cc over charges (+1, 0, -1)
