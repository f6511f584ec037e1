"""GPU trimer blocks (qodeapplications_gb300.trimer) against the oracle's restatement of
general-XRCC/build_H.py:103-188, which is itself pinned to the compiled reference kernels
(be_trimer_elements.npz) and to the 3-fragment FCI identity (test_oracle.py).
Tolerance: 1e-12 relative (FP64 GEMMs, different summation order)."""
import numpy as np
import pytest

import xr_oracle as O
from qodeapplications_gb300 import synthetic as S

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

CHG = (+1, 0, -1)


def _trimer_system(seed=21, n_orb=3, n_states=2, n_ref=4):
    sysd = S.make_system(n_frag=3, n_orb=n_orb, n_states=n_states, charges=CHG, n_elec_ref=n_ref, seed=seed)
    rng = np.random.default_rng(seed + 1)
    nsp = 3 * n_orb
    U = []
    for _k in range(3):
        b = rng.normal(0, 0.1, (nsp, nsp))
        U.append(S.spin_orbital_integrals(b + b.T, np.zeros((nsp,) * 4), [n_orb] * 3)[0])
    U = np.array(U)
    return sysd, sysd["h"] + U.sum(0), U


def test_trimer_blocks_match_oracle():
    from qodeapplications_gb300.densities import DensityBuilder, FragmentSpace
    from qodeapplications_gb300.hamiltonian import DeviceIntegrals
    from qodeapplications_gb300.trimer import XRTrimerPlan
    n_orb, n_ref = 3, 4
    sysd, htot, U = _trimer_system()
    ns = {c: sysd["states"][0][c][0].shape[0] for c in CHG}
    rho = []
    for m in range(3):
        sp = FragmentSpace({c: sysd["states"][m][c][1] for c in CHG}, n_orb, 0, n_ref)
        b = DensityBuilder(sp, ns)
        b.build({c: torch.as_tensor(sysd["states"][m][c][0], device="cuda") for c in CHG})
        rho.append(b.rho)
    ints = DeviceIntegrals(h=htot, V=sysd["V"], Ns=sysd["Ns"], U=U)
    plan = XRTrimerPlan(rho, ints, [n_ref] * 3, [CHG] * 3, [ns] * 3)
    plan.launch()
    torch.cuda.synchronize()
    oi = O.FragInts(htot, sysd["V"], sysd["Ns"], U=U)
    od = [O.build_densities({c: O.Sector(*sysd["states"][m][c]) for c in CHG}, n_orb, 0, n_ref,
                            ops=("a", "c", "ca", "aa", "cc")) for m in range(3)]
    n_checked = 0
    for ci in np.ndindex(3, 3, 3):
        for cj in np.ndindex(3, 3, 3):
            chg_i, chg_j = tuple(CHG[k] for k in ci), tuple(CHG[k] for k in cj)
            ref = O.gen_trimer_block(od, oi.T, oi.U, oi.V, [n_ref] * 3, (0, 1, 2), chg_i, chg_j)
            got = plan.block(chg_i, chg_j)
            if ref is None:
                assert got is None
                continue
            g = got.cpu().numpy()
            scale = max(1.0, np.abs(ref).max())
            assert np.abs(g - ref).max() <= 1e-12 * scale, (chg_i, chg_j, np.abs(g - ref).max())
            n_checked += 1
    assert n_checked == 96          # charge blocks with one of the three trimer cases


def test_trimer_relaunch_after_density_rebuild():
    """The plan reads the densities in place: new states, rebuild, launch again."""
    from qodeapplications_gb300.densities import DensityBuilder, FragmentSpace
    from qodeapplications_gb300.hamiltonian import DeviceIntegrals
    from qodeapplications_gb300.trimer import XRTrimerPlan
    n_orb, n_ref = 3, 4
    sysd, htot, U = _trimer_system(seed=22)
    sysd2 = S.make_system(n_frag=3, n_orb=n_orb, n_states=2, charges=CHG, n_elec_ref=n_ref, seed=99)
    ns = {c: 2 for c in CHG}
    builders = []
    for m in range(3):
        sp = FragmentSpace({c: sysd["states"][m][c][1] for c in CHG}, n_orb, 0, n_ref)
        builders.append(DensityBuilder(sp, ns))
    ints = DeviceIntegrals(h=htot, V=sysd["V"], Ns=sysd["Ns"], U=U)
    for b, m in zip(builders, range(3)):
        b.build({c: torch.as_tensor(sysd["states"][m][c][0], device="cuda") for c in CHG})
    plan = XRTrimerPlan([b.rho for b in builders], ints, [n_ref] * 3, [CHG] * 3, [ns] * 3)
    plan.launch()
    for b, m in zip(builders, range(3)):
        # same determinant lists, other coefficients
        b.build({c: torch.as_tensor(sysd2["states"][m][c][0], device="cuda") for c in CHG})
    plan.launch()
    torch.cuda.synchronize()
    oi = O.FragInts(htot, sysd["V"], sysd["Ns"], U=U)
    states2 = [{c: (sysd2["states"][m][c][0], sysd["states"][m][c][1]) for c in CHG} for m in range(3)]
    od = [O.build_densities({c: O.Sector(*states2[m][c]) for c in CHG}, n_orb, 0, n_ref,
                            ops=("a", "c", "ca", "aa", "cc")) for m in range(3)]
    for key in plan.keys():
        ref = O.gen_trimer_block(od, oi.T, oi.U, oi.V, [n_ref] * 3, (0, 1, 2), *key)
        assert np.abs(plan.block(*key).cpu().numpy() - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max())
