"""torch.autograd.Function over the device build and the adjoint (qodeapplications_gb300.autograd).

Tolerances: directional derivatives against central finite differences (step 1e-5) of the
FP64 oracle energy, relative 1e-6; split precision against FP64, relative 1e-5."""
import numpy as np
import pytest

import xr_oracle as O
from qodeapplications_gb300 import synthetic as S

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

CHG = (+1, 0, -1)
NORB = 4


def _system(seed=57):
    return S.make_system(n_frag=2, n_orb=NORB, n_states=3, charges=CHG, seed=seed)


def _inputs(sysd, requires_grad=True):
    h = torch.as_tensor(sysd["h"], device="cuda")
    V = torch.as_tensor(sysd["V"], device="cuda")
    z = [{c: torch.as_tensor(sysd["states"][m][c][0], device="cuda").requires_grad_(requires_grad) for c in CHG}
         for m in range(2)]
    return h, V, z


def _oracle_energy(sysd, h, V, states=None):
    E, _, _, _ = O.xr_energy(h, V, sysd["Ns"], NORB, 0, 4, states or sysd["states"], CHG)
    return E


def test_energy_matches_oracle_and_state_gradient_matches_fd():
    from qodeapplications_gb300.autograd import XRDimerEnergy
    sysd = _system()
    f = XRDimerEnergy.from_system(sysd)
    h, V, z = _inputs(sysd)
    E = f(h, V, z)
    assert abs(float(E) - _oracle_energy(sysd, sysd["h"], sysd["V"])) < 1e-10
    E.backward()
    rng = np.random.default_rng(3)
    eps = 1e-5
    for _ in range(2):
        dirs = [{c: rng.standard_normal(sysd["states"][m][c][0].shape) for c in CHG} for m in range(2)]
        an = sum(float((z[m][c].grad.cpu().numpy() * dirs[m][c]).sum()) for m in range(2) for c in CHG)
        Es = []
        for sgn in (+1, -1):
            st = [{c: (sysd["states"][m][c][0] + sgn * eps * dirs[m][c], sysd["states"][m][c][1]) for c in CHG}
                  for m in range(2)]
            Es.append(_oracle_energy(sysd, sysd["h"], sysd["V"], st))
        fd = (Es[0] - Es[1]) / (2 * eps)
        assert abs(an - fd) <= 1e-6 * max(1.0, abs(fd)), (an, fd)


def test_orbital_rotation_gradient_by_autograd_matches_fd():
    from qodeapplications_gb300.autograd import XRDimerEnergy, rotate_integrals
    sysd = _system(seed=58)
    f = XRDimerEnergy.from_system(sysd)
    h, V, z = _inputs(sysd, requires_grad=False)
    n_sp = 2 * NORB
    rng = np.random.default_rng(5)
    k0 = rng.normal(0.0, 1e-3, size=(n_sp, n_sp))
    k0 = k0 - k0.T
    kappa = torch.as_tensor(k0, device="cuda").requires_grad_(True)
    h2, V2 = rotate_integrals(h, V, kappa, [NORB, NORB])
    E = f(h2, V2, z)
    E.backward()
    G = kappa.grad.cpu().numpy()
    eps = 1e-5
    for _ in range(3):
        D = rng.standard_normal((n_sp, n_sp))
        D = D - D.T
        an = float((G * D).sum())
        Es = []
        for sgn in (+1, -1):
            hh, VV = S.rotate_integrals(sysd["h"], sysd["V"], k0 + sgn * eps * D, [NORB, NORB])
            Es.append(_oracle_energy(sysd, hh, VV))
        fd = (Es[0] - Es[1]) / (2 * eps)
        assert abs(an - fd) <= 1e-6 * max(1.0, abs(fd)), (an, fd)


def test_autograd_orbital_gradient_at_zero_equals_adjoint_formula():
    from qodeapplications_gb300.autograd import XRDimerEnergy, rotate_integrals
    sysd = _system(seed=59)
    f = XRDimerEnergy.from_system(sysd)
    h, V, z = _inputs(sysd, requires_grad=False)
    kappa = torch.zeros((2 * NORB, 2 * NORB), dtype=torch.float64, device="cuda", requires_grad=True)
    h2, V2 = rotate_integrals(h, V, kappa, [NORB, NORB])
    f(h2, V2, z).backward()
    U = torch.zeros((2,) + h.shape, dtype=torch.float64, device="cuda")
    K = f.adj.orbital_gradient(h, U, V, S.spin_orbital_spatial_index([NORB, NORB]))
    # autograd gives dE/dkappa over the full matrix; on antisymmetric directions it pairs
    # with the antisymmetric adjoint formula: G - G^T == K
    G = kappa.grad
    assert float((G - G.t() - K).abs().max()) < 1e-10


def test_backward_recomputes_after_another_forward():
    from qodeapplications_gb300.autograd import XRDimerEnergy
    sysd = _system(seed=60)
    f = XRDimerEnergy.from_system(sysd)
    h, V, z = _inputs(sysd)
    E1 = f(h, V, z)
    g_direct = torch.autograd.grad(E1, [z[0][0]], retain_graph=True)[0].clone()
    # another forward at other integrals overwrites the plan's densities and H
    f(h * 1.01, V, [{c: t.detach() for c, t in zm.items()} for zm in z])
    g_again = torch.autograd.grad(E1, [z[0][0]])[0]
    assert float((g_again - g_direct).abs().max()) < 1e-11


@pytest.mark.parametrize("precision", ["bf16x3", "tf32x3"])
def test_split_precision_autograd_within_1e5(precision):
    from qodeapplications_gb300.autograd import XRDimerEnergy, rotate_integrals
    sysd = _system(seed=61)
    out = {}
    for prec in ("fp64", precision):
        f = XRDimerEnergy.from_system(sysd, precision=prec)
        h, V, z = _inputs(sysd)
        kappa = torch.zeros((2 * NORB, 2 * NORB), dtype=torch.float64, device="cuda", requires_grad=True)
        h2, V2 = rotate_integrals(h, V, kappa, [NORB, NORB])
        E = f(h2, V2, z)
        E.backward()
        gz = torch.cat([z[m][c].grad.reshape(-1) for m in range(2) for c in CHG])
        out[prec] = (float(E), gz, kappa.grad.clone())
    E64, gz64, gk64 = out["fp64"]
    E32, gz32, gk32 = out[precision]
    assert abs(E32 - E64) < 1e-6
    assert float((gz32 - gz64).norm() / gz64.norm()) < 1e-5
    assert float((gk32 - gk64).norm() / gk64.norm()) < 1e-5
