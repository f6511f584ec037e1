"""Device optimizer iteration: CUDA-graph replay equals eager execution, the energy goes
down along the steepest-descent path, and each energy equals the FP64 oracle's lowest
eigenvalue for the states of that iteration."""
import numpy as np
import pytest

import xr_oracle as O
from qodeapplications_gb300 import synthetic as S

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu
CHG = (+1, 0, -1)


def _opt(use_graphs, precision="fp64"):
    from qodeapplications_gb300.iteration import XRStateOptimizer
    sysd = S.make_system(n_frag=2, n_orb=4, n_states=3, charges=CHG, seed=51)
    return sysd, XRStateOptimizer(sysd, precision=precision, step=0.05, lanczos_m=60, warm_m=40,
                                  use_graphs=use_graphs)


def test_graph_equals_eager_and_energy_decreases():
    _, eager = _opt(False)
    _, graphed = _opt(True)
    Es_e = [eager.iterate() for _ in range(5)]
    Es_g = [graphed.iterate() for _ in range(5)]
    np.testing.assert_allclose(Es_g, Es_e, rtol=0, atol=1e-10)
    assert all(b < a + 1e-12 for a, b in zip(Es_e, Es_e[1:])), Es_e
    assert Es_e[-1] < Es_e[0] - 1e-6


def test_iteration_energy_matches_oracle_for_current_states():
    sysd, opt = _opt(True)
    for _ in range(3):
        opt.iterate()
    states = [{c: (opt.plan.coeffs[m][c].cpu().numpy(), sysd["states"][m][c][1]) for c in CHG} for m in range(2)]
    E_next = opt.iterate()
    E_ref = O.xr_energy(sysd["h"], sysd["V"], sysd["Ns"], 4, 0, 4, states, CHG)[0]
    assert abs(E_next - E_ref) < 1e-10
    # states stay orthonormal after the Loewdin step
    for m in range(2):
        for c in CHG:
            z = opt.plan.coeffs[m][c]
            assert float((z @ z.t() - torch.eye(z.shape[0], device="cuda", dtype=torch.float64)).abs().max()) < 1e-12
