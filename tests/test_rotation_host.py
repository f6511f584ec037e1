"""Host-side pieces of the differentiable path (no GPU): the torch orbital rotation matches
the NumPy one the oracle finite differences use, and its autograd derivative at kappa = 0 is
the commutator formula."""
import numpy as np
import pytest

from qodeapplications_gb300 import synthetic as S

torch = pytest.importorskip("torch")


def test_torch_rotation_matches_numpy():
    from qodeapplications_gb300.autograd import rotate_integrals
    sysd = S.make_system(n_frag=2, n_orb=3, n_states=2, seed=9)
    rng = np.random.default_rng(2)
    k = rng.normal(0.0, 0.05, size=(6, 6))
    k = k - k.T
    h2, V2 = rotate_integrals(torch.as_tensor(sysd["h"]), torch.as_tensor(sysd["V"]), torch.as_tensor(k), [3, 3])
    h_ref, V_ref = S.rotate_integrals(sysd["h"], sysd["V"], k, [3, 3])
    assert np.abs(h2.numpy() - h_ref).max() < 1e-13
    assert np.abs(V2.numpy() - V_ref).max() < 1e-13


def test_rotation_keeps_antisymmetry():
    from qodeapplications_gb300.autograd import rotate_integrals
    sysd = S.make_system(n_frag=2, n_orb=3, n_states=2, seed=10)
    k = np.triu(np.random.default_rng(1).normal(0.0, 0.1, size=(6, 6)), 1)
    h2, V2 = rotate_integrals(torch.as_tensor(sysd["h"]), torch.as_tensor(sysd["V"]), torch.as_tensor(k - k.T), [3, 3])
    V2 = V2.numpy()
    assert np.abs(V2 + V2.transpose(1, 0, 2, 3)).max() < 1e-13
    assert np.abs(V2 + V2.transpose(0, 1, 3, 2)).max() < 1e-13
    assert np.abs(h2.numpy() - h2.numpy().T).max() < 1e-13
