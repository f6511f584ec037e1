"""Failure paths, exercised without faulting the GPU.

* A bounded device wait that runs out: the cooperative Lanczos loop with a grid-barrier poll
  limit of 0 (xrh_lanczos_coop_bounded) -- the first CTA to reach a barrier finds the others
  absent and gives up, writes XRH_ERR_TIMEOUT to the status word, and every CTA returns.  The
  context stays usable: the next, unbounded launch on the same buffers runs to the end (an
  orthonormal Krylov basis satisfying the Lanczos relation).  (This kernel has no asynchronous copies in flight when it waits.)
* Inputs the host rejects before any launch: a missing density block (RuntimeError), a
  density holding NaN (ValueError), sizes beyond a documented limit (XRH_ERR_CAPACITY).
"""
import numpy as np
import pytest

import xr_oracle as O
from qodeapplications_gb300 import synthetic as S

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def test_lanczos_barrier_timeout_returns_status_and_context_survives():
    from qodeapplications_gb300 import _lib
    L = _lib.lib()
    n, m = 300, 20
    rng = np.random.default_rng(1)
    A = rng.standard_normal((n, n))
    H = torch.as_tensor(A + A.T, device="cuda")
    v0 = torch.as_tensor(rng.standard_normal(n), device="cuda")
    v0 /= v0.norm()
    V = torch.zeros((m + 1, n), dtype=torch.float64, device="cuda")
    ab = torch.zeros(2 * m, dtype=torch.float64, device="cuda")
    work = torch.zeros(int(L.xrh_lanczos_coop_work(m)), dtype=torch.float64, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    s = _lib.stream_ptr()
    st = L.xrh_lanczos_coop_bounded(n, m, _lib.ptr(H), n, _lib.ptr(v0), _lib.ptr(V), _lib.ptr(ab),
                                    _lib.ptr(ab[m:]), _lib.ptr(work), work.numel(), _lib.ptr(status), 0, s)
    assert st == _lib.XRH_OK
    torch.cuda.synchronize()
    assert int(status.item()) == _lib.XRH_ERR_TIMEOUT
    # the same buffers, the default bound: a normal run
    status.zero_()
    _lib.call("xrh_lanczos_coop", n, m, _lib.ptr(H), n, _lib.ptr(v0), _lib.ptr(V), _lib.ptr(ab), _lib.ptr(ab[m:]),
              _lib.ptr(work), work.numel(), _lib.ptr(status), s)
    torch.cuda.synchronize()
    assert int(status.item()) == _lib.XRH_OK
    # the Lanczos relation H v_j = beta_{j-1} v_{j-1} + alpha_j v_j + beta_j v_{j+1} and an
    # orthonormal basis: the loop ran to the end with consistent data
    a, b = ab[:m].cpu().numpy(), ab[m:].cpu().numpy()
    Vh, Hh = V.cpu().numpy(), (A + A.T)
    for j in range(m):
        r = Hh @ Vh[j] - a[j] * Vh[j] - b[j] * Vh[j + 1] - (b[j - 1] * Vh[j - 1] if j else 0.0)
        assert np.abs(r).max() < 1e-10 * np.abs(Hh).max(), j
    np.testing.assert_allclose(Vh @ Vh.T, np.eye(m + 1), rtol=0, atol=1e-10)
    # a negative bound is an argument error, reported before any launch
    assert L.xrh_lanczos_coop_bounded(n, m, _lib.ptr(H), n, _lib.ptr(v0), _lib.ptr(V), _lib.ptr(ab),
                                      _lib.ptr(ab[m:]), _lib.ptr(work), work.numel(), _lib.ptr(status), -1,
                                      s) == _lib.XRH_ERR_ARG


def _dens(seed=21):
    chg = [+1, 0, -1]
    sysd = S.make_system(n_frag=2, n_orb=4, n_states=3, charges=chg, seed=seed)
    oi = O.FragInts(sysd["h"], sysd["V"], sysd["Ns"])
    dens = [O.build_densities({c: O.Sector(*sysd["states"][m][c]) for c in chg}, 4, 0, 4) for m in range(2)]
    return chg, oi, dens


def test_missing_density_block_is_reported():
    from qodeapplications_gb300.get_xr_result import get_xr_H
    chg, oi, dens = _dens()
    bad = dict(dens[0])
    bad["caa"] = {k: v for k, v in bad["caa"].items() if k != (0, -1)}
    with pytest.raises(RuntimeError, match="missing"):
        get_xr_H((oi, oi, None), [bad, dens[1]], 0, [chg, chg])


def test_nan_density_is_rejected():
    from qodeapplications_gb300.get_xr_result import get_xr_H
    chg, oi, dens = _dens()
    bad = dict(dens[1])
    bad["ca"] = dict(bad["ca"])
    arr = bad["ca"][(0, 0)].copy()
    arr[0, 1, 2, 3] = np.nan
    bad["ca"][(0, 0)] = arr
    with pytest.raises(ValueError, match="NaN"):
        get_xr_H((oi, oi, None), [dens[0], bad], 0, [chg, chg])


def test_capacity_limits_are_reported_before_any_launch():
    from qodeapplications_gb300 import _lib
    L = _lib.lib()
    x = torch.zeros((65, 65), dtype=torch.float64, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    assert L.xrh_expm_small(65, _lib.ptr(x), 65, _lib.ptr(x), 65, _lib.stream_ptr()) == _lib.XRH_ERR_CAPACITY
    assert L.xrh_inverse_small(65, _lib.ptr(x), 65, _lib.ptr(x), 65, _lib.ptr(st), _lib.stream_ptr()) == \
        _lib.XRH_ERR_CAPACITY
    assert L.xrh_lanczos_coop_work(0) < 0
