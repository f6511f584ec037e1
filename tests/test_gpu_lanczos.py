"""FP64 Lanczos modes (cooperative multi-CTA loop, one-CTA loop, per-step launches) against
dense torch.linalg.eigh on random symmetric matrices with a separated lowest eigenvalue.

All three are FP64 with the same recurrence (two classical Gram-Schmidt passes); they differ
only in summation order, so their tridiagonal coefficients agree to 1e-11 relative and the
lowest Ritz value matches eigh to 1e-10 relative once converged."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _matrix(n, seed):
    g = torch.Generator().manual_seed(seed)
    Q, _ = torch.linalg.qr(torch.randn(n, n, dtype=torch.float64, generator=g))
    w = torch.linspace(-1.0, 1.0, n, dtype=torch.float64)
    w[0] = -3.0                                   # a gap, so few steps converge
    A = (Q * w) @ Q.t()
    return 0.5 * (A + A.t()), float(w[0])


@pytest.mark.parametrize("n,m", [(300, 24), (2, 2), (1, 1), (1000, 60), (5003, 40)])
@pytest.mark.parametrize("mode", ["cluster", "coop", "small", "steps"])
def test_lanczos_modes(n, m, mode):
    from qodeapplications_gb300 import _lib
    from qodeapplications_gb300.eigen import Lanczos
    if mode == "cluster" and not _lib.lib().xrh_lanczos_cluster_fits(n, m, 0):
        pytest.skip("sector larger than the cluster loop takes")
    A, w0 = _matrix(n, n + m)
    Ad = A.cuda()
    lz = Lanczos(n, m=m, mode=mode)
    lz.krylov(Ad)
    lz.stage_to_host()
    torch.cuda.synchronize()
    w, resid = lz.solve(1)
    assert abs(w[0] - w0) <= 1e-10 * abs(w0) + resid, (w[0], w0, resid)
    if n >= 300:
        assert resid < 1e-8
        v = lz.ground_vector()
        r = Ad @ v - w[0] * v
        assert r.norm().item() < 1e-7


@pytest.mark.parametrize("n,m", [(300, 24), (4099, 30), (1000, 48)])
def test_lanczos_coop_matches_steps(n, m):
    from qodeapplications_gb300 import _lib
    from qodeapplications_gb300.eigen import Lanczos
    A, _ = _matrix(n, 5)
    Ad = A.cuda()
    out = {}
    modes = ["coop", "steps"] + (["cluster"] if _lib.lib().xrh_lanczos_cluster_fits(n, m, 0) else [])
    for mode in modes:
        lz = Lanczos(n, m=m, mode=mode)
        lz.krylov(Ad)
        lz.stage_to_host()
        torch.cuda.synchronize()
        out[mode] = lz._host[:2 * m].numpy().copy()
    b = out["steps"]
    for mode in modes[:1] + modes[2:]:
        assert np.abs(out[mode] - b).max() <= 1e-11 * np.abs(b).max(), mode


@pytest.mark.parametrize("mode", ["coop", "cluster"])
def test_lanczos_in_graph(mode):
    """The cooperative and the cluster launches are captured and replayed in a CUDA graph."""
    from qodeapplications_gb300.eigen import Lanczos
    A, w0 = _matrix(300, 9)
    Ad = A.cuda()
    lz = Lanczos(300, m=24, mode=mode)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        lz.krylov(Ad)
        lz.stage_to_host()
    torch.cuda.current_stream().wait_stream(s)
    torch.cuda.synchronize()
    lz.solve(1)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        lz.krylov(Ad)
        lz.stage_to_host()
    lz._host.zero_()
    g.replay()
    torch.cuda.synchronize()
    w, resid = lz.solve(1)
    assert abs(w[0] - w0) <= 1e-10 * abs(w0) + resid


@pytest.mark.parametrize("ctas", [1, 2, 4, 8])
def test_lanczos_cluster_sizes_agree(ctas):
    """The cluster loop with at most 1, 2, 4 or 8 CTAs gives the per-step launches' result."""
    from qodeapplications_gb300.eigen import Lanczos
    A, _ = _matrix(300, 11)
    Ad = A.cuda()
    out = {}
    for mode, kw in (("steps", {}), ("cluster", {"cluster_ctas": ctas})):
        lz = Lanczos(300, m=24, mode=mode, **kw)
        lz.krylov(Ad)
        lz.stage_to_host()
        torch.cuda.synchronize()
        out[mode] = lz._host[:48].numpy().copy()
    assert np.abs(out["cluster"] - out["steps"]).max() <= 1e-11 * np.abs(out["steps"]).max()
