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


@pytest.mark.parametrize("n", [1, 2047, 2048, 100_003])
def test_split_gemv_and_normalize(n):
    """Column-split products for few rows over long vectors against FP64 PyTorch (1e-13)."""
    from qodeapplications_gb300 import _lib
    L = _lib.lib()
    g = torch.Generator().manual_seed(n)
    rows = 31
    A = torch.randn(rows, n, generator=g, dtype=torch.float64).cuda()
    x = torch.randn(n, generator=g, dtype=torch.float64).cuda()
    y = torch.randn(rows, generator=g, dtype=torch.float64).cuda()
    y0 = y.clone()
    work = torch.zeros(int(L.xrh_gemv_split_work(rows, n)), dtype=torch.float64, device="cuda")
    _lib.call("xrh_gemv_rows_split", rows, n, _lib.ptr(A), n, _lib.ptr(x), 2.0, 0.5, _lib.ptr(y), _lib.ptr(work),
              work.numel(), _lib.stream_ptr())
    ref = 2.0 * (A @ x) + 0.5 * y0
    torch.cuda.synchronize()
    assert float((y - ref).abs().max()) <= 1e-13 * float(ref.abs().max())
    v = torch.empty_like(x)
    beta = torch.zeros(1, dtype=torch.float64, device="cuda")
    _lib.call("xrh_lanczos_normalize_split", n, _lib.ptr(x), _lib.ptr(v), _lib.ptr(beta), _lib.ptr(work),
              work.numel(), _lib.stream_ptr())
    torch.cuda.synchronize()
    nrm = float(x.norm())
    assert abs(float(beta) - nrm) <= 1e-13 * nrm
    assert float((v - x / nrm).abs().max()) <= 1e-15 * float((x / nrm).abs().max()) * 10
    assert L.xrh_gemv_rows_split(rows, n, _lib.ptr(A), n, _lib.ptr(x), 1.0, 0.0, _lib.ptr(y), _lib.ptr(work),
                                 work.numel() - 1, None) == _lib.XRH_ERR_CAPACITY


def test_krylov_operator_known_spectrum():
    """The matrix-free loop (split products) on an operator with a known spectrum:
    A = Q diag(d) Q with the Householder reflection Q = 1 - 2 u u^T, n = 100 003."""
    from qodeapplications_gb300.eigen import Lanczos
    n = 100_003
    g = torch.Generator().manual_seed(2)
    d = torch.linspace(-3.0, 5.0, n, dtype=torch.float64)
    d[0] = -4.0
    u = torch.randn(n, generator=g, dtype=torch.float64)
    u = (u / u.norm()).cuda()
    d = d.cuda()

    def apply(x, y):
        t = x - 2.0 * u * torch.dot(u, x)
        t = d * t
        y.copy_(t - 2.0 * u * torch.dot(u, t))

    lz = Lanczos(n, m=60, mode="steps")
    lz.krylov_operator(apply)
    lz.stage_to_host()
    torch.cuda.synchronize()
    w, resid = lz.solve(1)
    assert abs(w[0] + 4.0) <= 1e-10 * 4.0 + resid and resid < 1e-6
