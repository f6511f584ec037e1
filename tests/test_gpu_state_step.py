"""The grouped state update (StateStepper) and the small-output A B^T kernel against plain
PyTorch FP64.

The reference step per block (StateSpaceOptimizer/state_solver.py:207-453, in NumPy):
t = g - 1/2 (g z^T + z g^T) z, z' = z - eps t, z <- (z' z'^T)^-1/2 z'.  All of it is FP64
on the GPU, so the tolerance is relative 1e-12 (summation order only).  xrh_abt_small in
FP64 is held to 1e-12 relative, in FP32 to 2e-6 relative to the sum of |terms| (FP32
rounding of the inputs and of 32-term partial sums)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _torch_step(z, g, eps, iters=6):
    t = g - 0.5 * (g @ z.t() + z @ g.t()) @ z
    zn = z - eps * t
    S = zn @ zn.t()
    n = S.shape[0]
    I = torch.eye(n, dtype=S.dtype, device=S.device)
    Y, Z = S.clone(), I.clone()
    for _ in range(iters):
        T = 0.5 * (3.0 * I - Z @ Y)
        Y = Y @ T
        Z = T @ Z
    return Z @ zn, float((t * t).sum())


def _orthonormal_rows(n, K, gen):
    a = torch.randn(K, n, dtype=torch.float64, generator=gen)
    q, _ = torch.linalg.qr(a)
    return q.t().contiguous()


@pytest.mark.parametrize("shapes", [[(10, 1000), (10, 257), (3, 1), (10, 15876)],
                                    [(40, 3001), (12, 256), (1, 77)],
                                    [(64, 600)]])
@pytest.mark.parametrize("with_f32", [False, True])
def test_state_stepper_matches_torch(shapes, with_f32):
    from qodeapplications_gb300.iteration import StateStepper
    gen = torch.Generator().manual_seed(7 + len(shapes))
    eps = 0.02
    zs, gs, ref, sq_ref = [], [], [], 0.0
    for n, K in shapes:
        if n > K:
            continue
        z = _orthonormal_rows(n, K, gen)
        gT = torch.randn(K, n, dtype=torch.float64, generator=gen) * 0.3
        gT32 = (torch.randn(K, n, dtype=torch.float64, generator=gen) * 1e-3).to(torch.float32) if with_f32 else None
        g = (gT + (gT32.double() if gT32 is not None else 0.0)).t()
        zr, sq = _torch_step(z, g, eps)
        ref.append(zr)
        sq_ref += sq
        zs.append(z.cuda())
        gs.append((gT.cuda(), gT32.cuda() if gT32 is not None else None))
    st = StateStepper(zs, gs, eps)
    sq = float(st.launch())
    torch.cuda.synchronize()
    for z, zr in zip(zs, ref):
        err = (z.cpu() - zr).abs().max().item()
        assert err <= 1e-12 * max(1.0, zr.abs().max().item()), err
        # rows stay orthonormal
        I = torch.eye(z.shape[0], dtype=torch.float64)
        assert (z.cpu() @ z.cpu().t() - I).abs().max().item() < 1e-12
    assert abs(sq - sq_ref) <= 1e-12 * max(1.0, sq_ref)


def test_state_stepper_repeat_is_stable():
    """Ten steps in a row: the zeroed accumulators are reset every launch."""
    from qodeapplications_gb300.iteration import StateStepper
    gen = torch.Generator().manual_seed(3)
    z = _orthonormal_rows(6, 500, gen)
    gT = torch.randn(500, 6, dtype=torch.float64, generator=gen) * 0.1
    zc = z.cuda()
    st = StateStepper([zc], [(gT.cuda(), None)], 0.05)
    zr = z
    for _ in range(10):
        st.launch()
        zr, _ = _torch_step(zr, gT.t(), 0.05)
    torch.cuda.synchronize()
    assert (zc.cpu() - zr).abs().max().item() < 1e-11


@pytest.mark.parametrize("m,n,K", [(36, 36, 46656), (5, 64, 1), (64, 7, 257), (1, 1, 100000)])
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_abt_small(m, n, K, prec):
    from qodeapplications_gb300 import _lib
    from qodeapplications_gb300._lib import call, ptr, stream_ptr
    gen = torch.Generator().manual_seed(m * 1000 + n)
    A = torch.randn(m, K, dtype=torch.float64, generator=gen)
    B = torch.randn(n, K, dtype=torch.float64, generator=gen)
    C0 = torch.randn(m, n, dtype=torch.float64, generator=gen)
    dt = torch.float64 if prec == "fp64" else torch.float32
    Ad, Bd = A.to(dt).cuda(), B.to(dt).cuda()
    C = C0.clone().cuda()
    call("xrh_abt_small", _lib.PRECISIONS[prec], m, n, K, ptr(Ad), K, ptr(Bd), K, 0.75, ptr(C), stream_ptr())
    torch.cuda.synchronize()
    ref = C0 + 0.75 * (A @ B.t())
    scale = 0.75 * (A.abs() @ B.abs().t()) + C0.abs()
    tol = 1e-12 if prec == "fp64" else 2e-6
    assert ((C.cpu() - ref).abs() / scale).max().item() < tol
