"""The allocation-free density entry point, xrh_density_build_noalloc.

Some callers cannot allocate device memory (code running inside another application's CUDA
context whose allocator owns the device, or a host program with no device allocator of its
own).  They call this variant, which keeps its scratch in a fixed array inside the library,
instead of xrh_density_accumulate + xrh_transpose with a caller-provided buffer.  These tests
call it through the C ABI twice in a row, with different coefficients, in FP64 and in FP32,
and check the results against the allocating path (FP64: 1e-13, the tolerance of the other
FP64 density tests; FP32: the same kernel in both paths, so equal to 1e-12 of the largest
element, and within 2e-6 relative of FP64).  A synthetic coupling list that fills the scratch
exactly (K * n_b * n_k = 2^20 doubles) checks its far end, and one element more is rejected
before any device work.  The file is named to be collected last."""
import ctypes

import numpy as np
import pytest

from qodeapplications_gb300 import synthetic as S

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

CAPACITY = 1 << 20          # doubles in the library's scratch array


def _noalloc(L, _lib, prec, K, idx_ptr, P, Q, sign, zbT, nb, zkT, nk, out, stream=None):
    return L.xrh_density_build_noalloc(prec, K, _lib.ptr(idx_ptr), _lib.ptr(P), _lib.ptr(Q), _lib.ptr(sign),
                                       _lib.ptr(zbT), nb, _lib.ptr(zkT), nk, _lib.ptr(out),
                                       _lib.stream_ptr() if stream is None else stream)


def _allocating(L, _lib, prec, K, idx_ptr, P, Q, sign, zbT, nb, zkT, nk):
    """The allocating path: caller-provided [K, n_b n_k] scratch, then the transpose."""
    tmp = torch.empty((K, nb * nk), dtype=torch.float64, device="cuda")
    out = torch.empty((nb, nk, K), dtype=torch.float64, device="cuda")
    s = _lib.stream_ptr()
    st = L.xrh_density_accumulate(prec, K, _lib.ptr(idx_ptr), _lib.ptr(P), _lib.ptr(Q), _lib.ptr(sign),
                                  _lib.ptr(zbT), nb, _lib.ptr(zkT), nk, _lib.ptr(tmp), s)
    assert st == 0, L.xrh_status_string(st)
    st = L.xrh_transpose(_lib.ptr(tmp), K, nb * nk, _lib.ptr(out), s)
    assert st == 0, L.xrh_status_string(st)
    return out


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_noalloc_density_matches_allocating_path(precision):
    from qodeapplications_gb300 import _lib
    from qodeapplications_gb300.densities import DensityBuilder, FragmentSpace
    chg = (+1, 0, -1)
    L = _lib.lib()
    prec = _lib.PRECISIONS[precision]
    for seed in (41, 42):              # two calls in a row, different states
        sysd = S.make_system(n_frag=1, n_orb=5, n_states=4, charges=chg, seed=seed)
        st = sysd["states"][0]
        space = FragmentSpace({c: st[c][1] for c in chg}, 5, 0, 4)
        b = DensityBuilder(space, {c: 4 for c in chg})
        rho = b.build({c: torch.as_tensor(st[c][0], device="cuda") for c in chg})
        for key in (("caa", 0, -1), ("ca", 0, 0)):
            cp = space.couplings[key]
            op, bc, kc = key
            out = torch.full_like(rho[op][(bc, kc)], float("nan"))
            status = _noalloc(L, _lib, prec, cp.K, cp.idx_ptr, cp.P, cp.Q, cp.sign, b.zbT[bc], 4, b.zT[kc], 4, out)
            assert status == 0, L.xrh_status_string(status)
            torch.cuda.synchronize()
            got = out.cpu().numpy()
            ref64 = rho[op][(bc, kc)].cpu().numpy()
            if precision == "fp64":
                np.testing.assert_allclose(got, ref64, rtol=0, atol=1e-13)
            else:
                ref = _allocating(L, _lib, prec, cp.K, cp.idx_ptr, cp.P, cp.Q, cp.sign, b.zbT[bc], 4, b.zT[kc], 4)
                scale = max(np.abs(ref64).max(), 1e-30)
                np.testing.assert_allclose(got, ref.cpu().numpy().reshape(got.shape), rtol=0, atol=1e-12 * scale)
                np.testing.assert_allclose(got, ref64, rtol=0, atol=2e-6 * scale)
    # beyond the 2^20-double scratch: rejected before any device work
    for p in (_lib.FP64, _lib.FP32):
        assert L.xrh_density_build_noalloc(p, CAPACITY, _lib.ptr(cp.idx_ptr), None, None, None,
                                           _lib.ptr(b.zbT[0]), 2, _lib.ptr(b.zT[0]), 1, _lib.ptr(out),
                                           ctypes.c_void_p(0)) == _lib.XRH_ERR_CAPACITY


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_noalloc_density_fills_the_whole_scratch(precision):
    """A synthetic coupling list with K * n_b * n_k equal to the scratch size, twice in a row
    with different coefficients, against the allocating path."""
    from qodeapplications_gb300 import _lib
    L = _lib.lib()
    prec = _lib.PRECISIONS[precision]
    nb = nk = 16
    K = CAPACITY // (nb * nk)
    n_conf_b, n_conf_k = 700, 900
    rng = np.random.default_rng(7)
    counts = rng.integers(0, 9, size=K)
    idx_ptr = np.zeros(K + 1, dtype=np.int64)
    idx_ptr[1:] = np.cumsum(counts)
    n_c = int(idx_ptr[-1])
    dev = dict(device="cuda")
    P = torch.as_tensor(rng.integers(0, n_conf_b, size=n_c).astype(np.int32), **dev)
    Q = torch.as_tensor(rng.integers(0, n_conf_k, size=n_c).astype(np.int32), **dev)
    sign = torch.as_tensor(rng.choice(np.array([-1, 1], dtype=np.int8), size=n_c), **dev)
    idx = torch.as_tensor(idx_ptr, **dev)
    for call in range(2):
        zbT = torch.as_tensor(rng.standard_normal((n_conf_b, nb)), **dev)
        zkT = torch.as_tensor(rng.standard_normal((n_conf_k, nk)), **dev)
        out = torch.full((nb, nk, K), float("nan"), dtype=torch.float64, **dev)
        status = _noalloc(L, _lib, prec, K, idx, P, Q, sign, zbT, nb, zkT, nk, out)
        assert status == 0, L.xrh_status_string(status)
        ref = _allocating(L, _lib, prec, K, idx, P, Q, sign, zbT, nb, zkT, nk)
        torch.cuda.synchronize()
        scale = float(ref.abs().max())
        tol = 1e-13 if precision == "fp64" else 1e-12
        assert float((out - ref).abs().max()) <= tol * max(scale, 1.0), call
        if precision == "fp64":
            # the far end of the scratch (the last operator index) against a host sum
            k = K - 1
            zb, zk = zbT.cpu().numpy(), zkT.cpu().numpy()
            c0, c1 = int(idx_ptr[k]), int(idx_ptr[k + 1])
            Pn, Qn, sn = P.cpu().numpy(), Q.cpu().numpy(), sign.cpu().numpy()
            host = sum(sn[c] * np.outer(zb[Pn[c]], zk[Qn[c]]) for c in range(c0, c1)) if c1 > c0 else 0.0
            np.testing.assert_allclose(out[:, :, k].cpu().numpy(), host + np.zeros((nb, nk)), rtol=0, atol=1e-12)
    assert L.xrh_density_build_noalloc(prec, K + 1, _lib.ptr(idx), None, None, None, _lib.ptr(zbT), nb,
                                       _lib.ptr(zkT), nk, _lib.ptr(out), ctypes.c_void_p(0)) == _lib.XRH_ERR_CAPACITY
