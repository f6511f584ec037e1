"""The allocation-free density entry point, xrh_density_build_noalloc.

Some callers cannot allocate device memory (code running inside another application's CUDA
context whose allocator owns the device, or a host program with no device allocator of its
own).  They call this variant, which keeps its scratch in a fixed array inside the library,
instead of xrh_density_accumulate + xrh_transpose with a caller-provided buffer.  This test
calls it through the C ABI twice in a row, with different coefficients, and checks both
results against the allocating path at the FP64 parity tolerance of the other density
tests (1e-13); it also checks that a size beyond the documented limit is rejected.
The file is named to be collected last."""
import ctypes

import numpy as np
import pytest

from qodeapplications_gb300 import synthetic as S

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def test_noalloc_density_matches_allocating_path():
    from qodeapplications_gb300 import _lib
    from qodeapplications_gb300.densities import DensityBuilder, FragmentSpace
    chg = (+1, 0, -1)
    L = _lib.lib()
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
            status = L.xrh_density_build_noalloc(
                _lib.FP64, cp.K, _lib.ptr(cp.idx_ptr), _lib.ptr(cp.P), _lib.ptr(cp.Q), _lib.ptr(cp.sign),
                _lib.ptr(b.zbT[bc]), 4, _lib.ptr(b.zT[kc]), 4, _lib.ptr(out), _lib.stream_ptr())
            assert status == 0, L.xrh_status_string(status)
            torch.cuda.synchronize()
            np.testing.assert_allclose(out.cpu().numpy(), rho[op][(bc, kc)].cpu().numpy(), rtol=0, atol=1e-13)
    # beyond the 2^20-double scratch: rejected before any device work
    assert L.xrh_density_build_noalloc(_lib.FP64, 1 << 20, _lib.ptr(cp.idx_ptr), None, None, None,
                                       _lib.ptr(b.zbT[0]), 2, _lib.ptr(b.zT[0]), 1, _lib.ptr(out),
                                       ctypes.c_void_p(0)) == _lib.XRH_ERR_CAPACITY
