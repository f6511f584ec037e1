"""Operator-pair symmetries of the density kernels (xrh_antisym_rows, densities.canonical_couplings).

The density build and its adjoint run over the canonical index tuples of an operator pair --
o_u < o_u+1 for two anticommuting operators of one kind (aa, cc, caa, cca), p <= q for the
Hermitian ca pair between the same states -- and one row pass fills (forward) or folds
(adjoint) the other tuples.  Checked here: every mode of the row pass against PyTorch FP64
index arithmetic (exact), and the builder's densities with canonical lists against the full
lists (FP64 1e-13, FP32 products 1e-6 relative)."""
import numpy as np
import pytest

from qodeapplications_gb300 import synthetic as S

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _swap(idx, N, L, u):
    w_lo = N ** (L - 2 - u)
    w_hi = w_lo * N
    a, b = (idx // w_hi) % N, (idx // w_lo) % N
    return idx + (b - a) * w_hi + (a - b) * w_lo, a, b


@pytest.mark.parametrize("N,L,u,n", [(5, 3, 1, 3), (6, 2, 0, 4), (4, 3, 0, 2)])
def test_row_pass_modes_match_index_arithmetic(N, L, u, n):
    from qodeapplications_gb300 import _lib
    K, R = N ** L, n * n
    g = torch.Generator().manual_seed(11)
    base = torch.randn(K, R, generator=g, dtype=torch.float64)
    idx = torch.arange(K)
    partner, a, b = _swap(idx, N, L, u)
    for mode in (0, 1, 2, 3):
        rows = base.clone().cuda()
        _lib.AntisymRows([(rows, R, N, L, u, mode)], rows.device).run()
        ref = base.clone()
        tgt = (a > b) if mode in (0, 2) else (a < b)
        src = base[partner]
        if mode >= 2:
            src = src.view(K, n, n).transpose(1, 2).reshape(K, R)
        if mode == 0:
            ref[tgt] = -src[tgt]
        elif mode == 1:
            ref[tgt] -= src[tgt]
        elif mode == 2:
            ref[tgt] = src[tgt]
        else:
            ref[tgt] += src[tgt]
        assert torch.equal(rows.cpu(), ref), mode


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_canonical_densities_match_full_lists(precision):
    from qodeapplications_gb300.densities import DensityBuilder, FragmentSpace
    chg = (+1, 0, -1)
    sysd = S.make_system(n_frag=2, n_orb=5, n_states=20, charges=chg, seed=5)
    space = FragmentSpace({c: sysd["states"][0][c][1] for c in chg}, 5, 0, 4)
    ns = {c: 20 for c in chg}
    coeffs = {c: torch.as_tensor(sysd["states"][0][c][0], device="cuda") for c in chg}
    full = DensityBuilder(space, ns, precision=precision, antisym=False).build(coeffs)
    full = {op: {k: t.clone() for k, t in blocks.items()} for op, blocks in full.items()}
    canon_b = DensityBuilder(space, ns, precision=precision, antisym=True)
    assert canon_b._canon, "no block took the canonical lists"
    canon = canon_b.build(coeffs)
    tol = 1e-13 if precision == "fp64" else 1e-6
    for op, blocks in full.items():
        for k, t in blocks.items():
            err = float((canon[op][k] - t).abs().max()) / max(float(t.abs().max()), 1e-300)
            assert err <= tol, (op, k, err)
