"""Split-precision tensor-core path (tcgen05): GEMM unit checks and the XR-H build.

Tolerances are those of the arithmetic: 3xBF16 keeps about 16 significant bits per operand
(relative error of a product term ~1e-5), 3xTF32 about 21 bits (~5e-7), both accumulated
in FP32; they are stated per test against an FP64 result."""
import numpy as np
import pytest

import xr_oracle as O
from qodeapplications_gb300 import synthetic as S

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = {"bf16x3": 3e-5, "tf32x3": 2e-6}


def _rel(a, b):
    return float((a - b).abs().max() / b.abs().max())


@pytest.mark.parametrize("prec", ["bf16x3", "tf32x3"])
def test_tc_gemm_store_and_splitk(prec):
    from qodeapplications_gb300.gemm import SplitRegistry, TCGroupedGemm
    g = torch.Generator().manual_seed(3)
    A = torch.randn(300, 200, generator=g, dtype=torch.float64).cuda()
    B = torch.randn(150, 200, generator=g, dtype=torch.float64).cuda()
    A2 = torch.randn(300, 70, generator=g, dtype=torch.float64).cuda()
    B2 = torch.randn(150, 70, generator=g, dtype=torch.float64).cuda()
    reg = SplitRegistry(prec)
    C0 = torch.zeros(300, 150, dtype=torch.float64, device="cuda")
    C1 = torch.zeros(300, 150, dtype=torch.float64, device="cuda")
    tc = TCGroupedGemm(reg)
    tc.add(300, 150, [(A, 200, B, 200, 200, 1.0)], C0, 150, mode=0)
    tc.add(300, 150, [(A, 200, B, 200, 200, 1.0), (A2, 70, B2, 70, 70, -1.0)], C1, 150, mode=1, splitk=3)
    reg.upload()
    tc.finalize()
    reg.split("in")
    tc.run()
    torch.cuda.synchronize()
    tc.check()
    ref0 = A @ B.t()
    ref1 = ref0 - A2 @ B2.t()
    assert _rel(C0, ref0) < TOL[prec], _rel(C0, ref0)
    assert _rel(C1, ref1) < TOL[prec], _rel(C1, ref1)


@pytest.mark.parametrize("prec", ["bf16x3", "tf32x3"])
def test_tc_dimer_H_close_to_oracle(prec):
    from qodeapplications_gb300.densities import FragmentSpace
    from qodeapplications_gb300.hamiltonian import DeviceIntegrals, XRDimerPlan
    chg = (+1, 0, -1)
    sysd = S.make_system(n_frag=2, n_orb=5, n_states=4, charges=chg, seed=21)
    spaces = [FragmentSpace({c: sysd["states"][m][c][1] for c in chg}, 5, 0, 4) for m in range(2)]
    ns = [{c: 4 for c in chg}] * 2
    plan = XRDimerPlan(spaces, ns, [list(chg)] * 2, DeviceIntegrals(h=sysd["h"], V=sysd["V"], Ns=sysd["Ns"]),
                       precision=prec)
    coeffs = [{c: torch.as_tensor(sysd["states"][m][c][0], device="cuda") for c in chg} for m in range(2)]
    H = plan.build(coeffs)
    torch.cuda.synchronize()
    plan.check_status()
    ints = O.FragInts(sysd["h"], sysd["V"], sysd["Ns"])
    dens = [O.build_densities({c: O.Sector(*sysd["states"][m][c]) for c in chg}, 5, 0, 4) for m in range(2)]
    H1, H2 = O.get_xr_H0(ints, dens, [list(chg)] * 2)
    Href = O.full_H(H1, H2)
    err = np.abs(H.cpu().numpy() - Href).max()
    e_gpu = np.linalg.eigvalsh(H.cpu().numpy())[0]
    e_ref = np.linalg.eigvalsh(Href)[0]
    print(f"{prec}: max|dH| = {err:.3e}, |dE0| = {abs(e_gpu - e_ref):.3e}")
    assert err < {"bf16x3": 1e-3, "tf32x3": 2e-5}[prec]
    assert abs(e_gpu - e_ref) < 1e-6 if prec == "tf32x3" else abs(e_gpu - e_ref) < 1e-4


@pytest.mark.parametrize("prec", ["bf16x3", "tf32x3"])
def test_tc_gemm_every_tile_policy(prec):
    """Every (N-tile cap, split-K divisor) the autotuner may pick gives the same result."""
    from qodeapplications_gb300.gemm import SplitRegistry, TCGroupedGemm
    g = torch.Generator().manual_seed(4)
    A = torch.randn(260, 512, generator=g, dtype=torch.float64).cuda()
    B = torch.randn(200, 512, generator=g, dtype=torch.float64).cuda()
    B2 = torch.randn(40, 512, generator=g, dtype=torch.float64).cuda()
    reg = SplitRegistry(prec)
    C = torch.zeros(260, 200, dtype=torch.float64, device="cuda")
    C2 = torch.zeros(260, 40, dtype=torch.float64, device="cuda")
    tc = TCGroupedGemm(reg)
    tc.add(260, 200, [(A, 512, B, 512, 512, 1.0)], C, 200, mode=1)
    tc.add(260, 40, [(A, 512, B2, 512, 512, -1.0)], C2, 40, mode=1)
    reg.upload()
    reg.split("in")
    ref, ref2 = A @ B.t(), -(A @ B2.t())
    for cap in TCGroupedGemm.BN_CAPS:
        for div in TCGroupedGemm.SK_DIVS:
            tc.finalize((cap, div))
            reg.split("in")
            C.zero_()
            C2.zero_()
            tc.run()
            torch.cuda.synchronize()
            tc.check()
            assert _rel(C, ref) < TOL[prec], (cap, div, _rel(C, ref))
            assert _rel(C2, ref2) < TOL[prec], (cap, div, _rel(C2, ref2))
    tc.autotune()
    assert tc.tuning is not None and tc.policy in [p for p, _ in tc.tuning]


@pytest.mark.parametrize("prec", ["bf16x3", "tf32x3"])
def test_tc_gemm_many_short_segments_wide_output(prec):
    """The shape of the three-fragment H x v's stage B in small: M < N (concurrent tiles walk
    the M tiles of one N tile), 40 K-concatenated segments of K = 28 (one padded chunk each);
    stored and split-K accumulated."""
    from qodeapplications_gb300.gemm import SplitRegistry, TCGroupedGemm
    g = torch.Generator().manual_seed(5)
    M, N, K, S_ = 280, 1000, 28, 40
    As = [torch.randn(M, K, generator=g, dtype=torch.float64).cuda() for _ in range(S_)]
    Bs = [torch.randn(N, K, generator=g, dtype=torch.float64).cuda() for _ in range(S_)]
    reg = SplitRegistry(prec)
    C0 = torch.zeros(M, N, dtype=torch.float64, device="cuda")
    C1 = torch.zeros(M, N, dtype=torch.float64, device="cuda")
    tc = TCGroupedGemm(reg)
    segs = [(A, K, B, K, K, 1.0 if i % 3 else -1.0) for i, (A, B) in enumerate(zip(As, Bs))]
    tc.add(M, N, segs, C0, N, mode=0)
    tc.add(M, N, segs, C1, N, mode=1, splitk=4)
    reg.upload()
    tc.finalize()
    reg.split("in")
    tc.run()
    torch.cuda.synchronize()
    tc.check()
    ref = sum(s[5] * (s[0] @ s[2].t()) for s in segs)
    assert _rel(C0, ref) < TOL[prec], _rel(C0, ref)
    assert _rel(C1, ref) < TOL[prec], _rel(C1, ref)


def test_tc_gemm_precontraction_shape():
    """One 3xTF32 launch at the shape of the 2 x 14 / 60-state precontractions (M = 3600 state
    pairs, N = 784, K = 784) against FP64, and its CUDA-event time (printed): the launch the
    tensor-pipe counters of the profile summary were taken on."""
    from qodeapplications_gb300.gemm import SplitRegistry, TCGroupedGemm
    g = torch.Generator().manual_seed(6)
    M, N, K = 3600, 784, 784
    A = torch.randn(M, K, generator=g, dtype=torch.float64).cuda()
    B = torch.randn(N, K, generator=g, dtype=torch.float64).cuda()
    C = torch.zeros(M, N, dtype=torch.float64, device="cuda")
    reg = SplitRegistry("tf32x3")
    tc = TCGroupedGemm(reg)
    tc.add(M, N, [(A, K, B, K, K, 1.0)], C, N, mode=0)
    reg.upload()
    tc.finalize()
    reg.split("in")
    tc.run()
    torch.cuda.synchronize()
    tc.check()
    assert _rel(C, A @ B.t()) < TOL["tf32x3"]
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(10):
        tc.run()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / 10
    print(f"tf32x3 GEMM {M}x{N}x{K}: {ms:.3f} ms, {2.0 * M * N * K / ms / 1e9:.1f} TFLOP/s algorithmic")


def test_tc_gemm_stage_b_shape():
    """One 3xTF32 launch of the three-fragment H x v's stage B at 3 x 14 orbitals / 40 states
    (M = 40 x 28, N = 40 x 40, 40 K-concatenated segments of K = 28) against FP64, and its
    CUDA-event time (printed): the launch the stage-B profile summary was taken on."""
    from qodeapplications_gb300.gemm import SplitRegistry, TCGroupedGemm
    g = torch.Generator().manual_seed(7)
    M, N, K, S_ = 1120, 1600, 28, 40
    A = torch.randn(S_, M, K, generator=g, dtype=torch.float64).cuda()
    B = torch.randn(S_, N, K, generator=g, dtype=torch.float64).cuda()
    C = torch.zeros(M, N, dtype=torch.float64, device="cuda")
    reg = SplitRegistry("tf32x3")
    tc = TCGroupedGemm(reg)
    tc.add(M, N, [(A[i], K, B[i], K, K, 1.0) for i in range(S_)], C, N, mode=0)
    reg.upload()
    tc.finalize()
    reg.split("in")
    tc.run()
    torch.cuda.synchronize()
    tc.check()
    assert _rel(C, torch.einsum("smk,snk->mn", A, B)) < TOL["tf32x3"]
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(10):
        tc.run()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / 10
    print(f"tf32x3 stage-B GEMM {M}x{N}x({S_}x{K}): {ms:.3f} ms, {2.0 * M * N * K * S_ / ms / 1e9:.1f} TFLOP/s algorithmic")
