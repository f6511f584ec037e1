"""One optimizer iteration on the device: densities -> XR-H -> lowest eigenpair -> gradients.

The per-iteration unit of the reference's state optimisation
(StateSpaceOptimizer/state_solver.py:207-453 calls state_gradients, which rebuilds densities
and H with bra_det/ket_det densities, state_gradients.py:144-185) is done here as

  1. densities of both fragments from the current states, the XR-H build (FP64 or split
     precision), all inside one planned launch sequence;
  2. FP64 Lanczos on the total-charge sector that holds the ground state, warm-started from
     the previous eigenvector (the first iteration scans every sector);
  3. the reverse pass (XRDimerAdjoint): dE/dz of both fragments, projected on the tangent
     space of the orthonormal states, and dE/dkappa of the orbital rotations;
  4. a steepest-descent step on the states followed by Loewdin orthonormalisation
     (z <- (z z^T)^-1/2 z, the inverse square root by Newton-Schulz iterations, FP64), for
     all (fragment, charge) blocks at once in five grouped launches (StateStepper).

Steps 1-2 and 3-4 are each replayed as a CUDA graph; between them the host solves the
m x m tridiagonal Lanczos matrix (one small device-to-host copy).
"""
import numpy as np
import torch

from . import _lib
from ._lib import call, ptr, stream_ptr
from .densities import FragmentSpace
from .eigen import Lanczos
from .gradients import XRDimerAdjoint
from .hamiltonian import DeviceIntegrals, XRDimerPlan
from .synthetic import spin_orbital_spatial_index


NS_ITERS = 6


class NewtonSchulzGrouped:
    """M_i = S_i^-1/2 for every state block i (n <= 64) by coupled Newton-Schulz iterations
    (Y_0 = S, Z_0 = I; T = (3 I - Z Y) / 2, Y <- Y T, Z <- T Z; Z -> S^-1/2) in FP64, two
    xrh_small_mm_grouped launches per iteration over all blocks.  The task tables are built
    once over persistent buffers, so run() can be captured in a CUDA graph."""

    def __init__(self, S_views, M_views, iters, device):
        f64 = dict(dtype=torch.float64, device=device)
        self.keep = []
        per = []
        for S, M in zip(S_views, M_views):
            n = S.shape[0]
            if n > 64:
                raise ValueError("Newton-Schulz blocks are limited to 64 states")
            b = dict(n=n, S=S, M=M, Y=[torch.empty((n, n), **f64) for _ in range(2)],
                     Z=[torch.empty((n, n), **f64) for _ in range(2)], T=torch.empty((n, n), **f64),
                     I=torch.eye(n, **f64))
            self.keep.append(b)
            per.append(b)
        self.launches = []
        for it in range(iters):
            first, last = it == 0, it == iters - 1
            a_tasks, b_tasks = [], []
            for b in per:
                Yin = b["S"] if first else b["Y"][(it - 1) % 2]
                Zin = b["I"] if first else b["Z"][(it - 1) % 2]
                Zout = b["M"] if last else b["Z"][it % 2]
                a_tasks.append((Zin, Yin, b["T"], b["n"], -0.5, 1.5))
                if not last:
                    b_tasks.append((Yin, b["T"], b["Y"][it % 2], b["n"], 1.0, 0.0))
                b_tasks.append((b["T"], Zin, Zout, b["n"], 1.0, 0.0))
            self.launches.append(self._table(a_tasks, device))
            self.launches.append(self._table(b_tasks, device))

    @staticmethod
    def _table(tasks, device):
        tab = np.zeros(len(tasks), dtype=_lib.SMALL_MM_TASK_DTYPE)
        cta = 0
        for i, (A, B, C, n, alpha, beta) in enumerate(tasks):
            e = tab[i]
            e["A"], e["B"], e["C"], e["n"], e["alpha"], e["beta"], e["cta_begin"] = (
                A.data_ptr(), B.data_ptr(), C.data_ptr(), n, alpha, beta, cta)
            cta += (n + 3) // 4
        return torch.from_numpy(tab.view(np.uint8).copy()).to(device), len(tab), cta

    def run(self):
        s = stream_ptr()
        for tab, n_t, ctas in self.launches:
            call("xrh_small_mm_grouped", ptr(tab), n_t, ctas, s)


class StateStepper:
    """The state update z <- (z' z'^T)^-1/2 z', z' = z - step * (tangent part of dE/dz), over
    every (fragment, charge) block in grouped FP64 launches: G = g z^T, the tangent step with
    its squared norm, S = z' z'^T, M = S^-1/2 (Newton-Schulz; one CTA per block for n <= 32,
    NewtonSchulzGrouped above), z = M z'.  coeffs[i] is the n x K state block (updated in
    place); grads[i] = (gT, gT32) with dE/dz = (gT + gT32)^T, gT32 None or FP32, both K x n.
    All buffers are persistent, so launch() may be captured in a CUDA graph."""

    def __init__(self, coeffs, grads, step):
        self.coeffs = coeffs
        self.step = float(step)
        dev = coeffs[0].device
        nb = len(coeffs)
        ns = [int(z.shape[0]) for z in coeffs]
        for z, (gT, gT32) in zip(coeffs, grads):
            n, K = z.shape
            if z.dtype != torch.float64 or not z.is_contiguous() or n > 64:
                raise ValueError("state blocks must be contiguous FP64 with at most 64 states")
            if gT.shape != (K, n) or gT.dtype != torch.float64 or not gT.is_contiguous():
                raise ValueError("gradient block must be a contiguous FP64 (n_conf x n) array")
            if gT32 is not None and (gT32.shape != (K, n) or gT32.dtype != torch.float32 or not gT32.is_contiguous()):
                raise ValueError("FP32 gradient part must be a contiguous (n_conf x n) array")
        self.zn = [torch.empty_like(z) for z in coeffs]
        sq = [n * n for n in ns]
        # G and S of every block and the squared norm are zeroed together before each step
        self.zeroed = torch.zeros(2 * sum(sq) + 1, dtype=torch.float64, device=dev)
        self.M = torch.zeros(sum(sq), dtype=torch.float64, device=dev)
        self.sq = self.zeroed[-1:]
        tasks = np.zeros(nb, dtype=_lib.STATE_TASK_DTYPE)
        off, cta = 0, 0
        self.S_views, self.M_views = [], []
        for i, (z, (gT, gT32)) in enumerate(zip(coeffs, grads)):
            n, K = z.shape
            G = self.zeroed[off:off + n * n]
            S = self.zeroed[sum(sq) + off:sum(sq) + off + n * n]
            M = self.M[off:off + n * n]
            self.S_views.append(S.view(n, n))
            self.M_views.append(M.view(n, n))
            t = tasks[i]
            t["gT"], t["gT32"] = gT.data_ptr(), (gT32.data_ptr() if gT32 is not None else 0)
            t["z"], t["zn"] = z.data_ptr(), self.zn[i].data_ptr()
            t["G"], t["S"], t["M"] = G.data_ptr(), S.data_ptr(), M.data_ptr()
            t["K"], t["n"], t["cta_begin"] = K, n, cta
            cta += int(_lib.lib().xrh_state_ctas(K))
            off += n * n
        self.total_ctas = cta
        self.n_tasks = nb
        self.tasks = torch.from_numpy(tasks.view(np.uint8).copy()).to(dev)
        self.small_ns = max(ns) <= 32
        self.ns_grouped = None if self.small_ns else NewtonSchulzGrouped(self.S_views, self.M_views, NS_ITERS, dev)

    def launch(self):
        """One step on the current stream; returns the squared tangent-gradient norm (device)."""
        s = stream_ptr()
        tp = ptr(self.tasks)
        _lib.zero_(self.zeroed)
        call("xrh_gram_grouped", tp, self.n_tasks, self.total_ctas, 0, s)
        call("xrh_tangent_step", tp, self.n_tasks, self.total_ctas, self.step, ptr(self.sq), s)
        call("xrh_gram_grouped", tp, self.n_tasks, self.total_ctas, 1, s)
        if self.small_ns:
            call("xrh_inv_sqrt_small", tp, self.n_tasks, NS_ITERS, s)
        else:
            self.ns_grouped.run()
        call("xrh_left_multiply", tp, self.n_tasks, self.total_ctas, s)
        return self.sq[0]


class XRStateOptimizer:
    def __init__(self, sysd, precision="fp64", step=0.02, lanczos_m=48, warm_m=24, orbital_gradient=True,
                 use_graphs=True, device="cuda"):
        self.sysd = sysd
        self.charges = list(sysd["charges"])
        chg = self.charges
        dev = torch.device(device)
        self.device = dev
        self.spaces = [FragmentSpace({c: sysd["states"][m][c][1] for c in chg}, sysd["n_orb"], sysd["n_core"],
                                     sysd["n_elec_ref"], device=dev) for m in range(2)]
        ns = [{c: sysd["states"][m][c][0].shape[0] for c in chg} for m in range(2)]
        self.ints = DeviceIntegrals(h=sysd["h"], V=sysd["V"], Ns=sysd["Ns"], device=dev)
        self.plan = XRDimerPlan(self.spaces, ns, [chg, chg], self.ints, output="full", precision=precision,
                                layout="sectors")
        self.adj = XRDimerAdjoint(self.plan)
        for m in range(2):
            for c in chg:
                self.plan.coeffs[m][c].copy_(torch.as_tensor(sysd["states"][m][c][0], device=dev))
        self.step_size = step
        parts = self.adj.state_gradient_parts()
        self.stepper = StateStepper([self.plan.coeffs[m][c] for m, c, _, _ in parts],
                                    [(gT, gT32) for _, _, gT, gT32 in parts], step)
        self.lz = {t: Lanczos(sec["dim"], m=lanczos_m, device=dev) for t, sec in self.plan.sectors.items()}
        self.lz_warm = {t: Lanczos(sec["dim"], m=warm_m, device=dev) for t, sec in self.plan.sectors.items()}
        self.target = None
        self.d_product = torch.zeros(self.plan.tot[0] * self.plan.tot[1], dtype=torch.float64, device=dev)
        self.orbital = orbital_gradient
        if orbital_gradient:
            self.T = torch.as_tensor(sysd["h"], device=dev)
            self.U = torch.zeros((2,) + self.T.shape, dtype=torch.float64, device=dev)
            self.V = torch.as_tensor(sysd["V"], device=dev)
            self.sidx = spin_orbital_spatial_index([sysd["n_orb"]] * 2)
        self.kappa_grad = None
        self.grad_norm = None
        self.use_graphs = use_graphs
        self._graphs = None
        self.energy = None
        self.residual = None

    # -------------------------------------------------------------------- device parts --
    def _forward(self, sectors, warm):
        self.plan.launch()
        for t in sectors:
            lz = (self.lz_warm if warm else self.lz)[t]
            lz.krylov(self.plan.sectors[t]["H"])
            lz.stage_to_host()

    def _backward(self, t, warm):
        lz = (self.lz_warm if warm else self.lz)[t]
        d = lz.ground_vector()
        self._scatter_ground(t, d)
        # the warm start of the next iteration
        self.lz_warm[t].v0.copy_(d)
        self.adj.launch(self.d_product)
        self._gsq = self.stepper.launch()
        if self.orbital:
            self.kappa_grad = self.adj.orbital_gradient(self.T, self.U, self.V, self.sidx)

    # ----------------------------------------------------------------------- iteration --
    def _solve(self, sectors, warm):
        best = None
        for t in sectors:
            lz = (self.lz_warm if warm else self.lz)[t]
            w, resid = lz.solve(1)
            if best is None or w[0] < best[0]:
                best = (w[0], t, resid)
        return best

    def iterate(self):
        """One optimizer iteration; returns the energy of the states it started from."""
        torch_stream = torch.cuda.current_stream()
        if self.target is None:
            sectors = list(self.plan.sectors)
            self._forward(sectors, warm=False)
            torch_stream.synchronize()
            E, t, resid = self._solve(sectors, warm=False)
            self.target = t
            self._backward(t, warm=False)
        else:
            t = self.target
            if self.use_graphs:
                if self._graphs is None:
                    self._capture(t)
                self._graphs[0].replay()
            else:
                self._forward([t], warm=True)
            torch_stream.synchronize()
            E, _, resid = self._solve([t], warm=True)
            if self.use_graphs:
                self.lz_warm[t].y.copy_(torch.from_numpy(self._ritz_padded(t)))
                self._graphs[1].replay()
            else:
                self._backward(t, warm=True)
        self.energy, self.residual = float(E), float(resid)
        return self.energy

    def _ritz_padded(self, t):
        lz = self.lz_warm[t]
        y = np.zeros(lz.m + 1)
        y[:lz._cut] = lz._ritz
        return y

    def _capture(self, t):
        """Record the forward (build + Krylov) and backward (adjoint + update) launch sequences."""
        lz = self.lz_warm[t]
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):          # warm the allocator and caches outside capture
            self._forward([t], warm=True)
        torch.cuda.current_stream().wait_stream(s)
        torch.cuda.synchronize()
        lz.solve(1)
        g0, g1 = torch.cuda.CUDAGraph(), torch.cuda.CUDAGraph()
        saved = [{c: self.plan.coeffs[m][c].clone() for c in self.charges} for m in range(2)]
        v0 = lz.v0.clone()
        from . import _lib
        n0 = _lib.LaunchCounter.count
        with torch.cuda.graph(g0):
            self._forward([t], warm=True)
        with torch.cuda.graph(g1):
            self._backward_graphed(t)
        self.graph_kernels = _lib.LaunchCounter.count - n0
        _lib.LaunchCounter.count = n0
        # capture does not execute: restore nothing, but keep the warm vector and states intact
        lz.v0.copy_(v0)
        for m in range(2):
            for c in self.charges:
                self.plan.coeffs[m][c].copy_(saved[m][c])
        torch.cuda.synchronize()
        self._graphs = (g0, g1)

    def _backward_graphed(self, t):
        lz = self.lz_warm[t]
        d = lz.vec
        _lib.zero_(d)
        call("xrh_gemv_cols", lz.m, lz.n, ptr(lz.V), lz.n, ptr(lz.y), 1.0, ptr(d), stream_ptr())
        self._scatter_ground(t, d)
        lz.v0.copy_(d)
        self.adj.launch(self.d_product)
        self._gsq = self.stepper.launch()
        if self.orbital:
            self.kappa_grad = self.adj.orbital_gradient(self.T, self.U, self.V, self.sidx)

    def _scatter_ground(self, t, d):
        """d_product (product order, zero outside sector t) from the sector's ground vector."""
        rows = self.plan.sectors[t]["rows"]
        _lib.zero_(self.d_product)
        call("xrh_index_move", rows.numel(), ptr(rows), ptr(d), ptr(self.d_product), 0, stream_ptr())

    @property
    def gradient_norm(self):
        return float(self._gsq.sqrt())
