"""The lowest XR-H eigenvalue as a differentiable torch function.

E(h, V, z) = lowest eigenvalue of the order-0 excitonic Hamiltonian of a dimer built from
the one-electron integrals h (supersystem spin orbitals, U folded in), the antisymmetrised
two-electron integrals V and the fragment-state coefficients z[m][charge].

forward   sets the integrals and states of a resident XRDimerPlan, launches the build and
          solves for the lowest eigenpair with restarted FP64 Lanczos to a residual tolerance;
backward  runs the adjoint (XRDimerAdjoint) with the ground vector d, E = d^T H d
          (Hellmann-Feynman): dE/dz of every fragment and charge, dE/dh and dE/dV.

This replaces the gradient quantities of the reference's state optimisation:
state_gradients (StateSpaceOptimizer/state_gradients.py:121-244) is dE/dz projected on the
tangent space of the orthonormal states (gradients.tangent_project), and orb_grads
(StateSpaceOptimizer/orb_grads.py:976-1000) is dE/dkappa, obtained here by autograd through
the rotation R = matrix_exp(kappa), h' = R^T h R, V' = V x R^4 (rotate_integrals below).

Densities are not kept for the backward pass when the plan has been reused since the forward
(another forward in between): backward then recomputes them from the saved inputs.
"""
import numpy as np
import torch

from .densities import FragmentSpace
from .eigen import Lanczos
from .gradients import XRDimerAdjoint
from .hamiltonian import DeviceIntegrals, XRDimerPlan
from .synthetic import spin_orbital_spatial_index


class XRDimerEnergy:
    """Resident plan + adjoint + eigensolver for one dimer; call it like a function.

    spaces:    two FragmentSpace objects;  n_states: two {charge: n};  charges: two lists
    Ns:        spin orbitals per fragment;  h0, V0: initial integrals (device FP64) for the plan
    precision: 'fp64' | 'bf16x3' | 'tf32x3'
    tol:       Lanczos residual tolerance of the lowest eigenpair."""

    def __init__(self, spaces, n_states, charges, Ns, h0, V0, precision="fp64", lanczos_m=64, tol=1e-9,
                 max_restarts=100):
        self.Ns = list(Ns)
        self.charges = [list(c) for c in charges]
        ints = DeviceIntegrals.from_tensors(h0, V0, self.Ns)
        self.plan = XRDimerPlan(spaces, n_states, self.charges, ints, output="full", precision=precision,
                                layout="sectors")
        self.adj = XRDimerAdjoint(self.plan)
        self.device = self.plan.device
        self.lz = {t: Lanczos(sec["dim"], m=lanczos_m, device=self.device) for t, sec in self.plan.sectors.items()}
        self.tol, self.max_restarts = tol, max_restarts
        self.d_product = torch.zeros(self.plan.tot[0] * self.plan.tot[1], dtype=torch.float64, device=self.device)
        self.version = 0
        self.sector = None
        self.residual = None

    @classmethod
    def from_system(cls, sysd, precision="fp64", device="cuda", **kw):
        """From a synthetic.make_system dictionary (integrals and masks; the states are inputs)."""
        chg = list(sysd["charges"])
        dev = torch.device(device)
        spaces = [FragmentSpace({c: sysd["states"][m][c][1] for c in chg}, sysd["n_orb"], sysd["n_core"],
                                sysd["n_elec_ref"], device=dev) for m in range(2)]
        ns = [{c: sysd["states"][m][c][0].shape[0] for c in chg} for m in range(2)]
        h0 = torch.as_tensor(sysd["h"], device=dev)
        V0 = torch.as_tensor(sysd["V"], device=dev)
        return cls(spaces, ns, [chg, chg], sysd["Ns"], h0, V0, precision=precision, **kw)

    def flat(self, coeffs):
        return [coeffs[m][c] for m in (0, 1) for c in self.charges[m]]

    def unflat(self, zs):
        it = iter(zs)
        return [{c: next(it) for c in self.charges[m]} for m in (0, 1)]

    # --------------------------------------------------------------------------------------
    def _build(self, h, V, zs):
        self.plan.set_integrals(DeviceIntegrals.from_tensors(h.detach().contiguous(), V.detach().contiguous(),
                                                             self.Ns))
        self.plan.set_coeffs(self.unflat([z.detach() for z in zs]))
        self.plan.launch()
        self.version += 1

    def _eigen(self):
        """Lowest eigenpair over the sectors (all on the first call, then the sector found)."""
        sectors = list(self.plan.sectors) if self.sector is None else [self.sector]
        best = None
        for t in sectors:
            lz = self.lz[t]
            H = self.plan.sectors[t]["H"]
            for _ in range(self.max_restarts):
                lz.krylov(H)
                lz.stage_to_host()
                torch.cuda.current_stream().synchronize()
                w, res = lz.solve(1)
                v = lz.ground_vector()
                lz.v0.copy_(v / v.norm())
                if res < self.tol:
                    break
            if best is None or w[0] < best[0]:
                best = (float(w[0]), t, float(res))
        E, t, res = best
        self.sector, self.residual = t, res
        d = self.lz[t].v0
        self.d_product.zero_()
        self.d_product.index_copy_(0, self.plan.sectors[t]["rows"], d)
        return E

    def _gradients(self):
        self.adj.launch(self.d_product)
        g = self.adj.state_gradient()
        gz = [g[m][c].clone() for m in (0, 1) for c in self.charges[m]]
        dT, _dU, dV = self.adj.integral_gradients()
        return dT, dV, gz

    def __call__(self, h, V, coeffs):
        """E (0-d FP64 tensor on the device); coeffs = two {charge: (n_states, n_conf)} dicts."""
        return _XRLowestEnergy.apply(self, h, V, *self.flat(coeffs))


class _XRLowestEnergy(torch.autograd.Function):
    @staticmethod
    def forward(ctx, engine, h, V, *zs):
        engine._build(h, V, zs)
        E = engine._eigen()
        ctx.engine = engine
        ctx.version = engine.version
        ctx.save_for_backward(h, V, *zs)
        return torch.tensor(E, dtype=torch.float64, device=h.device)

    @staticmethod
    def backward(ctx, gE):
        engine = ctx.engine
        h, V, *zs = ctx.saved_tensors
        if engine.version != ctx.version:
            # the plan has been rebuilt since: recompute densities, H and the ground vector
            engine._build(h, V, zs)
            engine._eigen()
        dT, dV, gz = engine._gradients()
        return (None, gE * dT, gE * dV) + tuple(gE * g for g in gz)


def rotation_matrix(kappa, frag_sizes):
    """Spin-orbital rotation R = expm(kappa) for an antisymmetric spatial kappa (same rotation
    for both spins; alpha block then beta block per fragment)."""
    R_sp = torch.matrix_exp(kappa)
    sidx = spin_orbital_spatial_index(frag_sizes)
    seen, spins = {}, []
    for sp in sidx:
        spins.append(seen.get(sp, 0))
        seen[sp] = seen.get(sp, 0) + 1
    idx = torch.as_tensor(sidx, device=kappa.device)
    spins = torch.as_tensor(np.array(spins), device=kappa.device)
    same = (spins[:, None] == spins[None, :]).to(kappa.dtype)
    return R_sp[idx[:, None], idx[None, :]] * same


def rotate_integrals(h, V, kappa, frag_sizes):
    """h' = R^T h R, V'_pqrs = sum R_ap R_bq R_cr R_ds V_abcd (differentiable in kappa)."""
    R = rotation_matrix(kappa, frag_sizes)
    h2 = R.t() @ h @ R
    t = V.shape[0]
    V2 = V
    for _ in range(4):        # rotate the leading index, then cycle it to the back
        V2 = (R.t() @ V2.reshape(t, -1)).reshape(t, t, t, t).permute(1, 2, 3, 0)
    return h2, V2.contiguous()
