"""get_xr_H with the reference's signature, on the device.

Drop-in for hermitian-XRCC/get_xr_result.get_xr_H (get_xr_result.py:45-355):

    H1, H2 = get_xr_H(ints, dens, xr_order, monomer_charges, bra_det=False, ket_det=False)

ints            (symm_ints, bior_ints, nuc_rep) as the reference's get_ints returns it
                (hermitian-XRCC/get_ints.py:116-155); structs with fragment-block accessors
                T[m, n], U[k, m, n], V[m, n, o, p] (and S[m, n]).
dens            two per-fragment density dictionaries in the layout of Be-states/densities.py
                (:210-231): dens[m][op][(bra_chg, ket_chg)] -> (n_bra, n_ket, N, ...), ops
                a, c, ca, aa, cc, caa, cca, ccaa, plus 'n_elec', 'n_states', 'n_states_bra'.
monomer_charges two charge lists; they fix the order of the charge blocks of H1 and of the
                product basis of H2.

Returns H1 = [H1_0, H1_1] (each sum_c n_c square, charge-block order) and H2 (product-state
order, get_xr_result.py:300-353), NumPy FP64 arrays as the reference returns them
(device=True keeps them as CUDA tensors).  The order-0 terms are those of
get_xr_result.py:86-132: monomers t00 + u000 + v0000 and the dimer diagrams t01, u100, u001,
u101, v0101, v0001, v0100, v0011 with the biorthogonal integrals, contracted by this library's
grouped GEMM kernels (FP64 SIMT, or 3 x BF16 / 3 x TF32 on the tensor cores with
precision=...).  v0000 contracts the stored rho^ccaa blocks with V (SV_1mer_0.py:24).

Errors mirror the reference: NotImplementedError for an xr_order other than 0 (the S-dressed
orders need the S2^-1 recipe of get_xr_result.py:133-296, which this library does not build)
and for bra_det / ket_det (the reference builds those only to assemble state gradients,
StateSpaceOptimizer/state_gradients.py:170-185; here the adjoint in gradients.py gives the
gradient directly); RuntimeError for a density block the charges need that is missing;
ValueError for densities whose shapes disagree with their state counts or that hold NaN or
infinity.
"""
import torch

from ._external import (ExternalBuilder, ExternalSpace, check_complete, check_shapes, device_densities,
                        reference_electrons)
from .hamiltonian import DeviceIntegrals, XRDimerPlan


def dimer_plan_from_densities(dens, integrals, monomer_charges, precision="fp64", output="split",
                              convention="hermitian", monomer_2e="ccaa", device="cuda"):
    """An XRDimerPlan over densities given as reference dictionaries (the two fragments of
    dens), built once: launch() then forms H without rebuilding densities."""
    charges = [list(c) for c in monomer_charges]
    dev = torch.device(device)
    ints = DeviceIntegrals(source=integrals, device=dev)
    rho, spaces, ns = [], [], []
    for m in (0, 1):
        d = dens[m]
        ns_m = {c: int(d["n_states"][c]) for c in charges[m]}
        nsb = {c: int(d.get("n_states_bra", d["n_states"])[c]) for c in charges[m]}
        if nsb != ns_m:
            raise NotImplementedError("densities with bra states other than the ket states (bra_det / ket_det)")
        r = device_densities(d, dev)
        N = int(ints.T(m, m).shape[0])
        check_shapes(r, ns_m, N, f"fragment {m}")
        check_complete(r, charges[m], f"fragment {m}", skip=() if monomer_2e == "ccaa" else ("ccaa",))
        rho.append(r)
        spaces.append(ExternalSpace(r, N, reference_electrons(d, charges[m]), charges[m], dev))
        ns.append(ns_m)
    return XRDimerPlan(spaces, ns, charges, ints, output=output, precision=precision, convention=convention,
                       layout="product", builders=[ExternalBuilder(r) for r in rho], monomer_2e=monomer_2e,
                       autotune=False)


def get_xr_H(ints, dens, xr_order, monomer_charges, bra_det=False, ket_det=False, precision="fp64",
             device=False):
    if xr_order != 0:
        raise NotImplementedError(f"xr order {xr_order} is not implemented")
    if bra_det or ket_det:
        raise NotImplementedError("bra_det / ket_det builds are not provided: the state gradient comes from the "
                                  "adjoint (qodeapplications_gb300.gradients) instead")
    symm_ints, bior_ints, nuc_rep = ints
    plan = dimer_plan_from_densities(dens, bior_ints, monomer_charges, precision=precision)
    plan.launch(build_densities=False)
    H1 = plan.H1()
    H2 = plan.H
    if plan.tc:
        plan.check_status()
    if device:
        return H1, H2
    return [h.cpu().numpy() for h in H1], H2.cpu().numpy()
