"""Densities and integrals handed in by a caller of the reference-signature functions.

The reference passes fragment densities as dictionaries (Be-states/densities.py:210-231,
general-XRCC/build_density_tensors.py:57-160):

    dens[op][(bra_chg, ket_chg)]  ->  (n_bra, n_ket, N, ..., N) array, or a list (over I) of
                                      lists (over J) of (N, ..., N) arrays; general-XRCC
                                      stores 'ccaa' as one precontracted number per (I, J)
    dens['n_elec'][chg], dens['n_states'][chg], dens['n_states_bra'][chg]

and integrals as structs whose T[m, n], U[k, m, n], V[m, n, o, p] are fragment blocks.  This
module uploads the densities once as contiguous FP64 device tensors and presents them to the
planned builds (XRDimerPlan, XRTrimerPlan) in the form those read: a density "builder" whose
rho dictionary is already filled and a "space" that lists which blocks exist.
"""
import numpy as np
import torch

OPS = ("a", "c", "ca", "aa", "cc", "caa", "cca", "ccaa")


def _as_array(x):
    if isinstance(x, torch.Tensor):
        return x.detach().to(torch.float64)
    if isinstance(x, (list, tuple)):
        return torch.as_tensor(np.array([[np.asarray(xij, dtype=np.float64) for xij in xi] for xi in x]))
    return torch.as_tensor(np.asarray(x, dtype=np.float64))


def device_densities(dens, device="cuda", ops=OPS):
    """{op: {(bc, kc): CUDA float64 contiguous (n_b, n_k, N...)}} from a reference dictionary."""
    out = {}
    for op in ops:
        blocks = dens.get(op, {})
        out[op] = {}
        for key, val in blocks.items():
            out[op][tuple(key)] = _as_array(val).to(device).contiguous()
    return out


def reference_electrons(dens, charges):
    """n_elec of the neutral reference, n_elec[chg] + chg (the same for every charge)."""
    refs = {int(dens["n_elec"][c]) + int(c) for c in charges}
    if len(refs) != 1:
        raise ValueError(f"n_elec is inconsistent with the charges: {dens['n_elec']}")
    return refs.pop()


class ExternalSpace:
    """What a plan reads of a FragmentSpace: the spin orbitals, the reference electron count
    and which (op, bra charge, ket charge) blocks exist."""

    def __init__(self, rho, N, n_elec_ref, charges, device):
        self.N = int(N)
        self.n_elec_ref = int(n_elec_ref)
        self.charges = list(charges)
        self.device = torch.device(device)
        self.couplings = {(op, bc, kc): None for op, blocks in rho.items() for (bc, kc) in blocks}
        self.n_conf = {c: 0 for c in charges}


class ExternalBuilder:
    """A density 'builder' whose blocks were given: build() has nothing to do."""

    def __init__(self, rho):
        self.rho = rho
        self.zT = {}

    def build(self, coeffs=None, bra_coeffs=None):
        return self.rho


# op strings per (bra_chg - ket_chg) that an order-0 build reads (general-XRCC/
# build_density_tensors.py:90-157)
OPS_FOR_DCHG = {+2: ("aa",), +1: ("a", "caa"), 0: ("ca", "ccaa"), -1: ("c", "cca"), -2: ("cc",)}


def check_complete(rho, charges, where, skip=()):
    """Every density block an order-0 build of these charges reads is present and finite:
    RuntimeError for a missing block (as the reference's lookups fail), ValueError for a
    block holding NaN or infinity."""
    for bc in charges:
        for kc in charges:
            for op in OPS_FOR_DCHG.get(bc - kc, ()):
                if op in skip:
                    continue
                t = rho.get(op, {}).get((bc, kc))
                if t is None:
                    raise RuntimeError(f"{where}: density {op}{(bc, kc)} is missing")
                if not bool(torch.isfinite(t).all()):
                    raise ValueError(f"{where}: density {op}{(bc, kc)} holds NaN or infinity")


def check_shapes(rho, n_states, N, where):
    """Every block (n_b, n_k, N^k) with n_b, n_k the dictionary's state counts."""
    for op, blocks in rho.items():
        for (bc, kc), t in blocks.items():
            if op == "ccaa" and t.dim() == 2:
                want = (n_states[bc], n_states[kc])
            else:
                want = (n_states[bc], n_states[kc]) + (N,) * len(op)
            if tuple(t.shape) != want:
                raise ValueError(f"{where}: density {op}{(bc, kc)} has shape {tuple(t.shape)}, expected {want}")
