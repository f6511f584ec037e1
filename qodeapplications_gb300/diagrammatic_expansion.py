"""diagrammatic_expansion.blocks with the reference's interface, evaluated on the device.

Drop-in for hermitian-XRCC/diagrammatic_expansion.py:110-124:

    b = blocks(densities, integrals, diagrams, contract_cache, timings, precon_timings,
               bra_det=False, ket_det=False)
    b[subsystem][charges][label]     e.g. b[(0, 1)][((0, 0), (+1, +1))]["v0101"]

densities   per-fragment density dictionaries (Be-states/densities.py:210-231 layout)
integrals   struct with S and the family's T, U or V blocks (T[m, n], U[k, m, n], V[m, n, o, p])
diagrams    a catalog object: qodeapplications_gb300.diagrams.ST_diagrams / SU_diagrams /
            SV_diagrams (order-0 labels; diagrams.py)
contract_cache, timings, precon_timings   accepted for the signature; the precontractions are
            evaluated inside each label's body on the device

A label's block is the sum over the catalog's permutations of phase x body, transposed back to
the subsystem's fragment order (_build_block, diagrammatic_expansion.py:27-59): (i0, j0) for a
monomer, (i0, i1, j0, j1) for a dimer, as a NumPy FP64 array (or None when the charges admit
no term, as the reference leaves it).  Results are cached per label like the reference's
_charges object.  Errors: NotImplementedError for a label absent from the catalog and for
bra_det / ket_det.
"""
import torch

from ._external import device_densities


class _charges(object):
    def __init__(self, info, subsystem, charges, diagrams):
        self._info, self._subsystem, self._charges, self._diagrams = info, subsystem, charges, diagrams
        self._results = {}

    def __getitem__(self, label):
        if label not in self._results:
            order = len(self._subsystem)
            try:
                entry = self._diagrams.catalog[order][label]
            except (KeyError, AttributeError):
                raise NotImplementedError(f"diagram '{label}' not implemented for {order} bodies") from None
            total = None
            for tp in entry(self._info, tuple(zip(self._subsystem, self._charges))):
                if tp is None:
                    continue
                term, perm = tp
                r = term()
                if r is None:
                    continue
                reorder = list(perm) + [order + p for p in perm]
                r = r.permute(*reorder) if order > 1 else r
                total = r if total is None else total + r
            self._results[label] = None if total is None else total.contiguous().cpu().numpy()
        return self._results[label]


class _subsystem(object):
    def __init__(self, info, subsystem, diagrams):
        self._info, self._subsystem, self._diagrams = info, subsystem, diagrams
        self._items = {}

    def __getitem__(self, charges):
        charges = tuple(tuple(c) for c in (charges or ()))
        if charges not in self._items:
            self._items[charges] = _charges(self._info, self._subsystem, charges, self._diagrams)
        return self._items[charges]


class blocks(object):
    def __init__(self, densities, integrals, diagrams, contract_cache=None, timings=None, precon_timings=None,
                 bra_det=False, ket_det=False, device="cuda"):
        if bra_det or ket_det:
            raise NotImplementedError("bra_det / ket_det blocks are not provided: the state gradient comes from the "
                                      "adjoint (qodeapplications_gb300.gradients) instead")
        dev = torch.device(device)
        rho = []
        for d in densities:
            r = device_densities(d, dev)
            r["ns"] = {c: int(n) for c, n in d["n_states"].items()}
            r["n_elec"] = {c: int(n) for c, n in d["n_elec"].items()}
            rho.append(r)
        N = []
        for m in range(len(densities)):
            blk = integrals.S[m, m] if hasattr(integrals, "S") else None
            if blk is None:
                for kind in ("T", "V", "U"):
                    if hasattr(integrals, kind):
                        src = getattr(integrals, kind)
                        blk = src[(m, m)] if kind == "T" else (src[(m, m, m, m)] if kind == "V" else src[(m, m, m)])
                        break
            N.append(int(blk.shape[0]))
        self._info = {"rho": rho, "integrals": integrals, "N": N, "device": dev}
        self._diagrams = diagrams
        self._items = {}
        self.densities = densities

    def __getitem__(self, subsystem):
        subsystem = tuple(subsystem or ())
        if subsystem not in self._items:
            self._items[subsystem] = _subsystem(self._info, subsystem, self._diagrams)
        return self._items[subsystem]
