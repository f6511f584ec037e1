"""ctypes bindings to the reference's own general-XRCC C kernels, compiled from source by
oracle/build_ref.sh into oracle/_ref/.  TEST INFRASTRUCTURE ONLY: used by tests/, by the
golden-fixture generator and by bench.py's CPU baseline; never by the product path.

Signatures follow the reference sources:
  general-XRCC/density_tensors.c:162-556  (a/c/ca/aa/cc/caa/cca/ccaa_tensor)
  general-XRCC/H_contractions.c:22-252    (monomer*, dimer_*, trimer_*)
and the driver that packs their arguments, general-XRCC/build_density_tensors.py:57-160.
"""
import ctypes
import math
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_REF_DIR = os.path.join(_HERE, "_ref")

_i64 = ctypes.c_longlong
_dp = ctypes.POINTER(ctypes.c_double)
_lp = ctypes.POINTER(ctypes.c_longlong)

DENSITY_OPS = ("a", "c", "ca", "aa", "cc", "caa", "cca", "ccaa")
H_FUNCS = {
    # name: (number of int args, number of pointer args)
    "monomer": (1, 4), "monomer_1e": (1, 2), "monomer_2e": (1, 2), "monomer_extPot": (1, 2),
    "dimer_2min2pls": (2, 3), "dimer_1min1pls_1e": (2, 3), "dimer_1min1pls_2e": (2, 6),
    "dimer_ExEx": (2, 3),
    "trimer_2min1pls1pls": (3, 4), "trimer_2pls1min1min": (3, 4), "trimer_Ex1min1pls": (3, 4),
}


def available():
    return (os.path.exists(os.path.join(_REF_DIR, "libref_density_tensors.so")) and
            os.path.exists(os.path.join(_REF_DIR, "libref_H_contractions.so")))


_libs = {}


def _lib(name):
    if name not in _libs:
        path = os.path.join(_REF_DIR, f"libref_{name}.so")
        if not os.path.exists(path):
            raise FileNotFoundError(f"{path} missing: run oracle/build_ref.sh")
        lib = ctypes.CDLL(path)
        if name == "density_tensors":
            for op in DENSITY_OPS:
                f = getattr(lib, f"{op}_tensor")
                f.restype = None
                f.argtypes = [_dp, _i64, _i64, _lp, _lp, ctypes.POINTER(_dp), _lp,
                              ctypes.POINTER(_lp), _i64, _i64, ctypes.POINTER(_lp), _i64]
        else:
            for fname, (n_int, n_ptr) in H_FUNCS.items():
                f = getattr(lib, fname)
                f.restype = ctypes.c_double
                f.argtypes = [_i64] * n_int + [_dp] * n_ptr
        _libs[name] = lib
    return _libs[name]


def fci_combo_mat(n_elec, n_spin_orbs):
    """Binomial table in the layout general-XRCC/build_density_tensors.py:31-37 expects."""
    m = np.zeros((max(n_elec, 0), n_spin_orbs), dtype=np.int64)
    for i in range(n_elec):
        for j in range(i, n_spin_orbs):
            m[i, j] = math.comb(j, i)
    return m


def _ptr(a, t=_dp):
    return a.ctypes.data_as(t)


def ref_density(op, sectors, bra_idx, ket_idx, n_orbs, n_core):
    """Run the reference <op>_tensor kernel.

    sectors: list of (coeffs[n_states, n_conf] float64, occ[n_conf, n_e] int64) per charge
    index; occ lists must be the complete lexicographic valence enumeration the kernel's
    ranking assumes (general-XRCC/density_tensors.c:29-62).
    Returns ndarray (n_bra, n_ket, N, ..., N) with N = 2*n_orbs.
    """
    lib = _lib("density_tensors")
    n = len(sectors)
    N = 2 * n_orbs
    n_elec = np.array([s[1].shape[1] for s in sectors], dtype=np.int64)
    n_states = np.array([s[0].shape[0] for s in sectors], dtype=np.int64)
    n_configs = np.array([s[1].shape[0] for s in sectors], dtype=np.int64)
    coeffs = [np.ascontiguousarray(s[0], dtype=np.float64) for s in sectors]
    occs = [np.ascontiguousarray(s[1], dtype=np.int64) if s[1].size else np.zeros(1, np.int64)
            for s in sectors]
    combos = [fci_combo_mat(int(n_elec[i]) - 2 * n_core, N - 2 * n_core) for i in range(n)]
    combos = [c if c.size else np.zeros(1, np.int64) for c in combos]
    zp = (_dp * n)(*[_ptr(c) for c in coeffs])
    cp = (_lp * n)(*[_ptr(o, _lp) for o in occs])
    bp = (_lp * n)(*[_ptr(c, _lp) for c in combos])
    k = len(op)
    out = np.zeros(int(n_states[bra_idx] * n_states[ket_idx]) * N ** k, dtype=np.float64)
    getattr(lib, f"{op}_tensor")(_ptr(out), bra_idx, ket_idx, _ptr(n_elec, _lp), _ptr(n_states, _lp),
                                 zp, _ptr(n_configs, _lp), cp, n_orbs, n_core, bp, 1)
    return out.reshape((int(n_states[bra_idx]), int(n_states[ket_idx])) + (N,) * k)


def ref_h(fname, *args):
    """Call one reference H_contractions.c function; ints first, then float64 arrays."""
    lib = _lib("H_contractions")
    n_int, n_ptr = H_FUNCS[fname]
    ints = [int(a) for a in args[:n_int]]
    arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in args[n_int:]]
    assert len(arrs) == n_ptr
    return getattr(lib, fname)(*ints, *[_ptr(a) for a in arrs])
