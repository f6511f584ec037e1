"""Generate the golden fixtures in tests/golden/ from the reference itself.

Run on a machine that has the reference tree after `oracle/build_ref.sh` has compiled its
C kernels; the tree is the first argument, else $XRH_REFERENCE_ROOT, else /root/reference:

    python tests/golden/make_golden.py [REFERENCE_ROOT]

Inputs are the reference's own test fixtures, tests/ref_data/check_{states,configs}_0_*.pkl
(real frozen-core Be 6-31G fragment states, read with an unpickler that only admits NumPy
arrays and Python builtins), re-ordered into the lexicographic configuration order that
general-XRCC/density_tensors.c ranks by.  Outputs come from the compiled reference kernels:

* be_densities.npz: for every (op, bra charge, ket charge) the reference
  density_tensors.c builds, two probes per (I, J) state pair: a fixed analytic weighting
  sum_idx rho[I,J,idx] * cos(0.37 idx + 0.1) and the squared norm sum_idx rho[I,J,idx]^2,
  plus the full tensors of the 1- and 2-index operators (a, c, ca, aa, cc).
* h_elements.npz: H_contractions.c functions evaluated on seeded random inputs.
* be_dimer_elements.npz: dimer matrix elements of a Be2 system (fixture states on both
  fragments, seeded synthetic integrals, n_core = 1) computed element by element with the
  reference C kernels exactly as general-XRCC/build_H.py:56-102 dispatches them.
* be_trimer_elements.npz: trimer matrix elements of a Be3 system (fixture states on all
  three fragments, seeded synthetic integrals with nonzero nuclear potentials U) computed
  element by element with the reference C trimer kernels (H_contractions.c:184-252) as
  general-XRCC/build_H.py:103-188 dispatches them.  Only this file:
      python tests/golden/make_golden.py [REFERENCE_ROOT] --trimer
"""
import os
import pickle
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "oracle"))

import ref_ctypes as R  # noqa: E402
import xr_oracle as O   # noqa: E402

N_ORBS, N_CORE, N_ELEC_REF = 9, 1, 4
CHARGES = (+1, 0, -1)


class _NumpyOnly(pickle.Unpickler):
    def find_class(self, module, name):
        if module.startswith("numpy") or module == "builtins":
            import importlib
            return getattr(importlib.import_module(module), name)
        raise pickle.UnpicklingError(f"refused {module}.{name}")


def probe_weights(n):
    return np.cos(0.37 * np.arange(n) + 0.1)


def load_be_sectors(ref_root, frag=0):
    base = os.path.join(ref_root, "tests", "ref_data")
    out = {}
    for chg in CHARGES:
        st = np.array(_NumpyOnly(open(os.path.join(base, f"check_states_{frag}_{chg}.pkl"), "rb")).load())
        cf = np.array(_NumpyOnly(open(os.path.join(base, f"check_configs_{frag}_{chg}.pkl"), "rb")).load(),
                      dtype=np.uint64)
        lex = O.all_configs(N_ORBS, N_CORE, bin(int(cf[0])).count("1"))
        pos = {int(m): i for i, m in enumerate(cf)}
        perm = np.array([pos[int(m)] for m in lex])
        out[chg] = (np.ascontiguousarray(st[:, perm]), lex)
    return out


def main(ref_root):
    assert R.available(), "run oracle/build_ref.sh first"
    N = 2 * N_ORBS
    sectors = load_be_sectors(ref_root)
    secs = [(sectors[c][0], O.masks_to_occ(sectors[c][1], N)) for c in CHARGES]
    dd = {}
    for c in CHARGES:
        dd[f"coeffs_{c}"] = sectors[c][0]
        dd[f"masks_{c}"] = sectors[c][1]
    full_ref = {}
    for bi, bc in enumerate(CHARGES):
        for ki, kc in enumerate(CHARGES):
            for op in O.OPS_FOR_DCHG.get(bc - kc, ()):
                rho = R.ref_density(op, secs, bi, ki, N_ORBS, N_CORE)
                flat = rho.reshape(rho.shape[0], rho.shape[1], -1)
                dd[f"probe_{op}_{bc}_{kc}"] = flat @ probe_weights(flat.shape[2])
                dd[f"norm2_{op}_{bc}_{kc}"] = (flat ** 2).sum(-1)
                if len(op) <= 2:
                    dd[f"full_{op}_{bc}_{kc}"] = rho
                full_ref[(op, bc, kc)] = rho
    np.savez_compressed(os.path.join(HERE, "be_densities.npz"), **dd)

    # H_contractions.c on seeded random inputs
    rng = np.random.default_rng(20240611)
    n1, n2, n3 = 5, 4, 3
    hd = {}
    args = {
        "monomer_1e": (n1, rng.standard_normal(n1 ** 2), rng.standard_normal(n1 ** 2)),
        "monomer_2e": (n1, rng.standard_normal(n1 ** 4), rng.standard_normal(n1 ** 4)),
        "monomer_extPot": (n1, rng.standard_normal(n1 ** 2), rng.standard_normal(n1 ** 2)),
        "dimer_2min2pls": (n1, n2, rng.standard_normal(n1 ** 2), rng.standard_normal(n2 ** 2),
                           rng.standard_normal(n1 * n1 * n2 * n2)),
        "dimer_1min1pls_1e": (n1, n2, rng.standard_normal(n1), rng.standard_normal(n2),
                              rng.standard_normal(n1 * n2)),
        "dimer_1min1pls_2e": (n1, n2, rng.standard_normal(n1), rng.standard_normal(n1 ** 3),
                              rng.standard_normal(n2), rng.standard_normal(n2 ** 3),
                              rng.standard_normal(n1 ** 3 * n2), rng.standard_normal(n1 * n2 ** 3)),
        "dimer_ExEx": (n1, n2, rng.standard_normal(n1 ** 2), rng.standard_normal(n2 ** 2),
                       rng.standard_normal((n1 * n2) ** 2)),
        "trimer_2min1pls1pls": (n1, n2, n3, rng.standard_normal(n1 ** 2), rng.standard_normal(n2),
                                rng.standard_normal(n3), rng.standard_normal(n1 * n1 * n2 * n3)),
        "trimer_2pls1min1min": (n1, n2, n3, rng.standard_normal(n1 ** 2), rng.standard_normal(n2),
                                rng.standard_normal(n3), rng.standard_normal(n2 * n3 * n1 * n1)),
        "trimer_Ex1min1pls": (n1, n2, n3, rng.standard_normal(n1 ** 2), rng.standard_normal(n2),
                              rng.standard_normal(n3), rng.standard_normal(n1 * n2 * n1 * n3)),
    }
    for name, a in args.items():
        n_int = R.H_FUNCS[name][0]
        hd[f"{name}__ints"] = np.array(a[:n_int], dtype=np.int64)
        for i, arr in enumerate(a[n_int:]):
            hd[f"{name}__arg{i}"] = arr
        hd[f"{name}__out"] = np.array(R.ref_h(name, *a))
    np.savez_compressed(os.path.join(HERE, "h_elements.npz"), **hd)

    # Be2 dimer elements with the fixture states on both fragments
    from qodeapplications_gb300 import synthetic as S
    rng = np.random.default_rng(99)
    nsp = 2 * N_ORBS
    a = rng.normal(0, 0.1, (nsp, nsp))
    h_sp = np.triu(a) + np.triu(a, 1).T
    L = rng.normal(0, 0.05, (40, nsp, nsp))
    L = 0.5 * (L + L.transpose(0, 2, 1))
    h, V = S.spin_orbital_integrals(h_sp, np.einsum("kpq,krs->pqrs", L, L), [N_ORBS, N_ORBS])
    ints = O.FragInts(h, V, [N, N])
    rho = {}
    for (op, bc, kc), t in full_ref.items():
        rho.setdefault(op, {})[(bc, kc)] = t
    ns = {c: sectors[c][0].shape[0] for c in CHARGES}
    T, U, Vb = ints.T, ints.U, ints.V
    el = []
    rng2 = np.random.default_rng(5)
    while len(el) < 400:
        ci1, ci2, cj1 = (int(x) for x in rng2.choice(CHARGES, 3))
        cj2 = ci1 + ci2 - cj1
        if cj2 not in CHARGES or abs(ci1 - cj1) > 2:
            continue
        i1, i2 = int(rng2.integers(ns[ci1])), int(rng2.integers(ns[ci2]))
        j1, j2 = int(rng2.integers(ns[cj1])), int(rng2.integers(ns[cj2]))
        s2 = (-1) ** ((N_ELEC_REF - ci2) % 2)
        k1, k2 = (ci1, cj1), (ci2, cj2)
        if ci1 == cj1 - 2:
            v = R.ref_h("dimer_2min2pls", N, N, rho["cc"][k1][i1, j1], rho["aa"][k2][i2, j2], Vb[0, 0, 1, 1])
        elif ci1 == cj1 - 1:
            v = s2 * (R.ref_h("dimer_1min1pls_1e", N, N, rho["c"][k1][i1, j1], rho["a"][k2][i2, j2],
                              T[0, 1] + U[0, 0, 1] + U[1, 0, 1]) +
                      R.ref_h("dimer_1min1pls_2e", N, N, rho["c"][k1][i1, j1], rho["cca"][k1][i1, j1],
                              rho["a"][k2][i2, j2], rho["caa"][k2][i2, j2], Vb[0, 0, 0, 1], Vb[0, 1, 1, 1]))
        elif ci1 == cj1:
            v = R.ref_h("dimer_ExEx", N, N, rho["ca"][k1][i1, j1], rho["ca"][k2][i2, j2], Vb[0, 1, 0, 1])
        elif ci1 == cj1 + 1:
            v = -s2 * (R.ref_h("dimer_1min1pls_1e", N, N, rho["c"][k2][i2, j2], rho["a"][k1][i1, j1],
                               T[1, 0] + U[0, 1, 0] + U[1, 1, 0]) +
                       R.ref_h("dimer_1min1pls_2e", N, N, rho["c"][k2][i2, j2], rho["cca"][k2][i2, j2],
                               rho["a"][k1][i1, j1], rho["caa"][k1][i1, j1], Vb[1, 1, 1, 0], Vb[1, 0, 0, 0]))
        else:
            v = R.ref_h("dimer_2min2pls", N, N, rho["cc"][k2][i2, j2], rho["aa"][k1][i1, j1], Vb[1, 1, 0, 0])
        el.append((ci1, ci2, cj1, cj2, i1, i2, j1, j2, v))
    # monomer elements: Rccaa scalar (build_density_tensors.py:129-133) + monomer_1e
    mono = []
    for c in CHARGES:
        for i in range(ns[c]):
            for j in range(ns[c]):
                e2 = R.ref_h("monomer_2e", N, full_ref[("ccaa", c, c)][i, j], Vb[0, 0, 0, 0])
                e1 = R.ref_h("monomer_1e", N, full_ref[("ca", c, c)][i, j], T[0, 0] + U[0, 0, 0])
                mono.append((c, i, j, e1 + e2))
    np.savez_compressed(os.path.join(HERE, "be_dimer_elements.npz"),
                        h_sp=h_sp, L=L, elements=np.array(el, dtype=np.float64),
                        monomer=np.array(mono, dtype=np.float64))
    print("golden fixtures written to", HERE)


def trimer_elements(ref_root, n_el=300):
    assert R.available(), "run oracle/build_ref.sh first"
    from qodeapplications_gb300 import synthetic as S
    N = 2 * N_ORBS
    sectors = load_be_sectors(ref_root)
    secs = [(sectors[c][0], O.masks_to_occ(sectors[c][1], N)) for c in CHARGES]
    rho = {}
    for bi, bc in enumerate(CHARGES):
        for ki, kc in enumerate(CHARGES):
            for op in O.OPS_FOR_DCHG.get(bc - kc, ()):
                if op in ("a", "c", "ca", "aa", "cc"):
                    rho.setdefault(op, {})[(bc, kc)] = R.ref_density(op, secs, bi, ki, N_ORBS, N_CORE)
    ns = {c: sectors[c][0].shape[0] for c in CHARGES}
    rng = np.random.default_rng(777)
    nsp = 3 * N_ORBS
    a = rng.normal(0, 0.1, (nsp, nsp))
    h_sp = np.triu(a) + np.triu(a, 1).T
    L = rng.normal(0, 0.05, (20, nsp, nsp))
    L = 0.5 * (L + L.transpose(0, 2, 1))
    u_sp = []
    U = []
    for _k in range(3):
        b = rng.normal(0, 0.05, (nsp, nsp))
        b = np.triu(b) + np.triu(b, 1).T
        u_sp.append(b)
        U.append(S.spin_orbital_integrals(b, np.zeros((nsp,) * 4), [N_ORBS] * 3)[0])
    U = np.array(U)
    h, V = S.spin_orbital_integrals(h_sp, np.einsum("kpq,krs->pqrs", L, L), [N_ORBS] * 3)
    ints = O.FragInts(h + U.sum(0), V, [N, N, N], U=U)
    Ub, Vb = ints.U, ints.V
    el = []
    rng2 = np.random.default_rng(6)
    m1, m2, m3 = 0, 1, 2
    while len(el) < n_el:
        ci = [int(x) for x in rng2.choice(CHARGES, 3)]
        cj = [int(x) for x in rng2.choice(CHARGES, 3)]
        d = sorted(x - y for x, y in zip(ci, cj))
        if d not in ([-2, 1, 1], [-1, 0, 1], [-1, -1, 2]):
            continue
        I = [int(rng2.integers(ns[c])) for c in ci]
        J = [int(rng2.integers(ns[c])) for c in cj]
        k = [(ci[x], cj[x]) for x in range(3)]

        def r(op, x):
            return rho[op][k[x]][I[x], J[x]]
        s2 = (-1) ** ((N_ELEC_REF - ci[1]) % 2)
        s3 = (-1) ** ((N_ELEC_REF - ci[2]) % 2)
        t2m, t2p, tex, ext = "trimer_2min1pls1pls", "trimer_2pls1min1min", "trimer_Ex1min1pls", "dimer_1min1pls_1e"
        if ci[0] == cj[0] - 2:
            v = s3 * R.ref_h(t2m, N, N, N, r("cc", 0), r("a", 1), r("a", 2), Vb[m1, m1, m2, m3])
        elif ci[1] == cj[1] - 2:
            v = s2 * s3 * R.ref_h(t2m, N, N, N, r("cc", 1), r("a", 0), r("a", 2), Vb[m2, m2, m1, m3])
        elif ci[2] == cj[2] - 2:
            v = s2 * R.ref_h(t2m, N, N, N, r("cc", 2), r("a", 0), r("a", 1), Vb[m3, m3, m1, m2])
        elif ci[0] == cj[0] + 2:
            v = s3 * R.ref_h(t2p, N, N, N, r("aa", 0), r("c", 1), r("c", 2), Vb[m2, m3, m1, m1])
        elif ci[1] == cj[1] + 2:
            v = s2 * s3 * R.ref_h(t2p, N, N, N, r("aa", 1), r("c", 0), r("c", 2), Vb[m1, m3, m2, m2])
        elif ci[2] == cj[2] + 2:
            v = s2 * R.ref_h(t2p, N, N, N, r("aa", 2), r("c", 0), r("c", 1), Vb[m1, m2, m3, m3])
        else:
            # one fragment keeps its charge (Rca), one gains and one loses an electron
            ex = [x for x in range(3) if ci[x] == cj[x]][0]
            cr = [x for x in range(3) if ci[x] == cj[x] - 1][0]
            an = [x for x in range(3) if ci[x] == cj[x] + 1][0]
            mm = (m1, m2, m3)
            tmp = R.ref_h(tex, N, N, N, r("ca", ex), r("c", cr), r("a", an), Vb[mm[ex], mm[cr], mm[ex], mm[an]])
            if I[ex] == J[ex]:
                tmp += R.ref_h(ext, N, N, r("c", cr), r("a", an), Ub[mm[ex], mm[cr], mm[an]])
            # the phase of build_H.py:146-187 for each (Ex, creating, annihilating) placement
            sgn = {(0, 1, 2): s3, (0, 2, 1): -s3, (1, 0, 2): s2 * s3, (1, 2, 0): -s2 * s3,
                   (2, 0, 1): s2, (2, 1, 0): -s2}[(ex, cr, an)]
            v = sgn * tmp
        el.append(tuple(ci) + tuple(cj) + tuple(I) + tuple(J) + (v,))
    np.savez_compressed(os.path.join(HERE, "be_trimer_elements.npz"), h_sp=h_sp, L=L, u_sp=np.array(u_sp),
                        elements=np.array(el, dtype=np.float64))
    print("trimer fixture written to", HERE)


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    root = args[0] if args else os.environ.get("XRH_REFERENCE_ROOT", "/root/reference")
    if "--trimer" in sys.argv:
        trimer_elements(root)
    else:
        main(root)
        trimer_elements(root)
