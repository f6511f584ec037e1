"""Seeded synthetic inputs for the XR-H build (NumPy, host side).

No public dataset is involved: the workloads are fixed-seed synthetic systems with the
shapes and value distributions of the Be-chain test systems the reference is run on
(general-XRCC/Be631g.py: 9 spatial orbitals per Be, 3/4/5 electrons for charges +1/0/-1).

* One-electron integrals h: symmetric, entries N(0, 0.1), over the supersystem's spatial
  orbitals, spin-blocked (alpha block then beta block inside every fragment).
* Two-electron integrals: spatial (pq|rs) = sum_{K=1..40} L^K_pq L^K_rs with symmetric
  L^K ~ N(0, 0.05), turned into the antisymmetrised spin-orbital tensor the reference
  contracts, V_pqrs = (<pq|rs> - <pq|sr>)/4 with <pq|rs> = (pr|qs) delta_spin, so that
  H = sum h_pq c+_p a_q + sum V_pqrs c+_p c+_q a_s a_r.
* Fragment states: Gaussian CI vectors, each with a definite Sz (Sz=0 for even electron
  counts; alternating +1/2 and -1/2 for odd counts, so charge-transfer blocks do not vanish
  by spin), QR-orthonormalised within each Sz group of a charge sector.
* S = 1 (orthogonal fragments) and U = 0 (nuclear attraction folded into h).
"""
import itertools

import numpy as np


def _core_mask(n_orbs, n_core):
    m = 0
    for i in range(n_core):
        m |= (1 << i) | (1 << (n_orbs + i))
    return m


def sector_configs(n_orbs, n_core, n_elec, sz2_values):
    """Determinants (uint64 masks, spin-orbital i = alpha i, n_orbs+i = beta i) with a
    filled frozen core and 2*Sz in sz2_values, in lexicographic valence order."""
    val = [o for o in range(2 * n_orbs) if not (o < n_core or n_orbs <= o < n_orbs + n_core)]
    cm = _core_mask(n_orbs, n_core)
    k = n_elec - 2 * n_core
    out = []
    lo = (1 << n_orbs) - 1
    for comb in itertools.combinations(range(len(val)), k):
        m = cm
        for v in comb:
            m |= 1 << val[v]
        if bin(m & lo).count("1") - bin(m >> n_orbs).count("1") in sz2_values:
            out.append(m)
    return np.array(out, dtype=np.uint64)


def _sz2_of(masks, n_orbs):
    lo = np.uint64((1 << n_orbs) - 1)
    a = np.array([bin(int(m & lo)).count("1") for m in masks])
    b = np.array([bin(int(m >> np.uint64(n_orbs))).count("1") for m in masks])
    return a - b


def make_states(rng, n_orbs, n_core, n_elec, n_states):
    """n_states orthonormal Sz-definite Gaussian CI vectors; returns (coeffs, masks)."""
    if n_elec % 2 == 0:
        sz_list = [0] * n_states
    else:
        sz_list = [(+1 if i % 2 == 0 else -1) for i in range(n_states)]
    masks = sector_configs(n_orbs, n_core, n_elec, sorted(set(sz_list)))
    sz_of = _sz2_of(masks, n_orbs)
    coeffs = np.zeros((n_states, len(masks)))
    for sz in sorted(set(sz_list)):
        rows = [i for i, s in enumerate(sz_list) if s == sz]
        cols = np.nonzero(sz_of == sz)[0]
        if len(rows) > len(cols):
            raise ValueError(f"{len(rows)} states requested in a {len(cols)}-dimensional space")
        g = rng.standard_normal((len(cols), len(rows)))
        q, _ = np.linalg.qr(g)
        coeffs[np.ix_(rows, cols)] = q.T
    return coeffs, masks


def spin_orbital_integrals(h_sp, eri_sp, frag_sizes):
    """Spin-block spatial integrals fragment by fragment.  h_sp (n, n), eri_sp (pq|rs) (n^4),
    frag_sizes = spatial orbitals per fragment.  Returns h (N, N), V (N^4) with N = 2n."""
    n = h_sp.shape[0]
    so_sp = []   # spatial index of every spin orbital
    so_spin = []
    off = 0
    for nf in frag_sizes:
        for s in (0, 1):
            for i in range(nf):
                so_sp.append(off + i)
                so_spin.append(s)
        off += nf
    so_sp = np.array(so_sp)
    so_spin = np.array(so_spin)
    N = 2 * n
    h = h_sp[np.ix_(so_sp, so_sp)] * (so_spin[:, None] == so_spin[None, :])
    # <pq|rs> = (pr|qs) delta(sp,sr) delta(sq,ss)
    g = eri_sp[np.ix_(so_sp, so_sp, so_sp, so_sp)]             # (pr|qs) indexed [p,r,q,s]
    d = (so_spin[:, None] == so_spin[None, :]).astype(float)
    phys = g.transpose(0, 2, 1, 3) * d[:, None, :, None] * d[None, :, None, :]   # [p,q,r,s]
    V = 0.25 * (phys - phys.transpose(0, 1, 3, 2))
    assert h.shape == (N, N)
    return h, V


def make_system(n_frag=2, n_orb=9, n_states=10, charges=(+1, 0, -1), n_elec_ref=4, n_core=0,
                n_chol=40, seed=1234, rng_states=None):
    """A linear chain of identical-size fragments with seeded integrals and states.

    Returns a dict with keys n_frag, n_orb, n_core, n_elec_ref, charges, Ns (spin orbitals
    per fragment), h (ΣN x ΣN), V (ΣN^4), states[m][chg] = (coeffs, masks)."""
    rng = np.random.default_rng(seed)
    n = n_frag * n_orb
    a = rng.normal(0.0, 0.1, size=(n, n))
    h_sp = np.triu(a) + np.triu(a, 1).T
    L = rng.normal(0.0, 0.05, size=(n_chol, n, n))
    L = 0.5 * (L + L.transpose(0, 2, 1))
    eri = np.einsum("kpq,krs->pqrs", L, L)
    h, V = spin_orbital_integrals(h_sp, eri, [n_orb] * n_frag)
    srng = rng if rng_states is None else rng_states
    states = []
    for _m in range(n_frag):
        st = {}
        for c in charges:
            st[c] = make_states(srng, n_orb, n_core, n_elec_ref - c, n_states)
        states.append(st)
    return dict(n_frag=n_frag, n_orb=n_orb, n_core=n_core, n_elec_ref=n_elec_ref,
                charges=tuple(charges), Ns=[2 * n_orb] * n_frag, h=h, V=V, states=states)


class ChainIntegralSource:
    """The integrals of make_system (same seed, same random stream for h and the Cholesky
    vectors L^K) for chains and rings too large for the supersystem V: fragment blocks are
    formed on request, with the accessors of the reference's fragment-blocked integral
    structs (hermitian-XRCC/get_ints.py:116-155): T[m, n], U[k, m, n] (zero), V[m, n, o, p],
    S[m, n] (identity), each spin-blocked (alpha then beta inside a fragment) and V
    antisymmetrised as in spin_orbital_integrals."""

    def __init__(self, n_frag, n_orb, n_chol=40, seed=1234):
        rng = np.random.default_rng(seed)
        n = n_frag * n_orb
        a = rng.normal(0.0, 0.1, size=(n, n))
        self.h_sp = np.triu(a) + np.triu(a, 1).T
        L = rng.normal(0.0, 0.05, size=(n_chol, n, n))
        self.L = 0.5 * (L + L.transpose(0, 2, 1))
        self.rng = rng                      # continues with the states, as in make_system
        self.n_frag, self.n_orb = n_frag, n_orb
        sp = np.tile(np.arange(n_orb), 2)
        self._sp = [m * n_orb + sp for m in range(n_frag)]
        self._spin = np.repeat([0, 1], n_orb)
        outer = self

        class _Acc:
            def __init__(self, fn):
                self.fn = fn

            def __getitem__(self, key):
                return self.fn(*(key if isinstance(key, tuple) else (key,)))

        self.T = _Acc(self._T)
        self.U = _Acc(lambda k, m, n: np.zeros((2 * n_orb, 2 * n_orb)))
        self.V = _Acc(self._V)
        self.S = _Acc(lambda m, n: np.eye(2 * n_orb) if m == n else np.zeros((2 * n_orb, 2 * n_orb)))
        self._cache = {}
        del outer

    def _T(self, m, n):
        a, b = self._sp[m], self._sp[n]
        return self.h_sp[np.ix_(a, b)] * (self._spin[:, None] == self._spin[None, :])

    def _eri(self, a, b, c, d):
        """(ab|cd) for spatial index arrays."""
        return np.einsum("kab,kcd->abcd", self.L[:, a][:, :, b], self.L[:, c][:, :, d], optimize=True)

    def _V(self, m, n, o, p):
        key = (m, n, o, p)
        if key not in self._cache:
            sa, sb, sc, sd = self._sp[m], self._sp[n], self._sp[o], self._sp[p]
            sp = self._spin
            d = (sp[:, None] == sp[None, :]).astype(float)
            # <ab|cd> = (ac|bd) delta(s_a, s_c) delta(s_b, s_d)
            phys = self._eri(sa, sc, sb, sd).transpose(0, 2, 1, 3) * d[:, None, :, None] * d[None, :, None, :]
            # <ab|dc> = (ad|bc) delta(s_a, s_d) delta(s_b, s_c), indexed [a, b, c, d]
            physx = self._eri(sa, sd, sb, sc).transpose(0, 2, 3, 1) * d[:, None, None, :] * d[None, :, :, None]
            self._cache[key] = 0.25 * (phys - physx)
        return self._cache[key]

    def make_states(self, charges, n_states, n_elec_ref=4, n_core=0):
        """states[m][chg] = (coeffs, masks) from the continued random stream (make_system's)."""
        out = []
        for _m in range(self.n_frag):
            out.append({c: make_states(self.rng, self.n_orb, n_core, n_elec_ref - c, n_states) for c in charges})
        return out


def spin_block_one_electron(h_sp, frag_sizes):
    """A spatial one-electron matrix spin-blocked like spin_orbital_integrals' h."""
    sidx = np.array(spin_orbital_spatial_index(frag_sizes))
    spin = np.concatenate([np.repeat([0, 1], nf) for nf in frag_sizes])
    return h_sp[np.ix_(sidx, sidx)] * (spin[:, None] == spin[None, :])


def make_nuclear_potentials(n_frag, n_orb, scale=0.05, seed=4321):
    """Seeded fragment nuclear potentials U[k] (supersystem spin orbitals, symmetric spatial
    entries N(0, scale), spin-blocked), for inputs with U != 0: the integrals are then
    T = h - sum_k U[k] and U (the reference's fragment-blocked T and U,
    hermitian-XRCC/get_ints.py:116-155), with the total one-electron operator h unchanged."""
    rng = np.random.default_rng(seed)
    n = n_frag * n_orb
    out = []
    for _k in range(n_frag):
        a = rng.normal(0.0, scale, size=(n, n))
        out.append(spin_block_one_electron(np.triu(a) + np.triu(a, 1).T, [n_orb] * n_frag))
    return np.array(out)


def spin_orbital_spatial_index(frag_sizes):
    """Spatial orbital of every spin orbital (alpha block then beta block per fragment)."""
    out, off = [], 0
    for nf in frag_sizes:
        out += [off + i for i in range(nf)] * 2
        off += nf
    return out


def rotate_integrals(h, V, kappa_sp, frag_sizes):
    """Integrals in the orbitals rotated by R = expm(kappa) (kappa antisymmetric over the
    supersystem's spatial orbitals, the same rotation for both spins):
    h' = R^T h R, V'_pqrs = sum R_ap R_bq R_cr R_ds V_abcd."""
    from scipy.linalg import expm
    R_sp = expm(np.asarray(kappa_sp, dtype=np.float64))
    sidx = spin_orbital_spatial_index(frag_sizes)
    n = len(sidx)
    spins = []
    seen = {}
    for sp in sidx:
        spins.append(seen.get(sp, 0))
        seen[sp] = seen.get(sp, 0) + 1
    spins = np.array(spins)
    R = R_sp[np.ix_(sidx, sidx)] * (spins[:, None] == spins[None, :])
    h2 = R.T @ h @ R
    V2 = np.einsum("ap,bq,cr,ds,abcd->pqrs", R, R, R, R, V, optimize=True)
    assert h2.shape == (n, n)
    return h2, V2
