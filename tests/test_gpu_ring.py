"""Ring of fragments (qodeapplications_gb300.ring) against the oracle: every monomer, pair and
nearest-neighbour triple energy of a ring of 4 fragments (3 spatial orbitals, 3 states per
charge +1, 0, -1) is the lowest eigenvalue of the oracle's order-0 general-XRCC Hamiltonian
of those fragments (general_xr_H_full, pinned by test_oracle.py) in its neutral sector, to
1e-9 Eh; the state gradient of E2 matches central finite differences (step 1e-5) to 1e-6
relative; the 3xTF32 ring is within 1e-6 Eh (E2, E3) and 1e-5 relative (gradient) of FP64."""
import numpy as np
import pytest

import xr_oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

N_FRAG, N_ORB, N_STATES, N_REF = 4, 3, 3, 3


def _ring(**kw):
    from qodeapplications_gb300.ring import XRRing
    args = dict(n_frag=N_FRAG, n_orb=N_ORB, n_states=N_STATES, n_elec_ref=N_REF, precision="fp64", tol=1e-11,
                pair_m=40, triple_m=40, graph=False, autotune=False)
    args.update(kw)
    return XRRing(**args)


def _sub_ints(src, frags):
    N = 2 * src.n_orb
    k = len(frags)
    h = np.zeros((k * N, k * N))
    V = np.zeros((k * N,) * 4)
    sl = [slice(a * N, (a + 1) * N) for a in range(k)]
    for a, fa in enumerate(frags):
        for b, fb in enumerate(frags):
            h[sl[a], sl[b]] = src.T[fa, fb]
            for c, fc in enumerate(frags):
                for d, fd in enumerate(frags):
                    V[sl[a], sl[b], sl[c], sl[d]] = src.V[fa, fb, fc, fd]
    return O.FragInts(h, V, [N] * k)


def _oracle_energy(ring, frags):
    """Lowest eigenvalue of the oracle's Hamiltonian of these fragments, neutral sector."""
    dens = [O.build_densities({c: O.Sector(ring.coeffs[f][c].cpu().numpy(), ring.masks[c]) for c in ring.charges},
                              ring.n_orb, 0, ring.n_elec_ref) for f in frags]
    H = O.general_xr_H_full(dens, _sub_ints(ring.src, frags), ring.n_elec_ref, ring.charges, len(frags))
    chg = np.repeat(ring.charges, ring.n_states)
    tot = np.zeros(1, dtype=int)
    for _ in frags:
        tot = (tot[:, None] + chg[None, :]).reshape(-1)
    keep = np.flatnonzero(tot == 0)
    Hs = H[np.ix_(keep, keep)]
    return np.linalg.eigvalsh(0.5 * (Hs + Hs.T))[0]


def test_ring_subcluster_energies_match_oracle():
    from qodeapplications_gb300.ring import mbe_energies
    ring = _ring()
    out = ring.iterate()
    ring.check_status()
    assert len(ring.E_pair) == 6 and len(ring.E_triple) == 4 and len(ring.E_mono) == 4
    for F, E in ring.E_mono.items():
        assert abs(E - _oracle_energy(ring, (F,))) <= 1e-9, F
    for P, E in ring.E_pair.items():
        assert abs(E - _oracle_energy(ring, P)) <= 1e-9, P
    for T, E in ring.E_triple.items():
        assert abs(E - _oracle_energy(ring, T)) <= 1e-9, T
    E2, E3 = mbe_energies(ring.E_mono, ring.E_pair, ring.E_triple, N_FRAG)
    assert abs(out["E2"] - E2) <= 1e-12 and abs(out["E3"] - E3) <= 1e-12


def _directional(ring, dirs):
    g = ring.state_gradient()
    return sum(float((g[f][c].cpu() * dirs[f][c]).sum()) for f in range(ring.n_frag) for c in ring.charges)


def test_ring_state_gradient_matches_finite_differences():
    ring = _ring(triples=False)
    ring.iterate()
    rng = np.random.default_rng(5)
    dirs = [{c: torch.as_tensor(rng.normal(size=tuple(ring.coeffs[f][c].shape))) for c in ring.charges}
            for f in range(N_FRAG)]
    analytic = _directional(ring, dirs)
    base = [{c: z.clone() for c, z in zf.items()} for zf in ring.coeffs]
    eps, E = 1e-5, []
    for sgn in (1.0, -1.0):
        for f in range(N_FRAG):
            for c in ring.charges:
                ring.coeffs[f][c].copy_(base[f][c] + sgn * eps * dirs[f][c].cuda())
        E.append(ring.iterate()["E2"])
    fd = (E[0] - E[1]) / (2 * eps)
    assert abs(fd - analytic) <= 1e-6 * max(1.0, abs(analytic)), (fd, analytic)


def test_ring_split_precision_close_to_fp64():
    r64 = _ring()
    r32 = _ring(precision="tf32x3", hv_precision="tf32x3", graph=True)      # triples' Krylov loop as a graph
    a, b = r64.iterate(), r32.iterate()
    r32.check_status()
    assert abs(a["E2"] - b["E2"]) <= 1e-6 and abs(a["E3"] - b["E3"]) <= 1e-6
    g64, g32 = r64.state_gradient(), r32.state_gradient()
    num = sum(float((g64[f][c] - g32[f][c]).norm() ** 2) for f in range(N_FRAG) for c in r64.charges) ** 0.5
    den = sum(float(g64[f][c].norm() ** 2) for f in range(N_FRAG) for c in r64.charges) ** 0.5
    assert num <= 1e-5 * den, num / den
