"""Host-side bookkeeping of the ring (qodeapplications_gb300.ring): the nearest-neighbour
triples and the many-body-expansion energies, checked against the expansion written out
term by term for a ring of 5."""
import itertools

from qodeapplications_gb300.ring import mbe_energies, ring_pairs, ring_triples


def test_ring_pairs_and_triples():
    assert ring_pairs(4) == [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)]
    assert ring_triples(8) == [(i, (i + 1) % 8, (i + 2) % 8) for i in range(8)]
    assert ring_triples(3) == [(0, 1, 2)]
    assert ring_triples(2) == []


def test_mbe_energies_match_the_expansion():
    n = 5
    E1 = {i: -1.0 - 0.1 * i for i in range(n)}
    E2p = {p: E1[p[0]] + E1[p[1]] - 0.01 * (p[0] + 2 * p[1] + 1) for p in ring_pairs(n)}
    E3t = {t: sum(E1[i] for i in t) - 0.003 * (t[0] + 1) for t in ring_triples(n)}
    e2, e3 = mbe_energies(E1, E2p, E3t, n)
    ref2 = sum(E1.values()) + sum(E2p[(i, j)] - E1[i] - E1[j] for i, j in itertools.combinations(range(n), 2))
    ref3 = ref2
    for t in ring_triples(n):
        inc = E3t[t]
        for a, b in ((0, 1), (1, 2), (0, 2)):
            inc -= E2p[tuple(sorted((t[a], t[b])))]
        ref3 += inc + sum(E1[i] for i in t)
    assert abs(e2 - ref2) < 1e-12 and abs(e3 - ref3) < 1e-12
