"""The lazily blocked integrals of large chains and rings (synthetic.ChainIntegralSource) are
the blocks of make_system's supersystem arrays, and its states continue the same random
stream (CPU only)."""
import numpy as np

from qodeapplications_gb300 import synthetic as S


def test_chain_blocks_equal_make_system_blocks():
    n_frag, n_orb, seed = 3, 3, 9
    sysd = S.make_system(n_frag=n_frag, n_orb=n_orb, n_states=2, seed=seed)
    src = S.ChainIntegralSource(n_frag, n_orb, seed=seed)
    N = 2 * n_orb
    sl = [slice(m * N, (m + 1) * N) for m in range(n_frag)]
    for m in range(n_frag):
        for n in range(n_frag):
            np.testing.assert_allclose(src.T[m, n], sysd["h"][sl[m], sl[n]], rtol=0, atol=1e-15)
            for o in range(n_frag):
                for p in range(n_frag):
                    np.testing.assert_allclose(src.V[m, n, o, p], sysd["V"][sl[m], sl[n], sl[o], sl[p]],
                                               rtol=0, atol=1e-15)
    states = src.make_states([+1, 0, -1], 2)
    for m in range(n_frag):
        for c in (+1, 0, -1):
            np.testing.assert_array_equal(states[m][c][0], sysd["states"][m][c][0])
            np.testing.assert_array_equal(states[m][c][1], sysd["states"][m][c][1])
