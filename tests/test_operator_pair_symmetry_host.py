"""The symmetries the density kernels exploit, on the oracle's densities (CPU): two adjacent
operators of one kind anticommute, so rho^aa, rho^cc (pair 0,1), rho^caa (pair 1,2) and
rho^cca (pair 0,1) change sign under the swap of that pair; rho^ca between the same real
states is Hermitian, rho^ca[i, j, p, q] = rho^ca[j, i, q, p].  Exact up to rounding (1e-14)."""
import numpy as np

import xr_oracle as O
from qodeapplications_gb300 import synthetic as S

SWAP = {"aa": (0, 1), "cc": (0, 1), "caa": (1, 2), "cca": (0, 1)}


def _densities():
    chg = (+1, 0, -1)
    sysd = S.make_system(n_frag=2, n_orb=4, n_states=3, charges=chg, seed=9)
    return O.build_densities({c: O.Sector(*sysd["states"][0][c]) for c in chg}, 4, 0, 4), chg


def test_anticommuting_pairs_change_sign():
    dens, _ = _densities()
    seen = 0
    for op, (u, v) in SWAP.items():
        for key, r in dens[op].items():
            ax = list(range(r.ndim))
            ax[2 + u], ax[2 + v] = ax[2 + v], ax[2 + u]
            assert np.abs(r + r.transpose(ax)).max() <= 1e-14 * max(np.abs(r).max(), 1.0), (op, key)
            seen += 1
    assert seen >= 4


def test_ca_between_the_same_states_is_hermitian():
    dens, chg = _densities()
    for c in chg:
        r = dens["ca"][(c, c)]
        assert np.abs(r - r.transpose(1, 0, 3, 2)).max() <= 1e-14 * max(np.abs(r).max(), 1.0), c
