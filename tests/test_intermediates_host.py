"""Host logic of the density build through intermediate determinants (no GPU): the index
plans, evaluated with NumPy, give the oracle's transition densities (the restatement of
general-XRCC/density_tensors.c pinned to the compiled reference) for every operator string
and charge pair, with and without a frozen core."""
import numpy as np
import pytest

import xr_oracle as O
from qodeapplications_gb300 import synthetic as S
from qodeapplications_gb300.intermediates import OP_SPLIT, numpy_density, plan_block


@pytest.mark.parametrize("n_orb,n_core,seed", [(4, 0, 1), (5, 1, 2)])
def test_intermediate_densities_match_oracle(n_orb, n_core, seed):
    chg = (+1, 0, -1)
    sysd = S.make_system(n_frag=1, n_orb=n_orb, n_states=3, charges=chg, n_core=n_core, seed=seed)
    st = sysd["states"][0]
    dens = O.build_densities({c: O.Sector(*st[c]) for c in chg}, n_orb, n_core, 4,
                             ops=tuple(OP_SPLIT))
    N = 2 * n_orb
    checked = 0
    for bc in chg:
        for kc in chg:
            for op in O.OPS_FOR_DCHG.get(bc - kc, ()):
                if op not in OP_SPLIT:
                    continue
                plan = plan_block(op, st[bc][1], st[kc][1], N)
                ref = dens[op][(bc, kc)]
                if plan is None:
                    assert np.abs(ref).max() == 0.0
                    continue
                got = numpy_density(plan, st[bc][0].T, st[kc][0].T)
                np.testing.assert_allclose(got, ref, atol=1e-13)
                checked += 1
    assert checked >= 12
