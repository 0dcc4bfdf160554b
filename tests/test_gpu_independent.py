"""The GPU solves against the dense hierarchy of the published equations (tests/dense_heom.py),
with no oracle in between: interacting single-orbital and double-dot models at tier 2, Pade
M = 1, their steady states by the FP64 TFQMR and by the mixed-precision refinement, through
the C ABI.  Occupations within 1e-8, lead currents per spin within 1e-8 relative."""
import numpy as np
import pytest

import heomq
from test_independent_heom import INTERACTING, dense_model, observables_dense, oracle_cfg

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", list(INTERACTING))
@pytest.mark.parametrize("prec, crit", [(heomq.PREC_FP64, 1e-10), (heomq.PREC_MIXED, 1e-11)], ids=["fp64", "mixed"])
def test_gpu_steady_state_matches_dense_hierarchy(name, prec, crit):
    norbs, p = INTERACTING[name]
    h, a, n, idx, H = dense_model(norbs, ntier=2, **p)
    d_occ, d_cur, d_dbl, d_coh, d_spec = observables_dense(h, h.steady(), a, idx, norbs)
    m = heomq.Model(oracle_cfg(norbs, p, 2))
    ctx = heomq.Context(m, adjoint=False)
    rho, info = ctx.solve_tfqmr(crit=crit, precision=prec, maxit0=40000)
    assert info.converged and info.resid <= crit
    np.testing.assert_allclose(ctx.occupation(rho), d_occ, atol=1e-8)
    np.testing.assert_allclose(ctx.current(rho), d_cur, atol=1e-8 * np.abs(d_cur).max())
