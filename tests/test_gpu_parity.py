"""GPU parity of the apply, adjoint and derivative kernels against the oracle."""
import numpy as np
import pytest

import configs as cf
import heomq
import oracle_ffi as of

pytestmark = pytest.mark.gpu

CASES = {
    "siam_L2": cf.siam(ntier=3),
    "siam_L3": cf.CFG0,
    "dqd_L2": cf.dqd(ntier=3),
    "dqd_L4": cf.CFG1,
    "hund_L2": cf.CFG4,
    "dqd_L2_prony": dict(cf.dqd(ntier=3, nmats=1, T=0.3), psf=cf.prony_table()),
}


@pytest.fixture(scope="module", params=list(CASES))
def pair(request):
    cfg = CASES[request.param]
    m = heomq.Model(cfg)
    return request.param, m, heomq.Context(m), of.Model(cfg)


def rvec(n, seed):
    r = np.random.default_rng(seed)
    return r.standard_normal(n) + 1j * r.standard_normal(n)


def test_apply_fp64_matches_oracle(pair):
    name, m, ctx, ref = pair
    x = rvec(m.lunk + 1, 1)
    y = ctx.calc_ax_tfqmr_spa(x)
    y_ref = ref.calc_ax(x)
    # FP64, different summation order: relative error at the rounding level
    assert np.linalg.norm(y - y_ref) <= 1e-13 * np.linalg.norm(y_ref), name
    assert abs(y[-1] - y_ref[-1]) <= 1e-13 * abs(y_ref[-1])


def test_calcderiv_matches_oracle(pair):
    name, m, ctx, ref = pair
    x = rvec(m.lunk, 2)
    for t in (0.0, 0.7):
        y = ctx.calcderiv_spa(t, x)
        y_ref = ref.calcderiv(t, x)
        assert np.linalg.norm(y - y_ref) <= 1e-13 * np.linalg.norm(y_ref), (name, t)


def test_adjoint_identity(pair):
    """<u, A v> = <A^H u, v> in the real inner product Re(u^H v)."""
    name, m, ctx, ref = pair
    u, v = rvec(m.lunk + 1, 3), rvec(m.lunk + 1, 4)
    lhs = np.vdot(u, ctx.calc_ax_tfqmr_spa(v)).real
    rhs = np.vdot(ctx.calc_atrx(u), v).real
    assert abs(lhs - rhs) <= 1e-12 * (abs(lhs) + 1e-300) * 10 + 1e-12 * np.linalg.norm(u) * np.linalg.norm(v), name


def test_apply_fp32x2_matches_oracle(pair):
    """The packed FP32x2 apply of the mixed-precision inner solves (f32x2 instructions, about
    48-bit arithmetic) against the oracle's FP64 apply: the input is rounded to FP32x2 (2^-49
    relative per component) and every product and sum is error-free up to the low parts, so
    the result sits within a few hundred units of 2^-48 of the FP64 one."""
    name, m, ctx, ref = pair
    x = rvec(m.lunk + 1, 5)
    y = ctx.calc_ax_fp32x2(x)
    y_ref = ref.calc_ax(x)
    err = np.linalg.norm(y - y_ref) / np.linalg.norm(y_ref)
    assert err <= 1e-12, (name, err)
    assert abs(y[-1] - y_ref[-1]) <= 1e-12 * abs(y_ref[-1])


@pytest.mark.parametrize("precond", [True, False], ids=["preconditioned", "plain"])
def test_inner_operator_fp32x2_matches_fp64(pair, precond):
    """The operator the mixed-precision inner solves iterate with (the regularised operator,
    rows scaled by the inner preconditioner) in packed FP32x2 against the same operator in
    FP64: the Hermitian-part reads of the RDO block, the regularising blocks and the row
    scaling, which the plain apply does not exercise."""
    name, m, ctx, ref = pair
    x = rvec(m.lunk + 1, 6)
    y64 = ctx.calc_ax_inner(x, heomq.PREC_FP64_REFINED, precond)
    ydf = ctx.calc_ax_inner(x, heomq.PREC_MIXED, precond)
    err = np.linalg.norm(ydf - y64) / np.linalg.norm(y64)
    assert err <= 1e-12, (name, err)
    nz0 = int(m.array("nnz_spa")[0])
    rdo = np.linalg.norm(ydf[:nz0] - y64[:nz0]) / np.linalg.norm(y64[:nz0])
    assert rdo <= 1e-12, (name, rdo)
    assert abs(ydf[-1] - y64[-1]) <= 1e-12 * abs(y64[-1])
