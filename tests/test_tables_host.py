"""Host-side set-up of the product against the oracle (no GPU needed).

The ADO index tables (ball2drawer / buildcoefindex / findhighertier / findlowertier,
main/buildcoefindex.f90:192-362) and the sparse patterns (fermion/prelude_spa.f90:146-747)
built by the product's C++ host code must equal the oracle's bit for bit; bath
coefficients and H (main/evaluatepara.f90:1897-2020, main/calchs.f90) agree to rounding,
since the two use different eigensolvers for the Pade poles.
"""
from math import comb

import numpy as np
import pytest

import configs as cf
import heomq
import oracle_ffi as of

CASES = {
    "siam_L2": cf.siam(ntier=3, nmats=4),
    "siam_L3": cf.CFG0,
    "dqd_L2": cf.dqd(ntier=3),
    "hund_L1": cf.hund(ntier=2, nmats=2),
}

INT_TABLES = ["nfirst", "nlast", "indextable", "index_coef_ref", "indexcoef", "itypecoef", "ifactfcoef",
              "ifactrcoef", "nnz_spa", "ind_spa", "irow_spa", "icol_spa", "rowams", "colams", "sgnams",
              "mpm", "morbs", "mspin", "ilead", "mcor", "indexdraw"]
FLOAT_TABLES = ["cb", "cd", "cgamma", "dipm", "hs"]


@pytest.fixture(scope="module", params=sorted(CASES))
def pair(request):
    cfg = CASES[request.param]
    return heomq.Model(cfg), of.Model(cfg)


def test_sizes(pair):
    p, o = pair
    assert (p.lunk, p.nunk, p.lall, p.nrho) == (o.lunk, o.nunk, o.lall, o.nrho)


@pytest.mark.parametrize("name", INT_TABLES)
def test_integer_tables_bit_exact(pair, name):
    p, o = pair
    a = p.array(name)
    b = o.get(name)[: a.size]
    assert a.size == b.size
    np.testing.assert_array_equal(a.astype(np.int64), b.astype(np.int64))


@pytest.mark.parametrize("name", FLOAT_TABLES)
def test_coefficients(pair, name):
    p, o = pair
    a = p.array(name)
    b = o.get(name)[: a.size]
    scale = max(np.max(np.abs(b)), 1e-300)
    assert np.max(np.abs(a - b)) <= 1e-12 * scale


def test_lead_shift_at_infinity(pair):
    """eleadinfty(ialf, ispin), column-major in the product; [alf][spin] in the oracle."""
    p, o = pair
    a = p.array("eleadinfty").reshape(p.nspin, p.nalf).T
    b = o.get("eleadinfty").reshape(of.MAXALF, 2)[: p.nalf, : p.nspin]
    np.testing.assert_allclose(a, b, rtol=1e-14, atol=0)


def closed_form_tier_counts(nsgn_ops, ncor, ntier):
    """ADOs per tier as ball2drawer enumerates them (main/ball2drawer.f90:26-257): multisets
    of operators (sigma, spin, orbital, lead), each operator copy carrying a memory index
    k with non-decreasing k for equal operators, one representative per pair related by
    Hermitian conjugation (sigma -> -sigma on every operator, the jredex map)."""
    from itertools import combinations_with_replacement
    from collections import Counter

    ops = list(range(nsgn_ops))
    half = nsgn_ops // 2
    conj = lambda o: (o + half) % nsgn_ops
    out = [1]
    for n in range(1, ntier):
        seen, total = set(), 0
        for ms in combinations_with_replacement(ops, n):
            key = min(ms, tuple(sorted(conj(o) for o in ms)))
            if key in seen:
                continue
            seen.add(key)
            w = 1
            for mult in Counter(ms).values():
                w *= comb(ncor + mult - 1, mult)
            total += w
        out.append(total)
    return out


@pytest.mark.parametrize("cfg, nops", [(cf.CFG0, 8), (cf.siam(ntier=5, nmats=2), 8), (cf.hund(ntier=3, nmats=6), 24)],
                         ids=["siam_L3", "siam_L4", "hund_L2"])
def test_ado_count_closed_form(cfg, nops):
    """Tier sizes against the closed form (operators = 2 signs x spins x orbitals x leads)."""
    m = heomq.Model(cfg)
    nf, nl = m.array("nfirst"), m.array("nlast")
    got = [int(nl[k] - nf[k] + 1) for k in range(m.ntier)]
    assert got == closed_form_tier_counts(nops, m.ncor, m.ntier)
    if cfg is cf.CFG0:
        assert got == [1, 20, 460, 5740]


def test_coupling_rows_link_neighbouring_tiers():
    """index_coef_ref holds 1-based row starts; row n (n >= 1) lists its n lower-tier
    couplings (findlowertier) and then its higher-tier ones (findhighertier).  A direct
    coupling (itypecoef = 0) n -> m is matched by a direct coupling m -> n; a conjugate
    one (itypecoef = 1) targets the conjugation-class representative instead.  The RDO
    has no row: its tier-1 couplings are addressed through indexdraw
    (calc_ax_tfqmr_spa_omp.f90:136-205)."""
    m = heomq.Model(cf.siam(ntier=4, nmats=2))
    ref = m.array("index_coef_ref")
    idx = m.array("indexcoef")
    ity = m.array("itypecoef")
    nf, nl = m.array("nfirst"), m.array("nlast")
    tier = np.zeros(m.nunk, dtype=np.int64)
    for k in range(m.ntier):
        tier[nf[k] - 1: nl[k]] = k
    start = ref - 1
    end = np.append(ref[1:] - 1, m.lall)
    assert ref[0] == 0 and ref[1] == 1
    rows = [set()] + [set(idx[start[n]: end[n]].tolist()) for n in range(1, m.nunk)]
    direct = 0
    for n in range(1, m.nunk):
        t = tier[idx[start[n]: end[n]] - 1]
        assert np.all(t[: tier[n]] == tier[n] - 1)
        assert np.all(t[tier[n]:] == tier[n] + 1)
        for j in range(start[n], end[n]):
            tgt = idx[j] - 1
            if tgt > 0 and ity[j] == 0:
                assert n + 1 in rows[tgt]
                direct += 1
    assert direct > 0


@pytest.mark.parametrize("cfg, nunk, lall", [
    (cf.siam(ntier=3, nmats=4), 481, None),
    (cf.CFG0, 6221, 37360),
    (cf.siam(ntier=5, nmats=4), 70251, 523080),
    (cf.CFG1, 30453, 223904),
    (cf.CFG4, 7477, 28980),
], ids=["siam_L2", "siam_L3", "siam_L4", "dqd_L4", "hund_L2"])
def test_stored_sizes_match_an_independent_count(cfg, nunk, lall):
    """Stored ADO and coupling-entry counts of the reference's table rules, as counted by
    a separate restatement of ball2drawer / buildcoefindex (Hermitian-conjugate halves
    kept once, repeated drawers kept, lscreen dropping decoupled operators)."""
    m = heomq.Model(cfg)
    assert m.nunk == nunk
    if lall is not None:
        assert m.lall == lall


@pytest.mark.parametrize("spin", [1, 2])
def test_correlation_function_pattern_bit_exact(pair, spin):
    """corrfunc/prelude_cf_spa.f90:146-760: the library's structural propagation from the
    seed E0 (a + a^dag) E0 against the oracle's random-coefficient products."""
    p, o = pair
    for iorbs in range(1, p.norbs + 1):
        a = p.cf_pattern(iorbs, spin)
        c = of.CF(o, iorbs, spin)
        assert a["lunkcf_spa"] == c.lunkcf
        for k in ("nnzcf_spa", "indcf_spa", "irowcf_spa", "icolcf_spa"):
            np.testing.assert_array_equal(a[k].astype(np.int64), c.get(k).astype(np.int64))


def test_correlation_function_pattern_rejects_a_bad_spin_orbital(pair):
    p, _ = pair
    with pytest.raises(heomq.HeomError):
        p.cf_pattern(p.norbs + 1, 1)


def test_initial_guess_matches_oracle(pair):
    """heom_model_initial_guess (main/analyze_hs.f90:144-283 + fermion/initialize1_spa.f90:32-236)
    against orc_initial_guess: the Boltzmann RDO at the lead-1 temperature on the RDO pattern,
    every ADO zero.  The two diagonalise H with different eigensolvers, so the entries agree
    to rounding; the ADO part is exactly zero in both."""
    p, o = pair
    g, h = p.initial_guess(), o.initial_guess()
    nz = int(o.get("nnz_spa")[0])
    assert g.shape == h.shape
    np.testing.assert_allclose(g[:nz], h[:nz], rtol=0, atol=1e-12)
    assert not np.any(g[nz:]) and not np.any(h[nz:])
    assert abs(sum(g[q] for q in range(nz) if p.array("irow_spa")[q] == p.array("icol_spa")[q]) - 1) < 1e-12
