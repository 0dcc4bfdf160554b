"""The reference's input file and state files (host only).

The input text below follows the reference's positional records
(main/evaluatepara.f90:71-84) and namelist groups; the tables built from it must equal
those of the same model configured directly."""
import struct

import numpy as np
import pytest

import configs as cf
import heomq
from heomq import inputfile as inp

SIAM_INPUT = """2          ! init: steady state
4          ! ntier = truncation tier + 1
4          ! nmats
1          ! norbs
2          ! nspin
2          ! nalf
10.d0 10.d0
0.5 0.5
0.1 0.1
0.2 0.2 -0.2 -0.2
0.0
0.05
$jobinfo lsparse=T psdjob=T $end
$method methodss=2 $end
$converge crit=1.d-10 maxit0=40000 $end
$para1 eup=-1.d0 edown=-1.d0 uu=2.d0 $end
$field fieldtype=0 $end
0.0 0.0 0.0 0.0
"""

TABLES = ["nfirst", "nlast", "indextable", "index_coef_ref", "indexcoef", "itypecoef", "ifactfcoef", "ifactrcoef",
          "nnz_spa", "ind_spa", "irow_spa", "icol_spa"]


def _same_tables(a, b):
    assert (a.lunk, a.nunk, a.lall, a.nrho) == (b.lunk, b.nunk, b.lall, b.nrho)
    for name in TABLES:
        np.testing.assert_array_equal(a.array(name), b.array(name))
    for name in ("cb", "cd", "cgamma", "hs", "eleadinfty"):
        np.testing.assert_allclose(a.array(name), b.array(name), rtol=1e-14, atol=0)


def test_reference_style_input_builds_the_same_model():
    m, opts = inp.model_from_input(SIAM_INPUT)
    _same_tables(m, heomq.Model(cf.siam(ntier=4, nmats=4, V=0.4)))
    assert opts["crit"] == 1e-10 and opts["maxit0"] == 40000 and opts["init"] == 2


def test_repeat_counts_and_continued_records():
    text = SIAM_INPUT.replace("10.d0 10.d0", "2*10.0").replace("0.2 0.2 -0.2 -0.2", "0.2 0.2\n-0.2 -0.2")
    pos, groups, tchar = inp.parse(text)
    assert pos["bandwidth"] == [10.0, 10.0]
    assert pos["engyshift"] == [[0.2, 0.2], [-0.2, -0.2]]
    assert groups["para1"]["uu"] == 2.0 and groups["jobinfo"]["lsparse"] is True
    assert tchar == [[0.0, 0.0], [0.0, 0.0]]


@pytest.mark.parametrize("cfg", [cf.siam(ntier=3, nmats=2, V=0.6), cf.dqd(ntier=3, nmats=2)], ids=["siam", "dqd"])
def test_written_input_round_trips(cfg):
    text = inp.write_input(cfg, crit=1e-9)
    m, opts = inp.model_from_input(text)
    _same_tables(m, heomq.Model(cfg))
    assert opts["crit"] == 1e-9


def test_hamiltonian_file_path(tmp_path):
    cfg = cf.hund(ntier=2, nmats=2)
    ref = heomq.Model(cfg)
    hs = ref.get("hs", ref.nrho ** 2, np.complex128).reshape(ref.nrho, ref.nrho, order="F")
    path = tmp_path / "hamil_sys.data"
    inp.write_hamil_sys(path, hs)
    hs2 = inp.read_hamil_sys(path, ref.nrho)
    np.testing.assert_array_equal(hs, hs2)
    text = inp.write_input(dict(cfg, model=9))
    m, _ = inp.model_from_input(text, hamil_sys=hs2)
    _same_tables(m, ref)


def test_state_file_round_trip_and_layout(tmp_path):
    m = heomq.Model(cf.siam(ntier=3, nmats=2))
    rng = np.random.default_rng(3)
    rho = rng.standard_normal(m.lunk) + 1j * rng.standard_normal(m.lunk)
    path = tmp_path / "rho_spa.st"
    inp.write_rho_spa(path, m, rho)
    raw = path.read_bytes()
    assert len(raw) == 20 + 8 + 16 * m.lunk
    assert np.frombuffer(raw[:20], dtype="<i4").tolist() == [m.norbs, m.nspin, m.ncor, m.ntier, m.nalf]
    assert np.frombuffer(raw[20:28], dtype="<i8")[0] == m.nunk
    np.testing.assert_array_equal(inp.read_rho_spa(path, m), rho)


def test_lower_tier_state_seeds_a_higher_tier_job(tmp_path):
    low = heomq.Model(cf.siam(ntier=3, nmats=2))
    high = heomq.Model(cf.siam(ntier=4, nmats=2))
    rho = low.initial_guess() + 0.01
    path = tmp_path / "rho_spa.sav"
    inp.write_rho_spa(path, low, rho)
    seeded = inp.read_rho_spa(path, high)
    np.testing.assert_array_equal(seeded[: low.lunk], rho)
    assert not np.any(seeded[low.lunk:])


def test_prony_job_reads_the_callers_table():
    """$jobinfo psfjob = T itype_psf = 3: the fitted table of that type comes from the caller
    (the reference's built-in tables are not part of the library); without it the job is
    refused.  Restating the input's own Pade decomposition as a Prony table gives the Pade
    job's coefficient tables to rounding."""
    text = SIAM_INPUT.replace("psdjob=T", "psdjob=F psfjob=T itype_psf=3")
    with pytest.raises(ValueError):
        inp.to_config(text)
    tab = heomq.psf_table_from_pade(4, 10.0, 0.1, tpsf=1.5)
    m, _ = inp.model_from_input(text, psf_tables={3: tab})
    ref, _ = inp.model_from_input(SIAM_INPUT)
    for k in ("cb", "cd", "cgamma"):
        assert np.abs(m.array(k) - ref.array(k)).max() <= 1e-13 * np.abs(ref.array(k)).max(), k
    for k in TABLES:
        np.testing.assert_array_equal(m.array(k), ref.array(k), err_msg=k)


def test_unsupported_options_are_refused():
    with pytest.raises(ValueError):
        inp.to_config(SIAM_INPUT.replace("psdjob=T", "psdjob=F pfdjob=T"))
    with pytest.raises(ValueError):
        inp.to_config(SIAM_INPUT.replace("methodss=2", "methodss=0"))
    with pytest.raises(ValueError):
        inp.to_config(SIAM_INPUT.replace("$field fieldtype=0", "$field fieldtype=1"))


def test_resume_tape_round_trip_and_layout(tmp_path):
    m = heomq.Model(cf.siam(ntier=3, nmats=2))
    rng = np.random.default_rng(5)
    rho = rng.standard_normal(m.lunk) + 1j * rng.standard_normal(m.lunk)
    path = tmp_path / "TAPE_3.resume"
    inp.write_tape(path, m, 12.5, rho)
    raw = path.read_bytes()
    assert len(raw) == 8 + 24 + 8 + 4 + 8 + 16 * m.lunk
    assert np.frombuffer(raw[:8], dtype="<f8")[0] == 12.5
    assert np.frombuffer(raw[8:32], dtype="<i4").tolist() == [m.ntier, m.norbs, m.nspin, m.ncor, m.nalf, 0]
    assert np.frombuffer(raw[32:40], dtype="<i8")[0] == m.nunk
    assert np.frombuffer(raw[44:52], dtype="<i8")[0] == m.lunk
    t, back = inp.read_tape(path, m)
    assert t == 12.5
    np.testing.assert_array_equal(back, rho)
    other = heomq.Model(cf.siam(ntier=4, nmats=2))
    with pytest.raises(ValueError):
        inp.read_tape(path, other)


@pytest.mark.parametrize("cfg", [cf.siam(ntier=3), cf.dqd(ntier=3)], ids=["siam", "dqd_lscreen"])
def test_cached_tables_round_trip_and_layout(tmp_path, cfg):
    """coefindex.data / auxindex.data (main/buildcoefindex.f90:683-709) and sparse_index.data /
    sparse_info.data (fermion/prelude_spa.f90:798-820): written in the reference's stream
    layout, read back through the reference's compatibility checks, equal to the tables."""
    m = heomq.Model(cfg)
    ci, ai = tmp_path / "coefindex.data", tmp_path / "auxindex.data"
    si, sf = tmp_path / "sparse_index.data", tmp_path / "sparse_info.data"
    inp.write_coefindex(ci, m)
    inp.write_auxindex(ai, m)
    inp.write_sparse(si, sf, m)
    # byte counts of the streams
    nh = int((np.abs(inp.exp_hs(m)) >= 1e-32).sum())
    assert ci.stat().st_size == 36 + 28 + 12 + 4 + 8 + 4 + 12 + 8 + 11 * m.lall
    assert ai.stat().st_size == 8 + 8 * m.nunk
    assert si.stat().st_size == 36 + 28 + 16 + 4 + 24 * nh + 12 * m.nunk
    assert sf.stat().st_size == 28 + 8 + 8 * m.lunk
    raw = ci.read_bytes()
    assert struct.unpack("<9i", raw[:36]) == (m.ntier, m.ncor, m.norbs, m.nspin, m.nalf, 0, m.ntier, 0, 0)
    assert struct.unpack("<i", raw[36 + 28 + 12 + 4 + 8:36 + 28 + 12 + 4 + 8 + 4])[0] == (-1 if cfg.get("lscreen") else 0)
    coef = inp.read_coefindex(ci, m)
    for k in ("indexcoef", "itypecoef", "ifactfcoef", "ifactrcoef"):
        np.testing.assert_array_equal(coef[k], m.array(k))
    np.testing.assert_array_equal(inp.read_auxindex(ai, m), m.array("index_coef_ref"))
    sp = inp.read_sparse(si, sf, m)
    assert sp["lunk"] == m.lunk
    for k in ("nnz_spa", "ind_spa", "irow_spa", "icol_spa"):
        np.testing.assert_array_equal(sp[k], m.array(k))


def test_cached_tables_of_another_job_are_refused(tmp_path):
    m3, m4 = heomq.Model(cf.siam(ntier=3)), heomq.Model(cf.siam(ntier=4))
    inp.write_coefindex(tmp_path / "c", m3)
    inp.write_auxindex(tmp_path / "a", m3)
    inp.write_sparse(tmp_path / "i", tmp_path / "f", m3)
    with pytest.raises(ValueError, match="incompatible"):
        inp.read_coefindex(tmp_path / "c", m4)
    with pytest.raises(ValueError, match="auxindex"):
        inp.read_auxindex(tmp_path / "a", m4)
    with pytest.raises(ValueError, match="incompatible"):
        inp.read_sparse(tmp_path / "i", tmp_path / "f", m4)
    # same sizes, different Hamiltonian sparsity: the cached exp(0.314 H) does not match
    md = heomq.Model(cf.dqd(ntier=3, t=0.0))
    mt = heomq.Model(cf.dqd(ntier=3, t=0.5))
    inp.write_sparse(tmp_path / "i2", tmp_path / "f2", md)
    with pytest.raises(ValueError, match="sparsity"):
        inp.read_sparse(tmp_path / "i2", tmp_path / "f2", mt)
