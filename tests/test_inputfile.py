"""The reference's input file and state files (host only).

The input text below follows the reference's positional records
(main/evaluatepara.f90:71-84) and namelist groups; the tables built from it must equal
those of the same model configured directly."""
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


def test_unsupported_options_are_refused():
    with pytest.raises(ValueError):
        inp.to_config(SIAM_INPUT.replace("psdjob=T", "psdjob=F psfjob=T"))
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
