"""The reference's input file and its sparse state files, for drop-in workflows.

Input file (read on unit 5 by the reference):
- 12 list-directed records in the order of main/evaluatepara.f90:71-84:
  init, ntier, nmats, norbs, nspin, nalf, bandwidth(nalf), linewidth(norbs, per lead),
  temperature(nalf), engyshift(nspin, per lead), tmax, dt;
- Fortran namelist groups anywhere after them ($name ... $end or &name ... /), each read by
  name (main/main.f90:119-147, main/calchs.f90:17-27, main/evaluatepara.f90:27-28);
- after the $field group, the record of tchar(nspin, per lead) for fieldtype 0
  (main/evaluatepara.f90:2299-2330).

Supported subset: the Lorentzian PSD sparse path (psdjob = T, lsparse = T, methodss = 2,
fieldtype = 0) with $para1 (one orbital), $para4 (two orbitals, $ddots), or
$hamil_sys lreadhs = T (H from hamil_sys.data, internal units).  Anything else raises.

State files (Intel form='binary', i.e. raw streams without record markers; TAPE_n.resume
of a time propagation in write_tape / read_tape):
  rho_spa.st / .gr / .sav / .chk : int32 norbs, nspin, ncor, ntier0, nalf; int64 nunk;
                                   then the nnz_spa(n) complex128 entries of every ADO n with
                                   entries, in ADO order (main/main.f90:1087-1105,
                                   fermion/initialize2_spa.f90:24-110).
hamil_sys.data (form='unformatted', sequential): one record of nrho^2 complex128, column-major
                                   (main/calchs.f90:78-82).

Cached tables (raw streams; logicals 4 bytes, .true. = -1 as Intel writes them):
  coefindex.data, auxindex.data       : the coupling tables (main/buildcoefindex.f90:683-709)
  sparse_index.data, sparse_info.data : the per-ADO patterns (fermion/prelude_spa.f90:798-820)
The readers apply the reference's compatibility checks before the data are used.
"""
import re
import struct

import numpy as np

from . import models

_NUM = re.compile(r"^[+-]?(\d+\.?\d*|\.\d+)([eEdD][+-]?\d+)?$")


def _value(tok):
    t = tok.strip().strip(",")
    low = t.lower()
    if low in (".true.", "t", ".t.", "true"):
        return True
    if low in (".false.", "f", ".f.", "false"):
        return False
    if len(t) >= 2 and t[0] == t[-1] and t[0] in "'\"":
        return t[1:-1]
    if _NUM.match(t):
        v = float(t.replace("d", "e").replace("D", "e"))
        return int(v) if re.match(r"^[+-]?\d+$", t) else v
    raise ValueError(f"cannot read value {tok!r}")


def _tokens(line):
    """List-directed items of one record (r*value repeats expanded; '!' starts a comment)."""
    line = line.split("!")[0]
    out = []
    for tok in re.split(r"[\s,]+", line.strip()):
        if not tok:
            continue
        m = re.match(r"^(\d+)\*(.+)$", tok)
        if m:
            out += [m.group(2)] * int(m.group(1))
        else:
            out.append(tok)
    return out


def _namelists(text):
    groups = {}
    for m in re.finditer(r"[$&](\w+)(.*?)(?:[$&]end\b|/)", text, re.S | re.I):
        name, body = m.group(1).lower(), m.group(2)
        if name == "end":
            continue
        vals = {}
        for a in re.finditer(r"(\w+)\s*=\s*('[^']*'|\"[^\"]*\"|[^\s,=]+)", body):
            vals[a.group(1).lower()] = _value(a.group(2))
        groups[name] = vals
    return groups


def parse(text):
    """The positional records, the namelist groups and the record after $field."""
    lines = text.splitlines()
    pos = {}
    li = 0

    def read(count):
        nonlocal li
        vals = []
        while len(vals) < count:
            if li >= len(lines):
                raise ValueError("input file ends inside the positional records")
            toks = _tokens(lines[li])
            li += 1
            vals += [_value(t) for t in toks]
        return vals[:count]

    for key in ("init", "ntier", "nmats", "norbs", "nspin", "nalf"):
        pos[key] = int(read(1)[0])
    nalf, norbs, nspin = pos["nalf"], pos["norbs"], pos["nspin"]
    pos["bandwidth"] = [float(v) for v in read(nalf)]
    lw = read(nalf * norbs)
    pos["linewidth"] = [[float(v) for v in lw[a * norbs:(a + 1) * norbs]] for a in range(nalf)]
    pos["temperature"] = [float(v) for v in read(nalf)]
    es = read(nalf * nspin)
    pos["engyshift"] = [[float(v) for v in es[a * nspin:(a + 1) * nspin]] for a in range(nalf)]
    pos["tmax"] = float(read(1)[0])
    pos["dt"] = float(read(1)[0])
    rest = "\n".join(lines[li:])
    groups = _namelists(rest)
    tchar = None
    m = re.search(r"[$&]field\b.*?(?:[$&]end\b|/)[^\n]*\n(.*)", rest, re.S | re.I)
    if m:
        after = m.group(1).splitlines()
        toks = []
        for ln in after:
            toks += _tokens(ln)
            if len(toks) >= nalf * nspin:
                break
        if len(toks) >= nalf * nspin:
            vals = [float(_value(t)) for t in toks[: nalf * nspin]]
            tchar = [[vals[a * nspin + s] for s in range(nspin)] for a in range(nalf)]
    return pos, groups, tchar


def to_config(text, hamil_sys=None, psf_tables=None):
    """Model configuration (heomq.Model argument) and solver options of an input file.
    hamil_sys: H (nrho x nrho, internal units) when $hamil_sys lreadhs = T.
    psf_tables: for $jobinfo psfjob = T, the fitted Prony tables by itype_psf ({itype: {"coef",
    "pole", "tpsf", "rpsf"}}, the contents of main/zpout_psf.f90's tables); the reference's own
    tables are not part of this library."""
    pos, g, tchar = parse(text)
    job = g.get("jobinfo", {})
    if not job.get("lsparse", False):
        raise ValueError("only the sparse path (lsparse = T) is supported")
    psf = None
    if job.get("psfjob", False):
        itype = int(job.get("itype_psf", 1))                       # main/main.f90:177 default
        if not psf_tables or itype not in psf_tables:
            raise ValueError(f"psfjob = T needs the fitted Prony table itype_psf = {itype} (psf_tables)")
        psf = psf_tables[itype]
    elif not job.get("psdjob", False):
        raise ValueError("only the Pade (psdjob = T) and Prony (psfjob = T) decompositions are supported")
    for flag in ("mfdjob", "pfdjob", "psdlor", "psdfff", "lsimple", "ltrun_der"):
        if job.get(flag, False):
            raise ValueError(f"{flag} = T is not supported")
    if g.get("adiabatic", {}).get("lad", False):
        raise ValueError("lad = T is not supported")
    if g.get("method", {}).get("methodss", 2) != 2:
        raise ValueError("only methodss = 2 (TFQMR) is supported")
    if g.get("field", {}).get("fieldtype", 0) != 0:
        raise ValueError("only fieldtype = 0 is supported")
    cfg = dict(norbs=pos["norbs"], nspin=pos["nspin"], nalf=pos["nalf"], nmats=pos["nmats"], ntier=pos["ntier"],
               bandwidth=pos["bandwidth"], linewidth=pos["linewidth"], temperature=pos["temperature"],
               engyshift=pos["engyshift"], lscreen=int(bool(job.get("lscreen", False))),
               doubledot=int(bool(g.get("ddots", {}).get("doubledot", False))),
               tchar=(tchar if tchar else 0.0))
    if psf is not None:
        cfg["psf"] = psf
        cfg["nmats"] = len(psf["coef"])
    hs = None
    if g.get("hamil_sys", {}).get("lreadhs", False):
        if hamil_sys is None:
            raise ValueError("lreadhs = T needs the hamil_sys.data matrix")
        hs = np.asarray(hamil_sys, dtype=np.complex128)
        cfg["model"] = 9
    elif pos["norbs"] == 1 and pos["nspin"] == 2:
        p = g.get("para1", {})
        cfg.update(model=1, eup=p.get("eup", 0.0), edown=p.get("edown", 0.0), uu=p.get("uu", 0.0))
    elif pos["norbs"] == 2 and pos["nspin"] == 2:
        p = g.get("para4", {})
        cfg.update(model=4, **{k: float(p.get(k, 0.0)) for k in ("e1up", "e1down", "e2up", "e2down", "uu1", "uu2",
                                                                  "u12", "t12")})
    else:
        raise ValueError("this orbital/spin count needs $hamil_sys lreadhs = T")
    conv = g.get("converge", {})
    opts = dict(init=pos["init"], crit=float(conv.get("crit", 1e-8)), maxit0=int(conv.get("maxit0", 20000)),
                tmax=pos["tmax"], dt=pos["dt"])
    return cfg, hs, opts


def model_from_input(text, hamil_sys=None, psf_tables=None):
    """heomq.Model of an input file, with its solver options."""
    from . import Model

    cfg, hs, opts = to_config(text, hamil_sys, psf_tables)
    return Model(cfg, hs=hs), opts


# ---- state files -----------------------------------------------------------------
def write_rho_spa(path, model, rho):
    """rho_spa.st layout: header, then the entries of every ADO in ADO order."""
    rho = np.ascontiguousarray(rho, dtype=np.complex128)
    if rho.size != model.lunk:
        raise ValueError("rho must hold lunk entries")
    with open(path, "wb") as f:
        f.write(struct.pack("<5i", model.norbs, model.nspin, model.ncor, model.ntier, model.nalf))
        f.write(struct.pack("<q", model.nunk))
        f.write(rho.tobytes())


def read_rho_spa(path, model):
    """A saved state as the initial guess of `model` (fermion/initialize2_spa.f90 without the
    changed-pattern branch): header fields must match; a state saved at a lower tier fills the
    ADOs it holds and leaves the rest zero."""
    with open(path, "rb") as f:
        norbs, nspin, ncor, jtier, nalf = struct.unpack("<5i", f.read(20))
        (nunk_saved,) = struct.unpack("<q", f.read(8))
        data = np.frombuffer(f.read(), dtype=np.complex128)
    if (norbs, nspin, ncor, nalf) != (model.norbs, model.nspin, model.ncor, model.nalf) or jtier <= 1:
        raise ValueError("state file does not match the model (norbs, nspin, ncor, nalf)")
    nnz = model.array("nnz_spa").astype(np.int64)
    if jtier >= model.ntier and nunk_saved != model.nunk:
        raise ValueError("incompatible state file: ADO count differs")
    count = int(nnz[: min(nunk_saved, model.nunk)].sum())
    if data.size < count:
        raise ValueError("state file is truncated")
    rho = np.zeros(model.lunk, dtype=np.complex128)
    rho[:count] = data[:count]
    return rho


def write_tape(path, model, t, rho):
    """Resume tape of a time propagation (td/resumejob.f90:83-105, sparse mode, no heat bath):
    float64 t; int32 ntier, norbs, nspin, ncor, nalf, numfff (0 without psdfff); int64 nunk;
    int32 lhb (0); int64 lunk; then the lunk complex128 entries."""
    rho = np.ascontiguousarray(rho, dtype=np.complex128)
    if rho.size != model.lunk:
        raise ValueError("rho must hold lunk entries")
    with open(path, "wb") as f:
        f.write(struct.pack("<d", float(t)))
        f.write(struct.pack("<6i", model.ntier, model.norbs, model.nspin, model.ncor, model.nalf, 0))
        f.write(struct.pack("<q", model.nunk))
        f.write(struct.pack("<i", 0))
        f.write(struct.pack("<q", model.lunk))
        f.write(rho.tobytes())


def read_tape(path, model):
    """(t, rho) from a resume tape written for `model` (td/resumejob.f90:17-70): every header
    field must match, as in the reference, and tapes with heat-bath data are refused."""
    with open(path, "rb") as f:
        (t,) = struct.unpack("<d", f.read(8))
        head = struct.unpack("<6i", f.read(24))
        (nunk,) = struct.unpack("<q", f.read(8))
        (lhb,) = struct.unpack("<i", f.read(4))
        if lhb:
            raise ValueError("resume tape carries heat-bath data (lhb = T), which is not supported")
        (lunk,) = struct.unpack("<q", f.read(8))
        data = np.frombuffer(f.read(16 * lunk), dtype=np.complex128)
    if head != (model.ntier, model.norbs, model.nspin, model.ncor, model.nalf, 0):
        raise ValueError(f"resume tape does not match the model: {head}")
    if nunk != model.nunk or lunk != model.lunk or data.size != lunk:
        raise ValueError("resume tape does not match the model's ADO count or stored entries")
    return t, data.copy()


# ---- cached tables (Intel form='binary': raw streams; logical = 4 bytes, .true. = -1) ----
_TRUE, _FALSE = -1, 0
_COEF_REC = np.dtype([("indexcoef", "<i8"), ("itypecoef", "i1"), ("ifactfcoef", "i1"), ("ifactrcoef", "i1")])
_HSYS_REC = np.dtype([("irow", "<i4"), ("icol", "<i4"), ("cval", "<c16")])
_NNZ_REC = np.dtype([("nnz_spa", "<i4"), ("ind_spa", "<i8")])
_RC_REC = np.dtype([("irow", "<i4"), ("icol", "<i4")])


def _lg(v):
    return _TRUE if v else _FALSE


def _truth(v):
    """Intel's test of a logical: the low bit."""
    return bool(v & 1)


def _head9(model):
    # ntier, ncor, norbs, nspin, nalf, numfff, ntier0, ndrawer_slow, ncor_slow (lad = F, no psdfff)
    return (model.ntier, model.ncor, model.norbs, model.nspin, model.nalf, 0, model.ntier, 0, 0)


def _lscreen(model):
    return bool(model.tables.lscreen)


def write_coefindex(path, model):
    """coefindex.data (main/buildcoefindex.f90:683-698): the job flags the reader checks, with
    the reference's defaults for the options outside the supported subset (lad, lfilter,
    ltrun_der, lsimple, lomit all F; lwalf T), then lall records of indexcoef (int64),
    itypecoef, ifactfcoef, ifactrcoef (int8)."""
    rec = np.zeros(model.lall, dtype=_COEF_REC)
    rec["indexcoef"] = model.array("indexcoef")
    rec["itypecoef"] = model.array("itypecoef")
    rec["ifactfcoef"] = model.array("ifactfcoef")
    rec["ifactrcoef"] = model.array("ifactrcoef")
    with open(path, "wb") as f:
        f.write(struct.pack("<9i", *_head9(model)))
        f.write(struct.pack("<3i2id", _lg(False), _lg(True), _lg(True), 1, 2, 0.9))   # lad, lad_fast, lset_fast, idegen_fast, ndegen_fast, dratio_fast
        f.write(struct.pack("<3i", _lg(False), 2, 3))                                 # lfilter, nfilter_count, nfilter_long
        f.write(struct.pack("<i", _lg(False)))                                        # ltrun_der
        f.write(struct.pack("<2i", _lg(False), _lg(True)))                            # lsimple, lwalf
        f.write(struct.pack("<i", _lg(_lscreen(model))))                              # lscreen
        f.write(struct.pack("<id", _lg(False), 4e-6))                                 # lomit, dfact_omit
        f.write(struct.pack("<q", model.lall))
        f.write(rec.tobytes())


def read_coefindex(path, model):
    """The coupling table of a coefindex.data file, with the reader's compatibility checks
    (main/buildcoefindex.f90:44-159): the nine sizes, then lad, lfilter, ltrun_der, lsimple and
    lwalf, lscreen and lomit must agree with the job.  Returns a dict of the four arrays."""
    with open(path, "rb") as f:
        head = struct.unpack("<9i", f.read(36))
        if head != _head9(model):
            raise ValueError(f"coefindex.data incompatible: sizes {head}")
        lad, _, _, _, _, _ = struct.unpack("<3i2id", f.read(28))
        lfilter, _, _ = struct.unpack("<3i", f.read(12))
        (ltrun_der,) = struct.unpack("<i", f.read(4))
        lsimple, lwalf = struct.unpack("<2i", f.read(8))
        (lscreen,) = struct.unpack("<i", f.read(4))
        lomit, _ = struct.unpack("<id", f.read(12))
        if _truth(lad) or _truth(lfilter) or _truth(ltrun_der) or _truth(lsimple) or not _truth(lwalf) or _truth(lomit):
            raise ValueError("coefindex.data written for options outside the supported subset")
        if _truth(lscreen) != _lscreen(model):
            raise ValueError("coefindex.data incompatible: lscreen differs")
        (lall,) = struct.unpack("<q", f.read(8))
        rec = np.frombuffer(f.read(lall * _COEF_REC.itemsize), dtype=_COEF_REC)
    if rec.size != lall:
        raise ValueError("coefindex.data is truncated")
    return {k: rec[k].copy() for k in _COEF_REC.names}


def write_auxindex(path, model):
    """auxindex.data (main/buildcoefindex.f90:700-709, lsimple = F): int64 nunk, then
    index_coef_ref (int64 per ADO)."""
    with open(path, "wb") as f:
        f.write(struct.pack("<q", model.nunk))
        f.write(model.array("index_coef_ref").astype("<i8").tobytes())


def read_auxindex(path, model):
    with open(path, "rb") as f:
        (nunk,) = struct.unpack("<q", f.read(8))
        if nunk != model.nunk:
            raise ValueError(f"auxindex.data: length {nunk}, expected {model.nunk}")
        ref = np.frombuffer(f.read(8 * nunk), dtype="<i8")
    if ref.size != nunk:
        raise ValueError("auxindex.data is truncated")
    return ref.copy()


def exp_hs(model, alpha=0.31415926, kmax=10):
    """E0 = 1 + sum_{k <= kmax} (alpha H)^k / k! (utility/calc_exp_hmat.f90), H in internal units."""
    n = model.nrho
    h = model.array("hs").reshape(n, n, order="F")
    out = np.eye(n, dtype=np.complex128)
    c1 = np.eye(n, dtype=np.complex128)
    f = 1.0
    for k in range(1, kmax + 1):
        f /= k
        c1 = alpha * (c1 @ h)
        out = out + f * c1
    return out


def _sparse_flags(model):
    # nunk, offcor, lequileads, lsimple, lscreen, lproj
    return struct.pack("<q5i", model.nunk, _lg(False), _lg(False), _lg(False), _lg(_lscreen(model)), _lg(False))


def _flags_match(raw, model):
    if len(raw) != 28:
        return False
    nunk, *flags = struct.unpack("<q5i", raw)
    return nunk == model.nunk and [_truth(v) for v in flags] == [False, False, False, _lscreen(model), False]


def write_sparse(index_path, info_path, model):
    """sparse_index.data and sparse_info.data (fermion/prelude_spa.f90:798-820): the sizes and
    job flags, the COO of E0 = exp(0.314 H) (|v| >= 1e-32, column-major, as zmat_dns2coo), the
    (nnz_spa, ind_spa) pairs of every ADO; then lunk and the (irow, icol) pairs of every entry."""
    n = model.nrho
    e0 = exp_hs(model)
    jj, ii = np.nonzero(np.abs(e0.T) >= 1e-32)      # column-major scan
    hs = np.zeros(ii.size, dtype=_HSYS_REC)
    hs["irow"], hs["icol"], hs["cval"] = ii + 1, jj + 1, e0[ii, jj]
    nz = np.zeros(model.nunk, dtype=_NNZ_REC)
    nz["nnz_spa"], nz["ind_spa"] = model.array("nnz_spa"), model.array("ind_spa")
    rc = np.zeros(model.lunk, dtype=_RC_REC)
    rc["irow"], rc["icol"] = model.array("irow_spa"), model.array("icol_spa")
    with open(index_path, "wb") as f:
        f.write(struct.pack("<9i", *_head9(model)))
        f.write(_sparse_flags(model))
        f.write(struct.pack("<i3i", _lg(False), 1, n, 1))      # lprocc, nproji, nprojf, nprocc
        f.write(struct.pack("<i", ii.size))
        f.write(hs.tobytes())
        f.write(nz.tobytes())
    with open(info_path, "wb") as f:
        f.write(_sparse_flags(model))
        f.write(struct.pack("<q", model.lunk))
        f.write(rc.tobytes())


def read_sparse(index_path, info_path, model):
    """The per-ADO patterns of a sparse_index.data / sparse_info.data pair, reused only when
    the reference would reuse them (fermion/prelude_spa.f90:65-133, 463-510): matching sizes
    and flags, and a cached E0 with the same sparsity as the job's.  Returns a dict of
    nnz_spa, ind_spa, irow_spa, icol_spa and lunk."""
    n = model.nrho
    with open(index_path, "rb") as f:
        head = struct.unpack("<9i", f.read(36))
        if head != _head9(model):
            raise ValueError(f"sparse_index.data incompatible -- 1: {head}")
        if not _flags_match(f.read(28), model):
            raise ValueError("sparse_index.data incompatible -- 2")
        f.read(16)                                              # projection fields (lproj = F)
        (nnz_h,) = struct.unpack("<i", f.read(4))
        if nnz_h <= 0 or nnz_h > n * n:
            raise ValueError(f"error nnz_hsys read from sparse_index.data: {nnz_h}")
        hs = np.frombuffer(f.read(nnz_h * _HSYS_REC.itemsize), dtype=_HSYS_REC)
        nz = np.frombuffer(f.read(model.nunk * _NNZ_REC.itemsize), dtype=_NNZ_REC)
    cached = np.zeros((n, n), dtype=bool)
    cached[hs["irow"] - 1, hs["icol"] - 1] = np.abs(hs["cval"]) >= 1e-32
    if not np.array_equal(cached, np.abs(exp_hs(model)) >= 1e-32):
        raise ValueError("incompatible sparse_index.data: the sparsity of exp(0.314 H) differs")
    if nz.size != model.nunk:
        raise ValueError("sparse_index.data is truncated")
    with open(info_path, "rb") as f:
        if not _flags_match(f.read(28), model):
            raise ValueError("sparse_info.data incompatible -- 1")
        (lunk,) = struct.unpack("<q", f.read(8))
        rc = np.frombuffer(f.read(lunk * _RC_REC.itemsize), dtype=_RC_REC)
    if rc.size != lunk:
        raise ValueError("sparse_info.data is truncated")
    return {"nnz_spa": nz["nnz_spa"].copy(), "ind_spa": nz["ind_spa"].copy(), "irow_spa": rc["irow"].copy(),
            "icol_spa": rc["icol"].copy(), "lunk": lunk}


def write_hamil_sys(path, hs):
    """hamil_sys.data: one sequential unformatted record (4-byte length markers)."""
    h = np.asfortranarray(np.asarray(hs, dtype=np.complex128))
    body = h.reshape(-1, order="F").tobytes()
    with open(path, "wb") as f:
        f.write(struct.pack("<i", len(body)))
        f.write(body)
        f.write(struct.pack("<i", len(body)))


def read_hamil_sys(path, nrho):
    with open(path, "rb") as f:
        (n,) = struct.unpack("<i", f.read(4))
        if n != 16 * nrho * nrho:
            raise ValueError(f"record of {n} bytes, expected {16 * nrho * nrho}")
        body = f.read(n)
        (n2,) = struct.unpack("<i", f.read(4))
    if n2 != n:
        raise ValueError("record markers differ")
    return np.frombuffer(body, dtype=np.complex128).reshape(nrho, nrho, order="F")


def write_input(cfg, crit=1e-8, maxit0=20000, init=2, tmax=0.0, dt=0.05):
    """Input-file text of a model configuration (the inverse of to_config for its subset)."""
    nalf, norbs, nspin = cfg["nalf"], cfg["norbs"], cfg["nspin"]
    lines = [str(init), str(cfg["ntier"]), str(cfg["nmats"]), str(norbs), str(nspin), str(nalf),
             " ".join(repr(float(w)) for w in cfg["bandwidth"][:nalf]),
             " ".join(repr(float(cfg["linewidth"][a][o])) for a in range(nalf) for o in range(norbs)),
             " ".join(repr(float(t)) for t in cfg["temperature"][:nalf]),
             " ".join(repr(float(cfg["engyshift"][a][s])) for a in range(nalf) for s in range(nspin)),
             repr(float(tmax)), repr(float(dt))]
    job = f"$jobinfo lsparse=T psdjob=T lscreen={'T' if cfg.get('lscreen') else 'F'} $end"
    lines += [job, "$method methodss=2 $end", f"$converge crit={crit!r} maxit0={maxit0} $end"]
    if cfg.get("model") == 1:
        lines.append(f"$para1 eup={cfg['eup']!r} edown={cfg['edown']!r} uu={cfg['uu']!r} $end")
    elif cfg.get("model") == 4:
        keys = ("e1up", "e1down", "e2up", "e2down", "uu1", "uu2", "u12", "t12")
        lines.append("$para4 " + " ".join(f"{k}={float(cfg.get(k, 0.0))!r}" for k in keys) + " $end")
        if cfg.get("doubledot"):
            lines.append("$ddots doubledot=T $end")
    else:
        lines.append("$hamil_sys lreadhs=T $end")
    lines.append("$field fieldtype=0 $end")
    tc = cfg.get("tchar", 0.0)
    lines.append(" ".join(repr(float(tc[a][s] if isinstance(tc, (list, tuple)) else tc))
                          for a in range(nalf) for s in range(nspin)))
    return "\n".join(lines) + "\n"


__all__ = ["parse", "to_config", "model_from_input", "write_rho_spa", "read_rho_spa", "write_hamil_sys",
           "read_hamil_sys", "write_input", "models"]
