"""The C-ABI boundary on a host without a GPU: the shared library loads, exports every
function that include/heom_gb300.h declares, builds models on the host, and refuses
device work loudly (an error code and message, never a CPU fallback)."""
import os
import re

import numpy as np
import pytest

import configs as cf
import heomq

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "heom_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(heom_\w+)\s*\(", text)))


def test_header_declares_the_reference_entry_points():
    names = declared_functions()
    for required in ("heom_ctx_create", "heom_ctx_destroy", "heom_calc_ax", "heom_calcderiv", "heom_calc_atrx",
                     "heom_solve_tfqmr", "heom_propagate"):
        assert required in names


def test_library_exports_every_declared_function():
    lib = heomq.lib()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_signatures_cover_the_header():
    assert set(declared_functions()) <= set(heomq.SIGNATURES)


def test_model_builds_on_the_host():
    m = heomq.Model(cf.siam(ntier=3, nmats=2))
    assert m.lunk > 0 and m.nunk > 0
    rho = m.initial_guess()
    assert rho.shape == (m.lunk,)
    assert np.isfinite(rho).all()


def test_bad_model_is_an_error_not_a_crash():
    cfg = cf.siam(ntier=3, nmats=2)
    cfg["norbs"] = 0
    with pytest.raises(heomq.HeomError):
        heomq.Model(cfg)


def _has_gpu():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="checks the no-device error path")
def test_context_without_a_device_fails_loudly():
    m = heomq.Model(cf.siam(ntier=3, nmats=2))
    with pytest.raises(heomq.HeomError) as e:
        heomq.Context(m)
    assert "device" in str(e.value).lower() or "cuda" in str(e.value).lower()
