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


def test_static_currents_are_requested_in_chunks_of_the_scratch_size(monkeypatch):
    """Batches above the static scratch's 4096 instances go through the C entry point in
    consecutive chunks: each call gets the offset device address, its count and the matching
    slice of the host output (the C call is replaced by a recorder; nothing runs on a device)."""
    assert heomq.static_current_chunks(4096) == [(0, 4096)]
    assert heomq.static_current_chunks(9000) == [(0, 4096), (4096, 4096), (8192, 808)]
    assert heomq.static_current_chunks(0) == []

    calls = []

    class FakeLib:
        @staticmethod
        def heom_batch_current_static(h, xptr, n, vs, out_ptr):
            calls.append((xptr.value, n, vs, out_ptr))
            return 0

    class FakeModel:
        nalf, nspin = 2, 2

    class FakeCtx:
        h = None
        model = FakeModel()

    monkeypatch.setattr(heomq, "lib", lambda: FakeLib)
    b = heomq.Batch.__new__(heomq.Batch)
    b.ctx, b.nbatch, b.stride = FakeCtx(), 9000, 128
    jt = b.currents_static(1 << 20)
    assert jt.shape == (9000, 2, 2)
    assert [(x - (1 << 20)) // (128 * 16) for x, _, _, _ in calls] == [0, 4096, 8192]
    assert [n for _, n, _, _ in calls] == [4096, 4096, 808]
    assert all(vs == 128 for _, _, vs, _ in calls)
    assert calls[1][3] - calls[0][3] == 4096 * 4 * 8   # output slice of the second chunk
