"""heom_batch_current_static (allocation-free batch currents) against heom_current.

Collected last on purpose: it must pass both alone and after every other GPU test has
used the device."""
import numpy as np
import pytest

import configs as cf
import heomq

pytestmark = pytest.mark.gpu

HB = 0.658211928


def _batch_states(cfg, biases):
    import torch

    m = heomq.Model(cfg)
    ctx = heomq.Context(m, adjoint=False)
    es = np.zeros((len(biases), m.nalf * m.nspin))
    for b, V in enumerate(biases):
        es[b] = np.array([[V / 2, V / 2], [-V / 2, -V / 2]]).T.reshape(-1) / HB
    batch = heomq.Batch(ctx, eshift_batch=es, nbatch=len(biases))
    x = torch.zeros((len(biases), batch.stride), dtype=torch.complex128, device="cuda")
    x[:, : m.lunk] = torch.from_numpy(m.initial_guess()).cuda()
    torch.cuda.synchronize()
    batch.solve_dev(x.data_ptr(), crit=1e-9, precision=heomq.PREC_MIXED)
    return m, ctx, batch, x


@pytest.mark.parametrize("cfg", [cf.siam(ntier=3, nmats=2), cf.dqd(ntier=3, nmats=2)], ids=["siam_L2", "dqd_L2"])
def test_static_currents_match_heom_current_twice(cfg):
    m, ctx, batch, x = _batch_states(cfg, [0.2, 0.5, 0.9])
    first = batch.currents_static(x.data_ptr())
    second = batch.currents_static(x.data_ptr())
    np.testing.assert_array_equal(first, second)
    for b in range(batch.nbatch):
        ref = ctx.current(x[b, : m.lunk].cpu().numpy())
        np.testing.assert_allclose(first[b], ref, rtol=1e-12, atol=1e-9 * np.max(np.abs(ref)))


def test_static_currents_reject_oversize_batches():
    """The C entry point refuses more than 4096 instances and a stride shorter than a vector
    before it launches anything (the buffer here holds one instance); the Python wrapper
    refuses to read beyond its own batch."""
    m, ctx, batch, x = _batch_states(cf.siam(ntier=3, nmats=2), [0.4])
    jt = np.zeros(4097 * 4)
    rc = heomq.lib().heom_batch_current_static(ctx.h, x.data_ptr(), 4097, batch.stride, jt.ctypes.data)
    assert rc == -1 and "4096" in heomq.lib().heom_last_error().decode()
    rc = heomq.lib().heom_batch_current_static(ctx.h, x.data_ptr(), 1, m.lunk, jt.ctypes.data)
    assert rc == -1
    with pytest.raises(heomq.HeomError):
        batch.currents_static(x.data_ptr(), nbatch=2)
    # the context still works after the refusals
    np.testing.assert_array_equal(batch.currents_static(x.data_ptr()), batch.currents_static(x.data_ptr()))
