"""The allocation-free colour-flow entry point (usx_cu_color_flow_noalloc).

Some callers of this library cannot allocate device memory while they run: a
real-time acquisition loop with a fixed memory budget, or a host application
that owns the device's allocator and lends the library only a stream. For them, usx_cu_color_flow_noalloc keeps its
working memory in a fixed 8 MiB array reserved by the library, takes a stream
instead of a context, and must give exactly what usx_cu_color_flow gives.

This file is collected last (its name sorts after the others), so a run that
stops at the first failure has already run everything else; it also passes
when run alone in a fresh process.
"""

from __future__ import annotations

import numpy as np
import pytest

from gold import rel_l2

pytestmark = pytest.mark.gpu


def _ensemble(rng, n, n0, n1):
    ph = np.exp(-1j * 0.3 * np.arange(n))[:, None, None] * np.exp(-1j * 0.8 * np.arange(n1))[None, None, :]
    noise = rng.normal(size=(n, n0, n1)) + 1j * rng.normal(size=(n, n0, n1))
    return (5.0 * np.exp(0.02j * np.arange(n))[:, None, None] + 2.0 * ph + 0.3 * noise).astype(np.complex64)


def _maps(torch, n0, n1):
    out = [torch.empty((n0, n1), dtype=torch.float32, device="cuda") for _ in range(3)]
    out.append(torch.empty((n0, n1), dtype=torch.uint8, device="cuda"))
    return out


def test_noalloc_color_flow_equals_color_flow_on_two_calls():
    import torch
    from usx import capi

    assert torch.cuda.is_available()
    ctx = capi.Context(0, stream=torch.cuda.current_stream().cuda_stream)
    rng = np.random.default_rng(7)
    cfg = capi.doppler_config(wall_filter=1, polynomial_order=2)
    # Two calls in a row with different sizes: the second must not see the
    # first call's leftovers in the shared scratch (e.g. its maximum power).
    for n, n0, n1 in ((12, 64, 100), (8, 40, 150)):
        ens = _ensemble(rng, n, n0, n1)
        ens[:, :, : n1 // 3] *= 0.01 if n == 8 else 100.0  # change the frame's peak power between calls
        axis1 = np.linspace(0.02, 0.03, n1).astype(np.float32)
        d = torch.from_numpy(ens).cuda()
        ref = _maps(torch, n0, n1)
        got = _maps(torch, n0, n1)
        nyq_ref = ctx.color_flow(d.data_ptr(), n, n0, n1, axis1, 5e6, 5000.0, 1540.0, cfg,
                                 *[t.data_ptr() for t in ref])
        nyq = capi.color_flow_noalloc(torch.cuda.current_stream().cuda_stream, d.data_ptr(), n, n0, n1, axis1,
                                      5e6, 5000.0, 1540.0, cfg, *[t.data_ptr() for t in got])
        torch.cuda.synchronize()
        assert nyq == nyq_ref
        for a, b in zip(got[:3], ref[:3]):
            assert rel_l2(a.cpu().numpy(), b.cpu().numpy()) <= 1e-5
        assert np.array_equal(got[3].cpu().numpy(), ref[3].cpu().numpy())
        assert got[3].cpu().numpy().sum() > 0
    ctx.close()


@pytest.mark.parametrize("n,n0,n1,wt", [(64, 128, 128, 1), (16, 64, 96, 0)])
def test_noalloc_color_flow_at_the_limit_and_without_wall_filter(n, n0, n1, wt):
    """Exactly the 1,048,576 complex samples the scratch holds (64 frames,
    whose wall filter needs more than 48 KiB of shared memory per block), and
    the wall filter switched off, each twice in a row."""
    import torch
    from usx import capi

    ctx = capi.Context(0, stream=torch.cuda.current_stream().cuda_stream)
    rng = np.random.default_rng(11)
    cfg = capi.doppler_config(wall_filter=wt, polynomial_order=2)
    ens = _ensemble(rng, n, n0, n1)
    axis1 = np.linspace(0.02, 0.03, n1).astype(np.float32)
    d = torch.from_numpy(ens).cuda()
    ref = _maps(torch, n0, n1)
    ctx.color_flow(d.data_ptr(), n, n0, n1, axis1, 5e6, 5000.0, 1540.0, cfg, *[t.data_ptr() for t in ref])
    for _ in range(2):
        got = _maps(torch, n0, n1)
        capi.color_flow_noalloc(torch.cuda.current_stream().cuda_stream, d.data_ptr(), n, n0, n1, axis1,
                                5e6, 5000.0, 1540.0, cfg, *[t.data_ptr() for t in got])
        torch.cuda.synchronize()
        for a, b in zip(got[:3], ref[:3]):
            assert rel_l2(a.cpu().numpy(), b.cpu().numpy()) <= 1e-5
        assert np.array_equal(got[3].cpu().numpy(), ref[3].cpu().numpy())
    ctx.close()


def test_noalloc_color_flow_rejects_ensembles_beyond_its_scratch():
    import torch
    from usx import capi

    n, n0, n1 = 17, 256, 256  # 1,114,112 complex samples > 1,048,576
    d = torch.zeros((n, n0, n1), dtype=torch.complex64, device="cuda")
    maps = _maps(torch, n0, n1)
    with pytest.raises(ValueError, match="static scratch"):
        capi.color_flow_noalloc(0, d.data_ptr(), n, n0, n1, np.linspace(0.02, 0.03, n1), 5e6, 5000.0, 1540.0,
                                capi.doppler_config(), *[t.data_ptr() for t in maps])
