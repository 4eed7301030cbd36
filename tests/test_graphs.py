"""Beamforming plans under CUDA graphs: after one warm-up execution a plan
launches kernels only (no allocation, no host synchronisation), so a frame
loop can be captured once and replayed; the replayed frames equal direct
executions bit for bit. Covers the delay-and-sum, tensor-core minimum
variance and learned minimum-variance (subspace refinement) paths."""

from __future__ import annotations

import numpy as np
import pytest

from gold import BF_CASES, sim_setup, txset

pytestmark = pytest.mark.gpu


def _channel(capi, s):
    from test_gpu_parity import c_channel
    pr, med, acq = sim_setup(s)
    return c_channel(capi, pr, med, acq, txset(s, "pw"), is_iq=True, fdem=5e6)


@pytest.mark.parametrize("kind", ["das", "mv", "learned"])
def test_plan_capture_and_replay(golden, kind):
    import torch
    from usx import capi, learned

    g = golden("bf")
    s = golden("sim")
    stream = torch.cuda.Stream()
    ctx = capi.Context(0, stream=stream.cuda_stream)
    try:
        grid = capi.Grid(0, g["ax0"], g["ax1"], g["pts"])
        ch = _channel(capi, s)
        if kind == "das":
            cfg = capi.bf_config(f_number=1.5)
        elif kind == "mv":
            cfg = capi.bf_config(**dict(BF_CASES["mv"]))
        else:
            cfg = capi.bf_config(**dict(BF_CASES["mv"], combiner=learned.COMB_LEARNED_MV))
        plan = ctx.plan(ch, grid, cfg)
        mlp = None
        if kind == "mv":
            plan.set_mv_mode(1)
        if kind == "learned":
            mlp = capi.Mlp(ctx, learned.DIMS, seed=3)
            p = np.zeros(mlp.n_params, np.float32)
            _, b = mlp.layers(p)[-1]
            b[0::2] = 1.0 + 0.3 * np.cos(np.arange(64) * 0.9)
            mlp.set_params(p)
            plan.set_learned(mlp, float("inf"))
            plan.set_learned_refine(6)
        iq = torch.from_numpy(np.ascontiguousarray(g["iq"])).cuda()
        out = torch.empty(grid.shape, dtype=torch.complex64, device="cuda")
        with torch.cuda.stream(stream):
            plan.execute(iq.data_ptr(), out.data_ptr())        # warm-up: sizes the scratch arena
            stream.synchronize()
            graph = torch.cuda.CUDAGraph()
            with torch.cuda.graph(graph, stream=stream):
                plan.execute(iq.data_ptr(), out.data_ptr())
        frames_direct, frames_graph = [], []
        for scale in (1.0, 0.5 - 0.25j, 2.0j):
            data = torch.from_numpy(np.ascontiguousarray(g["iq"] * scale).astype(np.complex64)).cuda()
            with torch.cuda.stream(stream):
                iq.copy_(data)
                graph.replay()
            stream.synchronize()
            frames_graph.append(out.cpu().numpy().copy())
            with torch.cuda.stream(stream):
                plan.execute(iq.data_ptr(), out.data_ptr())
            stream.synchronize()
            frames_direct.append(out.cpu().numpy().copy())
        for a, b in zip(frames_graph, frames_direct):
            assert np.array_equal(a, b)
        assert not np.array_equal(frames_graph[0], frames_graph[1])
        plan.close()
        if mlp is not None:
            mlp.close()
    finally:
        ctx.close()
