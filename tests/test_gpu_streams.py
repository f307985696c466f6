"""Occlusion calls that overlap on the GPU. Each vxl_trace_occlusion call
takes its own work-queue counter, so calls on two non-blocking streams of one
context run at the same time without sharing one. A call captured into a CUDA
graph keeps its counter for the graph's life, on a slot no direct call gets,
and a context refuses captured calls once those slots are used up. Every
output is compared bit for bit with the same call run alone."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KEYS = ("shadow", "ao", "ao_vis", "spec", "spec_t")


def _scene(vxl, ctx, n, W, H, seed):
    from voxelengine_gb300 import scenes as S

    return S.make_scene(ctx, n, W, H, seed, thresh=0.55)


def _outs(npix):
    import torch

    return {k: torch.full((npix,), -1.0, dtype=torch.float32, device="cuda") for k in KEYS}


def _trace(vxl, ctx, sc, outs, stream=None):
    vxl.trace_occlusion(ctx, sc["grid"], sc["pos"], sc["nrm"], sc["rough"], sc["npix"], sc["params"],
                        stream=stream, **outs)


def _assert_same(got, want, what):
    import torch

    for k in KEYS:
        assert torch.equal(got[k], want[k]), (what, k)


def test_two_streams_overlap(vxl, ctx):
    import torch

    a = _scene(vxl, ctx, 128, 320, 180, 31)
    b = _scene(vxl, ctx, 96, 256, 144, 32)
    want_a, want_b = _outs(a["npix"]), _outs(b["npix"])
    _trace(vxl, ctx, a, want_a)
    _trace(vxl, ctx, b, want_b)
    torch.cuda.synchronize()
    s1 = torch.cuda.Stream()
    s2 = torch.cuda.Stream()
    got_a, got_b = _outs(a["npix"]), _outs(b["npix"])
    torch.cuda.synchronize()
    for _ in range(8):  # no synchronisation between the two streams
        _trace(vxl, ctx, a, got_a, stream=s1)
        _trace(vxl, ctx, b, got_b, stream=s2)
    torch.cuda.synchronize()
    _assert_same(got_a, want_a, "stream 1")
    _assert_same(got_b, want_b, "stream 2")


def test_captured_call_keeps_its_counter(vxl):
    import torch

    ctx = vxl.Context(0)
    a = _scene(vxl, ctx, 64, 96, 64, 41)
    b = _scene(vxl, ctx, 64, 80, 48, 42)
    want_a, want_b = _outs(a["npix"]), _outs(b["npix"])
    _trace(vxl, ctx, a, want_a)
    _trace(vxl, ctx, b, want_b)
    torch.cuda.synchronize()
    got_a, got_b = _outs(a["npix"]), _outs(b["npix"])
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, capture_error_mode="relaxed"):
        _trace(vxl, ctx, a, got_a)
    s1 = torch.cuda.Stream()
    s2 = torch.cuda.Stream()
    torch.cuda.synchronize()
    # more direct calls than the ring holds, with graph replays among them:
    # no direct call may take the captured call's counter
    for i in range(4500):
        _trace(vxl, ctx, b, got_b, stream=s2)
        if i % 64 == 0:
            with torch.cuda.stream(s1):
                g.replay()
    torch.cuda.synchronize()
    _assert_same(got_a, want_a, "graph replays")
    _assert_same(got_b, want_b, "direct calls")
    del g, a, b
    ctx.close()


def test_captured_calls_are_bounded(vxl):
    import torch

    ctx = vxl.Context(0)
    a = _scene(vxl, ctx, 32, 16, 8, 43)
    o = _outs(a["npix"])
    g = torch.cuda.CUDAGraph()
    err = None
    with torch.cuda.graph(g, capture_error_mode="relaxed"):
        for i in range(4097):
            try:
                _trace(vxl, ctx, a, o)
            except vxl.VxlError as e:
                err = (i, e)
                break
    assert err is not None and err[0] == 4096, err
    assert err[1].status == 7 and "captured" in str(err[1])
    del g
    torch.cuda.synchronize()
    # direct calls still work on that context
    want = _outs(a["npix"])
    _trace(vxl, ctx, a, want)
    torch.cuda.synchronize()
    assert float(want["shadow"].min()) >= 0.0
    del a
    ctx.close()
