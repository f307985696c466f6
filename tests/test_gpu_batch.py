"""Batched tracing (vxl_batch_*: many scenes in one persistent launch,
replayed from a CUDA graph) and tile-shape / queue-granularity knobs: every
scene's buffers must equal the oracle's (oracle.occlusion on the scene's
exported ShadowVox grid, Light.frag:29-81 driven as vxl_trace_occlusion
drives it) and a separate vxl_trace_occlusion of that scene, bit for bit, and
the single-scene outputs must not depend on the tuning."""
import ctypes as C

import numpy as np
import pytest

import oracle
from tests.gpu_util import export_r8, same_bits

pytestmark = pytest.mark.gpu

KEYS = ("shadow", "ao", "ao_vis", "spec", "spec_t")


@pytest.fixture(scope="module")
def scenes(vxl, ctx):
    from voxelengine_gb300 import scenes as S

    out = []
    rng = np.random.default_rng(3)
    for i, (n, W, H) in enumerate([(64, 120, 70), (128, 200, 90), (96, 33, 17), (192, 160, 160), (66, 80, 40)]):
        sc = S.make_scene(ctx, n, W, H, 100 + i, thresh=float(rng.uniform(0.45, 0.65)))
        if i == 2:  # different ray mix in one batch
            sc["params"] = vxl.make_params(cam_pos=sc["cam"], n_shadow=1, n_ao=4, ao_len=16.0, n_spec=0, seed=5)
        if i == 4:
            sc["params"] = vxl.make_params(cam_pos=sc["cam"], n_shadow=0, n_ao=12, ao_len=24.0, n_spec=2, seed=6)
        out.append(S.add_outputs(sc))
    return out


@pytest.fixture(scope="module")
def oracle_outs(scenes):
    out = []
    for sc in scenes:
        op = oracle.Params()
        C.memmove(C.byref(op), C.byref(sc["params"]), C.sizeof(op))  # same layout as vxl_trace_params
        out.append(oracle.occlusion(export_r8(sc["grid"]), sc["pos"].cpu().numpy(), sc["nrm"].cpu().numpy(),
                                    sc["rough"].cpu().numpy(), op))
    return out


@pytest.mark.parametrize("use_graph", [True, False])
@pytest.mark.parametrize("tune", [None, (32, 4, 2, 2, 8, 2)])
def test_batch_matches_oracle(vxl, ctx, scenes, oracle_outs, use_graph, tune):
    """The batched kernel runs its own template instance (two step counters,
    the bounds test at every step, every ray's t kept): its outputs are
    checked against the oracle directly, not only against the single-scene
    kernel."""
    import torch

    before = ctx.get_tuning()
    try:
        if tune:
            ctx.set_tuning(*tune)
        b = vxl.Batch(ctx, scenes, use_graph=use_graph)
        for rep in range(2):
            for sc in scenes:
                for k in KEYS:
                    sc[k].fill_(-1.0)
            b.run()
            torch.cuda.synchronize()
            for i, (sc, w) in enumerate(zip(scenes, oracle_outs)):
                for k in KEYS:
                    ok = same_bits(sc[k].cpu().numpy(), w[k])
                    assert ok.all(), "scene %d (%d^3) %s rep %d: %d of %d values differ" % (
                        i, sc["n"], k, rep, int((~ok).sum()), ok.size)
        b.close()
    finally:
        ctx.set_tuning(**before)


def _single(vxl, ctx, sc):
    import torch

    o = {k: torch.empty(sc["npix"], dtype=torch.float32, device="cuda") for k in KEYS}
    vxl.trace_occlusion(ctx, sc["grid"], sc["pos"], sc["nrm"], sc["rough"], sc["npix"], sc["params"], **o)
    return o


@pytest.mark.parametrize("use_graph", [True, False])
def test_batch_matches_single_scene_calls(vxl, ctx, scenes, use_graph):
    import torch

    want = [_single(vxl, ctx, sc) for sc in scenes]
    b = vxl.Batch(ctx, scenes, use_graph=use_graph)
    for rep in range(2):  # replays reset the shared work queue
        for sc in scenes:
            for k in KEYS:
                sc[k].fill_(-1.0)
        b.run()
        torch.cuda.synchronize()
        for sc, w in zip(scenes, want):
            for k in KEYS:
                assert torch.equal(sc[k], w[k]), (sc["n"], k, rep)
    tiles, rays = b.info()
    assert rays == sum(sc["npix"] * (sc["params"].n_shadow + sc["params"].n_ao + sc["params"].n_spec)
                       for sc in scenes)
    b.close()


@pytest.mark.parametrize("tune", [(16, 8, 2, 1, 4, 1), (16, 4, 2, 2, 8, 2), (32, 2, 2, 1, 8, 4), (32, 8, 2, 1, 32, 1),
                                  (16, 1, 1, 1, 4, 2)])
def test_tuning_does_not_change_results(vxl, ctx, scenes, tune):
    import torch

    sc = scenes[3]
    base = _single(vxl, ctx, sc)
    before = ctx.get_tuning()
    try:
        ctx.set_tuning(*tune)
        got = _single(vxl, ctx, sc)
        b = vxl.Batch(ctx, scenes[:4])
        b.run()
        torch.cuda.synchronize()
        for k in KEYS:
            assert torch.equal(got[k], base[k]), k
            assert torch.equal(sc[k], base[k]), k
        b.close()
    finally:
        ctx.set_tuning(**before)
