"""The headline configuration as a test: 512^3 grid (seeded 3-octave value
noise, threshold 0.55, frequency 1/32, ground slab y < 8, plus 2000 boxes of
4-48 voxels per side), 1920x1080 G-buffer from the seeded camera outside the
grid, 1 shadow (maxt 100) + 8 cosine AO (maxt 32) + 1 GGX specular (maxt 256)
rays per pixel through the exact DDA (Light.frag:29-81). The same scene and
parameters as the default benchmark.

Checked against the oracle:
  - all five occlusion buffers of the whole frame, bit for bit, on the
    default (no-records) kernel the benchmark times;
  - the per-ray records (hit cell, t bits, fetch count, exit reason) of every
    8th band of 32 image rows, from the records pass the benchmark uses for
    S_ref.
"""
import numpy as np
import pytest

import oracle
from tests.gpu_util import assert_recs_equal, export_r8, recs_np, same_bits

pytestmark = pytest.mark.gpu

N, W, H, SEED = 512, 1920, 1080, 2024
KEYS = ("shadow", "ao", "ao_vis", "spec", "spec_t")
PARAMS = dict(bias=0.5, shadow_len=100.0, ao_len=32.0, spec_len=256.0, n_shadow=1, n_ao=8, n_spec=1, seed=SEED)


@pytest.fixture(scope="module")
def c2(vxl, ctx):
    import torch

    from voxelengine_gb300 import scenes as S

    G = vxl.Grid(ctx, N, N, N)
    G.scene_noise(SEED, 0.55, 1.0 / 32.0, 8)
    G.scene_boxes(SEED, 2000, 4, 48)
    cam, tgt = S.camera(N)
    npix = W * H
    pos = torch.empty(npix * 3, dtype=torch.float32, device="cuda")
    nrm = torch.empty_like(pos)
    rough = torch.empty(npix, dtype=torch.float32, device="cuda")
    vxl.scene_gbuffer(ctx, G, cam, tgt, W, H, SEED, pos, nrm, rough)
    ld = S.light_dir(SEED)
    P = vxl.make_params(light_dir=ld, cam_pos=cam, **PARAMS)
    OP = oracle.make_params(light_dir=ld, cam_pos=cam, **PARAMS)
    torch.cuda.synchronize()
    return dict(G=G, pos=pos, nrm=nrm, rough=rough, P=P, OP=OP, g=export_r8(G), pos_h=pos.cpu().numpy(),
                nrm_h=nrm.cpu().numpy(), rough_h=rough.cpu().numpy())


def test_c2_frame_bit_exact(vxl, ctx, c2):
    import torch

    npix = W * H
    outs = {k: torch.full((npix,), -1.0, dtype=torch.float32, device="cuda") for k in KEYS}
    vxl.trace_occlusion(ctx, c2["G"], c2["pos"], c2["nrm"], c2["rough"], npix, c2["P"], width=W, height=H, **outs)
    torch.cuda.synchronize()
    want = oracle.occlusion(c2["g"], c2["pos_h"], c2["nrm_h"], c2["rough_h"], c2["OP"])
    for k in KEYS:
        got = outs[k].cpu().numpy()
        ok = same_bits(got, want[k])
        assert ok.all(), "%s: %d of %d values differ (max |d| %g)" % (
            k, int((~ok).sum()), ok.size, float(np.nanmax(np.abs(got - want[k]))))
    # the frame is neither all lit nor all shadowed
    assert 0.05 < float(want["shadow"].mean()) < 0.95
    assert 0.05 < float(want["ao_vis"].mean()) < 0.95


def test_c2_records_bit_exact(vxl, ctx, c2):
    import torch

    npix = W * H
    R = 10
    rec = torch.zeros(npix * R * 6, dtype=torch.int32, device="cuda")
    vxl.trace_occlusion(ctx, c2["G"], c2["pos"], c2["nrm"], c2["rough"], npix, c2["P"], records=rec, width=W,
                        height=H)
    torch.cuda.synchronize()
    got = recs_np(rec)
    rays = 0
    for y0 in range(0, H, 32 * 8):
        y1 = min(H, y0 + 32)
        want = oracle.occlusion_range(c2["g"], c2["pos_h"], c2["nrm_h"], c2["rough_h"], c2["OP"], y0 * W, y1 * W)
        assert_recs_equal(got[y0 * W * R:y1 * W * R], want["recs"], "rows %d-%d" % (y0, y1))
        rays += (y1 - y0) * W * R
    assert rays >= 5 * 32 * W * R
