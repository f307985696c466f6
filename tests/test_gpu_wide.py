"""The wide trace layout (bit addresses of 33-37 bits, z term in 64 bits,
per-ray cached word: k_occl_lean_w) on a non-cubic grid, 2048 x 256 x 2048,
whose x and z extents need it: the whole occlusion frame (1 shadow + 8 AO +
1 spec rays per pixel through the exact DDA, Light.frag:29-81) bit for bit
against the oracle, and against the exact-step kernel's records pass."""
import numpy as np
import pytest

import oracle
from tests.gpu_util import assert_recs_equal, export_r8, rec_buffer, recs_np, same_bits

pytestmark = pytest.mark.gpu

KEYS = ("shadow", "ao", "ao_vis", "spec", "spec_t")


@pytest.mark.parametrize("light", [(0.3, 0.8, -0.5), (0.0, 0.8, -0.6)])
def test_wide_layout_frame_bit_exact(vxl, ctx, light):
    """light (0, 0.8, -0.6): every shadow ray has a zero x component and takes
    the literal form of the DDA, after the stepping loop."""
    import torch

    nx, ny, nz, W, H, seed = 2048, 256, 2048, 256, 144, 31
    G = vxl.Grid(ctx, nx, ny, nz)
    d = G.describe()
    assert d.trace_words and d.trace_wide == 1
    G.scene_noise(seed, 0.6, 1.0 / 24.0, 8)
    G.scene_boxes(seed, 400, 4, 48)
    cam = np.array([0.5 * nx, 1.6 * ny, -0.05 * nz], np.float32)
    tgt = np.array([0.5 * nx, 0.3 * ny, 0.35 * nz], np.float32)
    npix = W * H
    pos = torch.empty(npix * 3, dtype=torch.float32, device="cuda")
    nrm = torch.empty_like(pos)
    rough = torch.empty(npix, dtype=torch.float32, device="cuda")
    vxl.scene_gbuffer(ctx, G, cam, tgt, W, H, seed, pos, nrm, rough)
    kw = dict(light_dir=light, cam_pos=cam, bias=0.5, shadow_len=256.0, ao_len=48.0, spec_len=256.0,
              n_shadow=1, n_ao=8, n_spec=1, seed=seed)
    P = vxl.make_params(**kw)
    outs = {k: torch.full((npix,), -1.0, dtype=torch.float32, device="cuda") for k in KEYS}
    vxl.trace_occlusion(ctx, G, pos, nrm, rough, npix, P, width=W, height=H, **outs)
    R = 10
    rec = rec_buffer(npix * R)
    outs_r = {k: torch.empty(npix, dtype=torch.float32, device="cuda") for k in KEYS}
    vxl.trace_occlusion(ctx, G, pos, nrm, rough, npix, P, records=rec, **outs_r)
    torch.cuda.synchronize()
    for k in KEYS:
        assert torch.equal(outs[k].view(torch.int32), outs_r[k].view(torch.int32)), k
    g = export_r8(G)
    want = oracle.occlusion(g, pos.cpu().numpy(), nrm.cpu().numpy(), rough.cpu().numpy(),
                            oracle.make_params(**kw), with_recs=True)
    for k in KEYS:
        got = outs[k].cpu().numpy()
        ok = same_bits(got, want[k])
        assert ok.all(), "%s: %d of %d values differ" % (k, int((~ok).sum()), ok.size)
    assert_recs_equal(recs_np(rec), want["recs"], "records")
    # the frame has hits and misses of every kind, and long rays
    sky = (nrm.view(-1, 3).abs().sum(1) == 0).cpu().numpy()
    assert 0.02 < float(sky.mean()) < 0.95
    if light[0] != 0.0:  # (a zero direction component: the reference's loop reports no hit, all lit)
        assert 0.05 < float(want["shadow"][~sky].mean()) < 0.95
    assert 0.05 < float(want["ao_vis"][~sky].mean()) < 0.95
    assert int(want["recs"]["steps"].max()) > 100
    G.close()
