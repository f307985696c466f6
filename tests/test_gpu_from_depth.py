"""vxl_trace_occlusion_from_depth on the GPU against the oracle bit for bit:
the positions are rebuilt from a linear-depth G-buffer (the view buffer's
inverse matrices, LightAmbient's placement) and traced; the oracle rebuilds
with vo_rebuild_from_depth and traces the same rays. The depth buffer comes
from a traced G-buffer of a noise scene, with sky and edge-case texels."""
import numpy as np
import pytest

import oracle
from tests import view_cases as vc
from tests.gpu_util import dev, export_r8, same_bits

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("W,H", [(96, 64), (131, 77)])
def test_from_depth_matches_oracle(vxl, ctx, W, H):
    import torch

    n = 128
    G = vxl.Grid(ctx, n, n, n)
    G.scene_noise(11, 0.55, 1.0 / 32.0, 8)
    G.scene_boxes(11, 30, 4, 24)
    cam = np.array([-0.3 * n, 0.8 * n, -0.45 * n], np.float32)  # fine units
    tgt = np.array([n / 2] * 3, np.float32)
    npix = W * H
    pos = torch.empty(npix * 3, dtype=torch.float32, device="cuda")
    nrm = torch.empty_like(pos)
    rough = torch.empty(npix, dtype=torch.float32, device="cuda")
    vxl.scene_gbuffer(ctx, G, cam, tgt, W, H, 7, pos, nrm, rough)
    torch.cuda.synchronize()
    pos_h, nrm_h = pos.cpu().numpy().reshape(-1, 3), nrm.cpu().numpy().reshape(-1, 3)
    # the view buffer of that camera (world units = fine / 10) and the depth GeometryVoxel writes
    iv, ip, view, _ = vc.view_mats(cam / 10.0, tgt / 10.0, 0.57735026, W, H)
    depth = vc.depth_of(pos_h / 10.0, view)
    depth[~(np.abs(nrm_h).sum(1) > 0)] = 1.0  # pixels that saw nothing: sky
    depth[:4] = [0.999, np.nan, 0.99899, -0.0]
    d_depth = dev(depth)
    P = vxl.make_params(cam_pos=cam, n_ao=6, ao_len=24.0, n_spec=1, seed=3)
    outs = {k: torch.empty(npix, dtype=torch.float32, device="cuda") for k in ("shadow", "ao", "ao_vis", "spec",
                                                                                "spec_t")}
    vxl.trace_occlusion_from_depth(ctx, G, d_depth, nrm, rough, W, H, iv, ip, P, **outs)
    torch.cuda.synchronize()
    wcp, n2 = oracle.rebuild_from_depth(depth, nrm_h, W, H, iv, ip)
    OP = oracle.make_params(cam_pos=cam, n_ao=6, ao_len=24.0, n_spec=1, seed=3)
    want = oracle.occlusion(export_r8(G), wcp, n2, rough.cpu().numpy(), OP)
    for k in outs:
        assert same_bits(outs[k].cpu().numpy(), want[k]).all(), k
    live = depth < 0.999
    live[:4] = False
    # the rebuilt surface is the traced one, pulled toward the camera by LightAmbient's
    # NEAR bias (about 0.1 / w of the distance, under 1% here)
    d_true = np.linalg.norm(pos_h[live] - cam, axis=1)
    d_back = np.linalg.norm(wcp[live] - cam, axis=1)
    assert np.all(np.abs(d_back / d_true - 1) < 0.02)
    assert (want["shadow"][live] == 0).any() and (want["shadow"][live] == 1).any()


def test_from_depth_rejects_bad_arguments(vxl, ctx):
    import torch

    G = vxl.Grid(ctx, 16, 16, 16)
    P = vxl.make_params()
    d = torch.zeros(16, dtype=torch.float32, device="cuda")
    eye = np.eye(4, dtype=np.float32).reshape(16)
    with pytest.raises(vxl.VxlError):
        vxl.trace_occlusion_from_depth(ctx, G, None, d, None, 4, 4, eye, eye, P, shadow=d)
    with pytest.raises(vxl.VxlError):
        vxl.trace_occlusion_from_depth(ctx, G, d, d, None, -1, 4, eye, eye, P, shadow=d)
    # an empty image is a no-op
    vxl.trace_occlusion_from_depth(ctx, G, d, d, None, 0, 0, eye, eye, P, shadow=d)
