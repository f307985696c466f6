"""The two-level map of empty space (grids too large for the trace layout,
whose bit addresses must fit in 32 bits; tuning leap = 3). A ray whose remaining path is proved empty
on the map (dilated 8^3 tiles, 64^3 regions) ends as a miss without more
steps; every output must still equal the exact stepping of the records pass
(which never uses the map) over the whole frame, and the oracle on bands of
rows. The scene is a heightfield terrain with Vox instances standing on it
under an empty sky, so that many rays leave the surface into clear space;
both pool forms run (16-pixel tiles at 10 rays per pixel, 8-pixel tiles at
18)."""
import numpy as np
import pytest

import oracle
from tests.gpu_util import export_r8, same_bits

pytestmark = pytest.mark.gpu

KEYS = ("shadow", "ao", "ao_vis", "spec", "spec_t")


@pytest.fixture(scope="module")
def terrain(vxl, ctx):
    from voxelengine_gb300 import scenes

    sc = scenes.make_terrain_scene(ctx, 1024, 640, 360, seed=9, n_instances=3000, edge=(8, 48), amplitude=256.0)
    sc["g"] = export_r8(sc["grid"])
    return sc


@pytest.mark.parametrize("n_ao,ao_len", [(8, 32.0), (16, 64.0)])
def test_clear_path_matches_exact_stepping(vxl, ctx, terrain, n_ao, ao_len):
    import torch

    sc = terrain
    npix = sc["W"] * sc["H"]
    kw = dict(bias=0.5, shadow_len=256.0, ao_len=ao_len, spec_len=256.0, n_shadow=1, n_ao=n_ao, n_spec=1, seed=21)
    from voxelengine_gb300 import scenes

    ld = scenes.light_dir(21)
    P = vxl.make_params(light_dir=ld, cam_pos=sc["cam"], **kw)
    R = 2 + n_ao
    outs = {k: torch.full((npix,), -1.0, dtype=torch.float32, device="cuda") for k in KEYS}
    exact = {k: torch.full((npix,), -1.0, dtype=torch.float32, device="cuda") for k in KEYS}
    rec = torch.zeros(npix * R * 6, dtype=torch.int32, device="cuda")
    before = ctx.get_tuning()
    try:
        ctx.set_tuning(leap=3)
        vxl.trace_occlusion(ctx, sc["grid"], sc["pos"], sc["nrm"], sc["rough"], npix, P, width=sc["W"],
                            height=sc["H"], **outs)
    finally:
        ctx.set_tuning(**before)
    vxl.trace_occlusion(ctx, sc["grid"], sc["pos"], sc["nrm"], sc["rough"], npix, P, records=rec, **exact)
    torch.cuda.synchronize()
    for k in KEYS:
        assert torch.equal(outs[k], exact[k]), k
    # the sky is reached: many misses
    assert 0.2 < float(exact["shadow"].mean()) < 0.98
    OP = oracle.make_params(light_dir=ld, cam_pos=sc["cam"], **kw)
    pos, nrm, rough = sc["pos"].cpu().numpy(), sc["nrm"].cpu().numpy(), sc["rough"].cpu().numpy()
    W = sc["W"]
    for y0 in (0, 120, 240, 344):
        want = oracle.occlusion_range(sc["g"], pos, nrm, rough, OP, y0 * W, (y0 + 16) * W)
        for k in KEYS:
            got = outs[k][y0 * W:(y0 + 16) * W].cpu().numpy()
            assert same_bits(got, want[k]).all(), (k, y0)
