"""The shipped FarmHouse scene end to end on the GPU: its 67 placements
(tests/golden/farmhouse_scene.npz, from PrefabAsset::Spawn and the
reference's own RealculateMatrix) voxelized into a ShadowVox grid of the
engine's size (524x188x524 bytes), a G-buffer traced by primary visibility,
then shadow / AO / specular-occlusion rays from it; every stage bit-exact
against the oracle doing the same."""
import os

import numpy as np
import pytest

import oracle
from tests.gpu_util import dev, export_r8, same_bits

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def farm():
    z = np.load(os.path.join(HERE, "golden", "farmhouse_scene.npz"))
    vols, off = [], 0
    for shp in z["volume_shapes"]:
        n = int(np.prod(shp))
        vols.append(z["volumes"][off:off + n].reshape(tuple(shp)))
        off += n
    return dict(vols=vols, vol_of=z["vol_of"], matrix=z["matrix"], palette=z["palette"])


def test_farmhouse_frame(vxl, ctx, farm):
    import torch

    vols, vol_of, M = farm["vols"], farm["vol_of"], farm["matrix"]
    assert len(M) == 67
    # ShadowVox grid of the engine's size (ShadowVoxSystem.cpp:56-58): 524 x 188 x 524 bytes
    nx, ny, nz = 2 * 524, 2 * 188, 2 * 524
    G = vxl.Grid(ctx, nx, ny, nz)
    d_models = [dev(v) for v in vols]
    mdesc = [(d.data_ptr(),) + v.shape[::-1] for v, d in zip(vols, d_models)]
    vxl.voxelize(ctx, G, mdesc, [(M[k], int(vol_of[k]), vxl.OP_SET) for k in range(len(M))])
    want_g = np.zeros((nz // 2, ny // 2, nx // 2), np.uint8)
    for k in range(len(M)):
        oracle.voxelize_model(want_g, vols[vol_of[k]], M[k], 1)
    got_g = export_r8(G)
    assert np.array_equal(got_g, want_g)
    assert oracle.r8_to_fine(got_g).sum() > 100000
    # primary visibility from above the farm
    cam = np.array([32.0, 18.0, -4.0], np.float32)
    tgt = np.array([32.0, 2.0, 22.0], np.float32)
    W, H = 320, 180
    vs = vxl.VolumeSet(ctx, vols)
    n = W * H
    pos = torch.empty(n * 3, dtype=torch.float32, device="cuda")
    nrm = torch.empty_like(pos)
    depth = torch.empty(n, dtype=torch.float32, device="cuda")
    mat = torch.empty(n, dtype=torch.int32, device="cuda")
    inst = torch.empty(n, dtype=torch.int32, device="cuda")
    vxl.trace_primary(ctx, vs, M, vol_of, cam, tgt, W, H, pos, nrm, depth, mat, inst, frame=3)
    torch.cuda.synchronize()
    want = oracle.primary(vols, M, vol_of, cam, tgt, W, H, frame=3)
    assert same_bits(pos.cpu().numpy().reshape(n, 3), want["pos"]).all()
    assert same_bits(nrm.cpu().numpy().reshape(n, 3), want["nrm"]).all()
    assert same_bits(depth.cpu().numpy(), want["depth"]).all()
    assert np.array_equal(mat.cpu().numpy(), want["material"])
    assert np.array_equal(inst.cpu().numpy(), want["instance"])
    hit = want["instance"] >= 0
    assert hit.mean() > 0.4 and len(np.unique(want["instance"][hit])) > 20
    # the palette colours those pixels would take (PALLETE_COLOR_TEXTURE at the material index)
    pal = farm["palette"].reshape(256, 7)
    assert pal[want["material"][hit], :3].any()
    # occlusion rays from that G-buffer over the ShadowVox grid
    P = vxl.make_params(light_dir=(0.4, 0.8, 0.3), cam_pos=cam * np.float32(10.0), n_ao=8, ao_len=32.0, n_spec=1,
                        seed=9)
    outs = {k: torch.empty(n, dtype=torch.float32, device="cuda") for k in ("shadow", "ao", "ao_vis", "spec",
                                                                             "spec_t")}
    rough = torch.full((n,), 0.3, dtype=torch.float32, device="cuda")
    vxl.trace_occlusion(ctx, G, pos, nrm, rough, n, P, width=W, height=H, **outs)
    torch.cuda.synchronize()
    OP = oracle.make_params(light_dir=(0.4, 0.8, 0.3), cam_pos=cam * np.float32(10.0), n_ao=8, ao_len=32.0,
                            n_spec=1, seed=9)
    wo = oracle.occlusion(want_g, want["pos"], want["nrm"], np.full(n, 0.3, np.float32), OP)
    for k in outs:
        assert same_bits(outs[k].cpu().numpy(), wo[k]).all(), k
    assert (wo["shadow"][hit] == 0).any() and (wo["shadow"][hit] == 1).any()
