"""Primary visibility on the GPU (vxl_volume_build_mips, vxl_trace_primary)
against the oracle, bit for bit: mips, and per pixel the hit position,
normal and depth bits, material and instance index; then the whole frame
path -- instances voxelized into the ShadowVox grid, the G-buffer from
primary visibility, occlusion rays from that G-buffer -- against the oracle
doing the same three steps."""
import numpy as np
import pytest

import oracle
from tests.gpu_util import dev, export_r8, same_bits

pytestmark = pytest.mark.gpu


def _volumes(seed, count, lo=8, hi=40):
    from voxelengine_gb300 import scenes

    return scenes.vox_models(seed, count, lo, hi, fill=0.35)


def _instances(rng, n_inst, vols, extent):
    from voxelengine_gb300 import scenes

    worlds, vol_of = [], []
    for _ in range(n_inst):
        vi = int(rng.integers(0, len(vols)))
        worlds.append(scenes.instance_matrix(rng, extent, vols[vi].shape))
        vol_of.append(vi)
    return np.array(worlds, np.float32), np.array(vol_of, np.int32)


def test_volume_mips_match_oracle(vxl, ctx):
    import torch

    rng = np.random.default_rng(2)
    for v in _volumes(3, 6, 4, 64):
        sz, sy, sx = v.shape
        d = oracle.mip_dims((sx, sy, sz))
        d1 = torch.zeros(int(np.prod(d[1])), dtype=torch.uint8, device="cuda")
        d2 = torch.zeros(int(np.prod(d[2])), dtype=torch.uint8, device="cuda")
        vxl.volume_build_mips(ctx, dev(v), sx, sy, sz, d1, d2)
        torch.cuda.synchronize()
        w1, w2 = oracle.volume_mips(v)
        assert np.array_equal(d1.cpu().numpy(), w1.reshape(-1))
        assert np.array_equal(d2.cpu().numpy(), w2.reshape(-1))
    del rng


def _run_primary(vxl, ctx, vols, worlds, vol_of, cam, tgt, W, H, frame):
    import torch

    vs = vxl.VolumeSet(ctx, vols)
    n = W * H
    pos = torch.empty(n * 3, dtype=torch.float32, device="cuda")
    nrm = torch.empty_like(pos)
    depth = torch.empty(n, dtype=torch.float32, device="cuda")
    mat = torch.empty(n, dtype=torch.int32, device="cuda")
    inst = torch.empty(n, dtype=torch.int32, device="cuda")
    vxl.trace_primary(ctx, vs, worlds, vol_of, cam, tgt, W, H, pos, nrm, depth, mat, inst, frame=frame)
    torch.cuda.synchronize()
    return dict(pos=pos.cpu().numpy().reshape(n, 3), nrm=nrm.cpu().numpy().reshape(n, 3), depth=depth.cpu().numpy(),
                material=mat.cpu().numpy(), instance=inst.cpu().numpy(), d_pos=pos, d_nrm=nrm)


def _assert_same(got, want):
    for k in ("pos", "nrm", "depth"):
        assert same_bits(got[k], want[k]).all(), k
    assert np.array_equal(got["material"], want["material"])
    assert np.array_equal(got["instance"], want["instance"])


@pytest.mark.parametrize("frame", [0, 1])
def test_primary_matches_oracle(vxl, ctx, frame):
    rng = np.random.default_rng(10 + frame)
    vols = _volumes(5, 7)
    extent = 96  # fine voxels: instances inside a 9.6-world-unit cube
    worlds, vol_of = _instances(rng, 60, vols, extent)
    cam = np.array([4.8, 11.0, -3.0], np.float32)
    tgt = np.array([4.8, 4.0, 4.8], np.float32)
    W, H = 160, 96
    got = _run_primary(vxl, ctx, vols, worlds, vol_of, cam, tgt, W, H, frame)
    want = oracle.primary(vols, worlds, vol_of, cam, tgt, W, H, frame=frame)
    _assert_same(got, want)
    hit = want["instance"] >= 0
    assert 0.1 < hit.mean() < 0.95
    assert len(np.unique(want["instance"][hit])) > 20


def test_primary_camera_among_instances(vxl, ctx):
    """Camera inside the instance field (boxes behind it, around it and
    containing it): the screen bins fall back to the whole screen there."""
    rng = np.random.default_rng(21)
    vols = _volumes(6, 5, 8, 24)
    worlds, vol_of = _instances(rng, 80, vols, 64)
    cam = np.array([3.2, 3.2, 3.2], np.float32)
    tgt = np.array([5.0, 2.0, 6.0], np.float32)
    W, H = 96, 64
    got = _run_primary(vxl, ctx, vols, worlds, vol_of, cam, tgt, W, H, 0)
    want = oracle.primary(vols, worlds, vol_of, cam, tgt, W, H, frame=0)
    _assert_same(got, want)
    assert (want["instance"] >= 0).mean() > 0.2


def test_primary_edge_cases(vxl, ctx):
    import torch

    vols = _volumes(7, 2, 8, 16)
    vs = vxl.VolumeSet(ctx, vols)
    W, H = 32, 16
    pos = torch.ones(W * H * 3, dtype=torch.float32, device="cuda")
    nrm = torch.ones_like(pos)
    inst = torch.zeros(W * H, dtype=torch.int32, device="cuda")
    # no instances: every pixel is sky
    vxl.trace_primary(ctx, vs, np.zeros((0, 16), np.float32), [], (0, 1, -5), (0, 0, 0), W, H, pos, nrm,
                      instance=inst)
    torch.cuda.synchronize()
    assert not pos.any() and not nrm.any() and bool((inst == -1).all())
    # a command naming a missing volume is rejected
    with pytest.raises(vxl.VxlError) as e:
        vxl.trace_primary(ctx, vs, np.eye(4, dtype=np.float32).reshape(1, 16), [5], (0, 1, -5), (0, 0, 0), W, H,
                          pos, nrm)
    assert e.value.status == vxl.VXL_ERR_OUT_OF_RANGE
    # more (command, screen tile) pairs than 32-bit list offsets hold are rejected before any work
    many = np.tile(np.eye(4, dtype=np.float32).reshape(1, 16), (2100, 1))
    with pytest.raises(vxl.VxlError) as e:
        vxl.trace_primary(ctx, vs, many, [0] * 2100, (0, 1, -5), (0, 0, 0), 16384, 16384, pos, nrm)
    assert e.value.status == vxl.VXL_ERR_INVALID_ARG
    # volumes smaller than 4 on an axis are rejected (VoxAsset sizes are multiples of 4)
    d0 = torch.zeros(2 * 8 * 8, dtype=torch.uint8, device="cuda")
    with pytest.raises(vxl.VxlError):
        vxl.volume_build_mips(ctx, d0, 2, 8, 8, d0, d0)


def test_frame_path_primary_then_occlusion(vxl, ctx):
    """Instances -> ShadowVox grid (vxl_voxelize) and G-buffer
    (vxl_trace_primary) -> occlusion rays (vxl_trace_occlusion), against the
    oracle running the same three steps."""
    import torch

    rng = np.random.default_rng(31)
    vols = _volumes(8, 6, 8, 32)
    n = 128
    worlds, vol_of = _instances(rng, 50, vols, n)
    # ShadowVox grid from the same instances (model voxels >= 16 are opaque)
    G = vxl.Grid(ctx, n, n, n)
    d_models = [dev(v) for v in vols]
    mdesc = [(d.data_ptr(),) + v.shape[::-1] for v, d in zip(vols, d_models)]
    vxl.voxelize(ctx, G, mdesc, [(worlds[k], int(vol_of[k]), vxl.OP_SET) for k in range(len(worlds))])
    want_g = np.zeros((n // 2, n // 2, n // 2), np.uint8)
    for k in range(len(worlds)):
        oracle.voxelize_model(want_g, vols[vol_of[k]], worlds[k], 1)
    assert np.array_equal(export_r8(G), want_g)
    cam = np.array([6.4, 14.0, -4.0], np.float32)
    tgt = np.array([6.4, 5.0, 6.4], np.float32)
    W, H = 128, 80
    got = _run_primary(vxl, ctx, vols, worlds, vol_of, cam, tgt, W, H, 0)
    want = oracle.primary(vols, worlds, vol_of, cam, tgt, W, H, frame=0)
    _assert_same(got, want)
    npix = W * H
    cam_fine = cam * np.float32(10.0)
    P = vxl.make_params(light_dir=(0.3, 0.8, 0.5), cam_pos=cam_fine, n_ao=6, ao_len=24.0, n_spec=1, seed=4)
    outs = {k: torch.empty(npix, dtype=torch.float32, device="cuda") for k in ("shadow", "ao", "ao_vis", "spec",
                                                                                "spec_t")}
    rough = torch.full((npix,), 0.4, dtype=torch.float32, device="cuda")
    vxl.trace_occlusion(ctx, G, got["d_pos"], got["d_nrm"], rough, npix, P, **outs)
    torch.cuda.synchronize()
    OP = oracle.make_params(light_dir=(0.3, 0.8, 0.5), cam_pos=cam_fine, n_ao=6, ao_len=24.0, n_spec=1, seed=4)
    wo = oracle.occlusion(want_g, want["pos"], want["nrm"], np.full(npix, 0.4, np.float32), OP)
    for k in outs:
        assert same_bits(outs[k].cpu().numpy(), wo[k]).all(), k
    hit = want["instance"] >= 0
    assert hit.mean() > 0.2 and (wo["shadow"][hit] == 0).any() and (wo["shadow"][hit] == 1).any()


def test_primary_list_overflow_is_exact(vxl, ctx):
    """A frame whose screen-bin lists outgrow the capacity sized from the
    previous frame scans every command instead (same result); the next frame
    runs with grown lists."""
    rng = np.random.default_rng(41)
    vols = _volumes(9, 3, 32, 40)
    c2 = vxl.Context(0)  # fresh list capacity
    W, H = 128, 96
    cam = np.array([2.0, 2.0, -6.0], np.float32)
    tgt = np.array([2.0, 2.0, 2.0], np.float32)
    few_w, few_v = _instances(rng, 1, vols, 32)
    _run_primary(vxl, c2, vols, few_w, few_v, cam, tgt, W, H, 0)
    # 600 boxes of 3.2-4 world units 2.5-4.5 units in front of the camera: each
    # covers most of the 8x6 screen tiles, far beyond the 16 per command the
    # capacity allows for
    many = []
    for _ in range(600):
        m = np.eye(4, dtype=np.float32)
        m[:3, 3] = rng.uniform(-0.5, 2.5, 3)
        m[2, 3] = rng.uniform(-3.5, -1.5)
        many.append(np.ascontiguousarray(m.T).reshape(16))
    many = np.array(many, np.float32)
    many_v = rng.integers(0, len(vols), len(many)).astype(np.int32)
    want = oracle.primary(vols, many, many_v, cam, tgt, W, H, frame=0)
    for _ in range(2):  # first call overflows, second runs with grown lists
        got = _run_primary(vxl, c2, vols, many, many_v, cam, tgt, W, H, 0)
        _assert_same(got, want)
    assert (want["instance"] >= 0).mean() > 0.5
