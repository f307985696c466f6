"""Differentiable soft-opacity pass on the GPU (vxl_trace_soft_fwd/_bwd)
against the FP64 oracle model and FP64 central finite differences.

Tolerances: image within 2e-5 absolute of FP64 (fp32 products and sums);
gradient within 1e-3 of FP64 in relative L2 norm over the whole grid, and
each of 64 finite-difference voxels (h = 1e-4, FP64) within 1e-3 relative.
"""
import numpy as np
import pytest

import oracle
from tests.gpu_util import dev

pytestmark = pytest.mark.gpu

AMAX = 1.0 - 1.0 / 4096.0


def _scene(vxl, ctx, n=64, W=64, H=48, seed=3, n_ao=8, albedo_seed=1):
    from voxelengine_gb300 import scenes

    P = vxl.make_soft_params(light_dir=scenes.light_dir(seed), bias=0.5, length=24.0, k_sun=0.7, k_amb=0.5,
                             n_shadow=1, n_ao=n_ao, seed=seed)
    return scenes.make_soft_scene(ctx, n, W, H, seed, albedo_seed=albedo_seed, params=P)


def _oracle_params(P):
    return oracle.make_soft_params(light_dir=list(P.light_dir), bias=P.bias, length=P.len, k_sun=P.k_sun,
                                   k_amb=P.k_amb, n_shadow=P.n_shadow, n_ao=P.n_ao, seed=P.seed)


def _fwd(vxl, ctx, sc, soft=None):
    import torch

    soft = sc["soft"] if soft is None else soft
    img = torch.empty((sc["npix"], 3), dtype=torch.float32, device="cuda")
    light = torch.empty_like(img)
    vxl.trace_soft_fwd(ctx, soft, sc["pos"], sc["nrm"], sc["npix"], sc["soft_params"], img, light)
    torch.cuda.synchronize()
    return img, light


def test_soft_forward_matches_fp64(vxl, ctx):
    sc = _scene(vxl, ctx)
    img, light = _fwd(vxl, ctx, sc)
    vox = sc["soft"].cpu().numpy()
    pos, nrm = sc["pos3"].cpu().numpy(), sc["nrm3"].cpu().numpy()
    want = oracle.soft_render(vox, pos, nrm, _oracle_params(sc["soft_params"]))
    got = img.cpu().numpy()
    assert np.abs(got - want).max() < 2e-5
    assert (want > 0).mean() > 0.3  # most pixels see a surface
    # image = surface albedo * light
    s = np.floor(pos - 0.5 * nrm).astype(np.int64)
    live = np.any(nrm != 0, 1) & np.all((s >= 0) & (s < sc["n"]), 1)
    rs = vox[s[live, 2], s[live, 1], s[live, 0], 1:]
    assert np.array_equal(got[live], (rs * light.cpu().numpy()[live]).astype(np.float32))
    assert not got[~live].any()


def test_soft_forward_deterministic(vxl, ctx):
    sc = _scene(vxl, ctx, n=32, W=40, H=30)
    a, la = _fwd(vxl, ctx, sc)
    b, lb = _fwd(vxl, ctx, sc)
    assert np.array_equal(a.cpu().numpy().view(np.int32), b.cpu().numpy().view(np.int32))
    assert np.array_equal(la.cpu().numpy().view(np.int32), lb.cpu().numpy().view(np.int32))


def test_soft_adjoint_matches_fp64_and_finite_differences(vxl, ctx):
    import torch

    sc = _scene(vxl, ctx)
    img, light = _fwd(vxl, ctx, sc)
    rng = np.random.default_rng(5)
    gi = rng.standard_normal((sc["npix"], 3)).astype(np.float32)
    grad = torch.zeros_like(sc["soft"])
    vxl.trace_soft_bwd(ctx, sc["soft"], sc["pos"], sc["nrm"], sc["npix"], sc["soft_params"], dev(gi), light, grad)
    torch.cuda.synchronize()
    got = grad.cpu().numpy().astype(np.float64)
    vox = sc["soft"].cpu().numpy()
    pos, nrm = sc["pos3"].cpu().numpy(), sc["nrm3"].cpu().numpy()
    op = _oracle_params(sc["soft_params"])
    _, want = oracle.soft_render(vox, pos, nrm, op, gi)
    for c in range(4):
        rel = np.linalg.norm(got[..., c] - want[..., c]) / np.linalg.norm(want[..., c])
        assert rel < 1e-3, (c, rel)
    assert np.count_nonzero(want[..., 0]) > 1000

    # FP64 central differences on 64 voxels (largest gradients, inside the clamp)
    a = vox[..., 0].ravel()
    ga = want[..., 0].ravel()
    cand = np.flatnonzero((a > 2e-4) & (a < AMAX - 2e-4) & (ga != 0))
    pick = cand[np.argsort(-np.abs(ga[cand]))[:64]]
    assert len(pick) == 64
    h = 1e-4

    def loss(v, d):
        return float((oracle.soft_render(vox, pos, nrm, op, perturb_voxel=v, perturb_delta=d) * gi).sum())

    fd = np.array([(loss(v, h) - loss(v, -h)) / (2 * h) for v in pick])
    g64 = got[..., 0].ravel()[pick]
    err = np.abs(g64 - fd) / np.maximum(np.abs(fd), 1e-3 * np.abs(fd).max())
    assert err.max() < 1e-3, err.max()


def test_soft_autograd_mse(vxl, ctx):
    """torch.autograd.Function around the kernels: MSE against a target
    rendered with a second albedo seed; the gradient equals the adjoint
    called directly with dL/dimage = 2 (I - I_t) / numel."""
    import torch

    from tests.soft_autograd import soft_occlusion

    sc = _scene(vxl, ctx, n=64, W=64, H=64, n_ao=16)
    tgt = _scene(vxl, ctx, n=64, W=64, H=64, n_ao=16, albedo_seed=2)
    with torch.no_grad():
        target = soft_occlusion(tgt["soft"], tgt["pos3"], tgt["nrm3"], tgt["soft_params"], ctx)
    soft = sc["soft"].clone().requires_grad_(True)
    img = soft_occlusion(soft, sc["pos3"], sc["nrm3"], sc["soft_params"], ctx)
    loss = ((img - target) ** 2).mean()
    loss.backward()
    img2, light = _fwd(vxl, ctx, sc)
    gi = (2.0 * (img2 - target) / img2.numel()).contiguous()
    grad = torch.zeros_like(sc["soft"])
    vxl.trace_soft_bwd(ctx, sc["soft"], sc["pos"], sc["nrm"], sc["npix"], sc["soft_params"], gi, light, grad)
    torch.cuda.synchronize()
    g1, g2 = soft.grad.cpu().numpy(), grad.cpu().numpy()
    assert np.abs(g1 - g2).max() <= 1e-5 * np.abs(g2).max()
    assert float(loss.detach()) > 0 and np.abs(g2).max() > 0


def test_soft_binary_opacity_is_the_dda_shadow(vxl, ctx):
    """With opacity 1 - 2^-12 on the bit grid's voxels and 0 elsewhere, the soft
    shadow transmittance is <= 2^-12 exactly where the DDA-mode occlusion pass
    reports a shadow hit (same rays, same cells)."""
    import torch

    from voxelengine_gb300 import scenes

    n, W, H, seed = 96, 80, 60, 6
    sc = scenes.make_scene(ctx, n, W, H, seed, boxes=20)
    G = sc["grid"]
    r8 = torch.zeros((n // 2) ** 3, dtype=torch.uint8, device="cuda")
    G.export_r8(r8)
    torch.cuda.synchronize()
    fine = oracle.r8_to_fine(r8.cpu().numpy().reshape(n // 2, n // 2, n // 2))
    vox = np.zeros((n, n, n, 4), np.float32)
    vox[..., 0] = np.where(fine, np.float32(AMAX), np.float32(0.0))
    vox[..., 1:] = 1.0
    soft = dev(vox)
    L = 40.0
    hp = vxl.make_params(light_dir=scenes.light_dir(seed), bias=0.5, shadow_len=L, ao_len=1.0, spec_len=1.0,
                         n_shadow=1, n_ao=0, n_spec=0, seed=seed)
    shadow = torch.empty(sc["npix"], dtype=torch.float32, device="cuda")
    vxl.trace_occlusion(ctx, G, sc["pos"], sc["nrm"], sc["rough"], sc["npix"], hp, shadow=shadow)
    sp = vxl.make_soft_params(light_dir=list(hp.light_dir), bias=0.5, length=L, k_sun=1.0, k_amb=0.0, n_shadow=1,
                              n_ao=0, seed=seed)
    sc["soft_params"] = sp
    img, light = _fwd(vxl, ctx, sc, soft=soft)
    pos, nrm = sc["pos"].view(-1, 3).cpu().numpy(), sc["nrm"].view(-1, 3).cpu().numpy()
    s = np.floor(pos - 0.5 * nrm).astype(np.int64)
    live = np.any(nrm != 0, 1) & np.all((s >= 0) & (s < n), 1)
    T = light.cpu().numpy()[live, 0]
    sh = shadow.cpu().numpy()[live]
    assert live.sum() > 0.3 * W * H
    assert np.array_equal(T <= 1.0 / 4096.0, sh == 0.0)
    assert (sh == 0.0).any() and (sh == 1.0).any()


def test_scene_soft_matches_noise_grid(vxl, ctx):
    import torch

    n = 64
    G = vxl.Grid(ctx, n, n, n)
    G.scene_noise(9, 0.55, 1.0 / 32.0, 8)
    soft = torch.empty((n, n, n, 4), dtype=torch.float32, device="cuda")
    vxl.scene_soft(ctx, soft, 9, 0.55, 8.0, 1.0 / 32.0, 8, 3)
    r8 = torch.zeros((n // 2) ** 3, dtype=torch.uint8, device="cuda")
    G.export_r8(r8)
    torch.cuda.synchronize()
    fine = oracle.r8_to_fine(r8.cpu().numpy().reshape(n // 2, n // 2, n // 2))
    v = soft.cpu().numpy()
    assert np.mean((v[..., 0] > 0.5) != fine) < 1e-4
    assert v[..., 1:].min() >= 0.0 and v[..., 1:].max() < 1.0
    assert np.all(v[:, :8, :, 0] == 1.0)  # ground slab y < 8 (array order z, y, x)


def test_soft_edge_cases(vxl, ctx):
    import torch

    sc = _scene(vxl, ctx, n=32, W=16, H=8)
    soft, pos, nrm, P = sc["soft"], sc["pos"], sc["nrm"], sc["soft_params"]
    img = torch.zeros((sc["npix"], 3), dtype=torch.float32, device="cuda")
    # no pixels: nothing to do
    vxl.trace_soft_fwd(ctx, soft, pos, nrm, 0, P, img)
    # zero normals and surfaces off the grid trace nothing
    z = torch.zeros_like(pos)
    vxl.trace_soft_fwd(ctx, soft, pos, z, sc["npix"], P, img)
    far = torch.full_like(pos, 1e4)
    img2 = torch.ones_like(img)
    vxl.trace_soft_fwd(ctx, soft, far, nrm, sc["npix"], P, img2)
    torch.cuda.synchronize()
    assert not img.any() and not img2.any()
    bad = [
        dict(n_shadow=2, n_ao=4),
        dict(n_shadow=1, n_ao=32),
        dict(n_shadow=0, n_ao=0),
    ]
    for kw in bad:
        Q = vxl.make_soft_params(**kw)
        with pytest.raises(vxl.VxlError) as e:
            vxl.trace_soft_fwd(ctx, soft, pos, nrm, sc["npix"], Q, img)
        assert e.value.status == vxl.VXL_ERR_INVALID_ARG
    odd = torch.zeros((31, 32, 32, 4), dtype=torch.float32, device="cuda")
    with pytest.raises(vxl.VxlError):
        vxl.trace_soft_fwd(ctx, odd, pos, nrm, sc["npix"], P, img)
    flat = torch.zeros(32 * 32 * 32 * 4 + 1, dtype=torch.float32, device="cuda")
    mis = flat[1:].view(32, 32, 32, 4)  # 4-byte aligned only
    with pytest.raises(vxl.VxlError):
        vxl.trace_soft_fwd(ctx, mis, pos, nrm, sc["npix"], P, img)
