"""CUDA path vs the oracle, through libvxl's C ABI: ray records (hit cell,
t bits, fetch count, exit reason) must be identical, and so must the grids
and the occlusion buffers (bit-exact: both sides are IEEE fp32 without
contraction)."""
import numpy as np
import pytest

import oracle
from tests import cases
from tests.gpu_util import assert_recs_equal, dev, empty, export_r8, grid_from_r8, rec_buffer, recs_np, same_bits

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def g64():
    return cases.noise_grid(64, seed=3)


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_trace_rays_bit_exact(vxl, ctx, g64, mode):
    import torch

    G = grid_from_r8(vxl, ctx, g64)
    rays = np.concatenate([cases.edge_rays(64), cases.random_rays(64, 50000, seed=21 + mode)])
    want = oracle.trace_rays(g64, rays, mode=mode)
    rec = rec_buffer(len(rays))
    vxl.trace_rays(ctx, G, dev(rays), len(rays), mode, rec)
    torch.cuda.synchronize()
    assert_recs_equal(recs_np(rec), want, "mode %d" % mode)
    assert (want["flags"] & 1).any() and not (want["flags"] & 1).all()


def test_grid_roundtrip_and_count(vxl, ctx):
    import torch

    rng = np.random.default_rng(5)
    for dims in [(64, 64, 64), (6, 10, 14), (130, 66, 34)]:
        f = rng.random(dims[::-1]) < 0.3
        r8 = oracle.fine_to_r8(f)
        G = grid_from_r8(vxl, ctx, r8)
        assert np.array_equal(export_r8(G), r8)
        assert G.count() == int(f.sum())
        pal = np.where(f, rng.integers(16, 256, f.shape), rng.integers(0, 16, f.shape)).astype(np.uint8)
        G2 = vxl.Grid(ctx, *dims)
        G2.import_palette(dev(pal), 16)
        assert np.array_equal(export_r8(G2), r8)
        G.clear()
        assert G.count() == 0


def test_scene_generators_match_oracle(vxl, ctx):
    import torch

    for n, seed in [(64, 1), (256, 2)]:
        G = vxl.Grid(ctx, n, n, n)
        G.scene_noise(seed, 0.55, 1.0 / 32.0, 8)
        G.scene_boxes(seed, 50, 4, 48)
        want = oracle.scene_noise(n, n, n, seed=seed)
        oracle.scene_boxes(want, seed, 50, 4, 48)
        assert np.array_equal(export_r8(G), want)


def _c1_scene(vxl, ctx, n=256, W=640, H=360, seed=7):
    import torch

    G = vxl.Grid(ctx, n, n, n)
    G.scene_noise(seed, 0.55, 1.0 / 32.0, 8)
    cam = np.array([-0.35 * n, 0.9 * n, -0.45 * n], np.float32)
    tgt = np.array([n / 2, n / 2, n / 2], np.float32)
    pos, nrm, rough = empty(W * H * 3, torch.float32), empty(W * H * 3, torch.float32), empty(W * H, torch.float32)
    vxl.scene_gbuffer(ctx, G, cam, tgt, W, H, seed, pos, nrm, rough)
    return G, cam, tgt, pos, nrm, rough


def test_gbuffer_matches_oracle(vxl, ctx):
    import torch

    n, W, H = 128, 320, 180
    G, cam, tgt, pos, nrm, rough = _c1_scene(vxl, ctx, n, W, H)
    g = export_r8(G)
    p2, n2, r2 = oracle.gbuffer(g, cam, tgt, W, H, 7)
    torch.cuda.synchronize()
    assert same_bits(pos.cpu().numpy().reshape(-1, 3), p2).all()
    assert np.array_equal(nrm.cpu().numpy().reshape(-1, 3), n2)
    assert np.array_equal(rough.cpu().numpy(), r2)
    assert (np.abs(n2).sum(1) > 0).mean() > 0.3  # the camera sees mostly geometry


@pytest.mark.parametrize("n_spec,kstep", [(0, 0), (1, 0), (1, 4), (1, 16)])
def test_occlusion_c1_bit_exact(vxl, ctx, n_spec, kstep):
    """C1: 256^3 noise grid, 640x360 G-buffer, 1 shadow + 4 AO (L=16) [+ 1 GGX spec];
    the trace-layout kernel also with batches of 4 and 16 DDA iterations
    (tuning kstep; 0 = the default 8)."""
    import torch

    G, cam, tgt, pos, nrm, rough = _c1_scene(vxl, ctx)
    npix = 640 * 360
    P = vxl.make_params(light_dir=(0.3, 0.8, 0.5), cam_pos=cam, n_ao=4, ao_len=16.0, n_spec=n_spec, seed=99)
    R = 1 + 4 + n_spec
    outs = {k: empty(npix, torch.float32) for k in ("shadow", "ao", "ao_vis", "spec", "spec_t")}
    rec = rec_buffer(npix * R)
    vxl.trace_occlusion(ctx, G, pos, nrm, rough, npix, P, records=rec, **outs)
    torch.cuda.synchronize()
    g = export_r8(G)
    OP = oracle.make_params(light_dir=(0.3, 0.8, 0.5), cam_pos=cam, n_ao=4, ao_len=16.0, n_spec=n_spec, seed=99)
    want = oracle.occlusion(g, pos.cpu().numpy(), nrm.cpu().numpy(), rough.cpu().numpy(), OP, with_recs=True)
    assert_recs_equal(recs_np(rec), want["recs"], "records")
    for k in outs:
        assert same_bits(outs[k].cpu().numpy(), want[k]).all(), k
    # without records (the trace-layout kernel): same buffers
    outs2 = {k: empty(npix, torch.float32) for k in outs}
    before = ctx.get_tuning()
    try:
        if kstep:
            ctx.set_tuning(kstep=kstep)
        vxl.trace_occlusion(ctx, G, pos, nrm, rough, npix, P, **outs2)
        torch.cuda.synchronize()
    finally:
        ctx.set_tuning(**before)
    for k in outs:
        assert torch.equal(outs[k], outs2[k]), k


@pytest.mark.parametrize("light", [(0.0, 0.8, 0.6), (0.0, 1.0, 0.0)])
def test_occlusion_literal_rays_bit_exact(vxl, ctx, light):
    """Shadow rays whose direction has zero components take the literal
    4-pass form of raycastShadowVolume (Light.frag:29-81), traced after the
    trace-layout kernel's stepping loop: C1 scene, outputs and records equal
    to the oracle, and the same buffers without records."""
    import torch

    G, cam, tgt, pos, nrm, rough = _c1_scene(vxl, ctx)
    npix = 640 * 360
    kw = dict(light_dir=light, cam_pos=cam, n_ao=4, ao_len=16.0, n_spec=1, seed=7)
    P = vxl.make_params(**kw)
    outs = {k: empty(npix, torch.float32) for k in ("shadow", "ao", "ao_vis", "spec", "spec_t")}
    rec = rec_buffer(npix * 6)
    vxl.trace_occlusion(ctx, G, pos, nrm, rough, npix, P, records=rec, **outs)
    outs2 = {k: empty(npix, torch.float32) for k in outs}
    vxl.trace_occlusion(ctx, G, pos, nrm, rough, npix, P, width=640, height=360, **outs2)
    torch.cuda.synchronize()
    want = oracle.occlusion(export_r8(G), pos.cpu().numpy(), nrm.cpu().numpy(), rough.cpu().numpy(),
                            oracle.make_params(**kw), with_recs=True)
    assert_recs_equal(recs_np(rec), want["recs"], "records")
    for k in outs:
        assert same_bits(outs[k].cpu().numpy(), want[k]).all(), k
        assert torch.equal(outs[k], outs2[k]), k
    # (with a zero direction component the reference's t_max for that axis is 0/0 or x/0, and its loop
    # reports no hit: every shadow ray is lit, here as in the oracle)


@pytest.mark.parametrize("scene,ao_len,shadow_len", [("boxes", 32.0, 100.0), ("boxes", 64.0, 130.0),
                                                     ("noise", 24.0, 60.0)])
def test_occlusion_leap_matches_exact(vxl, ctx, scene, ao_len, shadow_len):
    """With the leap enabled (tuning leap = 1) and no per-ray records, the
    kernel crosses empty bricks in one leap; its buffers, those of the default
    exact stepping (8-pixel tiles at 14 rays per pixel) and those of the
    records mode must all equal the oracle."""
    import torch

    n, W, H = 192, 320, 200
    G = vxl.Grid(ctx, n, n, n)
    if scene == "boxes":
        G.scene_boxes(11, 60, 2, 30)
    else:
        G.scene_noise(12, 0.62, 1.0 / 16.0, 4)
    cam = np.array([0.5 * n, 1.1 * n, -0.2 * n], np.float32)
    tgt = np.array([n / 2] * 3, np.float32)
    npix = W * H
    pos, nrm, rough = empty(npix * 3, torch.float32), empty(npix * 3, torch.float32), empty(npix, torch.float32)
    vxl.scene_gbuffer(ctx, G, cam, tgt, W, H, 5, pos, nrm, rough)
    P = vxl.make_params(light_dir=(-0.2, 0.9, 0.4), cam_pos=cam, n_ao=12, ao_len=ao_len, shadow_len=shadow_len,
                        n_spec=1, seed=17)
    keys = ("shadow", "ao", "ao_vis", "spec", "spec_t")
    leap = {k: empty(npix, torch.float32) for k in keys}
    exact = {k: empty(npix, torch.float32) for k in keys}
    plain = {k: empty(npix, torch.float32) for k in keys}
    before = ctx.get_tuning()
    try:
        ctx.set_tuning(leap=1)
        vxl.trace_occlusion(ctx, G, pos, nrm, rough, npix, P, **leap)
        torch.cuda.synchronize()
    finally:
        ctx.set_tuning(**before)
    vxl.trace_occlusion(ctx, G, pos, nrm, rough, npix, P, **plain)
    vxl.trace_occlusion(ctx, G, pos, nrm, rough, npix, P, records=rec_buffer(npix * 14), **exact)
    torch.cuda.synchronize()
    OP = oracle.make_params(light_dir=(-0.2, 0.9, 0.4), cam_pos=cam, n_ao=12, ao_len=ao_len, shadow_len=shadow_len,
                            n_spec=1, seed=17)
    want = oracle.occlusion(export_r8(G), pos.cpu().numpy(), nrm.cpu().numpy(), rough.cpu().numpy(), OP)
    for k in keys:
        assert same_bits(leap[k].cpu().numpy(), exact[k].cpu().numpy()).all(), k
        assert same_bits(leap[k].cpu().numpy(), want[k]).all(), k
        assert same_bits(plain[k].cpu().numpy(), want[k]).all(), k
    assert 0.0 < float(leap["shadow"].mean()) < 1.0


@pytest.mark.parametrize("pinned", [True, False])
def test_occlusion_host_entry_matches_device(vxl, ctx, pinned):
    """Host buffers: pinned ones are read and written in place by the kernel,
    pageable ones go through staged copies; both equal the device call."""
    import torch

    G, cam, tgt, pos, nrm, rough = _c1_scene(vxl, ctx, 128, 200, 120)
    npix = 200 * 120
    P = vxl.make_params(cam_pos=cam, n_ao=8, ao_len=32.0, n_spec=1, seed=3)
    outs = {k: empty(npix, torch.float32) for k in ("shadow", "ao", "ao_vis", "spec", "spec_t")}
    vxl.trace_occlusion(ctx, G, pos, nrm, rough, npix, P, **outs)
    pin = (lambda t: t.pin_memory()) if pinned else (lambda t: t)
    hp, hn, hr = pin(pos.cpu()), pin(nrm.cpu()), pin(rough.cpu())
    hout = {k: pin(torch.zeros(npix, dtype=torch.float32)) for k in outs}
    vxl.trace_occlusion_host(ctx, G, hp, hn, hr, npix, P, h_shadow=hout["shadow"], h_ao=hout["ao"],
                             h_ao_vis=hout["ao_vis"], h_spec=hout["spec"], h_spec_t=hout["spec_t"])
    torch.cuda.synchronize()
    for k in outs:
        assert torch.equal(outs[k].cpu(), hout[k]), k


@pytest.mark.parametrize("W,H,n_ao,pinned", [(1280, 720, 6, False), (1333, 777, 6, False), (1024, 640, 16, False),
                                              (1333, 777, 6, True)])
def test_occlusion_host_pipeline_matches_one_launch(vxl, ctx, W, H, n_ao, pinned):
    """Pageable host buffers of >= 2^19 pixels go through the chunked
    copy/compute pipeline (pixel chunks on two streams, global pixel index
    seeding the rays), pinned ones are used in place: the outputs equal the
    one-launch device call bit for bit. With 18 rays per pixel both run
    8-pixel tiles."""
    import torch

    G, cam, tgt, pos, nrm, rough = _c1_scene(vxl, ctx, 128, W, H)
    npix = W * H
    P = vxl.make_params(cam_pos=cam, n_ao=n_ao, ao_len=24.0, n_spec=1, seed=5)
    outs = {k: empty(npix, torch.float32) for k in ("shadow", "ao", "ao_vis", "spec", "spec_t")}
    vxl.trace_occlusion(ctx, G, pos, nrm, rough, npix, P, **outs)
    pin = (lambda t: t.pin_memory()) if pinned else (lambda t: t)
    hp, hn, hr = pin(pos.cpu()), pin(nrm.cpu()), pin(rough.cpu())
    hout = {k: pin(torch.full((npix,), -3.0, dtype=torch.float32)) for k in outs}
    vxl.trace_occlusion_host(ctx, G, hp, hn, hr, npix, P, h_shadow=hout["shadow"], h_ao=hout["ao"],
                             h_ao_vis=hout["ao_vis"], h_spec=hout["spec"], h_spec_t=hout["spec_t"])
    torch.cuda.synchronize()
    for k in outs:
        assert torch.equal(outs[k].cpu(), hout[k]), k


def test_light_passes_bit_exact(vxl, ctx, g64):
    import torch

    G = grid_from_r8(vxl, ctx, g64)
    rng = np.random.default_rng(8)
    n = 20000
    axes = np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1]], np.float32)
    wcp = rng.uniform(-4, 68, (n, 3)).astype(np.float32)
    nrm = axes[rng.integers(0, 6, n)]
    depth = rng.uniform(0, 0.3, n).astype(np.float32)
    noise = rng.random((n, 4)).astype(np.float32)
    rough = rng.uniform(0.05, 1, n).astype(np.float32)
    vr = rng.normal(size=(n, 3)).astype(np.float32)
    sh, irr, r_amb = oracle.light_ambient(g64, wcp, nrm, depth, noise)
    d_sh, d_irr, d_rec = empty(n, torch.float32), empty(n, torch.float32), rec_buffer(2 * n)
    vxl.light_ambient(ctx, G, dev(wcp), dev(nrm), dev(depth), dev(noise), n, d_sh, d_irr, d_rec)
    t, r_ref = oracle.light_reflection(g64, wcp, nrm, vr, rough, noise)
    d_t, d_rec2 = empty(n, torch.float32), rec_buffer(n)
    vxl.light_reflection(ctx, G, dev(wcp), dev(nrm), dev(vr), dev(rough), dev(noise), n, d_t, d_rec2)
    torch.cuda.synchronize()
    assert np.array_equal(d_sh.cpu().numpy(), sh)
    assert same_bits(d_irr.cpu().numpy(), irr).all()
    assert_recs_equal(recs_np(d_rec), r_amb, "ambient")
    assert same_bits(d_t.cpu().numpy(), t).all()
    assert_recs_equal(recs_np(d_rec2), r_ref, "reflection")
    wpos = rng.uniform(0.2, 6.2, (n, 3)).astype(np.float32)
    for spot in (False, True):
        lp = np.array([3.2, 4.1, 2.7], np.float32)
        want, r_pt = oracle.light_point(g64, wpos, nrm, noise, lp, 2.5, spot=spot)
        d_s = dev(np.full(n, -7.0, np.float32))
        d_rec3 = rec_buffer(n)
        vxl.light_point(ctx, G, dev(wpos), dev(nrm), dev(noise), n, lp, 2.5, spot, d_s, d_rec3)
        torch.cuda.synchronize()
        assert np.array_equal(d_s.cpu().numpy(), want), spot
        assert_recs_equal(recs_np(d_rec3), r_pt, "point/spot")


def test_light_points_fused_matches_per_light(vxl, ctx, g64):
    """vxl_light_points (64 point and spot lights in one launch) against the
    oracle's per-light pass: bit l of the masks = in range / in range and lit."""
    import torch

    G = grid_from_r8(vxl, ctx, g64)
    rng = np.random.default_rng(17)
    n = 12000
    axes = np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1]], np.float32)
    wpos = rng.uniform(0.2, 6.2, (n, 3)).astype(np.float32)
    nrm = axes[rng.integers(0, 6, n)]
    noise = rng.random((n, 4)).astype(np.float32)
    lights = [(rng.uniform(0.5, 6.0, 3).astype(np.float32), float(rng.uniform(0.8, 4.0)), bool(l % 3 == 2))
              for l in range(64)]
    lit = torch.full((n,), -1, dtype=torch.int64, device="cuda")
    inr = torch.full((n,), -1, dtype=torch.int64, device="cuda")
    vxl.light_points(ctx, G, dev(wpos), dev(nrm), dev(noise), n, lights, lit, inr)
    torch.cuda.synchronize()
    got_lit = lit.cpu().numpy().view(np.uint64)
    got_in = inr.cpu().numpy().view(np.uint64)
    want_lit = np.zeros(n, np.uint64)
    want_in = np.zeros(n, np.uint64)
    for l, (lp, r, spot) in enumerate(lights):
        sh, _ = oracle.light_point(g64, wpos, nrm, noise, lp, r, spot=spot, init=np.full(n, -7.0, np.float32))
        b = np.uint64(1) << np.uint64(l)
        want_in |= np.where(sh != -7.0, b, np.uint64(0))
        want_lit |= np.where(sh == 1.0, b, np.uint64(0))
    assert np.array_equal(got_in, want_in)
    assert np.array_equal(got_lit, want_lit)
    assert (want_in != 0).mean() > 0.5 and (want_in != want_lit).any()
    with pytest.raises(vxl.VxlError):
        vxl.light_points(ctx, G, dev(wpos), dev(nrm), dev(noise), n, lights + lights[:1], lit)


def test_light_points_warp_culling_is_exact(vxl, ctx, g64):
    """Positions laid out like an image (each warp's 32 pixels close together)
    so that warps skip the lights whose sphere misses their box; pixels placed
    at exactly a light's range, a warp of one repeated boundary position, NaN
    and infinite positions: masks equal the oracle's per-light pass."""
    import torch

    G = grid_from_r8(vxl, ctx, g64)
    rng = np.random.default_rng(23)
    side = 96
    n = side * side
    u, v = np.meshgrid(np.arange(side), np.arange(side))
    wpos = np.stack([0.2 + u * 0.063, 1.5 + 0.8 * np.sin(u * 0.07) * np.cos(v * 0.05), 0.2 + v * 0.063],
                    -1).reshape(n, 3).astype(np.float32)
    axes = np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1]], np.float32)
    nrm = axes[rng.integers(0, 6, n)]
    noise = rng.random((n, 4)).astype(np.float32)
    lights = [(rng.uniform(0.3, 6.0, 3).astype(np.float32), float(rng.uniform(0.3, 1.2)), bool(l % 3 == 2))
              for l in range(64)]
    # pixels at exactly a light's range along an axis, and a whole warp at one such point
    for j in range(40):
        lp, r, _ = lights[j]
        wpos[j * 37 + 5] = lp + np.float32(r) * axes[j % 6]
    lp, r, _ = lights[3]
    wpos[32 * 100:32 * 101] = lp + np.float32(r) * axes[2]
    wpos[32 * 50 + 7] = np.nan
    wpos[32 * 60 + 3] = [np.inf, 1.0, 1.0]
    wpos[32 * 61 + 9] = [-np.inf, np.inf, 2.0]
    lit = torch.full((n,), -1, dtype=torch.int64, device="cuda")
    inr = torch.full((n,), -1, dtype=torch.int64, device="cuda")
    vxl.light_points(ctx, G, dev(wpos), dev(nrm), dev(noise), n, lights, lit, inr)
    torch.cuda.synchronize()
    want_lit = np.zeros(n, np.uint64)
    want_in = np.zeros(n, np.uint64)
    for l, (lp, r, spot) in enumerate(lights):
        sh, _ = oracle.light_point(g64, wpos, nrm, noise, lp, r, spot=spot, init=np.full(n, -7.0, np.float32))
        b = np.uint64(1) << np.uint64(l)
        want_in |= np.where(sh != -7.0, b, np.uint64(0))
        want_lit |= np.where(sh == 1.0, b, np.uint64(0))
    assert np.array_equal(inr.cpu().numpy().view(np.uint64), want_in)
    assert np.array_equal(lit.cpu().numpy().view(np.uint64), want_lit)
    # the layout lets warps skip most lights: few pairs are in range
    bits = sum(bin(int(x)).count("1") for x in want_in)
    assert 0 < bits < n * 64 * 0.2


def test_light_points_pair_list_overflow_is_exact(vxl, ctx, g64):
    """Every (pixel, light) pair in range: far more pairs than the list holds
    (two per pixel), so most are traced in the first pass; masks equal the
    oracle's per-light pass."""
    import torch

    G = grid_from_r8(vxl, ctx, g64)
    rng = np.random.default_rng(29)
    n = 20000
    axes = np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1]], np.float32)
    wpos = rng.uniform(0.2, 6.2, (n, 3)).astype(np.float32)
    nrm = axes[rng.integers(0, 6, n)]
    noise = rng.random((n, 4)).astype(np.float32)
    lights = [(rng.uniform(0.5, 6.0, 3).astype(np.float32), 100.0, bool(l % 3 == 2)) for l in range(64)]
    lit = torch.full((n,), -1, dtype=torch.int64, device="cuda")
    inr = torch.full((n,), -1, dtype=torch.int64, device="cuda")
    vxl.light_points(ctx, G, dev(wpos), dev(nrm), dev(noise), n, lights, lit, inr)
    torch.cuda.synchronize()
    want_lit = np.zeros(n, np.uint64)
    for l, (lp, r, spot) in enumerate(lights):
        sh, _ = oracle.light_point(g64, wpos, nrm, noise, lp, r, spot=spot, init=np.full(n, -7.0, np.float32))
        want_lit |= np.where(sh == 1.0, np.uint64(1) << np.uint64(l), np.uint64(0))
    assert np.array_equal(inr.cpu().numpy().view(np.uint64), np.full(n, np.uint64(2**64 - 1)))
    assert np.array_equal(lit.cpu().numpy().view(np.uint64), want_lit)
    assert (want_lit != 0).any() and (want_lit != np.uint64(2**64 - 1)).any()
