"""The oracle's depth -> position step (vo_rebuild_from_depth, the placement
of LightAmbient.vert:32-36 / LightAmbient.frag:136-150) against a float64
restatement of the same formula, and its geometry: every texel's position lies
on the ray through that texel's NDC (row 0 is the top of the view), sky texels
are masked."""
import numpy as np

import oracle
from tests import view_cases as vc


def _frame(W, H, seed):
    rng = np.random.default_rng(seed)
    cam, tgt = np.array([3.0, 4.0, -6.0]), np.array([2.0, 1.0, 5.0])
    iv, ip, view, proj = vc.view_mats(cam, tgt, 0.57735026, W, H)
    # world points on random surfaces in front of the camera, through each texel's centre
    jj, ii = np.mgrid[0:H, 0:W]
    ndc = np.stack([(ii + 0.5) * 2 / W - 1, 1 - (jj + 0.5) * 2 / H], -1).reshape(-1, 2)
    far = np.c_[ndc, np.ones((W * H, 2))] @ np.linalg.inv(proj).T
    dirs_v = far[:, :3] / far[:, 3:]
    dist = rng.uniform(2.0, 60.0, W * H)
    pts_v = dirs_v / np.linalg.norm(dirs_v, axis=1, keepdims=True) * dist[:, None]
    cw = np.linalg.inv(view)
    pts_w = (np.c_[pts_v, np.ones(W * H)] @ cw.T)[:, :3]
    depth = vc.depth_of(pts_w, view)
    sky = rng.random(W * H) < 0.1
    depth[sky] = 1.0
    depth[:3] = [0.999, np.nan, 0.99899]
    nrm = rng.normal(size=(W * H, 3)).astype(np.float32)
    return iv, ip, depth, nrm, pts_w, cam


def test_rebuild_matches_float64_restatement():
    W, H = 37, 23
    iv, ip, depth, nrm, _, _ = _frame(W, H, 1)
    wcp, n2 = oracle.rebuild_from_depth(depth, nrm, W, H, iv, ip)
    IP = iv.reshape(4, 4).T.astype(np.float64), ip.reshape(4, 4).T.astype(np.float64)
    live = depth < 0.999
    jj, ii = np.mgrid[0:H, 0:W]
    ndc = np.stack([(ii + 0.5) * 2 / W - 1, 1 - (jj + 0.5) * 2 / H, np.ones_like(ii), np.ones_like(ii)],
                   -1).reshape(-1, 4)
    v = ndc @ IP[1].T
    pos = v[:, :3] / v[:, 3:] * (depth.astype(np.float64) * (1 + 1 / 4096))[:, None]
    want = (np.c_[pos, np.ones(W * H)] @ IP[0].T)[:, :3] * 10
    assert np.allclose(wcp[live], want[live], rtol=2e-5, atol=2e-4)
    assert not wcp[~live].any() and not n2[~live].any()
    assert np.array_equal(n2[live], nrm[live])
    # the three edge cases: 0.999 and NaN are sky, 0.99899 is not
    assert not live[0] and not live[1] and live[2]


def test_rebuild_places_texels_on_their_rays():
    W, H = 48, 30
    iv, ip, depth, nrm, pts_w, cam = _frame(W, H, 2)
    wcp, _ = oracle.rebuild_from_depth(depth, nrm, W, H, iv, ip)
    live = depth < 0.999
    live[:3] = False  # the edge-case depths planted in the first texels lie off their surfaces
    a = wcp[live] / 10.0 - cam
    b = pts_w[live] - cam
    cosang = (a * b).sum(1) / np.linalg.norm(a, axis=1) / np.linalg.norm(b, axis=1)
    assert cosang.min() > 1 - 1e-6  # same direction from the camera
    # the pass's placement puts the point at FarVec * depth * (1 + 1/FAR): about
    # (1 - NEAR / w) of the true distance
    ratio = np.linalg.norm(a, axis=1) / np.linalg.norm(b, axis=1)
    w = np.linalg.norm(b, axis=1)  # >= the view depth; the bound below allows for it
    assert np.all(ratio > 1 - 0.1 / w * 1.5 - 1e-4) and np.all(ratio < 1 + 3e-4)
    # row 0 is the top of the view: for this upright camera its rays point higher
    dirs_top = (wcp.reshape(H, W, 3)[0][live.reshape(H, W)[0]] / 10 - cam)
    dirs_bot = (wcp.reshape(H, W, 3)[-1][live.reshape(H, W)[-1]] / 10 - cam)
    el = lambda d: (d[:, 1] / np.linalg.norm(d, axis=1)).mean()
    assert el(dirs_top) > el(dirs_bot)
