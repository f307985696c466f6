"""The FP64 adjoint of the soft-opacity model (oracle) against FP64 central
finite differences, and the soft walk against the reference DDA: with opacity
(1 - 2^-12) on occupied voxels and 0 elsewhere, a shadow ray's transmittance
falls to 2^-12 or below exactly when the reference DDA reports a hit."""
import numpy as np

import oracle

AMAX = 1.0 - 1.0 / 4096.0


def _soft_grid(rng, n, fill=0.3):
    vox = np.zeros((n, n, n, 4), np.float32)
    on = rng.random((n, n, n)) < fill
    vox[..., 0] = np.where(on, rng.uniform(0.02, 0.9, (n, n, n)), 0.0)
    vox[..., 1:] = rng.uniform(0.1, 1.0, (n, n, n, 3))
    return vox


def _floor_points(rng, n, npix, y=4.0):
    pos = np.stack([rng.uniform(2, n - 2, npix), np.full(npix, y), rng.uniform(2, n - 2, npix)], 1)
    nrm = np.tile([0.0, 1.0, 0.0], (npix, 1))
    return pos.astype(np.float32), nrm.astype(np.float32)


def test_soft_adjoint_matches_finite_differences(oracle_lib):
    rng = np.random.default_rng(11)
    n = 24
    vox = _soft_grid(rng, n)
    pos, nrm = _floor_points(rng, n, 96)
    p = oracle.make_soft_params(light_dir=(0.3, 0.8, 0.5), length=14.0, n_shadow=1, n_ao=6, seed=5)
    gi = rng.standard_normal((96, 3)).astype(np.float32)
    _, g = oracle.soft_render(vox, pos, nrm, p, gi)

    def loss(v, d):
        return float((oracle.soft_render(vox, pos, nrm, p, perturb_voxel=v, perturb_delta=d) * gi).sum())

    # 64 voxels with the largest opacity gradients, away from the clamp's kinks
    a = vox[..., 0].ravel()
    ga = g[..., 0].ravel()
    inside = (a > 2e-4) & (a < AMAX - 2e-4)
    cand = np.flatnonzero(inside & (ga != 0))
    pick = cand[np.argsort(-np.abs(ga[cand]))[:64]]
    assert len(pick) == 64
    h = 1e-4
    fd = np.array([(loss(v, h) - loss(v, -h)) / (2 * h) for v in pick])
    scale = np.abs(fd).max()
    err = np.abs(ga[pick] - fd) / np.maximum(np.abs(fd), 1e-3 * scale)
    assert err.max() < 1e-5, err.max()


def test_soft_albedo_gradient_is_exact_derivative(oracle_lib):
    rng = np.random.default_rng(12)
    n = 16
    vox = _soft_grid(rng, n, fill=0.4)
    pos, nrm = _floor_points(rng, n, 48)
    p = oracle.make_soft_params(length=10.0, n_shadow=1, n_ao=4, seed=9)
    gi = rng.standard_normal((48, 3)).astype(np.float32)
    _, g = oracle.soft_render(vox, pos, nrm, p, gi)
    gr = g[..., 1:].reshape(-1, 3)
    flat = vox.reshape(-1, 4)
    picks = np.argsort(-np.abs(gr).sum(1))[:12]
    for v in picks:
        for ch in range(3):
            vp, vm = vox.copy(), vox.copy()
            vp.reshape(-1, 4)[v, 1 + ch] += np.float32(0.05)
            vm.reshape(-1, 4)[v, 1 + ch] -= np.float32(0.05)
            dp = float(vp.reshape(-1, 4)[v, 1 + ch]) - float(flat[v, 1 + ch])
            dm = float(flat[v, 1 + ch]) - float(vm.reshape(-1, 4)[v, 1 + ch])
            lp = float((oracle.soft_render(vp, pos, nrm, p) * gi).sum())
            lm = float((oracle.soft_render(vm, pos, nrm, p) * gi).sum())
            fd = (lp - lm) / (dp + dm)  # the image is linear in each albedo value
            assert abs(fd - gr[v, ch]) <= 1e-9 + 1e-7 * abs(fd), (v, ch, fd, gr[v, ch])


def test_soft_walk_is_the_reference_dda(oracle_lib):
    """Binary opacity: the soft shadow ray and the reference DDA agree on every pixel."""
    n = 64
    g = oracle.scene_noise(n, n, n, seed=4, thresh=0.55, freq=1.0 / 16.0, ground_y=6)
    oracle.scene_boxes(g, 4, 12, 2, 10)
    fine = oracle.r8_to_fine(g)
    vox = np.zeros((n, n, n, 4), np.float32)
    vox[..., 0] = np.where(fine, np.float32(AMAX), np.float32(0.0))
    vox[..., 1:] = 1.0
    W, H = 48, 40
    pos, nrm, rough = oracle.gbuffer(g, (n * 1.2, n * 0.9, -n * 0.3), (n * 0.5, n * 0.2, n * 0.5), W, H, 4)
    pos = pos.reshape(-1, 3)
    nrm = nrm.reshape(-1, 3)
    L = 40.0
    light = (0.35, 0.8, 0.45)
    hard = oracle.make_params(light_dir=light, bias=0.5, shadow_len=L, n_shadow=1, n_ao=0, n_spec=0, seed=1)
    sh = oracle.occlusion(g, pos, nrm, rough, hard)["shadow"]
    sp = oracle.make_soft_params(light_dir=list(hard.light_dir), bias=0.5, length=L, k_sun=1.0, k_amb=0.0, n_shadow=1, n_ao=0)
    img = oracle.soft_render(vox, pos, nrm, sp)
    # surface voxels lie in the grid for these pixels; sky pixels trace nothing
    live = np.any(nrm != 0, axis=1)
    s = np.floor(pos - 0.5 * nrm).astype(int)
    live &= np.all((s >= 0) & (s < n), axis=1)
    assert live.sum() > 0.5 * W * H
    T = img[live, 0]
    assert np.array_equal(T <= 1.0 / 4096.0 + 1e-12, sh[live] == 0.0)
    assert (sh[live] == 0.0).any() and (sh[live] == 1.0).any()
