"""Seeded synthetic scene sets for benchmarks and tests (device-generated).

A scene is a noise grid (3-octave value noise at frequency 1/32, threshold
`thresh`, ground slab y < 8), optional boxes and voxelized Vox-model
instances, and a primary-hit G-buffer from a camera outside the grid looking
at its centre. Device buffers are torch CUDA tensors.
"""
from __future__ import annotations

import math

import numpy as np

import voxelengine_gb300 as V


def camera(n):
    """Above and in front of an n^3 grid, looking at its centre."""
    cam = np.array([0.5 * n, 1.15 * n, -0.1 * n], np.float32)
    tgt = np.array([0.5 * n, 0.5 * n, 0.5 * n], np.float32)
    return cam, tgt


def light_dir(seed):
    rng = np.random.default_rng(seed)
    v = rng.normal(size=3)
    v[1] = abs(v[1]) + 0.8  # above the horizon
    return (v / np.linalg.norm(v)).astype(np.float32)


def image_for_pixels(npix):
    """16:9-ish W x H with about npix pixels."""
    h = max(8, int(round(math.sqrt(npix * 9.0 / 16.0))))
    w = max(8, int(round(npix / h)))
    return w, h


def rotation_matrix(rng):
    """Uniform random rotation (unit quaternion from three uniforms, Shoemake)."""
    u1, u2, u3 = rng.random(3)
    x = math.sqrt(1 - u1) * math.sin(2 * math.pi * u2)
    y = math.sqrt(1 - u1) * math.cos(2 * math.pi * u2)
    z = math.sqrt(u1) * math.sin(2 * math.pi * u3)
    w = math.sqrt(u1) * math.cos(2 * math.pi * u3)
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def vox_models(seed, count, edge_min=8, edge_max=64, fill=0.4):
    """Dense uint8 palette blocks [sz, sy, sx]: opaque indices 16..255 with
    probability `fill`, a few glass indices 1..15, zeros elsewhere."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        sx, sy, sz = (int(v) for v in rng.integers(edge_min, edge_max + 1, 3))
        m = rng.integers(16, 256, (sz, sy, sx)).astype(np.uint8)
        m[rng.random((sz, sy, sx)) >= fill] = 0
        glass = rng.random((sz, sy, sx)) < 0.02
        m[glass] = rng.integers(1, 16, int(glass.sum())).astype(np.uint8)
        out.append(m)
    return out


def instance_matrix(rng, n, model_shape):
    """Column-major 4x4: uniform rotation, model centre inside an n^3 grid
    (positions in world units: 10 fine voxels per unit)."""
    m = np.eye(4)
    R = rotation_matrix(rng)
    m[:3, :3] = R
    sz, sy, sx = model_shape
    half = 0.05 * np.array([sx, sy, sz])  # model half extent in world units
    centre = rng.uniform(0.0, n / 10.0, 3)
    m[:3, 3] = centre - R @ half
    return np.ascontiguousarray(m.T.astype(np.float32)).reshape(16)


def make_scene(ctx, n, W, H, seed, thresh=0.55, boxes=0, params=None, device_tensors=True, palette=False):
    """palette: give the grid its 4-bit palette plane with seeded indices for
    the set voxels (vxl_scene_palette); the traversal does not read it."""
    import torch

    G = V.Grid(ctx, n, n, n)
    G.scene_noise(seed, thresh, 1.0 / 32.0, 8)
    if boxes:
        G.scene_boxes(seed, boxes, 4, 48)
    if palette:
        G.palette_alloc()
        G.scene_palette(seed)
    cam, tgt = camera(n)
    npix = W * H
    pos = torch.empty(npix * 3, dtype=torch.float32, device="cuda")
    nrm = torch.empty_like(pos)
    rough = torch.empty(npix, dtype=torch.float32, device="cuda")
    V.scene_gbuffer(ctx, G, cam, tgt, W, H, seed, pos, nrm, rough)
    P = params or V.make_params(light_dir=light_dir(seed), cam_pos=cam, bias=0.5, shadow_len=100.0, ao_len=32.0,
                                spec_len=256.0, n_shadow=1, n_ao=8, n_spec=1, seed=seed)
    return dict(grid=G, n=n, W=W, H=H, width=W, height=H, npix=npix, pos=pos, nrm=nrm, rough=rough, params=P,
                cam=cam, seed=seed)


def make_soft_scene(ctx, n, W, H, seed, albedo_seed=1, thresh=0.55, sharpness=8.0, params=None):
    """Differentiable workload: soft grid [n,n,n,4] with opacity
    sigmoid(sharpness * (noise - thresh)) and uniform albedo, plus the G-buffer
    of the matching binary scene (the voxels with opacity > 0.5)."""
    import torch

    sc = make_scene(ctx, n, W, H, seed, thresh=thresh)
    soft = torch.empty((n, n, n, 4), dtype=torch.float32, device="cuda")
    V.scene_soft(ctx, soft, seed, thresh, sharpness, 1.0 / 32.0, 8, albedo_seed)
    P = params or V.make_soft_params(light_dir=light_dir(seed), bias=0.5, length=24.0, k_sun=0.7, k_amb=0.5,
                                     n_shadow=1, n_ao=16, seed=seed)
    sc.update(soft=soft, soft_params=P, pos3=sc["pos"].view(-1, 3), nrm3=sc["nrm"].view(-1, 3))
    return sc


def batch_set(ctx, count=64, seed=7, edge_range=(64, 512), rays_range=(64 * 1024, 2 * 1024 * 1024),
              thresh_range=(0.45, 0.65), rays_per_pixel=10, palette=False):
    """The uneven scene mix: edges log-uniform in edge_range (even), noise
    threshold uniform in thresh_range, rays per scene log-uniform in rays_range."""
    rng = np.random.default_rng(seed)
    scenes = []
    for i in range(count):
        n = int(round(math.exp(rng.uniform(math.log(edge_range[0]), math.log(edge_range[1]))) / 2)) * 2
        rays = math.exp(rng.uniform(math.log(rays_range[0]), math.log(rays_range[1])))
        W, H = image_for_pixels(rays / rays_per_pixel)
        thresh = float(rng.uniform(*thresh_range))
        scenes.append(make_scene(ctx, n, W, H, seed * 1000 + i, thresh=thresh, palette=palette))
    return scenes


def add_outputs(scene):
    import torch

    for k in ("shadow", "ao", "ao_vis", "spec", "spec_t"):
        scene[k] = torch.empty(scene["npix"], dtype=torch.float32, device="cuda")
    return scene


def instance_set(scenes, n_instances, models, seed):
    """n_instances placements spread uniformly over the scenes: per scene a
    list of (matrix16, model index, op)."""
    rng = np.random.default_rng(seed)
    per = [[] for _ in scenes]
    for _ in range(n_instances):
        s = int(rng.integers(0, len(scenes)))
        mi = int(rng.integers(0, len(models)))
        per[s].append((instance_matrix(rng, scenes[s]["n"], models[mi].shape), mi, V.OP_SET))
    return per


def terrain_camera(n, top):
    """Above the terrain's near edge, looking down across it."""
    cam = np.array([0.5 * n, top + 0.35 * n, -0.15 * n], np.float32)
    tgt = np.array([0.5 * n, 0.5 * top, 0.55 * n], np.float32)
    return cam, tgt


def make_terrain_scene(ctx, n=2048, W=3840, H=2160, seed=5, n_instances=50000, n_models=48, edge=(16, 128),
                       base=None, amplitude=512.0, freq=None, octaves=6, params=None):
    """Stress scene: n^3 grid with a heightfield terrain (base + amplitude * fbm,
    `octaves` octaves) and n_instances Vox-model instances (edges in `edge`,
    uniform rotations) standing on the terrain, voxelized on the device;
    W x H G-buffer; 1 shadow ray, 16 AO rays of length 64 and 1 specular ray."""
    import torch

    base = n / 16.0 if base is None else base
    freq = 1.0 / (n / 4.0) if freq is None else freq
    G = V.Grid(ctx, n, n, n)
    d_h = torch.empty((n, n), dtype=torch.float32, device="cuda")
    G.scene_terrain(seed, base, amplitude, freq, octaves, d_height=d_h)
    h = d_h.cpu().numpy()
    models = vox_models(seed + 1, n_models, edge[0], edge[1], fill=0.4)
    d_models = [torch.from_numpy(m).cuda() for m in models]
    mdesc = [(d.data_ptr(),) + m.shape[::-1] for m, d in zip(models, d_models)]
    rng = np.random.default_rng(seed + 2)
    insts = []
    for _ in range(n_instances):
        mi = int(rng.integers(0, n_models))
        sz, sy, sx = models[mi].shape
        x, z = rng.uniform(0, n - 1, 2)
        y = float(h[int(z), int(x)]) - 0.25 * sy  # a quarter sunk into the ground
        m = np.eye(4)
        R = rotation_matrix(rng)
        m[:3, :3] = R
        half = 0.05 * np.array([sx, sy, sz])
        m[:3, 3] = np.array([x, y, z]) / 10.0 - R @ half
        insts.append((np.ascontiguousarray(m.T.astype(np.float32)).reshape(16), mi, V.OP_SET))
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    V.voxelize(ctx, G, mdesc, insts)
    e1.record()
    torch.cuda.synchronize()
    vox_s = e0.elapsed_time(e1) / 1e3
    top = float(h.max()) + amplitude * 0.1
    cam, tgt = terrain_camera(n, top)
    npix = W * H
    pos = torch.empty(npix * 3, dtype=torch.float32, device="cuda")
    nrm = torch.empty_like(pos)
    rough = torch.empty(npix, dtype=torch.float32, device="cuda")
    V.scene_gbuffer(ctx, G, cam, tgt, W, H, seed, pos, nrm, rough)
    P = params or V.make_params(light_dir=light_dir(seed), cam_pos=cam, bias=0.5, shadow_len=256.0, ao_len=64.0,
                                spec_len=256.0, n_shadow=1, n_ao=16, n_spec=1, seed=seed)
    src_voxels = sum(int(models[mi].size) for _, mi, _ in insts)
    return dict(grid=G, n=n, W=W, H=H, width=W, height=H, npix=npix, pos=pos, nrm=nrm, rough=rough, params=P,
                cam=cam, seed=seed, heights=d_h, models=models, d_models=d_models, mdesc=mdesc, instances=insts,
                voxelize_seconds=vox_s, source_voxels=src_voxels)
