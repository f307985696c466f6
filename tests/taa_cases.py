"""Seeded inputs for the temporal-accumulation pass: smooth fields with hard
edges (so the neighbourhood weights switch on and off), small motion with a
band pushed off screen (the disocclusion branch), sky pixels (depth 1)."""
import numpy as np


def frame(W, H, seed, band=4):
    rng = np.random.default_rng(seed)
    yy, xx = np.mgrid[0:H, 0:W].astype(np.float32)
    region = ((xx // 11 + yy // 7) % 3).astype(np.int32)
    light = np.stack([np.sin(xx * 0.05 + k) * 0.5 + 0.6 + rng.random((H, W)) * 0.2 for k in range(4)], -1)
    last = np.stack([np.cos(yy * 0.04 + k) * 0.5 + 0.6 for k in range(3)] + [rng.random((H, W))], -1)
    palette = rng.random((3, 3)).astype(np.float32)
    color = palette[region]
    normals = np.array([[0, 1, 0], [1, 0, 0], [0, 0.6, 0.8]], np.float32)
    normal = normals[region]
    mats = rng.random((3, 4)).astype(np.float32)
    material = mats[region]
    depth = (0.05 + 0.02 * region + 1e-4 * xx).astype(np.float32)
    depth[(yy < 3)] = 1.0  # sky rows
    motion = (rng.normal(size=(H, W, 2)) * 2e-3).astype(np.float32)
    motion[:, :band, 0] = -0.2  # pushed off the left edge: disocclusion branch
    noise = rng.random((H, W, 4)).astype(np.float32)
    f = lambda a: np.ascontiguousarray(a, np.float32)
    return dict(light=f(light), last=f(last), color=f(color), normal=f(normal), material=f(material),
                depth=f(depth[..., None]), motion=f(motion), noise=f(noise))
