"""Seeded voxelizer inputs: models and rigid transforms (column-major 4x4)."""
import os

import numpy as np


def rot_matrix(rng):
    # uniform rotation from a random unit quaternion (three uniforms)
    u1, u2, u3 = rng.random(3)
    q = np.array([np.sqrt(1 - u1) * np.sin(2 * np.pi * u2), np.sqrt(1 - u1) * np.cos(2 * np.pi * u2),
                  np.sqrt(u1) * np.sin(2 * np.pi * u3), np.sqrt(u1) * np.cos(2 * np.pi * u3)])
    x, y, z, w = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def world_matrix(rng, lo, hi, rotate=True):
    """column-major float32[16]: rotation (or identity) and translation in [lo, hi) world units"""
    m = np.eye(4)
    if rotate:
        m[:3, :3] = rot_matrix(rng)
    m[:3, 3] = rng.uniform(lo, hi, 3)
    return np.ascontiguousarray(m.T.astype(np.float32)).reshape(16)


def random_model(rng, sx, sy, sz, fill=0.4):
    m = rng.integers(16, 256, (sz, sy, sx)).astype(np.uint8)
    m[rng.random((sz, sy, sx)) >= fill] = 0
    glass = rng.random((sz, sy, sx)) < 0.05
    m[glass] = rng.integers(1, 16, int(glass.sum())).astype(np.uint8)
    return m


def read_v(path):
    """.v asset: u32 SizeX, SizeY, SizeZ then raw bytes (VoxAsset::Serialize, VoxAsset.h:42-50)."""
    raw = open(path, "rb").read()
    sx, sy, sz = np.frombuffer(raw[:12], np.uint32)
    return np.frombuffer(raw[12:12 + int(sx) * sy * sz], np.uint8).reshape(int(sz), int(sy), int(sx))


def farmhouse_models(ref_root=None, limit=12):
    if ref_root is None:
        from oracle.ref.build_ref import reference_dir

        ref_root = reference_dir()
    d = os.path.join(ref_root, "Assets", "Mods", "default", "FarmHouse")
    if not os.path.isdir(d):
        return []
    names = sorted(os.listdir(d), key=lambda s: int(s.split(".")[0]) if s.split(".")[0].isdigit() else 1 << 30)
    return [read_v(os.path.join(d, n)) for n in names if n.endswith(".v")][:limit]


def rayvox_cases(rng, shapes, n_per_model=400):
    """Seeded picking rays for RayVoxCast: (model index, obb float32[16]
    column-major, world origin float32[3], world direction float32[3]).
    The obb is a rigid placement (identity rotation for a quarter of the
    models, so that axis-aligned directions keep exact zero components and
    take the 1e-8 nudge); origins lie in and around the model's box
    (local cells -2 .. size+2, mapped by obb at 0.1 world units per cell)."""
    out = []
    for mi, (sz, sy, sx) in enumerate(shapes):
        plain = mi % 4 == 0
        obb = world_matrix(rng, -3.0, 3.0, rotate=not plain)
        M = obb.reshape(4, 4).T.astype(np.float64)
        for j in range(n_per_model):
            local = rng.uniform(-2.0, 1.0, 3) + rng.uniform(0.0, 1.0, 3) * (np.array([sx, sy, sz]) + 2.0)
            world = (M @ np.append(local * 0.1, 1.0))[:3]
            if plain and j % 5 == 0:
                d = np.zeros(3)
                d[j % 3] = 1.0 if (j // 3) % 2 == 0 else -1.0
            else:
                d = rng.normal(size=3)
                d /= np.linalg.norm(d)
            out.append((mi, obb, world.astype(np.float32), d.astype(np.float32)))
    return out
