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
