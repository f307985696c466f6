"""Seeded inputs shared by the parity tests: grids and ray sets that cover
the edge cases of the reference traversal (Light.frag:29-217)."""
import numpy as np

import oracle


def noise_grid(n=64, seed=3, thresh=0.55, ground=8):
    """reference R8 layout, uint8[n/2, n/2, n/2]"""
    return oracle.scene_noise(n, n, n, seed=seed, thresh=thresh, ground_y=ground, threads=4)


def edge_rays(n_fine):
    """Hand-picked rays: axis-aligned, exact diagonal ties (two and three axes),
    zero and tiny direction components, origins on cell faces, corners and
    negative coordinates, rays leaving through the +1 over-bound, and rays
    starting outside the grid."""
    N = float(n_fine)
    c = N / 2.0 + 0.25
    r = []
    for d in ([1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1]):
        r.append([c, c, c] + d + [200.0])
        r.append([c, 3.5, c] + d + [40.0])
    s2 = np.float32(0.70710677)
    s3 = np.float32(0.57735026)
    for d in ([s2, s2, 0], [-s2, s2, 0], [s2, 0, -s2], [0, -s2, -s2], [s3, s3, s3], [-s3, s3, -s3], [s3, -s3, s3]):
        for o in ([c, c, c], [10.0, 10.0, 10.0], [10.5, 10.5, 10.5], [11.0, 12.0, 13.0], [0.0, 0.0, 0.0]):
            r.append(list(o) + list(d) + [120.0])
    # zero components with origin on a cell face (0/0 -> NaN t_max) and tiny components
    r.append([5.5, 6.0, 7.5, 1, 0, 0, 50.0])
    r.append([5.0, 6.5, 7.5, 0, 0, -1, 50.0])
    r.append([5.5, 6.5, 7.5, 1e-35, 1, 1e-38, 50.0])
    r.append([5.5, 6.5, 7.5, -1e-31, 0.6, 0.8, 50.0])
    r.append([5.5, 6.5, 7.5, 0.6, -0.0, 0.8, 50.0])
    # negative coordinates, -1 cells (floor vs truncation), and outside the grid
    r.append([-0.5, 3.5, 3.5, 1, 0.2, 0.1, 60.0])
    r.append([-1.5, -0.25, 3.5, 0.5, 0.5, 0.70710677, 60.0])
    r.append([N + 0.5, 3.5, 3.5, -1, 0.1, 0.1, 60.0])
    r.append([N + 1.5, 3.5, 3.5, -1, 0.1, 0.1, 60.0])
    r.append([N + 2.5, 3.5, 3.5, -1, 0.1, 0.1, 60.0])
    # leaving through the +1 over-bound on every axis
    r.append([N - 0.5, N - 0.5, N - 0.5, 0.5, 0.6, 0.62449979, 60.0])
    # maxt <= 0 and huge maxt
    r.append([c, c, c, 0.3, 0.4, 0.866, 0.0])
    r.append([c, c, c, 0.3, 0.4, 0.866, -5.0])
    r.append([c, c, c, 0.3, 0.4, 0.866, 1e30])
    return np.array(r, np.float32)


def random_rays(n_fine, count, seed=0, margin=4.0, integer_frac=0.1):
    rng = np.random.default_rng(seed)
    o = rng.uniform(-margin, n_fine + margin, (count, 3)).astype(np.float32)
    k = int(count * integer_frac)
    o[:k] = np.floor(o[:k])  # origins on cell corners
    o[k:2 * k, 0] = np.floor(o[k:2 * k, 0]) + 0.5
    d = rng.normal(size=(count, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    maxt = rng.uniform(1.0, 260.0, count)
    return np.concatenate([o, d.astype(np.float32), maxt[:, None]], axis=1).astype(np.float32)
