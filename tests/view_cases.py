"""Camera matrices as the engine builds them (glm conventions, column-major):
CameraSystem::CalculateView (ViewMatrix = inverse(camera world matrix),
ProjectionMatrix = glm::perspective, right-handed, clip depth -1..1) and the
depth GeometryVoxel.frag:169 writes, (w - NEAR) / (FAR - NEAR) with the
shader constants NEAR = 0.1, FAR = 4096 (Common.frag:12-13)."""
import numpy as np

NEAR, FAR = 0.1, 4096.0


def camera_world(cam, target):
    """Camera-to-world matrix (float64 4x4): looks down its -z axis at target, y up."""
    cam = np.asarray(cam, np.float64)
    f = np.asarray(target, np.float64) - cam
    f /= np.linalg.norm(f)
    r = np.cross(f, [0.0, 1.0, 0.0])
    r /= np.linalg.norm(r)
    u = np.cross(r, f)
    m = np.eye(4)
    m[:3, 0], m[:3, 1], m[:3, 2], m[:3, 3] = r, u, -f, cam
    return m


def perspective(tan_half_fov, aspect, near=NEAR, far=FAR):
    """glm::perspective (right-handed, clip depth -1..1), float64 4x4."""
    f = 1.0 / tan_half_fov
    p = np.zeros((4, 4))
    p[0, 0] = f / aspect
    p[1, 1] = f
    p[2, 2] = -(far + near) / (far - near)
    p[3, 2] = -1.0
    p[2, 3] = -(2.0 * far * near) / (far - near)
    return p


def colmajor(m):
    """4x4 float64 -> float32[16] in glm's column-major storage."""
    return np.ascontiguousarray(np.asarray(m, np.float64).T.reshape(16), np.float32)


def view_mats(cam, target, tan_half_fov, W, H):
    """(inverse_view, inverse_projection) as the view buffer holds them, and the
    float64 view / projection matrices."""
    cw = camera_world(cam, target)
    pr = perspective(tan_half_fov, W / H)
    return colmajor(cw), colmajor(np.linalg.inv(pr)), np.linalg.inv(cw), pr


def depth_of(points_world, view):
    """Linear depth of world points as GeometryVoxel writes it."""
    p = np.concatenate([np.asarray(points_world, np.float64), np.ones((len(points_world), 1))], 1)
    w = -(p @ view.T)[:, 2]
    return ((w - NEAR) / (FAR - NEAR)).astype(np.float32)
