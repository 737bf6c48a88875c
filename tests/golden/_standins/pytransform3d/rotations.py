"""Stand-in rotations module (own code, small subset)."""
import numpy as np


def perpendicular_to_vector(a):
    """Return a vector perpendicular to ``a`` (any one)."""
    a = np.asarray(a, dtype=float)
    if abs(a[0]) > 1e-12 or abs(a[1]) > 1e-12:
        return np.array([-a[1], a[0], 0.0])
    return np.array([0.0, -a[2], a[1]])


def matrix_from_quaternion(q):
    w, x, y, z = np.asarray(q, dtype=float) / np.linalg.norm(q)
    return np.array([
        [1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
        [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
        [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])
