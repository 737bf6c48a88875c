"""Stand-in transformations module (own code, small subset)."""
import numpy as np
from .rotations import matrix_from_quaternion


def transform_from(R, p):
    A2B = np.eye(4)
    A2B[:3, :3] = R
    A2B[:3, 3] = p
    return A2B


def random_transform(random_state=None, mean=None, cov=None):
    if random_state is None:
        random_state = np.random.RandomState(0)
    q = random_state.randn(4)
    return transform_from(matrix_from_quaternion(q), random_state.randn(3))
