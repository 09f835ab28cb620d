"""Host-side geometry and numerics helpers (src/utils.jl of the reference).

These run on the CPU in double precision and are used to build geometry
(PMT layouts, rotations) and tables; the device has its own single-precision
versions inside the propagation kernel.
"""
from __future__ import annotations

import numpy as np

# 10-point Gauss-Legendre rule, utils.jl:17
GL10 = np.polynomial.legendre.leggauss(10)


def fast_linear_interp(x, xs, ys):
    """Linear interpolation with clamping (fast_linear_interp, utils.jl:24-53).

    Vectorised over ``x``; ``xs`` ascending.  Arithmetic in the dtype of ``xs``.
    """
    xs = np.asarray(xs)
    ys = np.asarray(ys, dtype=xs.dtype)
    x = np.clip(np.asarray(x, dtype=xs.dtype), xs[0], xs[-1])
    hi = np.searchsorted(xs, x, side="left")
    hi = np.clip(hi, 1, len(xs) - 1)
    lo = hi - 1
    along = (x - xs[lo]) / (xs[hi] - xs[lo])
    out = ys[lo] + (ys[hi] - ys[lo]) * along
    out = np.where(x == xs[0], ys[0], out)
    out = np.where(x == xs[-1], ys[-1], out)
    return out


def integrate_gauss_quad(f, a: float, b: float) -> float:
    """10-point Gauss-Legendre quadrature of f on [a, b] (utils.jl:91-103)."""
    nodes, weights = GL10
    half = (b - a) / 2.0
    mid = (a + b) / 2.0
    return float(np.dot(weights, [f(half * x + mid) * half for x in nodes]))


def sph_to_cart(theta, phi):
    """(theta, phi) -> unit vector (utils.jl:105-115)."""
    st, ct = np.sin(theta), np.cos(theta)
    sp, cp = np.sin(phi), np.cos(phi)
    return np.array([cp * st, sp * st, ct])


def cart_to_sph(x, y=None, z=None):
    """Unit vector -> (theta, phi) (utils.jl:118-135)."""
    if y is None:
        x, y, z = x
    if z == 1:
        return 0.0, 0.0
    if z == -1:
        return np.pi, 0.0
    theta = np.arccos(z)
    if x == 0 and y > 0:
        phi = np.pi / 2
    elif x == 0 and y < 0:
        phi = -np.pi / 2
    else:
        phi = np.arctan2(y, x)
    return theta, phi


def _ssc(v):
    return np.array([[0.0, -v[2], v[1]], [v[2], 0.0, -v[0]], [-v[1], v[0], 0.0]])


def calc_rot_matrix(a, b):
    """Rotation matrix taking a to b (utils.jl:173-184)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    if np.array_equal(a, b):
        return np.eye(3)
    c = np.cross(a, b)
    s = _ssc(c)
    return np.eye(3) + s + s @ s * (1 - np.dot(a, b)) / np.dot(c, c)


def apply_rot(a, b, operand):
    """Rotate operand by the rotation taking a to b, normalised (utils.jl:193-197)."""
    r = calc_rot_matrix(a, b) @ np.asarray(operand, dtype=np.float64)
    return r / np.linalg.norm(r)


def rot_to_ez_fast(a, operand):
    """Rotation taking a to e_z, applied to operand (utils.jl:200-225)."""
    a = np.asarray(a, dtype=np.float64)
    o = np.asarray(operand, dtype=np.float64)
    if abs(a[2]) == 1:
        return np.array([o[0], np.copysign(o[1], a[2]), np.copysign(o[2], a[2])])
    a1sq, a2sq = a[0] ** 2, a[1] ** 2
    fact = (1 - a[2]) / (a2sq + a1sq)
    a1a2 = a[0] * a[1]
    x = (1 - a1sq * fact) * o[0] - a1a2 * fact * o[1] - a[0] * o[2]
    y = -a1a2 * fact * o[0] + (1 - a2sq * fact) * o[1] - a[1] * o[2]
    z = a[0] * o[0] + a[1] * o[1] + a[2] * o[2]
    return np.array([x, y, z])


def rot_from_ez_fast(a, operand):
    """Rotation taking e_z to a, applied to operand (utils.jl:228-243)."""
    a = np.asarray(a, dtype=np.float64)
    o = np.asarray(operand, dtype=np.float64)
    if abs(a[2]) == 1:
        return np.array([o[0], np.copysign(o[1], a[2]), np.copysign(o[2], a[2])])
    a1sq, a2sq = a[0] ** 2, a[1] ** 2
    fact = (1 - a[2]) / (a2sq + a1sq)
    a1a2 = a[0] * a[1]
    x = (1 - a1sq * fact) * o[0] - a1a2 * fact * o[1] + a[0] * o[2]
    y = -a1a2 * fact * o[0] + (1 - a2sq * fact) * o[1] + a[1] * o[2]
    z = -a[0] * o[0] - a[1] * o[1] + a[2] * o[2]
    return np.array([x, y, z])


def random_rotation(rng: np.random.Generator) -> np.ndarray:
    """Uniformly distributed rotation matrix (rand(RotMatrix3) in the reference scripts)."""
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([
        [1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
        [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
        [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)],
    ])
