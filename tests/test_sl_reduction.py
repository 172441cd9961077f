"""The premise of the semi-Lagrangian kernels, checked on the CPU: the
reference's s = 0 bicubic spline (scipy RectBivariateSpline over the grid
padded by one periodic cell, vlapy/core/vlasov.py:42-80, 168-210), evaluated
where one coordinate is a grid node, equals the 1-D not-a-knot cubic spline of
that line, with departure points clamped to the padded range.  The line
spline below is the one the kernels solve (second derivatives M_k from the
not-a-knot conditions and the (1, 4, 1) interior system, then the cubic piece
holding each point); here it is written with NumPy's banded solver."""

import numpy as np
import pytest
from scipy.linalg import solve_banded

from oracle import vlapy_oracle as vo


def line_spline(y, p0, h, X):
    n = y.size
    sd = (y[:-2] + y[2:]) - 2.0 * y[1:-1]            # second differences at nodes 1 .. n-2
    M = np.zeros(n)
    M[1], M[n - 2] = sd[0] / h ** 2, sd[-1] / h ** 2
    m = n - 4
    if m > 0:
        rhs = 6.0 * sd[1:-1] / h ** 2
        rhs[0] -= M[1]
        rhs[-1] -= M[n - 2]
        ab = np.zeros((3, m))
        ab[0, 1:], ab[1, :], ab[2, :-1] = 1.0, 4.0, 1.0
        M[2:n - 2] = solve_banded((1, 1), ab, rhs)
    M[0], M[n - 1] = 2.0 * M[1] - M[2], 2.0 * M[n - 2] - M[n - 3]
    u = (np.clip(X, p0, p0 + (n - 1) * h) - p0) / h
    k = np.clip(np.floor(u).astype(int), 0, n - 2)
    t = u - k
    s = 1.0 - t
    return s * y[k] + t * y[k + 1] - h * h / 6.0 * t * s * ((2.0 - t) * M[k] + (1.0 + t) * M[k + 1])


def sl_by_lines(f, e, x, v, dt, along_x):
    out = np.empty_like(f)
    if along_x:
        h = x[2] - x[1]
        for j in range(f.shape[1]):
            y = np.concatenate([[f[-1, j]], f[:, j], [f[0, j]]])
            out[:, j] = line_spline(y, x[0] - h, h, x - v[j] * dt)
    else:
        h = v[2] - v[1]
        for i in range(f.shape[0]):
            y = np.concatenate([[f[i, -1]], f[i], [f[i, 0]]])
            out[i] = line_spline(y, v[0] - h, h, v - e[i] * dt)
    return out


SHAPES = [(4, 4), (5, 7), (8, 3), (3, 9), (16, 64), (12, 96), (33, 20), (64, 128)]


@pytest.mark.parametrize("nx,nv", SHAPES)
@pytest.mark.parametrize("dt", [0.1, -0.45, 2.5, 12.0])
def test_line_splines_equal_the_reference_bicubic(nx, nv, dt):
    rng = np.random.default_rng(nx * 1000 + nv)
    dx, x, kx, inv = vo.spatial_axis(0.0, 2 * np.pi / 0.3, nx)
    dv, v, kv = vo.velocity_axis(6.4, nv)
    f = vo.maxwellian(nx, nv, 6.4) * (1.0 + 0.05 * np.cos(0.3 * x))[:, None]
    f = f + 1e-3 * rng.standard_normal((nx, nv))
    e = 0.3 * rng.standard_normal(nx)
    if nx >= 3 and nv >= 4:
        ref = vo.vdfdx_sl(f, x, v, dt)
        assert np.linalg.norm(sl_by_lines(f, e, x, v, dt, True) - ref) <= 1e-13 * np.linalg.norm(ref)
    if nx >= 4 and nv >= 3:
        ref = vo.edfdv_sl(f, e, x, v, dt)
        assert np.linalg.norm(sl_by_lines(f, e, x, v, dt, False) - ref) <= 1e-12 * np.linalg.norm(ref)
