"""TEST ORACLE (checker only): numpy restatement of the 5-point heat stencil
of examples/cvode/CXX_serial/cv_heat2D.cpp:305-367 (without its forcing
term) on the nx x ny interior grid, zero Dirichlet boundaries, rounded in the
reference's order (cc u_c + cx (u_w + u_e)) + cy (u_s + u_n), and of the
Jacobi preconditioner of cv_heat2D.cpp:371-408."""
from __future__ import annotations

import numpy as np


def coefficients(nx, ny, kx=1.0, ky=1.0):
    dx, dy = 1.0 / (nx + 1), 1.0 / (ny + 1)
    cx, cy = kx / (dx * dx), ky / (dy * dy)
    return cx, cy, -2.0 * (cx + cy)


def jv(v, nx, ny, kx=1.0, ky=1.0):
    cx, cy, cc = coefficients(nx, ny, kx, ky)
    u = np.zeros((ny + 2, nx + 2))
    u[1:-1, 1:-1] = v.reshape(ny, nx)
    c = u[1:-1, 1:-1]
    w, e = u[1:-1, :-2], u[1:-1, 2:]
    s, n = u[:-2, 1:-1], u[2:, 1:-1]
    return ((cc * c + cx * (w + e)) + cy * (s + n)).reshape(-1)


def atimes(v, gamma, nx, ny, kx=1.0, ky=1.0):
    return v + (-gamma) * jv(v, nx, ny, kx, ky)


def jacobi(gamma, nx, ny, kx=1.0, ky=1.0):
    cc = coefficients(nx, ny, kx, ky)[2]
    return 1.0 / (1.0 - gamma * cc)
