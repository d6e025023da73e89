"""TEST ORACLE (checker only): the 3-D advection-reaction benchmark
(benchmarks/advection_reaction_3D/raja) in numpy -- its user functions
restated operation for operation (rhs3D.hpp: Advection 30-320, Reaction
322-383, AdvectionReaction 386-406, SolveReactionLinSys 441-552), its initial
condition (advection_reaction_3D.cpp:566-637, with numpy's exp / sqrt /
pow) -- and its CVODE configuration (cvode_driver.cpp:43-160: BDF, Newton,
SPGMR with left preconditioning and the default maxl, the difference-quotient
J v, PSolve = the per-cell reaction solve, no preconditioner setup; outputs
at t0 + k (tf - t0) / nout) run through the reference's CVode
(``run_reference``) and the CVODE restatement (``run_port_serial``).

Layout: cell (i, j, k) at ((i*ny + j)*nz + k)*3 + species, x slowest."""
from __future__ import annotations

import math

import numpy as np

from . import heat_cvode as hc

BLOCK_SOLVE_FN = hc.ct.CFUNCTYPE(hc.I, hc.VP, hc.VP, hc.VP, hc.D, hc.VP)

DEFAULTS = dict(xmax=1.0, A=1.0, B=3.5, k=(1.0, 1.0, 1.0, 1.0, 1.0 / 5.0e-6, 1.0 / 5.0e-6),
                c=0.01, rtol=1.0e-6, atol=1.0e-9, t0=0.0, tf=10.0, nout=10)


class Params:
    def __init__(self, nx, ny, nz, **kw):
        p = dict(DEFAULTS)
        p.update(kw)
        self.nx, self.ny, self.nz = nx, ny, nz
        self.xmax, self.A, self.B, self.c = p["xmax"], p["A"], p["B"], p["c"]
        self.k1, self.k2, self.k3, self.k4, self.k5, self.k6 = p["k"]
        self.k = tuple(p["k"])
        self.dx = (self.xmax - 0.0) / nx
        self.dy = (self.xmax - 0.0) / ny
        self.dz = (self.xmax - 0.0) / nz
        self.cx, self.cy, self.cz = -self.c / self.dx, -self.c / self.dy, -self.c / self.dz
        self.rtol, self.atol = p["rtol"], p["atol"]
        t0, tf, nout = p["t0"], p["tf"], p["nout"]
        dtout = (tf - t0) / nout
        self.touts, tout = [], t0 + dtout
        for _ in range(nout):
            self.touts.append(tout)
            tout = tout + dtout
            tout = tf if tout > tf else tout

    @property
    def n(self):
        return 3 * self.nx * self.ny * self.nz


def initial(q: Params) -> np.ndarray:
    alpha = 0.1
    mu = q.xmax / 2.0
    sigma = q.xmax / 4.0
    denom = 2.0 * math.sqrt((sigma * sigma * sigma) * math.pow(2 * math.pi, 3))

    def g(x):
        return alpha * np.exp(-((x - mu) * (x - mu) * (1.0 / sigma)) / denom)

    i = np.arange(q.nx)[:, None, None]
    j = np.arange(q.ny)[None, :, None]
    k = np.arange(q.nz)[None, None, :]
    p = (g(i * q.dx) + g(j * q.dy)) + g(k * q.dz)
    us = q.k1 * q.A / q.k4
    vs = q.k2 * q.k4 * q.B / (q.k1 * q.k3 * q.A)
    ws = 3.0
    y = np.stack([us + p, vs + p, ws + p], axis=-1)
    return np.ascontiguousarray(y).reshape(-1)


def advection(q: Params, y) -> np.ndarray:
    Y = y.reshape(q.nx, q.ny, q.nz, 3)
    if q.c == 0.0:
        return np.zeros_like(y)
    if q.c > 0.0:
        dx_, dy_, dz_ = (Y - np.roll(Y, 1, 0), Y - np.roll(Y, 1, 1), Y - np.roll(Y, 1, 2))
        i = np.arange(q.nx)[:, None, None, None] > 0
        j = np.arange(q.ny)[None, :, None, None] > 0
        k = np.arange(q.nz)[None, None, :, None] > 0
    else:
        dx_, dy_, dz_ = (np.roll(Y, -1, 0) - Y, np.roll(Y, -1, 1) - Y, np.roll(Y, -1, 2) - Y)
        i = np.arange(q.nx)[:, None, None, None] < q.nx - 1
        j = np.arange(q.ny)[None, :, None, None] < q.ny - 1
        k = np.arange(q.nz)[None, None, :, None] < q.nz - 1
    interior = (q.cz * dz_ + q.cy * dy_) + q.cx * dx_
    face = (q.cx * dx_ + q.cy * dy_) + q.cz * dz_
    return np.where(i & j & k, interior, face).reshape(-1)


def reaction_add(q: Params, y, d) -> np.ndarray:
    Y = y.reshape(-1, 3)
    D = d.reshape(-1, 3).copy()
    u, v, w = Y[:, 0], Y[:, 1], Y[:, 2]
    D[:, 0] = D[:, 0] + ((((q.k1 * q.A) - ((q.k2 * w) * u)) + (((q.k3 * u) * u) * v)) - (q.k4 * u))
    D[:, 1] = D[:, 1] + (((q.k2 * w) * u) - (((q.k3 * u) * u) * v))
    D[:, 2] = D[:, 2] + (((((-q.k2) * w) * u) + (q.k5 * q.B)) - (q.k6 * w))
    return D.reshape(-1)


def rhs(q: Params, y) -> np.ndarray:
    return reaction_add(q, y, advection(q, y))


def reaction(q: Params, y) -> np.ndarray:
    return reaction_add(q, y, np.zeros_like(y))


def solve_reaction(q: Params, y, b, gamma) -> np.ndarray:
    Y, Bv = y.reshape(-1, 3), b.reshape(-1, 3)
    u, v, w = Y[:, 0], Y[:, 1], Y[:, 2]
    b0, b1, b2 = Bv[:, 0], Bv[:, 1], Bv[:, 2]
    k2, k3, k4, k6 = q.k2, q.k3, q.k4, q.k6
    A0 = (((-k2) * w) + (((2.0 * k3) * u) * v)) - k4
    A1 = (k3 * u) * u
    A2 = (-k2) * u
    A3 = (k2 * w) - (((2.0 * k3) * u) * v)
    A4 = ((-k3) * u) * u
    A5 = k2 * u
    A6 = (-k2) * w
    A7 = np.zeros_like(u)
    A8 = ((-k2) * u) - k6
    A0 = 1.0 - (gamma * A0)
    A1 = (-gamma) * A1
    A2 = (-gamma) * A2
    A3 = (-gamma) * A3
    A4 = 1.0 - (gamma * A4)
    A5 = (-gamma) * A5
    A6 = (-gamma) * A6
    A7 = (-gamma) * A7
    A8 = 1.0 - (gamma * A8)
    s0, s1, s2, s3, s4, s5 = A4 * A8, A1 * A5, A2 * A7, A5 * A7, A1 * A8, A2 * A4
    s6 = 1.0 / (((((A0 * s0 - A0 * s3) + A3 * s2) - A3 * s4) + A6 * s1) - A6 * s5)
    s7, s8, s9, s10 = A2 * A3, A6 * b0, A2 * A6, A3 * b0
    s11 = 1.0 / A0
    s12 = A1 * s11
    s13 = ((-A6) * s12 + A7) / ((-A3) * s12 + A4)
    x0 = s6 * ((b0 * (s0 - s3) + b1 * (s2 - s4)) + b2 * (s1 - s5))
    x1 = s6 * (((b2 * (s7 - A0 * A5) + b1 * (A0 * A8 - s9)) + A5 * s8) - A8 * s10)
    x2 = (((-b2) + s11 * s8) + s13 * (b1 - s10 * s11)) / (((-A8) + s11 * s9) + s13 * (A5 - s11 * s7))
    return np.stack([x0, x1, x2], axis=1).reshape(-1)


class SerialBruss:
    """The benchmark's CVODE callbacks on NVECTOR_SERIAL vectors of the
    reference library: f = AdvectionReaction, no J v (difference quotient),
    no preconditioner setup, PSolve = the per-cell reaction solve."""

    def __init__(self, L, q: Params):
        self.q = q
        n = q.n

        def arr(v):
            return np.ctypeslib.as_array(L.N_VGetArrayPointer(v), shape=(n,))

        def f(t, y, ydot, data):
            arr(ydot)[:] = rhs(q, arr(y))
            return 0

        def psolve(t, y, fy, r, z, gamma, delta, lr, data):
            arr(z)[:] = solve_reaction(q, arr(y), arr(r), gamma)
            return 0

        def fe(t, y, ydot, data):
            arr(ydot)[:] = advection(q, arr(y))
            return 0

        def fi(t, y, ydot, data):
            arr(ydot)[:] = reaction(q, arr(y))
            return 0

        def block_solve(z, x, b, gamma, data):
            arr(x)[:] = solve_reaction(q, arr(z), arr(b), gamma)
            return 0

        self.cbs = (hc.RHS_FN(f), hc.PSOLVE_FN(psolve), hc.RHS_FN(fe), hc.RHS_FN(fi),
                    BLOCK_SOLVE_FN(block_solve))
        self.arr = arr

    def reaction_into(self, t, z, Fi):
        """The benchmark's Reaction(t, z, Fi) with add_reactions false."""
        self.arr(Fi)[:] = reaction(self.q, self.arr(z))
        return 0

    def block_solve(self, z, x, b, gamma):
        """SolveReactionLinSys(z, x, b, gamma) (rhs3D.hpp:441-552)."""
        self.arr(x)[:] = solve_reaction(self.q, self.arr(z), self.arr(b), gamma)
        return 0

    def block_solve_address(self):
        return hc.ct.cast(self.cbs[4], hc.VP).value

    def addresses(self):
        f, ps = (hc.ct.cast(c, hc.VP).value for c in self.cbs[:2])
        return (f, None, None, ps)

    def imex_addresses(self):
        """(Advection, Reaction): the ARK-IMEX splitting (arkode_driver.cpp:
        255-258, add_reactions false: Reaction = 0 + g)."""
        return tuple(hc.ct.cast(c, hc.VP).value for c in self.cbs[2:4])


def run_reference(q: Params, threads=None, fixed_point=None, adams=False):
    """cvode_driver.cpp's CV-BDF configuration through the reference's CVode
    (fixed_point = m: ``--nls fixedpoint --fpaccel m``; adams: its CV-ADAMS
    configuration, which always takes the fixed-point solver)."""
    return hc.run_reference_with(lambda L: SerialBruss(L, q), initial(q), q.touts, q.rtol,
                                 q.atol, threads=threads, fixed_point=fixed_point, adams=adams)


def run_port_serial(q: Params, fixed_point=None, adams=False):
    return hc.run_port_serial_with(lambda L: SerialBruss(L, q), initial(q), q.touts, q.rtol,
                                   q.atol, fixed_point=fixed_point, adams=adams)


def run_reference_arkode(q: Params, threads=None, imex=False, order=3, task_local=False,
                         fixed_point=None, erk=False, mxstep=100000):
    """The benchmark's ARK-DIRK (arkode_driver.cpp:51-160) or, imex, ARK-IMEX
    (239-370; task_local: with --nls tl-newton) configuration through the
    reference's ARKodeEvolve: (counters, reals, solutions, Butcher tables)."""
    from . import arkstep as ak
    return ak.run_reference_with(lambda L: SerialBruss(L, q), initial(q), q.touts, q.rtol, q.atol,
                                 order=order, threads=threads, imex=imex, task_local=task_local,
                                 fixed_point=fixed_point, erk=erk, mxstep=mxstep)


def run_port_serial_arkode(q: Params, tables, task_local=False, fixed_point=None):
    """The same through the ARKStep restatement on the reference's serial objects."""
    from . import arkstep as ak
    return ak.run_port_serial_with(lambda L: SerialBruss(L, q), initial(q), q.touts, tables,
                                   q.rtol, q.atol, task_local=task_local,
                                   fixed_point=fixed_point)
