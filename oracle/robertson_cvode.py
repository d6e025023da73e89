"""TEST ORACLE (checker only): the batched Robertson problem -- ncells
independent cells y1' = -k1 y1 + k3 y2 y3, y3' = k2 y2^2, y2' = -y1' - y3'
with k = (0.04, 3e7, 1e4) each scaled by exp(0.1 z), z ~ N(0, 1) per cell and
constant (seed 1), y0 = (1, 0, 0), outputs at 0.4 * 10^k, rtol 1e-4 and the
per-species absolute tolerances of the reference example (1e-8, 1e-14, 1e-6;
a scalar 1e-8 lets the reference's own solution blow up after t ~ 4e8 and
makes its counters depend on the summation order) -- integrated by
CVODE with BDF, Newton and SPGMR (left preconditioning, maxl 5), a user J v
and the exact block-Jacobi preconditioner of examples/cvode/serial/
cvDiurnal_kry.c:714-845 (jok reuses the saved Jacobian blocks; P = -gamma J,
P += I, SUNDlsMat_denseGETRF per 3x3 block; solve = SUNDlsMat_denseGETRS,
src/sundials/sundials_dense.c:85-193, restated here vectorised over cells in
the same floating-point order).

The serial callbacks round like the device ones of include/robertson_gb300.h
(f as examples/cvode/cuda/cvRoberts_block_cusolversp_batchqr.cu:316-333)."""
from __future__ import annotations

import numpy as np

from . import heat_cvode as hc

K0 = np.array([0.04, 3.0e7, 1.0e4])
TOUTS = [0.4 * 10.0 ** k for k in range(12)]
ATOL_SPECIES = np.array([1.0e-8, 1.0e-14, 1.0e-6])  # cvRoberts_block_cusolversp_batchqr.cu:56-59


def vector_atol(ncells: int) -> np.ndarray:
    return np.tile(ATOL_SPECIES, ncells)


def rates(ncells: int, seed: int = 1) -> np.ndarray:
    """k1, k2, k3 per cell, shape (ncells, 3)."""
    z = np.random.default_rng(seed).standard_normal((ncells, 3))
    return K0[None, :] * np.exp(0.1 * z)


def initial(ncells: int) -> np.ndarray:
    u = np.zeros((ncells, 3))
    u[:, 0] = 1.0
    return u.reshape(-1)


def rhs(k, y):
    k1, k2, k3 = k[:, 0], k[:, 1], k[:, 2]
    y = y.reshape(-1, 3)
    yd1 = (-k1) * y[:, 0] + (k3 * y[:, 1]) * y[:, 2]
    yd3 = (k2 * y[:, 1]) * y[:, 1]
    return np.stack([yd1, -yd1 - yd3, yd3], axis=1).reshape(-1)


def jac(k, y):
    """Jacobian blocks, J[c, col, row] (column-major per cell)."""
    k1, k2, k3 = k[:, 0], k[:, 1], k[:, 2]
    y = y.reshape(-1, 3)
    y2, y3 = y[:, 1], y[:, 2]
    J = np.zeros((len(k), 3, 3))
    J[:, 0, 0] = -k1
    J[:, 0, 1] = k1
    J[:, 1, 0] = k3 * y3
    J[:, 1, 1] = (-k3 * y3) - ((2.0 * k2) * y2)
    J[:, 1, 2] = (2.0 * k2) * y2
    J[:, 2, 0] = k3 * y2
    J[:, 2, 1] = -k3 * y2
    return J


def jtimes(k, y, v):
    J = jac(k, y)
    v = v.reshape(-1, 3)
    out = np.empty_like(v)
    for i in range(3):
        out[:, i] = (J[:, 0, i] * v[:, 0] + J[:, 1, i] * v[:, 1]) + J[:, 2, i] * v[:, 2]
    return out.reshape(-1)


def getrf(P):
    """SUNDlsMat_denseGETRF on every 3x3 block of P[c, col, row] in place;
    returns (pivots [c, 3], first zero-pivot column + 1 per block or 0)."""
    nb, n = P.shape[0], 3
    piv = np.zeros((nb, n), np.int64)
    fail = np.zeros(nb, np.int64)
    cells = np.arange(nb)
    with np.errstate(divide="ignore", invalid="ignore"):
        _getrf_steps(P, piv, fail, cells, n)
    return piv, fail


def _getrf_steps(P, piv, fail, cells, n):
    nb = P.shape[0]
    for k in range(n):
        ck = P[:, k, :]
        l = np.full(nb, k)
        for i in range(k + 1, n):
            l = np.where(np.abs(ck[cells, i]) > np.abs(ck[cells, l]), i, l)
        piv[:, k] = l
        zero = (ck[cells, l] == 0.0) & (fail == 0)
        fail[zero] = k + 1
        sw = (l != k)
        if np.any(sw):
            rows_l = P[cells, :, l].copy()
            rows_k = P[cells, :, k].copy()
            P[cells[sw], :, l[sw]] = rows_k[sw]
            P[cells[sw], :, k] = rows_l[sw]
        mult = 1.0 / P[:, k, k]
        for i in range(k + 1, n):
            P[:, k, i] = P[:, k, i] * mult
        for j in range(k + 1, n):
            akj = P[:, j, k].copy()
            nz = akj != 0.0
            for i in range(k + 1, n):
                P[:, j, i] = np.where(nz, P[:, j, i] - akj * P[:, k, i], P[:, j, i])


def getrs(P, piv, b):
    """SUNDlsMat_denseGETRS per block; b (ncells*3) -> solution."""
    b = b.reshape(-1, 3).copy()
    cells = np.arange(len(b))
    n = 3
    for k in range(n):
        pk = piv[:, k]
        bk = b[:, k].copy()
        bp = b[cells, pk].copy()
        b[:, k] = bp
        b[cells, pk] = np.where(pk != k, bk, b[cells, pk])
    for k in range(n - 1):
        for i in range(k + 1, n):
            b[:, i] = b[:, i] - P[:, k, i] * b[:, k]
    for k in range(n - 1, 0, -1):
        b[:, k] = b[:, k] / P[:, k, k]
        for i in range(k):
            b[:, i] = b[:, i] - P[:, k, i] * b[:, k]
    b[:, 0] = b[:, 0] / P[:, 0, 0]
    return b.reshape(-1)


class SerialRobertson:
    """The problem's callbacks on NVECTOR_SERIAL vectors of the reference library."""

    def __init__(self, L, k):
        self.k = k
        self.n = 3 * len(k)
        self.J = np.zeros((len(k), 3, 3))
        self.P = None
        self.piv = None

        def arr(v):
            return np.ctypeslib.as_array(L.N_VGetArrayPointer(v), shape=(self.n,))

        def f(t, y, ydot, data):
            arr(ydot)[:] = rhs(self.k, arr(y))
            return 0

        def jt(v, jv, t, y, fy, data, tmp):
            arr(jv)[:] = jtimes(self.k, arr(y), arr(v))
            return 0

        def psetup(t, y, fy, jok, jcur, gamma, data):
            if jok:
                jcur[0] = 0
            else:
                self.J = jac(self.k, arr(y))
                jcur[0] = 1
            P = (-gamma) * self.J
            for i in range(3):
                P[:, i, i] = P[:, i, i] + 1.0
            self.piv, fail = getrf(P)
            self.P = P
            return 1 if np.any(fail) else 0

        def psolve(t, y, fy, r, z, gamma, delta, lr, data):
            arr(z)[:] = getrs(self.P, self.piv, arr(r))
            return 0

        nc = len(k)
        cell = np.arange(nc)

        def jac_dense(t, y, fy, J, data, t1, t2, t3):
            # SUNDenseMatrix (column-major, zeroed by CVODE): the 3x3 blocks
            D = np.ctypeslib.as_array(L.SUNDenseMatrix_Data(J), shape=(self.n, self.n))
            Jb = jac(self.k, arr(y))
            for col in range(3):
                for row in range(3):
                    D[3 * cell + col, 3 * cell + row] = Jb[:, col, row]
            return 0

        self.cbs = (hc.RHS_FN(f), hc.JTIMES_FN(jt), hc.PSETUP_FN(psetup), hc.PSOLVE_FN(psolve))
        self.jac_cb = hc.JAC_FN(jac_dense)
        self.arr = arr

    def addresses(self):
        return tuple(hc.ct.cast(c, hc.VP).value for c in self.cbs)

    def jac_address(self):
        return hc.ct.cast(self.jac_cb, hc.VP).value


def run_reference(ncells: int, touts=TOUTS, rtol=1e-4, atol=None, threads=None):
    """SPGMR with the exact block-Jacobi preconditioner."""
    k = rates(ncells)
    atol = vector_atol(ncells) if atol is None else atol
    return hc.run_reference_with(lambda L: SerialRobertson(L, k), initial(ncells), touts, rtol,
                                 atol, threads=threads)


def run_port_serial(ncells: int, touts=TOUTS, rtol=1e-4, atol=None, direct=False):
    k = rates(ncells)
    atol = vector_atol(ncells) if atol is None else atol
    return hc.run_port_serial_with(lambda L: SerialRobertson(L, k), initial(ncells), touts, rtol,
                                   atol, direct=direct)


def run_reference_direct(ncells: int, touts=TOUTS, rtol=1e-4, atol=None, threads=None):
    """The reference example's configuration (cvRoberts_block_cusolversp_batchqr.cu:
    a direct solver on the block-diagonal Newton matrix with the user Jacobian),
    on the reference's CPU objects: SUNDenseMatrix + SUNLINSOL_DENSE, whose
    partial-pivoting LU of a block-diagonal matrix is the per-block LU."""
    k = rates(ncells)
    atol = vector_atol(ncells) if atol is None else atol
    return hc.run_reference_with(lambda L: SerialRobertson(L, k), initial(ncells), touts, rtol,
                                 atol, threads=threads, direct=True)


def run_reference_arkode_direct(ncells: int, touts=TOUTS, rtol=1e-4, atol=None, threads=None):
    """The same problem through the reference's ARKStep (DIRK, order 3,
    Newton) with the matrix-based direct path of ARKLS: SUNDenseMatrix +
    SUNLINSOL_DENSE and the user Jacobian (ARKodeSetJacFn), per-species
    absolute tolerances (ARKodeSVtolerances): (counters, reals, solutions,
    Butcher tables)."""
    from . import arkstep as ak
    k = rates(ncells)
    atol = vector_atol(ncells) if atol is None else atol
    return ak.run_reference_with(lambda L: SerialRobertson(L, k), initial(ncells), touts, rtol,
                                 atol, threads=threads, direct=True)


def run_port_serial_arkode_direct(ncells: int, tables, touts=TOUTS, rtol=1e-4, atol=None):
    """The same through the ARKStep restatement on the reference's objects."""
    from . import arkstep as ak
    k = rates(ncells)
    atol = vector_atol(ncells) if atol is None else atol
    return ak.run_port_serial_with(lambda L: SerialRobertson(L, k), initial(ncells), touts,
                                   tables, rtol, atol, direct=True)


def run_reference_arkode(ncells: int, touts=TOUTS, rtol=1e-4, atol=None, threads=None):
    """ARKStep (DIRK, order 3, Newton) with SPGMR (left, maxl 5), the user J v
    and the exact block-Jacobi preconditioner with its setup
    (ARKodeSetPreconditioner(psetup, psolve)): the iterative path of ARKLS."""
    from . import arkstep as ak
    k = rates(ncells)
    atol = vector_atol(ncells) if atol is None else atol
    return ak.run_reference_with(lambda L: SerialRobertson(L, k), initial(ncells), touts, rtol,
                                 atol, threads=threads)


def run_port_serial_arkode(ncells: int, tables, touts=TOUTS, rtol=1e-4, atol=None):
    from . import arkstep as ak
    k = rates(ncells)
    atol = vector_atol(ncells) if atol is None else atol
    return ak.run_port_serial_with(lambda L: SerialRobertson(L, k), initial(ncells), touts,
                                   tables, rtol, atol)
