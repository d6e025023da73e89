"""TEST ORACLE (checker only; never on the product path): a numpy restatement
of the reference's SPGMR solve, used to check the GB300 solver on inputs the
committed reference fixtures do not cover (other sizes and seeds).

Follows, step for step:
  SUNLinSolSolve_SPGMR   src/sunlinsol/spgmr/sunlinsol_spgmr.c:461-932
  SUNModifiedGS          src/sundials/sundials_iterative.c:45-105
  SUNClassicalGS         src/sundials/sundials_iterative.c:116-170
  SUNQRfact / SUNQRsol   src/sundials/sundials_iterative.c:181-329
Vector operations are numpy expressions, so dot products are summed in
numpy's order rather than the serial loop's: agreement with the reference
(tests/golden/spgmr_ref.npz, made by the reference itself) is to rounding,
which tests/test_spgmr_oracle.py checks.  The port also records the residual
norm of every iteration, so that fixture generation can reject cases whose
iteration count sits on the convergence threshold.
"""
from __future__ import annotations

import math

import numpy as np

SUCCESS, RES_REDUCED, CONV_FAIL = 0, 801, 802
QRFACT_FAIL, QRSOL_FAIL = 807, -811
PREC_NONE, PREC_LEFT, PREC_RIGHT, PREC_BOTH = 0, 1, 2, 3
MODIFIED_GS, CLASSICAL_GS = 1, 2
FACTOR = 1000.0


def _mgs(V, H, k, col):
    vk_norm = math.sqrt(float(np.dot(V[k], V[k])))
    for i in range(k):
        H[i, col] = float(np.dot(V[i], V[k]))
        V[k] = V[k] + (-H[i, col]) * V[i]
    new = math.sqrt(float(np.dot(V[k], V[k])))
    temp = FACTOR * vk_norm
    if temp + new != temp:
        return new
    nn2 = 0.0
    for i in range(k):
        p = float(np.dot(V[i], V[k]))
        temp = FACTOR * H[i, col]
        if temp + p == temp:
            continue
        H[i, col] += p
        V[k] = V[k] + (-p) * V[i]
        nn2 += p * p
    if nn2 != 0.0:
        prod = new * new - nn2
        new = math.sqrt(prod) if prod > 0.0 else 0.0
    return new


def _cgs(V, H, k, col):
    s = np.array([float(np.dot(V[k], V[j])) for j in range(k + 1)])
    vk_norm = math.sqrt(s[k])
    H[:k, col] = s[:k]
    w = V[k].copy()
    for j in range(k):
        w = w + (-s[j]) * V[j]
    V[k] = w
    new = math.sqrt(float(np.dot(V[k], V[k])))
    if FACTOR * new < vk_norm:
        s2 = np.array([float(np.dot(V[k], V[j])) for j in range(k)])
        H[:k, col] += s2
        w = V[k].copy()
        for j in range(k):
            w = w + (-s2[j]) * V[j]
        V[k] = w
        new = math.sqrt(float(np.dot(V[k], V[k])))
    return new


def _qr_add_column(n, H, q):
    col = n - 1
    for k in range(col):
        c, s = q[2 * k], q[2 * k + 1]
        t1, t2 = H[k, col], H[k + 1, col]
        H[k, col] = c * t1 - s * t2
        H[k + 1, col] = s * t1 + c * t2
    t1, t2 = H[col, col], H[col + 1, col]
    if t2 == 0.0:
        c, s = 1.0, 0.0
    elif abs(t2) >= abs(t1):
        t3 = t1 / t2
        s = -1.0 / math.sqrt(1.0 + t3 * t3)
        c = -s * t3
    else:
        t3 = t2 / t1
        c = 1.0 / math.sqrt(1.0 + t3 * t3)
        s = -c * t3
    q[2 * col], q[2 * col + 1] = c, s
    H[col, col] = c * t1 - s * t2
    return n if H[col, col] == 0.0 else 0


def _qr_solve(n, H, q, b):
    for k in range(n):
        c, s = q[2 * k], q[2 * k + 1]
        t1, t2 = b[k], b[k + 1]
        b[k] = c * t1 - s * t2
        b[k + 1] = s * t1 + c * t2
    for k in range(n - 1, -1, -1):
        if H[k, k] == 0.0:
            return k + 1
        b[k] /= H[k, k]
        for i in range(k):
            b[i] -= b[k] * H[i, k]
    return 0


def spgmr_solve(atimes, psolve, x, b, delta, *, maxl=5, max_restarts=0, gstype=MODIFIED_GS,
                pretype=PREC_NONE, s1=None, s2=None, zeroguess=False):
    """Solve A x = b.  ``atimes(v) -> A v``; ``psolve(r, lr) -> P^{-1} r``.

    Returns (flag, x, nli, resnorm, rho_history)."""
    x = np.array(x, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    left = pretype in (PREC_LEFT, PREC_BOTH)
    right = pretype in (PREC_RIGHT, PREC_BOTH)
    n = b.size
    V = np.zeros((maxl + 1, n))
    H = np.zeros((maxl + 1, maxl))
    q = np.zeros(2 * maxl)
    hist = []
    vt = b.copy() if zeroguess else b + (-1.0) * atimes(x)
    if left:
        vt = psolve(vt, PREC_LEFT)
    V[0] = s1 * vt if s1 is not None else vt
    r_norm = beta = math.sqrt(float(np.dot(V[0], V[0])))
    resnorm = r_norm
    nli = 0
    if r_norm <= delta:
        return SUCCESS, x, nli, resnorm, hist
    rho = beta
    xcor = np.zeros(n)
    converged = False
    krydim = 0
    for ntries in range(max_restarts + 1):
        H[:] = 0.0
        rot = 1.0
        V[0] = V[0] * (1.0 / r_norm)
        for l in range(maxl):
            nli += 1
            krydim = l + 1
            vt = V[l] / s2 if s2 is not None else V[l].copy()
            if right:
                vt = psolve(vt, PREC_RIGHT)
            w = atimes(vt)
            if left:
                w = psolve(w, PREC_LEFT)
            V[l + 1] = s1 * w if s1 is not None else w
            if gstype == CLASSICAL_GS:
                H[l + 1, l] = _cgs(V, H, l + 1, l)
            else:
                H[l + 1, l] = _mgs(V, H, l + 1, l)
            if _qr_add_column(krydim, H, q) != 0:
                return QRFACT_FAIL, x, nli, resnorm, hist
            rot *= q[2 * l + 1]
            resnorm = rho = abs(rot * r_norm)
            hist.append(rho)
            if rho <= delta:
                converged = True
                break
            V[l + 1] = V[l + 1] * (1.0 / H[l + 1, l])
        yg = np.zeros(krydim + 1)
        yg[0] = r_norm
        if _qr_solve(krydim, H, q, yg) != 0:
            return QRSOL_FAIL, x, nli, resnorm, hist
        acc = xcor.copy()
        for k in range(krydim):
            acc = acc + yg[k] * V[k]
        xcor = acc
        if converged or ntries == max_restarts:
            break
        sp = 1.0
        yg = np.zeros(krydim + 1)
        for i in range(krydim, 0, -1):
            yg[i] = sp * q[2 * i - 2]
            sp *= q[2 * i - 1]
        yg[0] = sp
        r_norm *= sp
        yg *= r_norm
        r_norm = abs(r_norm)
        acc = yg[0] * V[0]
        for k in range(1, krydim + 1):
            acc = acc + yg[k] * V[k]
        V[0] = acc
    if not converged and not rho < beta:
        return CONV_FAIL, x, nli, resnorm, hist
    if s2 is not None:
        xcor = xcor / s2
    vt = psolve(xcor, PREC_RIGHT) if right else xcor
    x = vt.copy() if zeroguess else x + vt
    return (SUCCESS if converged else RES_REDUCED), x, nli, resnorm, hist


# ---------------------------------------------------------------- operator
def tridiag_apply(v, s1, s2, diag, lo, hi):
    """z = S1^{-1} T S2 v for T = tridiag(lo, diag, hi), rounded like the
    reference unit test's ATimes (test_sunlinsol_spgmr_serial.c:ATimes):
    z_i = ((lo p_{i-1} + (diag v_i) s2_i) + hi p_{i+1}) / s1_i, p = v s2."""
    p = v * s2
    q = (diag * v) * s2
    z = q.copy()
    z[1:] = lo * p[:-1] + q[1:]
    z[:-1] = z[:-1] + hi * p[1:]
    return z / s1
