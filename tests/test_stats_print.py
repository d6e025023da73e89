"""CPU: SUNBatchBDF_GB300_PrintAllStats against the reference's own
CVodePrintAllStats (src/cvode/cvode_io.c:1626).

Where the reference library is built (oracle/_ref), a real CVODE run of the
Robertson problem with SUNLINSOL_DENSE and an analytic Jacobian prints its
statistics in both formats; the batch printer, given the same counters,
must print the same bytes.  Everywhere, the printer's layout is checked on
fixed counters (names, order, formats, argument checks)."""
import ctypes as ct
import os
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
REF = ROOT / "oracle" / "_ref" / "libsundials_ref.so"
libc = ct.CDLL(None)
libc.fopen.restype = ct.c_void_p
libc.fopen.argtypes = [ct.c_char_p, ct.c_char_p]
libc.fclose.argtypes = [ct.c_void_p]


def _print_batch(lib, rec, fmt, path):
    f = lib.SUNBatchBDF_GB300_PrintAllStats
    f.restype = ct.c_int
    f.argtypes = [ct.c_void_p, ct.c_int64, ct.c_int64, ct.c_void_p, ct.c_int]
    fp = libc.fopen(str(path).encode(), b"w")
    rc = f(rec.ctypes.data, rec.size, 0, fp, fmt)
    libc.fclose(fp)
    return rc, Path(path).read_text()


def _record(**kw):
    from sundials_gb300.kinetics import BATCH_STATS_DTYPE
    rec = np.zeros(1, BATCH_STATS_DTYPE)
    for k, v in kw.items():
        rec[k] = v
    return rec


def test_layout_on_fixed_counters(gb300_lib, tmp_path):
    rec = _record(tn=100.0, nst=1200, netf=44, ncfn=0, h0u=1e-9, hu=3.5, next_h=4.0, qu=5,
                  next_q=5, nfe=1518, nni=1515, nnf=0, nsetups=143, nje=22)
    rc, table = _print_batch(gb300_lib, rec, 0, tmp_path / "t.txt")
    assert rc == 0
    lines = table.splitlines()
    assert lines[0] == "Current time                  = 100"
    assert lines[1] == "Steps                         = 1200"
    assert "NLS iters per step            = 1.2625" in lines
    assert lines[-1] == "Root fn evals                 = 0"
    assert len(lines) == 27
    rc, csv = _print_batch(gb300_lib, rec, 1, tmp_path / "c.txt")
    assert rc == 0 and not csv.endswith("\n")
    fields = csv.split(",")
    assert fields[:4] == ["Current time", " 1.000000000000000e+02", "Steps", "1200"]
    assert len(fields) == 54
    assert _print_batch(gb300_lib, rec, 2, tmp_path / "x.txt")[0] == -9997


@pytest.mark.skipif(not REF.exists(), reason="reference library not built on this machine")
@pytest.mark.parametrize("fmt", [0, 1], ids=["table", "csv"])
def test_same_bytes_as_reference(gb300_lib, tmp_path, fmt):
    L = ct.CDLL(str(REF))
    vp, d, ci, i64 = ct.c_void_p, ct.c_double, ct.c_int, ct.c_int64
    for name, res, args in [
        ("SUNContext_Create", ci, [ci, ct.POINTER(vp)]),
        ("N_VNew_Serial", vp, [i64, vp]),
        ("N_VGetArrayPointer", ct.POINTER(d), [vp]),
        ("CVodeCreate", vp, [ci, vp]),
        ("CVodeInit", ci, [vp, vp, d, vp]),
        ("CVodeSStolerances", ci, [vp, d, d]),
        ("SUNDenseMatrix", vp, [i64, i64, vp]),
        ("SUNDenseMatrix_Column", ct.POINTER(d), [vp, i64]),
        ("SUNLinSol_Dense", vp, [vp, vp, vp]),
        ("CVodeSetLinearSolver", ci, [vp, vp, vp]),
        ("CVodeSetJacFn", ci, [vp, vp]),
        ("CVode", ci, [vp, d, vp, ct.POINTER(d), ci]),
        ("CVodePrintAllStats", ci, [vp, vp, ci]),
        ("CVodeGetActualInitStep", ci, [vp, ct.POINTER(d)]),
    ]:
        fn = getattr(L, name)
        fn.restype, fn.argtypes = res, args
    RHS = ct.CFUNCTYPE(ci, d, vp, vp, vp)
    JAC = ct.CFUNCTYPE(ci, d, vp, vp, vp, vp, vp, vp, vp)

    def arr(v):
        return np.ctypeslib.as_array(L.N_VGetArrayPointer(v), shape=(3,))

    @RHS
    def f(t, y, ydot, data):
        a, b = arr(y), arr(ydot)
        b[0] = -0.04 * a[0] + 1e4 * a[1] * a[2]
        b[2] = 3e7 * a[1] * a[1]
        b[1] = -b[0] - b[2]
        return 0

    @JAC
    def jac(t, y, fy, J, data, t1, t2, t3):
        a = arr(y)
        cols = [np.ctypeslib.as_array(L.SUNDenseMatrix_Column(J, j), shape=(3,)) for j in range(3)]
        cols[0][:] = [-0.04, 0.04, 0.0]
        cols[1][:] = [1e4 * a[2], -1e4 * a[2] - 6e7 * a[1], 6e7 * a[1]]
        cols[2][:] = [1e4 * a[1], -1e4 * a[1], 0.0]
        return 0

    ctx = vp()
    assert L.SUNContext_Create(0, ct.byref(ctx)) == 0
    y = L.N_VNew_Serial(3, ctx)
    arr(y)[:] = [1.0, 0.0, 0.0]
    mem = L.CVodeCreate(2, ctx)
    assert L.CVodeInit(mem, ct.cast(f, vp), 0.0, y) == 0
    assert L.CVodeSStolerances(mem, 1e-4, 1e-8) == 0
    A = L.SUNDenseMatrix(3, 3, ctx)
    LS = L.SUNLinSol_Dense(y, A, ctx)
    assert L.CVodeSetLinearSolver(mem, LS, A) == 0
    assert L.CVodeSetJacFn(mem, ct.cast(jac, vp)) == 0
    t = d()
    assert L.CVode(mem, 40.0, y, ct.byref(t), 1) == 0
    ref_path = tmp_path / "ref.txt"
    fp = libc.fopen(str(ref_path).encode(), b"w")
    assert L.CVodePrintAllStats(mem, fp, fmt) == 0
    libc.fclose(fp)
    ref = ref_path.read_text()
    # the reference's counters, read back from the same output (so the
    # printed digits are the ones both printers round)
    kv = {}
    if fmt == 0:
        for line in ref.splitlines():
            k, v = line.split("=")
            kv[k.strip()] = float(v)
    else:
        parts = ref.split(",")
        kv = {parts[i]: float(parts[i + 1]) for i in range(0, len(parts), 2)}
    assert kv["LS RHS fn evals"] == 0 and kv["LS iters"] == 0
    rec = _record(tn=kv["Current time"], nst=kv["Steps"], netf=kv["Error test fails"],
                  ncfn=kv["NLS step fails"], h0u=kv["Initial step size"],
                  hu=kv["Last step size"], next_h=kv["Current step size"],
                  qu=kv["Last method order"], next_q=kv["Current method order"],
                  nfe=kv["RHS fn evals"], nni=kv["NLS iters"], nnf=kv["NLS fails"],
                  nsetups=kv["LS setups"], nje=kv["Jac fn evals"])
    rc, ours = _print_batch(gb300_lib, rec, fmt, tmp_path / "ours.txt")
    assert rc == 0
    assert ours == ref


@pytest.mark.gpu
def test_batch_fills_print_fields(gb300_lib, tmp_path):
    """The integrator records the initial step, the next step and order; in
    the exact mode the step counters equal the CVODE restatement's."""
    from oracle import port
    from sundials_gb300 import kinetics as K
    from sundials_gb300.batch import BatchBDF
    batch = K.generate(256, seed=1).subset(np.arange(0, 256, 4))
    _, st = BatchBDF(batch).configure(1e-6, 1e-12, "fp64_exact").solve(100.0)
    pst, _ = port.bdf_batch(batch, dd_pow=True)
    assert np.array_equal(st["nst"], pst["nst"]) and np.array_equal(st["hu"], pst["hu"])
    assert np.all(st["h0u"] > 0) and np.all(st["next_h"] > 0)
    assert np.all((st["next_q"] >= 1) & (st["next_q"] <= 5))
    rc, table = _print_batch(gb300_lib, st[3:4].copy(), 0, tmp_path / "s.txt")
    assert rc == 0 and f"Steps                         = {int(st['nst'][3])}" in table
