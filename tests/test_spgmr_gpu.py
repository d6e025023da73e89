"""GPU parity of SUNLinSol_SPGMR_GB300 (fused Gram-Schmidt SPGMR) against the
reference's own SPGMR (tests/golden/spgmr_ref.npz, SUNLinSol_SPGMR over
NVECTOR_SERIAL) and against the numpy oracle at sizes beyond the fixtures.

The operator and preconditioner are the reference unit test's
(test_sunlinsol_spgmr_serial.c: tridiagonal, row/column scaled, Jacobi),
applied on the device with torch element-wise kernels rounded exactly like the
unit test's C loop, on the vectors' stream (the legacy default stream).

Tolerances.  The GPU and the reference differ only in the order of the dot
products' sums (and in fused multiply-adds, in the default FMA mode), so:
return flag and iteration count must be EQUAL; the solution within
1e-10 * max|x| (exact mode) / 1e-9 (FMA mode); the residual norm -- a product
of Givens sines near convergence, which amplifies relative error -- within
1e-6 relative."""
import numpy as np
import pytest

from oracle import spgmr_port as sp

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

GOLD = np.load(__import__("pathlib").Path(__file__).parent / "golden" / "spgmr_ref.npz")
NAMES = [str(s) for s in GOLD["names"]]
X_TOL = {False: 1e-10, True: 1e-9}
RES_RTOL = 1e-6


def _dview(handle, n):
    from sundials_gb300.spgmr import device_array
    ptr = device_array(handle)

    class _A:
        __cuda_array_interface__ = {"shape": (n,), "typestr": "<f8", "data": (ptr, False),
                                    "version": 2}
    return torch.as_tensor(_A(), device="cuda")


class Problem:
    """A = S1^{-1} tridiag(lo, dg, hi) S2 and P^{-1} r = r / dg on the GPU."""

    def __init__(self, n, dg, lo, hi, s1, s2):
        self.n, self.dg, self.lo, self.hi = n, dg, lo, hi
        self.s1 = torch.tensor(s1, dtype=torch.float64, device="cuda")
        self.s2 = torch.tensor(s2, dtype=torch.float64, device="cuda")
        self.natimes = 0
        self.npsolve = 0
        self.fail_atimes = 0
        self.fail_psolve = 0

    def atimes(self, v, z):
        self.natimes += 1
        if self.fail_atimes:
            return self.fail_atimes
        vv, zz = _dview(v, self.n), _dview(z, self.n)
        p = vv * self.s2
        q = (self.dg * vv) * self.s2
        t = q.clone()
        t[1:] = self.lo * p[:-1] + q[1:]
        t[:-1] = t[:-1] + self.hi * p[1:]
        torch.div(t, self.s1, out=zz)
        return 0

    def psolve(self, r, z, tol, lr):
        self.npsolve += 1
        if self.fail_psolve:
            return self.fail_psolve
        torch.div(_dview(r, self.n), self.dg, out=_dview(z, self.n))
        return 0


def _setup(name):
    from sundials_gb300.nvector import NVector
    gs, pre, s1_on, s2_on, maxl, maxrs, n, zg = (int(v) for v in GOLD[f"{name}_params"])
    dg, lo, hi, delta = (float(v) for v in GOLD[f"{name}_op"])
    s1, s2 = GOLD[f"{name}_s1"], GOLD[f"{name}_s2"]
    prob = Problem(n, dg, lo, hi, s1, s2)
    vec = dict(x=NVector.from_numpy(GOLD[f"{name}_x0"]), b=NVector.from_numpy(GOLD[f"{name}_b"]),
               s1=NVector.from_numpy(s1) if s1_on else None,
               s2=NVector.from_numpy(s2) if s2_on else None)
    cfg = dict(gs=gs, pre=pre, maxl=maxl, maxrs=maxrs, n=n, zg=bool(zg), delta=delta)
    return prob, vec, cfg


def _solver(prob, vec, cfg, fused=True):
    from sundials_gb300.spgmr import SPGMR
    S = SPGMR(vec["x"], cfg["pre"], cfg["maxl"])
    assert S.set_gs_type(cfg["gs"]) == 0
    assert S.set_max_restarts(cfg["maxrs"]) == 0
    assert S.set_fused(fused) == 0
    assert S.set_atimes(prob.atimes) == 0
    assert S.set_preconditioner(prob.psolve) == 0
    assert S.set_scaling_vectors(vec["s1"], vec["s2"]) == 0
    assert S.initialize() == 0
    assert S.setup() == 0
    assert S.set_zero_guess(cfg["zg"]) == 0
    return S


@pytest.mark.parametrize("fma", [False, True], ids=["exact", "fma"])
@pytest.mark.parametrize("fused", [True, False], ids=["fused", "ops"])
@pytest.mark.parametrize("name", NAMES)
def test_matches_reference_spgmr(name, fused, fma):
    prob, vec, cfg = _setup(name)
    for v in vec.values():
        if v is not None:
            v.set_fma(fma)
    S = _solver(prob, vec, cfg, fused)
    flag = S.solve(vec["x"], vec["b"], cfg["delta"])
    torch.cuda.synchronize()
    assert flag == int(GOLD[f"{name}_flag"][0])
    assert S.last_flag == flag
    assert S.num_iters == int(GOLD[f"{name}_nli"][0])
    rref = float(GOLD[f"{name}_resnorm"][0])
    assert abs(S.res_norm - rref) <= RES_RTOL * rref + 1e-300
    x, xref = vec["x"].get(), GOLD[f"{name}_x"]
    assert np.max(np.abs(x - xref)) <= X_TOL[fma] * max(1.0, np.max(np.abs(xref)))
    S.free()


def test_fused_path_synchronises_once_per_iteration():
    """Modified and classical GS, maxl 20, 16 iterations: the fused solver
    makes one stream synchronisation per Arnoldi step (+1 for the initial
    residual norm); the reference's operation sequence makes k+2 per step
    (MGS) or 2 (CGS)."""
    counts = {}
    for name in ("mgs_none", "cgs_none"):
        for fused in (True, False):
            prob, vec, cfg = _setup(name)
            S = _solver(prob, vec, cfg, fused)
            assert S.solve(vec["x"], vec["b"], cfg["delta"]) == 0
            counts[(name, fused)] = (S.num_syncs, S.num_iters)
            S.free()
    for name in ("mgs_none", "cgs_none"):
        syncs, nli = counts[(name, True)]
        assert syncs == nli + 1
    assert counts[("mgs_none", False)][0] > 5 * counts[("mgs_none", True)][0]
    assert counts[("cgs_none", False)][0] >= 2 * counts[("cgs_none", True)][0] - 2


@pytest.mark.parametrize("gs", [1, 2], ids=["mgs", "cgs"])
@pytest.mark.parametrize("n", [(1 << 20) + 3, 1 << 22])
def test_large_against_port(gs, n):
    """Sizes with odd tails and multi-block reductions, right preconditioning
    and both scalings, 3 restarts of maxl 8: against the numpy oracle."""
    from sundials_gb300.nvector import NVector
    rng = np.random.default_rng(n + gs)
    dg, lo, hi = 2.6, -1.0, -0.9
    s1 = 1.0 + 1000.0 * rng.uniform(0, 1, n)
    s2 = 1.0 + 1000.0 * rng.uniform(0, 1, n)
    xtrue = (1.0 + rng.uniform(0, 1, n)) / s2
    b = sp.tridiag_apply(xtrue, s1, s2, dg, lo, hi)
    delta = 1e-6 * np.sqrt(n)
    pflag, px, pnli, pres, hist = sp.spgmr_solve(
        lambda v: sp.tridiag_apply(v, s1, s2, dg, lo, hi), lambda r, lr: r / dg, np.zeros(n), b,
        delta, maxl=8, max_restarts=3, gstype=gs, pretype=sp.PREC_RIGHT, s1=s1, s2=s2,
        zeroguess=True)
    assert min(abs(h / delta - 1) for h in hist) > 0.01
    prob = Problem(n, dg, lo, hi, s1, s2)
    vec = dict(x=NVector(n), b=NVector.from_numpy(b), s1=NVector.from_numpy(s1),
               s2=NVector.from_numpy(s2))
    cfg = dict(gs=gs, pre=sp.PREC_RIGHT, maxl=8, maxrs=3, n=n, zg=True, delta=delta)
    S = _solver(prob, vec, cfg)
    flag = S.solve(vec["x"], vec["b"], delta)
    assert (flag, S.num_iters) == (pflag, pnli)
    assert abs(S.res_norm - pres) <= RES_RTOL * pres
    x = vec["x"].get()
    assert np.max(np.abs(x - px)) <= 1e-9 * np.max(np.abs(px))
    # and the solve is reproducible to the bit
    x1 = x.copy()
    vec["x"].set(np.zeros(n))
    S.set_zero_guess(True)
    assert S.solve(vec["x"], vec["b"], delta) == flag
    assert np.array_equal(vec["x"].get().view(np.int64), x1.view(np.int64))
    S.free()


@pytest.mark.parametrize("where,status,expect", [
    ("atimes", 1, 803), ("atimes", -1, -805), ("psolve", 1, 805), ("psolve", -1, -808)])
def test_callback_failures_map_to_reference_codes(where, status, expect):
    prob, vec, cfg = _setup("mgs_left")
    S = _solver(prob, vec, cfg)
    setattr(prob, "fail_" + where, status)
    assert S.solve(vec["x"], vec["b"], cfg["delta"]) == expect
    assert S.last_flag == expect
    S.free()


@pytest.mark.parametrize("status,expect", [(1, 804), (-1, -806), (0, 0)])
def test_psetup_status(status, expect):
    from sundials_gb300.nvector import NVector
    from sundials_gb300.spgmr import SPGMR
    y = NVector(64)
    S = SPGMR(y, 1, 5)
    S.set_atimes(lambda v, z: 0)
    S.set_preconditioner(lambda r, z, tol, lr: 0, psetup=lambda: status)
    assert S.initialize() == 0
    assert S.setup() == expect
    assert S.last_flag == expect
    S.free()


def test_object_contract():
    """Type, ID, option validation and workspace size as the reference's."""
    from sundials_gb300.nvector import NVector
    from sundials_gb300.spgmr import SPGMR
    y = NVector(1000)
    S = SPGMR(y, 7, 0)                         # illegal pretype -> NONE, maxl <= 0 -> 5
    assert S.gettype() == 1 and S.getid() == 8  # ITERATIVE, SUNLINEARSOLVER_SPGMR
    assert S.set_gs_type(3) == -9997 and S.set_prec_type(9) == -9997
    assert S.set_max_restarts(-4) == 0
    assert S.initialize() == -9999             # ATimes not set
    S.set_atimes(lambda v, z: 0)
    assert S.initialize() == 0
    lrw, liw = S.space()
    assert lrw == 1000 * (5 + 5) + 5 * (5 + 5) + 2
    assert S.resid()
    S.free()
