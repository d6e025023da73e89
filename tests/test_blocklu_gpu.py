"""Block-diagonal SUNMatrix and BlockLU SUNLinearSolver against the dense
restatement (oracle/dense_port.c, pinned to the reference's
SUNDlsMat_denseGETRF / GETRS), block by block.

Tolerances: FP64 precision -- factors, pivots and solutions BIT-EXACT per
block (the kernels perform the reference's operations in its order, without
FMA); ScaleAddI, ScaleAdd, Copy, Matvec bit-exact likewise.  MIXED precision
(FP32 inverse + one FP64 refinement sweep): |A x - b|_inf <= 1e-10 |b|_inf on
well-conditioned blocks, as in test_sunlinsol_dense.c's diagonally dominant
matrices."""
import numpy as np
import pytest

from sundials_gb300 import blockdiag as BD
from sundials_gb300.nvector import NVector

pytestmark = pytest.mark.gpu
SIZES = [1, 3, 3, 8, 9, 17, 32, 33, 64, 5, 2, 47]


@pytest.fixture(scope="module")
def port(oracle_lib):
    from oracle import port as p
    return p


def blocks_dd(sizes, seed):
    """Random blocks made diagonally dominant (test_sunlinsol_dense.c style)."""
    rng = np.random.default_rng(seed)
    out = []
    for n in sizes:
        a = rng.uniform(-1, 1, (n, n))
        a += np.diag(np.full(n, float(n)))
        out.append(a)
    return out


def exact_vec(a):
    v = NVector.from_numpy(a)
    v.set_fma(False)
    return v


def beq(a, b):
    return np.array_equal(np.asarray(a).view(np.int64), np.asarray(b).view(np.int64))


def test_fp64_factor_and_solve_bit_identical(gb300_lib, port):
    sizes = SIZES * 20
    M = BD.BlockDiag(sizes)
    blocks = blocks_dd(sizes, 1)
    M.set_blocks(blocks)
    N = int(np.sum(sizes))
    b = np.random.default_rng(2).uniform(-1, 1, N)
    X, B = exact_vec(np.zeros(N)), exact_vec(b)
    S = BD.BlockLU(B.v, M, BD.FP64)
    assert S.gettype(S.S) == 0  # SUNLINEARSOLVER_DIRECT
    assert S.initialize(S.S) == 0
    assert S.setup(S.S, M.A) == 0
    assert S.solve(S.S, M.A, X.v, B.v, 0.0) == 0
    x = X.get()
    lu = M.get_blocks()
    for k, a in enumerate(blocks):
        rl, rp, flag = port.dense_lu(a.T.copy())
        assert flag == 0
        assert beq(lu[k].T, rl), k
        xs = port.dense_solve(rl, rp, b[M.off[k]:M.off[k + 1]])
        assert beq(x[M.off[k]:M.off[k + 1]], xs), k
    S.free()


def test_mixed_solve_accuracy(gb300_lib):
    sizes = SIZES * 20
    M = BD.BlockDiag(sizes)
    blocks = blocks_dd(sizes, 3)
    M.set_blocks(blocks)
    N = int(np.sum(sizes))
    b = np.random.default_rng(4).uniform(-1, 1, N)
    X, B = exact_vec(np.zeros(N)), exact_vec(b)
    S = BD.BlockLU(B.v, M, BD.MIXED)
    assert S.setup(S.S, M.A) == 0
    assert S.solve(S.S, M.A, X.v, B.v, 0.0) == 0
    x = X.get()
    for k, a in enumerate(blocks):
        xs = x[M.off[k]:M.off[k + 1]]
        bs = b[M.off[k]:M.off[k + 1]]
        assert np.max(np.abs(a @ xs - bs)) <= 1e-10 * np.max(np.abs(bs)), k
    # the FP64 matrix is left intact by a MIXED setup
    for k, a in enumerate(M.get_blocks()):
        assert beq(a, blocks[k])
    S.free()


def test_mixed_falls_back_to_fp64_for_ill_conditioned_blocks(gb300_lib, port):
    """Newton matrices I - gamma J of Robertson cells late in an integration
    (gamma ~ 1e9, condition ~ 1e13, beyond FP32) among well-conditioned
    blocks: the ill-conditioned ones fail the setup's probe and are factored
    and solved by the FP64 path -- bit for bit SUNDlsMat_denseGETRF/GETRS --
    while the others keep the FP32 inverse (accurate to refinement level)."""
    rng = np.random.default_rng(8)
    sizes = [3] * 40
    blocks = []
    ill = set(range(0, 40, 3))
    for k in range(40):
        if k in ill:
            k1, k2, k3 = 0.04, 3e7, 1e4
            y2, y3 = 1e-12 * rng.uniform(1, 2), rng.uniform(0.5, 1.0)
            J = np.array([[-k1, k3 * y3, k3 * y2],
                          [k1, -k3 * y3 - 2 * k2 * y2, -k3 * y2],
                          [0.0, 2 * k2 * y2, 0.0]])
            blocks.append(np.eye(3) - 1e9 * rng.uniform(1, 3) * J)
        else:
            blocks.append(np.eye(3) * 4.0 + rng.uniform(-1, 1, (3, 3)))
    M = BD.BlockDiag(sizes)
    M.set_blocks(blocks)
    N = 3 * 40
    b = rng.uniform(-1, 1, N)
    X, B = exact_vec(np.zeros(N)), exact_vec(b)
    S = BD.BlockLU(B.v, M, BD.MIXED)
    assert S.setup(S.S, M.A) == 0
    assert S.solve(S.S, M.A, X.v, B.v, 0.0) == 0
    x = X.get()
    for k, a in enumerate(blocks):
        xs, bs = x[3 * k:3 * k + 3], b[3 * k:3 * k + 3]
        if k in ill:
            rl, rp, flag = port.dense_lu(a.T.copy())
            assert flag == 0
            assert beq(xs, port.dense_solve(rl, rp, bs)), k
        else:
            assert np.max(np.abs(a @ xs - bs)) <= 1e-10 * np.max(np.abs(bs)), k
    for k, a in enumerate(M.get_blocks()):  # the matrix is still left intact
        assert beq(a, blocks[k])
    S.free()


@pytest.mark.parametrize("precision", [BD.FP64, BD.MIXED])
def test_zero_pivot_is_recoverable_failure(gb300_lib, precision):
    sizes = [3, 4, 40]
    M = BD.BlockDiag(sizes)
    blocks = blocks_dd(sizes, 5)
    blocks[1][:, 2] = 0.0  # block 1 singular: zero column 2
    M.set_blocks(blocks)
    B = exact_vec(np.ones(int(np.sum(sizes))))
    S = BD.BlockLU(B.v, M, precision)
    assert S.setup(S.S, M.A) == 808  # SUNLS_LUFACT_FAIL
    assert S.lastflag(S.S) == 3 + 2 + 1  # global column of the zero pivot, plus 1
    S.free()


def test_matrix_ops_bit_identical(gb300_lib):
    sizes = SIZES * 10
    M = BD.BlockDiag(sizes)
    blocks = blocks_dd(sizes, 6)
    M.set_blocks(blocks)
    assert M.getid(M.A) == 10  # SUNMATRIX_CUSTOM
    C = M.clone()
    assert C.zero(C.A) == 0 and np.all(C.get_flat() == 0.0)
    assert M.copy(M.A, C.A) == 0 and beq(C.get_flat(), M.get_flat())
    # ScaleAddI: A = c A + I  (c*a, then +1 on the diagonal)
    c = -0.37
    assert C.scaleaddi(c, C.A) == 0
    for k, a in enumerate(C.get_blocks()):
        ref = blocks[k] * c
        ref[np.diag_indices(sizes[k])] = ref[np.diag_indices(sizes[k])] + 1.0
        assert beq(a, ref), k
    # ScaleAdd: C = 2 C + M
    assert C.scaleadd(2.0, C.A, M.A) == 0
    for k, a in enumerate(C.get_blocks()):
        ref = blocks[k] * c
        ref[np.diag_indices(sizes[k])] = ref[np.diag_indices(sizes[k])] + 1.0
        assert beq(a, 2.0 * ref + blocks[k]), k
    # Matvec: y_i = sum_j a_ij x_j in column order
    N = int(np.sum(sizes))
    x = np.random.default_rng(7).uniform(-1, 1, N)
    X, Y = exact_vec(x), exact_vec(np.zeros(N))
    assert M.matvec(M.A, X.v, Y.v) == 0
    y = Y.get()
    for k, a in enumerate(blocks):
        xs = x[M.off[k]:M.off[k + 1]]
        acc = np.zeros(sizes[k])
        for j in range(sizes[k]):
            acc = acc + a[:, j] * xs[j]
        assert beq(y[M.off[k]:M.off[k + 1]], acc), k
    C.destroy()
    M.destroy()


def test_many_small_blocks(gb300_lib, port):
    """2^16 blocks of 3x3 (the Robertson / Brusselator cell shape)."""
    nb = 1 << 16
    M = BD.BlockDiag([3] * nb)
    rng = np.random.default_rng(9)
    flat = rng.uniform(-1, 1, 9 * nb)
    for k in range(3):
        flat[k * 3 + k::9] += 3.0
    blocks = [flat[9 * b:9 * b + 9].reshape(3, 3).T for b in range(64)]
    assert M.lib.SUNMatrix_BlockDiag_GB300_CopyToDevice(M.A, flat.ctypes.data) == 0
    b = rng.uniform(-1, 1, 3 * nb)
    X, B = exact_vec(np.zeros(3 * nb)), exact_vec(b)
    S = BD.BlockLU(B.v, M, BD.FP64)
    assert S.setup(S.S, M.A) == 0 and S.solve(S.S, M.A, X.v, B.v, 0.0) == 0
    x = X.get()
    for k in range(64):
        rl, rp, _ = port.dense_lu(blocks[k].T.copy())
        assert beq(x[3 * k:3 * k + 3], port.dense_solve(rl, rp, b[3 * k:3 * k + 3]))
    S.free()
