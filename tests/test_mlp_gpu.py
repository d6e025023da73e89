"""GPU: the learned Newton predictor (include/sunmlp_gb300.h).

* the tensor-core training kernels' loss and gradients against the CPU oracle
  (oracle/mlp_port.py, same BF16 rounding points): relative error per
  parameter block <= 2e-3 (FP32 accumulation order and rare BF16 tie flips);
* the batched inference kernel (the integrator's arithmetic) against the
  oracle's forward pass: <= 1e-5 relative;
* training by the library's Adam steps fits a teacher network;
* the recorder writes well-formed rows;
* in the integrator the predictor leaves accuracy within the plain solver's
  error bound against the FP64 oracle (median <= 1.5x, p99 <= 2x, max <= 3x
  the reference CVODE's) with no failed system, and the trained network is
  kept far more often than an untrained one -- what training gains -- while
  the counters of that A/B run are printed."""
import numpy as np
import pytest

from oracle import mlp_port as mp

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _rand_rows(rng, m):
    X = rng.uniform(-1, 1, (m, mp.IN_PAD))
    X[:, 129:] = 0.0
    return mp.bf16_bits(X)


def _dev(a, dtype):
    return torch.from_numpy(np.ascontiguousarray(a)).to(dtype=dtype).cuda()


@pytest.mark.parametrize("m,seed", [(128, 1), (512, 2)])
def test_gradients_match_oracle(m, seed):
    from sundials_gb300.mlp import MLP
    rng = np.random.default_rng(seed)
    Xb = _rand_rows(rng, m)
    T = rng.uniform(-2, 2, (m, mp.OUT)).astype(np.float32)
    net = MLP(seed=seed + 10)
    p = net.get_params()
    dX = _dev(Xb.view(np.int16), torch.int16)
    dT = _dev(T, torch.float32)
    g = torch.zeros(mp.NPARAMS, dtype=torch.float32, device="cuda")
    loss = net.gradients(m, dX.data_ptr(), dT.data_ptr(), g.data_ptr())
    lref, gref = mp.loss_and_grad(p, mp.from_bits(Xb), T)
    assert abs(loss - lref) <= 1e-5 * lref
    gg = g.cpu().numpy().astype(np.float64)
    for a, b in [(mp.P_W1, mp.P_B1), (mp.P_B1, mp.P_W2), (mp.P_W2, mp.P_B2),
                 (mp.P_B2, mp.P_W3), (mp.P_W3, mp.P_B3), (mp.P_B3, mp.NPARAMS)]:
        err = np.linalg.norm(gg[a:b] - gref[a:b]) / np.linalg.norm(gref[a:b])
        assert err <= 2e-3, (a, err)


def test_gradients_reject_ragged_batch():
    from sundials_gb300.mlp import MLP
    net = MLP(seed=1)
    with pytest.raises(AssertionError):
        net.gradients(100, 0, 0, 0)


def test_forward_matches_oracle():
    from sundials_gb300.mlp import MLP
    rng = np.random.default_rng(4)
    m = 1000
    Xb = _rand_rows(rng, m)
    net = MLP(seed=3)
    out = torch.zeros((m, mp.OUT), dtype=torch.float32, device="cuda")
    dX = _dev(Xb.view(np.int16), torch.int16)
    net.forward(m, dX.data_ptr(), out.data_ptr())
    O, _ = mp.forward(net.get_params(), mp.from_bits(Xb))
    assert np.max(np.abs(out.cpu().numpy() - O)) <= 1e-5 * np.max(np.abs(O))


def test_training_fits_a_teacher():
    from sundials_gb300 import learned
    from sundials_gb300.mlp import MLP
    rng = np.random.default_rng(8)
    m = 128 * 64
    Xb = _rand_rows(rng, m)
    teacher = MLP(seed=99).get_params()
    T, _ = mp.forward(teacher, mp.from_bits(Xb))
    dX = _dev(Xb.view(np.int16), torch.int16)
    dT = _dev(T.astype(np.float32), torch.float32)
    net = MLP(seed=5)
    g = torch.zeros(mp.NPARAMS, dtype=torch.float32, device="cuda")
    l0 = net.gradients(m, dX.data_ptr(), dT.data_ptr(), g.data_ptr())
    learned.train(net, dX, dT, epochs=60, batch=1024, lr=2e-3)
    l1 = net.gradients(m, dX.data_ptr(), dT.data_ptr(), g.data_ptr())
    assert l1 < 0.2 * l0, (l0, l1)


def test_recorder_rows():
    from sundials_gb300 import kinetics as K, learned
    X, T = learned.record(256, [1001], 1 << 16)
    assert X.shape[0] > 1000
    Xh = mp.from_bits(X.cpu().numpy().view(np.uint16))
    Th = T.cpu().numpy()
    assert np.all(np.isfinite(Xh)) and np.all(np.isfinite(Th))
    assert np.all(Xh[:, 129:] == 0.0)
    assert np.all(np.abs(Th) <= learned.TARGET_CLIP)
    # y features of absent species are zero; present ones lie in [0, 1]
    assert np.all((Xh[:, :64] >= -1e-3) & (Xh[:, :64] <= 1.01))


def test_predictor_in_integrator_keeps_accuracy():
    import bench
    from sundials_gb300 import kinetics as K, learned
    from sundials_gb300.mlp import MLP
    X, T = learned.record(2048, range(1001, 1003), 1 << 19)
    trained = MLP(seed=7)
    losses = learned.train(trained, X, T, epochs=4)
    untrained = MLP(seed=7)
    full = K.generate(65536, seed=1)
    ids = np.arange(0, 65536, 64)  # the golden sample with FP64-oracle solutions
    test = full.subset(ids)
    ev = learned.evaluate(test, trained)
    ev0 = learned.evaluate(test, untrained)
    for k in ("plain", "learned"):
        yo = np.zeros(full.y0.size)
        for j, i in enumerate(ids):
            yo[full.y_off[i]:full.y_off[i + 1]] = ev[k]["y"][test.y_off[j]:test.y_off[j + 1]]
        acc = bench.accuracy_vs_oracle(full, yo)
        ref = acc["reference_cvode"]
        assert ev[k]["failed"] == 0
        assert acc["median"] <= 1.5 * ref["median"]
        assert acc["p99"] <= 2.0 * ref["p99"]
        assert acc["max"] <= 3.0 * ref["max"]
    kept_trained = ev["learned"]["kept"] / ev["learned"]["calls"]
    kept_untrained = ev0["learned"]["kept"] / ev0["learned"]["calls"]
    print(f"\nlearned predictor: loss {losses[0]:.3f} -> {losses[-1]:.3f}; kept "
          f"{100 * kept_trained:.1f}% (untrained {100 * kept_untrained:.1f}%); "
          f"nni {ev['plain']['nni']} -> {ev['learned']['nni']}, "
          f"nfe {ev['plain']['nfe']} -> {ev['learned']['nfe']}, kernel ms "
          f"{ev['plain']['kernel_ms']:.1f} -> {ev['learned']['kernel_ms']:.1f}")
    assert kept_trained > 2.0 * kept_untrained
