"""Pin the CVODE restatement (oracle/cvode_bdf_port.c) against the reference's
own CVODE runs stored in tests/golden/kinetics_cvode_ref.npz: every counter,
the return flag (one system ends in CV_ERR_FAILURE), the final t and h, and
the bits of y(100) must match exactly."""
from pathlib import Path

import numpy as np
import pytest

from sundials_gb300 import kinetics as K

GOLD = Path(__file__).resolve().parent / "golden" / "kinetics_cvode_ref.npz"


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(GOLD))


@pytest.fixture(scope="module")
def full_batch():
    return K.generate(65536, seed=1)


def test_generator_is_stable(full_batch):
    b = full_batch
    assert b.nsys == 65536 and b.n.min() >= 8 and b.n.max() <= 64
    assert abs(b.n.mean() - 36.0) < 0.5
    assert b.rk.size == 2 * int(b.n.sum())
    # distinct species within every reaction
    assert np.all(b.ra != b.rb)
    bi = b.rtype == 1
    assert np.all((b.rc[bi] != b.ra[bi]) & (b.rc[bi] != b.rb[bi]))
    assert np.all(b.rc[~bi] == -1)
    assert b.rk.min() >= 1e-2 and b.rk.max() <= 1e6
    # independent regeneration of a slice gives the same arrays
    s = K.generate(16, seed=1, first=1000)
    sub = b.subset(np.arange(1000, 1016))
    for f in ("n", "rtype", "ra", "rb", "rc", "rk", "y0"):
        assert np.array_equal(getattr(s, f), getattr(sub, f)), f


@pytest.mark.parametrize("tag", ["r6", "r4"])
def test_port_matches_reference_cvode(oracle_lib, gold, full_batch, tag):
    from oracle import port
    ids = gold[f"{tag}_ids"]
    sub = full_batch.subset(ids)
    st, yout = port.bdf_batch(sub, rtol=float(gold[f"{tag}_rtol"][0]), atol=1e-12, tout=100.0)
    for f in K.STATS_FIELDS + ["tn", "hu"]:
        mism = np.nonzero(st[f] != gold[f"{tag}_{f}"])[0]
        assert mism.size == 0, f"{f} differs for systems {ids[mism][:10]}"
    assert np.array_equal(yout.view(np.int64), gold[f"{tag}_y"].view(np.int64))
    if tag == "r4":
        assert (st["flag"] != 0).sum() >= 1  # the reference's own failure is reproduced


def test_reference_pow_sensitivity(oracle_lib, gold, full_batch):
    """The reference algorithm's own sensitivity to pow's last bit: the
    restatement with a correctly rounded pow against the reference's runs."""
    from oracle import port
    sub = full_batch.subset(gold["r6_ids"])
    st, yout = port.bdf_batch(sub, rtol=1e-6, atol=1e-12, tout=100.0, dd_pow=True)
    same = np.ones(sub.nsys, bool)
    for f in K.STATS_FIELDS:
        same &= st[f] == gold[f"r6_{f}"]
    assert same.mean() > 0.9  # counters unchanged for most systems
    assert np.all(st["flag"] == gold["r6_flag"])
