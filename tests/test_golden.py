"""Committed fixtures (tests/golden/oracle_small.npz, written by
tests/golden/make_golden.py from the CPU oracle): the oracle reproduces them
bit for bit on this host, so the restatement cannot drift unnoticed between
machines or edits.  The GPU side of the same fixtures is
tests/test_gpu_golden.py."""
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).with_name("golden") / "oracle_small.npz"
QOM, VUN = 200.0, 1.0 / 20.0


@pytest.fixture(scope="module")
def gold():
    with np.load(GOLDEN) as z:
        return {k: z[k] for k in z.files}


@pytest.mark.parametrize("method", ["rk5", "dop853"])
def test_oracle_reproduces_the_fixture(oracle_lib, gold, method):
    import oracle
    eta = float(gold[f"{method}_eta"])
    s, c, st = oracle.integrate(method, gold[f"{method}_params"], gold["time"], gold["uu"],
                                gold["bb"], gold["state0"].copy(), eta=eta,
                                jj=gold["jj"] if eta else None)
    assert (st == 0).all() and np.array_equal(st, gold[f"{method}_status"])
    assert np.array_equal(c, gold[f"{method}_cnt"])
    assert (c[:, 0] == c[:, 1] + c[:, 2]).all()
    assert np.array_equal(s.view(np.int64), gold[f"{method}_state"].view(np.int64))


def test_oracle_force_and_pow_reproduce_the_fixture(oracle_lib, gold):
    import oracle
    acc = np.stack([oracle.acceleration(QOM, VUN, gold["uu"], gold["bb"], v)
                    for v in gold["accel_vec"]])
    assert np.array_equal(acc.view(np.int64), gold["accel"].view(np.int64))
    pw = np.array([oracle.det_pow(a, b) for a, b in zip(gold["pow_x"], gold["pow_y"])])
    assert np.array_equal(pw.view(np.int64), gold["pow"].view(np.int64))
