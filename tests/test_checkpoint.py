"""Checkpoint files (host): round trip of every array, bit for bit."""
import numpy as np
import pytest

from particles_gb300 import checkpoint


def test_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    arrs = dict(state=rng.normal(size=(5, 4, 8)), cnt=rng.integers(0, 99, (5, 3)),
                carry=rng.integers(0, 255, 5 * 128).astype(np.uint8),
                status=np.array([0, 1, 2, -5, 1], np.int32), params=rng.normal(size=17),
                time=np.linspace(0, 1, 4))
    p = checkpoint.save(tmp_path / "run", t_reached=0.375, method="dop853", precision="fp32",
                        extra={"window": 3}, **arrs)
    out = checkpoint.load(p)
    for k, v in arrs.items():
        assert out[k].dtype == v.dtype and np.array_equal(out[k], v), k
    assert out["t_reached"] == 0.375 and out["meta"]["method"] == "dop853"
    assert out["meta"]["window"] == 3


def test_inconsistent_file_is_refused(tmp_path):
    p = tmp_path / "bad.npz"
    np.savez(p, state=np.zeros((3, 2, 8)), cnt=np.zeros((2, 3)), carry=np.zeros(384, np.uint8),
             status=np.zeros(3, np.int32), params=np.zeros(17), time=np.zeros(2),
             t_reached=np.float64(0), meta=np.array(repr({"format": 1})))
    with pytest.raises(ValueError):
        checkpoint.load(p)
