"""The checkpoint container of the learned correction (sctl_gb300/checkpoint.py): round trips
every array and the metadata exactly, and refuses damaged, truncated or foreign files."""
import numpy as np
import pytest

from sctl_gb300 import checkpoint as C


def sample():
    rng = np.random.default_rng(0)
    return {"w": rng.standard_normal(1000).astype(np.float32), "mu": rng.standard_normal((3, 5)),
            "idx": np.arange(7, dtype=np.int64), "flag": np.array(True), "empty": np.zeros((0, 4))}


def test_round_trip(tmp_path):
    a = sample()
    path = str(tmp_path / "m.ckpt")
    C.save(path, a, {"n_models": 2, "note": "x"})
    b, meta = C.load(path)
    assert meta == {"n_models": 2, "note": "x"}
    assert set(a) == set(b)
    for k in a:
        assert a[k].dtype == b[k].dtype and a[k].shape == b[k].shape
        assert np.array_equal(a[k], b[k])


@pytest.mark.parametrize("where", [20, -40, -1])
def test_damage_is_detected(where):
    blob = bytearray(C.dumps(sample(), {"k": 1}))
    blob[where] ^= 0x10
    with pytest.raises(C.CheckpointError):
        C.loads(bytes(blob))


def test_truncated_and_foreign_files_are_refused():
    blob = C.dumps(sample())
    with pytest.raises(C.CheckpointError):
        C.loads(blob[:-5])
    with pytest.raises(C.CheckpointError):
        C.loads(b"NOTACKPT" + blob[8:])
    with pytest.raises(C.CheckpointError):
        C.loads(b"")


def test_unsupported_dtype_is_refused():
    with pytest.raises(C.CheckpointError):
        C.dumps({"s": np.array(["a", "b"])})


def test_standardizer_from_arrays_matches_fitted():
    import torch
    from sctl_gb300.learned import Standardizer
    x = torch.randn(500, 7, dtype=torch.float64)
    a = Standardizer(x)
    b = Standardizer.from_arrays(a.mu.clone(), a.sd.clone())
    assert torch.equal(a.fwd(x), b.fwd(x))
    y = torch.randn(10, 7)
    assert torch.equal(a.inv(y), b.inv(y))
