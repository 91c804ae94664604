"""The batch-file format and the loader of the 4f training data
(toolbox.py:698-739) on the CPU: the reference's sampling (one random file,
batch_size random samples in index order) and its two datasets."""
import numpy as np
import pytest


def test_loader_reads_random_sorted_batches(tmp_path):
    torch = pytest.importorskip("torch")
    from xlumina_gb300 import datasets
    rng = np.random.default_rng(0)
    files = {}
    for k in range(2):
        inp = rng.uniform(0, 1, (7, 8, 8)).astype(np.float32)
        inp[:, 0, 0] = np.arange(7) + 100 * k          # sample id
        tgt = inp * 2
        p = datasets.write_batch_file(str(tmp_path / f"batch_{k}.hdf5"), inp, tgt)
        files[k] = (inp, tgt)
        assert p.endswith(".hdf5") or p.endswith(".npz")
    loader = datasets.MultiHDF5DataLoader(str(tmp_path), batch_size=3, device="cpu", seed=5)
    seen = set()
    for _ in range(6):
        a, b = next(loader)
        assert a.shape == (3, 8, 8) and b.shape == (3, 8, 8)
        ids = a[:, 0, 0].numpy()
        k = int(ids[0] // 100)
        idx = (ids - 100 * k).astype(int)
        assert list(idx) == sorted(idx) and len(set(idx)) == 3
        assert np.array_equal(a.numpy(), files[k][0][idx]) and np.array_equal(b.numpy(), files[k][1][idx])
        seen.add(k)
    loader.close()
    assert seen == {0, 1}


def test_empty_directory_raises(tmp_path):
    pytest.importorskip("torch")
    from xlumina_gb300 import datasets
    with pytest.raises(ValueError):
        datasets.MultiHDF5DataLoader(str(tmp_path), batch_size=2, device="cpu")
