"""Training data of the 4f tables: the batch files, their loader and the
synthetic generator (toolbox.py:698-739, experiments/generate_synthetic_data.py).

A batch file holds two datasets, ``"Input fields"`` (masks) and ``"Target
fields"`` (target intensities), with the samples along the first axis.  Files
are HDF5 (``.hdf5``) when h5py is importable; without it the same two
datasets are stored as ``.npz``, and the loader reads either.

``MultiHDF5DataLoader`` keeps the reference's sampling (a random file, then
``batch_size`` random samples from it, in index order) and returns device
tensors; a background thread reads the next batch into pinned host memory
and its copy to the device runs on a side stream, so a training step does not
wait for the disk or the copy.
"""
from __future__ import annotations

import os
import queue
import random
import threading

import numpy as np
import torch

INPUTS = "Input fields"
TARGETS = "Target fields"

try:   # optional: HDF5 files need h5py
    import h5py  # type: ignore
except Exception:   # pragma: no cover - depends on the environment
    h5py = None


def write_batch_file(path, input_fields, target_fields):
    """Write one batch file (``.hdf5`` with h5py, else ``.npz``); returns the path written."""
    inputs = np.asarray(input_fields.cpu() if isinstance(input_fields, torch.Tensor) else input_fields)
    targets = np.asarray(target_fields.cpu() if isinstance(target_fields, torch.Tensor) else target_fields)
    root, ext = os.path.splitext(path)
    if ext == ".hdf5" and h5py is not None:
        with h5py.File(path, "w") as f:
            f.create_dataset(INPUTS, data=inputs)
            f.create_dataset(TARGETS, data=targets)
        return path
    path = root + ".npz"
    np.savez(path, **{INPUTS: inputs, TARGETS: targets})
    return path


def _count(path):
    if path.endswith(".hdf5"):
        with h5py.File(path, "r") as f:
            return f[INPUTS].shape[0]
    with np.load(path, mmap_mode="r") as f:
        return f[INPUTS].shape[0]


def _read(path, idx):
    if path.endswith(".hdf5"):
        with h5py.File(path, "r") as f:
            return f[INPUTS][idx], f[TARGETS][idx]
    with np.load(path) as f:
        return f[INPUTS][idx], f[TARGETS][idx]


class MultiHDF5DataLoader:
    """toolbox.py:698-739: endless random batches from the batch files of a
    directory, as device tensors (``device=None``: the current CUDA device,
    else e.g. ``"cpu"``)."""

    def __init__(self, directory, batch_size, device=None, prefetch=2, seed=None):
        self.directory = directory
        self.batch_size = int(batch_size)
        exts = (".hdf5", ".npz") if h5py is not None else (".npz",)
        self.files = sorted(f for f in os.listdir(directory) if f.endswith(exts))
        if not self.files:
            raise ValueError(f"No HDF5 files found in directory: {directory}")
        self.device = torch.device(device) if device is not None else (
            torch.device("cuda", torch.cuda.current_device()) if torch.cuda.is_available() else torch.device("cpu"))
        self._rng = random.Random(seed)
        self._q: "queue.Queue" = queue.Queue(maxsize=max(1, prefetch))
        self._stop = threading.Event()
        self._thread = threading.Thread(target=self._produce, daemon=True)
        self._thread.start()
        self._stream = torch.cuda.Stream(self.device) if self.device.type == "cuda" else None

    def _sample(self):
        path = os.path.join(self.directory, self._rng.choice(self.files))
        n = _count(path)
        idx = sorted(self._rng.sample(range(n), self.batch_size))
        return _read(path, idx)

    def _produce(self):
        pin = self.device.type == "cuda"
        while not self._stop.is_set():
            try:
                a, b = self._sample()
                ta, tb = torch.from_numpy(np.ascontiguousarray(a)), torch.from_numpy(np.ascontiguousarray(b))
                if pin:
                    ta, tb = ta.pin_memory(), tb.pin_memory()
                item = (ta, tb)
            except Exception as exc:   # hand the failure to the consumer
                item = exc
            while not self._stop.is_set():
                try:
                    self._q.put(item, timeout=0.1)
                    break
                except queue.Full:
                    continue

    def __iter__(self):
        return self

    def __next__(self):
        item = self._q.get()
        if isinstance(item, Exception):
            raise item
        a, b = item
        if self._stream is None:
            return a.to(self.device), b.to(self.device)
        cur = torch.cuda.current_stream(self.device)
        with torch.cuda.stream(self._stream):
            da = a.to(self.device, non_blocking=True)
            db = b.to(self.device, non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(self._stream)
        cur.wait_event(ev)
        da.record_stream(cur)
        db.record_stream(cur)
        return da, db

    def close(self):
        self._stop.set()
        self._thread.join(timeout=5)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------- synthetic 4f training data --
# experiments/generate_synthetic_data.py:26-105: input masks and the intensity
# a 2x-magnifying 4f system should give for them (the mask scaled by 2 on a
# plane wave of amplitude 0.5), drawn on the device.

def _grid(n=1024, x_total=1500.0):
    from .toolbox import space
    x, y = space(x_total, n)
    dev = torch.device("cuda") if torch.cuda.is_available() else torch.device("cpu")
    X, Y = torch.meshgrid(torch.tensor(x, device=dev), torch.tensor(y, device=dev), indexing="xy")
    return X, Y


def generate_synthetic_circles(X, Y, num_samples, rng, amplitude=0.5):
    from .optical_elements import circular_mask
    ins, outs = [], []
    for _ in range(num_samples):
        r1, r2 = rng.uniform(100, 1000), rng.uniform(100, 1000)
        ins.append(circular_mask(X, Y, (r1, r2)))
        outs.append((amplitude ** 2) * circular_mask(X, Y, (2 * r1, 2 * r2)))
    return torch.stack(ins), torch.stack(outs)


def generate_synthetic_squares(X, Y, num_samples, rng, amplitude=0.5):
    from .optical_elements import rectangular_mask
    ins, outs = [], []
    for _ in range(num_samples):
        w, h, a = rng.uniform(100, 1000), rng.uniform(100, 1000), rng.uniform(0, 2 * np.pi)
        ins.append(rectangular_mask(X, Y, (0, 0), w, h, a))
        outs.append((amplitude ** 2) * rectangular_mask(X, Y, (0, 0), 2 * w, 2 * h, -a))
    return torch.stack(ins), torch.stack(outs)


def generate_synthetic_annular(X, Y, num_samples, rng, amplitude=0.5):
    from .optical_elements import annular_aperture
    ins, outs = [], []
    for _ in range(num_samples):
        di, do = rng.uniform(100, 500), rng.uniform(550, 1000)
        ins.append(annular_aperture(di, do, X, Y))
        outs.append((amplitude ** 2) * annular_aperture(2 * di, 2 * do, X, Y))
    return torch.stack(ins), torch.stack(outs)


def generate_synthetic_files(directory, n_files=1, num_samples=30, n=1024, seed=0, ext=".hdf5"):
    """The generator's loop: per file, ``num_samples`` circles, squares and
    annuli (inputs and targets stacked in that order)."""
    os.makedirs(directory, exist_ok=True)
    X, Y = _grid(n)
    rng = np.random.default_rng(seed)
    paths = []
    for s in range(n_files):
        parts = [f(X, Y, num_samples, rng) for f in (generate_synthetic_circles, generate_synthetic_squares,
                                                      generate_synthetic_annular)]
        inputs = torch.cat([p[0] for p in parts])
        targets = torch.cat([p[1] for p in parts])
        paths.append(write_batch_file(os.path.join(directory, f"synthetic_data_{s}{ext}"),
                                      inputs.to(torch.float32), targets.to(torch.float32)))
    return paths
