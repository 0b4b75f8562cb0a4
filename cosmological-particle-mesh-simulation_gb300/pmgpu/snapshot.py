"""Snapshots in the layout of src/save_data.py:7-32 (datasets x1..x3, vx1..vx3, a and,
optionally, density; positions in Mpc and velocities in km/s), written while the
simulation keeps running.

SnapshotWriter.submit() takes device tensors of a state that the caller no longer
modifies (Batch.get(..., device=True) returns fresh ones).  On a copy stream it waits for
the caller's stream, applies the unit conversions (float32 products, as numpy computes
them for float32 arrays and Python floats), copies into pinned host memory, and hands the
file write to a worker thread; the caller's stream is free to run the next steps at once.
HDF5 when h5py is importable, otherwise .npz with the same dataset names.
"""
from __future__ import annotations

import concurrent.futures as cf
import os

import numpy as np

try:
    import h5py
except ImportError:  # pragma: no cover - depends on the environment
    h5py = None


def units(a: float, box_size: float, n_cells: int, h0: float):
    """save_data.py:10-11: cells -> Mpc, code velocity -> km/s."""
    pos = 7.8 * (box_size / (n_cells / 128)) / 10 ** 3
    vel = 0.781 * box_size * h0 / (a * n_cells / 128)
    return pos, vel


def snapshot_path(directory: str, step: int) -> str:
    return os.path.join(directory, f"data.{step}." + ("hdf5" if h5py is not None else "npz"))


def write_file(path: str, data: dict):
    os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
    if h5py is not None:
        with h5py.File(path, "w") as hf:
            for k, v in data.items():
                hf.create_dataset(k, data=v)
    else:
        np.savez(path, **data)


def read_file(path: str) -> dict:
    if path.endswith(".hdf5"):
        with h5py.File(path, "r") as hf:
            return {k: np.array(hf.get(k)) for k in hf.keys()}
    with np.load(path) as f:
        return {k: np.array(f[k]) for k in f.files}


def host_snapshot(positions, velocities, a, box_size, n_cells, h0, rho=None) -> dict:
    """The datasets of one snapshot from host arrays (save_data.py:19-27)."""
    up, uv = units(a, box_size, n_cells, h0)
    d = {"x1": positions[0] * up, "x2": positions[1] * up, "x3": positions[2] * up,
         "vx1": velocities[0] * uv, "vx2": velocities[1] * uv, "vx3": velocities[2] * uv}
    if rho is not None:
        d["density"] = rho
    d["a"] = np.float64(a)
    return d


class SnapshotWriter:
    """Writes snapshots in the background: device-to-host copies on their own stream,
    files from worker threads.  close() waits for everything submitted."""

    def __init__(self, box_size: float, n_cells: int, h0: float, directory: str = "Data", workers: int = 2,
                 device: int = 0):
        import torch
        self.box, self.n, self.h0 = float(box_size), int(n_cells), float(h0)
        self.dir = directory
        self.device = device
        self.copy_stream = torch.cuda.Stream(device=device)
        self.pool = cf.ThreadPoolExecutor(max_workers=workers)
        self.futures = []

    def submit(self, step: int, positions, velocities, a: float, rho=None) -> str:
        """Queue snapshot `step` of (3, Np) device tensors (and the optional density grid)."""
        import torch
        path = snapshot_path(self.dir, step)
        up, uv = units(a, self.box, self.n, self.h0)
        ready = torch.cuda.Event()
        ready.record(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(self.copy_stream):
            self.copy_stream.wait_event(ready)
            conv = [positions[i] * up for i in range(3)] + [velocities[i] * uv for i in range(3)]
            if rho is not None:
                conv.append(rho)
            host = []
            for t in conv:
                h = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
                h.copy_(t, non_blocking=True)
                host.append(h)
            for t in (positions, velocities) + ((rho,) if rho is not None else ()):
                t.record_stream(self.copy_stream)  # keep the sources alive until copied
            done = torch.cuda.Event()
            done.record(self.copy_stream)
        self.futures.append(self.pool.submit(self._write, path, host, done, float(a)))
        return path

    @staticmethod
    def _write(path, host, done, a):
        done.synchronize()
        names = ("x1", "x2", "x3", "vx1", "vx2", "vx3", "density")
        d = {k: h.numpy() for k, h in zip(names, host)}
        d["a"] = np.float64(a)
        write_file(path, d)
        return path

    def wait(self):
        paths = [f.result() for f in self.futures]
        self.futures.clear()
        return paths

    def close(self):
        try:
            return self.wait()
        finally:
            self.pool.shutdown(wait=True)
