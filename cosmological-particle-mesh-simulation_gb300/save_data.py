"""Drop-in for save_data.py: snapshots with the reference's datasets and unit conversions.

Writes HDF5 when h5py is importable, otherwise an .npz file with the same dataset names
(pmgpu/snapshot.py; its SnapshotWriter writes the same files in the background).
"""
import numpy as np

from configure_me import BOX_SIZE, H0, N_CELLS, N_PARTS, SAVE_DENSITY
from pmgpu.snapshot import h5py, host_snapshot, snapshot_path, units, write_file

DATA_DIR = "Data"


def _units(a):
    return units(a, BOX_SIZE, N_CELLS, H0)


def _path(step):
    return snapshot_path(DATA_DIR, step)


def save_file(rho, positions, velocities, step, a):
    print("Writing to disk:", _path(step))
    d = host_snapshot(positions, velocities, a, BOX_SIZE, N_CELLS, H0,
                      rho if SAVE_DENSITY and rho is not None else None)
    write_file(_path(step), d)


def from_file(step):
    n3 = N_PARTS ** 3
    positions = np.zeros((3, n3), dtype=np.float32)
    velocities = np.zeros((3, n3), dtype=np.float32)
    if h5py is not None:
        hf = h5py.File(_path(step), "r")
        get = lambda k: np.array(hf.get(k))  # noqa: E731
    else:
        hf = np.load(_path(step))
        get = lambda k: np.array(hf[k])  # noqa: E731
    a = np.float32(get("a"))
    up, uv = _units(a)
    for i, k in enumerate(("x1", "x2", "x3")):
        positions[i] = get(k) / up
    for i, k in enumerate(("vx1", "vx2", "vx3")):
        velocities[i] = get(k) / uv
    return positions, velocities, a
