"""Drop-in for save_data.py: snapshots with the reference's datasets and unit conversions.

Writes HDF5 when h5py is importable, otherwise an .npz file with the same dataset names.
"""
import os

import numpy as np

from configure_me import BOX_SIZE, H0, N_CELLS, N_PARTS, SAVE_DENSITY

try:
    import h5py
except ImportError:  # pragma: no cover - depends on the environment
    h5py = None

DATA_DIR = "Data"


def _units(a):
    pos = 7.8 * (BOX_SIZE / (N_CELLS / 128)) / 10 ** 3       # cells -> Mpc
    vel = 0.781 * BOX_SIZE * H0 / (a * N_CELLS / 128)         # code units -> km/s
    return pos, vel


def _path(step):
    return os.path.join(DATA_DIR, f"data.{step}." + ("hdf5" if h5py is not None else "npz"))


def save_file(rho, positions, velocities, step, a):
    print("Writing to disk:", _path(step))
    os.makedirs(DATA_DIR, exist_ok=True)
    up, uv = _units(a)
    d = {"x1": positions[0] * up, "x2": positions[1] * up, "x3": positions[2] * up,
         "vx1": velocities[0] * uv, "vx2": velocities[1] * uv, "vx3": velocities[2] * uv, "a": np.float64(a)}
    if SAVE_DENSITY and rho is not None:
        d["density"] = rho
    if h5py is not None:
        with h5py.File(_path(step), "w") as hf:
            for k, v in d.items():
                hf.create_dataset(k, data=v)
    else:
        np.savez(_path(step), **d)


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
