"""Driver with the structure of the reference's pmesh.py, on the GPU engine.

RESIDENT = True (configure_me) keeps the simulation in HBM for the whole run (the batch
engine: CUDA graphs, fused kernels); RESIDENT = False runs the reference's loop body
(density -> advance_time) through the drop-in functions on host arrays.
"""
from time import time

from configure_me import (A_END, A_INIT, BOX_SIZE, H0, N_CELLS, N_PARTS, N_SAVE_FILES, OMEGA_M0,
                          PRINT_STATUS, RESTART, RESTART_FROM_N, SAVE_DATA, SAVE_DENSITY, STEPS)
import configure_me
from density import density
from fourier_utils import fourier_grid
from gaussian_random_field import gaussian_random_field
from integrate import advance_time
from save_data import from_file, save_file
from zeldovich import zeldovich


def simulator():
    print(f"Starting the simulation for {N_PARTS}^3 particles with {N_CELLS}^3 grid cells")
    particle_mass = 1.32 * 10 ** 5 * (OMEGA_M0 * H0 ** 2) * (BOX_SIZE / (N_PARTS / 128)) ** 3
    print("Particle mass in solar mass for this configuration: {:.3E}".format(particle_mass))
    dens_contrast = (N_CELLS / N_PARTS) ** 3
    print("Particle mass in code units: {:.3e}".format(dens_contrast))
    da = (A_END - A_INIT) / STEPS
    da_save = (A_END - A_INIT) / N_SAVE_FILES
    a_current = A_INIT
    n_file = 0
    if RESTART:
        n_file = RESTART_FROM_N
        positions, velocities, a_current = from_file(n_file)
    else:
        rho = gaussian_random_field()
        positions, velocities = zeldovich(rho)
        if SAVE_DATA:
            save_file(rho, positions, velocities, 0, a_current)
            n_file += 1
    if getattr(configure_me, "RESIDENT", False):
        return _resident(positions, velocities, a_current, da, da_save, n_file)
    ksq_inverse = fourier_grid()
    print("Starting the integrations...")
    while a_current < A_END - da:
        start_time = time()
        rho = density(positions, dens_contrast)
        positions, velocities = advance_time(rho, positions, velocities, ksq_inverse, a_current, da)
        a_current += da
        if a_current >= A_INIT + n_file * da_save:
            if SAVE_DATA:
                save_file(rho, positions, velocities, n_file, a_current)
            n_file += 1
        if PRINT_STATUS:
            print_status(a_current, start_time)
    return positions, velocities


def _resident(positions, velocities, a_current, da, da_save, n_file):
    from pmgpu.batch import Batch
    from pmgpu.config import step_count
    from pmgpu.dropin import config
    cfg = config()
    cfg.a_init = float(a_current)
    cfg.steps = max(1, int(round((A_END - a_current) / da)))
    nsteps = step_count(cfg.a_init, cfg.a_end, cfg.steps)
    b = Batch()
    sid = b.add(cfg, positions, velocities)
    writer = None
    if SAVE_DATA:  # snapshots are copied out and written while the next steps run
        from pmgpu.snapshot import SnapshotWriter
        from save_data import DATA_DIR
        writer = SnapshotWriter(BOX_SIZE, N_CELLS, H0, directory=DATA_DIR)
    print("Starting the integrations (resident on the GPU)...")
    while True:
        a, done = b.state(sid)
        if done >= nsteps:
            break
        start_time = time()
        # run up to the next snapshot boundary in one call
        target = A_INIT + n_file * da_save
        k = min(max(1, int((target - a) / da)) if SAVE_DATA else nsteps, nsteps - done)
        rho = None
        if SAVE_DATA and SAVE_DENSITY:
            # pmesh.py:60-67 saves the density the interval's last step was computed from
            if k > 1:
                b.step(k - 1)
            rho = b.density(sid)
            b.step(1)
        else:
            b.step(k)
        a, done = b.state(sid)
        if SAVE_DATA and a >= target:
            pos_d, vel_d, _, _ = b.get(sid, device=True)
            writer.submit(n_file, pos_d, vel_d, a, rho=rho)
            n_file += 1
        if PRINT_STATUS:
            print_status(a, start_time)
    b.check_device()
    positions, velocities, _, _ = b.get(sid)
    if writer is not None:
        writer.close()
    return positions, velocities


def print_status(a_current, start_time):
    percentile = 100 * (a_current - A_INIT) / (A_END - A_INIT)
    print("%.5f" % percentile, "%", " Save step time: --- %.5f seconds ---" % (time() - start_time))


if __name__ == "__main__":
    start_time = time()
    simulator()
    print("Finished in")
    print("--- %.2f seconds ---" % (time() - start_time))
