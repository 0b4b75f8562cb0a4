"""Drop-in for integrate.py: force gather, kick and drift on the GPU."""
from pmgpu import dropin


def advance_time(density, positions, velocities, fgrid, a, da):
    """potential -> f(a + da) -> integrate; positions and velocities updated in place."""
    return dropin.advance_time(density, positions, velocities, fgrid, a, da)


def integrate(positions, velocities, a_val, f_a1, da, potentials):
    """CIC-interpolated central-difference force, v += da f g, x = (x + da v f / (a + da)^2) mod N."""
    return dropin.integrate(positions, velocities, a_val, f_a1, da, potentials)
