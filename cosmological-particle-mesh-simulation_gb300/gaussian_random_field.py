"""Drop-in for gaussian_random_field.py (host numpy, runs once per simulation)."""
from pmgpu import ics
from pmgpu.dropin import config


def gaussian_random_field():
    """Real N_PARTS^3 float32 density field at A_INIT."""
    return ics.gaussian_random_field(config())
