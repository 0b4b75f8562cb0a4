"""Drop-in for cosmology.py: background functions (host, scalar)."""
import numpy as np

from configure_me import A_INIT, H0, OMEGA_K0, OMEGA_LAMBDA0, OMEGA_M0


def H(a, h0, cosmology):
    """Hubble rate for cosmology = [Omega_m, Omega_L, Omega_k]."""
    om, ol, ok = cosmology
    return np.sqrt(h0 ** 2 * (om / a ** 3 + ok / a ** 2 + ol))


def f(a, cosmology):
    """1 / (a' / H0): the leapfrog coefficient."""
    om, ol, ok = cosmology
    return 1 / np.sqrt((om + ok * a + ol * a ** 3) / a)


def Dt(a, cosmology):
    """Linear growth factor (fitting formula)."""
    om, ol, ok = cosmology
    return 5 / 2 / om / (om ** (4 / 7) - ol + (1 + om / 2) * (1 + ol / 70)) * a


class cosmo:
    def __init__(self):
        c = [OMEGA_M0, OMEGA_LAMBDA0, OMEGA_K0]
        self.Dt = Dt(A_INIT, c)
        self.H01 = H(A_INIT, H0, c)
        self.f0 = f(A_INIT, c)
