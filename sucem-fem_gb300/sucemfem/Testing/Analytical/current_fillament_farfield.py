"""Far field of a straight current filament of length L with a uniform
current I0 along z (sucemfem/Testing/Analytical/current_fillament_farfield.py:
24-43): the radiation integral of the line source gives

    E_theta = j omega mu I0 L exp(-j beta r) / (4 pi r) * sin(theta)
              * sin(beta L cos(theta) / 2) / (beta L cos(theta) / 2),

with beta = omega / c0 and mu = mu0 (the last factor is 1 at theta = pi/2
and tends to 1 where cos(theta) -> 0)."""
import numpy as np

from ...Consts import c0, mu0


def eval_E_theta(freq, L_val, I_val, theta_val, r_val=1):
    """E_theta (complex) at distance r_val and polar angle theta_val."""
    omega = 2 * np.pi * freq
    beta = omega / c0
    u = beta * L_val / 2 * np.cos(theta_val)
    factor = np.sinc(u / np.pi)          # sin(u) / u, 1 at u = 0
    return complex(1j * omega * mu0 * I_val * L_val * np.exp(-1j * beta * r_val)
                   / (4 * np.pi * r_val) * np.sin(theta_val) * factor)
