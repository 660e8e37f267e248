"""Mie-series bistatic RCS of a perfectly conducting sphere (test utility).

Written from the published series (Bohren & Huffman, "Absorption and
Scattering of Light by Small Particles", 1983, sections 4.4 and 4.8): for a
perfect conductor the coefficients reduce to a_n = psi_n'(x)/xi_n'(x) and
b_n = psi_n(x)/xi_n(x), with psi_n(x) = x j_n(x) and xi_n(x) = x h_n(x).
For an x-polarised wave travelling +z, the bistatic RCS in the phi = 0
plane is (lambda^2/pi)|S2(theta)|^2 and in the phi = 90 deg plane
(lambda^2/pi)|S1(theta)|^2.
"""
import numpy as np
from scipy.special import spherical_jn, spherical_yn


def _pi_tau(mu, nmax):
    pi = np.zeros((nmax + 1,) + mu.shape)
    tau = np.zeros_like(pi)
    pi[1] = 1.0
    tau[1] = mu
    for n in range(2, nmax + 1):
        pi[n] = ((2 * n - 1) / (n - 1)) * mu * pi[n - 1] - (n / (n - 1)) * pi[n - 2]
        tau[n] = n * mu * pi[n] - (n + 1) * pi[n - 1]
    return pi, tau


def pec_sphere_rcs(radius, freq, theta, c0=299792458.0):
    """Returns (sigma_E_plane, sigma_H_plane) in m^2 at the scattering angles theta."""
    k = 2 * np.pi * freq / c0
    x = k * radius
    nmax = int(np.ceil(x + 4 * x ** (1 / 3) + 2)) + 4
    n = np.arange(1, nmax + 1)
    jn = spherical_jn(n, x)
    jnp = spherical_jn(n, x, derivative=True)
    yn = spherical_yn(n, x)
    ynp = spherical_yn(n, x, derivative=True)
    hn = jn + 1j * yn
    hnp = jnp + 1j * ynp
    psi = x * jn
    dpsi = jn + x * jnp
    xi = x * hn
    dxi = hn + x * hnp
    a = dpsi / dxi
    b = psi / xi
    mu = np.cos(np.asarray(theta, dtype=float))
    pi, tau = _pi_tau(mu, nmax)
    s1 = np.zeros(mu.shape, dtype=complex)
    s2 = np.zeros(mu.shape, dtype=complex)
    for i, nn in enumerate(n):
        f = (2 * nn + 1) / (nn * (nn + 1))
        s1 += f * (a[i] * pi[nn] + b[i] * tau[nn])
        s2 += f * (a[i] * tau[nn] + b[i] * pi[nn])
    lam = 2 * np.pi / k
    return lam ** 2 / np.pi * np.abs(s2) ** 2, lam ** 2 / np.pi * np.abs(s1) ** 2
