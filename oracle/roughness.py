"""Gerekos et al. 2023 rough-facet response in float64 (oracle).

Restates soundersim ``roughness.py``: the coherent mean attenuation, the
incoherent variance series D_Phi (full Gaussian ACF through the Faddeeva
function; area-only Gaussian and exponential ACFs), the series length rule
and the speckle phasors.
"""

import functools

import numpy as np
from scipy.special import gammaln

INV_SQRT_PI = 1.0 / np.sqrt(np.pi)
SQRT_PI = np.sqrt(np.pi)


@functools.lru_cache(maxsize=None)
def weideman_coeffs(n=32):
    """Weideman (1994) rational-approximation constants (L, a) for w(z)
    (roughness.py:56-64): FFT of exp(-t^2)(L^2 + t^2) on the tangent grid
    t = L tan(pi k / 2M), M = 2n."""
    m = 2 * n
    big_l = np.sqrt(n / np.sqrt(2.0))
    k = np.arange(-m + 1, m)
    t = big_l * np.tan(np.pi * k / (2 * m))
    f = np.concatenate([[0.0], np.exp(-t * t) * (big_l * big_l + t * t)])
    a = np.real(np.fft.fft(np.fft.fftshift(f))) / (2 * m)
    return big_l, a[1:n + 1][::-1].copy()


def faddeeva(z, n=32):
    """w(z) = exp(-z^2) erfc(-iz), Im z >= 0 (roughness.py:67-80):
    w = 2 P(Z) / (L - iz)^2 + 1/(sqrt(pi) (L - iz)), Z = (L + iz)/(L - iz)."""
    big_l, a = weideman_coeffs(n)
    iz = 1j * np.asarray(z, np.complex128)
    den = big_l - iz
    zz = (big_l + iz) / den
    poly = np.polyval(a, zz)
    return 2.0 * poly / (den * den) + INV_SQRT_PI / den


def mean_attenuation(sigma, big_k):
    """exp(-sigma^2 K^2 / 2) (roughness.py:83-89)."""
    sk = sigma * big_k
    return np.exp(-0.5 * (sk * sk))


def f_factor(m, a0, edge, l):
    """One Eq 22-24 factor via the scaled Faddeeva combination
    (roughness.py:92-107): x = a0 l / (2 sqrt m), y = edge sqrt(m) / l."""
    sq = np.sqrt(m)
    x = a0 * l / (2.0 * sq)
    y = edge * sq / l
    ex2 = np.exp(-x * x)
    ey2 = np.exp(-y * y)
    wz = faddeeva(x + 1j * y)
    wx = faddeeva(x + 0j)
    rot = np.exp(1j * (a0 * edge))
    t1 = -y * ex2 - ey2 * np.real(1j * (x + 1j * y) * rot * wz)
    t2 = x * np.imag(wx)
    return 1.0 - ey2 * np.cos(edge * a0) + SQRT_PI * (t1 - t2)


def acf_spectrum(m, kb, l, acf="gaussian"):
    """W_m(k_B) of rho^m (roughness.py:113-124)."""
    if acf == "gaussian":
        return np.pi * (l * l) / m * np.exp(-(kb * kb) * (l * l) / (4.0 * m))
    if acf == "exponential":
        q = (l / m) ** 2
        return 2.0 * np.pi * q * (1.0 + (kb * kb) * q) ** -1.5
    raise ValueError(f"unknown roughness acf {acf!r}")


def d_phi(sigma, l, big_k, a0, b0, lx, ly, *, n_terms, area_only=False,
          acf="gaussian"):
    """Incoherent variance D_Phi (Eq 21) summed over m = 1..n_terms in order
    (roughness.py:127-186), Poisson weight in log space, clamped >= 0.
    ``sigma``/``l`` may be scalars or per-facet arrays."""
    if acf not in ("gaussian", "exponential"):
        raise ValueError(f"unknown roughness acf {acf!r}")
    if acf == "exponential" and not area_only:
        raise ValueError("acf='exponential' needs the area-only D_Phi")
    x = (sigma * big_k) ** 2
    x = np.asarray(x, np.float64)
    with np.errstate(divide="ignore"):
        logx = np.where(x > 0, np.log(np.where(x > 0, x, 1.0)), -np.inf)
    l = np.asarray(l, np.float64)
    acc = np.zeros(np.broadcast_shapes(x.shape, np.shape(a0), np.shape(b0),
                                       np.shape(lx), np.shape(ly), l.shape))
    kb2 = a0 * a0 + b0 * b0
    for m in range(1, n_terms + 1):
        mf = float(m)
        with np.errstate(invalid="ignore"):
            logp = mf * logx - gammaln(mf + 1.0) - x
        if area_only and acf == "exponential":
            term = np.exp(logp) * acf_spectrum(mf, np.sqrt(kb2), l,
                                               "exponential") * lx * ly
        elif area_only:
            term = (np.exp(logp - kb2 * (l * l) / (4.0 * mf))
                    * (np.pi * (l * l) / mf) * lx * ly)
        else:
            term = (np.exp(logp) * ((l * l) * (l * l) / (mf * mf))
                    * f_factor(mf, a0, lx, l) * f_factor(mf, b0, ly, l))
        acc = acc + term
    return np.maximum(acc, 0.0)


def n_terms_for(x_max):
    """Series length ceil(x + 6 sqrt(x) + 5) clipped to [10, 300]
    (roughness.py:189-196)."""
    x = float(x_max)
    return int(np.clip(np.ceil(x + 6.0 * np.sqrt(x) + 5.0), 10, 300))


def speckle_phasors(n, seed):
    """Unit-variance complex Gaussian phasors (roughness.py:199-204)."""
    rng = np.random.default_rng(seed)
    ph = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    return (ph / np.sqrt(2.0)).astype(np.complex64)
