"""Seeded synthetic surfaces for the benchmark configurations.

The reference measures on no public dataset; these generators are the whole
input suite.  All use ``numpy.random.default_rng(seed)`` (PCG64), nodes at
xi_j = 2 pi j / N and an Eulerian start x = xi, which is what the reference's
derivative code assumes (x - 2 pi j / N periodic, Derivatives.cuh:281-287).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

TWO_PI = 2.0 * np.pi


def nodes(n: int) -> np.ndarray:
    return TWO_PI * np.arange(n) / n


@dataclass
class Surface:
    x: np.ndarray
    y: np.ndarray
    phi: np.ndarray
    physics: str = "water"      # "water" | "helium"
    depth: float = 1.0          # helium film thickness h0
    A3: float | None = None     # helium van der Waals constant (None: h0^4 / 3)
    gravity: float = 1.0

    @property
    def n(self) -> int:
        return self.x.size


def linear_wave(n: int, amp: float, k: int = 1, g: float = 1.0) -> Surface:
    """y = amp cos(k xi), phi = amp sqrt(g/k) sin(k xi): a right-running linear
    deep-water wave (omega^2 = g k).  amp=0.05, n=128 is the CPU-runnable case;
    amp=0.3, n=8192 is the large steep case."""
    xi = nodes(n)
    return Surface(xi.copy(), amp * np.cos(k * xi), amp * np.sqrt(g / k) * np.sin(k * xi), gravity=g)


def random_modes(n: int, seed: int = 2, modes: int = 8, g: float = 1.0) -> Surface:
    """Sum of `modes` linear waves: a_m ~ U(0, 0.02)/m, theta_m ~ U(0, 2 pi)
    (all amplitudes drawn first, then all phases), y = sum a_m cos(m xi + theta_m),
    phi = sum a_m sqrt(g/m) sin(m xi + theta_m).  Seed 2 at n=1024 is the
    mixed-precision single-surface case; at n=4096 it is the headline case."""
    rng = np.random.default_rng(seed)
    m = np.arange(1, modes + 1)
    a = rng.uniform(0.0, 0.02, modes) / m
    theta = rng.uniform(0.0, TWO_PI, modes)
    xi = nodes(n)
    arg = m[:, None] * xi[None, :] + theta[:, None]
    y = (a[:, None] * np.cos(arg)).sum(0)
    phi = (a[:, None] * np.sqrt(g / m)[:, None] * np.sin(arg)).sum(0)
    return Surface(xi.copy(), y, phi, gravity=g)


def helium_batch(count: int = 512, seed: int = 3, n_min: int = 128, n_max: int = 2048) -> list[Surface]:
    """Uneven batch of helium films: per surface N = 32 * U{n_min/32 .. n_max/32},
    h0 ~ U(5, 20), A3 ~ U(0.5, 2) * 1e3, amp ~ U(0.01, 0.1) * h0, k ~ U{1..4};
    y = amp cos(k xi), phi = 0 (drawn in that order per surface)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        n = 32 * int(rng.integers(n_min // 32, n_max // 32 + 1))
        h0 = float(rng.uniform(5.0, 20.0))
        A3 = float(rng.uniform(0.5, 2.0) * 1e3)
        amp = float(rng.uniform(0.01, 0.1) * h0)
        k = int(rng.integers(1, 5))
        xi = nodes(n)
        out.append(Surface(xi.copy(), amp * np.cos(k * xi), np.zeros(n), physics="helium", depth=h0, A3=A3))
    return out


def fourier_surface(n: int, coeffs: np.ndarray) -> np.ndarray:
    """y(xi) = sum_m c_m cos(m xi) + s_m sin(m xi), coeffs = [c_1..c_M, s_1..s_M]."""
    M = coeffs.size // 2
    m = np.arange(1, M + 1)
    xi = nodes(n)
    return (coeffs[:M, None] * np.cos(m[:, None] * xi) + coeffs[M:, None] * np.sin(m[:, None] * xi)).sum(0)


def fit_coefficients(seed: int, modes: int = 32) -> np.ndarray:
    """(c_m, s_m) ~ N(0, 0.01/m): 2*modes coefficients (cosines then sines)."""
    rng = np.random.default_rng(seed)
    m = np.arange(1, modes + 1)
    c = rng.normal(0.0, 0.01 / m)
    s = rng.normal(0.0, 0.01 / m)
    return np.concatenate([c, s])


def helium_fit(n: int = 512, seed: int = 4, target_seed: int = 40, h0: float = 10.0, A3: float = 1e3):
    """Adjoint-fit case: initial film y from 64 seeded Fourier coefficients, phi = 0,
    and a target surface of the same form from `target_seed`."""
    c0 = fit_coefficients(seed)
    ct = fit_coefficients(target_seed)
    xi = nodes(n)
    s = Surface(xi.copy(), fourier_surface(n, c0), np.zeros(n), physics="helium", depth=h0, A3=A3)
    return s, c0, fourier_surface(n, ct)
