"""FH2Data builders: the input side of the split-operator propagator.

The reference drives its MEX entry with a MATLAB struct built by ``FH2main.m``
(grids ``:79-115``, Omega states ``:39-57``, options ``:149-155``, CRP fields
``:180-191``) and helpers ``InitWavePacket.m``, ``OmegaList.m`` and
``AssLegendreP.m``.  Several helpers it calls (``GaussLegendre2``,
``FH2PESJacobi``, ``H2VibRotWaveFunction``, ``EtaSq``, ``WoodsSaxon``) are not
part of the reference, so this module restates them from the underlying
mathematics:

* Gauss-Legendre nodes/weights (ascending nodes);
* fully normalised associated Legendre functions in MATLAB's
  ``legendre(l, x, 'norm')`` convention, i.e. sqrt((l+1/2)(l-m)!/(l+m)!)
  (1-x^2)^(m/2) d^m P_l/dx^m (the (-1)^m of the 'norm' definition cancels the
  Condon-Shortley phase), evaluated with the standard stable three-term
  recurrence;
* a London-Eyring-Polanyi-Sato (LEPS) surface for F + H2 in reactant Jacobi
  coordinates;
* a quadratic complex absorbing potential expressed through the reference's
  multiplicative mask mechanism (``dump1``/``dump2``, ``evolutionCUDAaux.cu:243-251``);
* the H2 vibrational ground state from a Fourier-grid Hamiltonian on the r grid;
* the incoming Gaussian of ``InitWavePacket.m:13-14`` times the H2 state times
  the normalised j=0 Legendre function (``InitWavePacket.m:35-40`` packing).

Array layout convention: every array is stored in the reference's
column-major memory order.  A MATLAB array of dims ``[n1, n2, n3]`` is a
C-contiguous numpy array of shape ``(n3, n2, n1)``; complex data is
``complex128`` (interleaved re/im, ``complex.h:27``).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence

import numpy as np

MASS_AU = 1.822888484929367e3          # FH2main.m:64
M_F = 18.998403
M_H = 1.007825

# LEPS parameters (Morse D [Eh], a [1/a0], re [a0], Sato Delta)
LEPS_FH = (0.2252, 1.1741, 1.7329, 0.167)
LEPS_HH = (0.1745, 1.0271, 1.4008, 0.106)
V_CAP = 1.0                              # repulsive wall cut-off [Eh]


# --------------------------------------------------------------------------
# quadrature and angular functions
# --------------------------------------------------------------------------

def gauss_legendre(n: int):
    """Gauss-Legendre nodes (ascending) and weights on [-1, 1]."""
    x, w = np.polynomial.legendre.leggauss(int(n))
    return np.ascontiguousarray(x), np.ascontiguousarray(w)


def normalized_associated_legendre(l_max: int, m: int, x) -> np.ndarray:
    """Columns l = m..l_max of the fully normalised associated Legendre functions.

    Returns shape ``(len(x), l_max - m + 1)``: the matrix ``AssLegendreP(m,
    l_max, x)`` of ``AssLegendreP.m:9-12`` (MATLAB ``legendre(l, x, 'norm')``
    row ``m+1``).  Normalisation: integral over [-1, 1] of N_l^m(x)^2 = 1.
    Recurrence: N_m^m = N_{m-1}^{m-1} sqrt((2m+1)/(2m)) sqrt(1-x^2),
    N_{m+1}^m = x sqrt(2m+3) N_m^m,
    N_l^m = a_l (x N_{l-1}^m - b_l N_{l-2}^m) with
    a_l = sqrt((4l^2-1)/(l^2-m^2)), b_l = sqrt(((l-1)^2-m^2)/(4(l-1)^2-1)).
    """
    x = np.asarray(x, dtype=np.float64)
    if l_max < m or m < 0:
        raise ValueError("need 0 <= m <= l_max")
    s = np.sqrt(np.maximum(0.0, 1.0 - x * x))
    pmm = np.full_like(x, math.sqrt(0.5))
    for k in range(1, m + 1):
        pmm = pmm * math.sqrt((2.0 * k + 1.0) / (2.0 * k)) * s
    out = np.empty((x.size, l_max - m + 1))
    out[:, 0] = pmm
    if l_max == m:
        return out
    p1 = x * math.sqrt(2.0 * m + 3.0) * pmm
    out[:, 1] = p1
    p0 = pmm
    for l in range(m + 2, l_max + 1):
        a = math.sqrt((4.0 * l * l - 1.0) / (l * l - m * m))
        b = math.sqrt(((l - 1.0) ** 2 - m * m) / (4.0 * (l - 1.0) ** 2 - 1.0))
        p2 = a * (x * p1 - b * p0)
        out[:, l - m] = p2
        p0, p1 = p1, p2
    return out


def omega_list(J: int, p: int, l_max: int, omega_cap: Optional[int] = None) -> List[int]:
    """Helicity list of ``OmegaList.m:1-16``; optional truncation at ``omega_cap``."""
    omega_max = min(J, l_max)
    if J == 0:
        return [0]
    omega_min = 0 if (J + p) % 2 == 0 else 1
    if omega_cap is not None:
        omega_max = min(omega_max, omega_cap)
    return list(range(omega_min, omega_max + 1))


# --------------------------------------------------------------------------
# potential energy surface
# --------------------------------------------------------------------------

def _leps_qj(d, D, a, re, delta):
    e1 = np.exp(-a * (d - re))
    e2 = e1 * e1
    c = D / (4.0 * (1.0 + delta))
    q = c * ((3.0 + delta) * e2 - (2.0 + 6.0 * delta) * e1)
    j = c * ((1.0 + 3.0 * delta) * e2 - (6.0 + 2.0 * delta) * e1)
    return q, j


def leps_fh2(R, r, cos_theta, v_cap: float = V_CAP):
    """LEPS energy of F + H2 at Jacobi (R, r, cos theta), capped at ``v_cap``.

    V = Q_1 + Q_2 + Q_3 - sqrt(((J_1-J_2)^2 + (J_2-J_3)^2 + (J_3-J_1)^2)/2) with
    Q = D/(4(1+d)) [(3+d) e^{-2a(x-re)} - (2+6d) e^{-a(x-re)}] and
    J = D/(4(1+d)) [(1+3d) e^{-2a(x-re)} - (6+2d) e^{-a(x-re)}].
    The F-H distances follow from the H2 centre of mass at the bond midpoint.
    """
    R = np.asarray(R, dtype=np.float64)
    r = np.asarray(r, dtype=np.float64)
    c = np.asarray(cos_theta, dtype=np.float64)
    half = 0.5 * r
    d1 = np.sqrt(np.maximum(R * R + half * half - R * r * c, 1e-12))
    d2 = np.sqrt(np.maximum(R * R + half * half + R * r * c, 1e-12))
    q1, j1 = _leps_qj(d1, *LEPS_FH)
    q2, j2 = _leps_qj(d2, *LEPS_FH)
    q3, j3 = _leps_qj(r, *LEPS_HH)
    v = q1 + q2 + q3 - np.sqrt(0.5 * ((j1 - j2) ** 2 + (j2 - j3) ** 2 + (j3 - j1) ** 2))
    return np.minimum(v, v_cap)


def morse_hh(r, v_cap: float = V_CAP):
    """Asymptotic H2 curve of the LEPS surface (singlet Morse), capped."""
    D, a, re, _ = LEPS_HH
    e1 = np.exp(-a * (np.asarray(r) - re))
    return np.minimum(D * (e1 * e1 - 2.0 * e1), v_cap)


# --------------------------------------------------------------------------
# grids, kinetic tables, initial state
# --------------------------------------------------------------------------

def fft_kinetic(n: int, dr: float, mass: float) -> np.ndarray:
    """k^2/2m in FFT order for a periodic box of length n*dr (``cudaMath.h:117-130``)."""
    if n % 2:
        raise ValueError("FFT grids must have an even number of points")
    i = np.arange(n)
    k = 2.0 * np.pi / (n * dr) * np.where(i <= n // 2, i, i - n)
    return k * k / (mass + mass)


def h2_ground_state(r: np.ndarray, dr: float, mass: float):
    """H2 v=0 on the r grid from a Fourier-grid Hamiltonian (same kinetic
    operator as the propagator).  Returns (energy, normalised real vector)."""
    n = r.size
    t = fft_kinetic(n, dr, mass)
    eye = np.eye(n)
    tmat = np.real(np.fft.ifft(t[:, None] * np.fft.fft(eye, axis=0), axis=0))
    tmat = 0.5 * (tmat + tmat.T)
    h = tmat + np.diag(morse_hh(r))
    e, v = np.linalg.eigh(h)
    chi = v[:, 0].copy()
    if chi[np.argmax(np.abs(chi))] < 0:
        chi = -chi
    chi /= math.sqrt(np.sum(chi * chi) * dr)
    return float(e[0]), chi


def woods_saxon(x, Cd: float, xd: float) -> np.ndarray:
    """Woods-Saxon absorbing mask 1 / (1 + exp(Cd (x - xd))) of the reference's
    front end (``FH2main.m:97-99,113-115``; the same function as
    ``cudaMath.h:159-162``), applied once per step as ``dump1``/``dump2``."""
    x = np.asarray(x, dtype=np.float64)
    # exp overflows to inf far beyond xd, where the mask is 0 anyway
    with np.errstate(over="ignore"):
        return 1.0 / (1.0 + np.exp(Cd * (x - xd)))


def cap_mask(x: np.ndarray, width: float, strength: float, dt: float) -> np.ndarray:
    """Multiplicative form exp(-strength (x-x0)^2 dt) of a quadratic absorbing
    potential -i strength (x-x0)^2 over the last ``width`` of the grid."""
    x0 = x[-1] - width
    d = np.where(x > x0, x - x0, 0.0)
    return np.exp(-strength * d * d * dt)


def eta_sq(energies_coll, mass: float, r0: float, delta: float, k0: float):
    """|a(E)|^2 for the incoming Gaussian (pi delta^2)^(-1/4) exp(-(R-R0)^2/(2 delta^2) - i k0 R):
    projection on energy-normalised incoming waves sqrt(mu/(2 pi k)) e^{-ikR},
    |a|^2 = (mu/k) (delta/sqrt(pi)) exp(-delta^2 (k-k0)^2)."""
    e = np.asarray(energies_coll, dtype=np.float64)
    k = np.sqrt(2.0 * mass * e)
    return mass / k * (delta / math.sqrt(math.pi)) * np.exp(-(delta ** 2) * (k - k0) ** 2)


def energy_window(eta_sq_values, rel: float = 1e-4) -> np.ndarray:
    """Energies the initial packet carries: |a(E)|^2 >= rel * max |a(E)|^2.

    P(E) = flux(E) / |a(E)|^2 is a probability only where the packet has weight;
    outside this window |a(E)|^2 falls to 1e-11 and below and P(E) divides
    rounding noise by it, so P(E) comparisons are made inside the window."""
    e = np.asarray(eta_sq_values, dtype=np.float64)
    return e >= rel * e.max()


def finite_difference_weights(n_points: int) -> np.ndarray:
    """First-derivative weights of the centred ``n_points`` stencil on a unit
    grid (Fornberg's recursion), offsets -(n-1)/2 .. (n-1)/2."""
    if n_points < 3 or n_points % 2 == 0:
        raise ValueError("n_gradient_points must be odd and >= 3")
    h = (n_points - 1) // 2
    xs = np.arange(-h, h + 1, dtype=np.float64)
    m = 1
    n = n_points - 1
    c = np.zeros((n + 1, m + 1))
    c1 = 1.0
    c4 = xs[0]
    c[0, 0] = 1.0
    for i in range(1, n + 1):
        mn = min(i, m)
        c2 = 1.0
        c5 = c4
        c4 = xs[i]
        for j in range(i):
            c3 = xs[i] - xs[j]
            c2 *= c3
            if j == i - 1:
                for k in range(mn, 0, -1):
                    c[i, k] = c1 * (k * c[i - 1, k - 1] - c5 * c[i - 1, k]) / c2
                c[i, 0] = -c1 * c5 * c[i - 1, 0] / c2
            for k in range(mn, 0, -1):
                c[j, k] = (c4 * c[j, k] - k * c[j, k - 1]) / c3
            c[j, 0] = c4 * c[j, 0] / c3
        c1 = c2
    return c[:, 1].copy()


# --------------------------------------------------------------------------
# configurations
# --------------------------------------------------------------------------

@dataclass
class FH2Config:
    """Physical and numerical parameters of one FH2Data build."""
    n1: int = 64
    r1_range: tuple = (0.5, 14.0)
    n2: int = 32
    r2_range: tuple = (0.5, 10.0)
    n_theta: int = 24
    l_max: int = 23
    J: int = 0
    parity: int = 0
    omega_cap: Optional[int] = None
    init_omega: int = 0
    dt: float = 10.0
    total_steps: int = 500
    # initial Gaussian in R
    R0: float = 9.0
    delta: float = 0.5
    e_coll: float = 0.05
    # absorbing potential: "cap" (quadratic CAP over the last cap_width of each grid) or
    # "woods_saxon" (the reference's own masks, FH2main.m:97-99,113-115: Cd, xd per coordinate)
    mask: str = "cap"
    cap_width: float = 2.0
    cap_strength: float = 0.01
    ws_r1: tuple = (4.0, 12.0)
    ws_r2: tuple = (4.0, 10.0)
    # flux / P(E)
    r_flux: float = 3.5
    n_gradient_points: int = 21
    n_energies: int = 400
    e_range: tuple = (0.01, 0.15)
    calculate_crp: int = 1
    precision: str = "fp64"
    steps_to_copy: int = 0
    name: str = "custom"


CONFIGS: Dict[str, FH2Config] = {
    # J=0 reference-scale case (64x32x24)
    "fh2_j0_64x32x24": FH2Config(name="fh2_j0_64x32x24"),
    # J=0 production grid 256x128x96
    "fh2_j0_256x128x96": FH2Config(n1=256, n2=128, n_theta=96, l_max=95, total_steps=20000,
                                   name="fh2_j0_256x128x96"),
    # Coriolis-coupled J=12, parity +, Omega=0..12 on the production grid
    "fh2_j12_256x128x96": FH2Config(n1=256, n2=128, n_theta=96, l_max=95, J=12, parity=0,
                                    total_steps=10000, name="fh2_j12_256x128x96"),
    # mixed-precision form of the production case
    "fh2_j0_256x128x96_mixed": FH2Config(n1=256, n2=128, n_theta=96, l_max=95, total_steps=20000,
                                         precision="mixed", name="fh2_j0_256x128x96_mixed"),
}


def batched_partial_waves(J_max: int = 40, omega_cap: int = 20, n1: int = 192, n2: int = 96,
                          n_theta: int = 80, l_max: int = 79, total_steps: int = 8000,
                          precision: str = "fp64") -> List[FH2Config]:
    """Configurations of the batched J=0..J_max partial-wave run (one per J).

    Each J takes the parity p = J mod 2, so that (J + p) mod 2 = 0 and its helicities start
    at Omega = 0 (``OmegaList.m:2-16``, ``CoriolisMatrix.C:52-61``): Omega = 0..min(J,
    omega_cap), 651 Omega blocks for J = 0..40 with omega_cap = 20."""
    out = []
    for J in range(J_max + 1):
        out.append(FH2Config(n1=n1, n2=n2, n_theta=n_theta, l_max=l_max, J=J, parity=J % 2,
                             omega_cap=omega_cap, total_steps=total_steps, precision=precision,
                             name=f"fh2_batched_J{J}"))
    return out


def _radial(n, lo, hi, mass):
    r = np.linspace(lo, hi, n)
    return {"n": np.int32(n), "left": float(r[0]), "dr": float(r[1] - r[0]), "mass": float(mass), "r": r}


def build_fh2data(cfg: FH2Config) -> dict:
    """Build the FH2Data struct (as nested dicts of numpy arrays) for ``cfg``.

    Field set and meaning follow the reference's MATLAB struct
    (``cudaOpenMPEvolution.C:27-70``, ``matlabStructures.C:17-153``).
    """
    mF, mH = M_F * MASS_AU, M_H * MASS_AU
    mu_R = mF * (2.0 * mH) / (mF + 2.0 * mH)          # FH2main.m:85-86
    mu_r = mH * mH / (mH + mH)                        # FH2main.m:108
    r1 = _radial(cfg.n1, *cfg.r1_range, mu_R)
    r2 = _radial(cfg.n2, *cfg.r2_range, mu_r)
    x, w = gauss_legendre(cfg.n_theta)
    theta = {"n": np.int32(cfg.n_theta), "m": np.int32(cfg.l_max), "x": x, "w": w,
             # (m+1) x n in MATLAB order: shape (n, m+1) here; parsed but unused on the path
             "associated_legendre": np.ascontiguousarray(
                 normalized_associated_legendre(cfg.l_max, 0, x))}

    Rg, rg, cg = np.meshgrid(r1["r"], r2["r"], x, indexing="ij")     # [n1, n2, nθ]
    pot = np.ascontiguousarray(leps_fh2(Rg, rg, cg).transpose(2, 1, 0))  # (nθ, n2, n1)

    omegas = omega_list(cfg.J, cfg.parity, cfg.l_max, cfg.omega_cap)
    n_om = len(omegas)
    n_cols = cfg.l_max - omegas[0] + 1
    P = np.zeros((n_om, n_cols, cfg.n_theta))        # MATLAB [nθ, n_cols, n_Ω]
    for b, om in enumerate(omegas):
        Pb = normalized_associated_legendre(cfg.l_max, om, x)   # (nθ, l_max-Ω+1)
        P[b, : Pb.shape[1], :] = Pb.T

    # initial wavepacket: Gaussian(R) x H2(v=0) x N_0^0(x)   (InitWavePacket.m:13-40)
    k0 = math.sqrt(2.0 * mu_R * cfg.e_coll)
    R = r1["r"]
    g = (1.0 / (math.pi * cfg.delta ** 2)) ** 0.25 * np.exp(
        -((R - cfg.R0) ** 2) / (2.0 * cfg.delta ** 2) - 1j * k0 * R)
    g /= math.sqrt(np.sum(np.abs(g) ** 2) * r1["dr"])
    e_h2, chi = h2_ground_state(r2["r"], r2["dr"], mu_r)
    ang = normalized_associated_legendre(0, 0, x)[:, 0]
    psi0 = ang[:, None, None] * chi[None, :, None] * g[None, None, :]   # (nθ, n2, n1)
    norm = np.sum(w[:, None, None] * np.abs(psi0) ** 2) * r1["dr"] * r2["dr"]
    psi0 = psi0 / math.sqrt(norm)
    wave_packets = np.zeros((n_om, cfg.n_theta, cfg.n2, cfg.n1), dtype=np.complex128)
    if cfg.init_omega in omegas:
        wave_packets[omegas.index(cfg.init_omega)] = psi0

    if cfg.mask == "woods_saxon":
        dump1 = {"dump": woods_saxon(r1["r"], *cfg.ws_r1)}
        dump2 = {"dump": woods_saxon(r2["r"], *cfg.ws_r2)}
    elif cfg.mask == "cap":
        dump1 = {"dump": cap_mask(r1["r"], cfg.cap_width, cfg.cap_strength, cfg.dt)}
        dump2 = {"dump": cap_mask(r2["r"], cfg.cap_width, cfg.cap_strength, cfg.dt)}
    else:
        raise ValueError(f"unknown mask kind {cfg.mask!r} (cap or woods_saxon)")

    n_ds = int(round((cfg.r_flux - r2["left"]) / r2["dr"]))
    e_coll = np.linspace(cfg.e_range[0], cfg.e_range[1], cfg.n_energies)
    crp = {
        "eDiatomic": e_h2,
        "n_dividing_surface": np.int32(n_ds),
        "n_gradient_points": np.int32(cfg.n_gradient_points),
        "n_energies": np.int32(cfg.n_energies),
        "energies": e_coll + e_h2,
        "eta_sq": eta_sq(e_coll, mu_R, cfg.R0, cfg.delta, k0),
        "CRP": np.zeros(cfg.n_energies),
        "calculate_CRP": np.int32(cfg.calculate_crp),
    }
    precision = {"fp64": 0, "mixed": 1}[cfg.precision]
    return {
        "r1": r1,
        "r2": r2,
        "theta": theta,
        "pot": pot,
        "psi": psi0,
        "time": {"total_steps": np.int32(cfg.total_steps), "time_step": float(cfg.dt),
                 "steps": np.int32(0)},
        "options": {"steps_to_copy_psi_from_device_to_host": np.int32(cfg.steps_to_copy),
                    "use_p2p_async": np.int32(0), "wave_to_matlab": None, "test_name": cfg.name,
                    "precision": np.int32(precision)},
        "dump1": dump1,
        "dump2": dump2,
        "CRP": crp,
        "OmegaStates": {"J": np.int32(cfg.J), "parity": np.int32(cfg.parity),
                        "l_max": np.int32(cfg.l_max), "n_omegas_max": np.int32(n_om),
                        "omegas": np.asarray(omegas, dtype=np.int32),
                        "associated_legendres": P, "wave_packets": wave_packets},
    }


def small_config(n1=16, n2=8, n_theta=6, l_max=5, J=0, parity=0, dt=10.0, steps=4, **kw) -> FH2Config:
    """A tiny grid for element-wise parity tests."""
    return FH2Config(n1=n1, n2=n2, n_theta=n_theta, l_max=l_max, J=J, parity=parity, dt=dt,
                     total_steps=steps, n_gradient_points=min(21, 2 * (n2 // 4) + 1),
                     r_flux=3.5, **kw)
