"""FP64 CPU oracle of the qd-openmp-cuda split-operator time step.

TEST INFRASTRUCTURE ONLY.  This module is the checker: tests, the smoke
entry and the CPU-baseline leg of the benchmark may call it; the product
path never does.

Parity status: **parity unpinned.**  The reference has no CPU propagator
(its ``FH2Matlab.m`` is a plotting callback), no test suite and no golden
vectors, and it cannot be built here (it needs MATLAB's ``mex.h``, the CUDA
samples' ``helper_cuda.h``, Intel MKL and sm_37/sm_52 targets).  This file
restates the reference's CUDA math step by step in numpy FP64, each function
citing the reference lines it follows.  It is pinned instead by the
reference's own invariants (norm guard, Legendre round trip of ``LTest.m``,
Coriolis reconstruction of ``test_coriolis_matrices``) and by independent
known answers (``scipy.linalg.expm`` of the Coriolis matrix, explicit DFT,
a flux normalisation test with P(E) = 1).

Layouts (``cudaMath.h:20-36``): index = (k*n2 + j)*n1 + i with i (R) fastest,
so theta-space psi of one Omega block is a C array of shape (ntheta, n2, n1)
and its Legendre-space form is (l_max - Omega + 1, n2, n1) holding slabs
l = Omega..l_max (the reference's ``legendre_psi_dev`` also keeps zero slabs
0..Omega-1, ``omegawavepacket.cu:11-15``; they never change and are not stored).
"""
from __future__ import annotations

import math
from typing import List, Optional

import os

import numpy as np
import scipy.fft
import scipy.linalg

_WORKERS = os.cpu_count() or 1


def _fd_weights(n_points: int) -> np.ndarray:
    """Centred first-derivative weights of order n_points-1 in closed form:
    w_{+-k} = +-(-1)^(k+1) (h!)^2 / (k (h-k)! (h+k)!), w_0 = 0 (h = (n-1)/2)."""
    h = (n_points - 1) // 2
    w = np.zeros(n_points)
    for k in range(1, h + 1):
        c = (-1) ** (k + 1) * math.factorial(h) ** 2 / (k * math.factorial(h - k) * math.factorial(h + k))
        w[h + k] = c
        w[h - k] = -c
    return w


def coriolis_dimension(J: int, p: int, l: int, omega_cap: Optional[int] = None):
    """``calculate_coriolis_matrix_dimension`` (CoriolisMatrix.C:52-61)."""
    if J == 0 and p != 0:
        raise ValueError("J == 0 requires p == 0")
    omega_min = 0 if (J + p) % 2 == 0 else 1
    omega_max = min(J, l)
    if omega_cap is not None:
        omega_max = min(omega_max, omega_cap)
    if l < omega_min:
        raise ValueError("l < omega_min")
    return omega_min, omega_max


def _lam(J: int, omega: int) -> float:
    # CoriolisMatrix.C:23-33 (sign%2 == 0 branch)
    return math.sqrt(J * (J + 1.0) - omega * (omega + 1.0)) if J >= omega else 0.0


def coriolis_matrix(J: int, p: int, l: int, omega_cap: Optional[int] = None):
    """Tridiagonal Coriolis matrix of ``setup_coriolis_matrix`` (CoriolisMatrix.C:63-99):
    diagonal J(J+1)-2 Omega^2, off-diagonal -lambda(J,Omega) lambda(l,Omega) sqrt(1+delta_{Omega,0})."""
    omega_min, omega_max = coriolis_dimension(J, p, l, omega_cap)
    n = omega_max - omega_min + 1
    d = np.array([J * (J + 1) - 2.0 * (k + omega_min) ** 2 for k in range(n)])
    e = np.array([-_lam(J, k + omega_min) * _lam(l, k + omega_min) * math.sqrt(1.0 + (k + omega_min == 0))
                  for k in range(n - 1)])
    return omega_min, omega_max, d, e


def coriolis_eigen(J, p, l, omega_cap=None):
    """Eigen-decomposition standing in for LAPACK ``dstev`` (CoriolisMatrix.C:94-95)."""
    omega_min, omega_max, d, e = coriolis_matrix(J, p, l, omega_cap)
    if d.size == 1:
        return omega_min, omega_max, d.copy(), np.ones((1, 1))
    ev, V = scipy.linalg.eigh_tridiagonal(d, e)
    return omega_min, omega_max, ev, V


class Oracle:
    """Propagates one FH2Data problem (all its Omega blocks) in FP64 on the CPU."""

    def __init__(self, data: dict, omega_cap: Optional[int] = None):
        self.d = data
        r1, r2, th = data["r1"], data["r2"], data["theta"]
        self.n1, self.n2, self.nth = int(r1["n"]), int(r2["n"]), int(th["n"])
        self.dr1, self.dr2 = float(r1["dr"]), float(r2["dr"])
        self.m1, self.m2 = float(r1["mass"]), float(r2["mass"])
        self.R = float(r1["left"]) + np.arange(self.n1) * self.dr1
        self.r = float(r2["left"]) + np.arange(self.n2) * self.dr2
        self.w = np.asarray(th["w"], dtype=np.float64)
        self.pot = np.asarray(data["pot"], dtype=np.float64)           # (nθ, n2, n1)
        om = data["OmegaStates"]
        self.J, self.p, self.l_max = int(om["J"]), int(om["parity"]), int(om["l_max"])
        self.omegas = [int(o) for o in om["omegas"]]
        self.omega_cap = omega_cap if omega_cap is not None else (
            self.omegas[-1] if self.J > 0 and self.omegas[-1] < min(self.J, self.l_max) else None)
        P = np.asarray(om["associated_legendres"], dtype=np.float64)   # (n_Ω, n_cols, nθ)
        self.P = []     # per block: (nθ, N_b)   (omegawavepacket.cu:134-155)
        self.wP = []    # per block: (nθ, N_b) = w_k P   (omegawavepacket.cu:157-181)
        for b, o in enumerate(self.omegas):
            Nb = self.l_max - o + 1
            Pb = P[b, :Nb, :].T.copy()
            self.P.append(Pb)
            self.wP.append(self.w[:, None] * Pb)
        wp = np.asarray(om["wave_packets"])
        self.psi = [wp[b].astype(np.complex128).copy() for b in range(len(self.omegas))]
        self.lpsi = [np.zeros((self.l_max - o + 1, self.n2, self.n1), np.complex128) for o in self.omegas]
        self.d1 = None if data.get("dump1") is None or data["dump1"].get("dump") is None else \
            np.asarray(data["dump1"]["dump"], dtype=np.float64)
        self.d2 = None if data.get("dump2") is None or data["dump2"].get("dump") is None else \
            np.asarray(data["dump2"]["dump"], dtype=np.float64)
        self.dt = float(data["time"]["time_step"])
        self.steps = int(data["time"]["steps"])
        # FFT kinetic tables (cudaMath.h:117-130)
        self.T1 = self._kin(self.n1, self.dr1, self.m1)
        self.T2 = self._kin(self.n2, self.dr2, self.m2)
        # inverse inertia tables (cudaMath.h:150-157)
        self.I1 = 1.0 / (2.0 * self.m1 * self.R * self.R)
        self.I2 = 1.0 / (2.0 * self.m2 * self.r * self.r)
        self._setup_coriolis()
        self.energies = {}
        self._setup_flux()

    # ------------------------------------------------------------------ setup
    @staticmethod
    def _kin(n, dr, mass):
        i = np.arange(n)
        k = 2.0 * math.pi / (n * dr) * np.where(i <= n // 2, i, i - n)
        return k * k / (mass + mass)

    def _setup_coriolis(self):
        # cudaOpenMP2.cu:158-209: matrices for l = omegas[0]..l_max
        self.cor = {}
        for l in range(self.omegas[0], self.l_max + 1):
            self.cor[l] = coriolis_eigen(self.J, self.p, l, self.omega_cap)

    def _setup_flux(self):
        c = self.d.get("CRP")
        self.flux_on = bool(c is not None and int(c["calculate_CRP"]) != 0)
        if not self.flux_on:
            return
        self.E = np.asarray(c["energies"], dtype=np.float64)
        self.eta_sq = np.asarray(c["eta_sq"], dtype=np.float64)
        self.n_ds = int(c["n_dividing_surface"])
        self.n_g = int(c["n_gradient_points"])
        h = (self.n_g - 1) // 2
        self.fd = _fd_weights(self.n_g) / self.dr2
        self.rows = np.arange(self.n_ds - h, self.n_ds + h + 1)
        nb = len(self.omegas)
        self.accA = np.zeros((nb, self.E.size, self.nth, self.n1), np.complex128)
        self.accD = np.zeros_like(self.accA)
        # exp(-i V dt/2) at the stencil rows: completes the Strang half step
        vs = self.pot[:, self.rows, :]                               # (nθ, n_g, n1)
        self.half_v = np.exp(-0.5j * self.dt * vs)

    # ------------------------------------------------------------------ stages
    def dump_wavepacket(self):
        """``_dump_wavepacket_`` (evolutionCUDAaux.cu:243-251)."""
        if self.d1 is None or self.d2 is None:
            return
        m = self.d2[:, None] * self.d1[None, :]
        for b in range(len(self.psi)):
            self.psi[b] *= m[None, :, :]

    def evolution_with_potential(self, dt):
        """``_evolution_with_potential_`` (evolutionCUDAaux.cu:5-11)."""
        cache = self.__dict__.setdefault("_pot_cache", {})
        if float(dt) not in cache:
            cache[float(dt)] = np.exp(-1j * dt * self.pot)
        ph = cache[float(dt)]
        for b in range(len(self.psi)):
            self.psi[b] *= ph

    def forward_legendre_transform(self):
        """ZGEMM psi[n1n2 x nθ] (w P)[nθ x N] (omegawavepacket.cu:200-219)."""
        M = self.n1 * self.n2
        for b in range(len(self.psi)):
            A = self.psi[b].reshape(self.nth, M)
            self.lpsi[b] = (self.wP[b].T @ A).reshape(-1, self.n2, self.n1)

    def backward_legendre_transform(self):
        """ZGEMM legendre_psi[n1n2 x N] P^T[N x nθ] (omegawavepacket.cu:221-240)."""
        M = self.n1 * self.n2
        for b in range(len(self.psi)):
            C = self.lpsi[b].reshape(-1, M)
            self.psi[b] = (self.P[b] @ C).reshape(self.nth, self.n2, self.n1)

    def rot_phase(self, omega, dt):
        """exp(-i dt l(l+1) (1/(2 m1 R^2) + 1/(2 m2 r^2))) for l = omega..l_max, cached per (omega, dt)."""
        key = (int(omega), float(dt))
        cache = self.__dict__.setdefault("_rot_cache", {})
        if key not in cache:
            l = np.arange(omega, self.l_max + 1, dtype=np.float64)
            ll = l * (l + 1.0)
            I = self.I2[:, None] + self.I1[None, :]
            cache[key] = np.exp(-1j * dt * ll[:, None, None] * I[None, :, :])
        return cache[key]

    def evolution_with_rotational(self, dt):
        """``_evolution_with_rotational_`` (evolutionCUDAaux.cu:33-54)."""
        for b, o in enumerate(self.omegas):
            self.lpsi[b] *= self.rot_phase(o, dt)

    def forward_fft(self):
        """cufft Z2Z forward over dims {n2, n1} (wavepackets1device.cu:186-201)."""
        for b in range(len(self.lpsi)):
            self.lpsi[b] = scipy.fft.fft2(self.lpsi[b], axes=(1, 2), workers=_WORKERS)

    def backward_fft(self):
        """cufft Z2Z inverse + ZDSCAL 1/(n1 n2) (omegawavepacket.cu:250-269)."""
        for b in range(len(self.lpsi)):
            self.lpsi[b] = scipy.fft.ifft2(self.lpsi[b], axes=(1, 2), workers=_WORKERS)

    def evolution_with_kinetic(self, dt):
        """``_evolution_with_kinetic_`` (evolutionCUDAaux.cu:13-31)."""
        T = self.T2[:, None] + self.T1[None, :]
        ph = np.exp(-1j * dt * T)
        for b in range(len(self.lpsi)):
            self.lpsi[b] *= ph[None, :, :]

    def coriolis_factors(self, l, dt):
        """U_{Omega Omega1}(R) = sum_a exp(-i dt e_a/(2 m1 R^2)) V[Omega,a] V[Omega1,a]
        (evolutionCUDAaux.cu:178-209), shape (n, n, n1)."""
        omin, omax, ev, V = self.cor[l]
        ph = np.exp(-1j * dt * ev[:, None] / (2.0 * self.m1 * self.R[None, :] ** 2))   # (n, n1)
        return np.einsum("pa,qa,ai->pqi", V, V, ph)

    def evolution_with_coriolis(self, dt, calculate_energy=False):
        """Coriolis half step (cudaOpenMP2.cu:392-423, wavepackets1device.cu:485-495,
        omegawavepacket.cu:430-489).  The coupling energy is evaluated on the
        pre-update psi (omegawavepacket.cu:503-553 runs before the D2D update).
        Per l, the blocks present in the l-matrix are stacked and updated together:
        psi'[Omega](R, r) = sum_Omega1 U_{Omega Omega1}(R) psi[Omega1](R, r)."""
        nb = len(self.omegas)
        if calculate_energy:
            # sum over pairs |Omega - Omega1| <= 1, weight 2 off the diagonal
            # (wavepackets1device.cu:515-530); H_{Omega Omega1} = sum_a e_a V V / (2 m1 R^2)
            ce = np.zeros(nb)
            inv2mR2 = 1.0 / (2.0 * self.m1 * self.R ** 2)
            for l in range(self.omegas[0], self.l_max + 1):
                omin, omax, ev, V = self.cor[l]
                present = [b for b, o in enumerate(self.omegas) if o <= l and omin <= o <= omax]
                for i in present:
                    for j in present:
                        oi, oj = self.omegas[i], self.omegas[j]
                        if oj < oi or oj - oi > 1:
                            continue
                        h = np.sum(ev * V[oi - omin] * V[oj - omin])
                        a = self.lpsi[i][l - oi]
                        bb = self.lpsi[j][l - oj]
                        dot = np.vdot(a * inv2mR2[None, :], bb) * h
                        if oi != oj:
                            dot *= 2.0
                        ce[i] += dot.real * self.dr1 * self.dr2
            self.energies["coriolis"] = ce
        new = [x.copy() for x in self.lpsi]
        for l in range(self.omegas[0], self.l_max + 1):
            omin, omax, ev, V = self.cor[l]
            present = [b for b, o in enumerate(self.omegas) if o <= l and omin <= o <= omax]
            if not present:
                continue
            U = self.coriolis_factors(l, dt)                          # (n, n, n1)
            idx = [self.omegas[b] - omin for b in present]
            Us = U[np.ix_(idx, idx)]                                  # (m, m, n1)
            S = np.stack([self.lpsi[b][l - self.omegas[b]] for b in present])   # (m, n2, n1)
            out = np.einsum("pqi,qji->pji", Us, S, optimize=True)
            for k, b in enumerate(present):
                new[b][l - self.omegas[b]] = out[k]
        self.lpsi = new

    # ------------------------------------------------------------- energies
    def kinetic_energy(self):
        """omegawavepacket.cu:364-395: dr1 dr2/(n1 n2) sum_l <psi_l|T|psi_l>."""
        T = self.T2[:, None] + self.T1[None, :]
        return np.array([np.sum(T[None] * np.abs(x) ** 2) * self.dr1 * self.dr2 / (self.n1 * self.n2)
                         for x in self.lpsi])

    def rotational_energy(self):
        """omegawavepacket.cu:397-428: dr1 dr2 sum_l l(l+1) <psi_l|I^-1|psi_l>."""
        I = self.I2[:, None] + self.I1[None, :]
        out = []
        for b, o in enumerate(self.omegas):
            l = np.arange(o, self.l_max + 1, dtype=np.float64)
            s = np.sum(np.abs(self.lpsi[b]) ** 2 * I[None], axis=(1, 2))
            out.append(np.sum(l * (l + 1) * s) * self.dr1 * self.dr2)
        return np.array(out)

    def potential_energy(self):
        """omegawavepacket.cu:101-132."""
        return np.array([np.sum(self.w[:, None, None] * self.pot * np.abs(x) ** 2) * self.dr1 * self.dr2
                         for x in self.psi])

    def module(self):
        """omegawavepacket.cu:76-99."""
        return np.array([np.sum(self.w[:, None, None] * np.abs(x) ** 2) * self.dr1 * self.dr2
                         for x in self.psi])

    # ------------------------------------------------------------------ flux
    def accumulate_flux(self):
        """Energy-resolved flux through r = r_s (the reference parses CRP but has
        no flux code; this is the project's own definition).  psi(t_{n+1}) on the
        stencil rows is exp(-i V dt/2) psi_theta; A_E += dt e^{iEt} psi(R, r_s, x_k),
        D_E += dt e^{iEt} d_r psi(R, r_s, x_k) with a centred FD stencil.  The
        surface values are buffered and added to the accumulators as one
        (energies x steps) @ (steps x points) product every 32 steps."""
        if not self.flux_on:
            return
        h = (self.n_g - 1) // 2
        surf = []
        for b in range(len(self.psi)):
            s = self.half_v * self.psi[b][:, self.rows, :]              # (nθ, n_g, n1)
            surf.append((s[:, h, :], np.einsum("g,kgi->ki", self.fd, s)))
        buf = self.__dict__.setdefault("_flux_buf", [])
        buf.append(((self.steps + 1) * self.dt, surf))
        if len(buf) >= 32:
            self._flush_flux()

    def _flush_flux(self):
        buf = self.__dict__.get("_flux_buf", [])
        if not buf:
            return
        t = np.array([x[0] for x in buf])
        ph = self.dt * np.exp(1j * self.E[:, None] * t[None, :])         # (nE, n_steps)
        for b in range(len(self.psi)):
            A = np.stack([x[1][b][0] for x in buf]).reshape(len(buf), -1)
            D = np.stack([x[1][b][1] for x in buf]).reshape(len(buf), -1)
            self.accA[b] += (ph @ A).reshape(self.accA[b].shape)
            self.accD[b] += (ph @ D).reshape(self.accD[b].shape)
        buf.clear()

    def crp(self):
        """P(E) = Im sum_{Omega,k,i} w_k dR conj(A_E) D_E / (2 pi mu_r eta^2(E))."""
        if not self.flux_on:
            return None
        self._flush_flux()
        s = np.einsum("k,beki->e", self.w, np.conj(self.accA) * self.accD) * self.dr1
        return s.imag / (2.0 * math.pi * self.m2 * self.eta_sq)

    # ------------------------------------------------------------------ step
    def step(self):
        """One time step in the order of ``test_multiple_cards`` (cudaOpenMP2.cu:338-386)."""
        dt = self.dt
        self.dump_wavepacket()
        if self.steps == 0:
            self.evolution_with_potential(-dt / 2)
        self.evolution_with_potential(dt)
        self.forward_legendre_transform()
        self.evolution_with_rotational(dt / 4)
        self.evolution_with_coriolis(dt / 2)
        self.evolution_with_rotational(dt / 4)
        self.forward_fft()
        self.evolution_with_kinetic(dt)
        ke = self.kinetic_energy()
        self.backward_fft()
        self.evolution_with_rotational(dt / 4)
        self.evolution_with_coriolis(dt / 2, calculate_energy=True)
        self.evolution_with_rotational(dt / 4)
        re = self.rotational_energy()
        self.backward_legendre_transform()
        pe = self.potential_energy()
        mod = self.module()
        ce = self.energies.get("coriolis", np.zeros(len(self.omegas)))
        self.energies = {"module": mod, "potential": pe, "kinetic": ke, "rotational": re,
                         "coriolis": ce, "total": pe + ke + re + ce}
        self.accumulate_flux()
        self.steps += 1
        return self.energies

    def run(self, n_steps: int):
        rec = []
        for _ in range(n_steps):
            e = self.step()
            rec.append(np.stack([e["module"], e["potential"], e["kinetic"], e["rotational"],
                                 e["coriolis"], e["total"]], axis=1))
        return np.array(rec)        # (steps, n_Ω, 6)

    def wave_packets(self) -> np.ndarray:
        return np.stack(self.psi)
