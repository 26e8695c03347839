"""CPU checks of the FP64 oracle and of the input builders.

The reference has no golden vectors (no tests, no CPU propagator), so the
oracle is pinned by the reference's own invariants and by independent known
answers.
"""
import math

import numpy as np
import pytest
import scipy.linalg
import scipy.special


def test_legendre_matches_scipy(qd):
    """Normalised associated Legendre = MATLAB legendre(l, x, 'norm') (AssLegendreP.m:9-12)."""
    x = np.linspace(-0.97, 0.97, 11)
    for m in range(0, 5):
        P = qd.inputs.normalized_associated_legendre(9, m, x)
        for l in range(m, 10):
            norm = math.sqrt((l + 0.5) * math.factorial(l - m) / math.factorial(l + m))
            ref = (-1) ** m * norm * scipy.special.lpmv(m, l, x)   # remove Condon-Shortley phase
            np.testing.assert_allclose(P[:, l - m], ref, rtol=1e-12, atol=1e-13)


def test_legendre_orthonormal_and_round_trip(qd):
    """Gauss-Legendre quadrature makes P^T W P = I, so the LTest.m:43-48 round trip keeps the norm."""
    n, lmax = 24, 23
    x, w = qd.inputs.gauss_legendre(n)
    for m in (0, 1, 5, 12):
        P = qd.inputs.normalized_associated_legendre(lmax, m, x)
        np.testing.assert_allclose(P.T @ (w[:, None] * P), np.eye(lmax - m + 1), atol=1e-13)
    rng = np.random.default_rng(0)
    P = qd.inputs.normalized_associated_legendre(lmax, 0, x)
    psi = rng.standard_normal((50, n)) + 1j * rng.standard_normal((50, n))
    s0 = np.sum(w * np.sum(np.abs(psi) ** 2, 0))
    for _ in range(3):
        c = psi @ (w[:, None] * P)
        psi = c @ P.T
    # the first pass projects onto the span; afterwards the norm is invariant
    s1 = np.sum(w * np.sum(np.abs(psi) ** 2, 0))
    c = psi @ (w[:, None] * P)
    psi2 = c @ P.T
    s2 = np.sum(w * np.sum(np.abs(psi2) ** 2, 0))
    assert s1 <= s0 + 1e-12
    assert abs(s2 - s1) < 1e-12 * s1


@pytest.mark.parametrize("J,p", [(1, 0), (1, 1), (4, 1), (12, 0), (7, 1), (28, 0), (40, 0)])
def test_coriolis_matrix_exponential(oracle, J, p):
    """U = sum_a exp(-i dt e_a/I) V V^T equals expm(-i dt H / I) (evolutionCUDAaux.cu:178-209),
    V diag(e) V^T reconstructs H (evolutionCUDAaux.cu:114-128) and U is unitary; J = 28 and 40
    reach the 29- and 41-block groups of the large-group GPU cases."""
    for l in range((J + p) % 2, max(15, J + 6)):
        omin, omax, d, e = oracle.coriolis_matrix(J, p, l)
        H = np.diag(d) + np.diag(e, 1) + np.diag(e, -1)
        _, _, ev, V = oracle.coriolis_eigen(J, p, l)
        np.testing.assert_allclose(V @ np.diag(ev) @ V.T, H, atol=1e-11 * max(1, np.abs(H).max()))
        I = 2 * 3000.0 * 4.0 ** 2
        dt = 5.0
        U = V @ np.diag(np.exp(-1j * dt * ev / I)) @ V.T
        np.testing.assert_allclose(U, scipy.linalg.expm(-1j * dt * H / I), atol=1e-12)
        np.testing.assert_allclose(U.conj().T @ U, np.eye(U.shape[0]), atol=1e-12)


def test_j0_coriolis_is_identity(qd, oracle):
    cfg = qd.inputs.small_config(J=0)
    o = oracle.Oracle(qd.inputs.build_fh2data(cfg))
    rng = np.random.default_rng(1)
    o.lpsi = [rng.standard_normal(x.shape) + 1j * rng.standard_normal(x.shape) for x in o.lpsi]
    before = [x.copy() for x in o.lpsi]
    o.evolution_with_coriolis(5.0, calculate_energy=True)
    for a, b in zip(o.lpsi, before):
        np.testing.assert_array_equal(a, b)
    assert np.all(o.energies["coriolis"] == 0.0)


def test_fft_stage_is_the_unnormalised_dft(qd, oracle):
    cfg = qd.inputs.small_config(n1=8, n2=6, n_theta=4, l_max=3)
    o = oracle.Oracle(qd.inputs.build_fh2data(cfg))
    rng = np.random.default_rng(2)
    x = rng.standard_normal((4, 6, 8)) + 1j * rng.standard_normal((4, 6, 8))
    o.lpsi = [x.copy()]
    o.forward_fft()
    F1 = np.exp(-2j * np.pi * np.outer(np.arange(8), np.arange(8)) / 8)
    F2 = np.exp(-2j * np.pi * np.outer(np.arange(6), np.arange(6)) / 6)
    ref = np.einsum("ab,lbc,dc->lad", F2, x, F1)
    np.testing.assert_allclose(o.lpsi[0], ref, atol=1e-12)
    o.backward_fft()
    np.testing.assert_allclose(o.lpsi[0], x, atol=1e-13)


def _free_gaussian(x, x0, sig, k0, m, t):
    """Closed-form free-particle solution (hbar = 1) from exp(-(x-x0)^2/(4 sig^2) + i k0 x)."""
    a = 1 + 1j * t / (2 * m * sig ** 2)
    v = k0 / m
    return a ** -0.5 * np.exp(-(x - x0 - v * t) ** 2 / (4 * sig ** 2 * a)) * np.exp(1j * k0 * (x - v * t / 2))


def test_kinetic_stage_is_the_free_particle_propagator(qd, oracle):
    """Known answer for forward FFT + _evolution_with_kinetic_ + inverse FFT (evolutionCUDAaux.cu:13-31):
    a Gaussian packet (width L/24, momentum 0.3/dr in R and r) propagates as the closed-form
    free particle of masses m1, m2 (to 1e-12 at t = 50, before it reaches the periodic edge), and
    the kinetic-energy sum (omegawavepacket.cu:364-395) equals (k0^2 + 1/(4 sigma^2))/(2m) per
    coordinate times the norm."""
    cfg = qd.inputs.small_config(J=0, n1=128, n2=64, n_theta=6, l_max=5, steps=1)
    o = oracle.Oracle(qd.inputs.build_fh2data(cfg))
    LR, Lr = o.n1 * o.dr1, o.n2 * o.dr2
    sR, sr, kR, kr = LR / 24, Lr / 24, 0.3 / o.dr1, 0.3 / o.dr2
    x0R, x0r = o.R[0] + 0.45 * LR, o.r[0] + 0.45 * Lr

    def packet(t):
        return np.outer(_free_gaussian(o.r, x0r, sr, kr, o.m2, t), _free_gaussian(o.R, x0R, sR, kR, o.m1, t))

    psi0 = packet(0.0)
    o.lpsi[0][...] = 0
    o.lpsi[0][0] = psi0
    o.forward_fft()
    norm = np.sum(np.abs(psi0) ** 2) * o.dr1 * o.dr2
    ke = norm * ((kR ** 2 + 1 / (4 * sR ** 2)) / (2 * o.m1) + (kr ** 2 + 1 / (4 * sr ** 2)) / (2 * o.m2))
    np.testing.assert_allclose(o.kinetic_energy()[0], ke, rtol=1e-12)
    o.evolution_with_kinetic(50.0)
    o.backward_fft()
    assert np.abs(o.lpsi[0][0] - packet(50.0)).max() < 1e-12


@pytest.mark.parametrize("J,p", [(0, 0), (2, 0), (3, 1)])
def test_norm_conserved_without_mask(qd, oracle, J, p):
    """Without the absorbing mask every factor is unitary: the module stays 1."""
    cfg = qd.inputs.small_config(J=J, parity=p, n1=16, n2=8, n_theta=8, l_max=6)
    d = qd.inputs.build_fh2data(cfg)
    d["dump1"] = None
    d["dump2"] = None
    if J:   # put the packet in the lowest Omega and let Coriolis spread it
        pass
    o = oracle.Oracle(d)
    rec = o.run(8)
    np.testing.assert_allclose(rec[:, :, 0].sum(1), 1.0, atol=1e-12)


def test_flux_normalisation_known_answer(qd, oracle):
    """P(E) = 1 for a packet that crosses the dividing surface freely.

    A Gaussian moving toward +r (no potential along r) with R bound in a
    harmonic well: every energy component crosses r_s once, so the
    energy-normalised flux must be 1 across the packet's energy range.
    """
    inp = qd.inputs
    n1, n2, nth = 8, 192, 2
    mu_R, mu_r = 3000.0, 918.0
    R = np.linspace(1.0, 3.0, n1)
    r = np.linspace(0.5, 28.0, n2)
    dR, dr = R[1] - R[0], r[1] - r[0]
    x, w = inp.gauss_legendre(nth)
    omega = 0.02
    VR = 0.5 * mu_R * omega ** 2 * (R - 2.0) ** 2
    # R ground state of the FFT-kinetic Hamiltonian
    T = inp.fft_kinetic(n1, dR, mu_R)
    Tm = np.real(np.fft.ifft(T[:, None] * np.fft.fft(np.eye(n1), axis=0), axis=0))
    e0s, vs = np.linalg.eigh(0.5 * (Tm + Tm.T) + np.diag(VR))
    e0, phi = e0s[0], vs[:, 0] * np.sign(vs[np.argmax(np.abs(vs[:, 0])), 0])
    phi /= math.sqrt(np.sum(phi ** 2) * dR)
    r0, delta, ecoll = 6.0, 0.6, 0.05
    k0 = math.sqrt(2 * mu_r * ecoll)
    g = (1 / (math.pi * delta ** 2)) ** 0.25 * np.exp(-((r - r0) ** 2) / (2 * delta ** 2) + 1j * k0 * r)
    g /= math.sqrt(np.sum(np.abs(g) ** 2) * dr)
    psi = (1 / math.sqrt(2)) * g[None, :, None] * phi[None, None, :] * np.ones((nth, 1, 1))
    pot = np.broadcast_to(VR[None, None, :], (nth, n2, n1)).copy()
    dt, steps = 10.0, 260
    ecol = np.linspace(0.03, 0.07, 9)
    # flux of an outgoing e^{+ikr} packet: same |a(E)|^2 formula
    eta = mu_r / np.sqrt(2 * mu_r * ecol) * (delta / math.sqrt(math.pi)) * np.exp(
        -(delta ** 2) * (np.sqrt(2 * mu_r * ecol) - k0) ** 2)
    rs = 14.0
    d = {
        "r1": {"n": n1, "left": R[0], "dr": dR, "mass": mu_R},
        "r2": {"n": n2, "left": r[0], "dr": dr, "mass": mu_r},
        "theta": {"n": nth, "m": 1, "x": x, "w": w, "associated_legendre": None},
        "pot": pot, "psi": None,
        "time": {"total_steps": steps, "time_step": dt, "steps": 0},
        "options": {},
        "dump1": {"dump": np.ones(n1)},
        "dump2": {"dump": inp.cap_mask(r, 6.0, 0.002, dt)},
        "CRP": {"energies": ecol + e0, "eta_sq": eta, "CRP": np.zeros(ecol.size),
                "n_dividing_surface": int(round((rs - r[0]) / dr)), "n_gradient_points": 21,
                "n_energies": ecol.size, "calculate_CRP": 1},
        "OmegaStates": {"J": 0, "parity": 0, "l_max": 1, "n_omegas_max": 1, "omegas": np.array([0]),
                        "associated_legendres": inp.normalized_associated_legendre(1, 0, x).T[None],
                        "wave_packets": psi[None].astype(np.complex128)},
    }
    o = oracle.Oracle(d)
    o.run(steps)
    P = o.crp()
    np.testing.assert_allclose(P, 1.0, atol=3e-3)


def test_fd_weights_exact_on_polynomials(qd, oracle):
    for n in (3, 5, 11, 21):
        wi = qd.inputs.finite_difference_weights(n)
        wo = oracle._fd_weights(n)
        np.testing.assert_allclose(wi, wo, atol=1e-9)
        h = (n - 1) // 2
        xs = np.arange(-h, h + 1, dtype=float)
        for p in range(1, min(n - 1, 8)):
            np.testing.assert_allclose(np.sum(wi * xs ** p), p * 0.0 ** (p - 1), atol=1e-8)


def test_omega_list_and_leps(qd):
    inp = qd.inputs
    assert inp.omega_list(0, 0, 10) == [0]
    assert inp.omega_list(4, 1, 200) == [1, 2, 3, 4]      # FH2main.m:33
    assert inp.omega_list(3, 1, 200) == [0, 1, 2, 3]      # FH2main.m:31
    assert inp.omega_list(40, 0, 79, omega_cap=20) == list(range(0, 21))
    # asymptote of the LEPS surface is the H2 Morse curve
    r = np.linspace(0.8, 4.0, 7)
    np.testing.assert_allclose(inp.leps_fh2(60.0, r, 0.3), inp.morse_hh(r), atol=1e-12)
    assert inp.morse_hh(np.array([inp.LEPS_HH[2]]))[0] == pytest.approx(-inp.LEPS_HH[0])


def test_golden_fixture_regression(qd, oracle):
    """The oracle reproduces its committed outputs (tests/golden, made by make_golden.py)."""
    from pathlib import Path
    gold = Path(__file__).parent / "golden" / "oracle_small.npz"
    if not gold.exists():
        pytest.skip("golden fixture not generated")
    z = np.load(gold)
    for name in ("j0", "j2"):
        cfg = qd.inputs.small_config(n1=16, n2=8, n_theta=6, l_max=5, J=int(z[f"{name}_J"]), parity=0,
                                     steps=int(z[f"{name}_steps"]), n_energies=8)
        o = oracle.Oracle(qd.inputs.build_fh2data(cfg))
        rec = o.run(cfg.total_steps)
        np.testing.assert_allclose(o.wave_packets(), z[f"{name}_psi"], rtol=0, atol=1e-13)
        np.testing.assert_allclose(rec, z[f"{name}_energies"], rtol=1e-11, atol=1e-14)
        np.testing.assert_allclose(o.crp(), z[f"{name}_crp"], rtol=1e-9, atol=1e-12)
