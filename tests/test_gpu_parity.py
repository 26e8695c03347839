"""GPU parity: the CUDA path through the C ABI against the FP64 oracle.

Tolerances: FP64 form, element-wise relative L2 error of psi <= 1e-12 after a
few steps and <= 1e-10 after 1000 steps; energies to 1e-11 relative; P(E)
within 1e-8 absolute.  Mixed form: psi <= 1e-5 relative, P(E) within 1e-4
absolute.  P(E) is compared inside the initial packet's energy window
(|a(E)|^2 >= 1e-4 max |a|^2): outside it P = flux/|a|^2 divides rounding
noise by |a|^2 < 1e-11 and is not a probability in either form.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(np.asarray(b)), 1e-300))


def dP_window(qd, d, got, ref):
    """max |P_got - P_ref| over the energies the initial packet carries."""
    win = qd.inputs.energy_window(d["CRP"]["eta_sq"])
    assert win.any()
    return float(np.max(np.abs(np.asarray(got) - np.asarray(ref))[win]))


def make(qd, **kw):
    steps = kw.pop("steps", 4)
    cfg = qd.inputs.small_config(steps=steps, **kw)
    return cfg, qd.inputs.build_fh2data(cfg), qd.inputs.build_fh2data(cfg)


CASES = [
    dict(J=0, n1=16, n2=8, n_theta=6, l_max=5),
    dict(J=2, parity=0, n1=16, n2=8, n_theta=8, l_max=6),
    dict(J=3, parity=1, n1=24, n2=12, n_theta=8, l_max=7),
    # (J + p) odd: Omega = 1..4, so the packet starts in Omega = 1
    dict(J=4, parity=1, n1=32, n2=16, n_theta=10, l_max=8, n_energies=12, init_omega=1),
]


@pytest.fixture(scope="module")
def gpu(lib):
    return lib


def _random_state(o, rng):
    for b in range(len(o.psi)):
        o.psi[b] = (rng.standard_normal(o.psi[b].shape) + 1j * rng.standard_normal(o.psi[b].shape)) * 1e-2


@pytest.mark.parametrize("case", CASES[:3])
def test_stages_match_oracle(qd, oracle, gpu, case):
    """Each reference stage (omegawavepacket.h:79-126) on the same random state."""
    cfg, d, dref = make(qd, **case)
    o = oracle.Oracle(dref)
    rng = np.random.default_rng(7)
    _random_state(o, rng)
    dt = cfg.dt
    with qd.Session(d) as s:
        for b in range(len(o.psi)):
            s.set_psi("theta", b, o.psi[b])
        checks = [
            ("dump", 0.0, o.dump_wavepacket, "theta"),
            ("potential", dt, lambda: o.evolution_with_potential(dt), "theta"),
            ("forward_legendre", 0.0, o.forward_legendre_transform, "j"),
            ("rotational", dt / 4, lambda: o.evolution_with_rotational(dt / 4), "j"),
            ("coriolis", dt / 2, lambda: o.evolution_with_coriolis(dt / 2), "j"),
            ("fft_kinetic", dt, lambda: (o.forward_fft(), o.evolution_with_kinetic(dt), o.backward_fft()), "j"),
            ("coriolis_energy", dt / 2, lambda: o.evolution_with_coriolis(dt / 2, calculate_energy=True), "j"),
            ("backward_legendre", 0.0, o.backward_legendre_transform, "theta"),
        ]
        for stage, sdt, fn, space in checks:
            if stage == "fft_kinetic":
                ke_ref = None
                o.forward_fft(); o.evolution_with_kinetic(dt); ke_ref = o.kinetic_energy(); o.backward_fft()
            else:
                fn()
            s.apply(stage, sdt)
            for b in range(len(o.psi)):
                got = s.get_psi(space, b)
                ref = o.psi[b] if space == "theta" else o.lpsi[b]
                assert rel(got, ref) < 1e-13, (stage, b, rel(got, ref))
            if stage == "fft_kinetic":
                np.testing.assert_allclose(s.energies()[:, 2], ke_ref, rtol=1e-12, atol=1e-18)
            if stage == "coriolis_energy":
                np.testing.assert_allclose(s.energies()[:, 4], o.energies["coriolis"], rtol=1e-10, atol=1e-16)
        s.apply("energies")
        e = s.energies()
        np.testing.assert_allclose(e[:, 0], o.module(), rtol=1e-12)
        np.testing.assert_allclose(e[:, 1], o.potential_energy(), rtol=1e-11, atol=1e-16)
        np.testing.assert_allclose(e[:, 3], o.rotational_energy(), rtol=1e-11, atol=1e-16)


@pytest.mark.parametrize("case", CASES)
def test_evolve_matches_oracle(qd, oracle, gpu, case):
    """Full steps of test_multiple_cards (cudaOpenMP2.cu:338-386) via qd_evolve."""
    cfg, d, dref = make(qd, steps=6, **case)
    nb = len(d["OmegaStates"]["omegas"])
    d["options"]["energies"] = np.zeros((cfg.total_steps, nb, 6))
    o = oracle.Oracle(dref)
    rec = o.run(cfg.total_steps)
    qd.cudaOpenMPEvolution(d)
    assert int(d["time"]["steps"]) == cfg.total_steps
    assert rel(d["OmegaStates"]["wave_packets"], o.wave_packets()) < 1e-12
    np.testing.assert_allclose(d["options"]["energies"][:, :, :4], rec[:, :, :4], rtol=1e-10, atol=1e-15)
    np.testing.assert_allclose(d["options"]["energies"][:, :, 4], rec[:, :, 4], rtol=1e-8, atol=1e-14)
    assert np.abs(o.wave_packets()).max() > 0
    assert dP_window(qd, d, d["CRP"]["CRP"], o.crp()) <= 1e-8


def test_fp64_1000_steps_reference_grid(qd, oracle, gpu):
    """64x32x24, J=0, dt=10, 1000 steps: relative |dpsi| <= 1e-10 and |dP(E)| <= 1e-8 in the window."""
    cfg = qd.inputs.CONFIGS["fh2_j0_64x32x24"]
    d = qd.inputs.build_fh2data(cfg)
    d["time"]["total_steps"] = 1000
    o = oracle.Oracle(qd.inputs.build_fh2data(cfg))
    o.run(1000)
    qd.cudaOpenMPEvolution(d)
    assert rel(d["OmegaStates"]["wave_packets"], o.wave_packets()) < 1e-10
    crp = o.crp()
    win = qd.inputs.energy_window(d["CRP"]["eta_sq"])
    assert np.abs(crp[win]).max() > 1.0     # a propagated flux, not a vacuous comparison
    assert dP_window(qd, d, d["CRP"]["CRP"], crp) <= 1e-8


def test_batch_equals_separate_problems(qd, oracle, gpu):
    """Uneven Omega counts (J = 0, 1, 2, 3) stepped in one batch."""
    cfgs = [qd.inputs.small_config(J=J, parity=0, n1=16, n2=8, n_theta=8, l_max=6, steps=5, n_energies=8)
            for J in (0, 1, 2, 3)]
    ds = [qd.inputs.build_fh2data(c) for c in cfgs]
    qd.evolve_batch(ds)
    for c, d in zip(cfgs, ds):
        o = oracle.Oracle(qd.inputs.build_fh2data(c))
        o.run(c.total_steps)
        assert rel(d["OmegaStates"]["wave_packets"], o.wave_packets()) < 1e-12
        assert dP_window(qd, d, d["CRP"]["CRP"], o.crp()) <= 1e-8


def test_callback_sees_copied_wave_packets(qd, oracle, gpu):
    """wave_to_matlab fires when steps % N == 0, after the D2H copy (cudaOpenMP2.cu:380-384)."""
    cfg, d, dref = make(qd, J=0, n1=16, n2=8, n_theta=6, l_max=5, steps=7)
    d["options"]["wave_to_matlab"] = "FH2Matlab.m"
    d["options"]["steps_to_copy_psi_from_device_to_host"] = 3
    o = oracle.Oracle(dref)
    seen = []

    def cb(data):
        seen.append((int(data["time"]["steps"]), data["OmegaStates"]["wave_packets"].copy()))
        return 0

    qd.cudaOpenMPEvolution(d, callback=cb)
    assert [s for s, _ in seen] == [0, 3, 6]
    for st, psi in seen:
        while o.steps <= st:
            o.step()
        assert rel(psi, o.wave_packets()) < 1e-12


@pytest.mark.parametrize("J", [0, 2])
def test_mixed_graph_chunks_equal_single_steps(qd, gpu, J):
    """140 mixed steps replayed from 64-step graphs (device-side step counter, flux slot and
    record index) equal the same steps enqueued one at a time (a callback after every step):
    wave packets and energy records bit for bit; P(E) in the energy window to 1e-12 of its
    maximum there (a callback may flush the surface buffer at other steps, which regroups the
    FP64 sums)."""
    out = []
    for every_step in (False, True):
        cfg, d, _ = make(qd, J=J, parity=0, n1=32, n2=16, n_theta=8, l_max=6, steps=140, n_energies=8)
        d["options"]["precision"] = 1
        nb = len(np.ravel(d["OmegaStates"]["omegas"]))
        d["options"]["energies"] = np.zeros((cfg.total_steps, nb, 6))
        if every_step:
            d["options"]["wave_to_matlab"] = "FH2Matlab.m"
            d["options"]["steps_to_copy_psi_from_device_to_host"] = 1
            qd.cudaOpenMPEvolution(d, callback=lambda data: 0)
        else:
            qd.cudaOpenMPEvolution(d)
        assert int(d["time"]["steps"]) == cfg.total_steps
        out.append(d)
    a, b = out
    assert np.array_equal(a["OmegaStates"]["wave_packets"], b["OmegaStates"]["wave_packets"])
    assert np.array_equal(a["options"]["energies"], b["options"]["energies"])
    win = qd.inputs.energy_window(b["CRP"]["eta_sq"])
    assert dP_window(qd, b, a["CRP"]["CRP"], b["CRP"]["CRP"]) <= 1e-12 * np.abs(b["CRP"]["CRP"][win]).max()


def test_callback_error_aborts(qd, gpu):
    cfg, d, _ = make(qd, J=0, steps=4)
    d["options"]["wave_to_matlab"] = "FH2Matlab.m"
    d["options"]["steps_to_copy_psi_from_device_to_host"] = 2
    with pytest.raises(qd.QDError) as e:
        qd.cudaOpenMPEvolution(d, callback=lambda data: 1)
    assert e.value.status == 5


def test_norm_guard(qd, gpu):
    """insist(total_module <= 1) (cudaOpenMP2.cu:437-440) becomes QD_ERR_NORM."""
    cfg, d, _ = make(qd, J=0, steps=3)
    d["OmegaStates"]["wave_packets"] *= 1.5
    with pytest.raises(qd.QDError) as e:
        qd.cudaOpenMPEvolution(d)
    assert e.value.status == 4
    assert "step 0" in str(e.value)


def test_resume_in_two_calls(qd, gpu):
    """time.steps is in/out: two calls of N steps equal one call of 2N (V(-dt/2) only at steps == 0)."""
    cfg, d1, _ = make(qd, J=2, parity=0, n1=16, n2=8, n_theta=8, l_max=6, steps=8, n_energies=8)
    d2 = qd.inputs.build_fh2data(cfg)
    qd.cudaOpenMPEvolution(d1)
    nb = len(d2["OmegaStates"]["omegas"])
    acc = np.zeros((nb, 2, 8, cfg.n_theta, cfg.n1), np.complex128)
    d2["CRP"]["accumulators"] = acc
    d2["time"]["total_steps"] = 4
    qd.cudaOpenMPEvolution(d2)
    assert int(d2["time"]["steps"]) == 4
    qd.cudaOpenMPEvolution(d2)
    assert int(d2["time"]["steps"]) == 8
    assert rel(d2["OmegaStates"]["wave_packets"], d1["OmegaStates"]["wave_packets"]) < 1e-13
    np.testing.assert_allclose(d2["CRP"]["CRP"], d1["CRP"]["CRP"], rtol=1e-11, atol=1e-14)


def test_norm_conserved_at_production_grid(qd, gpu):
    """256x128x96, l_max=95, no mask: the module stays 1 (unitary factors) over 20 steps."""
    cfg = qd.inputs.CONFIGS["fh2_j0_256x128x96"]
    d = qd.inputs.build_fh2data(cfg)
    d["dump1"] = None
    d["dump2"] = None
    d["time"]["total_steps"] = 20
    d["CRP"]["calculate_CRP"] = 0
    d["options"]["energies"] = np.zeros((20, 1, 6))
    qd.cudaOpenMPEvolution(d)
    mod = d["options"]["energies"][:, 0, 0]
    np.testing.assert_allclose(mod, 1.0, atol=1e-12)
    tot = d["options"]["energies"][:, 0, 5]
    assert np.ptp(tot) < 1e-4 * abs(tot.mean())


def test_mixed_precision_close_to_fp64(qd, oracle, gpu):
    cfg, d, dref = make(qd, J=2, parity=0, n1=32, n2=16, n_theta=8, l_max=6, steps=20, n_energies=64)
    d["options"]["precision"] = 1
    o = oracle.Oracle(dref)
    o.run(cfg.total_steps)
    qd.cudaOpenMPEvolution(d)
    assert rel(d["OmegaStates"]["wave_packets"], o.wave_packets()) < 1e-5
    crp = o.crp()
    dp = dP_window(qd, d, d["CRP"]["CRP"], crp)
    win = qd.inputs.energy_window(d["CRP"]["eta_sq"])
    assert dp <= 1e-4
    assert dp <= 1e-3 * np.abs(crp[win]).max()


@pytest.mark.parametrize("case", [dict(J=0, n1=16, n2=8, n_theta=6, l_max=5),
                                  dict(J=2, parity=0, n1=32, n2=16, n_theta=24, l_max=23),
                                  dict(J=3, parity=1, n1=24, n2=12, n_theta=40, l_max=37),
                                  dict(J=0, n1=64, n2=32, n_theta=8, l_max=7),
                                  dict(J=1, parity=0, n1=256, n2=128, n_theta=8, l_max=7),
                                  dict(J=2, parity=0, n1=192, n2=96, n_theta=8, l_max=7)])
def test_mixed_stages_match_oracle(qd, oracle, gpu, case):
    """tcgen05 BF16x3 Legendre contractions and the FP32 FFT: FP32-level agreement (rel <= 3e-6)."""
    cfg, d, dref = make(qd, **case)
    d["options"]["precision"] = 1
    o = oracle.Oracle(dref)
    rng = np.random.default_rng(11)
    _random_state(o, rng)
    with qd.Session(d) as s:
        for b in range(len(o.psi)):
            s.set_psi("theta", b, o.psi[b])
        o.forward_legendre_transform()
        s.apply("forward_legendre")
        for b in range(len(o.psi)):
            assert rel(s.get_psi("j", b), o.lpsi[b]) < 3e-6
            s.set_psi("j", b, o.lpsi[b])   # restart the next stage from the exact state
        o.forward_fft(); o.evolution_with_kinetic(cfg.dt); ke = o.kinetic_energy(); o.backward_fft()
        s.apply("fft_kinetic", cfg.dt)
        for b in range(len(o.psi)):
            assert rel(s.get_psi("j", b), o.lpsi[b]) < 3e-6
            s.set_psi("j", b, o.lpsi[b])
        np.testing.assert_allclose(s.energies()[:, 2], ke, rtol=1e-5)
        o.backward_legendre_transform()
        s.apply("backward_legendre")
        s.apply("energies")
        for b in range(len(o.psi)):
            assert rel(s.get_psi("theta", b), o.psi[b]) < 3e-6
        np.testing.assert_allclose(s.energies()[:, 0], o.module(), rtol=1e-5)
        np.testing.assert_allclose(s.energies()[:, 1], o.potential_energy(), rtol=1e-5, atol=1e-12)


@pytest.mark.parametrize("J", [28, 40])
@pytest.mark.parametrize("prec", [0, 1])
def test_large_coriolis_groups(qd, oracle, gpu, J, prec):
    """29 and 41 coupled Omega blocks: the FP64 Coriolis variants for 25-32 and 33-48 blocks with
    complex128 (FP64 form) and complex64 (mixed form) storage, four full steps against the oracle."""
    cfg, d, dref = make(qd, J=J, parity=0, n1=16, n2=8, n_theta=44, l_max=42, steps=4)
    assert len(np.ravel(d["OmegaStates"]["omegas"])) == J + 1
    d["options"]["precision"] = prec
    o = oracle.Oracle(dref)
    o.run(cfg.total_steps)
    qd.cudaOpenMPEvolution(d)
    assert rel(d["OmegaStates"]["wave_packets"], o.wave_packets()) < (1e-12 if prec == 0 else 1e-5)


def test_mixed_production_grid_tracks_fp64(qd, gpu):
    """256x128x96: 40 steps of the mixed form stay within 1e-5 of the FP64 form; norm drift <= 1e-6."""
    cfg = qd.inputs.CONFIGS["fh2_j0_256x128x96"]
    out = {}
    for prec in (0, 1):
        d = qd.inputs.build_fh2data(cfg)
        d["time"]["total_steps"] = 40
        d["options"]["precision"] = prec
        d["options"]["energies"] = np.zeros((40, 1, 6))
        qd.cudaOpenMPEvolution(d)
        out[prec] = d
    a, b = out[1]["OmegaStates"]["wave_packets"], out[0]["OmegaStates"]["wave_packets"]
    assert rel(a, b) < 1e-5
    ma, mb = out[1]["options"]["energies"][:, 0, 0], out[0]["options"]["energies"][:, 0, 0]
    assert np.max(np.abs(ma - mb)) < 1e-6


def test_mixed_coupled_norm_tracks_fp64(qd, gpu):
    """J=4 (five coupled Omega blocks) on a 64x32x24 grid: 400 steps of the mixed form, whose
    Coriolis step runs in FP32, keep the module within 2e-6 of the FP64 form at every step
    (no systematic drift) and the wave packet within 1e-4."""
    cfg = qd.inputs.small_config(J=4, parity=0, n1=64, n2=32, n_theta=24, l_max=23, steps=400, n_energies=16)
    out = {}
    for prec in (0, 1):
        d = qd.inputs.build_fh2data(cfg)
        d["options"]["precision"] = prec
        d["options"]["energies"] = np.zeros((cfg.total_steps, len(np.ravel(d["OmegaStates"]["omegas"])), 6))
        qd.cudaOpenMPEvolution(d)
        out[prec] = d
    m1 = out[1]["options"]["energies"][:, :, 0].sum(axis=1)
    m0 = out[0]["options"]["energies"][:, :, 0].sum(axis=1)
    assert np.max(np.abs(m1 - m0)) < 2e-6
    assert rel(out[1]["OmegaStates"]["wave_packets"], out[0]["OmegaStates"]["wave_packets"]) < 1e-4


def test_snapshot_callback_writes_copied_packets(qd, gpu, tmp_path):
    """The headless snapshot callback receives the copied wave packets (steps 0, 2 of 4)."""
    cfg, d, _ = make(qd, J=0, n1=32, n2=16, n_theta=8, l_max=6, steps=4)
    d["options"]["wave_to_matlab"] = "PlotPotWave.m"
    d["options"]["steps_to_copy_psi_from_device_to_host"] = 2
    d["options"]["precision"] = 1
    qd.cudaOpenMPEvolution(d, callback=qd.snapshots.snapshot_callback(tmp_path))
    names = sorted(p.name for p in tmp_path.iterdir())
    assert names == ["density_000000.pgm", "density_000002.pgm", "psi_000000.npy", "psi_000002.npy"]
    psi2 = np.load(tmp_path / "psi_000002.npy")
    assert psi2.shape == d["OmegaStates"]["wave_packets"].shape and np.isfinite(psi2).all()
    assert qd.snapshots.read_pgm(tmp_path / "density_000002.pgm").max() == 255
