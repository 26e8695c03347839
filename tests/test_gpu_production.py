"""Both forms against the FP64 oracle at the production configurations.

* 256x128x96, J=0 (one Omega block, l_max = 95): 5 steps.
* 256x128x96, J=12, p=+ (13 Coriolis-coupled Omega blocks, the cudaOpenMP2.cu:392-423
  path): 3 steps.
* A sample of the batched J = 0..40 partial waves on 192x96x80 (l_max = 79, Omega =
  0..min(J, 20)): J = 0, 7, 20, 33, 40, 72 Omega blocks stepped together through
  qd_evolve_batch, 2 steps.

Tolerances: FP64 form, relative L2 error of psi <= 1e-12, module, potential, kinetic
and rotational energies to 1e-10 relative, Coriolis energy to 1e-8; mixed form psi
<= 1e-5 relative, module and energies to 1e-5 of their largest magnitude.  P(E) inside the
initial packet's energy window: FP64 within 1e-8 absolute, mixed within 1e-4 (the
spec gates).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PRODUCTION = {
    "j0": ("fh2_j0_256x128x96", 5),
    "j12": ("fh2_j12_256x128x96", 3),
}
BATCH_J = (0, 7, 20, 33, 40)


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(np.asarray(b)), 1e-300))


@pytest.fixture(scope="module")
def reference_runs():
    return {}


def _oracle(qd, oracle, cache, key, cfgs, steps):
    """Oracle wave packets, energy records and P(E) of each config (cached per module)."""
    if key not in cache:
        out = []
        for c in cfgs:
            o = oracle.Oracle(qd.inputs.build_fh2data(c))
            rec = o.run(steps)
            out.append((o.wave_packets(), rec, o.crp()))
        cache[key] = out
    return cache[key]


def _check(qd, d, ref, prec):
    wp, rec, crp = ref
    tol = 1e-12 if prec == 0 else 1e-5
    err = rel(d["OmegaStates"]["wave_packets"], wp)
    assert err < tol, f"relative |dpsi| {err:.3e}"
    e = d["options"]["energies"]
    if prec == 0:
        np.testing.assert_allclose(e[:, :, :4], rec[:, :, :4], rtol=1e-10, atol=1e-15)
        np.testing.assert_allclose(e[:, :, 4], rec[:, :, 4], rtol=1e-8, atol=1e-14)
    else:
        # FP32 wave packets: the module to 1e-5 of the largest module, every energy
        # (potential, kinetic, rotational, Coriolis) to 1e-5 of the largest energy
        np.testing.assert_allclose(e[:, :, 0], rec[:, :, 0], rtol=1e-5, atol=1e-5 * np.abs(rec[:, :, 0]).max())
        escale = np.abs(rec[:, :, 1:5]).max()
        np.testing.assert_allclose(e[:, :, 1:5], rec[:, :, 1:5], rtol=1e-5, atol=1e-5 * escale)
    win = qd.inputs.energy_window(d["CRP"]["eta_sq"])
    dp = float(np.max(np.abs(d["CRP"]["CRP"] - crp)[win]))
    assert dp <= (1e-8 if prec == 0 else 1e-4), f"|dP(E)| in the window {dp:.3e}"


def _prepare(qd, cfg, prec, steps):
    d = qd.inputs.build_fh2data(cfg)
    d["time"]["total_steps"] = steps
    d["options"]["precision"] = prec
    nb = len(np.ravel(d["OmegaStates"]["omegas"]))
    d["options"]["energies"] = np.zeros((steps, nb, 6))
    return d


@pytest.mark.parametrize("prec", [0, 1], ids=["fp64", "mixed"])
@pytest.mark.parametrize("case", list(PRODUCTION))
def test_production_config_matches_oracle(qd, oracle, lib, reference_runs, case, prec):
    """One problem at 256x128x96 through qd_evolve (cudaOpenMP2.cu:338-386 step order)."""
    name, steps = PRODUCTION[case]
    cfg = qd.inputs.CONFIGS[name]
    ref = _oracle(qd, oracle, reference_runs, case, [cfg], steps)[0]
    d = _prepare(qd, cfg, prec, steps)
    qd.cudaOpenMPEvolution(d)
    assert int(d["time"]["steps"]) == steps
    _check(qd, d, ref, prec)


@pytest.mark.parametrize("prec", [0, 1], ids=["fp64", "mixed"])
def test_batched_partial_waves_sample_matches_oracle(qd, oracle, lib, reference_runs, prec):
    """J = 0, 7, 20, 33, 40 of the batched configuration, stepped together (qd_evolve_batch)."""
    steps = 2
    cfgs = [c for c in qd.inputs.batched_partial_waves() if c.J in BATCH_J]
    refs = _oracle(qd, oracle, reference_runs, "batch", cfgs, steps)
    ds = [_prepare(qd, c, prec, steps) for c in cfgs]
    assert sum(len(np.ravel(d["OmegaStates"]["omegas"])) for d in ds) == 72
    qd.evolve_batch(ds)
    for d, ref in zip(ds, refs):
        assert int(d["time"]["steps"]) == steps
        _check(qd, d, ref, prec)


def test_mixed_pe_gate_at_production_grid(qd, lib):
    """The spec gate of the mixed form: 256x128x96, J=0, 2000 steps of both forms on the
    GPU; max |P_mixed(E) - P_fp64(E)| <= 1e-4 in the energy window, module within 1e-5, and a
    propagated flux (max P in the window above 0.1) so that the comparison is not vacuous."""
    cfg = qd.inputs.CONFIGS["fh2_j0_256x128x96"]
    out = {}
    for prec in (0, 1):
        d = qd.inputs.build_fh2data(cfg)
        d["time"]["total_steps"] = 2000
        d["options"]["precision"] = prec
        d["options"]["energies"] = np.zeros((2000, 1, 6))
        qd.cudaOpenMPEvolution(d)
        out[prec] = d
    win = qd.inputs.energy_window(out[0]["CRP"]["eta_sq"])
    pf, pm = out[0]["CRP"]["CRP"][win], out[1]["CRP"]["CRP"][win]
    assert np.abs(pf).max() > 0.1
    assert np.max(np.abs(pm - pf)) <= 1e-4
    mf, mm = out[0]["options"]["energies"][:, 0, 0], out[1]["options"]["energies"][:, 0, 0]
    assert np.max(np.abs(mm - mf)) <= 1e-5


@pytest.mark.parametrize("prec", [0, 1], ids=["fp64", "mixed"])
def test_woods_saxon_masks_match_oracle(qd, oracle, lib, prec):
    """The reference's own absorbing masks (Woods-Saxon, FH2main.m:97-99,113-115) through the
    dump1/dump2 mechanism (evolutionCUDAaux.cu:243-251), J=2 on 64x32x24, 20 steps."""
    cfg = qd.inputs.small_config(J=2, parity=0, n1=64, n2=32, n_theta=24, l_max=23, steps=20,
                                 n_energies=32, mask="woods_saxon")
    d = qd.inputs.build_fh2data(cfg)
    assert d["dump1"]["dump"][0] > 0.999 and d["dump1"]["dump"][-1] < 1e-2
    d["options"]["precision"] = prec
    o = oracle.Oracle(qd.inputs.build_fh2data(cfg))
    o.run(cfg.total_steps)
    qd.cudaOpenMPEvolution(d)
    assert rel(d["OmegaStates"]["wave_packets"], o.wave_packets()) < (1e-12 if prec == 0 else 1e-5)
