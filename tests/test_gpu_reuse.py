"""Reuse of the device state between qd_evolve calls of the same shape.

A call parks its session; the next call with the same grids, time step, precision,
Omega lists and flux surface reloads only its own inputs into it, and rebuilds the
tables whose inputs changed (potential compared on the device, masks, weights and
Legendre matrices on the host).  Every result must equal, bit for bit, that of a
fresh session on the same inputs.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(qd, cfg, prec, modify=None, record=False):
    d = qd.inputs.build_fh2data(cfg)
    d["options"]["precision"] = prec
    if modify:
        modify(d)
    if record:
        nb = len(np.ravel(d["OmegaStates"]["omegas"]))
        d["options"]["energies"] = np.zeros((cfg.total_steps, nb, 6))
    qd.cudaOpenMPEvolution(d)
    return d


def _same(a, b):
    assert np.array_equal(a["OmegaStates"]["wave_packets"], b["OmegaStates"]["wave_packets"])
    assert np.array_equal(a["CRP"]["CRP"], b["CRP"]["CRP"])
    assert int(a["time"]["steps"]) == int(b["time"]["steps"])


def _deeper_pot(d):
    d["pot"] = np.ascontiguousarray(d["pot"] * 1.01)


def _other_masks(d):
    d["dump1"]["dump"] = np.ascontiguousarray(d["dump1"]["dump"] ** 2)


@pytest.mark.parametrize("prec", [0, 1], ids=["fp64", "mixed"])
def test_reused_session_equals_fresh_session(qd, lib, prec):
    # 70 steps: step 0, one 64-step graph chunk and five single steps
    cfg = qd.inputs.small_config(J=2, parity=0, n1=32, n2=16, n_theta=8, l_max=6, steps=70, n_energies=8)
    fresh = {}
    for name, mod, rec in (("pot", _deeper_pot, True), ("mask", _other_masks, False), ("same", None, False)):
        qd.release_session_cache()
        fresh[name] = _run(qd, cfg, prec, mod, rec)
    qd.release_session_cache()
    _same(_run(qd, cfg, prec), fresh["same"])          # parks a session
    b = _run(qd, cfg, prec, _deeper_pot, True)           # another potential, energies recorded
    _same(b, fresh["pot"])
    assert np.array_equal(b["options"]["energies"], fresh["pot"]["options"]["energies"])
    _same(_run(qd, cfg, prec, _other_masks), fresh["mask"])
    _same(_run(qd, cfg, prec), fresh["same"])            # and back to the first inputs
    qd.release_session_cache()


def test_reuse_resumes_across_calls(qd, lib):
    """time.steps and the flux accumulators carried over two calls on one kept session
    equal one call of twice the steps."""
    cfg = qd.inputs.small_config(J=0, n1=32, n2=16, n_theta=8, l_max=6, steps=80, n_energies=8)
    qd.release_session_cache()
    whole = _run(qd, cfg, 1)
    d = qd.inputs.build_fh2data(cfg)
    d["options"]["precision"] = 1
    d["time"]["total_steps"] = 40
    d["CRP"]["accumulators"] = np.zeros((1, 2, 8, cfg.n_theta, cfg.n1), np.complex128)
    qd.cudaOpenMPEvolution(d)
    qd.cudaOpenMPEvolution(d)
    assert int(d["time"]["steps"]) == 80
    assert np.linalg.norm(d["OmegaStates"]["wave_packets"] - whole["OmegaStates"]["wave_packets"]) <= \
        1e-6 * np.linalg.norm(whole["OmegaStates"]["wave_packets"])
    qd.release_session_cache()


@pytest.mark.parametrize("grid", [(256, 128, 7), (192, 96, 7)])
def test_every_fft_candidate_matches_oracle(qd, oracle, lib, tmp_path, grid):
    """Each FFT kernel the autotuner may pick for a production grid, forced through the
    autotune cache file, gives the FP32-level FFT-kinetic stage (rel <= 3e-6 of the oracle)."""
    import re
    n1, n2, l_max = grid
    cfg = qd.inputs.small_config(J=0, n1=n1, n2=n2, n_theta=l_max + 1, l_max=l_max, steps=1, n_energies=8)
    d = qd.inputs.build_fh2data(cfg)
    d["options"]["precision"] = 1
    first = tmp_path / "tuned.txt"
    d["options"]["autotune_cache"] = str(first)
    with qd.Session(d) as s:
        text = s.tuning()
    key = first.read_text().splitlines()[0].split("\t")[0]
    ids = sorted(set(int(x) for x in re.findall(r"\[(\d+)\] =", text)))
    assert len(ids) >= 3, text
    rng = np.random.default_rng(3)
    for c in ids:
        forced = tmp_path / f"forced_{c}.txt"
        forced.write_text(f"{key}\t{c}\t1.0\n")
        d = qd.inputs.build_fh2data(cfg)
        d["options"]["precision"] = 1
        d["options"]["autotune_cache"] = str(forced)
        o = oracle.Oracle(qd.inputs.build_fh2data(cfg))
        lp = (rng.standard_normal(o.lpsi[0].shape) + 1j * rng.standard_normal(o.lpsi[0].shape)) * 1e-2
        o.lpsi[0] = lp.copy()
        with qd.Session(d) as s:
            assert f"[{c}] (cached" in s.tuning(), s.tuning()
            s.set_psi("j", 0, lp)
            s.apply("fft_kinetic", cfg.dt)
            got = s.get_psi("j", 0)
        o.forward_fft(); o.evolution_with_kinetic(cfg.dt); o.backward_fft()
        err = np.linalg.norm(got - o.lpsi[0]) / np.linalg.norm(o.lpsi[0])
        assert err < 3e-6, (c, err)


@pytest.mark.parametrize("prec", [0, 1], ids=["fp64", "mixed"])
def test_zero_step_call_on_kept_session(qd, lib, prec):
    """A call of zero steps on a kept session returns P(E) = 0: the accumulators the earlier
    call left on the device are not read (the first transform of a call writes them, and
    P(E) of accumulators no transform has written is zero), and psi comes back as it went
    in (exactly in the FP64 form, rounded to c64 once in the mixed form, where values below
    the smallest normal FP32 number become zero)."""
    cfg = qd.inputs.small_config(J=0, n1=32, n2=16, n_theta=8, l_max=6, steps=20, n_energies=8)
    qd.release_session_cache()
    first = _run(qd, cfg, prec)
    assert np.abs(first["CRP"]["CRP"]).max() > 0
    d = qd.inputs.build_fh2data(cfg)
    d["options"]["precision"] = prec
    d["time"]["total_steps"] = 0
    psi0 = d["OmegaStates"]["wave_packets"].copy()
    qd.cudaOpenMPEvolution(d)
    assert int(d["time"]["steps"]) == 0
    assert np.array_equal(d["CRP"]["CRP"], np.zeros_like(d["CRP"]["CRP"]))
    if prec == 0:
        assert np.array_equal(d["OmegaStates"]["wave_packets"], psi0)
    else:
        def narrow(x):
            return np.where(np.abs(x) < 2.0 ** -126, 0.0, x.astype(np.float32).astype(np.float64))
        c64 = narrow(psi0.real) + 1j * narrow(psi0.imag)
        assert np.array_equal(d["OmegaStates"]["wave_packets"], c64)
    qd.release_session_cache()
