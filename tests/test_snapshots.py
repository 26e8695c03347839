"""Headless snapshot callback (the stand-in for the reference's plotting script)."""
import numpy as np


def test_snapshot_files(qd, tmp_path):
    cfg = qd.inputs.small_config(J=2, parity=0, n1=32, n2=16, n_theta=8, l_max=6)
    d = qd.inputs.build_fh2data(cfg)
    d["time"]["steps"] = np.int32(12)
    cb = qd.snapshots.snapshot_callback(tmp_path)
    assert cb(d) == 0
    psi = np.load(tmp_path / "psi_000012.npy")
    np.testing.assert_array_equal(psi, d["OmegaStates"]["wave_packets"])
    img = qd.snapshots.read_pgm(tmp_path / "density_000012.pgm")
    rho = qd.snapshots.density(d)
    assert img.shape == (cfg.n2, cfg.n1) and img.dtype == np.uint8
    assert img.max() == 255 and np.unravel_index(img.argmax(), img.shape) == np.unravel_index(rho.argmax(), rho.shape)
    # the density integrates to the module: dr1 dr2 sum rho = sum_Omega <psi|psi>
    dV = d["r1"]["dr"] * d["r2"]["dr"]
    w = d["theta"]["w"]
    mod = dV * sum(np.einsum("k,kji->", w, np.abs(p) ** 2) for p in d["OmegaStates"]["wave_packets"])
    np.testing.assert_allclose(dV * rho.sum(), mod, rtol=1e-12)


def test_pgm_round_trip(qd, tmp_path):
    a = np.arange(12.0).reshape(3, 4)
    qd.snapshots.write_pgm(tmp_path / "a.pgm", a, vmax=11.0)
    g = qd.snapshots.read_pgm(tmp_path / "a.pgm")
    np.testing.assert_array_equal(g, np.rint(255 * a / 11.0).astype(np.uint8))
