"""Input builders (the reference's MATLAB front end restated): masks and the batched run."""
import numpy as np


def test_woods_saxon_mask_matches_reference_formula(qd):
    """1/(1 + exp(Cd (x - xd))) (cudaMath.h:159-162) with FH2main.m's Cd = 4, xd = 12 / 10."""
    cfg = qd.inputs.small_config(n1=64, n2=32, n_theta=8, l_max=6, mask="woods_saxon")
    d = qd.inputs.build_fh2data(cfg)
    R, r = d["r1"]["r"], d["r2"]["r"]
    np.testing.assert_allclose(d["dump1"]["dump"], 1.0 / (1.0 + np.exp(4.0 * (R - 12.0))), rtol=1e-15)
    np.testing.assert_allclose(d["dump2"]["dump"], 1.0 / (1.0 + np.exp(4.0 * (r - 10.0))), rtol=1e-15)
    assert qd.inputs.woods_saxon(np.array([1e4]), 4.0, 10.0)[0] == 0.0   # no overflow warning path


def test_batched_partial_waves_have_651_blocks(qd):
    """J = 0..40 with Omega = 0..min(J, 20): parity p = J mod 2 makes every J start at Omega = 0."""
    cfgs = qd.inputs.batched_partial_waves()
    lists = [qd.inputs.omega_list(c.J, c.parity, c.l_max, c.omega_cap) for c in cfgs]
    assert all(ls[0] == 0 for ls in lists)
    assert [len(ls) for ls in lists] == [min(J, 20) + 1 for J in range(41)]
    assert sum(len(ls) for ls in lists) == 651


def test_energy_window(qd):
    eta = np.array([1e-12, 1e-5, 0.5, 1.0, 2e-4])
    assert qd.inputs.energy_window(eta).tolist() == [False, False, True, True, True]
