"""Failure detection on the GPU without a fault: the bounded device-side wait.

Every wait in the library's pipelined kernels (the tensor-core contractions'
mbarrier hand-offs) gives up after its budget and records QD_ERR_TIMEOUT in the
device status word, which the host turns into an error; nothing traps or spins
forever.  qd_device_wait_selftest runs that same wait on an mbarrier that nothing
arrives at (a flag that nothing sets), with a short budget.
"""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_bounded_wait_gives_up_with_timeout_status(qd, lib):
    t0 = time.perf_counter()
    with pytest.raises(qd.QDError) as e:
        qd.device_wait_selftest(20.0, arrive=False)
    assert e.value.status == 8                       # QD_ERR_TIMEOUT
    assert "gave up" in str(e.value)
    assert time.perf_counter() - t0 >= 0.02          # it waited its whole budget ...
    qd.device_wait_selftest(20.0, arrive=True)       # ... and a wait that is satisfied returns


def test_context_usable_after_a_timeout(qd, oracle, lib):
    with pytest.raises(qd.QDError):
        qd.device_wait_selftest(5.0, arrive=False)
    cfg = qd.inputs.small_config(J=2, parity=0, n1=16, n2=8, n_theta=8, l_max=6, steps=3, n_energies=8)
    d = qd.inputs.build_fh2data(cfg)
    d["options"]["precision"] = 1
    qd.cudaOpenMPEvolution(d)
    o = oracle.Oracle(qd.inputs.build_fh2data(cfg))
    o.run(cfg.total_steps)
    ref = o.wave_packets()
    assert np.linalg.norm(d["OmegaStates"]["wave_packets"] - ref) / np.linalg.norm(ref) < 1e-5
