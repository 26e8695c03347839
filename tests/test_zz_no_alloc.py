"""The allocation-free rotational-energy call against the session's reduction.

qd_rotational_energy_noalloc is for callers that cannot call cudaMalloc (their
device memory is owned by another allocator, here PyTorch's caching pool): they
pass their own device input and output buffers, and the library uses a fixed
scratch array of its own.  It must agree with the rotational energy that the
session computes (with scratch it allocates) for the same Legendre-space
wavepacket, on two calls in a row (the shared scratch keeps the last call's
contents).  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_rotational_energy_noalloc_matches_session(qd, lib):
    torch = pytest.importorskip("torch")
    cfg = qd.inputs.small_config(J=2, parity=0, n1=32, n2=16, n_theta=10, l_max=9, steps=1)
    d = qd.inputs.build_fh2data(cfg)
    rng = np.random.default_rng(5)
    r1, r2 = d["r1"], d["r2"]
    with qd.Session(d) as s:
        for block, omega in enumerate(s.block_omegas):
            shape = (s.l_max - omega + 1, s.n2, s.n1)
            psi = (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) * 0.01
            s.set_psi("j", block, psi)
            s.apply("energies")
            ref = s.energies()[block, 3]
            dev_psi = torch.from_numpy(psi).to("cuda")
            out = torch.zeros(1, dtype=torch.float64, device="cuda")
            for call in range(2):
                st = lib.qd_rotational_energy_noalloc(
                    C.c_void_p(dev_psi.data_ptr()), s.n1, s.n2, omega, s.l_max,
                    float(r1["left"]), float(r1["dr"]), float(r1["mass"]),
                    float(r2["left"]), float(r2["dr"]), float(r2["mass"]),
                    C.c_void_p(out.data_ptr()), None)
                assert st == 0, lib.qd_last_error().decode()
                torch.cuda.synchronize()
                got = float(out.item())
                assert got == pytest.approx(ref, rel=1e-12), (block, call, got, ref)
                out.zero_()


def test_rotational_energy_noalloc_rejects_oversize(qd, lib):
    torch = pytest.importorskip("torch")
    buf = torch.zeros(2, dtype=torch.float64, device="cuda")
    st = lib.qd_rotational_energy_noalloc(C.c_void_p(buf.data_ptr()), 2, 2, 0, 5000, 0.5, 0.1, 1.0, 0.5, 0.1, 1.0,
                                          C.c_void_p(buf.data_ptr()), None)
    assert st == 1
    assert "exceed the fixed scratch" in lib.qd_last_error().decode()
