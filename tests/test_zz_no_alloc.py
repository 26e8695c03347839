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


def _rot_energy_numpy(psi, omega, r1, r2):
    """dr1 dr2 sum_l l(l+1) sum (1/(2 m1 R^2) + 1/(2 m2 r^2)) |psi_l|^2 in FP64 on the host."""
    n_l, n2, n1 = psi.shape
    R = r1["left"] + np.arange(n1) * r1["dr"]
    r = r2["left"] + np.arange(n2) * r2["dr"]
    inertia = 1.0 / (2 * r2["mass"] * r[:, None] ** 2) + 1.0 / (2 * r1["mass"] * R[None, :] ** 2)
    l = omega + np.arange(n_l, dtype=np.float64)
    per_l = np.sum(np.abs(psi) ** 2 * inertia[None], axis=(1, 2))
    return float(np.sum(l * (l + 1) * per_l) * r1["dr"] * r2["dr"])


def _call(lib, torch, psi, omega, r1, r2):
    dev = torch.from_numpy(np.ascontiguousarray(psi)).to("cuda")
    out = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
    n_l, n2, n1 = psi.shape
    st = lib.qd_rotational_energy_noalloc(C.c_void_p(dev.data_ptr()), n1, n2, omega, omega + n_l - 1,
                                          r1["left"], r1["dr"], r1["mass"], r2["left"], r2["dr"], r2["mass"],
                                          C.c_void_p(out.data_ptr()), None)
    torch.cuda.synchronize()
    return st, float(out.item())


def test_rotational_energy_noalloc_limit_and_stale_partials(lib):
    """The scratch limit is exact: 4096 slabs (2x2 grid) are accepted and summed correctly,
    4097 are rejected.  A small call after the largest one reads none of the larger call's
    leftover partial sums."""
    torch = pytest.importorskip("torch")
    r1 = {"left": 0.5, "dr": 0.25, "mass": 3321.0}
    r2 = {"left": 0.6, "dr": 0.125, "mass": 918.6}
    rng = np.random.default_rng(9)
    big = (rng.standard_normal((4096, 2, 2)) + 1j * rng.standard_normal((4096, 2, 2))) * 1e-3
    st, got = _call(lib, torch, big, 0, r1, r2)
    assert st == 0, lib.qd_last_error().decode()
    assert got == pytest.approx(_rot_energy_numpy(big, 0, r1, r2), rel=1e-12)
    small = (rng.standard_normal((3, 2, 2)) + 1j * rng.standard_normal((3, 2, 2))) * 1e-3
    for _ in range(2):
        st, got = _call(lib, torch, small, 5, r1, r2)
        assert st == 0, lib.qd_last_error().decode()
        assert got == pytest.approx(_rot_energy_numpy(small, 5, r1, r2), rel=1e-12)
    over = np.zeros((4097, 2, 2), np.complex128)
    st, _ = _call(lib, torch, over, 0, r1, r2)
    assert st == 1
    assert "exceed the fixed scratch" in lib.qd_last_error().decode()
