"""Host-side checks that need no GPU: the C ABI exports, input validation."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def test_library_exports_every_declared_symbol(lib):
    header = (ROOT / "include" / "qd.h").read_text()
    names = re.findall(r"^\s*(?:int|const char \*|void \*)\s*(qd_\w+)\s*\(", header, flags=re.M)
    assert len(names) >= 16
    for n in names:
        assert hasattr(lib, n), n
    assert lib.qd_version() == 10000


def test_python_bindings_cover_the_header(qd, lib):
    header = (ROOT / "include" / "qd.h").read_text()
    names = set(re.findall(r"^\s*(?:int|const char \*|void \*)\s*(qd_\w+)\s*\(", header, flags=re.M))
    assert names == set(qd.EXPORTED)


def test_struct_layout_matches_header(qd):
    # offsets that the C compiler would choose on LP64 (x86_64 and aarch64 agree)
    assert C.sizeof(qd.RadialCoordinate) == 32
    assert C.sizeof(qd.EvolutionTime) == 24
    assert qd.FH2Data.OmegaStates.offset > qd.FH2Data.CRP.offset


def _bad(qd, mutate):
    cfg = qd.inputs.small_config()
    d = qd.inputs.build_fh2data(cfg)
    mutate(d)
    with pytest.raises(qd.QDError) as e:
        qd.cudaOpenMPEvolution(d)
    return e.value


@pytest.mark.parametrize("mutate,needle", [
    (lambda d: d["OmegaStates"].__setitem__("parity", 1), "p == 0 when J == 0"),
    (lambda d: d["OmegaStates"].__setitem__("l_max", 9), "theta.n >= l_max + 1"),
    (lambda d: d["OmegaStates"].__setitem__("omegas", np.array([1], np.int32)), "omegas[0]"),
    (lambda d: d["OmegaStates"].__setitem__("n_omegas_max", 0), "n_omegas_max"),
    (lambda d: d["CRP"].__setitem__("n_gradient_points", 4), "odd"),
    (lambda d: d["CRP"].__setitem__("n_dividing_surface", 0), "stencil"),
    (lambda d: d["options"].__setitem__("wave_to_matlab", "FH2Matlab"), "steps_to_copy"),
    (lambda d: d["options"].__setitem__("precision", 7), "precision"),
])
def test_invalid_inputs_are_rejected_before_any_device_work(qd, lib, mutate, needle):
    err = _bad(qd, mutate)
    assert err.status == 1
    assert needle in str(err)


def test_odd_grid_is_unsupported(qd, lib):
    cfg = qd.inputs.small_config()
    d = qd.inputs.build_fh2data(cfg)
    d["r1"]["n"] = 15
    with pytest.raises(qd.QDError) as e:
        qd.cudaOpenMPEvolution(d)
    assert e.value.status == 6


def test_output_arrays_must_be_writable_in_place(qd, lib):
    cfg = qd.inputs.small_config()
    d = qd.inputs.build_fh2data(cfg)
    d["OmegaStates"]["wave_packets"] = d["OmegaStates"]["wave_packets"].astype(np.complex64)
    with pytest.raises(qd.QDError):
        qd.cudaOpenMPEvolution(d)


def test_bench_algorithmic_bytes_of_the_headline(qd):
    """The roofline numerator: algorithmic bytes per launch at 256x128x96, J=0, mixed form
    (8 B per c64 value of psi; forward reads psi_theta and the potential's shear pair and
    writes psi_l, backward reads psi_l and w V and writes psi_theta, the slab FFT reads and
    writes every psi_l value once)."""
    import importlib.util

    spec = importlib.util.spec_from_file_location("bench", Path(__file__).resolve().parents[1] / "bench.py")
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    d = qd.inputs.build_fh2data(qd.inputs.CONFIGS["fh2_j0_256x128x96"])
    d["options"]["precision"] = 1
    npt, nth, nl = 256 * 128, 96, 96
    assert bench.algorithmic("legendre_forward", d) == ("hbm", 8.0 * npt * (nth + nth + nl), "GB/s")
    assert bench.algorithmic("legendre_backward", d) == ("hbm", npt * (8.0 * nl + 8.0 * nth + 4.0 * nth), "GB/s")
    assert bench.algorithmic("fft_slab", d) == ("hbm", 50_331_648.0, "GB/s")
    assert bench.algorithmic("legendre_forward", d)[1] == 75_497_472.0
    assert bench.algorithmic("legendre_backward", d)[1] == 62_914_560.0
