"""The MATLAB MEX shim (qd_mex.c) without MATLAB.

The shim is compiled against a stand-in of MATLAB's MEX header (tests/mex/mex.h, the
documented calls it uses) and run on a minimal MEX runtime (tests/mex/fake_mex.c): an
FH2main.m-shaped struct goes through mexFunction, MATLAB scripts are Python callbacks,
and mexErrMsgTxt unwinds with longjmp as MATLAB does.  On the CPU the shim is linked with
a stand-in of qd_evolve (tests/mex/stub_qd.c) that follows libqd's host contract; the GPU
test links it with libqd itself.  What is checked is the drop-in behaviour of the
reference's entry point (cudaOpenMPEvolution.C:15-79):

* the wave_to_matlab script sees FH2Data.time.steps = 0, N, 2N, ... in MATLAB's own
  memory (bound by reference, matlabStructures.C:42; read by FH2Matlab.m:18) and the
  copied wave packets;
* a MATLAB error inside the script comes back through mexCallMATLABWithTrap, so libqd
  returns normally (its session clean-up runs) and the script's error is raised once;
* malformed structs (missing time.steps, wrong class, short wave_packets) raise an
  insist-style MATLAB error instead of reading or writing out of bounds.
"""
import ctypes as C
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
MEX = ROOT / "tests" / "mex"
SHIM = ROOT / "qd-openmp-cuda_gb300" / "csrc" / "qd_mex.c"
PKG = ROOT / "qd-openmp-cuda_gb300"
mxCHAR, mxDOUBLE, mxINT32 = 4, 6, 12
SCRIPT = C.CFUNCTYPE(C.c_int, C.c_char_p)


def _cc():
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    return cc


def _flags():
    return ["-std=c11", "-D_POSIX_C_SOURCE=200809L", "-Wall", "-Werror", "-I", str(MEX), "-I", str(ROOT / "include")]


def build_shim(tmp: Path, real_library: bool) -> C.CDLL:
    """cudaOpenMPEvolution shim + fake MEX runtime as one shared library."""
    out = tmp / ("shim_gpu.so" if real_library else "shim_stub.so")
    srcs = [str(MEX / "fake_mex.c"), str(SHIM)]
    link = ["-L", str(PKG), "-lqd", f"-Wl,-rpath,{PKG}"] if real_library else [str(MEX / "stub_qd.c")]
    r = subprocess.run([_cc(), *_flags(), "-shared", "-fPIC", "-Wl,-Bsymbolic", *srcs, *link, "-o", str(out)],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    lib = C.CDLL(str(out))
    lib.fm_struct.restype = C.c_void_p
    lib.fm_numeric.restype = C.c_void_p
    lib.fm_numeric.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_size_t), C.c_void_p]
    lib.fm_string.restype = C.c_void_p
    lib.fm_string.argtypes = [C.c_char_p]
    lib.fm_set.argtypes = [C.c_void_p, C.c_char_p, C.c_void_p]
    lib.fm_remove.argtypes = [C.c_void_p, C.c_char_p]
    lib.fm_run.argtypes = [C.c_void_p, C.c_char_p, C.c_size_t]
    lib.fm_set_script_handler.argtypes = [SCRIPT]
    return lib


class MxTree:
    """An FH2Data dict (inputs.build_fh2data) as fake mxArrays borrowing numpy memory."""

    def __init__(self, lib, d: dict, script=None):
        self.lib, self.keep = lib, []
        self.root = self.struct({
            "r1": self.radial(d["r1"]), "r2": self.radial(d["r2"]),
            "theta": self.struct({"n": self.i32(d["theta"]["n"]), "m": self.i32(d["theta"]["m"]),
                                  "x": self.f64(d["theta"]["x"]), "w": self.f64(d["theta"]["w"])}),
            "pot": self.f64(d["pot"], dims=(d["pot"].shape[2], d["pot"].shape[1], d["pot"].shape[0])),
            "time": self.struct({"total_steps": self.i32(d["time"]["total_steps"]),
                                 "time_step": self.f64(d["time"]["time_step"]),
                                 "steps": self.i32(d["time"]["steps"], name="steps")}),
            "options": self.struct({"steps_to_copy_psi_from_device_to_host":
                                    self.i32(d["options"]["steps_to_copy_psi_from_device_to_host"]),
                                    "use_p2p_async": self.i32(0), "test_name": self.text("FH2"),
                                    "precision": self.i32(d["options"].get("precision", 0)),
                                    **({"wave_to_matlab": self.text(script)} if script else {})}),
            "dump1": self.struct({"dump": self.f64(d["dump1"]["dump"])}),
            "dump2": self.struct({"dump": self.f64(d["dump2"]["dump"])}),
            "CRP": self.struct({k: self.i32(d["CRP"][k]) for k in
                                ("n_dividing_surface", "n_gradient_points", "n_energies", "calculate_CRP")} |
                               {"energies": self.f64(d["CRP"]["energies"]), "eta_sq": self.f64(d["CRP"]["eta_sq"]),
                                "CRP": self.f64(d["CRP"]["CRP"], name="CRP")}),
            "OmegaStates": self.omega_states(d["OmegaStates"]),
        })

    def struct(self, fields):
        s = self.lib.fm_struct()
        for k, v in fields.items():
            self.lib.fm_set(s, k.encode(), v)
        return s

    def numeric(self, cls, a, dims):
        self.keep.append(a)
        d = (C.c_size_t * len(dims))(*dims)
        return self.lib.fm_numeric(cls, len(dims), d, a.ctypes.data)

    def i32(self, v, name=None):
        a = np.array([int(v)], dtype=np.int32)
        if name:
            setattr(self, name, a)
        return self.numeric(mxINT32, a, (1, 1))

    def f64(self, v, dims=None, name=None):
        a = np.asarray(v, dtype=np.float64)
        if not (isinstance(v, np.ndarray) and v.dtype == np.float64 and v.flags.c_contiguous):
            a = np.ascontiguousarray(a)
        if name:
            setattr(self, name, a)
        return self.numeric(mxDOUBLE, a, dims or ((a.size, 1) if a.ndim <= 1 else a.shape[::-1]))

    def text(self, s):
        return self.lib.fm_string(s.encode())

    def radial(self, r):
        return self.struct({"n": self.i32(r["n"]), "left": self.f64(r["left"]), "dr": self.f64(r["dr"]),
                            "mass": self.f64(r["mass"])})

    def omega_states(self, om):
        wp = om["wave_packets"]                       # complex (n_Omega, n_theta, n2, n1), in place
        self.wave_packets = wp
        n_om, nth, n2, n1 = wp.shape
        P = np.ascontiguousarray(om["associated_legendres"])   # (n_Omega, n_cols, n_theta)
        omegas = np.ascontiguousarray(om["omegas"], dtype=np.int32)
        self.keep += [wp, P, omegas]
        return self.struct({
            "J": self.i32(om["J"]), "parity": self.i32(om["parity"]), "l_max": self.i32(om["l_max"]),
            "n_omegas_max": self.i32(om["n_omegas_max"]),
            "omegas": self.numeric(mxINT32, omegas, (1, omegas.size)),
            "associated_legendres": self.numeric(mxDOUBLE, P, (P.shape[2], P.shape[1], P.shape[0])),
            "wave_packets": self.numeric(mxDOUBLE, wp, (2 * n1, n2, nth, n_om)),
        })


def run(lib, tree):
    msg = C.create_string_buffer(1024)
    rc = lib.fm_run(tree.root, msg, 1024)
    return rc, msg.value.decode()


def small(qd, steps=7, every=3, **kw):
    cfg = qd.inputs.small_config(J=2, parity=0, n1=16, n2=8, n_theta=8, l_max=6, steps=steps, n_energies=16, **kw)
    d = qd.inputs.build_fh2data(cfg)
    d["options"]["steps_to_copy_psi_from_device_to_host"] = np.int32(every)
    return cfg, d


def test_mex_shim_compiles():
    """qd_mex.c compiles warning-free against the MEX header stand-in and the C ABI header."""
    r = subprocess.run([_cc(), *_flags(), "-fsyntax-only", str(SHIM)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr


def test_mex_callback_sees_live_steps(qd, tmp_path, monkeypatch):
    lib = build_shim(tmp_path, real_library=False)
    monkeypatch.chdir(tmp_path)
    (tmp_path / "FH2Matlab.m").write_text("% plotting script\n")
    _, d = small(qd)
    tree = MxTree(lib, d, script="FH2Matlab.m")
    seen = []

    @SCRIPT
    def script(name):
        seen.append((name.decode(), int(tree.steps[0]), float(tree.wave_packets.reshape(-1)[0].real)))
        return 0

    lib.fm_set_script_handler(script)
    rc, msg = run(lib, tree)
    assert rc == 0, msg
    assert seen == [("FH2Matlab", 0, 1.0), ("FH2Matlab", 3, 4.0), ("FH2Matlab", 6, 7.0)]
    assert int(tree.steps[0]) == 7
    assert lib.fm_errors() == 0 and lib.fm_live_strings() == 0
    assert lib.stub_live_sessions() == 0


def test_mex_script_error_is_trapped(qd, tmp_path, monkeypatch):
    lib = build_shim(tmp_path, real_library=False)
    monkeypatch.chdir(tmp_path)
    (tmp_path / "FH2Matlab.m").write_text("% plotting script\n")
    _, d = small(qd)
    tree = MxTree(lib, d, script="FH2Matlab")
    calls = []

    @SCRIPT
    def script(name):
        calls.append(int(tree.steps[0]))
        return 1 if len(calls) == 2 else 0

    lib.fm_set_script_handler(script)
    rc, msg = run(lib, tree)
    assert rc == 1 and msg == "error in script FH2Matlab"
    assert calls == [0, 3]
    assert lib.fm_errors() == 1 and lib.fm_rethrows() == 1
    assert lib.stub_live_sessions() == 0          # libqd returned normally: no unwinding through it
    assert lib.fm_live_strings() == 0             # script name and test name freed
    assert int(tree.steps[0]) == 4                # steps done, written back in place


def test_mex_script_absent_is_skipped(qd, tmp_path, monkeypatch):
    """wavepacket_to_matlab runs the script only if script.m exists (wave2matlab.C:19-26)."""
    lib = build_shim(tmp_path, real_library=False)
    monkeypatch.chdir(tmp_path)
    _, d = small(qd)
    tree = MxTree(lib, d, script="FH2Matlab")
    seen = []

    @SCRIPT
    def script(name):
        seen.append(name)
        return 0

    lib.fm_set_script_handler(script)
    rc, msg = run(lib, tree)
    assert rc == 0, msg
    assert seen == [] and int(tree.steps[0]) == 7


@pytest.mark.parametrize("defect", ["no_steps", "steps_double", "short_packets", "short_pot"])
def test_mex_rejects_malformed_struct(qd, tmp_path, defect):
    lib = build_shim(tmp_path, real_library=False)
    _, d = small(qd)
    tree = MxTree(lib, d)
    lib.mxGetField.restype = C.c_void_p
    lib.mxGetField.argtypes = [C.c_void_p, C.c_size_t, C.c_char_p]
    time_s = lib.mxGetField(tree.root, 0, b"time")
    om = lib.mxGetField(tree.root, 0, b"OmegaStates")
    if defect == "no_steps":
        lib.fm_remove(time_s, b"steps")
        expect = "insist failed: field steps"
    elif defect == "steps_double":
        lib.fm_set(time_s, b"steps", tree.f64(0.0))
        expect = "insist failed: class of field steps"
    elif defect == "short_packets":
        short = np.zeros(10)
        lib.fm_set(om, b"wave_packets", tree.numeric(mxDOUBLE, short, (10, 1)))
        expect = "insist failed: size of field wave_packets"
    else:
        lib.fm_set(tree.root, b"pot", tree.f64(np.zeros(5)))
        expect = "insist failed: size of field pot"
    rc, msg = run(lib, tree)
    assert rc == 1 and msg.startswith(expect), msg
    assert lib.stub_live_sessions() == 0


@pytest.mark.gpu
def test_mex_shim_on_libqd_matches_python_binding(qd, lib, tmp_path, monkeypatch):
    """FH2main.m-shaped struct through mexFunction and libqd on the GPU: the script sees the
    copied wave packets at steps 0, 2, 4 and the final state and P(E) equal those of the
    same run through the Python binding."""
    shim = build_shim(tmp_path, real_library=True)
    monkeypatch.chdir(tmp_path)
    (tmp_path / "FH2Matlab.m").write_text("% plotting script\n")
    _, d = small(qd, steps=5, every=2)
    tree = MxTree(shim, d, script="FH2Matlab")
    seen = []

    @SCRIPT
    def script(name):
        seen.append((int(tree.steps[0]), tree.wave_packets.copy()))
        return 0

    shim.fm_set_script_handler(script)
    rc, msg = run(shim, tree)
    assert rc == 0, msg
    assert int(tree.steps[0]) == 5
    _, ref = small(qd, steps=5, every=2)
    ref["options"]["wave_to_matlab"] = "FH2Matlab"
    ref_seen = []
    qd.cudaOpenMPEvolution(ref, callback=lambda data: ref_seen.append(
        (int(data["time"]["steps"]), data["OmegaStates"]["wave_packets"].copy())) or 0)
    assert [s for s, _ in seen] == [s for s, _ in ref_seen] == [0, 2, 4]
    for (_, a), (_, b) in zip(seen, ref_seen):
        assert np.array_equal(a, b)
    assert np.array_equal(tree.wave_packets, ref["OmegaStates"]["wave_packets"])
    assert np.array_equal(tree.CRP, ref["CRP"]["CRP"])
