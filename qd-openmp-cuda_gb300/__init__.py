"""GB300 split-operator wavepacket propagator: Python host side.

The product is ``libqd.so`` (CUDA kernels for sm_103a behind the C ABI in
``include/qd.h``).  This module binds it with ctypes and mirrors the
reference's MATLAB entry point ``cudaOpenMPEvolution(FH2Data)``
(``cudaOpenMPEvolution.C:15-79``, called at ``FH2main.m:213``): the same
struct fields, in-place outputs (``OmegaStates.wave_packets``,
``time.steps``, ``CRP.CRP``) and error behaviour (the reference's
``mexErrMsgTxt`` unwinding becomes a :class:`QDError`).

There is no CPU fallback: if the library is missing or no GPU is present the
calls raise.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path
from typing import Callable, List, Optional, Sequence

import numpy as np

from . import inputs  # noqa: F401  (FH2Data builders)
from . import snapshots  # noqa: F401  (headless wave-packet snapshots for the callback)

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "libqd.so"

QD_OK = 0
STATUS_NAMES = {0: "QD_OK", 1: "QD_ERR_INVALID", 2: "QD_ERR_CUDA", 3: "QD_ERR_NOMEM", 4: "QD_ERR_NORM",
                5: "QD_ERR_CALLBACK", 6: "QD_ERR_UNSUPPORTED", 7: "QD_ERR_NO_DEVICE", 8: "QD_ERR_TIMEOUT"}
PRECISION = {"fp64": 0, "mixed": 1}
STAGES = {"dump": 0, "potential": 1, "forward_legendre": 2, "backward_legendre": 3, "rotational": 4,
          "coriolis": 5, "coriolis_energy": 6, "fft_kinetic": 7, "energies": 8, "flux": 9}
ENERGY_FIELDS = ("module", "potential", "kinetic", "rotational", "coriolis", "total")


class QDError(RuntimeError):
    """Raised for every non-zero qd_status; ``status`` holds the code."""

    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


# ----------------------------------------------------------------- structs
class RadialCoordinate(C.Structure):
    _fields_ = [("n", C.c_int32), ("left", C.c_double), ("dr", C.c_double), ("mass", C.c_double)]


class AngleCoordinate(C.Structure):
    _fields_ = [("n", C.c_int32), ("m", C.c_int32), ("x", C.POINTER(C.c_double)), ("w", C.POINTER(C.c_double)),
                ("associated_legendre", C.POINTER(C.c_double))]


class EvolutionTime(C.Structure):
    _fields_ = [("total_steps", C.c_int32), ("time_step", C.c_double), ("steps", C.c_int32)]


class Options(C.Structure):
    _fields_ = [("wave_to_matlab", C.c_char_p), ("test_name", C.c_char_p),
                ("steps_to_copy_psi_from_device_to_host", C.c_int32), ("use_p2p_async", C.c_int32),
                ("precision", C.c_int32), ("print_energies", C.c_int32), ("energies", C.POINTER(C.c_double)),
                ("autotune_cache", C.c_char_p)]


class DumpFunction(C.Structure):
    _fields_ = [("dump", C.POINTER(C.c_double))]


class CRP(C.Structure):
    _fields_ = [("energies", C.POINTER(C.c_double)), ("eta_sq", C.POINTER(C.c_double)),
                ("CRP", C.POINTER(C.c_double)), ("n_dividing_surface", C.c_int32),
                ("n_gradient_points", C.c_int32), ("n_energies", C.c_int32), ("calculate_CRP", C.c_int32),
                ("accumulators", C.POINTER(C.c_double))]


class OmegaStates(C.Structure):
    _fields_ = [("J", C.c_int32), ("parity", C.c_int32), ("l_max", C.c_int32), ("n_omegas_max", C.c_int32),
                ("n_omegas", C.c_int32), ("omegas", C.POINTER(C.c_int32)),
                ("associated_legendres", C.POINTER(C.c_double)), ("n_cols", C.c_int32),
                ("wave_packets", C.POINTER(C.c_double))]


class FH2Data(C.Structure):
    _fields_ = [("r1", RadialCoordinate), ("r2", RadialCoordinate), ("theta", AngleCoordinate),
                ("pot", C.POINTER(C.c_double)), ("psi", C.POINTER(C.c_double)), ("time", EvolutionTime),
                ("options", Options), ("dump1", DumpFunction), ("dump2", DumpFunction), ("CRP", CRP),
                ("OmegaStates", OmegaStates)]


CALLBACK = C.CFUNCTYPE(C.c_int, C.POINTER(FH2Data), C.c_void_p)

_lib = None

EXPORTED = ("qd_evolve", "qd_evolve_batch", "qd_release_session_cache", "qd_last_error", "qd_version", "qd_session_create",
            "qd_session_destroy", "qd_session_run", "qd_session_synchronize", "qd_session_flush", "qd_session_download",
            "qd_session_upload", "qd_session_stream", "qd_session_info", "qd_session_apply", "qd_session_get_psi",
            "qd_session_set_psi", "qd_session_get_energies", "qd_session_profile", "qd_device_fma_peaks",
            "qd_device_wait_selftest", "qd_session_tuning", "qd_device_dmma_peak",
            "qd_rotational_energy_noalloc")


def library_path() -> Path:
    return Path(os.environ.get("QD_LIBRARY", LIB_PATH))


def load_library():
    """Load libqd.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    p = library_path()
    if not p.exists():
        raise QDError(7, f"{p} not built: run build() first")
    lib = C.CDLL(str(p))
    P = C.POINTER
    lib.qd_version.restype = C.c_int
    lib.qd_last_error.restype = C.c_char_p
    lib.qd_evolve.argtypes = [P(FH2Data), CALLBACK, C.c_void_p]
    lib.qd_evolve_batch.argtypes = [P(P(FH2Data)), C.c_int32, CALLBACK, C.c_void_p]
    lib.qd_release_session_cache.argtypes = []
    lib.qd_session_create.argtypes = [P(P(FH2Data)), C.c_int32, P(C.c_void_p)]
    lib.qd_session_destroy.argtypes = [C.c_void_p]
    lib.qd_session_run.argtypes = [C.c_void_p, C.c_int32]
    lib.qd_session_synchronize.argtypes = [C.c_void_p]
    lib.qd_session_flush.argtypes = [C.c_void_p]
    lib.qd_session_download.argtypes = [C.c_void_p, P(P(FH2Data)), C.c_int32]
    lib.qd_session_upload.argtypes = [C.c_void_p, P(P(FH2Data)), C.c_int32]
    lib.qd_session_stream.argtypes = [C.c_void_p]
    lib.qd_session_stream.restype = C.c_void_p
    lib.qd_session_info.argtypes = [C.c_void_p, P(C.c_int32), P(C.c_int32)]
    lib.qd_session_apply.argtypes = [C.c_void_p, C.c_int32, C.c_double]
    lib.qd_session_get_psi.argtypes = [C.c_void_p, C.c_int32, C.c_int32, P(C.c_double), C.c_size_t]
    lib.qd_session_set_psi.argtypes = [C.c_void_p, C.c_int32, C.c_int32, P(C.c_double), C.c_size_t]
    lib.qd_session_get_energies.argtypes = [C.c_void_p, P(C.c_double), C.c_size_t]
    lib.qd_session_profile.argtypes = [C.c_void_p, C.c_int32, C.c_char_p, C.c_size_t, P(C.c_double),
                                       P(C.c_int32), C.c_int32, P(C.c_int32)]
    lib.qd_device_fma_peaks.argtypes = [P(C.c_double), P(C.c_double)]
    lib.qd_device_wait_selftest.argtypes = [C.c_double, C.c_int32]
    lib.qd_session_tuning.argtypes = [C.c_void_p, C.c_char_p, C.c_size_t]
    lib.qd_device_dmma_peak.argtypes = [P(C.c_double)]
    lib.qd_rotational_energy_noalloc.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                                 C.c_double, C.c_double, C.c_double, C.c_double, C.c_double,
                                                 C.c_double, C.c_void_p, C.c_void_p]
    _lib = lib
    return lib


def _check(status: int):
    if status != QD_OK:
        msg = _lib.qd_last_error().decode(errors="replace") if _lib is not None else ""
        raise QDError(status, msg)


def _dptr(a: Optional[np.ndarray]):
    if a is None:
        return C.POINTER(C.c_double)()
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _f64(a) -> np.ndarray:
    a = np.asarray(a)
    if a.dtype != np.float64 or not a.flags.c_contiguous:
        a = np.ascontiguousarray(a, dtype=np.float64)
    return a


class _Marshalled:
    """A C FH2Data struct whose pointers borrow the arrays of a Python FH2Data dict.

    Output arrays (``wave_packets``, ``CRP.CRP``, ``options.energies``,
    ``CRP.accumulators``) must already be contiguous with the right dtype so
    that the library writes into them in place.
    """

    def __init__(self, d: dict):
        self.keep = []
        s = FH2Data()
        for key in ("r1", "r2"):
            r = d[key]
            setattr(s, key, RadialCoordinate(int(r["n"]), float(r["left"]), float(r["dr"]), float(r["mass"])))
        th = d["theta"]
        x, w = self._in(th["x"]), self._in(th["w"])
        al = self._in(th["associated_legendre"]) if th.get("associated_legendre") is not None else None
        s.theta = AngleCoordinate(int(th["n"]), int(th["m"]), _dptr(x), _dptr(w), _dptr(al))
        s.pot = _dptr(self._in(d["pot"]))
        s.psi = _dptr(self._in(d["psi"]) if d.get("psi") is not None and np.isrealobj(d["psi"]) else None)
        t = d["time"]
        s.time = EvolutionTime(int(t["total_steps"]), float(t["time_step"]), int(t["steps"]))
        op = d.get("options", {})
        wtm = op.get("wave_to_matlab")
        tn = op.get("test_name")
        self.wtm = wtm.encode() if isinstance(wtm, str) else None
        self.tn = tn.encode() if isinstance(tn, str) else None
        en = op.get("energies")
        if en is not None:
            self._out(en, np.float64)
        atc = op.get("autotune_cache")
        self.atc = str(atc).encode() if atc else None
        s.options = Options(self.wtm, self.tn, int(op.get("steps_to_copy_psi_from_device_to_host", 0)),
                            int(op.get("use_p2p_async", 0)), int(op.get("precision", 0)),
                            int(op.get("print_energies", 0)), _dptr(en), self.atc)
        for key in ("dump1", "dump2"):
            dm = d.get(key)
            arr = None if dm is None or dm.get("dump") is None else self._in(dm["dump"])
            setattr(s, key, DumpFunction(_dptr(arr)))
        c = d.get("CRP")
        if c is not None and int(c.get("calculate_CRP", 0)):
            self._out(c["CRP"], np.float64)
            acc = c.get("accumulators")
            if acc is not None:
                self._out(acc, np.complex128)
            s.CRP = CRP(_dptr(self._in(c["energies"])), _dptr(self._in(c["eta_sq"])), _dptr(c["CRP"]),
                        int(c["n_dividing_surface"]), int(c["n_gradient_points"]), int(c["n_energies"]),
                        int(c["calculate_CRP"]),
                        C.cast(acc.ctypes.data, C.POINTER(C.c_double)) if acc is not None else _dptr(None))
        else:
            s.CRP = CRP()
        om = d["OmegaStates"]
        omegas = np.ascontiguousarray(om["omegas"], dtype=np.int32).ravel()
        self.keep.append(omegas)
        P = self._in(om["associated_legendres"])
        if P.ndim == 2:
            P = P[None]
        wp = om["wave_packets"]
        self._out(wp, np.complex128)
        s.OmegaStates = OmegaStates(int(om["J"]), int(om["parity"]), int(om["l_max"]), int(om["n_omegas_max"]),
                                    int(omegas.size), omegas.ctypes.data_as(C.POINTER(C.c_int32)), _dptr(P),
                                    int(P.shape[1]), C.cast(wp.ctypes.data, C.POINTER(C.c_double)))
        self.struct = s
        self.d = d

    def _in(self, a):
        a = _f64(a)
        self.keep.append(a)
        return a

    def _out(self, a, dtype):
        if not isinstance(a, np.ndarray) or a.dtype != dtype or not a.flags.c_contiguous:
            raise QDError(1, f"output arrays must be C-contiguous {np.dtype(dtype).name} numpy arrays")
        self.keep.append(a)

    def write_back(self):
        self.d["time"]["steps"] = np.int32(self.struct.time.steps)


def _callback(fn, marshalled: List[_Marshalled]):
    if fn is None:
        return CALLBACK()

    def cb(ptr, user):
        try:
            for m in marshalled:
                if C.addressof(m.struct) == C.addressof(ptr.contents):
                    m.write_back()
                    return int(fn(m.d) or 0)
            return 1
        except Exception:   # a Python error in the callback aborts the run
            return 1

    return CALLBACK(cb)


def cudaOpenMPEvolution(FH2Data: dict, callback: Optional[Callable[[dict], int]] = None) -> None:
    """Propagate ``FH2Data['time']['total_steps']`` steps on the GPU, in place.

    Drop-in for the reference's MEX call ``cudaOpenMPEvolution(FH2Data)``
    (``FH2main.m:213``).  ``callback`` stands in for the MATLAB script named by
    ``options.wave_to_matlab`` (``cudaOpenMP2.cu:380-384``).
    """
    lib = load_library()
    m = _Marshalled(FH2Data)
    cb = _callback(callback, [m])
    st = lib.qd_evolve(C.byref(m.struct), cb, None)
    m.write_back()
    _check(st)


def evolve_batch(problems: Sequence[dict], callback=None) -> None:
    """Step several total-J problems together (``qd_evolve_batch``)."""
    lib = load_library()
    ms = [_Marshalled(d) for d in problems]
    arr = (C.POINTER(FH2Data) * len(ms))(*[C.pointer(m.struct) for m in ms])
    cb = _callback(callback, ms)
    st = lib.qd_evolve_batch(arr, len(ms), cb, None)
    for m in ms:
        m.write_back()
    _check(st)


def release_session_cache() -> None:
    """Release the device state that qd_evolve keeps for its next call of the same shape."""
    _check(load_library().qd_release_session_cache())


class Session:
    """Device-resident propagation state (``qd_session_*``)."""

    def __init__(self, problems):
        if isinstance(problems, dict):
            problems = [problems]
        self.lib = load_library()
        self.ms = [_Marshalled(d) for d in problems]
        self.arr = (C.POINTER(FH2Data) * len(self.ms))(*[C.pointer(m.struct) for m in self.ms])
        h = C.c_void_p()
        _check(self.lib.qd_session_create(self.arr, len(self.ms), C.byref(h)))
        self.h = h
        nb, lp = C.c_int32(), C.c_int32()
        _check(self.lib.qd_session_info(self.h, C.byref(nb), C.byref(lp)))
        self.n_blocks, self.launches_per_step = nb.value, lp.value
        d0 = problems[0]
        self.n1, self.n2 = int(d0["r1"]["n"]), int(d0["r2"]["n"])
        self.nth, self.l_max = int(d0["theta"]["n"]), int(d0["OmegaStates"]["l_max"])
        self.block_omegas = [int(o) for d in problems for o in np.ravel(d["OmegaStates"]["omegas"])]

    def close(self):
        if getattr(self, "h", None):
            self.lib.qd_session_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def run(self, n_steps: int):
        _check(self.lib.qd_session_run(self.h, int(n_steps)))

    def synchronize(self):
        _check(self.lib.qd_session_synchronize(self.h))

    def flush(self):
        """Enqueue the flux transform of the steps buffered so far (no host sync)."""
        _check(self.lib.qd_session_flush(self.h))

    def download(self):
        _check(self.lib.qd_session_download(self.h, self.arr, len(self.ms)))
        for m in self.ms:
            m.write_back()

    def upload(self):
        _check(self.lib.qd_session_upload(self.h, self.arr, len(self.ms)))

    def stream(self) -> int:
        return int(self.lib.qd_session_stream(self.h) or 0)

    def apply(self, stage: str, dt: float = 0.0):
        _check(self.lib.qd_session_apply(self.h, STAGES[stage], float(dt)))

    def get_psi(self, which: str, block: int) -> np.ndarray:
        if which == "theta":
            shape = (self.nth, self.n2, self.n1)
        else:
            shape = (self.l_max - self.block_omegas[block] + 1, self.n2, self.n1)
        out = np.empty(shape, np.complex128)
        _check(self.lib.qd_session_get_psi(self.h, 0 if which == "theta" else 1, block,
                                           C.cast(out.ctypes.data, C.POINTER(C.c_double)), out.size * 2))
        return out

    def set_psi(self, which: str, block: int, value: np.ndarray):
        v = np.ascontiguousarray(value, dtype=np.complex128)
        _check(self.lib.qd_session_set_psi(self.h, 0 if which == "theta" else 1, block,
                                           C.cast(v.ctypes.data, C.POINTER(C.c_double)), v.size * 2))

    def profile(self, n_steps: int) -> dict:
        """Mean per-launch duration (ms) and launches per step of every kernel over n_steps."""
        names = C.create_string_buffer(4096)
        avg = (C.c_double * 64)()
        cnt = (C.c_int32 * 64)()
        nk = C.c_int32()
        _check(self.lib.qd_session_profile(self.h, int(n_steps), names, 4096, avg, cnt, 64, C.byref(nk)))
        keys = names.value.decode().split("\n")
        return {k: {"ms": avg[i], "per_step": cnt[i] / n_steps} for i, k in enumerate(keys[: nk.value])}

    def tuning(self) -> str:
        """The autotuner's choice of FFT kernel for this session (and its timings)."""
        buf = C.create_string_buffer(8192)
        _check(self.lib.qd_session_tuning(self.h, buf, 8192))
        return buf.value.decode()

    def energies(self) -> np.ndarray:
        out = np.empty((self.n_blocks, 6))
        _check(self.lib.qd_session_get_energies(self.h, _dptr(out), out.size))
        return out


def fma_peaks() -> tuple:
    """Measured (FP64, FP32) FMA throughput of the current device in TFLOP/s."""
    lib = load_library()
    a, b = C.c_double(), C.c_double()
    _check(lib.qd_device_fma_peaks(C.byref(a), C.byref(b)))
    return a.value, b.value


def dmma_peak() -> float:
    """Measured FP64 tensor-core (DMMA) throughput of the current device in TFLOP/s."""
    lib = load_library()
    a = C.c_double()
    _check(lib.qd_device_dmma_peak(C.byref(a)))
    return a.value


def device_wait_selftest(budget_ms: float, arrive: bool) -> None:
    """Run the bounded-wait self-test (qd_device_wait_selftest); raises QDError
    (status QD_ERR_TIMEOUT) when the wait gave up."""
    lib = load_library()
    _check(lib.qd_device_wait_selftest(float(budget_ms), 1 if arrive else 0))


def build(force: bool = False) -> Path:
    """Compile libqd.so for sm_103a (in-tree)."""
    from . import buildlib
    return buildlib.build(force=force)
