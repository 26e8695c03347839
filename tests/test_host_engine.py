"""The host engine of libqd on a CPU, over a stand-in CUDA runtime (tests/mockcuda).

A child process preloads the stand-in, so device memory is host memory and kernels do
nothing: the numbers are not checked, the host logic is.  qd_evolve twice with the same
shape reuses the kept session (and with another potential, reloads it); callbacks fire
after the steps whose counter is a multiple of steps_to_copy_psi_from_device_to_host;
time.steps is written back; runs shorter than a flux chunk replay 2^k-step graphs;
sessions and the autotuner's cache file round-trip (tuned once, then read back as "cached"
in a fresh process)."""
import os
import shutil
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]

CHILD = r'''
import sys, json
sys.path.insert(0, sys.argv[1])
import numpy as np
import __graft_entry__ as e
qd = e.load_package(); qd.load_library()
out = {}
cfg = qd.inputs.small_config(J=2, parity=0, n1=16, n2=8, n_theta=8, l_max=6, steps=7, n_energies=8)
for prec in (0, 1):
    seen = []
    d = qd.inputs.build_fh2data(cfg); d["options"]["precision"] = prec
    d["options"]["wave_to_matlab"] = "FH2Matlab"; d["options"]["steps_to_copy_psi_from_device_to_host"] = 3
    qd.cudaOpenMPEvolution(d, callback=lambda data: seen.append(int(data["time"]["steps"])) or 0)
    out[f"callbacks_{prec}"] = seen
    out[f"steps_{prec}"] = int(d["time"]["steps"])
    qd.cudaOpenMPEvolution(d)                       # same shape: the kept session
    out[f"steps2_{prec}"] = int(d["time"]["steps"])
    d2 = qd.inputs.build_fh2data(cfg); d2["options"]["precision"] = prec
    d2["pot"] = d2["pot"] * 1.01
    qd.cudaOpenMPEvolution(d2)                      # same shape, another potential
    out[f"steps3_{prec}"] = int(d2["time"]["steps"])
qd.release_session_cache()
# a 20-step run from step 0: step 0 on its own, then 16 + 2 steps from graphs and one more step
import ctypes
mock = ctypes.CDLL(None)
small = qd.inputs.small_config(J=0, n1=16, n2=8, n_theta=8, l_max=7, steps=1, n_energies=8)
d = qd.inputs.build_fh2data(small); d["options"]["precision"] = 1
with qd.Session(d) as s:
    g0 = mock.mock_graph_launches()
    s.run(20); s.synchronize()
    out["graphs_20"] = mock.mock_graph_launches() - g0
    g0 = mock.mock_graph_launches()
    s.run(20); s.synchronize()   # steps 20-39: 16 + 4
    out["graphs_20b"] = mock.mock_graph_launches() - g0
big = qd.inputs.small_config(J=0, n1=256, n2=128, n_theta=8, l_max=7, steps=1, n_energies=8)
d = qd.inputs.build_fh2data(big); d["options"]["precision"] = 1
with qd.Session(d) as s:
    out["tuning"] = s.tuning()
    s.run(70); s.flush(); s.synchronize()
print("RESULT " + json.dumps(out))
'''


def _run_child(tmp_path, cache):
    mock = tmp_path / "libmockcuda.so"
    if not mock.exists():
        cc = shutil.which("gcc") or shutil.which("cc")
        if cc is None:
            pytest.skip("no C compiler")
        r = subprocess.run([cc, "-shared", "-fPIC", "-O1", "-Wall", "-Werror", str(ROOT / "tests" / "mockcuda" / "mockcuda.c"),
                            "-o", str(mock)], capture_output=True, text=True, timeout=120)
        assert r.returncode == 0, r.stderr
    env = dict(os.environ, LD_PRELOAD=str(mock), QD_AUTOTUNE_CACHE=str(cache))
    r = subprocess.run([sys.executable, "-c", CHILD, str(ROOT)], capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    line = [x for x in r.stdout.splitlines() if x.startswith("RESULT ")][-1]
    import json
    return json.loads(line[len("RESULT "):])


def test_host_engine_over_stand_in_runtime(lib, tmp_path):
    cache = tmp_path / "autotune.txt"
    out = _run_child(tmp_path, cache)
    # runs shorter than a flux chunk replay 2^k-step graphs
    assert out["graphs_20"] == 2 and out["graphs_20b"] == 2
    for prec in (0, 1):
        assert out[f"callbacks_{prec}"] == [0, 3, 6]
        assert out[f"steps_{prec}"] == 7 and out[f"steps2_{prec}"] == 14 and out[f"steps3_{prec}"] == 7
    # first process: every FFT candidate of 256x128 timed, the choice written to the file
    assert out["tuning"].startswith("fft: ") and "tuned:" in out["tuning"]
    assert "threads=512" in out["tuning"] and "three-pass" in out["tuning"]
    assert "two-pass 24 warps/SM" in out["tuning"] and "two-pass 32 warps/SM" in out["tuning"]
    lines = cache.read_text().splitlines()
    assert all(x.startswith("fft_mixed ") and len(x.split("\t")) == 3 for x in lines)
    assert sum("grid 256x128 slabs 8 coupled 0" in x for x in lines) == 1
    assert sum("grid 16x8 slabs 18 coupled 1" in x for x in lines) == 1
    # a fresh process reads the choices back instead of timing again
    again = _run_child(tmp_path, cache)
    assert "(cached," in again["tuning"]
    assert again["tuning"].split(" (")[0] == out["tuning"].split(" (")[0]
    assert cache.read_text().splitlines() == lines
