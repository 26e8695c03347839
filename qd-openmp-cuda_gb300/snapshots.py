"""Headless wave-packet snapshots.

The reference shows the wave packet by running a MATLAB script through
``options.wave_to_matlab`` every ``steps_to_copy_psi_from_device_to_host``
steps, after the device-to-host copy (``cudaOpenMP2.cu:380-384``,
``wave2matlab.C:19-26``); its plotting scripts (``PlotPotWave.m``,
``FH2Matlab.m``) need a display.  ``snapshot_callback`` is the headless
equivalent for ``cudaOpenMPEvolution(..., callback=...)``: at each callback it
writes the complex128 wave packets as ``psi_<step>.npy`` and the reduced
density

    rho(R, r) = sum_Omega sum_k w_k |psi_Omega(R, r, x_k)|^2

as an 8-bit grey-scale PGM image ``density_<step>.pgm`` (R across, r upwards),
a format any image viewer reads and that needs no graphics library to write.
"""
from __future__ import annotations

from pathlib import Path
from typing import Callable, Optional

import numpy as np


def density(data: dict) -> np.ndarray:
    """rho[j, i] over the (r, R) grid of the FH2Data ``data`` (shape (n2, n1))."""
    wp = np.asarray(data["OmegaStates"]["wave_packets"])   # (n_Omega, n_theta, n2, n1)
    w = np.asarray(data["theta"]["w"], dtype=np.float64)
    return np.einsum("k,okji->ji", w, wp.real ** 2 + wp.imag ** 2)


def write_pgm(path, image: np.ndarray, vmax: Optional[float] = None) -> None:
    """Binary PGM (P5), 0..255 linear in ``image / vmax`` (default: its maximum);
    row 0 of ``image`` is drawn at the bottom."""
    a = np.asarray(image, dtype=np.float64)
    top = float(a.max()) if vmax is None else float(vmax)
    g = np.zeros(a.shape, np.uint8) if top <= 0 else np.clip(np.rint(255.0 * a / top), 0, 255).astype(np.uint8)
    g = np.ascontiguousarray(g[::-1])
    with open(path, "wb") as f:
        f.write(b"P5\n%d %d\n255\n" % (g.shape[1], g.shape[0]))
        f.write(g.tobytes())


def read_pgm(path) -> np.ndarray:
    """The grey levels of a binary PGM written by ``write_pgm``, row 0 at the bottom."""
    raw = Path(path).read_bytes()
    fields, pos = [], 0
    while len(fields) < 4:   # magic, width, height, maxval
        while raw[pos:pos + 1].isspace():
            pos += 1
        start = pos
        while not raw[pos:pos + 1].isspace():
            pos += 1
        fields.append(raw[start:pos])
    if fields[0] != b"P5":
        raise ValueError("not a binary PGM")
    w, h = int(fields[1]), int(fields[2])
    img = np.frombuffer(raw[pos + 1:pos + 1 + w * h], dtype=np.uint8).reshape(h, w)
    return img[::-1]


def snapshot_callback(outdir, psi: bool = True, image: bool = True) -> Callable[[dict], int]:
    """A ``cudaOpenMPEvolution`` callback writing ``psi_<step>.npy`` and
    ``density_<step>.pgm`` into ``outdir``; returns 0 (continue)."""
    out = Path(outdir)
    out.mkdir(parents=True, exist_ok=True)

    def cb(data: dict) -> int:
        step = int(data["time"]["steps"])
        if psi:
            np.save(out / f"psi_{step:06d}.npy", np.asarray(data["OmegaStates"]["wave_packets"]))
        if image:
            write_pgm(out / f"density_{step:06d}.pgm", density(data))
        return 0

    return cb
