"""Regenerate tests/golden/oracle_small.npz: outputs of the FP64 oracle on two
tiny deterministic problems (J=0 and J=2, 16x8x6 grid, l_max=5).

The reference has no golden vectors of its own (no tests, no CPU
propagator); this fixture pins the oracle across machines (x86 container and
Arm GPU machine) so that a change in the oracle or its libraries is noticed.
Run from the repository root:  python tests/golden/make_golden.py
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
import __graft_entry__ as entry  # noqa: E402


def main():
    qd = entry.load_package()
    oracle = entry.load_oracle()
    out = {}
    for name, J, steps in (("j0", 0, 5), ("j2", 2, 5)):
        cfg = qd.inputs.small_config(n1=16, n2=8, n_theta=6, l_max=5, J=J, parity=0, steps=steps, n_energies=8)
        o = oracle.Oracle(qd.inputs.build_fh2data(cfg))
        rec = o.run(steps)
        out[f"{name}_J"] = J
        out[f"{name}_steps"] = steps
        out[f"{name}_psi"] = o.wave_packets()
        out[f"{name}_energies"] = rec
        out[f"{name}_crp"] = o.crp()
    np.savez_compressed(Path(__file__).parent / "oracle_small.npz", **out)


if __name__ == "__main__":
    main()
