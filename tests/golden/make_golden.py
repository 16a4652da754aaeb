"""Generates the golden fixtures of tests/test_oracle.py from the oracle.

The reference cannot be built or imported in this image (CSXCAD, fparser,
TinyXML, HDF5, Boost and VTK are missing) and its TESTSUITE ships no golden
vectors, so these fixtures freeze the oracle's output on small scenes: any
later change to the oracle, the operator build or the scene generators that
alters a single bit shows up as a fixture mismatch.

    python tests/golden/make_golden.py
"""
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
from wipems_gb300 import Operator, scenes  # noqa: E402

CASES = [("p64_200", "p64", 2000, 200), ("mini_upml_150", "upml", 400, 150), ("mini_mixed_120", "mixed", 400, 120)]


def main():
    out = Path(__file__).resolve().parent
    for name, kind, nr_ts, steps in CASES:
        sc = scenes.p64(nr_ts=nr_ts) if kind == "p64" else scenes.mini(kind, nr_ts=nr_ts)
        op = Operator(sc)
        r = oracle.run(op.desc, op.probes, steps, op.probe_interval, engine=oracle.BASIC)
        np.savez_compressed(out / f"{name}.npz", values=r["values"], energy=r["energy"])
        meta = dict(scene=kind, nr_ts=nr_ts, steps=steps, dT=op.dT, interval=op.probe_interval,
                    volt_xor=int(np.bitwise_xor.reduce(r["volt"].view(np.uint32).ravel())))
        (out / f"{name}.json").write_text(json.dumps(meta, indent=1) + "\n")
        print(name, r["values"].shape)


if __name__ == "__main__":
    main()
