"""Fixture of the reference's own test inputs (TESTS/TEST_2D, TEST_BOX,
TEST_BW): the parameters, run information, cell-centre topography and
restart state that this library's readers make of them, so that the GPU
tests can run those cases without the reference tree.

    python tests/golden/make_reference_fixtures.py /path/to/reference
    SFLOW_REFERENCE_DIR=/path/to/reference python tests/golden/make_reference_fixtures.py

Writes tests/golden/reference_tests.npz (compressed).
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))

from imex_sflow2d_dev_gb300 import lib as L  # noqa: E402
from imex_sflow2d_dev_gb300.params import params_to_dict  # noqa: E402

CASES = ("TEST_2D", "TEST_BOX", "TEST_BW")


def main(ref):
    meta, arrays = {}, {}
    for name in CASES:
        d = os.path.join(ref, "TESTS", name)
        p, run = L.read_input(os.path.join(d, "IMEX_SfloW2D.inp"))
        B, nd = L.read_dem(os.path.join(d, run["topography_file"]), p)
        q, idx = L.read_q2d(os.path.join(d, run["restart_file"]), p)
        meta[name] = {"params": params_to_dict(p), "run": run, "output_idx": idx}
        arrays[name + "_B"] = B
        arrays[name + "_q"] = q
        arrays[name + "_nodata"] = nd
    out = os.path.join(HERE, "reference_tests.npz")
    np.savez_compressed(out, meta=np.array(json.dumps(meta)), **arrays)
    print("wrote", out, os.path.getsize(out), "bytes")


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SFLOW_REFERENCE_DIR", "")
    if not ref:
        sys.exit("usage: make_reference_fixtures.py /path/to/reference (or set SFLOW_REFERENCE_DIR)")
    main(ref)
