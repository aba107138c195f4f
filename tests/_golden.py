"""Readers for the golden fixtures in tests/golden (reference test data)."""
import json
import os
import struct

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_bin(name):
    """fn_load_matrix_from_binary_file format: uint rows, uint cols, column-major doubles."""
    with open(os.path.join(GOLDEN, name), "rb") as f:
        b = f.read()
    r, c = struct.unpack("II", b[:8])
    return np.frombuffer(b[8:], dtype=np.float64).reshape(c, r).T.copy()


def elasticity_inputs():
    with open(os.path.join(GOLDEN, "elasticity_inputs.json")) as f:
        return json.load(f)
