"""Regenerate the golden fixtures in this folder from the reference checkout.

Run once where the reference source tree is available, with its root as the
argument:

    python tests/golden/make_golden.py <reference source tree>

It copies the reference's own shape-function and quadrature fixture files
(``projects/FEM/INT/test/data``: raw ``uint rows, uint cols`` + column-major
doubles, read by ``LINALG/src/fn_load_matrix_from_binary_file.hpp``) and
extracts the deterministic linear-element inputs of the elasticity IWG unit
tests (``FEM/INT/test/FEM_Test_Proxy/cl_FEM_Inputs_for_Elasticity_UT.cpp``,
``fill_xhat_Elast`` / ``fill_uhat_Elast``, interpolation order 1) into
``elasticity_inputs.json``.  It also extracts the 2 x 2 QUAD4 mesh of the
reference's plane-strain example (``projects/EXA/structure/linear/Plane_Strain/
4elements.e``, Exodus II in netCDF classic format, read with scipy's netCDF
reader) into ``plane_strain_4elements.json``: node coordinates, 0-based cell
connectivity and the side sets as (cell, side ordinal) pairs, where the
ordinal is the Exodus side number minus one (side k joins local nodes k and
k+1).  And it copies HMR's T-matrix fixture (``projects/HMR/test/data/
T-Matrix_test_values.hdf5``, read by ``tests/hdf5_min.py``).  Nothing at test
time reads the reference.
"""
import json
import os
import re
import shutil
import sys

BINS = [
    "points_2d.bin", "points_3d.bin",
    "lagrange_quad4_phihat.bin", "lagrange_quad4_phi.bin", "lagrange_quad4_dphidxi.bin",
    "lagrange_hex8_phihat.bin", "lagrange_hex8_phi.bin", "lagrange_hex8_dphidxi.bin",
    "integrate_quad_2x2.bin", "integrate_hex_2x2x2.bin", "integrate_hex_3x3x3.bin",
]


def _case_block(text, func, dim, order):
    """Return the brace initializer of `func` for (space dim, interp order)."""
    start = text.index("fill_%s(" % func)
    body = text[start:]
    dpos = body.index("case %d:" % dim)
    sub = body[dpos:]
    opos = sub.index("case %d:" % order)
    sub = sub[opos:]
    eq = sub.index("=")
    k = sub.index("{", eq)
    depth = 0
    for m in range(k, len(sub)):
        if sub[m] == "{":
            depth += 1
        elif sub[m] == "}":
            depth -= 1
            if depth == 0:
                break
    rows = re.findall(r"\{([^{}]*)\}", sub[k:m + 1])
    return [[float(x) for x in r.split(",") if x.strip()] for r in rows]


def plane_strain_mesh(ref):
    from scipy.io import netcdf_file
    path = os.path.join(ref, "projects", "EXA", "structure", "linear", "Plane_Strain", "4elements.e")
    f = netcdf_file(path, "r", mmap=False)
    v = f.variables

    def names(key):
        return [b"".join(r).decode().strip("\x00") for r in v[key][:]]

    coords = [[float(x), float(y)] for x, y in zip(v["coordx"][:], v["coordy"][:])]
    cells = (v["connect1"][:] - 1).tolist()
    sides = {}
    for k, name in enumerate(names("ss_names")):
        sides[name] = {"cells": (v["elem_ss%d" % (k + 1)][:] - 1).tolist(),
                       "ordinals": (v["side_ss%d" % (k + 1)][:] - 1).tolist()}
    return {"source": "projects/EXA/structure/linear/Plane_Strain/4elements.e", "coords": coords, "cells": cells,
            "block": names("eb_names")[0], "side_sets": sides}


def main(ref):
    here = os.path.dirname(os.path.abspath(__file__))
    data = os.path.join(ref, "projects", "FEM", "INT", "test", "data")
    for b in BINS:
        shutil.copyfile(os.path.join(data, b), os.path.join(here, b))
    # HMR's T-matrix fixture (HDF5, read by tests/hdf5_min.py)
    shutil.copyfile(os.path.join(ref, "projects", "HMR", "test", "data", "T-Matrix_test_values.hdf5"),
                    os.path.join(here, "T-Matrix_test_values.hdf5"))
    src = open(os.path.join(ref, "projects", "FEM", "INT", "test", "FEM_Test_Proxy",
                            "cl_FEM_Inputs_for_Elasticity_UT.cpp")).read()
    out = {}
    for dim in (2, 3):
        out["xhat_%dd" % dim] = _case_block(src, "xhat_Elast", dim, 1)
        out["uhat_%dd" % dim] = _case_block(src, "uhat_Elast", dim, 1)
    with open(os.path.join(here, "elasticity_inputs.json"), "w") as f:
        json.dump(out, f, indent=1)
    with open(os.path.join(here, "plane_strain_4elements.json"), "w") as f:
        json.dump(plane_strain_mesh(ref), f, indent=1)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <reference source tree>")
    main(sys.argv[1])
