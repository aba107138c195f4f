"""Field output (the reference's VIS path): the Exodus II writer read back by
an independent netCDF reader (scipy), and the device nodal field against the
extraction rows applied on the host."""
import numpy as np
import pytest

import moris_gb300 as mg
from moris_gb300 import vis

from common import problem, uniform01


def test_exodus_file_reads_back(tmp_path):
    netcdf = pytest.importorskip("scipy.io").netcdf_file
    mesh = mg.hmr_uniform_mesh(3, (3, 2, 2), (1.0, 1.0, 1.0), 1)
    n = len(mesh["coords"])
    fields = {"displacement_x": uniform01(1, n), "density": uniform01(2, n)}
    path = tmp_path / "out.exo"
    vis.write_exodus(path, mesh["coords"], mesh["cells"], fields, time=2.5)
    with netcdf(str(path), "r", mmap=False) as f:
        assert f.version_byte == 2
        assert f.dimensions["num_nodes"] == n and f.dimensions["num_elem"] == len(mesh["cells"])
        assert f.dimensions["num_dim"] == 3 and f.dimensions["num_nod_per_el1"] == 8
        assert f.dimensions["time_step"] is None  # the record dimension
        for d, ax in enumerate(("coordx", "coordy", "coordz")):
            assert np.array_equal(f.variables[ax][:], mesh["coords"][:, d])
        conn = f.variables["connect1"]
        assert np.array_equal(conn[:], mesh["cells"] + 1)
        assert conn.elem_type == b"HEX8"
        names = [b"".join(r).rstrip(b"\0").decode() for r in f.variables["name_nod_var"][:]]
        assert names == list(fields)
        assert f.variables["time_whole"][0] == 2.5
        for k, name in enumerate(fields):
            assert np.array_equal(f.variables["vals_nod_var%d" % (k + 1)][0], fields[name])
        assert f.variables["eb_prop1"].name == b"ID"


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    if not t.cuda.is_available():
        pytest.skip("no CUDA device")
    return t


@pytest.mark.gpu
def test_nodal_field_matches_extraction_rows(torch, tmp_path):
    """Quadratic B-splines: every node's value is the weighted sum over its
    extraction row, computed on the host from the same mesh arrays."""
    prod, _, mesh = problem(3, (3, 3, 2), 2, mg.SHAPE_RECTANGULAR, mg.RULE_HEX_3x3x3, False)
    prod.finalize()
    u = uniform01(5, prod.num_adofs) - 0.5
    got = vis.nodal_field(prod, torch.tensor(u, device="cuda")).cpu().numpy()
    rp, _ = prod.graph()
    nu = prod.num_adofs // 3
    # basis -> rank: the used bases in ascending order (level 0, all bases used)
    used = np.unique(mesh["t_bases"])
    rank = {b: i for i, b in enumerate(used)}
    assert len(used) == nu
    ref = np.zeros((3, len(mesh["coords"])))
    for nd in range(len(mesh["coords"])):
        for k in range(mesh["t_off"][nd], mesh["t_off"][nd + 1]):
            for f in range(3):
                ref[f, nd] += mesh["t_w"][k] * u[f * nu + rank[mesh["t_bases"][k]]]
    assert np.max(np.abs(got - ref)) <= 1e-13 * np.max(np.abs(ref))
    vis.write_exodus(tmp_path / "q.exo", mesh["coords"], mesh["cells"], {"ux": got[0], "uy": got[1], "uz": got[2]})
