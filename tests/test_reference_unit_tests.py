"""The reference's own unit tests (tests/unit/*.py), restated against this
package's host-side pieces.  The ones that need device arrays are in
test_gpu_parity.py."""
import numpy as np
import pytest
import torch

from pyminiweather_gb300.data import Constants, Quadrature
from pyminiweather_gb300.mesh import MeshData
from pyminiweather_gb300.utils import sample_ellipse_cosine
from tests.helpers import make_params


def test_constants():  # tests/unit/test_constants.py:7-19
    assert Constants.hv_beta == 0.05
    assert Constants.p0 == 1.0e5
    assert Constants.C0 == 27.5629410929725921310572974482
    assert Constants.gamma == 1.40027894002789400278940027894
    assert Constants.grav == 9.8
    assert Constants.cp == 1004.0
    assert Constants.cv == 717.0
    assert Constants.rd == 287
    assert Constants.pi == 3.14159265358979323846264338327
    assert Constants.theta0 == 300.0
    assert Constants.exner0 == 1.0


def test_quadrature_values():  # test_constants.py:22-45
    assert Quadrature.npoints == 3
    qp = np.array([0.112701665379258311482073460022, 0.5, 0.887298334620741688517926539980])
    qw = np.array([0.277777777777777777777777777779, 0.444444444444444444444444444444,
                   0.277777777777777777777777777779])
    assert np.allclose(qp, Quadrature.qpoints)
    assert np.allclose(qw, Quadrature.qweights)
    assert Quadrature.qweights.sum() == 1.0


def test_quadrature_immutable():  # test_constants.py:48-64
    for name, val in (("npoints", 4), ("qweights", 1), ("qpoints_grid_x", 3), ("qpoints_grid_z", 1),
                      ("qweights_grid_x", 3), ("qweights_grid_z", 1)):
        with pytest.raises(AttributeError):
            setattr(Quadrature, name, val)
    with pytest.raises(ValueError):
        Quadrature.qpoints[0] = 1.0


@pytest.fixture
def mesh_params():  # tests/unit/test_mesh.py:8-15
    p = {"nx": 64, "nz": 32, "xlen": 2e4, "zlen": 1e4, "hs": 2}
    p["dx"] = p["xlen"] / p["nx"]
    p["dz"] = p["zlen"] / p["nz"]
    return p


def test_mesh_coordinates(mesh_params):  # test_mesh.py:18-82
    p = mesh_params
    m = MeshData(p, device="cpu")
    xx, zz = m.get_mesh_int_ext()
    x = np.linspace(-p["hs"] * p["dx"], (p["nx"] + p["hs"]) * p["dx"], p["nx"] + 2 * p["hs"], endpoint=False)
    z = np.linspace(-p["hs"] * p["dz"], (p["nz"] + p["hs"]) * p["dz"], p["nz"] + 2 * p["hs"], endpoint=False)
    assert np.array_equal(x, xx[0, :].numpy()) and np.array_equal(z, zz[:, 0].numpy())
    xx, zz = m.get_mesh_cell_centers()
    x = np.linspace(p["dx"] / 2.0, p["xlen"] + p["dx"] / 2.0, p["nx"], endpoint=False)
    z = np.linspace(p["dz"] / 2.0, p["zlen"] + p["dz"] / 2.0, p["nz"], endpoint=False)
    assert np.array_equal(x, xx[0, :].numpy()) and np.array_equal(z, zz[:, 0].numpy())
    ze = np.linspace(0.0, (p["nz"] + 1) * p["dz"], p["nz"] + 1, endpoint=False)
    assert np.array_equal(ze, m.get_mesh_vertical_cell_edges().numpy())
    zc = np.linspace((-p["hs"] + 0.5) * p["dz"], (p["nz"] + p["hs"] + 0.5) * p["dz"], p["nz"] + 2 * p["hs"],
                     endpoint=False)
    assert np.array_equal(zc, m.get_mesh_vertical_cell_centers_int_ext().numpy())


def test_sample_ellipse_cosine():  # tests/unit/test_sample_cosine.py:9-36
    p = make_params(200, 100, "thermal")
    x, z = MeshData(p, device="cpu").get_mesh_int_ext()
    data = sample_ellipse_cosine(x, z, 1.0, p["xlen"] / 2.0, p["zlen"] / 2.0, 1e-4, 1e-4)
    assert int((data == 0.0).sum()) == data.numel() - 1


def test_sample_ellipse_cosine_cosine_dist():  # test_sample_cosine.py:39-73
    p = make_params(200, 100, "thermal")
    x, z = MeshData(p, device="cpu").get_mesh_int_ext()
    x0, z0, r = p["xlen"] / 2.0, p["zlen"] / 2.0, 1e4
    got = sample_ellipse_cosine(x, z, 1.0, x0, z0, r, r).numpy()
    xn, zn = x.numpy(), z.numpy()
    dist = np.sqrt(((xn - x0) / r) ** 2 + ((zn - z0) / r) ** 2) * Constants.pi.value / 2.0
    exp = np.where(dist <= Constants.pi.value / 2.0, np.cos(dist) ** 2.0, 0.0)
    assert np.allclose(got, exp)
