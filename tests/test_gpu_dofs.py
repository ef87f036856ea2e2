"""DOF enumeration on the device: identical to the host numbering (which
reproduces mesh_fem::enumerate_dof, pinned by the reference fixtures) for
PK and QK elements of every degree the plans take, qdim 1 and 3."""
import ctypes as C

import numpy as np
import pytest

import getfem_gb300 as g
from getfem_gb300 import _lib as L

from common import golden_names, load

pytestmark = pytest.mark.gpu


def both(mesh, degree, qdim):
    lib = L.lib()
    nb = C.c_int32()
    L.check(lib.gfgpu_nb_basis(mesh.dim, mesh.kind, degree, C.byref(nb)))
    out = []
    for fn in (lib.gfgpu_enumerate_dofs, lib.gfgpu_enumerate_dofs_device):
        d = np.empty((mesh.nb_convex(), nb.value), dtype=np.int64)
        n = C.c_int64()
        L.check(fn(mesh.dim, mesh.kind, degree, qdim, mesh.nb_convex(),
                   mesh.cvpts.ctypes.data_as(C.c_void_p), d.ctypes.data_as(C.c_void_p),
                   C.byref(n)))
        out.append((d, n.value))
    return out


@pytest.mark.parametrize("dim,kind,degree,qdim,nx", [
    (2, "simplex", 1, 1, 9), (2, "simplex", 2, 2, 7), (3, "simplex", 1, 3, 4),
    (3, "simplex", 2, 3, 5), (3, "simplex", 3, 1, 3), (2, "hex", 2, 1, 6),
    (3, "hex", 1, 3, 4), (3, "hex", 2, 3, 4), (3, "hex", 4, 1, 3)])
def test_device_numbering_equals_host(dim, kind, degree, qdim, nx):
    mesh = g.Mesh.regular_unit(dim, nx, kind)
    (dh, nh), (dd, nd) = both(mesh, degree, qdim)
    assert nh == nd
    assert np.array_equal(dh, dd)


@pytest.mark.parametrize("name", golden_names())
def test_device_numbering_matches_reference(name):
    rec = load(name)
    m = rec["meta"]
    mesh = g.Mesh.regular_unit(m["dim"], m["nx"], "simplex" if m["gt"] == "PK" else "hex",
                               jitter=rec.get("jitter"))
    mf = g.MeshFem(mesh, m["qdim"], degree=m["degree"])  # device numbering on a GPU machine
    assert mf.nb_dof() == m["n_dof"]
    assert np.array_equal(mf.dofs, rec["dofs"])
