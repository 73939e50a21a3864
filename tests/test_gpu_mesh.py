"""hx_cube_mesh (metric on the GPU, connectivity from integer corner positions) against
the numpy mesh generator, and a remap interval on each mesh."""
import numpy as np
import pytest

import hxtest as H
from hommexx_gb300 import abi, mesh as M, state as S

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("ne,hvs", [(1, 0.0), (2, 0.0), (4, 0.0), (4, 3.2), (16, 0.0), (30, 0.0)])
def test_cube_mesh_matches_numpy_generator(gpu_path, ne, hvs):
    d = H.lib(gpu_path).cube_mesh(ne, hvs)
    m = M.build_mesh(ne, hvs)
    assert np.array_equal(d.connections, m.connections)
    assert np.array_equal(d.dvv, m.dvv)
    assert np.array_equal(d.mp, m.mp)
    errs = {k: H.rel_err(getattr(d, k), getattr(m, k)) for k in
            ("D", "Dinv", "metinv", "metdet", "spheremp", "rspheremp", "fcor", "lat", "vec_sph2cart")}
    dl = np.angle(np.exp(1j * (d.lon - m.lon)))
    errs["lon"] = float(np.max(np.abs(dl))) / np.pi
    if hvs:
        errs["tensorvisc"] = H.rel_err(d.tensorvisc, m.tensorvisc)
    assert all(v < 1e-13 for v in errs.values()), errs
    # the mesh's area is 4 pi and rspheremp is the inverse assembled mass
    assert abs(np.sum(d.spheremp) - 4 * np.pi) < 1e-12 * 4 * np.pi


def test_remap_interval_on_device_mesh(gpu_path):
    """The same seeded state stepped on the device-generated mesh and on the numpy mesh."""
    L = H.lib(gpu_path)
    md = L.cube_mesh(4)
    mp_ = H.mesh(4)
    hv = H.hvc()
    st = S.initial_state(mp_, 4, hv)
    out = []
    for m in (md, mp_):
        if L.nelem:
            L.finalize()
        L.init(m, hv, abi.SimParams(qsize=4, nu=1e16, rsplit=3), st)
        L.run_subcycle(300.0)
        out.append(L.push_results())
    errs = {k: H.rel_err(out[0][k], out[1][k]) for k in out[1]}
    assert all(v < 1e-12 for v in errs.values()), errs
