"""The debug build with device index checks (libhxgpu_bc.so, compiled with
-DHX_BOUNDS_CHECK; hx_build_flags() bit 0): the DSS gathers check every table source
against the mesh, the remap its source cell, the tracer advection its Qdp slab, and a
violation would be reported as HX_ERR_CUDA by the interval that met it.  Whole remap
intervals on small meshes run clean and still match the oracle to 1e-12.

The debug library runs in a process of its own, as a debug build would be used: its
kernels carry the same names as the regular library's.
"""
import os
import subprocess
import sys
import textwrap

import numpy as np
import pytest

import hxtest as H
from hommexx_gb300 import build as B

pytestmark = pytest.mark.gpu

DT = 300.0

_RUN = textwrap.dedent("""
    import sys
    import numpy as np
    sys.path.insert(0, sys.argv[1])
    import hxtest as H
    from hommexx_gb300 import abi
    ne, Q, nint = int(sys.argv[3]), int(sys.argv[4]), int(sys.argv[5])
    kw = eval(sys.argv[6])
    L = H.lib(sys.argv[2])
    assert L.lib.hx_build_flags() & 1, "not the bounds-checked library"
    L.init(H.mesh(ne), H.hvc(), abi.SimParams(qsize=Q, nu=1e16, **kw), H.state(ne, Q))
    for _ in range(nint):
        L.run_subcycle(300.0)   # raises on a reported index violation
    np.savez(sys.argv[7], tl=np.array(L.tl), **L.push_results())
""")


@pytest.mark.parametrize("ne,Q,kw", [(2, 2, dict(rsplit=3)), (4, 4, dict(rsplit=1, limiter_option=9)),
                                     (3, 3, dict(rsplit=0))])
def test_bounds_checked_build_runs_clean_and_matches_oracle(oracle_path, tmp_path, ne, Q, kw):
    bc = B.build(bounds_check=True)
    out = str(tmp_path / "bc.npz")
    here = os.path.dirname(os.path.abspath(__file__))
    r = subprocess.run([sys.executable, "-c", _RUN, here, bc, str(ne), str(Q), "2", repr(kw), out],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    got = np.load(out)
    o = H.setup(oracle_path, ne, Q, nu=1e16, **kw)
    for _ in range(2):
        o.run_subcycle(DT)
    ro = o.push_results()
    assert got["tl"].tolist() == o.tl
    errs = {k: H.rel_err(got[k], ro[k]) for k in ro}
    assert all(v <= 1e-12 for v in errs.values()), errs
