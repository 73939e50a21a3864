"""The Fortran driver's call sequence, made from C on the GPU: tests/c/prim_main_from_c.c
(compiled here against include/hxgpu.h and libhxgpu.so) reads a mesh, namelist values
and an initial state from a file this test writes, makes the calls of
prim_driver_mod.F90:1045-1104 and prim_main.F90:297-317 with every argument by
reference, runs remap intervals and writes what cxx_push_results_to_f90 returns.  The
oracle runs the same intervals from the same inputs; every array agrees to 1e-12.
"""
import os
import subprocess

import numpy as np
import pytest

import hxtest as H
from hommexx_gb300 import abi

pytestmark = pytest.mark.gpu

NE, Q, NINT, DT = 4, 4, 2, 300.0


def _params():
    return abi.SimParams(qsize=Q, nu=1e16, rsplit=3, hypervis_subcycle=3, nu_top=2.5e5, limiter_option=8,
                         remap_alg=1)


def _write_input(path, mesh, hv, st, p):
    conns = np.array(list(mesh.f90_connections()), dtype=np.int32).reshape(-1, 8)
    hd = np.array([mesh.nelem, Q, conns.shape[0], NINT, p.rsplit, p.hypervis_subcycle, p.limiter_option,
                   p.remap_alg], dtype=np.int32)
    par = np.array([DT, p.nu, p.nu_top, hv.ps0], dtype=np.float64)
    f64 = lambda a: np.ascontiguousarray(a, dtype=np.float64).tobytes()
    with open(path, "wb") as f:
        f.write(hd.tobytes())
        f.write(par.tobytes())
        f.write(conns.tobytes())
        f.write(f64(mesh.dvv))
        for a in (hv.hyam, hv.hyai, hv.hybm, hv.hybi):
            f.write(f64(a))
        for a in (mesh.D, mesh.Dinv, mesh.fcor, mesh.mp, mesh.spheremp, mesh.rspheremp, mesh.metdet,
                  mesh.metinv, mesh.phis, mesh.tensorvisc, mesh.vec_sph2cart):
            f.write(f64(a))
        for k in ("v", "T", "dp3d", "Qdp", "ps_v"):
            f.write(f64(st[k]))


def _read_output(path, E):
    n3 = E * 72 * 16
    raw = open(path, "rb").read()
    dbl = np.frombuffer(raw[: len(raw) - 16], dtype=np.float64)
    shapes = dict(v=(E, 3, 72, 2, 4, 4), T=(E, 3, 72, 4, 4), dp3d=(E, 3, 72, 4, 4), Qdp=(E, 2, Q, 72, 4, 4),
                  Q=(E, Q, 72, 4, 4), ps_v=(E, 3, 4, 4), omega_p=(E, 72, 4, 4))
    out, o = {}, 0
    for k, sh in shapes.items():
        n = int(np.prod(sh))
        out[k] = dbl[o:o + n].reshape(sh)
        o += n
    assert o == n3 * (6 + 3 + 3 + 2 * Q + Q + 1) + E * 48
    tl = np.frombuffer(raw[-16:], dtype=np.int32).tolist()
    return out, tl


def test_fortran_call_sequence_from_c_matches_oracle(gpu_path, oracle_path, tmp_path):
    exe = str(tmp_path / "prim_main_from_c")
    libdir = os.path.dirname(gpu_path)
    subprocess.run(["gcc", "-std=c11", "-O1", "-Wall", "-Werror", "-I", os.path.join(H.ROOT, "include"),
                    os.path.join(H.ROOT, "tests", "c", "prim_main_from_c.c"), "-L", libdir, "-lhxgpu",
                    f"-Wl,-rpath,{libdir}", "-o", exe], check=True, capture_output=True)
    mesh, hv, st, p = H.mesh(NE), H.hvc(), H.state(NE, Q), _params()
    fin, fout = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    _write_input(fin, mesh, hv, st, p)
    r = subprocess.run([exe, fin, fout], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    got, tl = _read_output(fout, mesh.nelem)
    O = H.lib(oracle_path)
    if O.nelem:
        O.finalize()
    O.init(mesh, hv, p, st)
    for _ in range(NINT):
        O.run_subcycle(DT)
    ref = O.push_results()
    assert tl == [O.tl[3], O.tl[0], O.tl[1], O.tl[2]]
    errs = {k: H.rel_err(got[k], ref[k]) for k in ref}
    bad = {k: v for k, v in errs.items() if not v <= 1e-12}
    assert not bad, errs
