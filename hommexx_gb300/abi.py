"""ctypes driver for a library that exports the preqx C ABI of ``include/hxgpu.h``.

It makes the calls the Fortran driver makes (``src/share/prim_driver_mod.F90:1042-1105``
for initialisation, ``src/prim_main.F90:297-317`` for the time loop), with numpy arrays
in the Fortran layouts, so the same code drives the CUDA library (``libhxgpu.so``) and
the CPU oracle.  Python is only the test/benchmark harness here: every array crosses
the boundary as a plain pointer.
"""
from __future__ import annotations

import ctypes as C
import struct
from dataclasses import dataclass, field

import numpy as np

NP, NLEV = 4, 72

_c_int_p = C.POINTER(C.c_int)
_c_dbl_p = C.POINTER(C.c_double)


def _pp(a: np.ndarray):
    """Pointer-to-pointer argument (Fortran passes type(c_ptr) by reference)."""
    assert a.flags.c_contiguous and a.dtype == np.float64
    return C.byref(C.c_void_p(a.ctypes.data))


def _i(v: int):
    return C.byref(C.c_int(int(v)))


def _d(v: float):
    return C.byref(C.c_double(float(v)))


def _b(v: bool):
    return C.byref(C.c_bool(bool(v)))


@dataclass
class SimParams:
    """Namelist values ``init_simulation_params_c`` receives."""
    remap_alg: int = 1
    limiter_option: int = 8
    rsplit: int = 1
    qsplit: int = 1
    time_step_type: int = 5
    energy_fixer: int = 0
    qsize: int = 4
    state_frequency: int = 1_000_000
    nu: float = 1e16
    nu_p: float = -1.0
    nu_q: float = -1.0
    nu_s: float = -1.0
    nu_div: float = -1.0
    nu_top: float = 2.5e5
    hypervis_order: int = 2
    hypervis_subcycle: int = 3
    hypervis_scaling: float = 0.0
    ftype: int = -1
    prescribed_wind: bool = False
    moisture: bool = False
    disable_diagnostics: bool = True
    use_cpstar: bool = False
    use_semi_lagrangian_transport: bool = False

    def resolved(self) -> "SimParams":
        """Negative nu_s/nu_q/nu_p/nu_div default to nu (namelist_mod.F90:970-972)."""
        p = SimParams(**self.__dict__)
        for k in ("nu_s", "nu_q", "nu_p", "nu_div"):
            if getattr(p, k) < 0:
                setattr(p, k, p.nu)
        return p


class HxLibrary:
    """A loaded preqx library plus the arrays it was initialised with."""

    def __init__(self, path: str):
        self.path = path
        self.lib = C.CDLL(path)
        L = self.lib
        L.hx_last_error.restype = C.c_int
        L.hx_last_error.argtypes = [C.c_char_p, C.c_int]
        L.hx_set_precision.argtypes = [C.c_int]
        L.hx_get_field.argtypes = [C.c_char_p, C.c_int, C.c_void_p]
        L.hx_set_field.argtypes = [C.c_char_p, C.c_int, C.c_void_p]
        L.hx_run_caar_stage.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double]
        L.hx_run_rk5.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double]
        L.hx_run_hypervis.argtypes = [C.c_int, C.c_double, C.c_double]
        L.hx_run_euler_step.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_int]
        L.hx_run_tracers_rk2.argtypes = [C.c_double]
        L.hx_run_remap.argtypes = [C.c_int, C.c_int, C.c_double]
        L.hx_run_prim_step.argtypes = [C.c_double]
        L.hx_run_dss.argtypes = [C.c_char_p, C.c_int, C.c_int]
        L.hx_set_async_copies.argtypes = [C.c_int]
        L.hx_stream_results.argtypes = [C.c_void_p] * 7
        L.hx_write_restart.argtypes = [C.c_char_p]
        L.hx_read_restart.argtypes = [C.c_char_p]
        L.hx_launch_count.restype = C.c_longlong
        L.hx_kernel_stats.argtypes = [C.c_char_p, C.c_int, C.POINTER(C.c_longlong),
                                      C.POINTER(C.c_double), C.c_int]
        self.nelem = 0
        self.qsize = 0

    # -- status ----------------------------------------------------------------------
    def last_error(self):
        buf = C.create_string_buffer(512)
        code = self.lib.hx_last_error(buf, 512)
        return code, buf.value.decode(errors="replace")

    def check(self, what: str = ""):
        code, msg = self.last_error()
        if code:
            raise RuntimeError(f"{what}: error {code}: {msg}")

    # -- initialisation (prim_init1 / prim_init2 order) --------------------------------
    def init(self, mesh, hv, params: SimParams, state: dict, precision: int = 0,
             abort_on_error: bool = False, time_levels=(1, 2, 3), diagnostics: bool = False):
        L = self.lib
        p = params.resolved()
        L.hx_set_abort_on_error(0 if not abort_on_error else 1)
        L.initialize_hommexx_session()
        self.check("initialize_hommexx_session")
        L.reset_cxx_comm(_i(0))
        L.init_connectivity(_i(mesh.nelem))
        for t in mesh.f90_connections():
            L.add_connection(*[_i(x) for x in t])
        L.finalize_connectivity()
        self._keep = {}
        dvv = np.ascontiguousarray(mesh.dvv, dtype=np.float64)
        self._keep["dvv"] = dvv
        L.init_derivative_c(_pp(dvv))
        L.init_simulation_params_c(
            _i(p.remap_alg), _i(p.limiter_option), _i(p.rsplit), _i(p.qsplit),
            _i(p.time_step_type), _i(p.energy_fixer), _i(p.qsize), _i(p.state_frequency),
            _d(p.nu), _d(p.nu_p), _d(p.nu_q), _d(p.nu_s), _d(p.nu_div), _d(p.nu_top),
            _i(p.hypervis_order), _i(p.hypervis_subcycle), _d(p.hypervis_scaling),
            _i(p.ftype), _b(p.prescribed_wind), _b(p.moisture), _b(p.disable_diagnostics),
            _b(p.use_cpstar), _b(p.use_semi_lagrangian_transport))
        self.check("init_simulation_params_c")
        if L.hx_set_precision(int(precision)) != 0:
            self.check("hx_set_precision")
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (
            mesh.D, mesh.Dinv, mesh.fcor, mesh.mp, mesh.spheremp, mesh.rspheremp,
            mesh.metdet, mesh.metinv, mesh.phis, mesh.tensorvisc, mesh.vec_sph2cart)]
        self._keep["metric"] = arrs
        L.init_elements_2d_c(_i(mesh.nelem), *[_pp(a) for a in arrs],
                             _b(p.hypervis_scaling == 0.0))
        self.check("init_elements_2d_c")
        self.nelem = mesh.nelem
        self.qsize = p.qsize
        self.set_state(state)
        if diagnostics:
            self.init_diagnostics()
        hyam = np.ascontiguousarray(hv.hyam)
        hyai = np.ascontiguousarray(hv.hyai)
        hybm = np.ascontiguousarray(hv.hybm)
        hybi = np.ascontiguousarray(hv.hybi)
        self._keep["hv"] = (hyam, hyai, hybm, hybi)
        L.init_hvcoord_c(_d(hv.ps0), _pp(hyam), _pp(hyai), _pp(hybm), _pp(hybi))
        L.init_boundary_exchanges_c()
        self.check("init_boundary_exchanges_c")
        nm1, n0, np1 = time_levels
        L.init_time_level_c(_i(nm1), _i(n0), _i(np1), _i(0), _i(0))
        self.tl = [nm1 - 1, n0 - 1, np1 - 1, 0]
        return self

    DIAG_NAMES = ("Q", "Qvar", "Qmass", "Q1mass", "IEner", "IEner_wet", "KEner", "PEner")

    def init_diagnostics(self, fill: float = np.nan):
        """init_diagnostics_c with host arrays in the Fortran layouts of elem%state%Q and
        elem%accum (np,np,nlev,qsize) / (np,np,qsize,4) / (np,np,qsize) / (np,np,4) /
        (np,np), filled with ``fill``; the library writes them whenever a remap interval
        computes diagnostics.  Returns the dict of arrays."""
        E, Q = self.nelem, self.qsize
        shapes = dict(Q=(E, Q, NLEV, NP, NP), Qvar=(E, 4, Q, NP, NP), Qmass=(E, 4, Q, NP, NP),
                      Q1mass=(E, Q, NP, NP), IEner=(E, 4, NP, NP), IEner_wet=(E, NP, NP),
                      KEner=(E, 4, NP, NP), PEner=(E, 4, NP, NP))
        self.diag = {k: np.full(shapes[k], fill) for k in self.DIAG_NAMES}
        self.lib.init_diagnostics_c(*[_pp(self.diag[k]) for k in self.DIAG_NAMES])
        self.check("init_diagnostics_c")
        return self.diag

    def set_state(self, state: dict):
        arrs = [np.ascontiguousarray(state[k], dtype=np.float64)
                for k in ("v", "T", "dp3d", "Qdp", "ps_v")]
        self.lib.init_elements_states_c(*[_pp(a) for a in arrs])
        self.check("init_elements_states_c")

    # -- time stepping -----------------------------------------------------------------
    def run_subcycle(self, dt: float, last_step: int = 1 << 30):
        nstep, nm1, n0, np1 = (C.c_int(self.tl[3]), C.c_int(self.tl[0]),
                               C.c_int(self.tl[1]), C.c_int(self.tl[2]))
        self.lib.prim_run_subcycle_c(_d(dt), C.byref(nstep), C.byref(nm1), C.byref(n0),
                                     C.byref(np1), _i(last_step))
        self.check("prim_run_subcycle_c")
        self.tl = [nm1.value, n0.value, np1.value, nstep.value]
        return self.tl

    # -- cubed-sphere mesh generated by the library (hx_cube_mesh) ----------------------
    def cube_mesh(self, ne: int, hypervis_scaling: float = 0.0):
        """The mesh of ``mesh.build_mesh(ne)`` computed by hx_cube_mesh (metric on the
        GPU), as a ``mesh.Mesh``."""
        from . import mesh as M
        E = 6 * ne * ne
        a = dict(dvv=np.empty((NP, NP)), D=np.empty((E, 2, 2, NP, NP)), Dinv=np.empty((E, 2, 2, NP, NP)),
                 fcor=np.empty((E, NP, NP)), mp=np.empty((E, NP, NP)), spheremp=np.empty((E, NP, NP)),
                 rspheremp=np.empty((E, NP, NP)), metdet=np.empty((E, NP, NP)),
                 metinv=np.empty((E, 2, 2, NP, NP)), tensorvisc=np.empty((E, 2, 2, NP, NP)),
                 vec_sph2cart=np.empty((E, 2, 3, NP, NP)), lat=np.empty((E, NP, NP)),
                 lon=np.empty((E, NP, NP)))
        conn_f = np.empty((E, 8, 2), dtype=np.int32)
        order = ("dvv", "D", "Dinv", "fcor", "mp", "spheremp", "rspheremp", "metdet", "metinv",
                 "tensorvisc", "vec_sph2cart", "lat", "lon")
        rc = self.lib.hx_cube_mesh(C.c_int(ne), C.c_double(hypervis_scaling),
                                   *[C.c_void_p(a[k].ctypes.data) for k in order],
                                   C.c_void_p(conn_f.ctypes.data))
        if rc:
            self.check("hx_cube_mesh")
        # (remote element, remote add_connection position), 1-based, by position ->
        # the Mesh's [e][C slot] = (remote element, remote C slot), 0-based
        slot_of_pos = np.array([2, 3, 0, 1, 4, 5, 6, 7])
        conn = -np.ones((E, 8, 2), dtype=np.int64)
        for s in range(8):
            col = conn_f[:, M.F90_POS_OF_SLOT[s] - 1]
            ok = col[:, 0] > 0
            conn[ok, s, 0] = col[ok, 0] - 1
            conn[ok, s, 1] = slot_of_pos[col[ok, 1] - 1]
        return M.Mesh(ne=ne, nelem=E, dvv=a["dvv"], D=a["D"], Dinv=a["Dinv"], metinv=a["metinv"],
                      metdet=a["metdet"], mp=a["mp"], spheremp=a["spheremp"], rspheremp=a["rspheremp"],
                      fcor=a["fcor"], phis=np.zeros((E, NP, NP)), lat=a["lat"], lon=a["lon"],
                      vec_sph2cart=a["vec_sph2cart"], tensorvisc=a["tensorvisc"], connections=conn)

    # -- copies that overlap the step --------------------------------------------------
    def set_async_copies(self, on: bool = True) -> None:
        """hx_set_async_copies: Qdp streams in while the next interval's dynamics run."""
        if self.lib.hx_set_async_copies(C.c_int(1 if on else 0)):
            self.check("hx_set_async_copies")

    def stream_results(self, out: dict | None) -> None:
        """hx_stream_results: every interval copies its results into ``out`` (the arrays
        ``push_results`` fills) as they become final; None stops."""
        keys = ("v", "T", "dp3d", "Qdp", "Q", "ps_v", "omega_p")
        ptrs = [C.c_void_p(out[k].ctypes.data) if out is not None else C.c_void_p(None) for k in keys]
        self._keep["stream"] = out
        if self.lib.hx_stream_results(*ptrs):
            self.check("hx_stream_results")

    # -- restart files (format of include/hxgpu.h) -------------------------------------
    RESTART_HEADER = struct.Struct("<8sII6i5iiQQ48s")

    def write_restart(self, path) -> None:
        rc = self.lib.hx_write_restart(str(path).encode())
        if rc:
            self.check(f"hx_write_restart({path})")

    def read_restart(self, path) -> None:
        """Replace the session's state and time levels with the file's."""
        rc = self.lib.hx_read_restart(str(path).encode())
        if rc:
            self.check(f"hx_read_restart({path})")
        h = self.read_restart_header(path)
        self.tl = [h["nm1"] - 1, h["n0"] - 1, h["np1"] - 1, h["nstep"]]

    @classmethod
    def read_restart_header(cls, path) -> dict:
        with open(path, "rb") as f:
            raw = f.read(cls.RESTART_HEADER.size)
        v = cls.RESTART_HEADER.unpack(raw)
        keys = ("magic", "version", "header_bytes", "nelem", "np", "nlev", "qsize", "timelevels",
                "qsize_timelevels", "nm1", "n0", "np1", "nstep", "nstep0", "reserved0",
                "record_bytes", "checksum", "reserved")
        return dict(zip(keys, v))

    def push_results(self, out: dict | None = None):
        E, Q = self.nelem, self.qsize
        if out is None:
            out = dict(
                v=np.empty((E, 3, NLEV, 2, NP, NP)), T=np.empty((E, 3, NLEV, NP, NP)),
                dp3d=np.empty((E, 3, NLEV, NP, NP)), Qdp=np.empty((E, 2, Q, NLEV, NP, NP)),
                Q=np.empty((E, Q, NLEV, NP, NP)), ps_v=np.empty((E, 3, NP, NP)),
                omega_p=np.empty((E, NLEV, NP, NP)))
        self.lib.cxx_push_results_to_f90(*[_pp(out[k]) for k in
                                           ("v", "T", "dp3d", "Qdp", "Q", "ps_v", "omega_p")])
        self.check("cxx_push_results_to_f90")
        return out

    # -- field access and per-phase entry points ---------------------------------------
    _SHAPES = {"v": (2, NLEV * 0 + NLEV), "vn0": (2, NLEV)}

    def field_shape(self, name: str):
        E, Q = self.nelem, self.qsize
        if name in ("v", "vn0"):
            return (E, NLEV, 2, NP, NP)
        if name in ("Qdp", "Q"):
            return (E, Q, NLEV, NP, NP)
        if name == "ps_v":
            return (E, NP, NP)
        return (E, NLEV, NP, NP)

    def get(self, name: str, tl: int = 0) -> np.ndarray:
        out = np.empty(self.field_shape(name))
        rc = self.lib.hx_get_field(name.encode(), int(tl), out.ctypes.data)
        if rc:
            raise RuntimeError(f"hx_get_field({name}) -> {rc}")
        return out

    def set(self, name: str, tl: int, arr: np.ndarray):
        a = np.ascontiguousarray(arr, dtype=np.float64).reshape(self.field_shape(name))
        rc = self.lib.hx_set_field(name.encode(), int(tl), a.ctypes.data)
        if rc:
            raise RuntimeError(f"hx_set_field({name}) -> {rc}")

    def call(self, fn: str, *args):
        rc = getattr(self.lib, fn)(*args)
        if rc:
            code, msg = self.last_error()
            raise RuntimeError(f"{fn}{args} -> {rc}: {msg}")
        return rc

    def kernel_stats(self, maxn: int = 64):
        names = C.create_string_buffer(64 * maxn)
        la = (C.c_longlong * maxn)()
        ms = (C.c_double * maxn)()
        n = self.lib.hx_kernel_stats(names, 64, la, ms, maxn)
        out = []
        for i in range(min(n, maxn)):
            nm = names.raw[64 * i: 64 * (i + 1)].split(b"\0", 1)[0].decode()
            out.append((nm, int(la[i]), float(ms[i])))
        return out

    # -- CAM forcing (the calls the Fortran prim_run_subcycle makes around each step) ----
    def push_forcing(self, FM: np.ndarray, FT: np.ndarray, FQ: np.ndarray, Qdp: np.ndarray):
        """f90_push_forcing_to_cxx: FM (E,72,2,4,4), FT (E,72,4,4), FQ (E,Q,72,4,4),
        Qdp (E,2,Q,72,4,4)."""
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (FM, FT, FQ, Qdp)]
        self.lib.f90_push_forcing_to_cxx(*[C.c_void_p(a.ctypes.data) for a in arrs])
        self.check("f90_push_forcing_to_cxx")

    def pull_forcing(self):
        """cxx_push_forcing_to_f90 -> dict(FM, FT, FQ)."""
        E, Q = self.nelem, self.qsize
        out = dict(FM=np.zeros((E, NLEV, 2, NP, NP)), FT=np.zeros((E, NLEV, NP, NP)),
                   FQ=np.zeros((E, Q, NLEV, NP, NP)))
        self.lib.cxx_push_forcing_to_f90(*[C.c_void_p(out[k].ctypes.data) for k in ("FM", "FT", "FQ")])
        self.check("cxx_push_forcing_to_f90")
        return out

    # -- dry-dynamics trajectory and its adjoint -----------------------------------------
    def _dyn_arrays(self, st=None):
        E = self.nelem
        shapes = {"v": (E, NLEV, 2, NP, NP), "T": (E, NLEV, NP, NP), "dp3d": (E, NLEV, NP, NP)}
        if st is None:
            return {k: np.empty(s) for k, s in shapes.items()}
        return {k: np.ascontiguousarray(st[k], dtype=np.float64).reshape(shapes[k])
                for k in shapes}

    def _traj(self, fn: str, inp: dict):
        a = self._dyn_arrays(inp)
        out = self._dyn_arrays()
        rc = fn(C.c_void_p(a["v"].ctypes.data), C.c_void_p(a["T"].ctypes.data),
                C.c_void_p(a["dp3d"].ctypes.data), C.c_void_p(out["v"].ctypes.data),
                C.c_void_p(out["T"].ctypes.data), C.c_void_p(out["dp3d"].ctypes.data))
        if rc:
            raise RuntimeError(f"{fn.__name__} -> {rc}: {self.last_error()[1]}")
        return out

    def traj_forward(self, x0: dict, nsteps: int, dt: float) -> dict:
        """hx_traj_forward: ``x0``/result hold one time level of v, T, dp3d."""
        a = self._dyn_arrays(x0)
        out = self._dyn_arrays()
        rc = self.lib.hx_traj_forward(
            C.c_void_p(a["v"].ctypes.data), C.c_void_p(a["T"].ctypes.data),
            C.c_void_p(a["dp3d"].ctypes.data), C.c_int(nsteps), C.c_double(dt),
            C.c_void_p(out["v"].ctypes.data), C.c_void_p(out["T"].ctypes.data),
            C.c_void_p(out["dp3d"].ctypes.data))
        if rc:
            raise RuntimeError(f"hx_traj_forward -> {rc}: {self.last_error()[1]}")
        return out

    def traj_vjp(self, bar: dict) -> dict:
        """hx_traj_vjp: cotangent of the final state -> gradient w.r.t. the initial one."""
        return self._traj(self.lib.hx_traj_vjp, bar)

    def traj_jvp(self, tan: dict) -> dict:
        """hx_traj_jvp: tangent of the initial state -> tangent of the final one."""
        return self._traj(self.lib.hx_traj_jvp, tan)

    def traj_checkpointing(self, mode: int):
        """hx_traj_set_checkpointing: 0 automatic, 1 every stage input, 2 step inputs."""
        rc = self.lib.hx_traj_set_checkpointing(C.c_int(mode))
        if rc:
            raise RuntimeError(f"hx_traj_set_checkpointing -> {rc}: {self.last_error()[1]}")

    def finalize(self):
        self.lib.finalize_hommexx_session()
