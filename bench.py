"""Benchmark of the GB300 preqx dycore step: simulated years per day (SYPD) at ne30L72.

Workload (the FP64 plain-form configuration): equiangular cubed sphere ne=30 (5400
elements), np=4, 72 levels, 10 tracers, dt=300 s, rsplit=3 (remap every 3 dynamics
steps), hyperviscosity nu=1e15 with 3 subcycles, nu_top=2.5e5, limiter 8, PPM
mirrored remap; seeded smooth synthetic initial state (spherical harmonics of degree
<= 6).  One benchmark step = one ``prim_run_subcycle_c`` call = one remap interval =
3 dynamics steps = 900 simulated seconds.  SYPD = simulated years per wall-clock day.

* ``value``: device time of K steps with the state resident in HBM (CUDA events on the
  library's stream); the working set (~1.9 GB) is far larger than L2, so no flush.
* ``e2e``: the same through the C ABI with host buffers, each step copying the state in
  (``init_elements_states_c``) and the results out (``cxx_push_results_to_f90``) from
  pinned host memory, wall clock.  The copies overlap the step where their data allow
  (``hx_set_async_copies``: v, T, dp3d and ps_v as whole arrays before the first kernel,
  Qdp during the first dynamics step; ``hx_stream_results``: each result piece is copied
  out once it is final, the last ones chunk by chunk of the final remap); every byte
  still crosses the host link inside the timed region.  The ``e2e`` block also records
  the host link rates measured just before the loop and the wall time of each call.
* ``mixed``: the mixed-precision form timed the same way, with its error against the
  FP64 form after ``--error-days`` simulated days.
* ``roofline``: the kernel with the largest share of device time; algorithmic bytes per
  launch from the field-pass model below, divided by its CUDA-event launch time.
* ``cpu_baseline``: the C++/OpenMP oracle (a restatement of the reference's algorithm;
  the reference itself needs Kokkos and cannot be built here) on all host cores, on a
  bounded sample of the same workload.
* ``adjoint``: the hand-written adjoint of the dry dynamics (RK5 caar + hyperviscosity
  + PPM remap) at ne16 L72, 24 steps of 300 s: device time of the forward trajectory
  and of the vector-Jacobian product (state on the device, CUDA events), the cost of
  a gradient relative to a forward run, and its checks: central finite differences of
  J = sum spheremp T_final^2 along 10 seeded smooth directions (eps = 1e-6), the
  dot-product test against the CUDA tangent-linear model (``hx_traj_jvp``, also timed),
  and the mixed form's gradient error against the FP64 one.  (The dot product against
  the oracle's tangent-linear model is a GPU test, tests/test_gpu_adjoint.py.)

``--impl reference`` times that CPU implementation alone and prints its own line.
Multi-GPU: the step does not shard here (one GPU per box), so N>1 runs N independent
replicas, one per rank, and reports their aggregate.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NE, QSIZE, DT, RSPLIT, HSUB, NU = 30, 10, 300.0, 3, 3, 1e15
SIM_SECONDS_PER_STEP = DT * RSPLIT
MEASURED_PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0


# Per launch, measured by ncu at ne16 L72 q10 (1536 elements) over the launches of one
# remap interval (profiles/kernel_counts_ne16_fp64_mixed.md gives the command and the
# build): DRAM bytes read + written (dram__bytes_read.sum + dram__bytes_write.sum), FP64
# floating-point operations DADD + DMUL + 2 DFMA and FP64 instructions DADD + DMUL + DFMA
# (smsp__sass_thread_inst_executed_op_{dadd,dmul,dfma}_pred_on.sum), each averaged over the
# kernel's launches in that interval and scaled to the run's size by the element count
# (levels and tracers fixed).  A kernel that changes invalidates its row: the table is
# re-captured with the kernels it describes.
NCU_NE16 = {
    "fp64": {
        "ppm_remap": (327.6e6, 1245.0e6, 939.2e6),
        "euler_bih_post": (282.3e6, 668.9e6, 376.0e6),
        "euler_bih_pre": (260.8e6, 583.9e6, 300.8e6),
        "euler_aal_tracer": (426.3e6, 489.6e6, 299.0e6),
        "hv_laplace2": (162.0e6, 352.9e6, 210.4e6),
        "caar_stage": (200.4e6, 320.0e6, 197.9e6),
        "hv_laplace1": (77.6e6, 292.9e6, 164.6e6),
        "update_q": (239.2e6, 107.9e6, 63.7e6),
        "euler_dss_qdp": (326.0e6, 52.2e6, 46.3e6),
        "precompute_divdp": (29.3e6, 41.9e6, 25.0e6),
        "euler_qminmax": (214.5e6, 35.5e6, 26.7e6),
        "hv_dss_update": (117.7e6, 35.4e6, 30.1e6),
        "dss_caar": (79.1e6, 15.9e6, 15.9e6),
        "dp3d_from_ps": (0.2e6, 5.3e6, 3.5e6),
        "euler_dss_fvar": (14.8e6, 4.0e6, 4.0e6),
        "euler_bih_weight": (14.2e6, 1.8e6, 1.8e6),
        "euler_minmax_nbr": (17.8e6, 0.0e6, 0.0e6),
        "prim_step_init": (53.1e6, 0.0e6, 0.0e6),
    },
    "mixed": {
        "ppm_remap": (327.4e6, 345.9e6, 253.1e6),
        "update_q": (239.1e6, 107.9e6, 63.7e6),
        "euler_aal_tracer": (424.5e6, 55.4e6, 55.4e6),
        "euler_dss_qdp": (326.2e6, 52.2e6, 46.3e6),
        "caar_stage": (188.2e6, 52.0e6, 45.1e6),
        "euler_bih_post": (274.3e6, 43.7e6, 43.7e6),
        "hv_laplace2": (150.3e6, 28.0e6, 23.1e6),
        "dss_caar": (79.3e6, 15.9e6, 15.9e6),
        "hv_dss_update": (116.5e6, 15.9e6, 15.9e6),
        "dp3d_from_ps": (0.2e6, 5.3e6, 3.5e6),
        "euler_dss_fvar": (14.8e6, 4.0e6, 4.0e6),
        "hv_laplace1": (70.2e6, 3.5e6, 3.5e6),
        "euler_bih_weight": (14.2e6, 1.8e6, 1.8e6),
        "euler_qminmax": (214.6e6, 0.1e6, 0.1e6),
        "precompute_divdp": (28.8e6, 0.0e6, 0.0e6),
        "euler_minmax_nbr": (17.8e6, 0.0e6, 0.0e6),
        "euler_bih_pre": (257.3e6, 0.0e6, 0.0e6),
        "prim_step_init": (53.3e6, 0.0e6, 0.0e6),
    },
}
NCU_NE16_ELEMENTS = 1536


def ncu_row(form: str, kernel: str, E: int, Q: int):
    """(DRAM bytes, FP64 FLOPs, FP64 instructions) per launch scaled to E elements, or
    Nones."""
    v = NCU_NE16.get(form, {}).get(kernel)
    if v is None or Q != 10:
        return None, None, None
    sc = E / NCU_NE16_ELEMENTS
    return tuple(x * sc for x in v)


def measure_link(nbytes: int = 1 << 30, reps: int = 3):
    """Host link rates of this machine: best of ``reps`` pinned -> device and device -> pinned
    copies of ``nbytes`` (CUDA events on the copying stream), in GB/s."""
    import torch
    h = torch.empty(nbytes // 8, dtype=torch.float64, pin_memory=True)
    d = torch.empty(nbytes // 8, dtype=torch.float64, device="cuda")
    st = torch.cuda.Stream()
    out = {}
    with torch.cuda.stream(st):
        for name, f in (("h2d_gbs", lambda: d.copy_(h, non_blocking=True)),
                        ("d2h_gbs", lambda: h.copy_(d, non_blocking=True))):
            best = None
            for _ in range(reps):
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(st)
                f()
                b.record(st)
                b.synchronize()
                ms = a.elapsed_time(b)
                best = ms if best is None else min(best, ms)
            out[name] = nbytes / (best * 1e-3) / 1e9
    del h, d
    return out


def fp64_peak(lib_path: str):
    """Measured FP64 FMA throughput of the device in TFLOP/s (hx_fp64_peak)."""
    import ctypes
    lib = ctypes.CDLL(lib_path)
    v = ctypes.c_double(0.0)
    rc = lib.hx_fp64_peak(ctypes.byref(v))
    return v.value if rc == 0 else None


def sypd(steps: int, seconds: float) -> float:
    return steps * SIM_SECONDS_PER_STEP / (365.0 * seconds)


# ---- algorithmic bytes per remap interval, per kernel -----------------------------------
def kernel_bytes(E: int, Q: int, rsize: int, rsplit: int = RSPLIT, hsub: int = HSUB,
                 nu_p_positive: bool = True):
    """(launches, bytes) per remap interval for every kernel: each launch reads each
    input field once and writes each output field once (one field = E*16*72 values;
    dynamics fields in the form's type, tracer mass in double)."""
    F = E * 16 * 72 * rsize
    Fd = E * 16 * 72 * 8
    qlim = E * Q * 2 * 72 * 8
    d = {}

    def add(name, launches, nbytes):
        a, b = d.get(name, (0, 0))
        d[name] = (a + launches, b + nbytes)

    for _ in range(rsplit):
        add("prim_step_init", 1, 8 * F)
        # caar: stage 1 (19F: n0 4, nm1 4, vn0 4, omega_p 2, phi 1, out 4), stages 2-4
        # (13F: no vn0/omega_p accumulation), stage 5 (27F: + RK combine 8F)
        add("caar_stage", 5, (19 + 13 * 3 + 27) * F)
        add("dss_caar", 5, 5 * 8 * F)
        add("hv_laplace1", hsub, hsub * 8 * F)
        add("hv_laplace2", hsub, hsub * 13 * F)
        add("hv_dss_update", hsub, hsub * 11 * F)
        if Q > 0:
            add("precompute_divdp", 1, 4 * F)
            for stage in range(3):
                last = stage == 2
                add("euler_qminmax", 1, Q * Fd + 2 * F + qlim + (Q * F if last else 0)
                    + (qlim if stage == 1 else 0))
                if stage != 1:
                    add("euler_minmax_nbr", 1, 2 * qlim)
                if last:
                    add("euler_bih_pre", 1, 2 * Q * F + F)
                    add("euler_bih_post", 1, 2 * Q * F)
                # setup phase fused into the tracer kernel: derived_dp, divdp_proj, divdp,
                # vn0 (2), f_dss in, fscr out (+ dpdiss_bih in the biharmonic stage)
                add("euler_aal_tracer", 1, Q * Fd + Q * F + 7 * F + (F if (last and nu_p_positive) else 0)
                    + (Q * F if last else 0) + 2 * qlim)
                add("euler_dss_qdp", 1, Q * F + Q * Fd + (Q * Fd if last else 0))
                add("euler_dss_fvar", 1, 2 * F)
    add("dp3d_from_ps", 1, F)
    add("ppm_remap", 1, 7 * F + 2 * Q * Fd)
    add("update_q", 1, 2 * Q * Fd)
    return d


# ---- clocks sampled during the timed region ------------------------------------------------
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.samples = []
        self._stop = threading.Event()
        self._th = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", os.environ.get("HX_SMI_INDEX", "0"),
                                      f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits"],
                                     capture_output=True, text=True, timeout=5).stdout.strip()
                if out:
                    self.samples.append([x.strip() for x in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._th = threading.Thread(target=self._run, daemon=True)
        self._th.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._th:
            self._th.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4)
                          if len(s) > 3 + i and s[3 + i].lower().startswith("active")})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.samples)}


def _peaks():
    try:
        with open(MEASURED_PEAKS) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def _setup(lib_path, precision, mesh, hv, state, qsize=QSIZE):
    from hommexx_gb300 import abi
    L = abi.HxLibrary(lib_path)
    p = abi.SimParams(qsize=qsize, nu=NU, rsplit=RSPLIT, hypervis_subcycle=HSUB, nu_top=2.5e5,
                      limiter_option=8, remap_alg=1)
    L.init(mesh, hv, p, state, precision=precision, abort_on_error=True)
    return L


def _device_time(L, steps):
    L.lib.hx_timer_start()
    for _ in range(steps):
        L.run_subcycle(DT)
    import ctypes
    ms = ctypes.c_double(0)
    L.lib.hx_timer_stop(ctypes.byref(ms))
    return ms.value / 1e3


def run_gpu(args, rank, world):
    from hommexx_gb300 import build as B, mesh as M, state as S
    lib_path = B.build()
    mesh = M.build_mesh(NE)
    hv = S.hybrid_coordinate()
    state = S.initial_state(mesh, QSIZE, hv)
    out = {}
    forms = [f for f in args.forms.split(",") if f]
    for precision, tag in ((0, "fp64"), (1, "mixed")):
        if tag not in forms or (tag == "mixed" and args.no_mixed):
            continue
        L = _setup(lib_path, precision, mesh, hv, state)
        for _ in range(args.warmup):
            L.run_subcycle(DT)
        L.lib.hx_synchronize()
        _barrier(world)
        launches0 = L.lib.hx_launch_count()
        L.lib.hx_enable_timing(1)
        with ClockSampler() as cs:
            t = _device_time(L, args.steps)
        L.lib.hx_enable_timing(0)
        launches = L.lib.hx_launch_count() - launches0
        stats = L.kernel_stats()
        t = _max_over_ranks(t, world)
        # end-to-end through the C ABI with host buffers page-locked at allocation
        # (cudaHostAlloc through torch's pinned allocator, which raises rather than fall
        # back to pageable memory)
        import torch
        keep = []

        def pinned(shape, fill=None):
            t = torch.empty(tuple(shape), dtype=torch.float64, pin_memory=True)
            keep.append(t)
            a = t.numpy()
            if fill is not None:
                a[...] = fill
            return a

        # The state arrays are the source of init_elements_states_c and the destination
        # of cxx_push_results_to_f90, as the coupled driver's elem%state arrays are
        # (prim_driver_mod.F90:1380-1405): each interval starts from the previous one's
        # result; Q and omega_p are results only.
        res0 = L.push_results()
        host_in = {k: pinned(state[k].shape, state[k]) for k in ("v", "T", "dp3d", "Qdp", "ps_v")}
        res = {k: host_in[k] if k in host_in else pinned(v.shape) for k, v in res0.items()}
        del res0
        h2d = sum(a.nbytes for a in host_in.values())
        d2h = sum(a.nbytes for a in res.values())
        link = measure_link()  # the host link as this run sees it, just before the e2e loop
        L.set_async_copies(True)
        L.stream_results(res)
        L.set_state(host_in)
        L.run_subcycle(DT)
        L.push_results(res)
        _barrier(world)
        tp = [0.0, 0.0, 0.0]
        t0 = time.perf_counter()
        for _ in range(args.steps):
            ta = time.perf_counter()
            L.set_state(host_in)
            tb = time.perf_counter()
            L.run_subcycle(DT)
            tc = time.perf_counter()
            L.push_results(res)
            td = time.perf_counter()
            tp[0] += tb - ta
            tp[1] += tc - tb
            tp[2] += td - tc
        te = time.perf_counter() - t0
        te = _max_over_ranks(te, world)
        L.stream_results(None)
        L.set_async_copies(False)
        link_after = measure_link()  # the same test right after the loop
        calls = {"init_elements_states_c_ms": 1e3 * tp[0] / args.steps,
                 "prim_run_subcycle_c_ms": 1e3 * tp[1] / args.steps,
                 "cxx_push_results_to_f90_ms": 1e3 * tp[2] / args.steps}
        # init_elements_states_c returns once v, T, dp3d and ps_v are on the device: their
        # bytes over its wall time is the rate the host link gave this loop (the link test
        # above is a single copy with nothing else in flight)
        dyn_in = sum(host_in[k].nbytes for k in ("v", "T", "dp3d", "ps_v"))
        calls["init_h2d_gbs_effective"] = dyn_in / (tp[0] / args.steps) / 1e9 if tp[0] > 0 else None
        print(f"[e2e {tag}] per interval: " + ", ".join(f"{k[:-3]} {v:.2f} ms" for k, v in calls.items()
                                                      if k.endswith("_ms"))
              + f"; link h2d {link['h2d_gbs']:.1f} GB/s, d2h {link['d2h_gbs']:.1f} GB/s", file=sys.stderr)
        del keep
        out[tag] = dict(t=t, te=te, launches=launches, stats=stats, clocks=cs.summary(),
                        h2d=h2d, d2h=d2h, link=link, link_after=link_after, calls=calls)
        if tag == "fp64":
            out["fp64_state_after"] = None
        L.finalize()
    # error of the mixed form against the FP64 form after --error-days simulated days
    if not args.no_mixed and args.error_days > 0 and rank == 0:
        nsub = int(round(args.error_days * 86400.0 / SIM_SECONDS_PER_STEP))
        finals = {}
        for precision in (0, 1):
            L = _setup(lib_path, precision, mesh, hv, state)
            for _ in range(nsub):
                L.run_subcycle(DT)
            finals[precision] = L.push_results()
            L.finalize()
        a, b = finals[1], finals[0]
        err = {}
        for k, lab in (("v", "uv"), ("T", "T"), ("dp3d", "dp3d"), ("Qdp", "Qdp"), ("ps_v", "ps")):
            err[lab] = float(np.max(np.abs(a[k] - b[k])) / np.max(np.abs(b[k])))
        sm = mesh.spheremp
        m0 = float(np.sum(state["ps_v"][:, 1] * sm))
        out["mixed_error"] = dict(days=args.error_days, subcycles=nsub, rel_err=err,
                                  mass_drift_fp64=float(np.sum(b["ps_v"][:, 1] * sm) / m0 - 1.0),
                                  mass_drift_mixed=float(np.sum(a["ps_v"][:, 1] * sm) / m0 - 1.0))
    return out, mesh


ADJ_NE, ADJ_STEPS, ADJ_QSIZE = 16, 24, 4
LARGE_NE, LARGE_Q, LARGE_DT, LARGE_NU, LARGE_STEPS = 120, 40, 75.0, 1e13, 12
TRACER_KERNELS = ("precompute_divdp", "euler_qminmax", "euler_bih_pre", "euler_bih_post",
                  "euler_minmax_nbr", "euler_aal_setup", "euler_aal_tracer", "euler_dss_qdp",
                  "euler_dss_fvar")


def run_large(lib_path):
    """Large-mesh leg: ne120 L72 q40, dt 75 s, nu 1e13, 12 steps (4 remap intervals) in
    the mixed form against the FP64 form at the same size; SYPD of both, tracer-advection
    GB/s (field-pass bytes of the tracer kernels over their CUDA-event time), the mixed
    form's error after the 12 steps and the mass drift."""
    from hommexx_gb300 import abi, mesh as M, state as S
    t0 = time.perf_counter()
    mesh = M.build_mesh(LARGE_NE)
    hv = S.hybrid_coordinate()
    st = S.initial_state(mesh, LARGE_Q, hv)
    t_gen = time.perf_counter() - t0
    E = mesh.nelem
    nint = LARGE_STEPS // RSPLIT
    params = abi.SimParams(qsize=LARGE_Q, nu=LARGE_NU, rsplit=RSPLIT, hypervis_subcycle=HSUB,
                           nu_top=2.5e5, limiter_option=8, remap_alg=1)
    res, finals = {}, {}
    for precision, tag in ((0, "fp64"), (1, "mixed")):
        L = abi.HxLibrary(lib_path)
        L.init(mesh, hv, params, st, precision=precision, abort_on_error=True)
        L.lib.hx_enable_timing(1)
        import ctypes
        L.lib.hx_timer_start()
        for _ in range(nint):
            L.run_subcycle(LARGE_DT)
        ms = ctypes.c_double(0)
        L.lib.hx_timer_stop(ctypes.byref(ms))
        L.lib.hx_enable_timing(0)
        t = ms.value / 1e3
        stats = L.kernel_stats()
        model = kernel_bytes(E, LARGE_Q, 8)
        tr_ms = sum(r[2] for r in stats if r[0] in TRACER_KERNELS)
        tr_bytes = sum(model[r[0]][1] / model[r[0]][0] * r[1] for r in stats
                       if r[0] in TRACER_KERNELS and r[0] in model)
        n0 = L.tl[1]
        i_temp = (L.tl[3] - 1) // params.qsplit  # tracer level the last remap wrote
        q_tl = 1 if i_temp % 2 == 0 else 0
        finals[tag] = {"T": L.get("T", n0), "dp3d": L.get("dp3d", n0), "v": L.get("v", n0),
                       "ps_v": L.get("ps_v", n0), "Qdp": L.get("Qdp", q_tl)}
        res[tag] = {"sypd": nint * RSPLIT * LARGE_DT / (365.0 * t), "ms_per_interval": t / nint * 1e3,
                    "tracer_advection_gbs": tr_bytes / (tr_ms * 1e-3) / 1e9 if tr_ms else None,
                    "tracer_share": tr_ms / (sum(r[2] for r in stats) or 1.0)}
        L.finalize()
    a, b = finals["mixed"], finals["fp64"]
    res["mixed_rel_err"] = {k: float(np.max(np.abs(a[k] - b[k])) / np.max(np.abs(b[k])))
                            for k in ("v", "T", "dp3d", "Qdp", "ps_v")}
    sm = mesh.spheremp
    m0 = float(np.sum(st["ps_v"][:, 1] * sm))
    res["mass_drift"] = {tag: float(np.sum(finals[tag]["ps_v"] * sm) / m0 - 1.0) for tag in finals}
    res["speedup_mixed_vs_fp64"] = res["mixed"]["sypd"] / res["fp64"]["sypd"]
    res["workload"] = (f"ne{LARGE_NE} L72 ({E} elements) q{LARGE_Q}, dt {LARGE_DT:.0f} s, hv nu "
                       f"{LARGE_NU:g} x{HSUB} subcycles, remap every {RSPLIT} steps, "
                       f"{LARGE_STEPS} steps; input generation {t_gen:.0f} s on the host")
    return res


def _traj_call(fn, ins, outs, *mid):
    import ctypes
    a = [ctypes.c_void_p(t.data_ptr()) for t in ins]
    b = [ctypes.c_void_p(t.data_ptr()) for t in outs]
    rc = fn(*a, *mid, *b)
    if rc:
        raise RuntimeError(f"{fn.__name__} -> {rc}")


def _timed(L, f, reps=3):
    import ctypes
    ts = []
    for _ in range(reps):
        L.lib.hx_timer_start()
        f()
        ms = ctypes.c_double(0)
        L.lib.hx_timer_stop(ctypes.byref(ms))
        ts.append(ms.value)
    return float(np.median(ts))


def run_adjoint(lib_path, dot_check=True, forms=("fp64", "mixed")):
    """Adjoint leg: timings with the state resident on the device, then the checks."""
    import ctypes
    import torch
    from hommexx_gb300 import abi, mesh as M, state as S
    mesh = M.build_mesh(ADJ_NE)
    hv = S.hybrid_coordinate()
    st = S.initial_state(mesh, ADJ_QSIZE, hv)
    x0 = {"v": st["v"][:, 1], "T": st["T"][:, 1], "dp3d": st["dp3d"][:, 1]}
    w = mesh.spheremp[:, None]
    keys = ("v", "T", "dp3d")
    dev = lambda d: [torch.from_numpy(np.ascontiguousarray(d[k])).cuda() for k in keys]
    params = abi.SimParams(qsize=ADJ_QSIZE, nu=NU, rsplit=RSPLIT, hypervis_subcycle=HSUB,
                           nu_top=2.5e5)
    res = {}
    grads = {}
    for precision, tag in ((0, "fp64"), (1, "mixed")):
        if tag not in forms:
            continue
        L = abi.HxLibrary(lib_path)
        L.init(mesh, hv, params, st, precision=precision, abort_on_error=True)
        xin = dev(x0)
        xout = [torch.empty_like(t) for t in xin]
        gout = [torch.empty_like(t) for t in xin]
        torch.cuda.synchronize()
        fwd = lambda: _traj_call(L.lib.hx_traj_forward, xin, xout, ctypes.c_int(ADJ_STEPS),
                                 ctypes.c_double(DT))
        L.traj_checkpointing(2)
        fwd()
        t_plain = _timed(L, fwd)
        xf = {k: t.cpu().numpy() for k, t in zip(keys, xout)}
        bar = {"v": np.zeros_like(xf["v"]), "T": 2.0 * w * xf["T"], "dp3d": np.zeros_like(xf["dp3d"])}
        bard = dev(bar)
        torch.cuda.synchronize()
        vjp = lambda: _traj_call(L.lib.hx_traj_vjp, bard, gout)
        t_b2 = _timed(L, vjp)
        L.traj_checkpointing(1)
        fwd()
        t_f1 = _timed(L, fwd)
        t_b1 = _timed(L, vjp)
        # tangent-linear model: the trajectory again with its tangent beside it
        rng = np.random.default_rng(2025)
        tin = dev({k: rng.standard_normal(x0[k].shape) for k in keys})
        tout = [torch.empty_like(t) for t in xin]
        torch.cuda.synchronize()
        jvp = lambda: _traj_call(L.lib.hx_traj_jvp, tin, tout)
        t_j = _timed(L, jvp)
        L.lib.hx_enable_timing(1)
        vjp()
        L.lib.hx_enable_timing(0)
        stats = sorted(L.kernel_stats(), key=lambda r: -r[2])
        tot = sum(r[2] for r in stats) or 1.0
        grads[tag] = {k: t.cpu().numpy() for k, t in zip(keys, gout)}
        res[tag] = dict(forward_ms=t_plain, forward_checkpointed_ms=t_f1, vjp_ms=t_b1,
                        vjp_recompute_ms=t_b2,
                        gradient_cost_vs_forward=(t_f1 + t_b1) / t_plain,
                        reverse_sweep_vs_forward=t_b1 / t_plain,
                        recompute_mode_cost_vs_forward=(t_plain + t_b2) / t_plain,
                        jvp_ms=t_j, tangent_cost_vs_forward=t_j / t_plain,
                        vjp_kernels=[dict(kernel=n, launches=c, total_ms=round(ms, 3),
                                          share=round(ms / tot, 4)) for n, c, ms in stats[:6]])
        if tag == "fp64":
            # central finite differences of J along 10 smooth directions (host API)
            eps, worst = 1e-6, 0.0
            g = grads["fp64"]
            L.traj_checkpointing(2)
            for i in range(10):
                d = S.dynamics_direction(mesh, 7000 + i, hv)
                tp = L.traj_forward({k: x0[k] + eps * d[k] for k in keys}, ADJ_STEPS, DT)["T"]
                tm = L.traj_forward({k: x0[k] - eps * d[k] for k in keys}, ADJ_STEPS, DT)["T"]
                fd = float(np.sum(w * (tp - tm) * (tp + tm))) / (2 * eps)
                ad = sum(float(np.vdot(g[k], d[k])) for k in keys)
                worst = max(worst, abs(fd - ad) / abs(fd))
            res["fd_max_rel_err"] = worst
            if dot_check:
                rng = np.random.default_rng(2024)
                dx = {k: rng.standard_normal(x0[k].shape) for k in keys}
                dy = {k: rng.standard_normal(x0[k].shape) for k in keys}
                L.traj_forward(x0, ADJ_STEPS, DT)
                rhs = sum(float(np.vdot(dx[k], v)) for k, v in L.traj_vjp(dy).items())
                lhs_gpu = sum(float(np.vdot(v, dy[k])) for k, v in L.traj_jvp(dx).items())
                res["dot_product_gpu"] = dict(tlm_dot=lhs_gpu, adjoint_dot=rhs,
                                              rel_err=abs(lhs_gpu - rhs) / abs(lhs_gpu),
                                              tlm="CUDA tangent-linear model (hx_traj_jvp)")
        L.finalize()
    if len(grads) == 2:
        res["mixed_gradient_rel_err"] = {
            k: float(np.max(np.abs(grads["mixed"][k] - grads["fp64"][k])) / np.max(np.abs(grads["fp64"][k])))
            for k in keys}
    res["workload"] = (f"dry dynamics ne{ADJ_NE} L72 ({6 * ADJ_NE * ADJ_NE} elements), {ADJ_STEPS} steps "
                       f"of {DT:.0f} s, RK5 caar + hyperviscosity (nu {NU:g}, {HSUB} subcycles) + PPM "
                       f"remap every {RSPLIT} steps; J = sum spheremp T_final^2; gradient w.r.t. "
                       "initial u, v, T, dp3d")
    res["checkpoints"] = ("forward_checkpointed keeps every RK-stage, hyperviscosity-subcycle and "
                          "remap input; vjp_recompute keeps the step inputs only and recomputes each "
                          "step's stage inputs while reversing it")
    return res


def _barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def _max_over_ranks(x, world):
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def roofline(stats, E, Q, rsize, steps, form="fp64", hbm_peak=None, fp64_peak_tflops=None):
    """Per kernel: launches, CUDA-event time and share, algorithmic (field-pass) bytes per
    launch and the GB/s they give with their fraction of the HBM peak; the ncu DRAM bytes
    per launch; the FP64 FLOPs per launch (ncu instruction counts) and the TFLOP/s they
    give with their fraction of the measured FP64 peak."""
    model = kernel_bytes(E, Q, rsize)
    total = sum(ms for _, _, ms in stats) or 1.0
    rows = []
    for name, launches, ms in stats:
        nb = model.get(name)
        per_launch = nb[1] / nb[0] if nb else None
        t_launch = ms / launches * 1e-3 if launches else None
        gbs = per_launch / t_launch / 1e9 if (per_launch and t_launch) else None
        traffic, flops, inst = ncu_row(form, name, E, Q)
        tf = flops / t_launch / 1e12 if (flops and t_launch) else None
        ti = inst / t_launch / 1e12 if (inst and t_launch) else None
        rows.append(dict(kernel=name, launches=launches, total_ms=ms, share=ms / total,
                         bytes_per_launch=per_launch, gbs=gbs,
                         hbm_frac=gbs / hbm_peak if (gbs and hbm_peak) else None,
                         dram_bytes_per_launch_ncu=traffic,
                         fp64_flops_per_launch=flops, fp64_tflops=tf,
                         fp64_frac=tf / fp64_peak_tflops if (tf and fp64_peak_tflops) else None,
                         # FP64 instructions against the pipe's instruction rate (half the
                         # FMA FLOP peak): DADD and DMUL take a full slot for one FLOP
                         fp64_inst_frac=ti / (fp64_peak_tflops / 2) if (ti and fp64_peak_tflops) else None))
    rows.sort(key=lambda r: -r["total_ms"])
    return rows


def _rounded(r):
    return {k: (round(v, 4) if isinstance(v, float) and abs(v) < 1e6 else v) for k, v in r.items()}


def _oracle(mesh=None, state=None):
    from hommexx_gb300 import mesh as M, state as S
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    mesh = mesh or M.build_mesh(NE)
    hv = S.hybrid_coordinate()
    state = state or S.initial_state(mesh, QSIZE, hv)
    L = _setup(os.path.join(ROOT, "oracle", "liboracle.so"), 0, mesh, hv, state)
    L.lib.hx_oracle_threads.restype = int
    return L


def cpu_baseline(seconds_budget: float = 20.0, L=None):
    """Time the oracle on the machine's host cores on a bounded sample: ne30 with the same
    parameters for as many remap intervals as fit the budget (at least one)."""
    own = L is None
    L = L or _oracle()
    threads = L.lib.hx_oracle_threads()
    t0 = time.perf_counter()
    n = 0
    while True:
        L.run_subcycle(DT)
        n += 1
        if time.perf_counter() - t0 > seconds_budget / 2 or n >= 4:
            break
    t = time.perf_counter() - t0
    if own:
        L.finalize()
    return dict(value=sypd(n, t), unit="SYPD", cores=threads, kind="port",
                sample=f"ne{NE} L72 q{QSIZE}, {n} remap interval(s) of 3 x 300 s steps, "
                       f"{t:.1f} s on {threads} OpenMP threads")


def main():
    global NE, QSIZE
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--no-mixed", action="store_true")
    ap.add_argument("--forms", default="fp64,mixed",
                    help="forms to time: fp64, mixed or both (profiling runs time one; with "
                         "--only-adjoint, the adjoint leg's forms)")
    ap.add_argument("--error-days", type=float, default=1.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--ne", type=int, default=NE, help="cubed-sphere resolution (profiling cases)")
    ap.add_argument("--qsize", type=int, default=QSIZE, help="tracer count (profiling cases)")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint leg")
    ap.add_argument("--no-dot-check", action="store_true",
                    help="skip the dot-product check of the adjoint leg")
    ap.add_argument("--only-adjoint", action="store_true",
                    help="run the adjoint leg alone and print its JSON (profiling runs)")
    ap.add_argument("--large", action="store_true",
                    help="run the ne120 q40 mixed-vs-FP64 leg alone and print its JSON "
                         "(needs ~200 GB of device and ~150 GB of host memory)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    NE, QSIZE = args.ne, args.qsize

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local_rank)
        os.environ["HX_SMI_INDEX"] = str(local_rank)
        import torch.distributed as dist
        dist.init_process_group("gloo")

    config = {"workload": f"preqx step ne{NE} L72 np4 qsize{QSIZE}, dt 300 s, rsplit 3, hv nu 1e15 x3 "
                          "subcycles, limiter 8, PPM mirrored remap",
              "elements": 6 * NE * NE, "nlev": 72, "qsize": QSIZE, "step": "one remap interval "
              "(prim_run_subcycle_c) = 3 x 300 s", "l2": "working set 1.9 GB >> 129 MB L2, no flush",
              "parallelism": f"replicas x{world}" if world > 1 else "single GPU"}

    if args.impl == "reference":
        if rank != 0:
            return
        L = _oracle()
        threads = L.lib.hx_oracle_threads()
        times = []
        for i in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            L.run_subcycle(DT)
            if i >= args.warmup:
                times.append(time.perf_counter() - t0)
        L.finalize()
        v = sypd(len(times), float(np.sum(times)))
        per = [dict(value=v, unit="SYPD", cores=threads, kind="port",
                    sample=f"ne{NE} L72 q{QSIZE}, one remap interval (3 x 300 s) per step, "
                           f"{np.mean(times):.2f} s per step on {threads} OpenMP threads")]
        line = {"metric": "ne30L72 SYPD (FP64 preqx step)", "value": v, "unit": "SYPD",
                "impl": "reference", "n_gpus": 0, "steps": args.steps, "warmup": args.warmup,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic seeded spherical-harmonic state", "config": config,
                "cpu_baseline": dict(per[-1], value=v),
                "e2e": {"value": v, "unit": "SYPD", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    if args.large:
        if rank == 0:
            from hommexx_gb300 import build as B
            print(json.dumps(run_large(B.build())))
        return
    if args.only_adjoint:
        if rank == 0:
            from hommexx_gb300 import build as B
            print(json.dumps(run_adjoint(B.build(), dot_check=not args.no_dot_check,
                                         forms=[f for f in args.forms.split(",") if f])))
        return
    out, mesh = run_gpu(args, rank, world)
    if rank != 0:
        return
    E = mesh.nelem
    if "fp64" not in out:  # profiling run of the mixed form alone
        m = out["mixed"]
        print(json.dumps({"metric": "ne30L72 SYPD (mixed preqx step)", "value": sypd(args.steps, m["t"]),
                          "unit": "SYPD", "ms_per_step": m["t"] / args.steps * 1e3,
                          "kernels": roofline(m["stats"], E, QSIZE, 8, args.steps, "mixed")}))
        return
    f = out["fp64"]
    peak, peak_kind = _peaks()
    from hommexx_gb300 import build as B
    f64peak = fp64_peak(B.build())
    rows = roofline(f["stats"], E, QSIZE, 8, args.steps, "fp64", peak, f64peak)
    top = rows[0]
    # The binding roof of the top kernel: the FP64 pipe when its FP64 fraction is the
    # larger, else HBM.
    if top["fp64_frac"] is not None and top["fp64_frac"] > (top["hbm_frac"] or 0.0):
        roof = {"bound": "fp64", "kernel": top["kernel"], "achieved": top["fp64_tflops"], "peak": f64peak,
                "unit": "TFLOP/s", "frac": top["fp64_frac"], "fp64_inst_frac": top["fp64_inst_frac"],
                "peak_source": "measured in this run (hx_fp64_peak: independent DFMA chains, full occupancy)",
                "hbm": {"achieved": top["gbs"], "peak": peak, "unit": "GB/s", "frac": top["hbm_frac"],
                        "peak_source": peak_kind}}
    else:
        roof = {"bound": "hbm", "kernel": top["kernel"], "achieved": top["gbs"], "peak": peak, "unit": "GB/s",
                "frac": top["hbm_frac"], "peak_source": peak_kind, "fp64_peak_tflops": f64peak}
    roof["traffic"] = top["dram_bytes_per_launch_ncu"]
    roof["traffic_source"] = "ncu DRAM bytes per launch at ne16, scaled by elements"
    roof["achieved_source"] = ("algorithmic bytes (field passes) or ncu FP64 FLOPs per launch over the "
                               "kernel's CUDA-event launch time in this run")
    value = sypd(args.steps, f["t"]) * world
    ms_dev = f["t"] / args.steps * 1e3
    ms_e2e = f["te"] / args.steps * 1e3
    line = {
        "metric": "ne30L72 SYPD (FP64 preqx step)", "value": value, "unit": "SYPD",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_dev, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic seeded spherical-harmonic state",
        "config": config,
        "e2e": {"value": sypd(args.steps, f["te"]) * world, "unit": "SYPD",
                "h2d_bytes_per_step": f["h2d"], "d2h_bytes_per_step": f["d2h"],
                "ms_per_step": ms_e2e, "exposed_ms_per_step": ms_e2e - ms_dev,
                "link": f["link"], "link_after_loop": f["link_after"], "calls": f["calls"],
                "copies": "init_elements_states_c / prim_run_subcycle_c / cxx_push_results_to_f90 "
                          "with the state arrays (page-locked at allocation) both source and "
                          "destination, as the coupled driver's; Qdp in and the results out overlap "
                          "the step (hx_set_async_copies, hx_stream_results)"},
        "gpu_launches": f["launches"],
        "clocks": f["clocks"],
        "roofline": roof,
        "kernels": [_rounded(r) for r in rows],
    }
    if "mixed" in out:
        mx = out["mixed"]
        mrows = roofline(mx["stats"], E, QSIZE, 8, args.steps, "mixed", peak, f64peak)
        ms_m = mx["t"] / args.steps * 1e3
        line["mixed"] = {"value": sypd(args.steps, mx["t"]) * world, "unit": "SYPD",
                         "speedup_vs_fp64": f["t"] / mx["t"],
                         "e2e": sypd(args.steps, mx["te"]) * world,
                         "e2e_ms_per_step": mx["te"] / args.steps * 1e3, "ms_per_step": ms_m,
                         "e2e_calls": mx["calls"],
                         "top_kernels": [{k: r[k] for k in ("kernel", "share", "gbs", "hbm_frac")}
                                         for r in mrows[:3]],
                         "interval_hbm_frac": (sum(v[1] for v in kernel_bytes(E, QSIZE, 8).values())
                                               / (ms_m * 1e-3) / 1e9 / peak),
                         "kernels": [_rounded(r) for r in mrows],
                         "clocks": mx["clocks"]}
        if "mixed_error" in out:
            line["mixed"]["error_vs_fp64"] = out["mixed_error"]
    if not args.no_adjoint:
        line["adjoint"] = run_adjoint(os.path.join(ROOT, "hommexx_gb300", "libhxgpu.so"),
                                      dot_check=not args.no_dot_check)
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline()
    print(json.dumps(line))


if __name__ == "__main__":
    main()
