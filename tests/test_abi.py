"""The C ABI: libhxgpu.so loads without a GPU and exports every function
include/hxgpu.h declares; the oracle exports the same reference-facing set."""
import ctypes
import os
import re
import subprocess

import pytest

import hxtest as H

HEADER = os.path.join(H.ROOT, "include", "hxgpu.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?(?:void|int|long long|double)\s*\**\s*(\w+)\s*\(",
                       src, flags=re.M)
    return sorted(set(names))


REFERENCE_SYMBOLS = [
    "initialize_hommexx_session", "finalize_hommexx_session", "reset_cxx_comm",
    "init_connectivity", "add_connection", "finalize_connectivity", "init_derivative_c",
    "init_simulation_params_c", "init_hvcoord_c", "init_elements_2d_c",
    "init_elements_states_c", "init_diagnostics_c", "init_boundary_exchanges_c",
    "init_time_level_c", "prim_run_subcycle_c", "cxx_push_results_to_f90",
]


def exported(path):
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True,
                         check=True).stdout
    return {l.split()[-1] for l in out.splitlines() if " T " in l}


def test_header_declares_reference_surface():
    decl = declared_functions()
    for s in REFERENCE_SYMBOLS:
        assert s in decl
    assert len(decl) >= len(REFERENCE_SYMBOLS) + 20


def test_gpu_library_exports_every_declared_function(gpu_lib_cpu):
    ctypes.CDLL(gpu_lib_cpu)          # loads without a GPU
    exp = exported(gpu_lib_cpu)
    missing = [n for n in declared_functions() if n not in exp]
    assert not missing, missing


def test_bounds_checked_build_exports_every_declared_function():
    """The debug build with device index checks (HX_BOUNDS_CHECK) compiles, loads without
    a GPU and says so in hx_build_flags."""
    import sys
    from hommexx_gb300 import build as B
    path = B.build(bounds_check=True)
    # loaded in a process of its own: its kernels carry the regular library's names
    r = subprocess.run([sys.executable, "-c", f"import ctypes; print(ctypes.CDLL({path!r}).hx_build_flags())"],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == "1", r.stdout + r.stderr
    exp = exported(path)
    missing = [n for n in declared_functions() if n not in exp]
    assert not missing, missing


def test_oracle_exports_reference_surface(oracle_path):
    exp = exported(oracle_path)
    device_only = ("hx_dss_noalloc", "hx_cube_mesh", "hx_fp64_peak", "hx_build_flags")
    missing = [n for n in declared_functions() if n not in exp and n not in device_only]
    assert not missing, missing


def test_no_fallback_symbols_in_product(gpu_lib_cpu):
    """The product library carries no CPU implementation of the step: none of the
    oracle's test hooks, and it needs the CUDA runtime."""
    exp = exported(gpu_lib_cpu)
    assert not any(n.startswith("hx_oracle") for n in exp)
    deps = subprocess.run(["ldd", gpu_lib_cpu], capture_output=True, text=True).stdout
    assert "libcudart" in deps


def test_host_side_errors_without_gpu(gpu_lib_cpu):
    """Without a device the library reports instead of falling back."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    L = ctypes.CDLL(gpu_lib_cpu)
    L.hx_set_abort_on_error(0)
    L.initialize_hommexx_session()
    buf = ctypes.create_string_buffer(256)
    assert L.hx_last_error(buf, 256) == 200
    assert L.hx_run_prim_step.restype is not None
    L.hx_run_prim_step.argtypes = [ctypes.c_double]
    assert L.hx_run_prim_step(300.0) == 201   # no session: state error, not a CPU run


def test_c_driver_links_and_reports(gpu_lib_cpu, tmp_path):
    """include/hxgpu.h compiles as C, a C driver links libhxgpu.so and gets the status
    codes of the host-side paths (tests/c/abi_from_c.c)."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    exe = str(tmp_path / "abi_from_c")
    libdir = os.path.dirname(gpu_lib_cpu)
    subprocess.run(["gcc", "-std=c11", "-Wall", "-Werror", "-I", os.path.join(H.ROOT, "include"),
                    os.path.join(H.ROOT, "tests", "c", "abi_from_c.c"), "-L", libdir, "-lhxgpu",
                    f"-Wl,-rpath,{libdir}", "-o", exe], check=True, capture_output=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr
