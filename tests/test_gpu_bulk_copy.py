"""The bulk asynchronous copy helpers of hx_device.cuh (bulk_load, mbar_wait), which the
tracer advection uses to stream each tracer's Qdp slab into shared memory: slabs
streamed one ahead through one shared buffer arrive bit for bit, and a wait on a
barrier phase that never completes gives up after its bounded polls, so the kernel
exits and the context stays usable (tests/cuda/bulk_copy_check.cu)."""
import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def test_bulk_copies_and_bounded_wait(tmp_path):
    from hommexx_gb300 import build as B
    exe = str(tmp_path / "bulk_copy_check")
    subprocess.run([B.nvcc(), *B.flags(), "-o", exe, os.path.join(HERE, "cuda", "bulk_copy_check.cu")],
                   check=True, capture_output=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
