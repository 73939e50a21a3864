"""Restart files of the CUDA library against the oracle's (same format, include/hxgpu.h):
byte-identical files from identical states, bit-identical continuation through a
restart, files exchanged between the two libraries, multi-chunk streaming, and a
mixed-form session reading an FP64 file."""
import numpy as np
import pytest

import hxtest as H
from test_restart import HX_ERR_IO, parse_restart, splitmix_checksum

pytestmark = pytest.mark.gpu

DT = 300.0
TOL = 1e-12


def test_restart_file_matches_oracle_bytes(gpu_path, oracle_path, tmp_path):
    fg, fo = tmp_path / "g.bin", tmp_path / "o.bin"
    H.setup(gpu_path, 4, 4, rsplit=3).write_restart(fg)
    H.setup(oracle_path, 4, 4, rsplit=3).write_restart(fo)
    assert fg.read_bytes() == fo.read_bytes()


@pytest.mark.parametrize("precision,rsplit", [(0, 3), (1, 3), (0, 0)])
def test_restart_continuation_gpu(gpu_path, tmp_path, precision, rsplit):
    """Two intervals in one run equal one interval, restart, one interval (bit for bit),
    in the FP64 and mixed forms and with the vertically Eulerian step."""
    f = tmp_path / "r.bin"
    L = H.setup(gpu_path, 4, 4, precision=precision, rsplit=rsplit)
    L.run_subcycle(DT)
    L.write_restart(f)
    L.run_subcycle(DT)
    want, tl = L.push_results(), list(L.tl)
    L = H.setup(gpu_path, 4, 4, precision=precision, rsplit=rsplit)
    L.read_restart(f)
    L.run_subcycle(DT)
    got = L.push_results()
    assert L.tl == tl
    for k in want:
        assert np.array_equal(got[k], want[k]), k


@pytest.mark.parametrize("writer", ["gpu", "oracle"])
def test_restart_exchanged_between_libraries(gpu_path, oracle_path, tmp_path, writer):
    """One interval on the writer, the file read by the other library, one more interval
    on both: within the FP64 parity bound."""
    f = tmp_path / "r.bin"
    paths = dict(gpu=gpu_path, oracle=oracle_path)
    reader = "oracle" if writer == "gpu" else "gpu"
    W = H.setup(paths[writer], 4, 4, rsplit=3)
    W.run_subcycle(DT)
    W.write_restart(f)
    W.run_subcycle(DT)
    rw = W.push_results()
    R = H.setup(paths[reader], 4, 4, rsplit=3)
    R.read_restart(f)
    R.run_subcycle(DT)
    rr = R.push_results()
    errs = {k: H.rel_err(rr[k], rw[k]) for k in rw}
    assert all(v <= TOL for v in errs.values()), errs


def test_restart_multi_chunk_and_mixed_reader(gpu_path, tmp_path):
    """ne16 q4: 340 MB of records, more than one 256 MiB staging buffer.  The file is
    written by an FP64 session and read by a mixed-form session (all state is FP64 in
    both forms; phis is converted for the FP32 operators)."""
    f = tmp_path / "r.bin"
    L = H.setup(gpu_path, 16, 4, rsplit=3)
    L.run_subcycle(DT)
    L.write_restart(f)
    r64 = L.push_results()
    E = L.nelem
    h, seg, words = parse_restart(f, E, 4)
    assert h["record_bytes"] * E > 256 << 20
    assert splitmix_checksum(words) == h["checksum"]
    for k in ("v", "T", "dp3d", "ps_v", "Qdp", "Q"):
        assert np.array_equal(seg[k], r64[k].reshape(E, -1)), k
    M = H.setup(gpu_path, 16, 4, precision=1, rsplit=3)
    M.read_restart(f)
    rm = M.push_results()
    for k in ("v", "T", "dp3d", "ps_v", "Qdp", "Q"):  # omega_p is derived, not restarted
        assert np.array_equal(rm[k], r64[k]), k
    M.run_subcycle(DT)
    L = H.setup(gpu_path, 16, 4, rsplit=3)
    L.read_restart(f)
    L.run_subcycle(DT)
    a, b = M.push_results(), L.push_results()
    assert H.rel_err(a["T"], b["T"]) < 1e-6 and H.rel_err(a["dp3d"], b["dp3d"]) < 1e-6


def test_restart_errors_gpu(gpu_path, tmp_path):
    f = tmp_path / "r.bin"
    L = H.setup(gpu_path, 4, 4, rsplit=3)
    L.write_restart(f)
    raw = bytearray(f.read_bytes())
    raw[128 + 99991] ^= 0x01
    bad = tmp_path / "bad.bin"
    bad.write_bytes(bytes(raw))
    # the checksum is verified before anything is uploaded: a failed read leaves the
    # session's state as it was
    L.run_subcycle(DT)
    before = L.push_results()
    assert L.lib.hx_read_restart(str(bad).encode()) == HX_ERR_IO
    assert "checksum" in L.last_error()[1]
    short = tmp_path / "short.bin"
    short.write_bytes(f.read_bytes()[: len(raw) - 4096])
    assert L.lib.hx_read_restart(str(short).encode()) == HX_ERR_IO
    assert "short read" in L.last_error()[1]
    after = L.push_results()
    for k in before:
        assert np.array_equal(before[k], after[k]), k
    assert L.lib.hx_read_restart(str(tmp_path / "none.bin").encode()) == HX_ERR_IO
    L2 = H.setup(gpu_path, 4, 3, rsplit=3)
    assert L2.lib.hx_read_restart(str(f).encode()) == HX_ERR_IO
    assert "does not match" in L2.last_error()[1]
