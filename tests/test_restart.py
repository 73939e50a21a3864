"""Restart files of the oracle (hx_write_restart / hx_read_restart; the format of
include/hxgpu.h, which stands in for src/restart_io_mod.F90): the documented layout and
checksum, bit-identical continuation of a run through a restart, and the errors the
reader reports (size mismatch as CheckRestartHeader, src/restart_io_mod.F90:440-471;
corruption; missing file)."""
import numpy as np
import pytest

import hxtest as H
from hommexx_gb300 import abi

DT = 300.0
NE, Q = 2, 3
HX_ERR_IO = 202


def splitmix_checksum(words: np.ndarray) -> int:
    """The format's checksum: sum mod 2^64 of splitmix64(w_k + (k+1) * golden)."""
    k = np.arange(1, words.size + 1, dtype=np.uint64)
    z = words + k * np.uint64(0x9E3779B97F4A7C15)
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    z = z ^ (z >> np.uint64(31))
    return int(np.sum(z, dtype=np.uint64))


def record_segments(E, Qs):
    """(name, words) of one element record, in file order."""
    return [("v", 3 * 72 * 2 * 16), ("T", 3 * 72 * 16), ("dp3d", 3 * 72 * 16), ("ps_v", 48),
            ("phis", 16), ("Q", Qs * 72 * 16), ("Qdp", 2 * Qs * 72 * 16)]


def parse_restart(path, E, Qs):
    h = abi.HxLibrary.read_restart_header(path)
    raw = np.fromfile(path, dtype=np.uint8)
    words = raw[128:].view(np.uint64)
    rw = sum(w for _, w in record_segments(E, Qs))
    rec = raw[128:].view(np.float64).reshape(E, rw)
    out, off = {}, 0
    for name, w in record_segments(E, Qs):
        out[name] = rec[:, off:off + w]
        off += w
    return h, out, words


@pytest.fixture
def ora(oracle_path):
    return oracle_path


def test_restart_layout_and_checksum(ora, tmp_path):
    L = H.setup(ora, NE, Q, rsplit=3)
    L.run_subcycle(DT)
    f = tmp_path / "r.bin"
    L.write_restart(f)
    r = L.push_results()
    E = L.nelem
    h, seg, words = parse_restart(f, E, Q)
    assert h["magic"] == b"HXRESTRT" and h["version"] == 1 and h["header_bytes"] == 128
    assert (h["nelem"], h["np"], h["nlev"], h["qsize"], h["timelevels"], h["qsize_timelevels"]) == \
        (E, 4, 72, Q, 3, 2)
    assert [h["nm1"] - 1, h["n0"] - 1, h["np1"] - 1, h["nstep"]] == L.tl
    rw = sum(w for _, w in record_segments(E, Q))
    assert h["record_bytes"] == 8 * rw
    assert f.stat().st_size == 128 + E * 8 * rw
    for k in ("v", "T", "dp3d", "ps_v", "Q", "Qdp"):
        assert np.array_equal(seg[k], r[k].reshape(E, -1)), k
    assert np.array_equal(seg["phis"], H.mesh(NE).phis.reshape(E, -1))
    assert splitmix_checksum(words) == h["checksum"]


@pytest.mark.parametrize("rsplit", [3, 0])
def test_restart_continuation_is_bit_identical(ora, tmp_path, rsplit):
    """Two intervals in one run equal one interval, a restart into a fresh session
    (initialised from a different state), and the second interval."""
    f = tmp_path / "r.bin"
    L = H.setup(ora, NE, Q, rsplit=rsplit)
    L.run_subcycle(DT)
    L.write_restart(f)
    L.run_subcycle(DT)
    want, tl = L.push_results(), list(L.tl)
    L = H.setup(ora, NE, Q, rsplit=rsplit)
    st = {k: v.copy() for k, v in H.state(NE, Q).items()}
    st["T"] += 1.0
    L.set_state(st)
    L.read_restart(f)
    L.run_subcycle(DT)
    got = L.push_results()
    assert L.tl == tl
    for k in want:
        assert np.array_equal(got[k], want[k]), k


def test_restart_errors(ora, tmp_path):
    f = tmp_path / "r.bin"
    L = H.setup(ora, NE, Q, rsplit=3)
    L.write_restart(f)
    # a corrupted record byte fails the checksum
    raw = bytearray(f.read_bytes())
    raw[128 + 4321] ^= 0x10
    bad = tmp_path / "bad.bin"
    bad.write_bytes(bytes(raw))
    assert L.lib.hx_read_restart(str(bad).encode()) == HX_ERR_IO
    assert "checksum" in L.last_error()[1]
    # a truncated file
    short = tmp_path / "short.bin"
    short.write_bytes(bytes(raw[: len(raw) // 2]))
    assert L.lib.hx_read_restart(str(short).encode()) == HX_ERR_IO
    # not a restart file; missing file
    junk = tmp_path / "junk.bin"
    junk.write_bytes(b"\0" * 256)
    assert L.lib.hx_read_restart(str(junk).encode()) == HX_ERR_IO
    assert L.lib.hx_read_restart(str(tmp_path / "none.bin").encode()) == HX_ERR_IO
    # a session of another size (qsize) rejects the file
    L2 = H.setup(ora, NE, Q - 1, rsplit=3)
    assert L2.lib.hx_read_restart(str(f).encode()) == HX_ERR_IO
    assert "does not match" in L2.last_error()[1]
