"""Direct-stiffness-summation gather tables built from element connections.

Restates the connection bookkeeping of the reference DSS:

* point lists per connection slot and direction:
  ``src/share/cxx/mpi/ConnectivityHelpers.hpp:150-205``;
* direction of a (local slot, remote slot) pair:
  ``src/share/cxx/mpi/ConnectivityHelpers.hpp:129-139``;
* pack reads the sender's points ``CONNECTION_PTS[dir][sender_slot]``
  (``src/share/cxx/mpi/BoundaryExchange.cpp:343-364``);
* unpack accumulation order ``for k: for edge in S,N,W,E`` then corners
  ``SW,SE,NW,NE`` (``src/share/cxx/mpi/BoundaryExchange.cpp:505-538``).

The result is, for every (element, point), the ordered list of (source element,
source point) values that are added to the element's own value.  The CUDA library
builds the same table in C++ from the ``add_connection`` calls; this copy serves the
mesh generator (``rspheremp``) and the tests.
"""
from __future__ import annotations

import numpy as np

NP = 4
S, N, W, E, SW, SE, NW, NE = range(8)
FWD, BWD = 0, 1

_PTS_FWD = {
    S: [0, 1, 2, 3], N: [12, 13, 14, 15], W: [0, 4, 8, 12], E: [3, 7, 11, 15],
    SW: [0], SE: [3], NW: [12], NE: [15],
}
_PTS_BWD = {k: (list(reversed(v)) if k < 4 else v) for k, v in _PTS_FWD.items()}

_DIR = [
    [BWD, FWD, FWD, BWD],   # S with remote S,N,W,E
    [FWD, BWD, BWD, FWD],   # N
    [FWD, BWD, BWD, FWD],   # W
    [BWD, FWD, FWD, BWD],   # E
]

MAX_SRC = 3


def connection_points(direction: int, slot: int):
    return (_PTS_FWD if direction == FWD else _PTS_BWD)[slot]


def direction(local_slot: int, remote_slot: int) -> int:
    if local_slot < 4:
        return _DIR[local_slot][remote_slot]
    return FWD


def build_gather_table(conn: np.ndarray):
    """conn[e][slot] = (remote elem, remote slot) or -1.  Returns (src_e, src_p, cnt)
    with shapes (E,16,3), (E,16,3), (E,16) in the reference accumulation order."""
    nelem = conn.shape[0]
    src_e = np.zeros((nelem, 16, MAX_SRC), dtype=np.int32)
    src_p = np.zeros((nelem, 16, MAX_SRC), dtype=np.int32)
    cnt = np.zeros((nelem, 16), dtype=np.int32)

    def add(e, p, se, sp):
        c = cnt[e, p]
        src_e[e, p, c] = se
        src_p[e, p, c] = sp
        cnt[e, p] = c + 1

    for e in range(nelem):
        for k in range(NP):
            for slot in (S, N, W, E):
                r, rs = int(conn[e, slot, 0]), int(conn[e, slot, 1])
                if r < 0:
                    continue
                d = direction(rs, slot)
                add(e, _PTS_FWD[slot][k], r, connection_points(d, rs)[k])
        for slot in (SW, SE, NW, NE):
            r, rs = int(conn[e, slot, 0]), int(conn[e, slot, 1])
            if r < 0:
                continue
            add(e, _PTS_FWD[slot][0], r, _PTS_FWD[rs][0])
    return src_e, src_p, cnt
