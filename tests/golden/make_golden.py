"""Regenerates tests/golden/oracle_ne2_q2.npz: the CPU oracle's results for one remap
interval at ne=2 (24 elements), 72 levels, 2 tracers, dt=300 s, rsplit=1, on the
seeded state of hommexx_gb300.state.  A regression pin of the oracle across hosts
(x86_64 here, aarch64 on the GPU machine; the oracle is built without FMA contraction).

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

LEVELS = [0, 1, 2, 35, 70, 71]


def run_case():
    import hxtest as H
    H.build_oracle()
    L = H.setup(H.ORACLE_SO, 2, 2, nu=1e16, rsplit=1)
    L.run_subcycle(300.0)
    r = L.push_results()
    n0 = L.tl[1]
    out = {
        "T": r["T"][:, n0][:, LEVELS], "dp3d": r["dp3d"][:, n0][:, LEVELS],
        "v": r["v"][:, n0][:, LEVELS], "Qdp": r["Qdp"][:, :, :, LEVELS],
        "Q": r["Q"][:, :, LEVELS], "ps_v": r["ps_v"][:, n0], "omega_p": r["omega_p"][:, LEVELS],
    }
    sums = {f"sum_{k}": np.array([np.sum(r[k]), np.sum(np.abs(r[k]))]) for k in r}
    out.update(sums)
    return out


if __name__ == "__main__":
    np.savez_compressed(os.path.join(HERE, "oracle_ne2_q2.npz"), **run_case())
    print("written")
