"""The CPU oracle's dry-dynamics trajectory, its tangent-linear model and its adjoint.

* the trajectory forward equals the full oracle step (v, T and the remapped dp3d);
* the tangent-linear model (the oracle's own templated step run with dual numbers)
  matches central finite differences of the forward;
* the hand-written adjoint passes the dot-product test <L dx, dy> = <dx, L^T dy>
  against that tangent-linear model, for the option combinations the step has
  (remap every step or every third, remap_alg 1 and 2, nu_top on and off,
  nu_div != nu);
* the gradient of J = sum spheremp T_final^2 matches central finite differences
  (eps = 1e-6) along 10 seeded smooth directions.
"""
import numpy as np
import pytest

import hxtest as H
from hommexx_gb300 import abi, state as S

DT = 300.0


def _x0(ne):
    st = H.state(ne, 1)
    return {"v": st["v"][:, 1], "T": st["T"][:, 1], "dp3d": st["dp3d"][:, 1]}


def _rand(x0, seed):
    rng = np.random.default_rng(seed)
    sc = {"v": 1.0, "T": 1.0, "dp3d": 10.0}
    return {k: rng.standard_normal(x0[k].shape) * sc[k] for k in x0}


def _dot(a, b):
    return sum(float(np.vdot(a[k], b[k])) for k in a)


def test_trajectory_step_equals_full_step(oracle_path):
    ne = 2
    L = H.setup(oracle_path, ne, 2, rsplit=1)
    x1 = L.traj_forward(_x0(ne), 1, DT)
    L = H.setup(oracle_path, ne, 2, rsplit=1)
    L.run_subcycle(DT)
    r = L.push_results()
    n0 = L.tl[1]
    assert np.array_equal(x1["v"], r["v"][:, n0])
    assert np.array_equal(x1["T"], r["T"][:, n0])
    hv = H.hvc()
    dp = (np.diff(hv.hyai)[None, :, None, None] * hv.ps0
          + np.diff(hv.hybi)[None, :, None, None] * r["ps_v"][:, n0][:, None])
    assert H.rel_err(x1["dp3d"], dp) < 1e-15


def test_tangent_matches_finite_differences(oracle_path):
    """Without a remap the step is smooth: TLM = central FD to round-off."""
    ne = 2
    L = H.setup(oracle_path, ne, 1, rsplit=2)
    x0 = _x0(ne)
    L.traj_forward(x0, 1, DT)
    d = _rand(x0, 11)
    tl = L.traj_jvp(d)
    eps = 1e-6
    fp = L.traj_forward({k: x0[k] + eps * d[k] for k in x0}, 1, DT)
    fm = L.traj_forward({k: x0[k] - eps * d[k] for k in x0}, 1, DT)
    for k in tl:
        fd = (fp[k] - fm[k]) / (2 * eps)
        assert H.rel_err(fd, tl[k]) < 1e-6, k


@pytest.mark.parametrize("nsteps,kw", [
    (3, dict(rsplit=3)),
    (2, dict(rsplit=1)),
    (2, dict(rsplit=1, remap_alg=2, nu_top=0.0)),
    (2, dict(rsplit=1, nu_div=2.5e16, hypervis_subcycle=1)),
    (4, dict(rsplit=2, nu_s=5e15, nu_p=2e16)),
])
def test_dot_product(oracle_path, nsteps, kw):
    ne = 2
    L = H.setup(oracle_path, ne, 1, **kw)
    x0 = _x0(ne)
    L.traj_forward(x0, nsteps, DT)
    dx, dy = _rand(x0, 21), _rand(x0, 22)
    lhs = _dot(L.traj_jvp(dx), dy)
    rhs = _dot(dx, L.traj_vjp(dy))
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs), (lhs, rhs)


def test_gradient_matches_finite_differences(oracle_path):
    """J = sum spheremp T^2 at the end of 3 steps with a remap after each; central FD
    with eps = 1e-6 along 10 seeded smooth directions.  The FD of J is formed as
    sum w (T+ - T-)(T+ + T-) / (2 eps) so that it does not cancel in J itself."""
    ne, nsteps = 2, 3
    L = H.setup(oracle_path, ne, 1, rsplit=1)
    m = H.mesh(ne)
    w = m.spheremp[:, None]
    x0 = _x0(ne)
    xf = L.traj_forward(x0, nsteps, DT)
    bar = {"v": np.zeros_like(xf["v"]), "T": 2.0 * w * xf["T"],
           "dp3d": np.zeros_like(xf["dp3d"])}
    g = L.traj_vjp(bar)
    eps = 1e-6
    worst = 0.0
    for i in range(10):
        d = S.dynamics_direction(m, 7000 + i)
        tp = L.traj_forward({k: x0[k] + eps * d[k] for k in x0}, nsteps, DT)["T"]
        tm = L.traj_forward({k: x0[k] - eps * d[k] for k in x0}, nsteps, DT)["T"]
        fd = float(np.sum(w * (tp - tm) * (tp + tm))) / (2 * eps)
        worst = max(worst, abs(fd - _dot(g, d)) / abs(fd))
    assert worst < 1e-4, worst


def test_trajectory_errors(oracle_path):
    L = H.setup(oracle_path, 2, 1)
    L.lib.hx_set_abort_on_error(0)
    x0 = _x0(2)
    with pytest.raises(RuntimeError, match="201"):
        L.traj_vjp(x0)                       # no forward trajectory yet
    bad = {k: v.copy() for k, v in x0.items()}
    bad["dp3d"][0, 5] = -1.0
    with pytest.raises(RuntimeError, match="101"):
        L.traj_forward(bad, 1, DT)
    m = H.M.build_mesh(2, hypervis_scaling=3.2)
    L.finalize()
    L.init(m, H.hvc(), abi.SimParams(qsize=1, nu=3e-8, hypervis_scaling=3.2), H.state(2, 1))
    with pytest.raises(RuntimeError, match="12"):
        L.traj_forward(x0, 1, DT)
