"""The CUDA library's dry-dynamics trajectory and its hand-written adjoint, against the
CPU oracle (forward, vector-Jacobian product and tangent-linear model) and against
central finite differences of the CUDA forward.

* forward trajectory = oracle trajectory to 1e-12 (relative, per field);
* VJP = oracle VJP to 1e-10 after 3 steps (remap every step, and every third step);
* dot-product test <L dx, dy> (oracle tangent-linear model) = <dx, L^T dy> (CUDA
  adjoint) to 1e-10;
* both checkpointing modes (every stage input kept / recomputed per step) give
  bit-identical gradients;
* the gradient of J = sum spheremp T_final^2 matches central finite differences of
  the CUDA forward (eps = 1e-6) along 10 seeded smooth directions;
* the mixed form's gradient is close to the FP64 one.
"""
import numpy as np
import pytest

import hxtest as H
from hommexx_gb300 import state as S

pytestmark = pytest.mark.gpu

DT = 300.0
NE = 4


def _x0(ne):
    st = H.state(ne, 1)
    return {"v": st["v"][:, 1], "T": st["T"][:, 1], "dp3d": st["dp3d"][:, 1]}


def _rand(x0, seed):
    rng = np.random.default_rng(seed)
    sc = {"v": 1.0, "T": 1.0, "dp3d": 10.0}
    return {k: rng.standard_normal(x0[k].shape) * sc[k] for k in x0}


def _dot(a, b):
    return sum(float(np.vdot(a[k], b[k])) for k in a)


def _both(oracle_path, gpu_path, **kw):
    o = H.setup(oracle_path, NE, 1, **kw)
    g = H.setup(gpu_path, NE, 1, **kw)
    return o, g


@pytest.mark.parametrize("nsteps,rsplit", [(3, 1), (3, 3)])
def test_forward_and_vjp_match_oracle(oracle_path, gpu_path, nsteps, rsplit):
    o, g = _both(oracle_path, gpu_path, rsplit=rsplit)
    x0 = _x0(NE)
    fo = o.traj_forward(x0, nsteps, DT)
    fg = g.traj_forward(x0, nsteps, DT)
    for k in fo:
        assert H.rel_err(fg[k], fo[k]) < 1e-12, k
    bar = _rand(x0, 31)
    go = o.traj_vjp(bar)
    gg = g.traj_vjp(bar)
    for k in go:
        assert H.rel_err(gg[k], go[k]) < 1e-10, (k, H.rel_err(gg[k], go[k]))


def test_dot_product_with_oracle_tangent(oracle_path, gpu_path):
    o, g = _both(oracle_path, gpu_path, rsplit=1)
    x0 = _x0(NE)
    o.traj_forward(x0, 3, DT)
    g.traj_forward(x0, 3, DT)
    dx, dy = _rand(x0, 41), _rand(x0, 42)
    lhs = _dot(o.traj_jvp(dx), dy)
    rhs = _dot(dx, g.traj_vjp(dy))
    assert abs(lhs - rhs) <= 1e-10 * abs(lhs), (lhs, rhs)


def test_checkpointing_modes_agree(gpu_path):
    g = H.setup(gpu_path, NE, 1, rsplit=1)
    x0 = _x0(NE)
    bar = _rand(x0, 51)
    out = []
    for mode in (1, 2):
        g.traj_checkpointing(mode)
        g.traj_forward(x0, 2, DT)
        out.append(g.traj_vjp(bar))
    g.traj_checkpointing(0)
    for k in out[0]:
        assert np.array_equal(out[0][k], out[1][k]), k


def test_gradient_matches_finite_differences(gpu_path):
    g = H.setup(gpu_path, NE, 1, rsplit=1)
    m = H.mesh(NE)
    w = m.spheremp[:, None]
    x0 = _x0(NE)
    nsteps = 3
    xf = g.traj_forward(x0, nsteps, DT)
    bar = {"v": np.zeros_like(xf["v"]), "T": 2.0 * w * xf["T"], "dp3d": np.zeros_like(xf["dp3d"])}
    grad = g.traj_vjp(bar)
    eps = 1e-6
    worst = 0.0
    for i in range(10):
        d = S.dynamics_direction(m, 7000 + i)
        tp = g.traj_forward({k: x0[k] + eps * d[k] for k in x0}, nsteps, DT)["T"]
        tm = g.traj_forward({k: x0[k] - eps * d[k] for k in x0}, nsteps, DT)["T"]
        fd = float(np.sum(w * (tp - tm) * (tp + tm))) / (2 * eps)
        worst = max(worst, abs(fd - _dot(grad, d)) / abs(fd))
    assert worst < 1e-4, worst


def test_mixed_gradient_close_to_fp64(gpu_path):
    m = H.mesh(NE)
    w = m.spheremp[:, None]
    x0 = _x0(NE)
    grads = []
    for prec in (0, 1):
        g = H.setup(gpu_path, NE, 1, precision=prec, rsplit=1)
        xf = g.traj_forward(x0, 3, DT)
        bar = {"v": np.zeros_like(xf["v"]), "T": 2.0 * w * xf["T"],
               "dp3d": np.zeros_like(xf["dp3d"])}
        grads.append(g.traj_vjp(bar))
    for k in grads[0]:
        assert H.rel_err(grads[1][k], grads[0][k]) < 1e-3, (k, H.rel_err(grads[1][k], grads[0][k]))
