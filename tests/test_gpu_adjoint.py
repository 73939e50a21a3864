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
* the mixed form's gradient is close to the FP64 one;
* the CUDA tangent-linear model (hx_traj_jvp) = the oracle's dual-number tangent to
  1e-10 (remap every step and every third step, remap_alg 1 and 2, with and without
  the nu_top sponge), passes the dot-product test against the CUDA adjoint to 1e-12,
  matches central finite differences of the CUDA forward, leaves the adjoint of the
  trajectory unchanged, and in the mixed form stays close to the FP64 tangent.
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


@pytest.mark.parametrize("nsteps,kw", [(3, dict(rsplit=1)), (3, dict(rsplit=3)),
                                       (2, dict(rsplit=1, remap_alg=2, nu_top=0.0)),
                                       (2, dict(rsplit=2, nu_div=3e16))])
def test_jvp_matches_oracle(oracle_path, gpu_path, nsteps, kw):
    o, g = _both(oracle_path, gpu_path, **kw)
    x0 = _x0(NE)
    o.traj_forward(x0, nsteps, DT)
    g.traj_forward(x0, nsteps, DT)
    dx = _rand(x0, 61)
    to = o.traj_jvp(dx)
    tg = g.traj_jvp(dx)
    for k in to:
        assert H.rel_err(tg[k], to[k]) < 1e-10, (k, H.rel_err(tg[k], to[k]))


@pytest.mark.parametrize("rsplit", [1, 3])
def test_gpu_dot_product(gpu_path, rsplit):
    """<L dx, dy> = <dx, L^T dy> with both sides on the GPU."""
    g = H.setup(gpu_path, NE, 1, rsplit=rsplit)
    x0 = _x0(NE)
    g.traj_forward(x0, 3, DT)
    dx, dy = _rand(x0, 71), _rand(x0, 72)
    lhs = _dot(g.traj_jvp(dx), dy)
    rhs = _dot(dx, g.traj_vjp(dy))
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs), (lhs, rhs)


def test_jvp_matches_finite_differences(gpu_path):
    """Without a remap the step is smooth: the tangent = central FD of the CUDA forward
    per field; with remaps (PPM limiters are only piecewise smooth, so single points
    near a limiter switch differ) the projections on seeded random fields agree."""
    m = H.mesh(NE)
    x0 = _x0(NE)
    eps = 1e-6
    g = H.setup(gpu_path, NE, 1, rsplit=3)
    g.traj_forward(x0, 2, DT)  # 2 steps, no remap
    for i in range(2):
        d = S.dynamics_direction(m, 7100 + i)
        tl = g.traj_jvp(d)
        fp = g.traj_forward({k: x0[k] + eps * d[k] for k in x0}, 2, DT)
        fm = g.traj_forward({k: x0[k] - eps * d[k] for k in x0}, 2, DT)
        for k in tl:
            fd = (fp[k] - fm[k]) / (2 * eps)
            assert H.rel_err(tl[k], fd) < 1e-6, (i, k, H.rel_err(tl[k], fd))
        g.traj_forward(x0, 2, DT)
    g = H.setup(gpu_path, NE, 1, rsplit=1)
    g.traj_forward(x0, 3, DT)
    w = _rand(x0, 97)
    for i in range(3):
        d = S.dynamics_direction(m, 7200 + i)
        tl = g.traj_jvp(d)
        fp = g.traj_forward({k: x0[k] + eps * d[k] for k in x0}, 3, DT)
        fm = g.traj_forward({k: x0[k] - eps * d[k] for k in x0}, 3, DT)
        fd = {k: (fp[k] - fm[k]) / (2 * eps) for k in tl}
        a, b = _dot(tl, w), _dot(fd, w)
        assert abs(a - b) <= 1e-4 * abs(b), (i, a, b)
        g.traj_forward(x0, 3, DT)


def test_jvp_leaves_vjp_unchanged(gpu_path):
    g = H.setup(gpu_path, NE, 1, rsplit=1)
    x0 = _x0(NE)
    bar = _rand(x0, 81)
    for mode in (1, 2):
        g.traj_checkpointing(mode)
        g.traj_forward(x0, 2, DT)
        want = g.traj_vjp(bar)
        g.traj_jvp(_rand(x0, 82))
        got = g.traj_vjp(bar)
        for k in want:
            assert np.array_equal(got[k], want[k]), (mode, k)
    g.traj_checkpointing(0)


def test_mixed_jvp_close_to_fp64(gpu_path):
    x0 = _x0(NE)
    dx = _rand(x0, 91)
    tans = []
    for prec in (0, 1):
        g = H.setup(gpu_path, NE, 1, precision=prec, rsplit=1)
        g.traj_forward(x0, 3, DT)
        tans.append(g.traj_jvp(dx))
    for k in tans[0]:
        assert H.rel_err(tans[1][k], tans[0][k]) < 1e-3, (k, H.rel_err(tans[1][k], tans[0][k]))


def test_jvp_of_no_steps_is_identity(gpu_path):
    g = H.setup(gpu_path, NE, 1, rsplit=1)
    x0 = _x0(NE)
    g.traj_forward(x0, 0, DT)
    dx = _rand(x0, 95)
    got = g.traj_jvp(dx)
    for k in dx:
        assert np.array_equal(got[k], dx[k]), k
