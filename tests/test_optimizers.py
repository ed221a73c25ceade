"""The host optimizers of mole_gb300/api.py against the update rules of
src/optimize/src/optimizers.rs:45-192, fed a fixed gradient sequence through a
stub sampler result: MomentumDescent (m -= step g; delta = mu m),
NesterovMomentum (m_prev = m; m = mu m + step g; delta = -(mu m_prev + (1 + mu) m))
and OnlineLbfgs (the two-loop recursion over a history of curvature pairs,
with the reference's 1e-10 first-step scale, its averaged later scale, its
oldest-first history wrap-around and its second update_curvature_pairs call
after the direction, which stores every pair twice). The first updates are
also worked out by hand."""
import numpy as np

from mole_gb300 import api


class Stub:
    def __init__(self, g):
        self.g = np.asarray(g, dtype=np.float64)

    def energy_gradient(self):
        return self.g.copy()


GRADS = [np.array(v) for v in ([1.0, -2.0], [0.5, 0.5], [-0.25, 1.5], [0.8, -0.1], [0.3, 0.9], [-1.2, 0.4], [0.05, -0.7])]
PARS = [np.array(v) for v in ([0.9, 0.4], [1.1, 0.35], [1.0, 0.6], [0.95, 0.5], [1.2, 0.45], [1.05, 0.55], [0.98, 0.52])]


def test_momentum_descent():
    opt = api.MomentumDescent(0.1, 0.9, 2)
    d0 = opt.compute_parameter_update(PARS[0], Stub(GRADS[0]))
    np.testing.assert_allclose(d0, [-0.09, 0.18], rtol=0, atol=1e-15)  # m = [-0.1, 0.2]
    d1 = opt.compute_parameter_update(PARS[1], Stub(GRADS[1]))
    np.testing.assert_allclose(d1, [-0.135, 0.135], rtol=0, atol=1e-15)  # m = [-0.15, 0.15]
    m = np.array([-0.15, 0.15])
    for p, g in zip(PARS[2:], GRADS[2:]):
        m = m - 0.1 * g
        np.testing.assert_allclose(opt.compute_parameter_update(p, Stub(g)), 0.9 * m, rtol=0, atol=1e-15)


def test_nesterov_momentum():
    opt = api.NesterovMomentum(0.1, 0.9, 2)
    d0 = opt.compute_parameter_update(PARS[0], Stub(GRADS[0]))
    np.testing.assert_allclose(d0, [-0.19, 0.38], rtol=0, atol=1e-15)  # m = [0.1, -0.2]
    d1 = opt.compute_parameter_update(PARS[1], Stub(GRADS[1]))
    np.testing.assert_allclose(d1, [-0.356, 0.427], rtol=0, atol=1e-15)  # m = [0.14, -0.13]
    m_prev, m = np.array([0.1, -0.2]), np.array([0.14, -0.13])
    for p, g in zip(PARS[2:], GRADS[2:]):
        m_prev, m = m, 0.9 * m + 0.1 * g
        np.testing.assert_allclose(opt.compute_parameter_update(p, Stub(g)), -(0.9 * m_prev + 1.9 * m),
                                   rtol=0, atol=1e-15)


def lbfgs_reference(step, history, pars_seq, grad_seq):
    """optimizers.rs:109-192 written out with plain lists (oldest pair first)."""
    n = len(pars_seq[0])
    s_list, y_list = [], []
    grad_prev, pars_prev = [1e-5] * n, [1e-5] * n
    it = 0
    out = []

    def dot(a, b):
        return sum(x * y for x, y in zip(a, b))

    def push(pars, g):
        s = [a - b for a, b in zip(pars, pars_prev)]
        y = [a - b for a, b in zip(g, grad_prev)]
        if len(s_list) >= history:
            s_list.pop(0)
        s_list.append(s)
        if len(y_list) >= history:
            y_list.pop(0)
        y_list.append(y)

    for pars, g in zip(pars_seq, grad_seq):
        pars, g = list(pars), list(g)
        push(pars, g)
        p = [-v for v in g]
        alphas = []
        for s, y in zip(reversed(s_list), reversed(y_list)):  # newest first
            a = dot(s, p) / dot(s, y)
            p = [pi - a * yi for pi, yi in zip(p, y)]
            alphas.append(a)
        if it == 0:
            scale = 1e-10
        else:
            scale = sum(dot(s, y) / dot(y, y) for s, y in zip(s_list, y_list)) / min(it, history)
        p = [pi * scale for pi in p]
        for a, s, y in zip(reversed(alphas), s_list, y_list):  # oldest first
            c = a - dot(y, p) / dot(y, s)
            p = [pi + c * si for pi, si in zip(p, s)]
        out.append([-step * v for v in p])
        push(pars, g)  # the reference stores the pair a second time
        grad_prev, pars_prev = g, pars
        it += 1
    return out


def test_online_lbfgs_matches_two_loop_recursion_with_wraparound():
    step, history = 0.5, 3
    opt = api.OnlineLbfgs(step, history, 2)
    ref = lbfgs_reference(step, history, PARS, GRADS)
    for k, (p, g) in enumerate(zip(PARS, GRADS)):
        d = opt.compute_parameter_update(p, Stub(g))
        np.testing.assert_allclose(d, ref[k], rtol=1e-12, atol=1e-300)
        # two pushes per call, capped at the history length (oldest dropped)
        assert len(opt.s) == min(2 * (k + 1), history)
    # the first step by hand: one pair s = p0 - 1e-5, y = g0 - 1e-5, scale 1e-10
    s = PARS[0] - 1e-5
    y = GRADS[0] - 1e-5
    p = -GRADS[0]
    a = s.dot(p) / s.dot(y)
    p = (p - a * y) * 1e-10
    p = p + (a - y.dot(p) / y.dot(s)) * s
    np.testing.assert_allclose(ref[0], -step * p, rtol=1e-14)
    # history wrap-around: after the second call the oldest copy of the first pair is gone
    opt2 = api.OnlineLbfgs(step, history, 2)
    opt2.compute_parameter_update(PARS[0], Stub(GRADS[0]))
    opt2.compute_parameter_update(PARS[1], Stub(GRADS[1]))
    np.testing.assert_allclose(opt2.s[0], PARS[0] - 1e-5)
    np.testing.assert_allclose(opt2.s[1], PARS[1] - PARS[0])
    np.testing.assert_allclose(opt2.s[2], PARS[1] - PARS[0])
