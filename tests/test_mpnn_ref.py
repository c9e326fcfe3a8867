"""CPU checks of the network's FP64 restatement (oracle/mpnn_ref.py), the
checker of the CUDA forward/backward kernels: its backward pass against
central finite differences, its aggregation adjoint, and BF16 rounding."""
import numpy as np

from oracle import mpnn_ref as R


def _graph(n, rng, G):
    ptr, idx, val = [0], [], []
    for i in range(n):
        k = int(rng.integers(1, 5))
        nb = rng.choice(np.setdiff1d(np.arange(n), [i]), size=k, replace=False)
        w = rng.uniform(0.2, 1.0, k)
        idx += list(nb)
        val += list(w / w.sum())
        ptr.append(len(idx))
    return np.array(ptr), np.array(idx), np.array(val), rng.standard_normal((n, G))


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(0)
    F, H, O, L, G, N = 7, 6, 5, 2, 3, 12
    params = R.init_params(F, H, O, L, G, seed=1)
    for k in params:
        if k.startswith("b"):
            params[k] = rng.standard_normal(params[k].shape) * 0.1
    graph = _graph(N, rng, G)
    x = rng.standard_normal((N, F))
    t = rng.standard_normal((N, O))
    # eps = 1e-4: central differences are O(eps^2) here, and smaller steps
    # lose digits to cancellation on gradients of order 1e-6
    assert R.finite_difference_check(params, x, graph, t, L, n_probe=8, eps=1e-4) <= 1e-5


def test_aggregate_adjoint():
    rng = np.random.default_rng(2)
    wp, wi, wv, _ = _graph(15, rng, 1)
    a = rng.standard_normal((15, 4))
    b = rng.standard_normal((15, 4))
    lhs = np.sum(R.aggregate(wp, wi, wv, a) * b)
    rhs = np.sum(a * R.aggregate_T(wp, wi, wv, b))
    assert abs(lhs - rhs) <= 1e-13 * max(abs(lhs), 1.0)


def test_bf16_round_ties_to_even():
    x = np.array([1.0, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -8, -2.5, 1.0 + 2.0 ** -9])
    got = R.bf16_round(x)
    assert got[0] == 1.0
    assert got[1] == 1.0                      # tie -> even mantissa
    assert got[2] == 1.0 + 4 * 2.0 ** -8      # tie -> even (rounds up)
    assert got[3] == -2.5
    assert got[4] == 1.0


def test_gated_backward_matches_finite_differences():
    rng = np.random.default_rng(3)
    Np, B = 2, 2
    nd = 3 * Np
    F, H, L, G, N = B * nd + 3, 6, 1, 3, 10
    O = 6 * B
    params = R.init_params(F, H, O, L, G, seed=4)
    for k in params:
        if k.startswith("b"):
            params[k] = rng.standard_normal(params[k].shape) * 0.1
    graph = _graph(N, rng, G)
    x = rng.standard_normal((N, F))
    t = rng.standard_normal((N, 2 * nd))
    assert R.finite_difference_check(params, x, graph, t, L, n_probe=8, eps=1e-4, gate=(nd, B)) <= 1e-5


def test_gate_adjoint():
    rng = np.random.default_rng(5)
    nd, B, N = 9, 3, 4
    x = rng.standard_normal((N, B * nd + 2))
    y = rng.standard_normal((N, 6 * B))
    g = rng.standard_normal((N, 2 * nd))
    lhs = np.sum(R.gate_apply(y, x, nd, B) * g)
    rhs = np.sum(y * R.gate_adjoint(g, x, nd, B))
    assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), 1.0)
