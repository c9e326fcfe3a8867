"""GPU tests of the learned surrogate: the network's CUDA kernels against the
FP64 numpy restatement in oracle/mpnn_ref.py, the device-built surrogate
block, the leapfrog energy, the fallback controller, and what the trained
network gains over the extrapolation it corrects.

Bars (written in each assertion):
  * forward output, loss and every parameter gradient: normwise relative
    difference <= 2e-5 (FP32 activations and accumulation on the device,
    FP64 in the oracle; the same BF16-rounded weights on both sides);
  * one Adam step: the FP32 update formula in numpy, <= 1e-6 relative;
  * the surrogate block without the network equals the extrapolation
    u1 + k d1 + k(k+1)/2 d2 computed in numpy, <= 1e-14 relative;
  * leapfrog energy: the oracle's blocks and mass matrices, <= 1e-12;
  * the residual after the closing plain step: the host's, <= 1e-10;
  * a network whose predictions fail the residual or energy check leaves
    the state bit for bit where the plain stepper puts it, and so do judged
    blocks;
  * the trained network's mean relative prediction error on held-out solver
    trajectories is below 0.8 x that of the extrapolation alone.
"""
import math
from ctypes import byref, c_double

import numpy as np
import pytest

from lymph3d_apsc_gb300 import MatrixFree, _lib, mesh as M
from lymph3d_apsc_gb300 import ensemble as E
from lymph3d_apsc_gb300 import surrogate as S
from oracle import mpnn_ref as R

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    d = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (d if d > 0 else 1.0))


def _random_graph(n, rng, G):
    ptr = [0]
    idx, val = [], []
    for i in range(n):
        k = int(rng.integers(1, 7))
        nb = rng.choice(np.setdiff1d(np.arange(n), [i]), size=k, replace=False)
        w = rng.uniform(0.2, 1.0, k)
        idx += list(nb)
        val += list(w / w.sum())
        ptr.append(len(idx))
    g = rng.standard_normal((n, G))
    return (np.array(ptr, np.int32), np.array(idx, np.int32), np.array(val, np.float32), g.astype(np.float32))


def _net_and_ref(F=21, H=32, O=10, L=2, G=8, N=64, seed=0, gate=None):
    """A network, its parameters in the oracle's form, a random graph and
    inputs.  Draws are repeated until no pre-activation of the oracle's
    forward lies within 1e-5 of its tensor's largest magnitude from the ReLU
    kink (ten times the device's FP32 rounding there), so that rounding
    cannot flip a ReLU mask (a flipped mask changes a gradient by an O(1)
    amount in one entry)."""
    net = S.MPNN(F, O, H=H, L=L, G=G, seed=seed, gate=gate)
    for attempt in range(200):
        rng = np.random.default_rng(seed + 1000 * attempt)
        flat = net.init_params(seed + 1000 * attempt)
        d = net.unpack(flat)
        for k, v in d.items():  # non-zero biases and a visible output layer
            if k.startswith("b"):
                v[...] = rng.standard_normal(v.shape) * 0.1
        flat = np.concatenate([d[k].ravel() for k, _ in net.shapes()]).astype(np.float32)
        flat[-O - H * O:-O] *= 10.0
        graph = _random_graph(N, rng, G)
        ref = {}
        for k, v in net.unpack(flat).items():
            ref[k] = R.bf16_round(v) if k.startswith("W") else v.astype(np.float64)
        g64 = tuple(np.asarray(a, np.float64) if a.dtype.kind == "f" else a for a in graph)
        x = rng.standard_normal((N, F)).astype(np.float32)
        _, cache = R.forward(ref, x.astype(np.float64), g64, L, keep=True, gate=gate)
        zs = [cache["z0"]] + [z for l in range(L) for z in (cache[l][1], cache[l][4])]
        if all(np.abs(z).min() > 1e-5 * np.abs(z).max() for z in zs):
            break
    else:
        raise AssertionError("no draw without near-kink pre-activations")
    net.set_params(flat)
    net.set_graph(graph)
    return net, flat, ref, g64, x


GATED = dict(F=32, O=12, gate=(9, 2))  # Np = 3, two basis blocks of 9 DOFs


# F = 21 (not a multiple of 4) runs the SIMT forward GEMMs, F = 24 the
# tensor-core ones (tcgen05, TF32 hi/lo split of the activations)
@pytest.mark.parametrize("F,gated", [(21, False), (24, False), (32, True)])
def test_forward_matches_oracle(require_gpu, F, gated):
    net, _, ref, graph, x = _net_and_ref(F=F, **({k: v for k, v in GATED.items() if k != "F"} if gated else {}))
    y = net.forward(x)
    y_ref = R.forward(ref, x.astype(np.float64), graph, net.L, gate=net.gate)
    assert rel(y, y_ref) <= 2e-5
    net.close()


@pytest.mark.parametrize("L,gated,F", [(0, False, 21), (1, False, 24), (3, False, 24), (2, True, 32)])
def test_gradients_match_oracle(require_gpu, L, gated, F):
    net, _, ref, graph, x = _net_and_ref(L=L, seed=L + 1, F=F, **({k: v for k, v in GATED.items() if k != "F"}
                                                                     if gated else {}))
    t = np.random.default_rng(9).standard_normal((x.shape[0], net.out_width)).astype(np.float32)
    loss = net.loss_grad(x, t)
    loss_ref, g_ref = R.loss_and_grad(ref, x.astype(np.float64), graph, t.astype(np.float64), L, gate=net.gate)
    assert abs(loss - loss_ref) <= 2e-5 * loss_ref
    _, g = net.params_and_grads()
    gd = net.unpack(g)
    for k in g_ref:
        assert rel(gd[k], g_ref[k]) <= 2e-5, k
    net.close()


@pytest.mark.parametrize("ws", ["1", "0"])
def test_tensor_core_forward_equals_simt_on_a_large_graph(require_gpu, monkeypatch, ws):
    """1,000 nodes (8 row tiles, a partial last one), H = 256, three layers:
    the tcgen05 forward (the TMA warp-specialised kernel, ws = 1, and the
    cp.async kernel, ws = 0) and the SIMT forward agree to FP32 rounding (the
    activations' lo part keeps 10 of its 13 bits: ~2^-21 per operand)."""
    rng = np.random.default_rng(11)
    F, H, O, L, N = 64, 256, 24, 3, 1000
    graph = _random_graph(N, rng, 8)
    x = rng.standard_normal((N, F)).astype(np.float32)
    outs = []
    monkeypatch.setenv("LYMPH_UMMA_WS", ws)
    for simt in ("0", "1"):
        monkeypatch.setenv("LYMPH_MPNN_SIMT", simt)
        net = S.MPNN(F, O, H=H, L=L, seed=7)
        flat = net.init_params(7)
        flat[-O - H * O:-O] *= 10.0
        net.set_params(flat)
        net.set_graph(graph)
        outs.append(net.forward(x).astype(np.float64))
        net.close()
    assert rel(outs[0], outs[1]) <= 2e-5


def test_adam_step_matches_formula(require_gpu):
    net, flat, _, _, x = _net_and_ref(seed=4)
    t = np.zeros((x.shape[0], net.O), np.float32)
    net.loss_grad(x, t)
    p0, g = net.params_and_grads()
    lr, b1, b2, eps = 1e-3, 0.9, 0.999, 1e-8
    net.adam(lr, b1, b2, eps)
    p1, _ = net.params_and_grads()
    g = g.astype(np.float32)
    m = (1 - b1) * g
    v = (1 - b2) * g * g
    want = p0 - lr * (m / (1 - b1)) / (np.sqrt(v / (1 - b2)) + eps)
    assert rel(p1, want) <= 1e-6
    assert rel(p1, p0) > 0
    net.close()


def _free_vibration(n=3, p=2, seed=0, material=None):
    m = M.cube(n, bc="dirichlet", agglomeration="bfs", seed=seed, group=(4, 12), jitter=0.1,
               **({"material": material} if material else {}))
    s = MatrixFree(m, p, 1.0)
    s.MAKE_MATRICES_FREE()
    s.MAKE_RHS_FREE(_lib.RHS_STAT, _lib.F_NULL, _lib.GD_NULL, _lib.GN_NULL)
    s.MAKE_RHS_FREE(_lib.RHS_DYN, _lib.F_NULL, _lib.GD_NULL, _lib.GN_NULL)
    lam = E.max_eigenvalue(s, 80)
    E.set_dt(s, 0.8 * 2.0 / math.sqrt(lam))
    s.COMPUTE_MODAL_COEFFICIENTS_FREE(_lib.FUN_IC_DISPLACEMENT, _lib.SLOT_U0)
    s.COMPUTE_MODAL_COEFFICIENTS_FREE(_lib.FUN_IC_VELOCITY, _lib.SLOT_V0)
    _lib.check(s.lib.lymph_first_step_g(s.ctx, 0.0), "first_step_g")
    return m, s


def test_energy_matches_oracle_blocks(require_gpu):
    from oracle.oracle_py import Oracle
    m, s = _free_vibration(material=(1.0, 1.0, 1.0))
    S.run_plain(s, 5, lambda t: 0.0, 2 * s.dt)
    ua, ub = s.get_state(_lib.SLOT_U0), s.get_state(_lib.SLOT_UN)
    o = Oracle(m, s.degree, s.dt)
    o.make_matrices()
    nd = o.nd
    Ku = np.zeros_like(ua)
    for (P, Q), blk in o.block_dict(0).items():
        Ku[P] += blk @ ua[Q]
    kin = 0.0
    for P, Mp in enumerate(o.mass(0)):
        d = (ub[P] - ua[P]) / s.dt
        for i in range(3):
            sl = slice(i * o.Np, (i + 1) * o.Np)
            kin += d[sl] @ Mp @ d[sl]
    want = 0.5 * kin + 0.5 * float(np.sum(ub * Ku))
    assert abs(S.energy(s) - want) <= 1e-12 * abs(want)
    o.close()
    s.close()


def test_plain_leapfrog_conserves_energy(require_gpu):
    """lambda = mu: the operator is symmetric and the leapfrog energy is
    conserved to rounding; the controller's 1e-4 drift bar sits far above."""
    _, s = _free_vibration(material=(1.0, 1.0, 1.0))
    e0 = S.energy(s)
    S.run_plain(s, 300, lambda t: 0.0, s.dt)
    assert abs(S.energy(s) - e0) <= 1e-9 * abs(e0)
    s.close()


def _block_start(s, n_before=6):
    """Steps a little, then sets up a block: V0 = u^{n-1}; returns the host
    copies (um, u0, u1) after the block's opening plain step."""
    S.run_plain(s, n_before, lambda t: 0.0, s.dt)
    um = s.get_state(_lib.SLOT_U0).copy()
    _lib.check(s.lib.lymph_copy_state(s.ctx, _lib.SLOT_V0, _lib.SLOT_U0), "copy")
    S.run_plain(s, 1, lambda t: 0.0, 0.0)
    return um, s.get_state(_lib.SLOT_U0).copy(), s.get_state(_lib.SLOT_UN).copy()


def _host_a1(m, s, d1, gdiff=0.0):
    """dt^2 M^-1 (K d1 - gdiff F_dyn) from the oracle's blocks and mass
    matrices and the device's source vector."""
    from oracle.oracle_py import Oracle
    o = Oracle(m, s.degree, s.dt)
    o.make_matrices()
    Kd = np.zeros_like(d1)
    for (P, Q), blk in o.block_dict(0).items():
        Kd[P] += blk @ d1[Q]
    Kd -= gdiff * s.rhs(_lib.RHS_DYN)
    out = np.zeros_like(d1)
    for P, Mp in enumerate(o.mass(0)):
        for i in range(3):
            sl = slice(i * o.Np, (i + 1) * o.Np)
            out[P, sl] = np.linalg.solve(Mp, Kd[P, sl])
    o.close()
    return s.dt ** 2 * out


def test_block_without_network_is_the_extrapolation(require_gpu):
    """The block's prediction equals the Taylor extrapolation computed on the
    host from the device's a1 term (bit-level arithmetic check); a1 itself
    is checked against the oracle in test_device_features_match_host."""
    m, s = _free_vibration(p=3)
    um, u0, u1 = _block_start(s)
    K = 8
    feat = S.surrogate_net(s.degree, H=16, L=0)
    feat.set_graph(S.build_graph(m), "g")
    _, _, a1, _ = S.device_features(s, feat)  # the a1 the prediction below computes again
    sc = (c_double * 4)()
    _lib.check(s.lib.lymph_surrogate_predict(s.ctx, S._dummy_net().h, K, 0, 0.0, sc), "predict")
    d1 = u1 - u0
    d2 = (u1 - 2.0 * u0) + um
    assert rel(s.get_state(_lib.SLOT_U0), S.baseline(u1, d1, d2, a1, K - 3)) <= 1e-14
    assert rel(s.get_state(_lib.SLOT_UN), S.baseline(u1, d1, d2, a1, K - 2)) <= 1e-14
    assert np.array_equal(s.get_state(_lib.SLOT_V0), u0)
    assert np.array_equal(s.get_state(_lib.SLOT_UEX), u1)
    n = u1.size
    want = [math.sqrt(np.sum(v * v) / n) for v in (u1, d1, d2, a1)]
    assert max(abs(a - b) / b for a, b in zip(sc, want)) <= 1e-12
    feat.close()
    # the residual after the closing plain step, against the host's
    S.run_plain(s, 1, lambda t: 0.0, 0.0)
    ua, ub = s.get_state(_lib.SLOT_U0), s.get_state(_lib.SLOT_UN)
    r = c_double()
    _lib.check(s.lib.lymph_surrogate_residual(s.ctx, S._dummy_net().h, byref(r)), "residual")
    want_r = np.linalg.norm(ub - S.baseline(u1, d1, d2, a1, K - 1)) / np.linalg.norm(ub)
    assert abs(r.value - want_r) <= 1e-6 * want_r + 1e-10
    # the judge: keep this pair, redo the block plainly, compare on the device
    _lib.check(s.lib.lymph_surrogate_judge(s.ctx, S._dummy_net().h, 0, None), "judge")
    _lib.check(s.lib.lymph_copy_state(s.ctx, _lib.SLOT_U0, _lib.SLOT_V0), "copy")
    _lib.check(s.lib.lymph_copy_state(s.ctx, _lib.SLOT_UN, _lib.SLOT_UEX), "copy")
    S.run_plain(s, K - 1, lambda t: 0.0, 0.0)
    j = c_double()
    _lib.check(s.lib.lymph_surrogate_judge(s.ctx, S._dummy_net().h, 1, byref(j)), "judge")
    va, vb = s.get_state(_lib.SLOT_U0), s.get_state(_lib.SLOT_UN)
    want_j = np.linalg.norm(np.concatenate([va - ua, vb - ub])) / np.linalg.norm(np.concatenate([va, vb]))
    assert abs(j.value - want_j) <= 1e-10 * want_j
    s.close()


def test_device_features_match_host(require_gpu):
    m, s = _free_vibration(p=2)
    E.point_source(s, [0.41, 0.37, 0.63], [0.6, -0.48, 0.64])
    nd = 3 * s.Np
    F = S.feature_width(nd)
    net = S.surrogate_net(s.degree, H=32, L=1, seed=3)
    net.set_graph(S.build_graph(m), "g")
    um, u0, u1 = _block_start(s)
    gdiff = 0.37
    x, sc, a1_dev, sig = S.device_features(s, net, gdiff)
    a1 = _host_a1(m, s, u1 - u0, gdiff)
    assert rel(a1_dev, a1) <= 1e-11
    # with the FP32 copy of the blocks: FP32 rounding of each entry and FP32
    # accumulation, amplified by M^-1 (cond ~1e4 at p = 2)
    _lib.check(s.lib.lymph_surrogate_apply_fp32(s.ctx, 1), "apply_fp32")
    _, _, a1_32, _ = S.device_features(s, net, gdiff)
    _lib.check(s.lib.lymph_surrogate_apply_fp32(s.ctx, 0), "apply_fp32")
    assert 0 < rel(a1_32, a1) <= 1e-4
    # the rest of the features from the device's a1
    xh, sch, sigh, _, _ = S.features(um, u0, u1, a1_dev, S.poly_material(m), F)
    assert max(abs(a - b) / b for a, b in zip(sc, sch)) <= 1e-10
    # the per-polyhedron scales: sums of squares in FP64, the square roots in
    # FP32 (the device keeps scalar per-polyhedron math off the FP64 pipe)
    assert np.abs(sig / sigh - 1.0).max() <= 1e-6
    # float32 rows
    assert np.abs(x - xh).max() <= 1e-5 * np.abs(xh).max()
    assert rel(x[:, 3 * nd:4 * nd], xh[:, 3 * nd:4 * nd]) <= 1e-6
    net.close()
    s.close()


def test_block_with_network_uses_the_device_features(require_gpu):
    m, s = _free_vibration(p=2)
    nd = 3 * s.Np
    F = S.feature_width(nd)
    net = S.surrogate_net(s.degree, H=32, L=1, seed=3)
    flat = net.init_params(3)
    flat[-net.O:] = 0.5  # visible gate coefficients
    net.set_params(flat)
    net.set_graph(S.build_graph(m), "g")
    um, u0, u1 = _block_start(s)
    x, _, a1, sig = S.device_features(s, net)
    K = 8
    _lib.check(s.lib.lymph_surrogate_predict(s.ctx, net.h, K, 1, 0.0, None), "predict")
    y = net.forward(x).astype(np.float64)
    d1, d2 = u1 - u0, (u1 - 2.0 * u0) + um
    pa, pb, _ = S.predict_states(u1, d1, d2, a1, sig, K, y)
    # the corrections (the extrapolation itself is checked above)
    base_b = S.baseline(u1, d1, d2, a1, K - 2)
    got = s.get_state(_lib.SLOT_UN) - base_b
    want = pb - base_b
    assert np.linalg.norm(want) > 0 and rel(got, want) <= 1e-6
    base_a = S.baseline(u1, d1, d2, a1, K - 3)
    assert rel(s.get_state(_lib.SLOT_U0) - base_a, pa - base_a) <= 1e-6
    net.close()
    s.close()


def test_rejected_blocks_leave_the_plain_trajectory_bitwise(require_gpu):
    """A network with huge outputs fails every energy check: each block is
    redone by the plain stepper from the saved pair, so the hybrid run ends
    exactly where the plain run does."""
    m, s = _free_vibration(p=2, material=(1.0, 1.0, 1.0))
    nd = 3 * s.Np
    net = S.surrogate_net(s.degree, H=32, L=1, seed=5)
    flat = net.init_params(5)
    flat[-net.O:] = 1e3  # output bias: huge gate coefficients
    net.set_params(flat)
    graph = S.build_graph(m)
    u0, un = s.get_state(_lib.SLOT_U0).copy(), s.get_state(_lib.SLOT_UN).copy()
    _, stats = S.run_hybrid(s, net, 50, lambda t: 0.0, s.dt, K=8, check_every=0, graph=graph)
    assert stats["rejected"] == stats["blocks"] == 6 and stats["accepted"] == 0
    assert stats["rejected_residual"] + stats["rejected_energy"] == 6
    got = s.get_state(_lib.SLOT_UN).copy(), s.get_state(_lib.SLOT_U0).copy()
    s.set_state(_lib.SLOT_U0, u0)
    s.set_state(_lib.SLOT_UN, un)
    S.run_plain(s, 50, lambda t: 0.0, s.dt)
    assert np.array_equal(got[0], s.get_state(_lib.SLOT_UN))
    assert np.array_equal(got[1], s.get_state(_lib.SLOT_U0))
    net.close()
    s.close()


def test_judge_blocks_keep_the_plain_result(require_gpu):
    """With check_every = K every block is judged: the plain result is kept,
    so the run equals the plain run bit for bit and the prediction error of
    every block is recorded."""
    _, s = _free_vibration(p=2, material=(1.0, 1.0, 1.0))
    u0, un = s.get_state(_lib.SLOT_U0).copy(), s.get_state(_lib.SLOT_UN).copy()
    _, stats = S.run_hybrid(s, None, 40, lambda t: 0.0, s.dt, K=8, check_every=8)
    assert stats["judged"] == stats["blocks"] == 5
    assert 0.0 < stats["judge_err_max"] and np.isfinite(stats["judge_err_max"])
    got = s.get_state(_lib.SLOT_UN).copy()
    s.set_state(_lib.SLOT_U0, u0)
    s.set_state(_lib.SLOT_UN, un)
    S.run_plain(s, 40, lambda t: 0.0, s.dt)
    assert np.array_equal(got, s.get_state(_lib.SLOT_UN))
    s.close()


def test_trained_network_beats_the_extrapolation(require_gpu):
    """Trained on the GPU on 32 runs of the solver itself (seeded 4^3..6^3
    meshes, p = 2, Ricker point sources from rest, lognormal materials, dt a
    seeded fraction of the CFL bound), evaluated on four held-out runs: the
    network's correction lowers the mean relative error of the block's
    predicted states against the cubic Taylor extrapolation alone."""
    net, hist, _, _ = S.train_surrogate(2, n_traj=32, iters=6000, H=256, L=3, lr=1e-3)
    print(f"training loss {np.mean(hist[:50]):.3e} -> {np.mean(hist[-500:]):.3e}")
    assert np.mean(hist[-500:]) < np.mean(hist[:50])
    errs = S.held_out_errors(net, 2)
    ratios = [a / b for a, b in errs]
    print("held-out error ratios network / extrapolation:", np.round(ratios, 3))
    assert np.mean(ratios) < 0.85
    net.close()
