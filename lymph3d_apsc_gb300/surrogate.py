"""Learned surrogate: a per-polyhedron message-passing network that advances
the modal state K steps at a time, with the plain leapfrog stepper as its
fallback and judge.  No counterpart in the reference (the reference has no
learned component).

One surrogate block, from (u^{n-1}, u^n) at time t_n:
  1. one plain step gives u^{n+1};
  2. lymph_surrogate_predict builds the features on the device and predicts
     u^{n+K-2}, u^{n+K-1}, u^{n+K}: the constant-second-difference
     extrapolation of (u^{n-1}, u^n, u^{n+1}) plus the network's correction,
     two coefficients per DOF in the Newton basis of the extrapolation's
     cubic and quartic error terms (smooth in time by construction);
  3. one plain step from the predicted (u^{n+K-2}, u^{n+K-1}) gives u^{n+K};
     its distance from the predicted u^{n+K}, relative to the step's
     increment, is the residual: above `res_tol` the block is rejected;
  4. while the source is off, the discrete leapfrog energy of the final pair
     is compared with that of the last plain-verified pair: a relative drift
     above `drift_tol` (1e-4) rejects the block;
  5. a rejected block is redone from the saved (u^n, u^{n+1}) with K-1 plain
     steps; every `check_every` (64) steps the block is also redone plainly
     and the prediction's error recorded, the plain result being kept.
An accepted block costs 2 plain steps, the network and (without forcing)
one energy evaluation instead of K plain steps.
Training data are trajectories of the solver itself on small seeded meshes
(p = 3, BFS polyhedra, lognormal materials, Ricker point sources from rest);
training runs on the GPU through lymph_mpnn_loss_grad / _adam.
"""
from __future__ import annotations

import math
import time
from ctypes import byref, c_double, c_float, c_int64, c_void_p

import numpy as np

from . import _lib
from ._lib import check, ptr
from .matrix_free import MatrixFree
from . import mesh as M
from . import ensemble as E

G_FEATURES = 8


def feature_width(nd: int) -> int:
    """Feature columns for 3Np = nd: 4 nd + 6, rounded up to 16."""
    return ((4 * nd + 6 + 15) // 16) * 16


# ---------------------------------------------------------------------------
# graph of a mesh: face-area weights and aggregated shared-face geometry
# ---------------------------------------------------------------------------
FACE_V = np.array([[2, 1, 0], [0, 1, 3], [1, 2, 3], [2, 0, 3]])


def build_graph(mesh: M.Mesh):
    """w (CSR, rows normalised to 1) over face-adjacent polyhedra, weights
    proportional to the shared face area; g_i = sum_j w_ij e_ij with
    e_ij = [area-weighted unit normal (3), area / hk_i^2, (c_j - c_i)/hk_i (3), 1]."""
    X, tv, tp, nb = mesh.coords, mesh.tet_vert, mesh.tet_poly, mesh.neigh
    n_poly = mesh.n_poly
    t = np.repeat(np.arange(mesh.n_tet), 4)
    f = np.tile(np.arange(4), mesh.n_tet)
    e = nb.reshape(-1)
    sel = e >= 0
    t, f, e = t[sel], f[sel], e[sel]
    P, Q = tp[t], tp[e]
    sel = P != Q
    t, f, P, Q = t[sel], f[sel], P[sel], Q[sel]
    v = tv[t[:, None], FACE_V[f]]
    c1, c2, c3 = X[v[:, 0]], X[v[:, 1]], X[v[:, 2]]
    nvec = np.cross(c3 - c2, c1 - c2)  # the reference's (X3 - X2) x (X1 - X2), |.| = 2 area
    area = 0.5 * np.linalg.norm(nvec, axis=1)
    # polyhedron centres and sizes
    cent_t = X[tv].mean(axis=1)
    cnt = np.bincount(tp, minlength=n_poly).astype(np.float64)
    cent = np.zeros((n_poly, 3))
    np.add.at(cent, tp, cent_t)
    cent /= cnt[:, None]
    lo = np.full((n_poly, 3), np.inf)
    hi = np.full((n_poly, 3), -np.inf)
    np.minimum.at(lo, tp, X[tv].min(axis=1))
    np.maximum.at(hi, tp, X[tv].max(axis=1))
    hk = np.linalg.norm(hi - lo, axis=1)
    key = P.astype(np.int64) * n_poly + Q
    uniq, inv = np.unique(key, return_inverse=True)
    A = np.zeros(uniq.size)
    AN = np.zeros((uniq.size, 3))
    np.add.at(A, inv, area)
    np.add.at(AN, inv, nvec * 0.5)
    Pi, Qi = uniq // n_poly, uniq % n_poly
    rowA = np.zeros(n_poly)
    np.add.at(rowA, Pi, A)
    w = A / rowA[Pi]
    ef = np.zeros((uniq.size, G_FEATURES))
    ef[:, 0:3] = AN / A[:, None]
    ef[:, 3] = A / hk[Pi] ** 2
    ef[:, 4:7] = (cent[Qi] - cent[Pi]) / hk[Pi][:, None]
    ef[:, 7] = 1.0
    g = np.zeros((n_poly, G_FEATURES))
    np.add.at(g, Pi, w[:, None] * ef)
    ptr_ = np.zeros(n_poly + 1, np.int32)
    np.add.at(ptr_, Pi + 1, 1)
    ptr_ = np.cumsum(ptr_).astype(np.int32)
    return ptr_, Qi.astype(np.int32), w.astype(np.float32), g.astype(np.float32)


def poly_material(mesh: M.Mesh) -> np.ndarray:
    first = np.full(mesh.n_poly, -1)
    order = np.argsort(mesh.tet_poly, kind="stable")
    tp_sorted = mesh.tet_poly[order]
    starts = np.searchsorted(tp_sorted, np.arange(mesh.n_poly))
    first = order[starts]
    return mesh.mat[mesh.tet_mat[first]]


def features(um, u0, u1, a1, mat, F):
    """The device's k_features in numpy (float64 arithmetic, float32 out);
    a1 = dt^2 M^-1 (K d1 - gdiff F).  Returns (x, mesh-wide RMS s1..s4,
    per-polyhedron scales r [N, 4], d1, d2)."""
    d1 = u1 - u0
    d2 = (u1 - 2.0 * u0) + um
    vecs = (u1, d1, d2, a1)
    n = u1.size
    N, nd = u1.shape
    s = [math.sqrt(float(np.sum(v * v)) / n) for v in vecs]
    r = np.stack([np.sqrt(np.sum(v * v, axis=1) / nd) + 1e-3 * sg + 1e-300 for v, sg in zip(vecs, s)], axis=1)
    x = np.zeros((N, F))
    for b, v in enumerate(vecs):
        x[:, b * nd:(b + 1) * nd] = v / r[:, b:b + 1]
    x[:, 4 * nd] = np.log10(r[:, 1] / r[:, 0])
    x[:, 4 * nd + 1] = np.log10(r[:, 2] / r[:, 1])
    x[:, 4 * nd + 2] = np.log10(r[:, 3] / r[:, 2])
    x[:, 4 * nd + 3:4 * nd + 6] = mat[:, [1, 2, 0]]
    return x.astype(np.float32), tuple(s), r, d1, d2


def baseline(u1, d1, d2, a1, k):
    """Cubic Taylor extrapolation of u^{n+1+k}: u1 + k d1 + k(k+1)/2 d2
    - k(k+1)(k+2)/6 a1, with a1 = dt^2 M^-1 (K d1 - gdiff F) ~ -d3."""
    return u1 + k * d1 + 0.5 * k * (k + 1.0) * d2 - (k * (k + 1.0) * (k + 2.0) / 6.0) * a1


def newton_phi(k, K):
    """Newton basis of the remaining cubic and quartic error terms."""
    p3 = k * (k + 1.0) * (k + 2.0) / float(K) ** 3
    return p3, p3 * (k + 3.0) / K


def corr_scale(sig, K):
    """Per-polyhedron (r4^2 / r3) K^4 / 24 as a column [N, 1]: r4/r3 ~ omega dt,
    so the coefficients are O(1)."""
    return ((sig[:, 3] ** 2 / sig[:, 2]) * K ** 4 / 24.0)[:, None]


PRED_K = lambda K: (K - 3, K - 2, K - 1)  # noqa: E731  (offsets of the three predicted states)


def targets(u1, d1, d2, a1, sig, K, later):
    """Least-squares Newton coefficients [y3 | y4] of the extrapolation error
    over u^{n+1+k}, k = 1..K-1 (later[k-1] = u^{n+1+k})."""
    ks = np.arange(1, K, dtype=np.float64)
    Phi = np.stack(newton_phi(ks, K), axis=1)  # [K-1, 2]
    pinv = np.linalg.pinv(Phi)  # [2, K-1]
    sc = corr_scale(sig, K)
    E = np.stack([(later[k - 1] - baseline(u1, d1, d2, a1, k)) / sc for k in range(1, K)], axis=0)
    y = np.tensordot(pinv, E, axes=(1, 0))  # [2, N, nd]
    return np.concatenate([y[0], y[1]], axis=1).astype(np.float32)


def predict_states(u1, d1, d2, a1, sig, K, y):
    """The three predicted states of a block from coefficients y = [y3 | y4]."""
    nd = u1.shape[1]
    sc = corr_scale(sig, K)
    out = []
    for k in PRED_K(K):
        p3, p4 = newton_phi(float(k), K)
        out.append(baseline(u1, d1, d2, a1, k) + sc * (y[:, :nd] * p3 + y[:, nd:] * p4))
    return out


# ---------------------------------------------------------------------------
# network handle
# ---------------------------------------------------------------------------
class MPNN:
    """The CUDA network (lymph_mpnn_*).  gate = (nd, B) switches to the gated
    head: O = 6 B per-node coefficients over the first B feature blocks of nd
    DOFs, effective output width 2 nd."""

    def __init__(self, F: int, O: int, H: int = 256, L: int = 3, G: int = G_FEATURES, seed: int = 0, gate=None):
        self.lib = _lib.load()
        self.F, self.O, self.H, self.L, self.G = F, O, H, L, G
        self.gate = gate
        self.out_width = 2 * gate[0] if gate else O
        h = c_void_p()
        check(self.lib.lymph_mpnn_create(F, H, O, L, G, byref(h)), "lymph_mpnn_create")
        self.h = h
        self.n_par = self.lib.lymph_mpnn_num_params(h)
        if gate:
            check(self.lib.lymph_mpnn_set_gate(h, gate[0], gate[1]), "lymph_mpnn_set_gate")
        self.set_params(self.init_params(seed))
        self.graph_key = None

    def shapes(self):
        s = [("W0", (self.F, self.H)), ("b0", (self.H,))]
        for l in range(self.L):
            s += [(f"Wm{l}", (self.H, self.H)), (f"bm{l}", (self.H,)),
                  (f"Wu{l}", (2 * self.H + self.G, self.H)), (f"bu{l}", (self.H,))]
        s += [("Wo", (self.H, self.O)), ("bo", (self.O,))]
        return s

    def init_params(self, seed):
        rng = np.random.default_rng(seed)
        out = []
        for name, sh in self.shapes():
            if name.startswith("W"):
                scale = math.sqrt(2.0 / sh[0]) * (0.05 if name == "Wo" else 1.0)
                out.append((rng.standard_normal(sh) * scale).ravel())
            else:
                out.append(np.zeros(int(np.prod(sh))))
        return np.concatenate(out).astype(np.float32)

    def unpack(self, flat):
        d, o = {}, 0
        for name, sh in self.shapes():
            n = int(np.prod(sh))
            d[name] = flat[o:o + n].reshape(sh)
            o += n
        return d

    def set_params(self, flat):
        flat = np.ascontiguousarray(flat, dtype=np.float32)
        assert flat.size == self.n_par
        check(self.lib.lymph_mpnn_set_params(self.h, ptr(flat, c_float)), "lymph_mpnn_set_params")

    def params_and_grads(self):
        p = np.empty(self.n_par, np.float32)
        g = np.empty(self.n_par, np.float32)
        check(self.lib.lymph_mpnn_get_params(self.h, ptr(p, c_float), ptr(g, c_float)), "lymph_mpnn_get_params")
        return p, g

    def set_graph(self, graph, key=None):
        if key is not None and key == self.graph_key:
            return
        wp, wi, wv, g = graph
        wp, wi = np.ascontiguousarray(wp, np.int32), np.ascontiguousarray(wi, np.int32)
        wv, g = np.ascontiguousarray(wv, np.float32), np.ascontiguousarray(g, np.float32)
        check(self.lib.lymph_mpnn_set_graph(self.h, wp.size - 1, ptr(wp, _lib.c_int32), ptr(wi, _lib.c_int32),
                                            ptr(wv, c_float), ptr(g, c_float)), "lymph_mpnn_set_graph")
        self.graph_key = key

    def forward(self, x):
        x = np.ascontiguousarray(x, np.float32)
        y = np.empty((x.shape[0], self.out_width), np.float32)
        check(self.lib.lymph_mpnn_forward(self.h, ptr(x, c_float), ptr(y, c_float)), "lymph_mpnn_forward")
        return y

    def loss_grad(self, x, t):
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(t, np.float32)
        loss = c_double()
        check(self.lib.lymph_mpnn_loss_grad(self.h, ptr(x, c_float), ptr(t, c_float), byref(loss)), "loss_grad")
        return loss.value

    def adam(self, lr, b1=0.9, b2=0.999, eps=1e-8):
        check(self.lib.lymph_mpnn_adam(self.h, lr, b1, b2, eps), "lymph_mpnn_adam")

    def launch_count(self):
        n = c_int64()
        check(self.lib.lymph_mpnn_launch_count(self.h, byref(n)), "launch_count")
        return n.value

    def close(self):
        if getattr(self, "h", None):
            self.lib.lymph_mpnn_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------
# training data from the solver
# ---------------------------------------------------------------------------
def device_features(s: MatrixFree, net: MPNN, gdiff: float = 0.0):
    """Feature rows of the block whose V0, U0, UN the context holds, built
    on the device (lymph_surrogate_features); returns
    (x, mesh-wide RMS (s1, s2, s3, s4), a1, per-polyhedron scales [N, 4])."""
    x = np.empty((s.n_poly, net.F), np.float32)
    a1 = np.empty((s.n_poly, s.nd), np.float64)
    sig = np.empty((s.n_poly, 4), np.float64)
    sc = (c_double * 4)()
    check(s.lib.lymph_surrogate_features(s.ctx, net.h, gdiff, ptr(x, c_float), sc, ptr(a1, c_double),
                                         ptr(sig, c_double)), "lymph_surrogate_features")
    return x, tuple(sc), a1, sig


def solver_samples(seed: int, K: int, net: MPNN, p: int = 3, n: int = 5, steps: int | None = None, every: int = 32,
                   start: int = 40, cfl: float | None = None, f_dt: float | None = None, lognormal: bool = True,
                   keep_truth: bool = False, t0_cycles: float = 2.0):
    """Training or evaluation samples from one solver run from rest on a small
    seeded mesh: homogeneous Dirichlet, BFS polyhedra of 4-16 tets,
    lognormal lambda and mu, a Ricker point source centred at
    t0 = t0_cycles / f0 (2 cycles: the source starts smoothly from zero) at a
    random point and direction, dt = cfl x 2/sqrt(lambda_max) and
    f0 = f_dt / dt (f_dt = source cycles per step; cfl and f_dt drawn from
    the seed when None).  The run lasts `steps` (default: until the pulse
    has passed); a sample is taken every `every` steps, its features built
    on the device by the network handle `net` (its graph is set to this
    mesh).  Returns (samples, graph, material, meta)."""
    rng = np.random.default_rng(seed)
    cfl = float(rng.uniform(0.04, 0.15)) if cfl is None else cfl
    f_dt = float(rng.uniform(0.7e-3, 2e-3)) if f_dt is None else f_dt
    steps = int((t0_cycles + 1.5) / f_dt) if steps is None else steps
    base = M.cube(n, bc="dirichlet", agglomeration="bfs", seed=seed, group=(4, 16))
    mats = M.lognormal_materials(base.n_poly, seed=seed) if lognormal else None
    m = M.cube(n, bc="dirichlet", agglomeration="bfs", seed=seed, group=(4, 16), poly_materials=mats)
    mat = poly_material(m)
    graph = build_graph(m)
    net.set_graph(graph, ("samples", seed, n))
    s = MatrixFree(m, p, 1.0)
    samples = []
    try:
        s.MAKE_MATRICES_FREE()
        s.MAKE_RHS_FREE(_lib.RHS_STAT, _lib.F_NULL, _lib.GD_NULL, _lib.GN_NULL)
        lam = E.max_eigenvalue(s, 60)
        E.set_dt(s, cfl * 2.0 / math.sqrt(lam))
        f0 = f_dt / s.dt
        x0 = rng.uniform(0.2, 0.8, 3)
        d = rng.standard_normal(3)
        E.point_source(s, x0, d / np.linalg.norm(d))
        s.COMPUTE_MODAL_COEFFICIENTS_FREE(_lib.FUN_IC_DISPLACEMENT, _lib.SLOT_U0)  # zero at t = 0
        s.COMPUTE_MODAL_COEFFICIENTS_FREE(_lib.FUN_IC_DISPLACEMENT, _lib.SLOT_V0)
        gfun = lambda t: float(E.ricker(t, f0, t0_cycles / f0))  # noqa: E731
        check(s.lib.lymph_first_step_g(s.ctx, gfun(0.0)), "first_step_g")
        t, t_prev = s.dt, 0.0
        win, x, sc, a1, sig = {}, None, None, None, None
        for i in range(1, steps):  # UN holds u^i at time t
            r = (i - (start - 1)) % every
            if i >= start - 1 and r <= K + 1:
                win[r] = s.get_state(_lib.SLOT_UN).copy()
                if r == 1:  # V0 = u^{n-1} for the features after the next step
                    check(s.lib.lymph_copy_state(s.ctx, _lib.SLOT_V0, _lib.SLOT_U0), "copy")
                elif r == 2:
                    x, sc, a1, sig = device_features(s, net, gfun(t) - gfun(t_prev))
                elif r == K + 1:
                    um, u0, u1 = win[0], win[1], win[2]
                    d1 = u1 - u0
                    d2 = (u1 - 2.0 * u0) + um
                    if sc[2] > 1e-280 and sc[3] > 1e-280:
                        later = [win[2 + k] for k in range(1, K)]
                        tgt = targets(u1, d1, d2, a1, sig, K, later)
                        aux = (u1, d1, d2, a1, sig, [win[2 + k] for k in PRED_K(K)]) if keep_truth else None
                        samples.append((x, tgt, aux))
                    win = {}
            check(s.lib.lymph_step_g(s.ctx, gfun(t)), "step_g")
            t_prev = t
            t += s.dt
    finally:
        s.close()
    return samples, graph, mat, {"cfl": cfl, "f_dt": f_dt, "f0": f0, "steps": steps, "n_poly": m.n_poly}


def train(net: MPNN, datasets, iters: int, lr: float = 1e-3, seed: int = 0, log_every: int = 0):
    """Adam on (graph, samples, key) datasets, cosine-decayed learning rate;
    returns the loss history."""
    rng = np.random.default_rng(seed)
    hist = []
    for it in range(iters):
        graph, samples, key = datasets[int(rng.integers(len(datasets)))]
        x, t, _ = samples[int(rng.integers(len(samples)))]
        net.set_graph(graph, key)
        lr_t = lr * (0.5 * (1 + math.cos(math.pi * it / iters)) * 0.9 + 0.1)
        loss = net.loss_grad(x, t)
        net.adam(lr_t)
        hist.append(loss)
        if log_every and it % log_every == 0:
            print(f"iter {it} loss {loss:.4e}")
    return hist


def prediction_error(net: MPNN | None, graph, key, samples, K: int):
    """Mean over samples of the relative error of the three predicted states,
    with the network (net) or with the extrapolation alone (net = None)."""
    errs = []
    if net is not None:
        net.set_graph(graph, key)
    for x, t, (u1, d1, d2, a1, sig, truth) in samples:
        y = net.forward(x).astype(np.float64) if net is not None else np.zeros(t.shape)
        pred = predict_states(u1, d1, d2, a1, sig, K, y)
        errs.append(float(np.linalg.norm(np.concatenate(pred) - np.concatenate(truth)) /
                          np.linalg.norm(np.concatenate(truth))))
    return float(np.mean(errs))


# ---------------------------------------------------------------------------
# hybrid stepping
# ---------------------------------------------------------------------------
def energy(s: MatrixFree, a=_lib.SLOT_U0, b=_lib.SLOT_UN) -> float:
    e = c_double()
    check(s.lib.lymph_energy(s.ctx, a, b, byref(e)), "lymph_energy")
    return e.value


def run_plain(s: MatrixFree, n_steps: int, gfun, t: float) -> float:
    """n_steps plain leapfrog steps; t is the time of UN on entry (the step
    to u^{n+1} uses the source value at t_n); returns the time of UN."""
    for _ in range(n_steps):
        check(s.lib.lymph_step_g(s.ctx, gfun(t)), "step_g")
        t += s.dt
    return t


def run_hybrid(s: MatrixFree, net: MPNN | None, n_steps: int, gfun, t: float, K: int = 8, check_every: int = 64,
               drift_tol: float = 1e-4, res_tol: float = 1e-4, graph=None, g_scale: float = 1.0,
               apply_fp32: bool = False):
    """Advances n_steps with surrogate blocks of K steps (net = None: the
    extrapolation alone).  The context holds (u^{n-1}, u^n) with u^n at time
    t on entry and on exit.  A block is forced when a source value inside it
    exceeds 1e-9 x g_scale; its energy is then not checked.  apply_fp32
    computes the predictor's operator term with an FP32 copy of the blocks.
    Returns (t, stats)."""
    use_net = net is not None
    if use_net:
        net.set_graph(graph, ("hybrid", id(s)))
    check(s.lib.lymph_surrogate_apply_fp32(s.ctx, int(apply_fp32)), "lymph_surrogate_apply_fp32")
    hnet = net.h if use_net else _dummy_net().h
    stats = {"blocks": 0, "accepted": 0, "rejected": 0, "rejected_residual": 0, "rejected_energy": 0,
             "judged": 0, "judge_err_max": 0.0, "plain_steps": 0, "energy_evals": 0, "residual_max": 0.0,
             "drift_max": 0.0, "judge_err_accepted_max": 0.0}
    res = c_double()
    e_ref = None
    done = 0
    while done < n_steps:
        if n_steps - done < K:
            t = run_plain(s, n_steps - done, gfun, t)
            stats["plain_steps"] += n_steps - done
            break
        stats["blocks"] += 1
        tk, forced = t, False
        for _ in range(K + 1):
            forced = forced or abs(gfun(tk)) > 1e-9 * g_scale
            tk += s.dt
        if not forced and e_ref is None:
            e_ref = energy(s)
            stats["energy_evals"] += 1
        judge = check_every > 0 and (done // check_every) != ((done + K) // check_every)
        t0 = t
        check(s.lib.lymph_copy_state(s.ctx, _lib.SLOT_V0, _lib.SLOT_U0), "copy")
        t1 = run_plain(s, 1, gfun, t0)  # u^{n+1}
        gdiff = gfun(t1) - gfun(t0)
        check(s.lib.lymph_surrogate_predict(s.ctx, hnet, K, int(use_net), gdiff, None), "surrogate_predict")
        tpred = t1
        for _ in range(K - 2):
            tpred += s.dt  # time of the predicted u^{n+K-1}
        tend = run_plain(s, 1, gfun, tpred)  # u^{n+K} from the predicted pair
        stats["plain_steps"] += 2
        check(s.lib.lymph_surrogate_residual(s.ctx, hnet, byref(res)), "surrogate_residual")
        ok = res.value <= res_tol
        stats["residual_max"] = max(stats["residual_max"], res.value)
        if not ok:
            stats["rejected_residual"] += 1
        if ok and not forced:
            e = energy(s)
            stats["energy_evals"] += 1
            drift = abs(e - e_ref) / max(abs(e_ref), 1e-300)
            stats["drift_max"] = max(stats["drift_max"], drift)
            if drift > drift_tol:
                ok = False
                stats["rejected_energy"] += 1
        if judge or not ok:
            if judge:
                check(s.lib.lymph_surrogate_judge(s.ctx, hnet, 0, None), "surrogate_judge")
            check(s.lib.lymph_copy_state(s.ctx, _lib.SLOT_U0, _lib.SLOT_V0), "copy")
            check(s.lib.lymph_copy_state(s.ctx, _lib.SLOT_UN, _lib.SLOT_UEX), "copy")
            tend = run_plain(s, K - 1, gfun, t1)
            stats["plain_steps"] += K - 1
            if judge:
                err = c_double()
                check(s.lib.lymph_surrogate_judge(s.ctx, hnet, 1, byref(err)), "surrogate_judge")
                stats["judged"] += 1
                stats["judge_err_max"] = max(stats["judge_err_max"], err.value)
                if ok:
                    stats["judge_err_accepted_max"] = max(stats["judge_err_accepted_max"], err.value)
            if not forced:
                e_ref = energy(s)
                stats["energy_evals"] += 1
            else:
                e_ref = None
        if ok:
            stats["accepted"] += 1
        else:
            stats["rejected"] += 1
        if forced:
            e_ref = None
        t = tend
        done += K
    return t, stats


_DUMMY = None


def training_sets(net: MPNN, p: int, n_traj: int, K: int = 8, seed0: int = 0, every: int = 32, sizes=(4, 5, 6)):
    """Samples of n_traj solver runs (seeds seed0.., meshes n^3 x 6 with n
    cycling through `sizes`; larger meshes are sampled every 2 x `every`)."""
    sets = []
    for sd in range(seed0, seed0 + n_traj):
        n = sizes[sd % len(sizes)]
        sm, gr, _, _ = solver_samples(sd, K, net, p=p, n=n, every=every if n <= 6 else 2 * every)
        if sm:
            sets.append((gr, sm, ("train", p, sd)))
    return sets


def held_out_errors(net: MPNN, p: int, seeds=(100, 101, 102, 103), K: int = 8, every: int = 64):
    """(network, extrapolation-only) mean relative errors of the predicted
    states on solver runs the network was not trained on."""
    out = []
    for sd in seeds:
        sm, gr, _, _ = solver_samples(sd, K, net, p=p, n=4 + sd % 3, every=every, keep_truth=True)
        key = ("held", p, sd)
        out.append((prediction_error(net, gr, key, sm, K), prediction_error(None, gr, key, sm, K)))
    return out


def train_surrogate(p: int, n_traj: int = 200, iters: int = 20000, H: int = 256, L: int = 3, lr: float = 1e-3,
                    K: int = 8, seed: int = 0, sizes=(4, 5, 6)):
    """Builds the network for degree p and trains it on the GPU on n_traj
    runs of the solver.  Returns (net, loss history, seconds for data,
    seconds for training)."""
    net = surrogate_net(p, H=H, L=L, seed=seed)
    t0 = time.perf_counter()
    sets = training_sets(net, p, n_traj, K, sizes=sizes)
    t1 = time.perf_counter()
    hist = train(net, sets, iters, lr=lr, seed=seed)
    return net, hist, t1 - t0, time.perf_counter() - t1


def surrogate_net(p: int, H: int = 256, L: int = 3, seed: int = 0) -> MPNN:
    """The surrogate's network for degree p: gated head over the four
    feature blocks [u1, d1, d2, a1] (24 outputs per polyhedron)."""
    nd = 3 * (p + 1) * (p + 2) * (p + 3) // 6
    return MPNN(feature_width(nd), 6 * 4, H=H, L=L, seed=seed, gate=(nd, 4))


def _dummy_net():
    """A network handle for lymph_surrogate_predict with use_net = 0."""
    global _DUMMY
    if _DUMMY is None:
        _DUMMY = MPNN(16, 2, H=16, L=0)
    return _DUMMY
