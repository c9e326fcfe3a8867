"""The tensor-core self-block decomposition against the assembled block (CPU).

k_self_tc (csrc/selftc.cu) never forms the self block entry by entry: it
computes two matrix products over one K dimension of quadrature slots,
O_D = A B_D^T and O_S = A B_S^T, and combines them as
    K_PP[(i,a),(j,b)] = O_D[(i,a),(j,b)] + O_S[(j,a),(i,b)]
                        + delta_ij sum_k O_S[(k,a),(k,b)],
with, per slot, A = d_i phi_a (volume points and "d" face slots) or
n_i phi_a ("n phi" face slots) and the B rows weighted by the material,
theta, cI and the penalty (the table is in the kernel's header).  This test
restates that decomposition in FP64 numpy, with the kernel's quadrature (the
reference's collapsed Gauss rule on each sub-tetrahedron, the symmetric
triangle rule of lymph_mf_face_rule on each face), and checks it against the
oracle's assembled self blocks (MAKE_STIFFNESS_VOLUME +
MAKE_STIFFNESS_FACE's self terms): the same integrals, so they agree to FP64
rounding (1e-12 relative to the block's largest entry), for every theta,
Dirichlet and Neumann faces, jittered tetrahedra and lognormal materials.
k_nb_tc, for the neighbour blocks of LYMPH_MIXED, uses the same two products
with five slots per face point; the second test restates that form and
checks it against the oracle's neighbour blocks the same way.
"""
from ctypes import POINTER, byref, c_double, c_int32

import numpy as np
import pytest

from lymph3d_apsc_gb300 import _lib
from lymph3d_apsc_gb300 import mesh as M
from oracle.oracle_py import Oracle

# face vertex triples of the normals (k_geometry) and the face maps
# (basis_boundary's node_maps), as the device builds them
FACE_VERTS = [(2, 1, 0), (0, 1, 3), (1, 2, 3), (2, 0, 3)]
NODE_MAPS = np.zeros((4, 4, 4))
for f, r, c, v in [(0, 0, 1, 1), (0, 1, 0, 1), (0, 3, 3, 1), (1, 0, 0, 1), (1, 2, 1, 1), (1, 3, 3, 1),
                   (2, 0, 0, 1), (2, 1, 1, 1), (2, 2, 2, 1), (2, 3, 3, 1), (2, 2, 0, -1), (2, 2, 1, -1),
                   (3, 1, 1, 1), (3, 2, 0, 1), (3, 3, 3, 1)]:
    NODE_MAPS[f, r, c] = v


def _legendre(x, n):
    L = np.zeros((n + 1,) + np.shape(x))
    D = np.zeros_like(L)
    L[0] = 1
    if n >= 1:
        L[1] = x
        D[1] = 1
    for k in range(1, n):
        L[k + 1] = ((2 * k + 1) * x * L[k] - k * L[k - 1]) / (k + 1)
        D[k + 1] = D[k - 1] + (2 * k + 1) * L[k]
    return L, D


def _tabulate(xs, bb, p, blist):
    c = (bb[0::2] + bb[1::2]) / 2
    h = (bb[1::2] - bb[0::2]) / 2
    sc = 1 / np.sqrt(h.prod())
    xh = (xs - c) / h
    Lx, Dx = _legendre(xh[:, 0], p)
    Ly, Dy = _legendre(xh[:, 1], p)
    Lz, Dz = _legendre(xh[:, 2], p)
    phi = np.array([sc * Lx[a] * Ly[b] * Lz[cc] for a, b, cc in blist])
    grad = np.array([[sc / h[0] * Dx[a] * Ly[b] * Lz[cc] for a, b, cc in blist],
                     [sc / h[1] * Lx[a] * Dy[b] * Lz[cc] for a, b, cc in blist],
                     [sc / h[2] * Lx[a] * Ly[b] * Dz[cc] for a, b, cc in blist]])
    return phi, grad


def _decomposed_self_blocks(m, p, bbox, hk, alpha, theta):
    lib = _lib.load()
    n = c_int32()
    assert lib.lymph_mf_face_rule(p, byref(n), None) == 0
    xyw = np.zeros(3 * n.value)
    lib.lymph_mf_face_rule(p, byref(n), xyw.ctypes.data_as(POINTER(c_double)))
    xyw = xyw.reshape(-1, 3)
    NP = (p + 1) * (p + 2) * (p + 3) // 6
    ND = 3 * NP
    blist = [(a, b, c) for a in range(p, -1, -1) for b in range(p - a, -1, -1) for c in range(p - a - b, -1, -1)]
    g, w = np.polynomial.legendre.leggauss(p + 1)
    rp, rw = [], []
    for i in range(p + 1):
        for j in range(p + 1):
            for k in range(p + 1):
                a, b, cc = 0.5 * g[i] + 0.5, 0.5 * g[j] + 0.5, 0.5 * g[k] + 0.5
                rp.append((a, (1 - a) * b, (1 - a) * (1 - b) * cc))
                rw.append(abs((1 - b) * (1 - a) ** 2) * 0.125 * w[i] * w[j] * w[k])
    rp, rw = np.array(rp), np.array(rw)
    X, tv, tp = m.coords, m.tet_vert, m.tet_poly
    nb = m.neigh.reshape(-1, 4)
    out = []
    for P in range(m.n_poly):
        A, BD, BS = [], [], []
        for t in np.where(tp == P)[0]:
            V = X[tv[t]]
            F = np.stack([V[1] - V[0], V[2] - V[0], V[3] - V[0]], 1)
            lam, mu = m.mat[m.tet_mat[t], 1], m.mat[m.tet_mat[t], 2]
            phi, gr = _tabulate(V[0] + rp @ F.T, bbox[P], p, blist)
            wq = rw * abs(np.linalg.det(F))
            A.append(gr.reshape(ND, -1))
            BD.append((gr * (wq * lam)).reshape(ND, -1))
            BS.append((gr * (wq * mu)).reshape(ND, -1))
        for t in np.where(tp == P)[0]:
            for f in range(4):
                e2 = nb[t, f]
                if e2 == _lib.BC_DIRI:
                    dirichlet = True
                elif e2 >= 0 and tp[e2] != P:
                    dirichlet = False
                else:
                    continue
                V = X[tv[t]]
                F = np.concatenate([np.stack([V[1] - V[0], V[2] - V[0], V[3] - V[0]], 1), V[0][:, None]], 1)
                cm = F @ NODE_MAPS[f]
                c1, c2, c3 = (X[tv[t, v]] for v in FACE_VERTS[f])
                Qv, Pv = c1 - c2, c3 - c2
                nn = np.array([Pv[1] * Qv[2] - Pv[2] * Qv[1], -Pv[0] * Qv[2] + Pv[2] * Qv[0],
                               Pv[0] * Qv[1] - Pv[1] * Qv[0]])
                area = np.linalg.norm(nn)
                nv = nn / area
                lam, mu = m.mat[m.tet_mat[t], 1], m.mat[m.tet_mat[t], 2]
                hmin = hk[P] if dirichlet else min(hk[P], hk[tp[e2]])
                sigma = alpha * p * p / hmin * (lam + 2 * mu)
                cI = 1.0 if dirichlet else 0.5
                xs = (cm[:, 2] + cm[:, 3])[None, :] + xyw[:, :1] * cm[:, 0] + xyw[:, 1:2] * cm[:, 1]
                W = xyw[:, 2] * area
                phi, gr = _tabulate(xs, bbox[P], p, blist)
                nphi = nv[:, None, None] * phi[None]
                A.append(gr.reshape(ND, -1))                                   # "d" slots
                BD.append((nphi * (theta * cI * W * lam)).reshape(ND, -1))
                BS.append((nphi * (theta * cI * W * mu)).reshape(ND, -1))
                A.append(nphi.reshape(ND, -1))                                 # "n phi" slots
                BD.append((gr * (-cI * W * lam)).reshape(ND, -1))
                BS.append((nphi * (sigma * W / 2) + gr * (-cI * W * mu)).reshape(ND, -1))
        A = np.concatenate(A, 1)
        OD = (A @ np.concatenate(BD, 1).T).reshape(3, NP, 3, NP)
        OS = (A @ np.concatenate(BS, 1).T).reshape(3, NP, 3, NP)
        K = OD + np.transpose(OS, (2, 1, 0, 3))   # K[i,a,j,b] += OS[j,a,i,b]
        tr = OS[0, :, 0, :] + OS[1, :, 1, :] + OS[2, :, 2, :]
        for i in range(3):
            K[i, :, i, :] += tr
        out.append(K.reshape(ND, ND))
    return out


def _mesh(bc):
    m0 = M.cube(3, bc=bc, agglomeration="bfs", seed=1, group=(4, 12), jitter=0.15)
    return M.cube(3, bc=bc, agglomeration="bfs", seed=1, group=(4, 12), jitter=0.15,
                  poly_materials=M.lognormal_materials(m0.n_poly, seed=3))


@pytest.mark.parametrize("p,theta,bc", [(1, -1.0, "dirichlet"), (2, -1.0, "reference"), (3, 0.0, "dirichlet"),
                                        (4, -1.0, "dirichlet"), (2, 1.0, "reference"), (4, 1.0, "reference")])
def test_decomposition_reproduces_the_self_blocks(p, theta, bc):
    m = _mesh(bc)
    o = Oracle(m, p, 1e-3, theta=theta)
    o.make_matrices()
    blocks = o.block_dict(0)
    bbox, hk = o.poly_geometry()
    o.close()
    got = _decomposed_self_blocks(m, p, bbox, hk, 10.0, theta)
    worst = 0.0
    for P, K in enumerate(got):
        ref = blocks[(P, P)]
        worst = max(worst, float(np.abs(K - ref).max() / np.abs(ref).max()))
    print(f"p={p} theta={theta} bc={bc}: {m.n_poly} self blocks, worst {worst:.2e}")
    assert worst <= 1e-12, worst


def _decomposed_neighbour_blocks(m, p, bbox, hk, alpha, theta, pairs):
    """The neighbour blocks K_PQ by the same two products: per face point five
    slots -- "d" (A = d_i phi^P_a), "n phi" (A = n_i phi^P_a) and three
    "phi_k" slots (A = delta_ik phi^P_a) that carry the delta_ij part of the
    symmetry term, whose IT_E2 index order gives the block transpose of O_S
    lambda where that part needs mu."""
    lib = _lib.load()
    n = c_int32()
    lib.lymph_mf_face_rule(p, byref(n), None)
    xyw = np.zeros(3 * n.value)
    lib.lymph_mf_face_rule(p, byref(n), xyw.ctypes.data_as(POINTER(c_double)))
    xyw = xyw.reshape(-1, 3)
    NP = (p + 1) * (p + 2) * (p + 3) // 6
    ND = 3 * NP
    blist = [(a, b, c) for a in range(p, -1, -1) for b in range(p - a, -1, -1) for c in range(p - a - b, -1, -1)]
    X, tv, tp = m.coords, m.tet_vert, m.tet_poly
    nb = m.neigh.reshape(-1, 4)
    out = {}
    for P, Q in pairs:
        A, BD, BS = [], [], []
        for t in np.where(tp == P)[0]:
            for f in range(4):
                e2 = nb[t, f]
                if e2 < 0 or tp[e2] != Q:
                    continue
                V = X[tv[t]]
                F = np.concatenate([np.stack([V[1] - V[0], V[2] - V[0], V[3] - V[0]], 1), V[0][:, None]], 1)
                cm = F @ NODE_MAPS[f]
                c1, c2, c3 = (X[tv[t, v]] for v in FACE_VERTS[f])
                Qv, Pv = c1 - c2, c3 - c2
                nn = np.array([Pv[1] * Qv[2] - Pv[2] * Qv[1], -Pv[0] * Qv[2] + Pv[2] * Qv[0],
                               Pv[0] * Qv[1] - Pv[1] * Qv[0]])
                area = np.linalg.norm(nn)
                nv = nn / area
                lam, mu = m.mat[m.tet_mat[t], 1], m.mat[m.tet_mat[t], 2]
                sigma = alpha * p * p / min(hk[P], hk[Q]) * (lam + 2 * mu)
                xs = (cm[:, 2] + cm[:, 3])[None, :] + xyw[:, :1] * cm[:, 0] + xyw[:, 1:2] * cm[:, 1]
                W = xyw[:, 2] * area
                phP, grP = _tabulate(xs, bbox[P], p, blist)
                phQ, grQ = _tabulate(xs, bbox[Q], p, blist)
                nP = nv[:, None, None] * phP[None]
                nQ = nv[:, None, None] * phQ[None]
                dnQ = np.einsum("k,kbq->bq", nv, grQ)            # d_n phi^Q_b
                zero = np.zeros_like(grQ)
                A.append(grP.reshape(ND, -1))                      # "d"
                BD.append((nQ * (-0.5 * theta * W * lam)).reshape(ND, -1))
                BS.append((nQ * (-0.5 * theta * W * mu)).reshape(ND, -1))
                A.append(nP.reshape(ND, -1))                       # "n phi"
                BD.append((grQ * (-0.5 * mu * W)).reshape(ND, -1))
                BS.append((nQ * (-0.5 * sigma * W) + grQ * (-0.5 * lam * W)).reshape(ND, -1))
                for k in range(3):                                 # "phi_k"
                    a_k = np.zeros_like(grP)
                    a_k[k] = phP
                    b_k = np.zeros_like(grQ)
                    b_k[k] = dnQ * (0.5 * (lam - mu) * W)
                    A.append(a_k.reshape(ND, -1))
                    BD.append(b_k.reshape(ND, -1))
                    BS.append(zero.reshape(ND, -1))
        A = np.concatenate(A, 1)
        OD = (A @ np.concatenate(BD, 1).T).reshape(3, NP, 3, NP)
        OS = (A @ np.concatenate(BS, 1).T).reshape(3, NP, 3, NP)
        K = OD + np.transpose(OS, (2, 1, 0, 3))
        tr = OS[0, :, 0, :] + OS[1, :, 1, :] + OS[2, :, 2, :]
        for i in range(3):
            K[i, :, i, :] += tr
        out[(P, Q)] = K.reshape(ND, ND)
    return out


@pytest.mark.parametrize("p,theta", [(1, -1.0), (2, 0.0), (3, 1.0), (4, -1.0)])
def test_decomposition_reproduces_the_neighbour_blocks(p, theta):
    m = _mesh("dirichlet")
    o = Oracle(m, p, 1e-3, theta=theta)
    o.make_matrices()
    blocks = o.block_dict(0)
    bbox, hk = o.poly_geometry()
    o.close()
    pairs = [pq for pq in blocks if pq[0] != pq[1]][:40]
    got = _decomposed_neighbour_blocks(m, p, bbox, hk, 10.0, theta, pairs)
    worst = max(float(np.abs(got[pq] - blocks[pq]).max() / np.abs(blocks[pq]).max()) for pq in pairs)
    print(f"p={p} theta={theta}: {len(pairs)} neighbour blocks, worst {worst:.2e}")
    assert worst <= 1e-12, worst
