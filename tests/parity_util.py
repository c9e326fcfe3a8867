"""Helpers shared by the GPU parity tests (imported by tests only).

every_step_parity() runs the device path and the oracle side by side from the
same coefficients and checks u^n after every step against the bars stated in
tests/test_gpu_parity.py: ||u_gpu - u_ref|| / ||u_ref|| <= max(1e-12, 4 x
floor), floor = the largest spread so far of three oracle runs that evaluate
the same steps in other valid orders, and <= 1e-12 in the mass-matrix norm.
"""
import math

import numpy as np

from lymph3d_apsc_gb300 import _lib
from oracle.oracle_py import Oracle, load as oracle_load

TOL_STATE = 1e-12
# The operator apply K u alone (lymph_apply_operator), per polyhedron row,
# against the oracle's FP64 K u with random coefficients:
# max_P ||(K u)_P - (K u)_P,ref|| / ||(K u)_P,ref||.  FP64 blocks: 1e-13;
# FP32 evaluations (FP32 blocks, or FP32 self blocks with the matrix-free
# FP32 face terms): TOL_APPLY_FP32 (measured up to 5.3e-7 at p = 1..4).  A
# dropped or mis-signed face term moves rows by 2e-2 or more (tests/test_mf_formula.py plants each in the oracle).
TOL_APPLY_FP64 = 1e-13
TOL_APPLY_FP32 = 2e-6
# The state of an FP32 operator form after 20 leapfrog steps from the
# oracle's state, in the mass-matrix norm (the L2 norm of the field; the
# Euclidean norm of the coefficients is dominated by the directions the
# ill-conditioned bounding-box basis amplifies): relative <= TOL_STEPS_FP32
# (measured up to 6.5e-6 at p = 4).
TOL_STEPS_FP32 = 2e-5
# the step kernel's column slices per degree (the oracle's device-order variant)
DEVICE_SLICES = {1: 8, 2: 8, 3: 4, 4: 3}


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (den if den > 0 else 1.0))


def mass_norm_rel(o, a, b, Mm=None):
    """||a - b||_M / ||b||_M with the oracle's modal mass matrices."""
    Mm = o.mass(1) if Mm is None else Mm
    Np = o.Np
    d = (a - b).reshape(o.n_poly, 3, Np)
    bb = b.reshape(o.n_poly, 3, Np)
    num = np.einsum("pim,pmn,pin->", d, Mm, d)
    den = np.einsum("pim,pmn,pin->", bb, Mm, bb)
    return math.sqrt(max(num, 0.0) / den)


def start_same(g, o):
    """Same RHS data on both sides; initial coefficients projected by the
    oracle and copied to the device, so the comparison isolates the step."""
    g.MAKE_RHS_FREE(_lib.RHS_STAT, _lib.F_NULL, _lib.GD_NULL, _lib.GN_NULL)
    g.MAKE_RHS_FREE(_lib.RHS_DYN, _lib.F_TIME, _lib.GD, _lib.GN)
    o.make_rhs(0, 0, 0, 0)
    o.make_rhs(1, 1, 1, 1)
    o.modal_project(0, 0)
    o.modal_project(1, 2)
    g.set_state(_lib.SLOT_U0, o.get_state(0))
    g.set_state(_lib.SLOT_V0, o.get_state(2))


def every_step_parity(m, p, g, o, n_steps=25, floor_variants=True):
    """Steps both sides n_steps times (the first step included) and asserts
    the bars after every step.  Returns (last relative difference, floor,
    largest ratio of difference to bar)."""
    start_same(g, o)
    slices = DEVICE_SLICES[p]
    variants = [(1, 1, 0), (0, 1, 0), (0, 0, slices)] if floor_variants else []
    others = []
    for _ in variants:
        ox = Oracle(m, p, g.dt)
        ox.make_matrices()
        ox.make_rhs(0, 0, 0, 0)
        ox.make_rhs(1, 1, 1, 1)
        ox.set_state(0, o.get_state(0))
        ox.set_state(2, o.get_state(2))
        others.append(ox)
    lib = oracle_load()
    Mm = o.mass(1)
    t = 0.0
    worst = floor = e = 0.0
    try:
        for k in range(n_steps):
            if k == 0:
                g.FIRST_TIME_STEP_MATRIX_FREE(t)
                o.first_step(t)
            else:
                g.TIME_STEP_MATRIX_FREE(t)
                o.step(t)
            for (rev, inv, dev), ox in zip(variants, others):
                lib.oracle_set_reverse_sums(rev)
                lib.oracle_set_explicit_inverse(inv)
                lib.oracle_set_device_order(dev)
                try:
                    if k == 0:
                        ox.first_step(t)
                    else:
                        ox.step(t)
                finally:
                    lib.oracle_set_reverse_sums(0)
                    lib.oracle_set_explicit_inverse(0)
                    lib.oracle_set_device_order(0)
            t += g.dt
            ref = o.get_state(_lib.SLOT_UN)
            got = g.get_state(_lib.SLOT_UN)
            floor = max([floor] + [rel(ox.get_state(_lib.SLOT_UN), ref) for ox in others])
            e = rel(got, ref)
            bar = max(TOL_STATE, 4.0 * floor)
            worst = max(worst, e / bar)
            assert e <= bar, (k, e, floor)
            assert mass_norm_rel(o, got, ref, Mm) <= TOL_STATE, k
    finally:
        for ox in others:
            ox.close()
    return e, floor, worst


def row_rel_max(got, want):
    """max over polyhedra P of ||got_P - want_P|| / ||want_P||."""
    d = np.linalg.norm(np.asarray(got) - np.asarray(want), axis=1)
    w = np.linalg.norm(np.asarray(want), axis=1)
    return float(np.max(d / np.where(w > 0, w, 1.0)))


def oracle_apply(o, u, blocks=None):
    """K u from the oracle's assembled FP64 blocks, [n_poly][3Np]."""
    rp, col = o.pattern()
    vals = o.blocks(0) if blocks is None else blocks
    u = np.asarray(u).reshape(o.n_poly, o.nd)
    out = np.zeros_like(u)
    for P in range(o.n_poly):
        for k in range(rp[P], rp[P + 1]):
            out[P] += vals[k] @ u[col[k]]
    return out
