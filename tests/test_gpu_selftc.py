"""The tensor-core blocks of the mixed operators (csrc/selftc.cu) against the
FP64 assembly.

The matrix-free mixed path (LYMPH_MIXED_MF) stores only each polyhedron's
self block, in FP32, and the FP32-block path (LYMPH_MIXED) stores every block
of the block-CSR operator; the self blocks are assembled by k_self_tc<p>,
LYMPH_MIXED's neighbour blocks by k_nb_tc<p>, on the tcgen05 tensor cores:
kind::tf32 MMAs of
operands split into their nearest TF32 value and the TF32-rounded remainder
(four products, FP32-accurate), FP32 accumulation in tensor memory drained
to registers after every 32 quadrature slots (the tensor cores' accumulation
truncates).  Bars (written in each assertion):
  * the self block of every polyhedron against the FP64 path's self block
    (k_assemble, the reference's sums in FP64) with random coefficients:
    max_P ||(K_tc - K_64) u_P|| / ||K_64 u_P|| <= TOL_SELF (1e-6); the
    FP32 rounding of the FP64 block alone, printed beside it, is ~5e-8, and
    the algebra of the decomposition is checked in FP64 on the CPU
    (tests/test_selfblock_formula.py, 1e-12);
  * LYMPH_MIXED's whole operator (self and neighbour blocks) against the
    FP64 blocks, per polyhedron row of K u with random coefficients:
    <= TOL_SELF;
  * the mass matrices of the mixed contexts (the k_assemble CTAs with the
    stiffness skipped) equal the FP64 context's bit for bit;
  * the operator apply of the whole path stays within TOL_APPLY_FP32 of the
    oracle (tests/test_gpu_mf.py, every mesh kind and degree).
"""
import numpy as np
import pytest

from lymph3d_apsc_gb300 import MatrixFree, _lib
from test_gpu_parity import KINDS, _mesh

pytestmark = pytest.mark.gpu

TOL_SELF = 1e-6


def _self_and_mass(m, p, precision, theta=-1.0, blocks=False):
    with MatrixFree(m, p, 1e-3, precision=precision, theta=theta) as g:
        g.MAKE_MATRICES_FREE()
        out = (g.self_blocks(), g.mass(0), g.mass(1))
        return out + ((g.blocks(), g.pattern()) if blocks else ())


def _operator_rel(Ba, Bb, rp, col, seed):
    """max over rows P of ||sum_Q (Ba - Bb)_PQ u_Q|| / ||sum_Q Bb_PQ u_Q||."""
    n, nd = rp.size - 1, Ba.shape[1]
    u = np.random.default_rng(seed).standard_normal((n, nd))
    row = np.repeat(np.arange(n), np.diff(rp))
    ya, yb = np.zeros((n, nd)), np.zeros((n, nd))
    np.add.at(ya, row, np.einsum("krc,kc->kr", Ba, u[col]))
    np.add.at(yb, row, np.einsum("krc,kc->kr", Bb, u[col]))
    return float(np.max(np.linalg.norm(ya - yb, axis=1) / np.linalg.norm(yb, axis=1)))


def _apply_rel(Ka, Kb, seed):
    u = np.random.default_rng(seed).standard_normal((Ka.shape[0], Ka.shape[1]))
    ya = np.einsum("prc,pc->pr", Ka, u)
    yb = np.einsum("prc,pc->pr", Kb, u)
    return float(np.max(np.linalg.norm(ya - yb, axis=1) / np.linalg.norm(yb, axis=1)))


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("p", [1, 2, 3, 4])
def test_tensor_core_self_blocks_match_fp64_assembly(require_gpu, kind, p):
    m = _mesh(kind)
    K64, M64, Mm64, B64, (rp, col) = _self_and_mass(m, p, _lib.FP64, blocks=True)
    e_round = _apply_rel(K64.astype(np.float32).astype(np.float64), K64, 7 + p)
    for name, prec in (("mixed_mf", _lib.MIXED_MF), ("fp32_blocks", _lib.MIXED)):
        got = _self_and_mass(m, p, prec, blocks=(prec == _lib.MIXED))
        Ktc, Mtc, Mmtc = got[:3]
        e = _apply_rel(Ktc, K64, 7 + p)
        print(f"{kind} p={p} {name}: tensor-core self blocks {e:.2e} (FP32 rounding of the FP64 blocks {e_round:.2e})")
        assert e <= TOL_SELF, (name, e)
        assert np.array_equal(Mtc, M64) and np.array_equal(Mmtc, Mm64), name
        if prec == _lib.MIXED:
            e_all = _operator_rel(got[3], B64, rp, col, 13 + p)
            print(f"{kind} p={p} fp32_blocks: whole operator {e_all:.2e}")
            assert e_all <= TOL_SELF, e_all


def test_tensor_core_self_block_of_a_large_polyhedron(require_gpu):
    """One polyhedron of all 162 tetrahedra of a 3^3 x 6 cube, 108 Dirichlet
    faces: more tetrahedra and faces than k_self_tc keeps in shared memory
    (32 and 64), so the slots beyond them read the mesh arrays directly."""
    from lymph3d_apsc_gb300 import mesh as M
    m = M.cube(3, bc="dirichlet", agglomeration="hex", material=(1.0, 2.0, 1.0))
    m.tet_poly = np.zeros_like(m.tet_poly)
    for p in (2, 4):
        K64, M64, _ = _self_and_mass(m, p, _lib.FP64)
        Ktc, Mtc, _ = _self_and_mass(m, p, _lib.MIXED_MF)
        e = _apply_rel(Ktc, K64, 11)
        print(f"one polyhedron of {m.n_tet} tetrahedra, p={p}: {e:.2e}")
        assert e <= TOL_SELF, e
        assert np.array_equal(Mtc, M64)


@pytest.mark.parametrize("theta", [0.0, 1.0])
def test_tensor_core_blocks_other_theta(require_gpu, theta):
    """theta = 0 (IIPG) and 1 (NIPG): the symmetry terms enter O_D and O_S
    with other weights, and the blocks are no longer symmetric; the self
    blocks of the matrix-free context and the whole FP32-block operator."""
    m = _mesh("bfs_lognormal")
    K64, _, _, B64, (rp, col) = _self_and_mass(m, 3, _lib.FP64, theta, blocks=True)
    Ktc, _, _ = _self_and_mass(m, 3, _lib.MIXED_MF, theta)
    e = _apply_rel(Ktc, K64, 3)
    Bmx = _self_and_mass(m, 3, _lib.MIXED, theta, blocks=True)[3]
    e_all = _operator_rel(Bmx, B64, rp, col, 4)
    print(f"theta={theta}: self blocks {e:.2e}, whole FP32-block operator {e_all:.2e}")
    assert e <= TOL_SELF, e
    assert e_all <= TOL_SELF, e_all
    assert not np.allclose(K64, np.transpose(K64, (0, 2, 1)), rtol=1e-3)
