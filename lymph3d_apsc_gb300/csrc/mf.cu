// mf.cu -- the operator apply with matrix-free neighbour terms
// (LYMPH_MIXED_MF).
//
// The neighbour block K_PQ of the assembled operator is a sum over the
// triangles P shares with Q of face-quadrature terms (MAKE_STIFFNESS_FACE,
// src/assemble_element.f90:404-661, inserted by MAKE_MATRICES_FREE,
// src/matrix_free.f90:412-433):
//     K_PQ = -theta/2 I - S - IT/2
// with I, IT and S the consistency, symmetry and penalty integrals over each
// shared triangle, quadrature weights W_q = w_q |face|, P's outward normal n
// and the material of P's tetrahedron.  Contracting the block with u_Q point by point gives the
// same sums in another order:
//     (K_PQ u_Q)_(i,a) = sum_q  grad phi^P_a . G_i  +  phi^P_a s_i,
//     G_ik = -theta/2 W (lambda (n.v) delta_ik + mu (n_i v_k + v_i n_k)),
//     s_i  = -W (sigma (T v)_i + h_i / 2),
//     h_i  = lambda sum_j n_j D_ji + mu n_i tr D + mu sum_k n_k D_ik,
// where v = u_Q(x_q), D_jk = d_k u_Q,j (x_q) are Q's field and gradient at
// the point and T = (n_i^2 + sum_{k!=i} n_k^2 / 2 on the diagonal,
// n_i n_j / 2 off it).  h is the reference's symmetry term IT with its
// (i, j) order (it is the traction of u_Q only when lambda = mu).
//
// So the neighbour blocks are never stored.  One CTA per polyhedron P (or,
// for a batch of problems, persistent CTAs over (problem, polyhedron) items)
// evaluates u_Q and grad u_Q at the quadrature points of every triangle P
// shares with a neighbour Q, from the Legendre basis on Q's bounding box,
// forms G and s, tests them against P's basis, and applies its FP32 self
// block.  Everything runs in FP32 from per-triangle geometry precomputed
// once (quadrature origin and edge vectors, normal, area, material, penalty);
// both basis contractions are sum-factorised over the Legendre degree
// triples.  The row sums are combined in FP64 in a fixed order and finished
// exactly like the fused kernel (right-hand side, M^-1 in FP64, leapfrog
// update).  A step reads the self blocks (1/nb of the operator bytes) and the
// per-triangle geometry instead of every block.

#include <cstddef>
#include <cstring>

#include "step_body.cuh"

namespace {

using namespace stepk;

struct MfTri {          // one triangle of a neighbour block, seen from the row polyhedron P
    float oP[3];        // quadrature point x_q = c_P + oP + xi_q e1 + eta_q e2 (c_P: P's box centre)
    float oQ[3];        // the same point as c_Q + oQ + xi_q e1 + eta_q e2 (Q's box centre)
    float e1[3];
    float e2[3];
    float n[3];         // P's outward unit normal
    float area;         // W_q = w_q area
    float lam, mu;      // material of P's tetrahedron
    float sigma;        // penalty alpha p^2 / min(h_P, h_Q) (lambda + 2 mu)
    int32_t Q;          // neighbour polyhedron
};
static_assert(sizeof(MfTri) == 80, "MfTri is 5 x 16 bytes");
constexpr int MF_TRI_CHUNKS = (int)(sizeof(MfTri) / 16);

struct MfPoly {         // Legendre scaling of a bounding box: xp = (x - centre) ih, phi = sc L(xp_x) L(xp_y) L(xp_z)
    float ih[3];        // (the points are stored relative to the centres: MfTri)
    float sc;
};
static_assert(sizeof(MfPoly) == 16, "MfPoly is one 16-byte copy");

// The triangle rule of the neighbour terms.  The integrand of every term of
// K_PQ u_Q on a triangle is a polynomial of total degree <= 2p in the
// triangle's parameters (xi, eta): phi^P and u_Q are degree-p polynomials
// composed with affine maps, and the material is constant per tetrahedron.
// The reference's collapsed Gauss rule with (p+1)^2 points
// (mapping_quadrature_2D, Poly_ref_mappings.f90:137-186) is exact to that
// degree, and so is each rule below, with fewer points: 3 / 6 / 12 / 16 for
// p = 1..4 against 4 / 9 / 16 / 25.  Both give the same integrals in exact
// arithmetic.  These are fully symmetric rules with interior nodes and
// positive weights on the reference triangle (0,0), (1,0), (0,1), weights
// summing to 1/2 like the reference's.  Each orbit of the symmetry group
// (the centroid; (a, a, 1-2a) in barycentric coordinates, 3 points; (a, b,
// 1-a-b), 6 points) has one weight.  The nodes and weights solve the moment
// equations sum_q w_q xi^i eta^j = i! j! / (i+j+2)! for i + j <= 2p
// (derive_face_rules.py beside this file solves them to 40 digits;
// tests/test_abi_cpu.py checks every moment of the values below).
constexpr int MF_FACE_NQ[5] = {0, 3, 6, 12, 16};
constexpr int MF_FACE_NQ_MAX = 16;
// (xi, eta, w) per node, degrees 1..4 one after another
constexpr double kFaceRule[3 * (3 + 6 + 12 + 16)] = {
    // p = 1, exact to degree 2
    0.16666666666666666667, 0.16666666666666666667, 0.16666666666666666667,
    0.16666666666666666667, 0.66666666666666666667, 0.16666666666666666667,
    0.66666666666666666667, 0.16666666666666666667, 0.16666666666666666667,
    // p = 2, exact to degree 4
    0.09157621350977074346, 0.09157621350977074346, 0.054975871827660933819,
    0.09157621350977074346, 0.81684757298045851308, 0.054975871827660933819,
    0.81684757298045851308, 0.09157621350977074346, 0.054975871827660933819,
    0.44594849091596488632, 0.44594849091596488632, 0.11169079483900573285,
    0.44594849091596488632, 0.10810301816807022736, 0.11169079483900573285,
    0.10810301816807022736, 0.44594849091596488632, 0.11169079483900573285,
    // p = 3, exact to degree 6
    0.24928674517091042129, 0.24928674517091042129, 0.058393137863189683013,
    0.24928674517091042129, 0.50142650965817915742, 0.058393137863189683013,
    0.50142650965817915742, 0.24928674517091042129, 0.058393137863189683013,
    0.06308901449150222834, 0.06308901449150222834, 0.02542245318510340846,
    0.06308901449150222834, 0.87382197101699554332, 0.02542245318510340846,
    0.87382197101699554332, 0.06308901449150222834, 0.02542245318510340846,
    0.31035245103378440542, 0.053145049844816947353, 0.041425537809186787597,
    0.053145049844816947353, 0.31035245103378440542, 0.041425537809186787597,
    0.31035245103378440542, 0.63650249912139864723, 0.041425537809186787597,
    0.63650249912139864723, 0.31035245103378440542, 0.041425537809186787597,
    0.053145049844816947353, 0.63650249912139864723, 0.041425537809186787597,
    0.63650249912139864723, 0.053145049844816947353, 0.041425537809186787597,
    // p = 4, exact to degree 8
    0.33333333333333333333, 0.33333333333333333333, 0.072157803838893584126,
    0.45929258829272315603, 0.45929258829272315603, 0.047545817133642312397,
    0.45929258829272315603, 0.081414823414553687942, 0.047545817133642312397,
    0.081414823414553687942, 0.45929258829272315603, 0.047545817133642312397,
    0.17056930775176020662, 0.17056930775176020662, 0.051608685267359125141,
    0.17056930775176020662, 0.65886138449647958676, 0.051608685267359125141,
    0.65886138449647958676, 0.17056930775176020662, 0.051608685267359125141,
    0.050547228317030975458, 0.050547228317030975458, 0.016229248811599040155,
    0.050547228317030975458, 0.89890554336593804908, 0.016229248811599040155,
    0.89890554336593804908, 0.050547228317030975458, 0.016229248811599040155,
    0.72849239295540428124, 0.26311282963463811342, 0.013615157087217497132,
    0.26311282963463811342, 0.72849239295540428124, 0.013615157087217497132,
    0.72849239295540428124, 0.0083947774099576053372, 0.013615157087217497132,
    0.0083947774099576053372, 0.72849239295540428124, 0.013615157087217497132,
    0.26311282963463811342, 0.0083947774099576053372, 0.013615157087217497132,
    0.0083947774099576053372, 0.26311282963463811342, 0.013615157087217497132,
};
constexpr int face_rule_offset(int p) { return p <= 1 ? 0 : face_rule_offset(p - 1) + MF_FACE_NQ[p - 1]; }

constexpr int MF_THREADS = 128;
constexpr int MF_SLOTS = MF_THREADS / 3;   // test phase: point slots of three lanes (one per row component)

template <int PD> struct MfShape {
    static constexpr int NP = Deg<PD>::NP, ND = Deg<PD>::ND;
    static constexpr int L = PD + 1;              // Legendre degrees per direction
    static constexpr int NQ2 = MF_FACE_NQ[PD];    // quadrature points per triangle
    static constexpr int CT = MF_THREADS / NQ2;   // triangles per chunk
    static constexpr int NPT = CT * NQ2;          // points per chunk (one evaluating thread each)
    // a point's (L, L') values of the three directions, padded to an odd
    // number of 16-byte words so the points of a warp fall on distinct banks
    static constexpr int LEGW = ((3 * L + 1) / 2 % 2 == 1) ? 2 * ((3 * L + 1) / 2) : 2 * ((3 * L + 1) / 2) + 2;
    static_assert(ND <= MF_THREADS, "one thread per row of the self block");
};

// Position of basis function (a, b, c) in the reference's order.
template <int PD> struct Bidx {
    int i[PD + 1][PD + 1][PD + 1];
    constexpr Bidx() : i() {
        constexpr Blist<PD> BL{};
        for (int k = 0; k < Deg<PD>::NP; ++k) i[BL.d[k][0]][BL.d[k][1]][BL.d[k][2]] = k;
    }
};

// Field and gradient of the three components at a point by sum
// factorisation over the basis triples (a, b, c): with X_a = (L_a, L'_a)(x)
// and likewise Y, Z,
//   w0_ab = sum_c u_abc Z_c,  w1_ab = sum_c u_abc Z'_c,
//   r0_a = sum_b w0_ab Y_b,  r1_a = sum_b w0_ab Y'_b,  r2_a = sum_b w1_ab Y_b,
//   v = sum_a r0_a X_a, d_x = sum_a r0_a X'_a, d_y = sum_a r1_a X_a, d_z = sum_a r2_a X_a
// (unscaled: the caller applies the bounding-box factors).  uc[i] holds
// (u_0, u_1, u_2, 0) of basis function i.  Each w sum runs over c = p-a-b
// down to 0 (the basis order), each r sum over b = 0.., each output over
// a = 0..; one (a, b) group is live at a time, so the three components cost
// no more registers than one did with every w_ab held.
template <int PD>
__device__ __forceinline__ void eval_sf3(const float4* uc, const float2* X, const float2* Y, const float2* Z,
                                         float (&o)[3][4]) {
    constexpr Bidx<PD> BI{};
#pragma unroll
    for (int j = 0; j < 3; ++j) o[j][0] = o[j][1] = o[j][2] = o[j][3] = 0.0f;
#pragma unroll
    for (int a = 0; a <= PD; ++a) {
        float r[3][3];
#pragma unroll
        for (int j = 0; j < 3; ++j) r[j][0] = r[j][1] = r[j][2] = 0.0f;
#pragma unroll
        for (int b = 0; b <= PD - a; ++b) {
            float w0[3] = {0.0f, 0.0f, 0.0f}, w1[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
            for (int c = PD - a - b; c >= 0; --c) {
                const float4 uu = uc[BI.i[a][b][c]];
                const float u3[3] = {uu.x, uu.y, uu.z};
#pragma unroll
                for (int j = 0; j < 3; ++j) {
                    w0[j] = fmaf(u3[j], Z[c].x, w0[j]);
                    w1[j] = fmaf(u3[j], Z[c].y, w1[j]);
                }
            }
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                r[j][0] = fmaf(w0[j], Y[b].x, r[j][0]);
                r[j][1] = fmaf(w0[j], Y[b].y, r[j][1]);
                r[j][2] = fmaf(w1[j], Y[b].x, r[j][2]);
            }
        }
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            o[j][0] = fmaf(r[j][0], X[a].x, o[j][0]);
            o[j][1] = fmaf(r[j][0], X[a].y, o[j][1]);
            o[j][2] = fmaf(r[j][1], X[a].x, o[j][2]);
            o[j][3] = fmaf(r[j][2], X[a].x, o[j][3]);
        }
    }
}

// The transpose: acc_abc += X'_a Y_b Z_c gx + X_a Y'_b Z_c gy + X_a Y_b Z'_c gz
// + X_a Y_b Z_c s, factored the same way (one (a, b) factor pair live at a time).
template <int PD>
__device__ __forceinline__ void test_sf(float* acc, const float2* X, const float2* Y, const float2* Z, float gx, float gy,
                                        float gz, float s) {
    constexpr Bidx<PD> BI{};
#pragma unroll
    for (int a = 0; a <= PD; ++a) {
        const float t0 = fmaf(X[a].y, gx, X[a].x * s), t1 = X[a].x * gy, t2 = X[a].x * gz;
#pragma unroll
        for (int b = 0; b <= PD - a; ++b) {
            const float q0 = fmaf(Y[b].x, t0, Y[b].y * t1), q1 = Y[b].x * t2;
#pragma unroll
            for (int c = 0; c <= PD - a - b; ++c) {
                float& r = acc[BI.i[a][b][c]];
                r = fmaf(Z[c].x, q0, fmaf(Z[c].y, q1, r));
            }
        }
    }
}

struct MfArgs {
    StepArgs s;                 // CSR pattern, M^-1, right-hand sides, state, status
    const float* Kself;         // [n_poly][ND * ND] column-major self blocks
    const int32_t* qrec;        // per polyhedron MF_REC ints: triangle range and neighbours (k_mf_qrec)
    const MfTri* tri;           // parallel to the block face lists
    const MfPoly* poly;         // [n_poly]
    const float4* u32;          // operator input in FP32: [n_poly][Np] (u_0, u_1, u_2, 0)
    int64_t kself_bytes;        // size of Kself
    int64_t minv_bytes;         // size of the M^-1 array
    float quad[3 * MF_FACE_NQ_MAX];   // (xi, eta, w) of the triangle rule's nodes
    float theta;
};

// One record of MF_REC ints per polyhedron, read in one coalesced load at the
// start of its pass: [0, 1] the first triangle fb (int64, low word first),
// [2] the number of triangles, [4, 4 + MF_MAXT) the neighbour polyhedron of
// its first MF_MAXT triangles (the rest are read from the triangle records).
constexpr int MF_REC = 64;
constexpr int MF_MAXT = MF_REC - 4;   // triangles whose neighbour index is kept in shared memory

__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)), "l"(src)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N> __device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// Prefetch [p, p + bytes) of an allocation [base, base + total) into L2 (one
// bulk prefetch, range widened to 16-byte bounds inside the allocation).
__device__ __forceinline__ void prefetch_l2(const void* base, int64_t total, const void* p, int64_t bytes) {
    const uintptr_t b0 = (uintptr_t)base, lim = (b0 + (uintptr_t)total) & ~(uintptr_t)15;
    uintptr_t s = (uintptr_t)p & ~(uintptr_t)15, e = ((uintptr_t)p + (uintptr_t)bytes + 15) & ~(uintptr_t)15;
    if (e > lim) e = lim;
    if (s < b0 || e <= s) return;
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(s), "r"((uint32_t)(e - s)) : "memory");
}

// One CTA per polyhedron P.  At the start the CTA reads P's record (its
// triangles' range and neighbours, one coalesced load), and one thread
// prefetches into L2 what the CTA reads later (the FP32 self block, M^-1,
// the right-hand sides and the state rows).  The self-block rows (thread
// r < ND, K_PP streamed) are computed while the first chunk's copies are in
// flight (p = 4) or after the face loop (p <= 3).  Neighbour
// triangles, CT triangles at a time, their geometry, Q's box and Q's FP32
// coefficients copied into shared memory with cp.async one chunk ahead
// (double-buffered): thread t evaluates point t -- Q's field and gradient,
// the three components together by sum factorisation, the three flux rows,
// and P's Legendre values, kept in shared memory; then thread 3 k + i accumulates
// row component i of P's test sums over the points k, k + 42, ... of the
// chunk in Np registers (the sum-factorised transpose).  Then the 42 slots'
// partial rows are summed in a fixed order and added to the self-block rows.
// Shared-memory layout of one polyhedron's pass; the face-loop buffers and
// the final reduction share storage.
template <int PD> struct MfSmem {
    using S = MfShape<PD>;
    struct Loop {
        float2 leg[S::NPT][S::LEGW];   // P's (L, L') per point: direction-major, then degree
        float4 flux[S::NPT][3];        // (G_i0, G_i1, G_i2, s_i) per point, scaled by P's map
    };
    struct Fin {                       // after the face loop
        float red[MF_SLOTS][S::ND];    // the slots' partial rows
        double b[S::ND];               // the right-hand side of the M^-1 apply (beside red: the
                                       // last reads of red and the writes of b are not separated
                                       // by a barrier)
    };
    union Work {
        Loop loop;
        Fin fin;
    };
    Work w;
    float4 uQ[2][S::CT][S::NP];        // (u_0, u_1, u_2, 0) per basis function
    alignas(16) MfTri tri[2][S::CT];
    alignas(16) MfPoly polyQ[2][S::CT];
    float quad[3 * S::NQ2];
    float uP[S::ND];
    int rec[MF_REC];
};
// every cp.async destination starts on a 16-byte boundary (with the shared
// array itself 16-byte aligned)
template <int PD> constexpr bool mf_smem_aligned() {
    return offsetof(MfSmem<PD>, uQ) % 16 == 0 && offsetof(MfSmem<PD>, tri) % 16 == 0 &&
           offsetof(MfSmem<PD>, polyQ) % 16 == 0 && sizeof(MfTri) % 16 == 0 && sizeof(MfPoly) % 16 == 0;
}
static_assert(mf_smem_aligned<1>() && mf_smem_aligned<2>() && mf_smem_aligned<3>() && mf_smem_aligned<4>(),
              "cp.async destinations must be 16-byte aligned");

// The pass of polyhedron P (every thread of the CTA calls it; it
// synchronises): the per-problem tables come from A, the state, right-hand
// sides and M^-1 from sa.
template <int PD, int MODE>
__device__ __forceinline__ void mf_poly(const MfArgs& A, const StepArgs& sa, int P, char* smem) {
    using S = MfShape<PD>;
    constexpr int NP = S::NP, ND = S::ND, L = S::L, NQ2 = S::NQ2, CT = S::CT, NP2 = NP * NP;
    MfSmem<PD>& sm = *reinterpret_cast<MfSmem<PD>*>(smem);
    auto& s_w = sm.w;
    auto& s_tri = sm.tri;
    auto& s_polyQ = sm.polyQ;
    auto& s_uQ = sm.uQ;
    float* s_quad = sm.quad;
    float* s_uP = sm.uP;
    double* s_b = sm.w.fin.b;
    const int tid = threadIdx.x;
    // the polyhedron's record (triangle range and neighbours) in one load,
    // so the first chunk's staging waits on one global round trip, not three
    if (tid < MF_REC) sm.rec[tid] = A.qrec[(int64_t)P * MF_REC + tid];
    if (tid == 0) {
        const int64_t nb = (int64_t)ND * ND * 4, vb = (int64_t)ND * 8;
        prefetch_l2(A.Kself, A.kself_bytes, A.Kself + (int64_t)P * ND * ND, nb);
        prefetch_l2(sa.Minv, A.minv_bytes, sa.Minv + (int64_t)P * NP2, (int64_t)NP2 * 8);
        const int64_t sb = (int64_t)sa.n_poly * ND * 8;
        if (MODE == MODE_STEP || MODE == MODE_FIRST) {
            prefetch_l2(sa.rhs_stat, sb, sa.rhs_stat + (int64_t)P * ND, vb);
            prefetch_l2(sa.rhs_dyn, sb, sa.rhs_dyn + (int64_t)P * ND, vb);
        }
        prefetch_l2(sa.u0, sb, sa.u0 + (int64_t)P * ND, vb);
        prefetch_l2(sa.un, sb, sa.un + (int64_t)P * ND, vb);
    }
    for (int i = tid; i < 3 * NQ2; i += MF_THREADS) s_quad[i] = A.quad[i];
    for (int i = tid; i < ND; i += MF_THREADS) {
        const float4 w = A.u32[(int64_t)P * NP + i % NP];
        const int comp = i / NP;
        s_uP[i] = comp == 0 ? w.x : (comp == 1 ? w.y : w.z);
    }
    __syncthreads();
    const int64_t fb = (int64_t)(uint32_t)sm.rec[0] | ((int64_t)sm.rec[1] << 32);
    const int ntri = sm.rec[2];

    // neighbour of triangle i of P (shared memory for the first MF_MAXT)
    auto getQ = [&](int i) -> int { return i < MF_MAXT ? sm.rec[4 + i] : A.tri[fb + i].Q; };
    auto stage = [&](int c, int b) {  // chunk starting at triangle c into buffer b
        const int nt = (ntri - c) < CT ? ntri - c : CT;
        const char* src = (const char*)(A.tri + fb + c);
        for (int i = tid; i < nt * MF_TRI_CHUNKS; i += MF_THREADS) cp_async16((char*)s_tri[b] + 16 * i, src + 16 * i);
        for (int i = tid; i < nt; i += MF_THREADS) cp_async16(&s_polyQ[b][i], A.poly + getQ(c + i));
        for (int i = tid; i < nt * NP; i += MF_THREADS) {
            const int t = i / NP, bb = i - t * NP;
            cp_async16(&s_uQ[b][t][bb], A.u32 + (int64_t)getQ(c + t) * NP + bb);
        }
        cp_async_commit();
    };

    // ---- neighbour triangles ----
    const MfPoly pP = A.poly[P];
    const int slot = tid / 3, ci = tid - 3 * (tid / 3);   // test phase: point slot, row component
    const bool tact = slot < MF_SLOTS;
    if (ntri > 0) stage(0, 0);
    // ---- self block (FP32) rows, thread r < ND, K_PP streamed: at p = 4
    // while chunk 0's copies are in flight (its loads go out before the test
    // sums take their registers: 1 % faster on the 46,767-polyhedron mesh),
    // at p <= 3 after the face loop with the test sums parked (3 % faster
    // there); the same sums in the same order either way ----
    constexpr bool SELF_FIRST = PD >= 4;
    auto self_rows = [&]() -> float {
        float y = 0.0f;
        if (tid < ND) {
            const float* Kb = A.Kself + (int64_t)P * ND * ND + tid;
            float a0 = 0.0f, a1 = 0.0f;
#pragma unroll
            for (int c = 0; c < ND; c += 2) {
                a0 = fmaf(__ldcs(Kb + (int64_t)c * ND), s_uP[c], a0);
                if (c + 1 < ND) a1 = fmaf(__ldcs(Kb + (int64_t)(c + 1) * ND), s_uP[c + 1], a1);
            }
            y = a0 + a1;
        }
        return y;
    };
    float yself = 0.0f;
    if constexpr (SELF_FIRST) yself = self_rows();
    float acc[NP];
#pragma unroll
    for (int i = 0; i < NP; ++i) acc[i] = 0.0f;
    for (int c = 0, k = 0; c < ntri; c += CT, ++k) {
        const int b = k & 1, nt = (ntri - c) < CT ? ntri - c : CT;
        if (c + CT < ntri) stage(c + CT, b ^ 1);
        else cp_async_commit();
        cp_async_wait<1>();
        __syncthreads();  // chunk c staged for all threads; the previous test phase is done
        // ---- per point: u_Q and grad u_Q, the flux, P's Legendre values ----
        if (tid < nt * NQ2) {
            const int t = tid / NQ2, q = tid % NQ2;
            const MfTri& T = s_tri[b][t];
            const float xi = s_quad[3 * q], eta = s_quad[3 * q + 1];
            const float W = s_quad[3 * q + 2] * T.area;
            // the point relative to Q's and to P's box centre (small operands,
            // so the Legendre arguments keep FP32 relative accuracy)
            float xq[3], xp[3];
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const float r = fmaf(eta, T.e2[d], xi * T.e1[d]);
                xq[d] = T.oQ[d] + r;
                xp[d] = T.oP[d] + r;
            }
            const MfPoly& pq = s_polyQ[b][t];
            float2 X[L], Y[L], Z[L];
            legendre_f32<PD>(xq[0] * pq.ih[0], X);
            legendre_f32<PD>(xq[1] * pq.ih[1], Y);
            legendre_f32<PD>(xq[2] * pq.ih[2], Z);
            // Q's map: phi = sc L L L, d_k phi = sc ih_k (...)
            const float sq = pq.sc, gx = sq * pq.ih[0], gy = sq * pq.ih[1], gz = sq * pq.ih[2];
            float v[3], D[3][3];
            {
                float o[3][4];
                eval_sf3<PD>(s_uQ[b][t], X, Y, Z, o);
#pragma unroll
                for (int j = 0; j < 3; ++j) {
                    v[j] = o[j][0] * sq;
                    D[j][0] = o[j][1] * gx;
                    D[j][1] = o[j][2] * gy;
                    D[j][2] = o[j][3] * gz;
                }
            }
            const float* n = T.n;
            const float nv = n[0] * v[0] + n[1] * v[1] + n[2] * v[2];
            const float trD = D[0][0] + D[1][1] + D[2][2];
            const float cg = -0.5f * A.theta * W;
            const float nn0 = n[0] * n[0], nn1 = n[1] * n[1], nn2 = n[2] * n[2];
            const float Tdiag[3] = {nn0 + 0.5f * nn1 + 0.5f * nn2, nn1 + 0.5f * nn0 + 0.5f * nn2,
                                    nn2 + 0.5f * nn0 + 0.5f * nn1};
            const float sP = pP.sc, hx = sP * pP.ih[0], hy = sP * pP.ih[1], hz = sP * pP.ih[2];
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                float G[3];
#pragma unroll
                for (int kk = 0; kk < 3; ++kk)
                    G[kk] = cg * ((i == kk ? T.lam * nv : 0.0f) + T.mu * (n[i] * v[kk] + v[i] * n[kk]));
                float Tv = Tdiag[i] * v[i];
#pragma unroll
                for (int j = 0; j < 3; ++j)
                    if (j != i) Tv += 0.5f * n[i] * n[j] * v[j];
                const float h = T.lam * (n[0] * D[0][i] + n[1] * D[1][i] + n[2] * D[2][i]) + T.mu * n[i] * trD +
                                T.mu * (n[0] * D[i][0] + n[1] * D[i][1] + n[2] * D[i][2]);
                const float s = -W * (T.sigma * Tv + 0.5f * h);
                s_w.loop.flux[tid][i] = make_float4(G[0] * hx, G[1] * hy, G[2] * hz, s * sP);
            }
            // P's values, written as 16-byte words (the padded row keeps the
            // stores of a quarter-warp on distinct banks)
            constexpr int LW = (3 * L + 1) / 2;
            float2 LP[2 * LW];
            legendre_f32<PD>(xp[0] * pP.ih[0], LP);
            legendre_f32<PD>(xp[1] * pP.ih[1], LP + L);
            legendre_f32<PD>(xp[2] * pP.ih[2], LP + 2 * L);
            if (2 * LW > 3 * L) LP[2 * LW - 1] = make_float2(0.0f, 0.0f);
            float4* lw = reinterpret_cast<float4*>(s_w.loop.leg[tid]);
#pragma unroll
            for (int k = 0; k < LW; ++k) lw[k] = make_float4(LP[2 * k].x, LP[2 * k].y, LP[2 * k + 1].x, LP[2 * k + 1].y);
        }
        __syncthreads();
        // ---- test against P's basis: thread (slot, component) over the chunk's points ----
        if (tact) {
            for (int pt = slot; pt < nt * NQ2; pt += MF_SLOTS) {
                float2 LG[2 * ((3 * L + 1) / 2)];
                const float4* lp = reinterpret_cast<const float4*>(s_w.loop.leg[pt]);
#pragma unroll
                for (int k = 0; k < (3 * L + 1) / 2; ++k) {
                    const float4 q = lp[k];
                    LG[2 * k] = make_float2(q.x, q.y);
                    LG[2 * k + 1] = make_float2(q.z, q.w);
                }
                const float4 f = s_w.loop.flux[pt][ci];
                test_sf<PD>(acc, LG, LG + L, LG + 2 * L, f.x, f.y, f.z, f.w);
            }
        }
    }
    cp_async_wait<0>();
    __syncthreads();  // the loop buffers are free: reuse them for the slots' rows
    if (tact) {
#pragma unroll
        for (int i = 0; i < NP; ++i) s_w.fin.red[slot][ci * NP + i] = acc[i];
    }
    if constexpr (!SELF_FIRST) yself = self_rows();
    __syncthreads();
    double y = 0.0;
    if (tid < ND) {
        float t = 0.0f;
#pragma unroll 6
        for (int kk = 0; kk < MF_SLOTS; ++kk) t += s_w.fin.red[kk][tid];
        y = (double)yself + (double)t;
    }
    finish_poly<PD, MODE>(sa, P, y, s_b);
}

// CTAs per SM that the register budget is sized for, per degree (index p;
// measured on the 46,767-polyhedron mesh: more CTAs per SM pay while the
// registers still hold the test sums without spilling; at p = 1 shared
// memory holds 8).
constexpr int MF_MINB[5] = {5, 8, 8, 7, 5};
constexpr int MF_BATCH_MINB[5] = {5, 8, 8, 7, 5};   // the same for k_mf_batch<p>

template <int PD, int MODE>
__global__ void __launch_bounds__(MF_THREADS, MF_MINB[PD]) k_mf(const __grid_constant__ MfArgs A) {
    __shared__ __align__(16) char smem[sizeof(MfSmem<PD>)];
    mf_poly<PD, MODE>(A, A.s, blockIdx.x, smem);
}

// ---- many problems in one persistent launch per step (lymph_batch) ----

struct MfBatchProblem {
    MfArgs a;          // the problem's tables; a.s's state pointers are set per step
    double* buf[2];
    int cur0;          // buffer parity when the run started
    int p;
};

// Persistent CTAs pull (problem, polyhedron) items of degree PD from an
// atomic queue and run mf_poly on each: the same per-polyhedron pass as k_mf,
// so results equal stepping each problem alone.  One launch per degree
// present, so each degree runs with its own register and shared-memory
// budget (the CTAs per SM of k_mf).
template <int PD>
__global__ void __launch_bounds__(MF_THREADS, MF_BATCH_MINB[PD])
k_mf_batch(const MfBatchProblem* __restrict__ probs, const int2* __restrict__ items, int n_items, int* queue,
           const int64_t* step_idx, const double* gvals, int64_t g_stride) {
    __shared__ __align__(16) char smem[sizeof(MfSmem<PD>)];
    __shared__ int s_item;
    const int64_t k = *step_idx;
    for (;;) {
        if (threadIdx.x == 0) s_item = atomicAdd(queue, 1);
        __syncthreads();
        const int it = s_item;
        __syncthreads();
        if (it >= n_items) break;
        const int2 w = items[it];
        const MfBatchProblem& pb = probs[w.x];
        StepArgs s = pb.a.s;
        const int cur = pb.cur0 ^ (int)(k & 1);
        s.un = pb.buf[cur];
        s.u0 = pb.buf[cur ^ 1];
        s.out = pb.buf[cur ^ 1];
        s.gvals = gvals + (int64_t)w.x * g_stride;
        s.step_idx = step_idx;
        mf_poly<PD, MODE_STEP>(pb.a, s, w.y, smem);
    }
}

// The FP32 copies of every problem's u^n, a warp per (problem, polyhedron) item.
__global__ void k_mf_u32_batch(const MfBatchProblem* __restrict__ probs, const int2* __restrict__ items, int n_items,
                               const int64_t* step_idx) {
    const int64_t k = *step_idx;
    const int item = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (item >= n_items) return;
    const int2 w = items[item];
    const MfBatchProblem& pb = probs[w.x];
    const int NP = (pb.p + 1) * (pb.p + 2) * (pb.p + 3) / 6;
    const double* u = pb.buf[pb.cur0 ^ (int)(k & 1)] + (int64_t)w.y * 3 * NP;
    float4* o = const_cast<float4*>(pb.a.u32) + (int64_t)w.y * NP;
    for (int m = lane; m < NP; m += 32) o[m] = make_float4((float)u[m], (float)u[NP + m], (float)u[2 * NP + m], 0.0f);
}

// u32[P][m] = (u[P][0][m], u[P][1][m], u[P][2][m], 0): the operator input in
// FP32, converted once per pass instead of once per triangle that reads it.
__global__ void k_mf_u32(int64_t n, int NP, const double* __restrict__ u, float4* __restrict__ u32) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t P = i / NP, m = i - P * NP;
        const double* up = u + P * 3 * NP + m;
        u32[i] = make_float4((float)up[0], (float)up[NP], (float)up[2 * NP], 0.0f);
    }
}

// Per-triangle geometry of every neighbour block (FP64 set-up data rounded to
// FP32 once): the quadrature map of P's tetrahedron face (basis_boundary,
// basis_function.f90:560-577: x = Fk node_maps(:,:,f) (xi, eta, 1, 1)),
// normal, area, material and penalty.
__global__ void k_mf_tris(int64_t n_blocks, const int32_t* __restrict__ blk_row, const int32_t* __restrict__ col,
                          const int64_t* __restrict__ bf_ptr, const int32_t* __restrict__ bf,
                          const int32_t* __restrict__ neigh, const int32_t* __restrict__ tet_poly,
                          const int32_t* __restrict__ tet_mat, const double* __restrict__ mat,
                          const double* __restrict__ fk, const double* __restrict__ nrm,
                          const double* __restrict__ area, const double* __restrict__ hk,
                          const double* __restrict__ bbox, const RefTables* ref, double alpha, int p, MfTri* out,
                          int* status) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= n_blocks) return;
    const int P = blk_row[k], Q = col[k];
    if (P == Q) return;
    for (int64_t e = bf_ptr[k]; e < bf_ptr[k + 1]; ++e) {
        const int code = bf[e];
        const int t = code >> 2, f = code & 3;
        // every entry names the block's column Q, so the step kernel's reads
        // stay in bounds even when the check below fails
        if (neigh[code] < 0 || tet_poly[neigh[code]] != Q) atomicOr(status, ST_BAD_INDEX);
        MfTri T;
        const double* F = fk + (int64_t)t * 12;
        const double* nm = &ref->node_maps[f * 16];
        double cmap[3][4];
        for (int j = 0; j < 3; ++j)
            for (int l = 0; l < 4; ++l) {
                double s = 0.0;
                for (int m = 0; m < 4; ++m) s += F[j * 4 + m] * nm[m * 4 + l];
                cmap[j][l] = s;
            }
        for (int j = 0; j < 3; ++j) {
            const double o = cmap[j][2] + cmap[j][3];
            const double cP = (bbox[P * 6 + 2 * j] + bbox[P * 6 + 2 * j + 1]) / 2.0;
            const double cQ = (bbox[Q * 6 + 2 * j] + bbox[Q * 6 + 2 * j + 1]) / 2.0;
            T.oP[j] = (float)(o - cP);
            T.oQ[j] = (float)(o - cQ);
            T.e1[j] = (float)cmap[j][0];
            T.e2[j] = (float)cmap[j][1];
            T.n[j] = (float)nrm[(int64_t)t * 12 + f * 3 + j];
        }
        T.area = (float)area[(int64_t)t * 4 + f];
        const int mid = tet_mat[t];
        const double lam = mat[mid * 3 + 1], mu = mat[mid * 3 + 2];
        T.lam = (float)lam;
        T.mu = (float)mu;
        T.sigma = (float)(alpha * (double)(p * p) / fmin(hk[P], hk[Q]) * (lam + 2 * mu));
        T.Q = Q;
        out[e] = T;
    }
}

// The per-polyhedron records of mf_poly (MF_REC ints each): the neighbour
// triangles of row P are the blocks after the self block (which comes first
// in every row), bf_ptr[row_ptr[P] + 1] to bf_ptr[row_ptr[P + 1]].
__global__ void k_mf_qrec(int n_poly, const int32_t* __restrict__ row_ptr, const int64_t* __restrict__ bf_ptr,
                          const MfTri* __restrict__ tri, int32_t* __restrict__ rec) {
    const int P = blockIdx.x * blockDim.x + threadIdx.x;
    if (P >= n_poly) return;
    const int64_t fb = bf_ptr[row_ptr[P] + 1], fe = bf_ptr[row_ptr[P + 1]];
    int32_t* r = rec + (int64_t)P * MF_REC;
    r[0] = (int32_t)(uint32_t)((uint64_t)fb & 0xffffffffu);
    r[1] = (int32_t)(fb >> 32);
    r[2] = (int32_t)(fe - fb);
    r[3] = 0;
    for (int i = 0; i < MF_MAXT; ++i) r[4 + i] = i < fe - fb ? tri[fb + i].Q : -1;
}

__global__ void k_mf_polys(int n_poly, const double* __restrict__ bbox, MfPoly* out) {
    const int P = blockIdx.x * blockDim.x + threadIdx.x;
    if (P >= n_poly) return;
    MfPoly m;
    double hprod = 1.0;
    for (int d = 0; d < 3; ++d) {
        const double a = bbox[P * 6 + 2 * d], b = bbox[P * 6 + 2 * d + 1];
        const double hb = (b - a) / 2.0;
        m.ih[d] = (float)(1.0 / hb);
        hprod *= hb;
    }
    m.sc = (float)(1.0 / sqrt(hprod));
    out[P] = m;
}

// The context's tables in kernel arguments (s: the step's CSR pattern, state
// and right-hand sides).
MfArgs mf_args(const lymph_ctx* c, const StepArgs& s) {
    MfArgs a;
    a.s = s;
    a.Kself = (const float*)c->d_K;
    a.qrec = (const int32_t*)c->d_mf_range;
    a.tri = (const MfTri*)c->d_mf_tri;
    a.poly = (const MfPoly*)c->d_mf_poly;
    a.u32 = (const float4*)c->d_mf_u32;
    a.kself_bytes = (int64_t)c->n_poly * c->nd * c->nd * (int64_t)sizeof(float);
    a.minv_bytes = (int64_t)c->n_poly * c->Np * c->Np * (int64_t)sizeof(double);
    for (int i = 0; i < 3 * MF_FACE_NQ_MAX; ++i) a.quad[i] = c->mf_quad[i];
    a.theta = (float)c->theta;
    return a;
}

template <int PD, int MODE>
int launch_mf_t(lymph_ctx* c, const StepArgs& s) {
    const MfArgs a = mf_args(c, s);
    k_mf<PD, MODE><<<c->n_poly, MF_THREADS, 0, c->stream>>>(a);
    c->launches++;
    return LYMPH_OK;
}

template <int PD>
int launch_mf_p(lymph_ctx* c, int mode, const StepArgs& s) {
    const double* u = (mode == MODE_FIRST || mode == MODE_BILIN) ? s.u0 : s.un;
    const int64_t n = (int64_t)c->n_poly * c->Np;
    const int64_t nb = (n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096;
    k_mf_u32<<<(unsigned)nb, 256, 0, c->stream>>>(n, c->Np, u, (float4*)c->d_mf_u32);
    c->launches++;
    switch (mode) {
        case MODE_STEP: return launch_mf_t<PD, MODE_STEP>(c, s);
        case MODE_FIRST: return launch_mf_t<PD, MODE_FIRST>(c, s);
        case MODE_APPLY: return launch_mf_t<PD, MODE_APPLY>(c, s);
        case MODE_BILIN: return launch_mf_t<PD, MODE_BILIN>(c, s);
        case MODE_KU: return launch_mf_t<PD, MODE_KU>(c, s);
        default: lymph_set_error("matrix-free neighbour terms: unsupported mode"); return LYMPH_ERR_INVALID;
    }
}

}  // namespace

// The per-triangle and per-polyhedron FP32 tables of the matrix-free
// neighbour terms (after geometry and the block pattern exist).
int lymph_mf_setup(lymph_ctx* c, const RefTables& R) {
    (void)R;
    if (c->p < 1 || c->p > 4) { lymph_set_error("matrix-free neighbour terms: degree not supported"); return LYMPH_ERR_INVALID; }
    const int nq = MF_FACE_NQ[c->p];
    const double* rule = kFaceRule + 3 * face_rule_offset(c->p);
    for (int q = 0; q < MF_FACE_NQ_MAX; ++q)
        for (int k = 0; k < 3; ++k) c->mf_quad[3 * q + k] = q < nq ? (float)rule[3 * q + k] : 0.0f;
    if (!c->d_mf_tri) {
        void* p = nullptr;
        LYMPH_CUDA_TRY(cudaMalloc(&p, sizeof(MfTri) * (size_t)(c->n_block_faces > 0 ? c->n_block_faces : 1)));
        c->d_mf_tri = p;
        c->device_bytes += (int64_t)(sizeof(MfTri) * c->n_block_faces);
        LYMPH_CUDA_TRY(cudaMalloc(&p, sizeof(MfPoly) * (size_t)c->n_poly));
        c->d_mf_poly = p;
        c->device_bytes += (int64_t)(sizeof(MfPoly) * c->n_poly);
        LYMPH_CUDA_TRY(cudaMalloc(&p, sizeof(float4) * (size_t)c->n_poly * c->Np));
        c->d_mf_u32 = p;
        c->device_bytes += (int64_t)(sizeof(float4) * c->n_poly * c->Np);
        LYMPH_CUDA_TRY(cudaMalloc(&p, sizeof(int32_t) * MF_REC * (size_t)c->n_poly));
        c->d_mf_range = p;
        c->device_bytes += (int64_t)(sizeof(int32_t) * MF_REC * c->n_poly);
    }
    if (c->n_blocks > 0) {
        k_mf_tris<<<(unsigned)((c->n_blocks + 127) / 128), 128, 0, c->stream>>>(
            c->n_blocks, c->d_blk_row, c->d_col, c->d_bf_ptr, c->d_bf, c->d_neigh, c->d_tet_poly, c->d_tet_mat,
            c->d_mat, c->d_fk, c->d_normal, c->d_area, c->d_hk, c->d_bbox, c->d_ref, c->alpha, c->p,
            (MfTri*)c->d_mf_tri, c->d_status);
        c->launches++;
    }
    k_mf_polys<<<(c->n_poly + 127) / 128, 128, 0, c->stream>>>(c->n_poly, c->d_bbox, (MfPoly*)c->d_mf_poly);
    c->launches++;
    k_mf_qrec<<<(c->n_poly + 127) / 128, 128, 0, c->stream>>>(c->n_poly, c->d_row_ptr, c->d_bf_ptr,
                                                             (const MfTri*)c->d_mf_tri, (int32_t*)c->d_mf_range);
    c->launches++;
    LYMPH_CUDA_TRY(cudaGetLastError());
    return LYMPH_OK;
}

// The operator pass of one step mode with matrix-free neighbour terms.
int lymph_dev_mf(lymph_ctx* c, int mode, const stepk::StepArgs& s) {
    switch (c->p) {
        case 1: return launch_mf_p<1>(c, mode, s);
        case 2: return launch_mf_p<2>(c, mode, s);
        case 3: return launch_mf_p<3>(c, mode, s);
        case 4: return launch_mf_p<4>(c, mode, s);
        default: lymph_set_error("degree not supported on the device"); return LYMPH_ERR_INVALID;
    }
}

// ---- batch interface (batch.cu) ----

size_t lymph_mf_batch_problem_bytes() { return sizeof(MfBatchProblem); }

// CTAs of k_mf_batch<p> one SM holds (registers and shared memory).
int lymph_mf_batch_ctas_per_sm(int p) {
    int n = 0;
    cudaError_t e = cudaErrorInvalidValue;
    switch (p) {
        case 1: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_mf_batch<1>, MF_THREADS, 0); break;
        case 2: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_mf_batch<2>, MF_THREADS, 0); break;
        case 3: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_mf_batch<3>, MF_THREADS, 0); break;
        case 4: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_mf_batch<4>, MF_THREADS, 0); break;
        default: return 1;
    }
    return (e == cudaSuccess && n >= 1) ? n : 1;
}

// One problem's record for k_mf_batch; status: the batch's status word.
void lymph_mf_batch_problem(const lymph_ctx* c, int* status, void* out) {
    StepArgs s;
    s.row_ptr = c->d_row_ptr;
    s.col = c->d_col;
    s.K = c->d_K;
    s.Minv = c->d_Minv;
    s.rhs_stat = c->d_rhs_stat;
    s.rhs_dyn = c->d_rhs_dyn;
    s.gvals = nullptr;
    s.step_idx = nullptr;
    s.u0 = s.un = nullptr;
    s.out = nullptr;
    s.partial = nullptr;
    s.abs_idx = c->n_abs > 0 ? c->d_abs_idx : nullptr;
    s.Dabs = c->d_Dabs;
    s.Winv = c->d_Winv;
    s.dt = c->dt;
    s.status = status;
    s.n_poly = c->n_poly;
    MfBatchProblem pb;
    pb.a = mf_args(c, s);
    pb.buf[0] = c->d_buf[0];
    pb.buf[1] = c->d_buf[1];
    pb.cur0 = c->cur;
    pb.p = c->p;
    std::memcpy(out, &pb, sizeof(pb));
}

// One batched leapfrog step: the FP32 copies of every problem's u^n, then one
// persistent pass per degree over that degree's items, items[off[p - 1],
// off[p]) with grid[p - 1] CTAs and queue counter queue[p - 1] (the caller
// advances the step counter and clears the counters).  Returns the number of
// kernels launched in *launched.
int lymph_mf_batch_step(cudaStream_t st, const int* grid, const void* probs, const int2* items, const int* off,
                        int* queue, const int64_t* step_idx, const double* gvals, int64_t g_stride, int* launched) {
    const MfBatchProblem* pb = (const MfBatchProblem*)probs;
    const int n_all = off[4];
    int nl = 0;
    if (n_all > 0) {
        k_mf_u32_batch<<<(unsigned)((n_all + 3) / 4), 128, 0, st>>>(pb, items, n_all, step_idx);
        ++nl;
    }
    for (int p = 1; p <= 4; ++p) {
        const int n = off[p] - off[p - 1];
        if (n <= 0 || grid[p - 1] <= 0) continue;
        const int2* it = items + off[p - 1];
        int* q = queue + (p - 1);
        switch (p) {
            case 1: k_mf_batch<1><<<grid[0], MF_THREADS, 0, st>>>(pb, it, n, q, step_idx, gvals, g_stride); break;
            case 2: k_mf_batch<2><<<grid[1], MF_THREADS, 0, st>>>(pb, it, n, q, step_idx, gvals, g_stride); break;
            case 3: k_mf_batch<3><<<grid[2], MF_THREADS, 0, st>>>(pb, it, n, q, step_idx, gvals, g_stride); break;
            default: k_mf_batch<4><<<grid[3], MF_THREADS, 0, st>>>(pb, it, n, q, step_idx, gvals, g_stride); break;
        }
        ++nl;
    }
    if (launched) *launched = nl;
    LYMPH_CUDA_TRY(cudaGetLastError());
    return LYMPH_OK;
}

extern "C" int lymph_mf_face_rule(int32_t p, int32_t* n, double* xyw) {
    if (p < 1 || p > 4 || !n) return LYMPH_ERR_INVALID;
    *n = MF_FACE_NQ[p];
    if (xyw)
        for (int i = 0; i < 3 * MF_FACE_NQ[p]; ++i) xyw[i] = kFaceRule[3 * face_rule_offset(p) + i];
    return LYMPH_OK;
}
