// selftc.cu -- the FP32 operator blocks of the mixed precisions assembled on
// the 5th-generation tensor cores (tcgen05, kind::tf32): the self blocks of
// LYMPH_MIXED_MF and LYMPH_MIXED (k_self_tc) and LYMPH_MIXED's neighbour
// blocks (k_nb_tc).
//
// The self block K_PP of MAKE_MATRICES_FREE (src/matrix_free.f90:27-464) is
// the volume stiffness of P's sub-tetrahedra (MAKE_STIFFNESS_VOLUME,
// src/assemble_element.f90:24-77) plus the self part of the face terms on
// P's Dirichlet faces and on the faces it shares with other polyhedra
// (MAKE_STIFFNESS_FACE, :404-661).  Every one of its terms is a sum over
// quadrature points of a product of two basis tabulations, so with rows
// r = (i, a) and columns c = (j, b) (component, basis function) the block is
// two matrix products over a common K dimension of quadrature slots plus a
// re-indexing:
//     K_PP[(i,a),(j,b)] = O_D[(i,a),(j,b)] + O_S[(j,a),(i,b)]
//                         + delta_ij sum_k O_S[(k,a),(k,b)],
//     O_D = A B_D^T,  O_S = A B_S^T,
// where, per slot, the A row (i, a) and the B rows (j, b) are
//   volume point (w = weight |J|):   A = d_i phi_a,
//       B_D = w lambda d_j phi_b,  B_S = w mu d_j phi_b
//   face point, "d" slot (W = weight * area, cI = 1 on Dirichlet faces,
//   1/2 on shared ones, n P's outward normal):  A = d_i phi_a,
//       B_D = theta cI W lambda n_j phi_b,  B_S = theta cI W mu n_j phi_b
//   face point, "n phi" slot:  A = n_i phi_a,
//       B_D = -cI W lambda d_j phi_b,  B_S = sigma W / 2 n_j phi_b - cI W mu d_j phi_b.
// O_D gives lambda G_ij of the volume term and the lambda parts of the
// consistency and symmetry integrals; the block transpose of O_S gives
// mu G_ji, their mu parts and the penalty's n_i n_j part; the trace of O_S
// gives the delta_ij mu tr G term, the delta_ij mu n.H terms and the
// penalty's identity part (sum_k n_k^2 = 1).  Each face point enters twice
// (a "d" slot and an "n phi" slot); face integrals use the symmetric
// triangle rule exact to degree 2p of the matrix-free kernel (mf.cu), whose
// integrals equal the reference's collapsed rule's in exact arithmetic,
// volume integrals the reference's collapsed Gauss rule.
//
// A neighbour block K_PQ (P's test functions, Q's trial functions) has face
// terms only, -theta/2 I - S - IT/2 over the triangles P shares with Q,
// with P's normal and P's material; A comes from P's basis, B from Q's, and
// the same combination applies with five slots per face point:
//   "d":     A = d_i phi^P_a,  B_D = -theta/2 W lambda n_j phi^Q_b,  B_S = -theta/2 W mu n_j phi^Q_b
//   "n phi": A = n_i phi^P_a,  B_D = -mu W/2 d_j phi^Q_b,
//            B_S = -sigma W/2 n_j phi^Q_b - lambda W/2 d_j phi^Q_b
//   "phi_k", k = 0, 1, 2:  A = delta_ik phi^P_a,  B_D = delta_jk (lambda - mu)/2 W d_n phi^Q_b,  B_S = 0.
// The symmetry term's IT_E2 index order (assemble_element.f90:610-616) puts
// its lambda part into the block transpose of O_S, whose trace then carries
// lambda where that term's delta_ij part has mu; the "phi_k" slots add the
// difference on the diagonal component blocks.
//
// One CTA of 512 threads per polyhedron.  The K slots come in chunks of 32
// (the tetrahedra's volume points, then the faces).  P's tetrahedra (map,
// |J|, material) and faces (quadrature map, normal, area, weight factors)
// are staged in shared memory at CTA start; while warp 0 maps each slot of
// the next chunk to its physical point, weights and Legendre values, warps
// 1-15 write the current chunk's operands into shared memory, each value
// split into its nearest TF32 value and the TF32-rounded remainder (together
// within 2^-23 of the value), in the 128-byte-swizzled K-major layout the MMA
// reads, and lane 0 of warp 1 issues the four products A_hi B_hi + A_hi B_lo
// + A_lo B_hi + A_lo B_lo (FP32-accurate, not TF32 rounded) into an FP32
// accumulator in tensor memory.  Two operand stages let the tabulation of
// one chunk overlap the MMAs of the last.  The tensor
// cores add each MMA's products to the accumulator with truncation (round
// toward zero: an emulation with that rounding reproduces the measured
// errors, one with round-to-nearest gives 10x less), so the error grows
// with the number of MMAs an accumulator takes.  Each chunk's 16 MMAs
// therefore go into a fresh accumulator, drained into FP32 registers (round
// to nearest) two chunks later while the next chunk accumulates into the
// other of two accumulators: 3.5e-7 per row at p = 4 in that emulation,
// against 1.2-1.6e-6 with one drain every 4 chunks.  The epilogue
// stages O_D and O_S in shared memory, applies the re-indexing and writes
// the block column-major, coalesced.  Every mbarrier wait is bounded; on
// expiry the kernel sets ST_TIMEOUT, waits (bounded) for its MMAs in flight,
// frees its tensor memory and returns.

#include <cstddef>

#include "common.cuh"
#include "tc_prims.cuh"

extern "C" int lymph_mf_face_rule(int32_t p, int32_t* n, double* xyw);

namespace {

using namespace umma;

constexpr int ST_THREADS = 512;   // 16 warps: 4 per tensor-memory lane quadrant
constexpr int ST_BK = 32;         // K slots per chunk (4 MMAs of K = 8)
constexpr int ST_TMAX = 32;       // tetrahedra of a polyhedron kept in shared memory (the rest read from the arrays)
constexpr int ST_FMAX = 64;       // faces of a polyhedron kept in shared memory
constexpr int ST_FW = 18;         // floats per face entry of a self block (face_entry)
constexpr int ST_FWN = 28;        // floats per face entry of a neighbour block (face_entry_nb)
constexpr int ST_FACE_NQ[5] = {0, 3, 6, 12, 16};   // nodes of the symmetric triangle rule (mf.cu)

template <int PD, bool NB = false> struct TcShape {
    static constexpr int NP = (PD + 1) * (PD + 2) * (PD + 3) / 6;
    static constexpr int ND = 3 * NP;
    static constexpr int NQ3 = (PD + 1) * (PD + 1) * (PD + 1);
    static constexpr int NF = ST_FACE_NQ[PD];
    static constexpr int FPC = (ST_BK / (2 * NF)) > 0 ? ST_BK / (2 * NF) : 1;   // faces per chunk
    static constexpr int CPT = (NQ3 + ST_BK - 1) / ST_BK;                       // chunks per tetrahedron
    static constexpr int NH = (ND + 15) / 16 * 16;   // columns of O_D (and of O_S)
    static constexpr int NT = 2 * NH;                // the MMA's N: O_D | O_S
    static constexpr int NCOL = NT / 4;              // accumulator columns drained per thread
    static constexpr int TCOLS = 2 * NT <= 64 ? 64 : (2 * NT <= 128 ? 128 : (2 * NT <= 256 ? 256 : 512));
    // (L, L') pairs per slot (P's box; for a neighbour block also Q's), odd: no bank conflicts
    static constexpr int LS = ((NB ? 6 : 3) * (PD + 1)) | 1;
    static constexpr int FW = NB ? ST_FWN : ST_FW;
    static constexpr int SPF = 5 * NF;               // slots per face of a neighbour block
    static constexpr size_t A_TILE = 128 * 128;      // 128 rows x 32 TF32 slots
    static constexpr size_t B_TILE = (size_t)NT * 128;
    static constexpr size_t STAGE = 2 * A_TILE + 2 * B_TILE;
    static constexpr size_t LEG_OFF = 2 * STAGE;                             // two slot buffers
    static constexpr size_t COEF_OFF = LEG_OFF + 2 * (size_t)ST_BK * LS * 8;
    static constexpr size_t TET_OFF = COEF_OFF + 2 * (size_t)ST_BK * 3 * 16;
    static constexpr size_t FACE_OFF = TET_OFF + (size_t)ST_TMAX * 16 * 4;
    static constexpr size_t REF_OFF = FACE_OFF + (size_t)ST_FMAX * FW * 4;   // the volume rule in FP32
    static constexpr size_t BAR_OFF = REF_OFF + (size_t)NQ3 * 4 * 4;
    static constexpr size_t SMEM = BAR_OFF + 64 + 1024;   // + room to align the base to 1 KB
    static_assert(NT <= 256 && NT % 16 == 0, "MMA N");
    static_assert(2 * NT <= TCOLS, "two accumulators");
    static_assert(NCOL % 8 == 0, "drain in x16/x8 loads");
    static_assert(2 * (size_t)ND * ND * 4 <= 2 * STAGE, "epilogue staging fits the operand stages");
    static_assert(COEF_OFF % 16 == 0 && TET_OFF % 16 == 0 && FACE_OFF % 8 == 0 && REF_OFF % 16 == 0 && BAR_OFF % 8 == 0,
                  "alignment");
    static_assert(SMEM <= 232448, "shared memory per CTA");
};

// the reference's basis order as degree triples, per degree
__constant__ Blist<1> c_bl1 = Blist<1>{};
__constant__ Blist<2> c_bl2 = Blist<2>{};
__constant__ Blist<3> c_bl3 = Blist<3>{};
__constant__ Blist<4> c_bl4 = Blist<4>{};
template <int PD> __device__ __forceinline__ int3 blist_row(int a);
template <> __device__ __forceinline__ int3 blist_row<1>(int a) { return make_int3(c_bl1.d[a][0], c_bl1.d[a][1], c_bl1.d[a][2]); }
template <> __device__ __forceinline__ int3 blist_row<2>(int a) { return make_int3(c_bl2.d[a][0], c_bl2.d[a][1], c_bl2.d[a][2]); }
template <> __device__ __forceinline__ int3 blist_row<3>(int a) { return make_int3(c_bl3.d[a][0], c_bl3.d[a][1], c_bl3.d[a][2]); }
template <> __device__ __forceinline__ int3 blist_row<4>(int a) { return make_int3(c_bl4.d[a][0], c_bl4.d[a][1], c_bl4.d[a][2]); }

struct SelfTcArgs {
    const int32_t* poly_ptr;
    const int32_t* poly_tets;
    const int32_t* tet_poly;
    const int32_t* tet_mat;
    const int32_t* neigh;
    const double* mat;
    const double* fk;
    const double* jdet;
    const double* nrm;
    const double* area;
    const double* bbox;
    const double* hk;
    const RefTables* ref;
    const int32_t* row_ptr;
    const int32_t* blk_row;
    const int32_t* col;
    const int64_t* bf_ptr;
    const int32_t* bf;
    const int64_t* list;   // neighbour blocks: the blocks of this launch (one CTA each)
    double alpha, theta;
    float* out;            // column-major ND x ND blocks: P's self block at slot P or row_ptr[P]; a neighbour block at its own slot
    int slot_row_ptr;      // 1: the block-CSR operator of LYMPH_MIXED (self block first in each row)
    int* status;
    float frule[3 * 16];   // (xi, eta, w) of the symmetric triangle rule
};

// v rounded to the nearest TF32 value (10 explicit mantissa bits; ties away
// from zero), exact in TF32
__device__ __forceinline__ float tf32_rn(float v) { return __uint_as_float((__float_as_uint(v) + 0x1000u) & 0xFFFFE000u); }

// P's box: centre and inverse half-widths, in FP64.
struct Box {
    double c[3], ih[3];
};
__device__ __forceinline__ Box box_of(const double* bb) {
    Box b;
    for (int d = 0; d < 3; ++d) {
        b.c[d] = (bb[2 * d] + bb[2 * d + 1]) / 2.0;
        b.ih[d] = 2.0 / (bb[2 * d + 1] - bb[2 * d]);
    }
    return b;
}

// Tetrahedron tt in P's box coordinates (FP64 arithmetic, FP32 result):
// xhat = M (xi, eta, zeta) + v for the reference point (xi, eta, zeta) of
// jacobians' affine map (Poly_ref_mappings.f90:18-75), M = diag(ih) Fk[:, 0:3],
// v = diag(ih) (Fk[:, 3] - c); then |J|, lambda, mu.  out[16].
__device__ __noinline__ void tet_entry(const SelfTcArgs& A, const Box& bx, int tt, float* out) {
    const double* F = A.fk + (int64_t)tt * 12;
    for (int d = 0; d < 3; ++d) {
        for (int l = 0; l < 3; ++l) out[d * 3 + l] = (float)(F[d * 4 + l] * bx.ih[d]);
        out[9 + d] = (float)((F[d * 4 + 3] - bx.c[d]) * bx.ih[d]);
    }
    const int mid = A.tet_mat[tt];
    out[12] = (float)fabs(A.jdet[tt]);
    out[13] = (float)A.mat[mid * 3 + 1];
    out[14] = (float)A.mat[mid * 3 + 2];
    out[15] = 0.f;
}

// Entry e of P's self-block face list in P's box coordinates (FP64
// arithmetic, FP32 result): the quadrature map xhat = o + xi e1 + eta e2 of
// basis_boundary (basis_function.f90:560-577: x = Fk node_maps(:,:,f)
// (xi, eta, 1, 1)), P's outward normal, the area and the factors of the slot
// weights W = w_q area: theta cI lambda, theta cI mu, -cI lambda, -cI mu,
// sigma / 2 (cI = 1 on a Dirichlet face, 1/2 on a shared one; lambda, mu of
// P's tetrahedron).  out[ST_FW].
template <int PD>
__device__ __noinline__ void face_entry(const SelfTcArgs& A, int P, const Box& bx, int64_t e, float* out) {
    const int code = A.bf[e];
    const int tt = code >> 2, f = code & 3;
    const int E2 = A.neigh[code];
    const bool dir = (E2 == LYMPH_BC_DIRI);
    const double hmin = dir ? A.hk[P] : fmin(A.hk[P], A.hk[A.tet_poly[E2]]);
    const int mid = A.tet_mat[tt];
    const double lam = A.mat[mid * 3 + 1], mu = A.mat[mid * 3 + 2];
    const double sigma = A.alpha * (double)(PD * PD) / hmin * (lam + 2.0 * mu);
    const double cI = dir ? 1.0 : 0.5;
    const double* F = A.fk + (int64_t)tt * 12;
    const double* nm = A.ref->node_maps + f * 16;
    for (int d = 0; d < 3; ++d) {
        double cm[4];
        for (int l = 0; l < 4; ++l) {
            double s = 0.0;
            for (int m = 0; m < 4; ++m) s += F[d * 4 + m] * nm[m * 4 + l];
            cm[l] = s;
        }
        out[d] = (float)((cm[2] + cm[3] - bx.c[d]) * bx.ih[d]);
        out[3 + d] = (float)(cm[0] * bx.ih[d]);
        out[6 + d] = (float)(cm[1] * bx.ih[d]);
        out[9 + d] = (float)A.nrm[(int64_t)tt * 12 + f * 3 + d];
    }
    out[12] = (float)A.area[(int64_t)tt * 4 + f];
    out[13] = (float)(A.theta * cI * lam);
    out[14] = (float)(A.theta * cI * mu);
    out[15] = (float)(-cI * lam);
    out[16] = (float)(-cI * mu);
    out[17] = (float)(0.5 * sigma);
}

// Entry e of the face list of neighbour block (P, Q) (MAKE_STIFFNESS_FACE's
// E2 terms, assemble_element.f90:404-661, as MAKE_MATRICES_FREE inserts them,
// matrix_free.f90:412-433): the quadrature map in P's and in Q's box
// coordinates, P's outward normal, the area and the factors of the slot
// weights W = w_q area: -theta/2 lambda, -theta/2 mu, -mu/2, -lambda/2,
// -sigma/2 and (lambda - mu)/2 (lambda, mu of P's tetrahedron, the
// reference's choice for both sides).  out[ST_FWN].
template <int PD>
__device__ __noinline__ void face_entry_nb(const SelfTcArgs& A, int P, int Q, const Box& bp, const Box& bq, int64_t e,
                                           float* out) {
    const int code = A.bf[e];
    const int tt = code >> 2, f = code & 3;
    const int mid = A.tet_mat[tt];
    const double lam = A.mat[mid * 3 + 1], mu = A.mat[mid * 3 + 2];
    const double sigma = A.alpha * (double)(PD * PD) / fmin(A.hk[P], A.hk[Q]) * (lam + 2.0 * mu);
    const double* F = A.fk + (int64_t)tt * 12;
    const double* nm = A.ref->node_maps + f * 16;
    for (int d = 0; d < 3; ++d) {
        double cm[4];
        for (int l = 0; l < 4; ++l) {
            double s = 0.0;
            for (int m = 0; m < 4; ++m) s += F[d * 4 + m] * nm[m * 4 + l];
            cm[l] = s;
        }
        out[d] = (float)((cm[2] + cm[3] - bp.c[d]) * bp.ih[d]);
        out[3 + d] = (float)(cm[0] * bp.ih[d]);
        out[6 + d] = (float)(cm[1] * bp.ih[d]);
        out[9 + d] = (float)((cm[2] + cm[3] - bq.c[d]) * bq.ih[d]);
        out[12 + d] = (float)(cm[0] * bq.ih[d]);
        out[15 + d] = (float)(cm[1] * bq.ih[d]);
        out[18 + d] = (float)A.nrm[(int64_t)tt * 12 + f * 3 + d];
    }
    out[21] = (float)A.area[(int64_t)tt * 4 + f];
    out[22] = (float)(-0.5 * A.theta * lam);
    out[23] = (float)(-0.5 * A.theta * mu);
    out[24] = (float)(-0.5 * mu);
    out[25] = (float)(-0.5 * lam);
    out[26] = (float)(-0.5 * sigma);
    out[27] = (float)(0.5 * (lam - mu));
}

// value v into row `row`, slot k of a 128-byte-swizzled K-major tile pair:
// hi = v rounded to TF32, lo = the remainder v - hi (exact in FP32, at most
// 2^-11 |v|) rounded to TF32, so v = hi + lo to within 2^-23 |v| and the
// MMA, which reads only the TF32 bits, sees both exactly
__device__ __forceinline__ void put_split(char* hi, char* lo, int row, int k, float v) {
    const int off = row * 128 + ((((k >> 2) ^ (row & 7)) << 4) | ((k & 3) << 2));
    const float h = tf32_rn(v);
    *(float*)(hi + off) = h;
    *(float*)(lo + off) = tf32_rn(v - h);
}

// Adds this thread's NCOL accumulator columns (tensor-memory address taddr:
// its warp's lane quadrant, its column group) to run, 16 columns per load
// (fewer registers in flight than 32-column loads beside run).
template <int NCOL> __device__ __forceinline__ void drain(uint32_t taddr, float (&run)[NCOL]) {
    constexpr int N16 = NCOL / 16, N8 = (NCOL % 16) / 8;
#pragma unroll
    for (int q = 0; q < N16; ++q) {
        uint32_t r[16];
        tmem_ld16(taddr + 16 * q, r);
#pragma unroll
        for (int i = 0; i < 16; ++i) run[16 * q + i] += __uint_as_float(r[i]);
    }
    if (N8) {
        uint32_t r[8];
        tmem_ld8(taddr + 16 * N16, r);
#pragma unroll
        for (int i = 0; i < 8; ++i) run[16 * N16 + i] += __uint_as_float(r[i]);
    }
}

// One block of the operator per CTA: the self block of polyhedron
// blockIdx.x (NB = false) or neighbour block list[blockIdx.x] (NB = true).
template <int PD, bool NB>
__device__ __forceinline__ void block_tc(const SelfTcArgs& A) {
    using S = TcShape<PD, NB>;
    constexpr int NP = S::NP, ND = S::ND, L = PD + 1;
    extern __shared__ __align__(1024) char smem_raw[];
    // the swizzle pattern is a function of the address: align the stages to 1 KB
    char* smem = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
    float2* leg = (float2*)(smem + S::LEG_OFF);      // [2][32][LS]: (L, L') of x, y, z per slot
    float4* coef = (float4*)(smem + S::COEF_OFF);    // [2][32][3]: slot coefficients and normal
    float* s_tet = (float*)(smem + S::TET_OFF);      // [ST_TMAX][16]: P's tetrahedra (tet_entry)
    float* s_face = (float*)(smem + S::FACE_OFF);    // [ST_FMAX][ST_FW]: P's faces (face_entry)
    float4* s_ref = (float4*)(smem + S::REF_OFF);    // [NQ3]: the volume rule's (xi, eta, zeta, w)
    uint64_t* bars = (uint64_t*)(smem + S::BAR_OFF);
    uint32_t* tmem_slot = (uint32_t*)(bars + 2);
    __shared__ int s_ok;
    __shared__ float s_box[8];   // ih_x, ih_y, ih_z, sc of P's Legendre map, then Q's
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    const uint32_t sbase = smem_u32(smem);
    constexpr int ISSUER = 32;   // lane 0 of warp 1 waits on the barriers and issues the MMAs
    // after one CTA's wait ran out the launch has failed: the others return
    // at once instead of waiting out their own limits (one read, so the
    // whole CTA takes the same branch)
    if (t == 0) s_ok = (*(volatile int*)A.status & ST_TIMEOUT) ? 0 : 1;
    __syncthreads();
    if (!s_ok) return;

    int P, Q, t0, ntet;
    int64_t kblk;   // the block's slot in the block-CSR pattern
    if constexpr (NB) {
        kblk = A.list[blockIdx.x];
        P = A.blk_row[kblk];
        Q = A.col[kblk];
        t0 = 0;
        ntet = 0;   // face terms only
    } else {
        P = Q = blockIdx.x;
        kblk = A.row_ptr[P];   // the self block leads its row
        t0 = A.poly_ptr[P];
        ntet = A.poly_ptr[P + 1] - t0;
    }
    const int64_t f0 = A.bf_ptr[kblk];
    const int nface = (int)(A.bf_ptr[kblk + 1] - f0);
    const int nvc = ntet * S::CPT;
    const int nch = NB ? (nface * S::SPF + ST_BK - 1) / ST_BK : nvc + (nface + S::FPC - 1) / S::FPC;
    const double* bb = A.bbox + (int64_t)P * 6;
    const Box bx = box_of(bb);
    const Box bxq = NB ? box_of(A.bbox + (int64_t)Q * 6) : bx;

    // zero both operand stages: padding rows are never written again
    for (int i = t; i < (int)(2 * S::STAGE / 16); i += ST_THREADS) ((float4*)smem)[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    // P's tetrahedra and faces in its box coordinates, and the volume rule,
    // in shared memory and FP32, so the per-chunk slot set-up reads no global
    // memory and does no FP64 arithmetic (beyond ST_TMAX / ST_FMAX it forms
    // the entries from the arrays)
    if (t >= 64 && t - 64 < nface && t - 64 < ST_FMAX) {
        if constexpr (NB) face_entry_nb<PD>(A, P, Q, bx, bxq, f0 + (t - 64), s_face + (t - 64) * S::FW);
        else face_entry<PD>(A, P, bx, f0 + (t - 64), s_face + (t - 64) * S::FW);
    }
    if constexpr (!NB) {
        if (t < ntet && t < ST_TMAX) tet_entry(A, bx, A.poly_tets[t0 + t], s_tet + t * 16);
        for (int q = t; q < S::NQ3; q += ST_THREADS)
            s_ref[q] = make_float4((float)A.ref->nodtet3[q * 4], (float)A.ref->nodtet3[q * 4 + 1],
                                   (float)A.ref->nodtet3[q * 4 + 2], (float)A.ref->weitet3[q]);
    }
    if (t == 0) {
        for (int side = 0; side < (NB ? 2 : 1); ++side) {
            const double* bs = A.bbox + (int64_t)(side ? Q : P) * 6;
            double hprod = 1.0;
            for (int d = 0; d < 3; ++d) {
                const double h = (bs[2 * d + 1] - bs[2 * d]) / 2.0;
                s_box[4 * side + d] = (float)(1.0 / h);
                hprod *= h;
            }
            s_box[4 * side + 3] = (float)(1.0 / sqrt(hprod));
        }
        mbar_init(smem_u32(&bars[0]), 1);
        mbar_init(smem_u32(&bars[1]), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"((uint32_t)S::TCOLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");   // the zeroed stages, for the MMAs
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;
    const float sc = s_box[3], sx = sc * s_box[0], sy = sc * s_box[1], sz = sc * s_box[2];
    const float scq = s_box[7], sxq = scq * s_box[4], syq = scq * s_box[5], szq = scq * s_box[6];
    const int grp = warp >> 2;                                   // column group of the drain
    const uint32_t tq = tmem + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)(grp * S::NCOL);
    const uint32_t idesc = idesc_tf32(128, S::NT);

    // warp 0: slot `lane` of chunk c -> point (box coordinates), weights,
    // Legendre values, into buffer b; FP32 from the tables
    auto slot_setup = [&](int c, int b) {
        const int k = lane;
        float xh[3] = {0.f, 0.f, 0.f}, xq[3] = {0.f, 0.f, 0.f};
        float bd = 0.f, bn = 0.f, dd = 0.f, dn = 0.f, sd = 0.f, sn = 0.f, nv[3] = {0.f, 0.f, 0.f};
        float bphi = 0.f, dc = 0.f, kc = 0.f;
        if constexpr (NB) {
            // slot s of the block: face s / (5 NF); per point a "d", an "n phi"
            // and three "phi_k" slots (the delta_ij part of the symmetry term)
            const int sidx = c * ST_BK + k, fi = sidx / S::SPF, r = sidx % S::SPF;
            if (fi < nface) {
                float e[ST_FWN];
                if (fi < ST_FMAX) {
#pragma unroll
                    for (int i = 0; i < ST_FWN; ++i) e[i] = s_face[fi * ST_FWN + i];
                } else {
                    float ev[ST_FWN];
                    face_entry_nb<PD>(A, P, Q, bx, bxq, f0 + fi, ev);
#pragma unroll
                    for (int i = 0; i < ST_FWN; ++i) e[i] = ev[i];
                }
                const int kind = r / S::NF, q = r % S::NF;
                const float xi = A.frule[3 * q], eta = A.frule[3 * q + 1], W = A.frule[3 * q + 2] * e[21];
                for (int d = 0; d < 3; ++d) {
                    xh[d] = fmaf(eta, e[6 + d], fmaf(xi, e[3 + d], e[d]));
                    xq[d] = fmaf(eta, e[15 + d], fmaf(xi, e[12 + d], e[9 + d]));
                    nv[d] = e[18 + d];
                }
                if (kind == 0) {          // "d"
                    bd = 1.f;
                    dn = e[22] * W;
                    sn = e[23] * W;
                } else if (kind == 1) {   // "n phi"
                    bn = 1.f;
                    dd = e[24] * W;
                    sd = e[25] * W;
                    sn = e[26] * W;
                } else {                  // "phi_k", k = kind - 2
                    bphi = 1.f;
                    dc = e[27] * W;
                    kc = (float)(kind - 2);
                }
            }
        } else if (c < nvc) {
            const int q = (c % S::CPT) * ST_BK + k, j = c / S::CPT;
            if (q < S::NQ3) {
                float e[16];
                if (j < ST_TMAX) {
#pragma unroll
                    for (int i = 0; i < 16; ++i) e[i] = s_tet[j * 16 + i];
                } else {   // beyond the table (out of line: few registers on the common path)
                    float ev[16];
                    tet_entry(A, bx, A.poly_tets[t0 + j], ev);
#pragma unroll
                    for (int i = 0; i < 16; ++i) e[i] = ev[i];
                }
                const float4 r = s_ref[q];
                for (int d = 0; d < 3; ++d)
                    xh[d] = fmaf(e[d * 3 + 0], r.x, fmaf(e[d * 3 + 1], r.y, fmaf(e[d * 3 + 2], r.z, e[9 + d])));
                const float w = r.w * e[12];
                bd = 1.f;
                dd = w * e[13];
                sd = w * e[14];
            }
        } else {
            const int fi = (c - nvc) * S::FPC + k / (2 * S::NF), r = k % (2 * S::NF);
            if (k < S::FPC * 2 * S::NF && fi < nface) {
                float e[ST_FW];
                if (fi < ST_FMAX) {
#pragma unroll
                    for (int i = 0; i < ST_FW; ++i) e[i] = s_face[fi * ST_FW + i];
                } else {
                    float ev[ST_FW];
                    face_entry<PD>(A, P, bx, f0 + fi, ev);
#pragma unroll
                    for (int i = 0; i < ST_FW; ++i) e[i] = ev[i];
                }
                const int q = r % S::NF;
                const float xi = A.frule[3 * q], eta = A.frule[3 * q + 1], W = A.frule[3 * q + 2] * e[12];
                for (int d = 0; d < 3; ++d) {
                    xh[d] = fmaf(eta, e[6 + d], fmaf(xi, e[3 + d], e[d]));
                    nv[d] = e[9 + d];
                }
                if (r < S::NF) {   // "d" slot
                    bd = 1.f;
                    dn = e[13] * W;
                    sn = e[14] * W;
                } else {           // "n phi" slot
                    bn = 1.f;
                    dd = e[15] * W;
                    sd = e[16] * W;
                    sn = e[17] * W;
                }
            }
        }
        float2* lg = leg + (b * ST_BK + k) * S::LS;
#pragma unroll
        for (int d = 0; d < 3; ++d) legendre_f32<PD>(xh[d], lg + d * L);
        if constexpr (NB) {
#pragma unroll
            for (int d = 0; d < 3; ++d) legendre_f32<PD>(xq[d], lg + (3 + d) * L);
        }
        float4* cf = coef + (b * ST_BK + k) * 3;
        cf[0] = make_float4(bd, bn, dd, dn);
        cf[1] = make_float4(sd, sn, nv[0], nv[1]);
        cf[2] = make_float4(nv[2], bphi, dc, kc);
    };

    float run[S::NCOL];
#pragma unroll
    for (int j = 0; j < S::NCOL; ++j) run[j] = 0.0f;
    bool ok = true;
    int issued = 0;
    if (warp == 0 && nch > 0) slot_setup(0, 0);
    for (int c = 0; c < nch; ++c) {
        const int st = c & 1;
        // the MMAs of chunk c - 2 read this stage and wrote the accumulator
        // chunk c takes: the issuing thread waits for them
        if (c >= 2 && t == ISSUER) s_ok = mbar_wait(smem_u32(&bars[st]), (uint32_t)(((c - 2) >> 1) & 1)) ? 1 : 0;
        __syncthreads();
        if (c >= 2 && !s_ok) {
            ok = false;
            break;
        }
        if (c >= 2) {   // chunk c - 2's products, complete, into the running sums
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            drain<S::NCOL>(tq + (uint32_t)(st * S::NT), run);
        }
        if (warp == 0) {
            // the next chunk's slots while warps 1-15 write this chunk's operands
            if (c + 1 < nch) slot_setup(c + 1, (c + 1) & 1);
        } else {
            // ---- the operands of chunk c: basis function a = warp - 1 + 15 i, slot = lane ----
            char* ahi = smem + st * S::STAGE;
            char* alo = ahi + S::A_TILE;
            char* bhi = alo + S::A_TILE;
            char* blo = bhi + S::B_TILE;
            const int k = lane;
            const float4* cf = coef + (st * ST_BK + k) * 3;
            const float4 c0 = cf[0], c1 = cf[1], c2 = cf[2];
            const float n3[3] = {c1.z, c1.w, c2.x};
            const float2* lg = leg + (st * ST_BK + k) * S::LS;
            for (int a = warp - 1; a < NP; a += ST_THREADS / 32 - 1) {
                const int3 tr = blist_row<PD>(a);
                const float2 X = lg[tr.x], Y = lg[L + tr.y], Z = lg[2 * L + tr.z];
                const float yz = Y.x * Z.x;
                const float phi = sc * X.x * yz;
                const float g[3] = {sx * X.y * yz, sy * X.x * Y.y * Z.x, sz * X.x * Y.x * Z.y};
                if constexpr (NB) {
                    // A from P's basis, B from Q's; the "phi_k" slots put
                    // phi^P_a and (lambda - mu)/2 W d_n phi^Q_b on component kc
                    const float2 Xq = lg[3 * L + tr.x], Yq = lg[4 * L + tr.y], Zq = lg[5 * L + tr.z];
                    const float yzq = Yq.x * Zq.x;
                    const float phq = scq * Xq.x * yzq;
                    const float gq[3] = {sxq * Xq.y * yzq, syq * Xq.x * Yq.y * Zq.x, szq * Xq.x * Yq.x * Zq.y};
                    const float dnq = fmaf(n3[0], gq[0], fmaf(n3[1], gq[1], n3[2] * gq[2]));
                    const int kc = (int)c2.w;
#pragma unroll
                    for (int i = 0; i < 3; ++i) {
                        const int row = i * NP + a;
                        const float av = fmaf(c0.x, g[i], c0.y * (n3[i] * phi)) + (i == kc ? c2.y * phi : 0.f);
                        const float bdv = fmaf(c0.z, gq[i], c0.w * (n3[i] * phq)) + (i == kc ? c2.z * dnq : 0.f);
                        put_split(ahi, alo, row, k, av);
                        put_split(bhi, blo, row, k, bdv);
                        put_split(bhi, blo, S::NH + row, k, fmaf(c1.x, gq[i], c1.y * (n3[i] * phq)));
                    }
                } else {
#pragma unroll
                    for (int i = 0; i < 3; ++i) {
                        const float np_ = n3[i] * phi;
                        const int row = i * NP + a;
                        put_split(ahi, alo, row, k, fmaf(c0.x, g[i], c0.y * np_));
                        put_split(bhi, blo, row, k, fmaf(c0.z, g[i], c0.w * np_));
                        put_split(bhi, blo, S::NH + row, k, fmaf(c1.x, g[i], c1.y * np_));
                    }
                }
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");   // generic-proxy writes -> the MMAs
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
        if (t == ISSUER) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t ahi = sbase + (uint32_t)(st * S::STAGE), alo = ahi + (uint32_t)S::A_TILE;
            const uint32_t bhi = alo + (uint32_t)S::A_TILE, blo = bhi + (uint32_t)S::B_TILE;
            const uint32_t d = tmem + (uint32_t)(st * S::NT);
#pragma unroll
            for (int j = 0; j < ST_BK / 8; ++j) {   // k-step j: bytes 32 j .. 32 j + 31 of every row
                const uint64_t dah = sdesc_sw128(ahi + 32 * j), dal = sdesc_sw128(alo + 32 * j);
                const uint64_t dbh = sdesc_sw128(bhi + 32 * j), dbl = sdesc_sw128(blo + 32 * j);
                mma_tf32(d, dah, dbh, idesc, j == 0 ? 0u : 1u);
                mma_tf32(d, dah, dbl, idesc, 1u);
                mma_tf32(d, dal, dbh, idesc, 1u);
                mma_tf32(d, dal, dbl, idesc, 1u);
            }
            mma_commit(smem_u32(&bars[st]));
        }
        issued = c + 1;
    }
    // the last commit covers every MMA issued before it
    if (t == ISSUER) {
        bool done = true;
        if (issued > 0) done = mbar_wait(smem_u32(&bars[(issued - 1) & 1]), (uint32_t)(((issued - 1) >> 1) & 1));
        if (!done || !ok) atomicOr(A.status, ST_TIMEOUT);
        s_ok = (done && ok) ? 1 : 0;
    }
    __syncthreads();
    ok = s_ok != 0;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (ok) {
        // chunks 0 .. nch - 3 are drained; the last two are in the accumulators
        if (nch >= 2) drain<S::NCOL>(tq + (uint32_t)(((nch - 2) & 1) * S::NT), run);
        if (nch >= 1) drain<S::NCOL>(tq + (uint32_t)(((nch - 1) & 1) * S::NT), run);
        // ---- epilogue: O_D column-major and O_S row-major in the free stages ----
        float* Dm = (float*)smem;
        float* Sm = Dm + ND * ND;
        const int row = (warp & 3) * 32 + lane;
        if (row < ND) {
#pragma unroll
            for (int j = 0; j < S::NCOL; ++j) {
                const int col = grp * S::NCOL + j;
                if (col < ND) Dm[col * ND + row] = run[j];
                else if (col >= S::NH && col < S::NH + ND) Sm[row * ND + (col - S::NH)] = run[j];
            }
        }
        __syncthreads();
        float* out = A.out + ((NB || A.slot_row_ptr) ? kblk : (int64_t)P) * ND * ND;
        for (int e = t; e < ND * ND; e += ST_THREADS) {
            const int col = e / ND, r = e - col * ND;
            const int i = r / NP, a = r - i * NP, j = col / NP, b = col - j * NP;
            float v = Dm[e] + Sm[(j * NP + a) * ND + i * NP + b];
            if (i == j) v += (Sm[a * ND + b] + Sm[(NP + a) * ND + NP + b]) + Sm[(2 * NP + a) * ND + 2 * NP + b];
            out[e] = v;
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)S::TCOLS));
}

template <int PD>
__global__ void __launch_bounds__(ST_THREADS, 1) k_self_tc(const __grid_constant__ SelfTcArgs A) {
    block_tc<PD, false>(A);
}

template <int PD>
__global__ void __launch_bounds__(ST_THREADS, 1) k_nb_tc(const __grid_constant__ SelfTcArgs A) {
    block_tc<PD, true>(A);
}

// The kernel arguments of a context (out, the output flags and the list are
// the caller's); false if the degree has no triangle rule.
template <int PD> bool tc_args(lymph_ctx* c, SelfTcArgs& A) {
    A.poly_ptr = c->d_poly_ptr; A.poly_tets = c->d_poly_tets; A.tet_poly = c->d_tet_poly; A.tet_mat = c->d_tet_mat;
    A.neigh = c->d_neigh; A.mat = c->d_mat; A.fk = c->d_fk; A.jdet = c->d_jdet; A.nrm = c->d_normal; A.area = c->d_area;
    A.bbox = c->d_bbox; A.hk = c->d_hk; A.ref = c->d_ref; A.row_ptr = c->d_row_ptr; A.blk_row = c->d_blk_row;
    A.col = c->d_col; A.bf_ptr = c->d_bf_ptr; A.bf = c->d_bf; A.list = nullptr; A.alpha = c->alpha;
    A.theta = c->theta; A.out = nullptr; A.slot_row_ptr = 0; A.status = c->d_status;
    int32_t nq = 0;
    if (lymph_mf_face_rule(PD, &nq, nullptr) != LYMPH_OK || nq != ST_FACE_NQ[PD]) return false;
    double xyw[3 * 16];
    lymph_mf_face_rule(PD, &nq, xyw);
    for (int i = 0; i < 3 * nq; ++i) A.frule[i] = (float)xyw[i];
    return true;
}

template <int PD> int launch_nb_tc(lymph_ctx* c, float* out, const int64_t* list, int64_t n_list) {
    using S = TcShape<PD, true>;
    SelfTcArgs A;
    if (!tc_args<PD>(c, A)) {
        lymph_set_error("neighbour-block assembly: no triangle rule for this degree");
        return LYMPH_ERR_INVALID;
    }
    A.out = out;
    A.list = list;
    LYMPH_CUDA_TRY(cudaFuncSetAttribute(k_nb_tc<PD>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::SMEM));
    const int64_t chunk = 1 << 20;
    for (int64_t b0 = 0; b0 < n_list; b0 += chunk) {
        A.list = list + b0;
        const int64_t nb = n_list - b0 < chunk ? n_list - b0 : chunk;
        k_nb_tc<PD><<<(unsigned)nb, ST_THREADS, S::SMEM, c->stream>>>(A);
        c->launches++;
        LYMPH_CUDA_TRY(cudaGetLastError());
    }
    return LYMPH_OK;
}

template <int PD> int launch_self_tc(lymph_ctx* c, float* out, bool block_csr) {
    using S = TcShape<PD>;
    SelfTcArgs A;
    if (!tc_args<PD>(c, A)) {
        lymph_set_error("self-block assembly: no triangle rule for this degree");
        return LYMPH_ERR_INVALID;
    }
    A.out = out;
    A.slot_row_ptr = block_csr ? 1 : 0;
    LYMPH_CUDA_TRY(cudaFuncSetAttribute(k_self_tc<PD>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::SMEM));
    if (c->n_poly > 0) {
        k_self_tc<PD><<<c->n_poly, ST_THREADS, S::SMEM, c->stream>>>(A);
        c->launches++;
        LYMPH_CUDA_TRY(cudaGetLastError());
    }
    return LYMPH_OK;
}

}  // namespace

// The FP32 self block of every polyhedron on the tensor cores, column-major,
// into out[n_poly][nd * nd] or (block_csr) into the self-block slots
// row_ptr[P] of a block-CSR operator.
// The FP32 neighbour blocks list[0..n_list) of the block-CSR operator out,
// each into its own slot, on the tensor cores.
int lymph_dev_nb_tc(lymph_ctx* c, float* out, const int64_t* list, int64_t n_list) {
    switch (c->p) {
        case 1: return launch_nb_tc<1>(c, out, list, n_list);
        case 2: return launch_nb_tc<2>(c, out, list, n_list);
        case 3: return launch_nb_tc<3>(c, out, list, n_list);
        case 4: return launch_nb_tc<4>(c, out, list, n_list);
        default: lymph_set_error("degree not supported on the device"); return LYMPH_ERR_INVALID;
    }
}

int lymph_dev_self_tc(lymph_ctx* c, float* out, bool block_csr) {
    switch (c->p) {
        case 1: return launch_self_tc<1>(c, out, block_csr);
        case 2: return launch_self_tc<2>(c, out, block_csr);
        case 3: return launch_self_tc<3>(c, out, block_csr);
        case 4: return launch_self_tc<4>(c, out, block_csr);
        default: lymph_set_error("degree not supported on the device"); return LYMPH_ERR_INVALID;
    }
}
