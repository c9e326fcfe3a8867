// mf.cu -- the operator apply with matrix-free neighbour terms
// (LYMPH_MIXED_MF).
//
// The neighbour block K_PQ of the assembled operator is a sum over the
// triangles P shares with Q of face-quadrature terms (MAKE_STIFFNESS_FACE,
// src/assemble_element.f90:404-661, inserted by MAKE_MATRICES_FREE,
// src/matrix_free.f90:412-433):
//     K_PQ = -theta/2 I + S - IT/2 ... per triangle, per quadrature point q
// with weights W_q = w_q |face|, P's outward normal n and the material of
// P's tetrahedron.  Contracting the block with u_Q point by point gives the
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
// So the neighbour blocks are never stored: one CTA per polyhedron P applies
// its FP32 self block (streamed from HBM), then, for each triangle P shares
// with a neighbour, evaluates u_Q and grad u_Q at the triangle's quadrature
// points from the Legendre basis on Q's bounding box, forms G and s, and
// tests them against P's basis -- all in FP32 from per-triangle geometry
// precomputed once (quadrature origin and edge vectors, normal, area,
// material, penalty).  The row sums are combined in FP64 in a fixed order and
// finished exactly like the fused kernel (right-hand side, M^-1 in FP64,
// leapfrog update).  A step then reads the self blocks (1/nb of the
// operator bytes) and per-triangle geometry instead of every block.

#include "step_body.cuh"

namespace {

using namespace stepk;

struct MfTri {          // one triangle of a neighbour block, seen from the row polyhedron P
    float o[3];         // quadrature point x_q = o + xi_q e1 + eta_q e2
    float e1[3];
    float e2[3];
    float n[3];         // P's outward unit normal
    float area;         // W_q = w_q area
    float lam, mu;      // material of P's tetrahedron
    float sigma;        // penalty alpha p^2 / min(h_P, h_Q) (lambda + 2 mu)
    int32_t Q;          // neighbour polyhedron
    int32_t pad[3];
};
static_assert(sizeof(MfTri) == 80, "MfTri is 20 words");

struct MfPoly {         // Legendre map of a bounding box: xp = (x - c) ih, phi = sc L(xp_x) L(xp_y) L(xp_z)
    float c[3];
    float ih[3];
    float sc;
    float pad;
};
static_assert(sizeof(MfPoly) == 32, "MfPoly is 8 words");

constexpr int MF_THREADS = 128;

template <int PD> struct MfShape {
    static constexpr int NP = Deg<PD>::NP, ND = Deg<PD>::ND;
    static constexpr int L = PD + 1;              // Legendre degrees per direction
    static constexpr int NQ2 = L * L;             // quadrature points per triangle
    static constexpr int CT = MF_THREADS / NQ2;   // triangles per chunk
    static constexpr int NPT = CT * NQ2;          // points per chunk
    static constexpr int PARTS = MF_THREADS / NP; // point slices of the test phase
    static_assert(ND <= MF_THREADS, "one thread per row of the self block");
};

// The reference's basis order (basis_list, basis_function.f90:12-44): degree
// triples (x, y, z) for q1 = p..0, q2 = p-q1..0, q3 = p-q1-q2..0.
template <int PD> struct Blist {
    int d[Deg<PD>::NP][3];
    constexpr Blist() : d() {
        int ii = 0;
        for (int q1 = PD; q1 >= 0; --q1)
            for (int q2 = PD - q1; q2 >= 0; --q2)
                for (int q3 = PD - q1 - q2; q3 >= 0; --q3) {
                    d[ii][0] = q1;
                    d[ii][1] = q2;
                    d[ii][2] = q3;
                    ++ii;
                }
    }
};

// Legendre polynomials L_0..L_PD on [-1, 1] and their derivatives at x
// (Bonnet's recurrence; the reference evaluates the same polynomials in
// closed form, basis_function.f90:268-437).
template <int PD>
__device__ __forceinline__ void legendre(float x, float* Lv, float* Ld) {
    Lv[0] = 1.0f;
    Ld[0] = 0.0f;
    if (PD >= 1) {
        Lv[1] = x;
        Ld[1] = 1.0f;
    }
#pragma unroll
    for (int n = 1; n < PD; ++n) {
        Lv[n + 1] = ((2 * n + 1) * x * Lv[n] - n * Lv[n - 1]) * (1.0f / (n + 1));
        Ld[n + 1] = Ld[n - 1] + (2 * n + 1) * Lv[n];
    }
}

struct MfArgs {
    StepArgs s;                 // CSR pattern, M^-1, right-hand sides, state, status
    const float* Kself;         // [n_poly][ND * ND] column-major self blocks
    const int64_t* bf_ptr;      // per block: its triangles in tri[]
    const MfTri* tri;           // parallel to the block face lists
    const MfPoly* poly;         // [n_poly]
    const double* u;            // operator input
    float quad[3 * 25];         // (xi, eta, w) of the triangle quadrature points
    float theta;
};

template <int PD, int MODE>
__global__ void __launch_bounds__(MF_THREADS) k_mf(const __grid_constant__ MfArgs A) {
    using S = MfShape<PD>;
    constexpr int NP = S::NP, ND = S::ND, L = S::L, NQ2 = S::NQ2, CT = S::CT, NPT = S::NPT, PARTS = S::PARTS;
    constexpr Blist<PD> BL{};
    __shared__ __align__(16) float s_quad[3 * NQ2];
    __shared__ __align__(16) float s_uP[ND];
    __shared__ __align__(16) MfTri s_tri[CT];
    __shared__ __align__(16) MfPoly s_polyQ[CT];
    __shared__ __align__(16) float4 s_uQ[CT][NP];            // (u_0, u_1, u_2, 0) per basis function
    __shared__ __align__(16) float2 s_leg[NPT][3][L];        // P's (L, L') per point, direction, degree
    __shared__ __align__(16) float4 s_flux[NPT][3];          // (G_i0, G_i1, G_i2, s_i) per point, scaled by P's map
    __shared__ __align__(16) float s_red[PARTS][ND];
    __shared__ __align__(16) double s_b[ND];
    const int P = blockIdx.x, tid = threadIdx.x;
    const double* u = A.u;

    for (int i = tid; i < 3 * NQ2; i += MF_THREADS) s_quad[i] = A.quad[i];
    for (int i = tid; i < ND; i += MF_THREADS) s_uP[i] = (float)u[(int64_t)P * ND + i];
    __syncthreads();

    // ---- self block (FP32, streamed once) ----
    float yself = 0.0f;
    if (tid < ND) {
        const float* Kb = A.Kself + (int64_t)P * ND * ND + tid;
        float a0 = 0.0f, a1 = 0.0f;
#pragma unroll 8
        for (int c = 0; c < ND; c += 2) {
            a0 = fmaf(__ldcs(Kb + (int64_t)c * ND), s_uP[c], a0);
            if (c + 1 < ND) a1 = fmaf(__ldcs(Kb + (int64_t)(c + 1) * ND), s_uP[c + 1], a1);
        }
        yself = a0 + a1;
    }

    // ---- neighbour triangles ----
    const MfPoly pP = A.poly[P];
    const int ta = tid % NP, tpart = tid / NP;  // test phase: basis function, point slice
    int ax = 0, ay = 0, az = 0;
    if (tpart < PARTS) {
#pragma unroll
        for (int b = 0; b < NP; ++b)
            if (b == ta) { ax = BL.d[b][0]; ay = BL.d[b][1]; az = BL.d[b][2]; }
    }
    float acc0 = 0.0f, acc1 = 0.0f, acc2 = 0.0f;
    const int rb = A.s.row_ptr[P], re = A.s.row_ptr[P + 1];
    const int64_t fb = A.bf_ptr[rb + 1], fe = A.bf_ptr[re];
    for (int64_t c0 = fb; c0 < fe; c0 += CT) {
        const int nt = (fe - c0) < CT ? (int)(fe - c0) : CT;
        __syncthreads();  // the previous chunk's staging is consumed
        {
            const float* src = (const float*)(A.tri + c0);
            float* dst = (float*)s_tri;
            for (int i = tid; i < nt * 20; i += MF_THREADS) dst[i] = src[i];
        }
        __syncthreads();
        for (int i = tid; i < nt * 8; i += MF_THREADS) {
            const int t = i / 8, w = i % 8;
            ((float*)&s_polyQ[t])[w] = ((const float*)(A.poly + s_tri[t].Q))[w];
        }
        for (int i = tid; i < nt * NP; i += MF_THREADS) {
            const int t = i / NP, b = i % NP;
            const double* uq = u + (int64_t)s_tri[t].Q * ND + b;
            s_uQ[t][b] = make_float4((float)uq[0], (float)uq[NP], (float)uq[2 * NP], 0.0f);
        }
        __syncthreads();
        // ---- per point: u_Q and grad u_Q, the flux, P's Legendre values ----
        if (tid < nt * NQ2) {
            const int t = tid / NQ2, q = tid % NQ2;
            const MfTri& T = s_tri[t];
            const float xi = s_quad[3 * q], eta = s_quad[3 * q + 1];
            const float W = s_quad[3 * q + 2] * T.area;
            float x[3];
#pragma unroll
            for (int d = 0; d < 3; ++d) x[d] = fmaf(eta, T.e2[d], fmaf(xi, T.e1[d], T.o[d]));
            const MfPoly& pq = s_polyQ[t];
            float Lx[L], Dx[L], Ly[L], Dy[L], Lz[L], Dz[L];
            legendre<PD>((x[0] - pq.c[0]) * pq.ih[0], Lx, Dx);
            legendre<PD>((x[1] - pq.c[1]) * pq.ih[1], Ly, Dy);
            legendre<PD>((x[2] - pq.c[2]) * pq.ih[2], Lz, Dz);
            float v0 = 0, v1 = 0, v2 = 0;
            float d00 = 0, d01 = 0, d02 = 0, d10 = 0, d11 = 0, d12 = 0, d20 = 0, d21 = 0, d22 = 0;
#pragma unroll
            for (int b = 0; b < NP; ++b) {
                const int bx = BL.d[b][0], by = BL.d[b][1], bz = BL.d[b][2];
                const float yz = Ly[by] * Lz[bz];
                const float ph = Lx[bx] * yz;
                const float px = Dx[bx] * yz;
                const float py = Lx[bx] * (Dy[by] * Lz[bz]);
                const float pz = Lx[bx] * (Ly[by] * Dz[bz]);
                const float4 uu = s_uQ[t][b];
                v0 = fmaf(ph, uu.x, v0); v1 = fmaf(ph, uu.y, v1); v2 = fmaf(ph, uu.z, v2);
                d00 = fmaf(px, uu.x, d00); d01 = fmaf(py, uu.x, d01); d02 = fmaf(pz, uu.x, d02);
                d10 = fmaf(px, uu.y, d10); d11 = fmaf(py, uu.y, d11); d12 = fmaf(pz, uu.y, d12);
                d20 = fmaf(px, uu.z, d20); d21 = fmaf(py, uu.z, d21); d22 = fmaf(pz, uu.z, d22);
            }
            // Q's map: phi = sc L L L, d_k phi = sc ih_k (...)
            const float sq = pq.sc, gx = sq * pq.ih[0], gy = sq * pq.ih[1], gz = sq * pq.ih[2];
            const float v[3] = {v0 * sq, v1 * sq, v2 * sq};
            const float D[3][3] = {{d00 * gx, d01 * gy, d02 * gz}, {d10 * gx, d11 * gy, d12 * gz},
                                   {d20 * gx, d21 * gy, d22 * gz}};
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
                for (int k = 0; k < 3; ++k) G[k] = cg * ((i == k ? T.lam * nv : 0.0f) + T.mu * (n[i] * v[k] + v[i] * n[k]));
                float Tv = Tdiag[i] * v[i];
#pragma unroll
                for (int j = 0; j < 3; ++j)
                    if (j != i) Tv += 0.5f * n[i] * n[j] * v[j];
                const float h = T.lam * (n[0] * D[0][i] + n[1] * D[1][i] + n[2] * D[2][i]) + T.mu * n[i] * trD +
                                T.mu * (n[0] * D[i][0] + n[1] * D[i][1] + n[2] * D[i][2]);
                const float s = -W * (T.sigma * Tv + 0.5f * h);
                s_flux[tid][i] = make_float4(G[0] * hx, G[1] * hy, G[2] * hz, s * sP);
            }
            legendre<PD>((x[0] - pP.c[0]) * pP.ih[0], Lx, Dx);
            legendre<PD>((x[1] - pP.c[1]) * pP.ih[1], Ly, Dy);
            legendre<PD>((x[2] - pP.c[2]) * pP.ih[2], Lz, Dz);
#pragma unroll
            for (int l = 0; l < L; ++l) {
                s_leg[tid][0][l] = make_float2(Lx[l], Dx[l]);
                s_leg[tid][1][l] = make_float2(Ly[l], Dy[l]);
                s_leg[tid][2][l] = make_float2(Lz[l], Dz[l]);
            }
        }
        __syncthreads();
        // ---- test against P's basis: thread (a, slice) over the chunk's points ----
        if (tpart < PARTS) {
            for (int pt = tpart; pt < nt * NQ2; pt += PARTS) {
                const float2 lx = s_leg[pt][0][ax], ly = s_leg[pt][1][ay], lz = s_leg[pt][2][az];
                const float yz = ly.x * lz.x;
                const float ph = lx.x * yz, px = lx.y * yz, py = lx.x * (ly.y * lz.x), pz = lx.x * (ly.x * lz.y);
                const float4 f0 = s_flux[pt][0], f1 = s_flux[pt][1], f2 = s_flux[pt][2];
                acc0 = fmaf(px, f0.x, fmaf(py, f0.y, fmaf(pz, f0.z, fmaf(ph, f0.w, acc0))));
                acc1 = fmaf(px, f1.x, fmaf(py, f1.y, fmaf(pz, f1.z, fmaf(ph, f1.w, acc1))));
                acc2 = fmaf(px, f2.x, fmaf(py, f2.y, fmaf(pz, f2.z, fmaf(ph, f2.w, acc2))));
            }
        }
    }
    if (tpart < PARTS) {
        s_red[tpart][ta] = acc0;
        s_red[tpart][NP + ta] = acc1;
        s_red[tpart][2 * NP + ta] = acc2;
    }
    __syncthreads();
    double y = 0.0;
    if (tid < ND) {
        y = (double)yself;
#pragma unroll
        for (int k = 0; k < PARTS; ++k) y += (double)s_red[k][tid];
    }
    finish_poly<PD, MODE>(A.s, P, y, s_b);
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
                          const double* __restrict__ area, const double* __restrict__ hk, const RefTables* ref,
                          double alpha, int p, MfTri* out, int* status) {
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
            T.o[j] = (float)(cmap[j][2] + cmap[j][3]);
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
        T.pad[0] = T.pad[1] = T.pad[2] = 0;
        out[e] = T;
    }
}

__global__ void k_mf_polys(int n_poly, const double* __restrict__ bbox, MfPoly* out) {
    const int P = blockIdx.x * blockDim.x + threadIdx.x;
    if (P >= n_poly) return;
    MfPoly m;
    double hprod = 1.0;
    for (int d = 0; d < 3; ++d) {
        const double a = bbox[P * 6 + 2 * d], b = bbox[P * 6 + 2 * d + 1];
        const double hb = (b - a) / 2.0, mb = (b + a) / 2.0;
        m.c[d] = (float)mb;
        m.ih[d] = (float)(1.0 / hb);
        hprod *= hb;
    }
    m.sc = (float)(1.0 / sqrt(hprod));
    m.pad = 0.0f;
    out[P] = m;
}

template <int PD, int MODE>
int launch_mf_t(lymph_ctx* c, const StepArgs& s) {
    MfArgs a;
    a.s = s;
    a.Kself = (const float*)c->d_K;
    a.bf_ptr = c->d_bf_ptr;
    a.tri = (const MfTri*)c->d_mf_tri;
    a.poly = (const MfPoly*)c->d_mf_poly;
    a.u = (MODE == MODE_FIRST || MODE == MODE_BILIN) ? s.u0 : s.un;
    for (int i = 0; i < 3 * 25; ++i) a.quad[i] = c->mf_quad[i];
    a.theta = (float)c->theta;
    k_mf<PD, MODE><<<c->n_poly, MF_THREADS, 0, c->stream>>>(a);
    c->launches++;
    return LYMPH_OK;
}

template <int PD>
int launch_mf_p(lymph_ctx* c, int mode, const StepArgs& s) {
    switch (mode) {
        case MODE_STEP: return launch_mf_t<PD, MODE_STEP>(c, s);
        case MODE_FIRST: return launch_mf_t<PD, MODE_FIRST>(c, s);
        case MODE_APPLY: return launch_mf_t<PD, MODE_APPLY>(c, s);
        case MODE_BILIN: return launch_mf_t<PD, MODE_BILIN>(c, s);
        default: lymph_set_error("matrix-free neighbour terms: unsupported mode"); return LYMPH_ERR_INVALID;
    }
}

}  // namespace

// The per-triangle and per-polyhedron FP32 tables of the matrix-free
// neighbour terms (after geometry and the block pattern exist).
int lymph_mf_setup(lymph_ctx* c, const RefTables& R) {
    const int nq2 = (c->p + 1) * (c->p + 1);
    for (int q = 0; q < 25; ++q) {
        const bool in = q < nq2;
        c->mf_quad[3 * q + 0] = in ? (float)R.nodtria2[q * 4 + 0] : 0.0f;
        c->mf_quad[3 * q + 1] = in ? (float)R.nodtria2[q * 4 + 1] : 0.0f;
        c->mf_quad[3 * q + 2] = in ? (float)R.weitria2[q] : 0.0f;
    }
    if (!c->d_mf_tri) {
        void* p = nullptr;
        LYMPH_CUDA_TRY(cudaMalloc(&p, sizeof(MfTri) * (size_t)(c->n_block_faces > 0 ? c->n_block_faces : 1)));
        c->d_mf_tri = p;
        c->device_bytes += (int64_t)(sizeof(MfTri) * c->n_block_faces);
        LYMPH_CUDA_TRY(cudaMalloc(&p, sizeof(MfPoly) * (size_t)c->n_poly));
        c->d_mf_poly = p;
        c->device_bytes += (int64_t)(sizeof(MfPoly) * c->n_poly);
    }
    if (c->n_blocks > 0) {
        k_mf_tris<<<(unsigned)((c->n_blocks + 127) / 128), 128, 0, c->stream>>>(
            c->n_blocks, c->d_blk_row, c->d_col, c->d_bf_ptr, c->d_bf, c->d_neigh, c->d_tet_poly, c->d_tet_mat,
            c->d_mat, c->d_fk, c->d_normal, c->d_area, c->d_hk, c->d_ref, c->alpha, c->p, (MfTri*)c->d_mf_tri,
            c->d_status);
        c->launches++;
    }
    k_mf_polys<<<(c->n_poly + 127) / 128, 128, 0, c->stream>>>(c->n_poly, c->d_bbox, (MfPoly*)c->d_mf_poly);
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
