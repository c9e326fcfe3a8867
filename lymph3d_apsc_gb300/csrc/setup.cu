// setup.cu -- device set-up kernels: geometry, polyhedron bounding boxes,
// operator block assembly, mass matrices and their Cholesky factors, RHS
// vectors and L2 projections.  All arithmetic FP64.
//
// Assembly design.  The reference builds every (3Np)^2 block entry by entry
// at every quadrature point (MAKE_STIFFNESS_VOLUME, assemble_element.f90:24-77;
// MAKE_STIFFNESS_FACE, :404-661).  Here each CTA owns one block and
// accumulates, per pair of basis functions (m,n), a handful of scalar
// moments over the quadrature points, then folds them into the 9 component
// entries with the material and face constants:
//   volume:  G_kl(m,n) = sum_q w|J| d_k phi_m d_l phi_n,
//            V_ij = lambda G_ij + mu G_ji + delta_ij mu (G_11+G_22+G_33)
//   faces:   P(a,b) = sum W phi_a phi_b', H_k(a,b) = sum W d_k phi_a phi_b',
//            HT_k(a,b) = sum W phi_a d_k phi_b'  (W = weight * area)
//            S  = sigma T_ij P,  T_ii = n_i^2 + (n_j^2 + n_k^2)/2,  T_ij = n_i n_j / 2
//            I(i,j) = c [lambda n_j H_i + mu n_i H_j + delta_ij mu n.H]
// which is algebraically the reference's sum, with 9x fewer FP64 products.

#include "common.cuh"

namespace {

constexpr int ASM_THREADS = 256;
// AsmArgs::which for the mass matrices alone (the self blocks of the
// mixed operators come from the tensor-core assembly in selftc.cu)
constexpr int ASM_MASS_ONLY = 2;

template <int P> struct Deg {
    static constexpr int NP = (P + 1) * (P + 2) * (P + 3) / 6;
    static constexpr int ND = 3 * NP;
    static constexpr int NQ3 = (P + 1) * (P + 1) * (P + 1);
    static constexpr int NQ2 = (P + 1) * (P + 1);
    static constexpr int NPAIR = NP * NP;
};

// Vertex triples of the faces used for normals/areas,
// MAKE_PARTITION_AND_MPI_FILES.f90:1087-1096 (0-based local ids).
__constant__ int c_face_verts[4][3] = {{2, 1, 0}, {0, 1, 3}, {1, 2, 3}, {2, 0, 3}};

// jacobians (Poly_ref_mappings.f90:18-75) and CREATE_NORMAL_FACE
// (MAKE_PARTITION_AND_MPI_FILES.f90:1429-1504), one thread per tetrahedron.
__global__ void k_geometry(int n_tet, const double* __restrict__ X, const int32_t* __restrict__ tv, double* fk,
                           double* jdet, double* nrm, double* area, int* status) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_tet) return;
    double x[4], y[4], z[4];
    for (int v = 0; v < 4; ++v) {
        int id = tv[t * 4 + v];
        x[v] = X[id * 3 + 0]; y[v] = X[id * 3 + 1]; z[v] = X[id * 3 + 2];
    }
    double F[3][4];
    F[0][0] = x[1] - x[0]; F[0][1] = x[2] - x[0]; F[0][2] = x[3] - x[0]; F[0][3] = x[0];
    F[1][0] = y[1] - y[0]; F[1][1] = y[2] - y[0]; F[1][2] = y[3] - y[0]; F[1][3] = y[0];
    F[2][0] = z[1] - z[0]; F[2][1] = z[2] - z[0]; F[2][2] = z[3] - z[0]; F[2][3] = z[0];
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 4; ++b) fk[t * 12 + a * 4 + b] = F[a][b];
    double d = F[0][0] * F[1][1] * F[2][2] - F[0][0] * F[1][2] * F[2][1] - F[0][1] * F[1][0] * F[2][2] +
               F[0][1] * F[1][2] * F[2][0] + F[0][2] * F[1][0] * F[2][1] - F[1][1] * F[0][2] * F[2][0];
    jdet[t] = d;
    if (d == 0.0) atomicOr(status, ST_DEGENERATE);
    for (int f = 0; f < 4; ++f) {
        const double* c1 = &X[tv[t * 4 + c_face_verts[f][0]] * 3];
        const double* c2 = &X[tv[t * 4 + c_face_verts[f][1]] * 3];
        const double* c3 = &X[tv[t * 4 + c_face_verts[f][2]] * 3];
        double Qx = c1[0] - c2[0], Qy = c1[1] - c2[1], Qz = c1[2] - c2[2];
        double Px = c3[0] - c2[0], Py = c3[1] - c2[1], Pz = c3[2] - c2[2];
        double n1 = Py * Qz - Pz * Qy, n2 = -Px * Qz + Pz * Qx, n3 = Px * Qy - Py * Qx;
        double nn = sqrt(n1 * n1 + n2 * n2 + n3 * n3);
        if (nn == 0.0) atomicOr(status, ST_DEGENERATE);
        nrm[t * 12 + f * 3 + 0] = n1 / nn;
        nrm[t * 12 + f * 3 + 1] = n2 / nn;
        nrm[t * 12 + f * 3 + 2] = n3 / nn;
        area[t * 4 + f] = nn;
    }
}

// CREATE_BBOX_EL (MAKE_PARTITION_AND_MPI_FILES.f90:1510-1580): bounding box
// and diameter (largest vertex distance) of every polyhedron.
__global__ void k_bbox(int n_poly, const int32_t* __restrict__ pptr, const int32_t* __restrict__ ptets,
                       const int32_t* __restrict__ tv, const double* __restrict__ X, double* bbox, double* hk) {
    int P = blockIdx.x * blockDim.x + threadIdx.x;
    if (P >= n_poly) return;
    int t0 = pptr[P], t1 = pptr[P + 1];
    double mn[3] = {1e300, 1e300, 1e300}, mx[3] = {-1e300, -1e300, -1e300};
    int nv = 4 * (t1 - t0);
    for (int a = 0; a < nv; ++a) {
        const double* c = &X[tv[ptets[t0 + a / 4] * 4 + (a & 3)] * 3];
        for (int d = 0; d < 3; ++d) { mn[d] = fmin(mn[d], c[d]); mx[d] = fmax(mx[d], c[d]); }
    }
    double h = 0.0;
    for (int a = 0; a < nv; ++a) {
        const double* ca = &X[tv[ptets[t0 + a / 4] * 4 + (a & 3)] * 3];
        for (int b = a + 1; b < nv; ++b) {
            const double* cb = &X[tv[ptets[t0 + b / 4] * 4 + (b & 3)] * 3];
            double dist = sqrt((ca[0] - cb[0]) * (ca[0] - cb[0]) + (ca[1] - cb[1]) * (ca[1] - cb[1]) +
                               (ca[2] - cb[2]) * (ca[2] - cb[2]));
            if (dist > h) h = dist;
        }
    }
    for (int d = 0; d < 3; ++d) { bbox[P * 6 + 2 * d] = mn[d]; bbox[P * 6 + 2 * d + 1] = mx[d]; }
    hk[P] = h;
}

// Physical quadrature points of face f of tetrahedron t as basis_boundary
// forms them (basis_function.f90:560-577): temp = Fk node_maps(:,:,f),
// pt = temp nodtria2.
__device__ inline void face_point(const double* fk, const RefTables* ref, int f, int q, double pt[3]) {
    const double* nm = &ref->node_maps[f * 16];
    const double* nt = &ref->nodtria2[q * 4];
    for (int j = 0; j < 3; ++j) {
        double s = 0.0;
        for (int l = 0; l < 4; ++l) {
            double tmp = 0.0;
            for (int m = 0; m < 4; ++m) tmp = tmp + fk[j * 4 + m] * nm[m * 4 + l];
            s = s + tmp * nt[l];
        }
        pt[j] = s;
    }
}

// Physical point of tetrahedron quadrature node q (basis, :471-479).
__device__ inline void tet_point(const double* fk, const RefTables* ref, int q, double pt[3]) {
    const double* nt = &ref->nodtet3[q * 4];
    for (int j = 0; j < 3; ++j) {
        double s = 0.0;
        for (int l = 0; l < 4; ++l) s = s + fk[j * 4 + l] * nt[l];
        pt[j] = s;
    }
}

struct AsmArgs {
    const int32_t* blk_row;
    const int32_t* col;
    const int64_t* bf_ptr;
    const int32_t* bf;
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
    double alpha, theta;
    int which;        // LYMPH_BLOCKS_K or LYMPH_BLOCKS_ADG
    int out_fp32;     // store FP32 blocks
    void* out;        // [n][out_stride] blocks, each [ND][ND] column-major
    const int64_t* list;  // blocks to assemble (null: all, in order); output slot = position in the list
    int64_t out_stride;   // elements from one output block to the next (>= ND*ND)
    double* M;        // [n_poly][NP][NP] rho-weighted mass (self blocks only; may be null)
    double* Mm;       // unweighted (modal) mass
    int64_t block0;   // first block of this launch
};

// One CTA per operator block (row polyhedron P, column polyhedron Q).
template <int PD>
__global__ void __launch_bounds__(ASM_THREADS) k_assemble(AsmArgs A) {
    using D = Deg<PD>;
    constexpr int NP = D::NP, ND = D::ND, NQ3 = D::NQ3, NQ2 = D::NQ2;
    constexpr int PPT = (D::NPAIR + ASM_THREADS - 1) / ASM_THREADS;
    constexpr int QC = NQ3 < 32 ? NQ3 : 32;
    extern __shared__ double sm[];
    double* acc = sm;                   // [ND][ND] row-major
    double* tab = acc + ND * ND;        // tabulation area
    const int tid = threadIdx.x;
    const int64_t slot = A.block0 + blockIdx.x;
    const int64_t k = A.list ? A.list[slot] : slot;
    const int P = A.blk_row[k];
    const int Qc = A.col[k];
    const bool self = (Qc == P);
    const double pdeg2 = (double)(PD * PD);

    const bool mass_only = (A.which == ASM_MASS_ONLY);
    if (!mass_only)
        for (int i = tid; i < ND * ND; i += ASM_THREADS) acc[i] = 0.0;

    if (self) {
        // ---- volume terms and mass matrices over the sub-tetrahedra ----
        double* tphi = tab;                 // [QC][NP]
        double* tdphi = tphi + QC * NP;     // [QC][3][NP]
        double* tw = tdphi + QC * 3 * NP;   // [QC]
        double* ttl = tw + QC;              // [QC][3][p+1] (value, derivative) pairs
        double msum[PPT], mrho[PPT];
#pragma unroll
        for (int u = 0; u < PPT; ++u) { msum[u] = 0.0; mrho[u] = 0.0; }
        const double* bb = &A.bbox[P * 6];
        for (int kt = A.poly_ptr[P]; kt < A.poly_ptr[P + 1]; ++kt) {
            const int t = A.poly_tets[kt];
            const double* fk = &A.fk[t * 12];
            const int mid = A.tet_mat[t];
            const double rho = A.mat[mid * 3 + 0], lam = A.mat[mid * 3 + 1], mu = A.mat[mid * 3 + 2];
            const double aj = fabs(A.jdet[t]);
            double G[PPT][9], Mt[PPT];
#pragma unroll
            for (int u = 0; u < PPT; ++u) {
                Mt[u] = 0.0;
#pragma unroll
                for (int e = 0; e < 9; ++e) G[u][e] = 0.0;
            }
            for (int q0 = 0; q0 < NQ3; q0 += QC) {
                __syncthreads();
                if (mass_only) {
                    // phi alone, from one table of the 1-D factors per point
                    // (3 (p+1) legendre_1d calls instead of 3 Np), multiplied
                    // in basis_eval's order, and w phi_m once per (q, m): the
                    // same values and sums as the full assembly, bit for bit
                    constexpr int L1 = PD + 1;
                    double* tleg = tdphi;               // [QC][3][L1]
                    double* twphi = tdphi + QC * 3 * L1; // [QC][NP]
                    for (int it = tid; it < QC * 3 * L1; it += ASM_THREADS) {
                        const int qq = it / (3 * L1), r = it % (3 * L1), d = r / L1, deg = r % L1, q = q0 + qq;
                        if (q < NQ3) {
                            double pt[3], v, dv;
                            tet_point(fk, A.ref, q, pt);
                            legendre_1d(pt[d], deg, bb[2 * d], bb[2 * d + 1], &v, &dv);
                            tleg[it] = v;
                            if (r == 0) tw[qq] = A.ref->weitet3[q] * aj;
                        }
                    }
                    __syncthreads();
                    for (int it = tid; it < QC * NP; it += ASM_THREADS) {
                        const int qq = it / NP, f = it % NP, q = q0 + qq;
                        if (q < NQ3) {
                            const int* bl = &A.ref->blist[f * 3];
                            const double* tq = tleg + qq * 3 * L1;
                            const double ph = tq[bl[0]] * tq[L1 + bl[1]] * tq[2 * L1 + bl[2]];
                            tphi[qq * NP + f] = ph;
                            twphi[qq * NP + f] = tw[qq] * ph;
                        }
                    }
                    __syncthreads();
                    const int nq = (NQ3 - q0) < QC ? (NQ3 - q0) : QC;
#pragma unroll
                    for (int u = 0; u < PPT; ++u) {
                        const int pr = tid + u * ASM_THREADS;
                        if (pr < D::NPAIR) {
                            const int m = pr / NP, n = pr % NP;
                            for (int qq = 0; qq < nq; ++qq) Mt[u] += twphi[qq * NP + m] * tphi[qq * NP + n];
                        }
                    }
                    continue;
                }
                // basis_eval's 1-D factors (value, derivative) per point,
                // coordinate and degree, then their products in its order:
                // the same bits at 3 (p+1) legendre_1d calls per point
                // instead of 3 Np
                constexpr int L1 = PD + 1;
                for (int it = tid; it < QC * 3 * L1; it += ASM_THREADS) {
                    const int qq = it / (3 * L1), r = it % (3 * L1), d = r / L1, deg = r % L1, q = q0 + qq;
                    if (q < NQ3) {
                        double pt[3];
                        tet_point(fk, A.ref, q, pt);
                        legendre_1d(pt[d], deg, bb[2 * d], bb[2 * d + 1], &ttl[2 * it], &ttl[2 * it + 1]);
                        if (r == 0) tw[qq] = A.ref->weitet3[q] * aj;
                    }
                }
                __syncthreads();
                for (int it = tid; it < QC * NP; it += ASM_THREADS) {
                    const int qq = it / NP, f = it % NP, q = q0 + qq;
                    if (q < NQ3) {
                        const int* bl = &A.ref->blist[f * 3];
                        const double* tq = ttl + 2 * qq * 3 * L1;
                        const double vx = tq[2 * bl[0]], dx = tq[2 * bl[0] + 1];
                        const double vy = tq[2 * (L1 + bl[1])], dy = tq[2 * (L1 + bl[1]) + 1];
                        const double vz = tq[2 * (2 * L1 + bl[2])], dz = tq[2 * (2 * L1 + bl[2]) + 1];
                        tphi[qq * NP + f] = vx * vy * vz;
                        tdphi[(qq * 3 + 0) * NP + f] = dx * vy * vz;
                        tdphi[(qq * 3 + 1) * NP + f] = vx * dy * vz;
                        tdphi[(qq * 3 + 2) * NP + f] = vx * vy * dz;
                    }
                }
                __syncthreads();
                const int nq = (NQ3 - q0) < QC ? (NQ3 - q0) : QC;
#pragma unroll
                for (int u = 0; u < PPT; ++u) {
                    const int pr = tid + u * ASM_THREADS;
                    if (pr < D::NPAIR) {
                        const int m = pr / NP, n = pr % NP;
                        for (int qq = 0; qq < nq; ++qq) {
                            const double w = tw[qq];
                            const double a0 = w * tdphi[(qq * 3 + 0) * NP + m];
                            const double a1 = w * tdphi[(qq * 3 + 1) * NP + m];
                            const double a2 = w * tdphi[(qq * 3 + 2) * NP + m];
                            const double b0 = tdphi[(qq * 3 + 0) * NP + n];
                            const double b1 = tdphi[(qq * 3 + 1) * NP + n];
                            const double b2 = tdphi[(qq * 3 + 2) * NP + n];
                            G[u][0] += a0 * b0; G[u][1] += a0 * b1; G[u][2] += a0 * b2;
                            G[u][3] += a1 * b0; G[u][4] += a1 * b1; G[u][5] += a1 * b2;
                            G[u][6] += a2 * b0; G[u][7] += a2 * b1; G[u][8] += a2 * b2;
                            Mt[u] += (w * tphi[qq * NP + m]) * tphi[qq * NP + n];
                        }
                    }
                }
            }
            // fold V_t = lambda G_ij + mu G_ji + delta_ij mu tr G into the block
#pragma unroll
            for (int u = 0; u < PPT; ++u) {
                const int pr = tid + u * ASM_THREADS;
                if (pr < D::NPAIR) {
                    const int m = pr / NP, n = pr % NP;
                    const double tr = G[u][0] + G[u][4] + G[u][8];
                    if (!mass_only) {
#pragma unroll
                        for (int i = 0; i < 3; ++i)
#pragma unroll
                            for (int j = 0; j < 3; ++j) {
                                double v = lam * G[u][i * 3 + j] + mu * G[u][j * 3 + i];
                                if (i == j) v += mu * tr;
                                acc[(i * NP + m) * ND + j * NP + n] += v;
                            }
                    }
                    msum[u] += Mt[u];
                    mrho[u] += Mt[u] * rho;
                }
            }
        }
        if (A.M != nullptr) {
#pragma unroll
            for (int u = 0; u < PPT; ++u) {
                const int pr = tid + u * ASM_THREADS;
                if (pr < D::NPAIR) {
                    A.M[(int64_t)P * D::NPAIR + pr] = mrho[u];
                    A.Mm[(int64_t)P * D::NPAIR + pr] = msum[u];
                }
            }
        }
    }

    if (mass_only) return;

    // ---- face terms ----
    {
        double* fpt = tab;                        // [NQ2][3]
        double* fphi = fpt + NQ2 * 3;             // [2][NQ2][NP]
        double* fdphi = fphi + 2 * NQ2 * NP;      // [2][NQ2][3][NP]
        double* ftl = fdphi + 2 * NQ2 * 3 * NP;   // [2][NQ2][3][p+1] (value, derivative) pairs
        const double* bbp = &A.bbox[P * 6];
        for (int64_t e = A.bf_ptr[k]; e < A.bf_ptr[k + 1]; ++e) {
            const int code = A.bf[e];
            const int t = code >> 2, f = code & 3;
            const int E2 = A.neigh[code];
            const bool dir = (E2 == LYMPH_BC_DIRI);
            const int Qn = dir ? -1 : A.tet_poly[E2];
            const double* fk = &A.fk[t * 12];
            const int mid = A.tet_mat[t];
            const double lam = A.mat[mid * 3 + 1], mu = A.mat[mid * 3 + 2];
            const double n0 = A.nrm[t * 12 + f * 3 + 0], n1 = A.nrm[t * 12 + f * 3 + 1], n2 = A.nrm[t * 12 + f * 3 + 2];
            const double ar = A.area[t * 4 + f];
            const double Dbar = lam + 2 * mu;
            const double hk1 = A.hk[P];
            const double sigma = dir ? A.alpha * pdeg2 / hk1 * Dbar : A.alpha * pdeg2 / fmin(hk1, A.hk[Qn]) * Dbar;
            const double cI = dir ? 1.0 : 0.5;
            const int nside = self ? 1 : 2;
            __syncthreads();
            for (int q = tid; q < NQ2; q += ASM_THREADS) face_point(fk, A.ref, f, q, &fpt[q * 3]);
            __syncthreads();
            constexpr int L1 = PD + 1;
            for (int it = tid; it < nside * NQ2 * 3 * L1; it += ASM_THREADS) {
                const int s = it / (NQ2 * 3 * L1), rem = it % (NQ2 * 3 * L1), q = rem / (3 * L1);
                const int d = (rem % (3 * L1)) / L1, deg = rem % L1;
                const double* bb = (s == 0) ? bbp : &A.bbox[Qn * 6];
                legendre_1d(fpt[q * 3 + d], deg, bb[2 * d], bb[2 * d + 1], &ftl[2 * it], &ftl[2 * it + 1]);
            }
            __syncthreads();
            for (int it = tid; it < nside * NQ2 * NP; it += ASM_THREADS) {
                const int s = it / (NQ2 * NP), rem = it % (NQ2 * NP), q = rem / NP, fb = rem % NP;
                const int* bl = &A.ref->blist[fb * 3];
                const double* tq = ftl + 2 * (s * NQ2 + q) * 3 * L1;
                const double vx = tq[2 * bl[0]], dx = tq[2 * bl[0] + 1];
                const double vy = tq[2 * (L1 + bl[1])], dy = tq[2 * (L1 + bl[1]) + 1];
                const double vz = tq[2 * (2 * L1 + bl[2])], dz = tq[2 * (2 * L1 + bl[2]) + 1];
                fphi[(s * NQ2 + q) * NP + fb] = vx * vy * vz;
                fdphi[((s * NQ2 + q) * 3 + 0) * NP + fb] = dx * vy * vz;
                fdphi[((s * NQ2 + q) * 3 + 1) * NP + fb] = vx * dy * vz;
                fdphi[((s * NQ2 + q) * 3 + 2) * NP + fb] = vx * vy * dz;
            }
            __syncthreads();
            const double nv[3] = {n0, n1, n2};
            const double T00 = fabs(n0) * fabs(n0) + 0.5 * (fabs(n1) * fabs(n1)) + 0.5 * (fabs(n2) * fabs(n2));
            const double T11 = fabs(n1) * fabs(n1) + 0.5 * (fabs(n0) * fabs(n0)) + 0.5 * (fabs(n2) * fabs(n2));
            const double T22 = fabs(n2) * fabs(n2) + 0.5 * (fabs(n0) * fabs(n0)) + 0.5 * (fabs(n1) * fabs(n1));
            const int sb = self ? 0 : 1;  // side of the trial functions (column polyhedron)
#pragma unroll
            for (int u = 0; u < PPT; ++u) {
                const int pr = tid + u * ASM_THREADS;
                if (pr >= D::NPAIR) continue;
                const int a = pr / NP, b = pr % NP;
                // Pab = sum W phi+_a phi^s_b ; H_k = sum W d_k phi+_a phi^s_b ;
                // HT_k = sum W phi+_a d_k phi^s_b
                double Pab = 0, H0 = 0, H1 = 0, H2 = 0, T0 = 0, T1 = 0, T2 = 0;
                for (int q = 0; q < NQ2; ++q) {
                    const double W = A.ref->weitria2[q] * ar;
                    const double pa = fphi[q * NP + a];
                    const double pb = fphi[(sb * NQ2 + q) * NP + b];
                    const double wa = W * pa, wb = W * pb;
                    Pab += wa * pb;
                    H0 += wb * fdphi[(q * 3 + 0) * NP + a];
                    H1 += wb * fdphi[(q * 3 + 1) * NP + a];
                    H2 += wb * fdphi[(q * 3 + 2) * NP + a];
                    T0 += wa * fdphi[((sb * NQ2 + q) * 3 + 0) * NP + b];
                    T1 += wa * fdphi[((sb * NQ2 + q) * 3 + 1) * NP + b];
                    T2 += wa * fdphi[((sb * NQ2 + q) * 3 + 2) * NP + b];
                }
                const double H[3] = {H0, H1, H2}, HT[3] = {T0, T1, T2};
                const double nH = n0 * H0 + n1 * H1 + n2 * H2;
                const double nHT = n0 * T0 + n1 * T1 + n2 * T2;
#pragma unroll
                for (int i = 0; i < 3; ++i)
#pragma unroll
                    for (int j = 0; j < 3; ++j) {
                        const double Tij = (i == j) ? (i == 0 ? T00 : (i == 1 ? T11 : T22)) : 0.5 * nv[i] * nv[j];
                        const double S = sigma * Tij * Pab;
                        double v;
                        if (self) {
                            if (A.which == LYMPH_BLOCKS_ADG) {
                                v = S;
                            } else {
                                // S_E1 + theta I_E1(i,j,a,b) - I_E1(j,i,b,a)
                                double I = lam * nv[j] * H[i] + mu * nv[i] * H[j] + (i == j ? mu * nH : 0.0);
                                double IT = lam * nv[i] * HT[j] + mu * nv[j] * HT[i] + (i == j ? mu * nHT : 0.0);
                                v = S + A.theta * cI * I - cI * IT;
                            }
                        } else {
                            if (A.which == LYMPH_BLOCKS_ADG) {
                                v = -S;
                            } else {
                                // theta I_E2 + S_E2 - IT_E2 (IT_E2 carries the reference's index
                                // order, assemble_element.f90:610-616)
                                double I = lam * nv[j] * H[i] + mu * nv[i] * H[j] + (i == j ? mu * nH : 0.0);
                                double IT = lam * nv[j] * HT[i] + mu * nv[i] * HT[j] + (i == j ? mu * nHT : 0.0);
                                v = -0.5 * A.theta * I - S - 0.5 * IT;
                            }
                        }
                        acc[(i * NP + a) * ND + j * NP + b] += v;
                    }
            }
        }
    }
    __syncthreads();
    // write the block column-major (entry (r,c) at c*ND + r)
    const int64_t base = slot * A.out_stride;
    if (A.out_fp32) {
        float* o = (float*)A.out;
        for (int i = tid; i < ND * ND; i += ASM_THREADS) {
            const int c = i / ND, r = i % ND;
            o[base + i] = (float)acc[r * ND + c];
        }
    } else {
        double* o = (double*)A.out;
        for (int i = tid; i < ND * ND; i += ASM_THREADS) {
            const int c = i / ND, r = i % ND;
            o[base + i] = acc[r * ND + c];
        }
    }
}

template <int PD> size_t asm_smem() {
    using D = Deg<PD>;
    constexpr int QC = D::NQ3 < 32 ? D::NQ3 : 32;
    size_t vol = (size_t)QC * D::NP * 4 + QC + (size_t)QC * 3 * (PD + 1) * 2;
    size_t face = (size_t)D::NQ2 * 3 + 2 * (size_t)D::NQ2 * D::NP * 4 + 2 * (size_t)D::NQ2 * 3 * (PD + 1) * 2;
    return sizeof(double) * ((size_t)D::ND * D::ND + (vol > face ? vol : face));
}

// cholesky (vet_mat_operations.f90:84-120) of the NP x NP matrix of every
// polyhedron, one warp each; writes R (row-major upper) and R^T.
__global__ void k_cholesky(int n_poly, int NP, const double* __restrict__ A, double* R, double* RT, int* status) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= n_poly) return;
    extern __shared__ double shm[];
    double* r = shm + (threadIdx.x >> 5) * NP * NP;
    const double* a = A + (int64_t)warp * NP * NP;
    for (int i = lane; i < NP * NP; i += 32) r[i] = 0.0;
    __syncwarp();
    bool ok = true;
    for (int j = 0; j < NP; ++j) {
        double sum = a[j * NP + j];
        for (int kk = 0; kk < j; ++kk) sum = sum - r[kk * NP + j] * r[kk * NP + j];
        if (!(sum > 0.0)) { ok = false; sum = 1.0; }
        const double rjj = sqrt(sum);
        for (int i = j + 1 + lane; i < NP; i += 32) {
            double s = a[j * NP + i];
            for (int kk = 0; kk < j; ++kk) s = s - r[kk * NP + j] * r[kk * NP + i];
            r[j * NP + i] = s / rjj;
        }
        if (lane == 0) r[j * NP + j] = rjj;
        __syncwarp();
    }
    if (!ok && lane == 0) atomicOr(status, ST_NOT_SPD);
    for (int i = lane; i < NP * NP; i += 32) {
        const int row = i / NP, c = i % NP;
        R[(int64_t)warp * NP * NP + i] = r[i];
        RT[(int64_t)warp * NP * NP + c * NP + row] = r[i];
    }
}

// Inverse of the mass matrix from its Cholesky factor: column k of M^-1 is
// solve_LU(R^T, R, e_k) (vet_mat_operations.f90:123-153, reference operation
// order), one lane per column.  Stored column-major: Minv[c*NP + r] = (M^-1)(r,c),
// so that lane r of a warp reads consecutive addresses when applying it.
__global__ void k_mass_inverse(int n_poly, int NP, const double* __restrict__ R, double* Minv) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= n_poly) return;
    const double* r = R + (int64_t)warp * NP * NP;
    double* out = Minv + (int64_t)warp * NP * NP;
    for (int k = lane; k < NP; k += 32) {
        double* x = out + (int64_t)k * NP;  // column k, solved in place
        for (int i = 0; i < NP; ++i) x[i] = (i == k) ? 1.0 : 0.0;
        for (int i = 0; i < NP; ++i) {
            double y = x[i];
            for (int j = 0; j < i; ++j) y = y - r[j * NP + i] * x[j];
            x[i] = y / r[i * NP + i];
        }
        for (int i = NP - 1; i >= 0; --i) {
            double v = x[i];
            for (int j = i + 1; j < NP; ++j) v = v - r[i * NP + j] * x[j];
            x[i] = v / r[i * NP + i];
        }
    }
}

// ---- data functions (problem_data_and_properties.f90) ----
__device__ inline void dev_u_space(const double p[3], double r[3]) {
    const double PI = 3.141592653589793;
    r[0] = cos(PI * p[0]) * sin(PI * p[1]) * sin(PI * p[2]);
    r[1] = sin(PI * p[0]) * cos(PI * p[1]) * sin(PI * p[2]);
    r[2] = sin(PI * p[0]) * sin(PI * p[1]) * cos(PI * p[2]);
}

__device__ inline void dev_forcing(int id, double lam, double mu, const double p[3], double rho, double r[3]) {
    const double PI = 3.141592653589793;
    if (id == LYMPH_F_TIME) {
        const double c = (-2.0 * rho + 3.0 * (lam + 2.0 * mu)) * PI * PI;
        r[0] = c * cos(PI * p[0]) * sin(PI * p[1]) * sin(PI * p[2]);
        r[1] = c * sin(PI * p[0]) * cos(PI * p[1]) * sin(PI * p[2]);
        r[2] = c * sin(PI * p[0]) * sin(PI * p[1]) * cos(PI * p[2]);
    } else if (id == LYMPH_F_STAT) {
        r[0] = 3 * PI * PI * cos(PI * p[0]) * sin(PI * p[1]) * sin(PI * p[2]) * (lam + 2 * mu);
        r[1] = 3 * PI * PI * cos(PI * p[1]) * sin(PI * p[0]) * sin(PI * p[2]) * (lam + 2 * mu);
        r[2] = 3 * PI * PI * cos(PI * p[2]) * sin(PI * p[0]) * sin(PI * p[1]) * (lam + 2 * mu);
    } else {
        r[0] = r[1] = r[2] = 0.0;
    }
}

__device__ inline void dev_dirichlet(int id, const double p[3], int tag, double r[3]) {
    if (id == LYMPH_GD) {
        if (tag == 1 || tag == 2 || tag == 3) dev_u_space(p, r);
        else r[0] = r[1] = r[2] = 0.0;
    } else if (id == LYMPH_GD_STAT) {
        r[0] = r[1] = r[2] = 2.0;
    } else {
        r[0] = r[1] = r[2] = 0.0;
    }
}

__device__ inline void dev_neumann(int id, double lam, double mu, const double n[3], const double p[3], int tag,
                                   double r[3]) {
    const double PI = 3.141592653589793;
    r[0] = r[1] = r[2] = 0.0;
    if (id != LYMPH_GN || !(tag == 1 || tag == 2 || tag == 3)) return;
    double s[3][3];
    const double d = -PI * sin(PI * p[0]) * sin(PI * p[1]) * sin(PI * p[2]) * (3.0 * lam + 2.0 * mu);
    s[0][0] = d; s[1][1] = d; s[2][2] = d;
    s[0][1] = 2.0 * mu * PI * cos(PI * p[0]) * cos(PI * p[1]) * sin(PI * p[2]); s[1][0] = s[0][1];
    s[0][2] = 2.0 * mu * PI * cos(PI * p[0]) * cos(PI * p[2]) * sin(PI * p[1]); s[2][0] = s[0][2];
    s[1][2] = 2.0 * mu * PI * cos(PI * p[1]) * cos(PI * p[2]) * sin(PI * p[0]); s[2][1] = s[1][2];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) r[i] = r[i] + s[i][j] * n[j];
}

__device__ inline void dev_analytic(int id, const double p[3], double r[3]) {
    const double PI = 3.141592653589793, SQ2 = 1.4142135623730951;
    if (id == LYMPH_FUN_IC_VELOCITY) {
        r[0] = SQ2 * PI * cos(PI * p[0]) * sin(PI * p[1]) * sin(PI * p[2]);
        r[1] = SQ2 * PI * sin(PI * p[0]) * cos(PI * p[1]) * sin(PI * p[2]);
        r[2] = SQ2 * PI * sin(PI * p[0]) * sin(PI * p[1]) * cos(PI * p[2]);
    } else if (id == LYMPH_FUN_UEX) {
        dev_u_space(p, r);
    } else {
        r[0] = r[1] = r[2] = 0.0;
    }
}

struct VecArgs {
    const int32_t* poly_ptr;
    const int32_t* poly_tets;
    const int32_t* tet_mat;
    const int32_t* neigh;
    const int32_t* fun_tag;
    const double* mat;
    const double* fk;
    const double* jdet;
    const double* nrm;
    const double* area;
    const double* bbox;
    const double* hk;
    const RefTables* ref;
    double alpha, theta;
    int mode;            // 0 = RHS (MAKE_RHS_FREE), 1 = L2 projection
    int fid, did, nid;   // data function ids
    const double* R;     // modal factor (projection only)
    const double* RT;
    double scale;
    double* out;         // [n_poly][ND]
};

constexpr int VEC_THREADS = 128;

// solve_LU(R^T, R, b) (vet_mat_operations.f90:123-153) in the reference's
// operation order, one lane: forward substitution y_i = (b_i - sum_{j<i}
// R(j,i) y_j) / R(i,i), then back substitution x_i = (y_i - sum_{j>i} R(i,j)
// x_j) / R(i,i), both sums in increasing j.  Used by the set-up projection,
// where the solve sees the full coefficient vector and its rounding matters
// most; O(Np^2) sequential work once per polyhedron.
__device__ inline void lane_solve_rtr(int NP, const double* __restrict__ R, double* b) {
    for (int i = 0; i < NP; ++i) {
        double y = b[i];
        for (int j = 0; j < i; ++j) y = y - R[j * NP + i] * b[j];
        b[i] = y / R[i * NP + i];
    }
    for (int i = NP - 1; i >= 0; --i) {
        double x = b[i];
        for (int j = i + 1; j < NP; ++j) x = x - R[i * NP + j] * b[j];
        b[i] = x / R[i * NP + i];
    }
}

// MAKE_RHS_FREE (matrix_free.f90:467-843) with MAKE_RHS_VOLUME / MAKE_RHS_FACE
// (assemble_element.f90:171-390), or COMPUTE_MODAL_COEFFICIENTS_FREE
// (matrix_free.f90:847-997): one CTA per polyhedron.
template <int PD>
__global__ void __launch_bounds__(VEC_THREADS) k_vector(VecArgs A) {
    using D = Deg<PD>;
    constexpr int NP = D::NP, ND = D::ND, NQ3 = D::NQ3, NQ2 = D::NQ2;
    extern __shared__ double vsm[];
    double* s_acc = vsm;                  // [ND]
    double* s_phi = s_acc + ND;           // [NQ3][NP]
    double* s_dphi = s_phi + NQ3 * NP;    // [NQ2][3][NP]
    double* s_dat = s_dphi + NQ2 * 3 * NP;// [NQ3][3]
    double* s_w = s_dat + NQ3 * 3;        // [NQ3]
    double* s_pt = s_w + NQ3;             // [NQ2][3]
    // 1-D factors of basis_eval (legendre_1d of each coordinate and degree):
    // volume [NQ3][3][L1] values, faces [NQ2][3][L1] (value, derivative)
    // pairs; the basis values are their products in basis_eval's order, so
    // they are the same bits at 3 (p+1) instead of 3 Np legendre_1d calls
    constexpr int L1 = PD + 1;
    static_assert(NQ3 >= 2 * NQ2, "the face table fits the volume table's space");
    double* s_tab = s_pt + NQ2 * 3;
    const int tid = threadIdx.x, P = blockIdx.x;
    const double* bb = &A.bbox[P * 6];
    for (int i = tid; i < ND; i += VEC_THREADS) s_acc[i] = 0.0;
    for (int kt = A.poly_ptr[P]; kt < A.poly_ptr[P + 1]; ++kt) {
        const int t = A.poly_tets[kt];
        const double* fk = &A.fk[t * 12];
        const int mid = A.tet_mat[t];
        const double rho = A.mat[mid * 3 + 0], lam = A.mat[mid * 3 + 1], mu = A.mat[mid * 3 + 2];
        const double aj = fabs(A.jdet[t]);
        __syncthreads();
        for (int it = tid; it < NQ3 * 3 * L1; it += VEC_THREADS) {
            const int q = it / (3 * L1), rr = it % (3 * L1), d = rr / L1, deg = rr % L1;
            double pt[3], v, dv;
            tet_point(fk, A.ref, q, pt);
            legendre_1d(pt[d], deg, bb[2 * d], bb[2 * d + 1], &v, &dv);
            s_tab[it] = v;
            if (rr == 0) {
                double r[3];
                if (A.mode == 0) dev_forcing(A.fid, lam, mu, pt, rho, r);
                else dev_analytic(A.fid, pt, r);
                s_dat[q * 3 + 0] = r[0]; s_dat[q * 3 + 1] = r[1]; s_dat[q * 3 + 2] = r[2];
                s_w[q] = aj * A.ref->weitet3[q];
            }
        }
        __syncthreads();
        for (int it = tid; it < NQ3 * NP; it += VEC_THREADS) {
            const int q = it / NP, f = it % NP;
            const int* bl = &A.ref->blist[f * 3];
            const double* tq = s_tab + q * 3 * L1;
            s_phi[q * NP + f] = tq[bl[0]] * tq[L1 + bl[1]] * tq[2 * L1 + bl[2]];
        }
        __syncthreads();
        for (int r = tid; r < ND; r += VEC_THREADS) {
            const int i = r / NP, m = r % NP;
            // RHS: per-tetrahedron integral added to the polyhedron's vector
            // (MAKE_RHS_VOLUME then the row copy, matrix_free.f90:711-717);
            // projection: one running integral over all sub-tetrahedra
            // (uex_integral, matrix_free.f90:960-972)
            double s = (A.mode == 0) ? 0.0 : s_acc[r];
            for (int q = 0; q < NQ3; ++q) s = s + s_w[q] * s_dat[q * 3 + i] * s_phi[q * NP + m];
            if (A.mode == 0) s_acc[r] += s;
            else s_acc[r] = s;
        }
        if (A.mode != 0) continue;
        // boundary faces of this tetrahedron (only boundary faces are added, :809-819)
        for (int f = 0; f < 4; ++f) {
            const int E2 = A.neigh[t * 4 + f];
            if (E2 != LYMPH_BC_DIRI && E2 != LYMPH_BC_NEUM) continue;
            const int tag = A.fun_tag ? A.fun_tag[t * 4 + f] : 1;
            const double nv[3] = {A.nrm[t * 12 + f * 3], A.nrm[t * 12 + f * 3 + 1], A.nrm[t * 12 + f * 3 + 2]};
            const double ar = A.area[t * 4 + f];
            __syncthreads();
            for (int q = tid; q < NQ2; q += VEC_THREADS) {
                face_point(fk, A.ref, f, q, &s_pt[q * 3]);
                // data points as MAKE_RHS_FACE forms them (assemble_element.f90:313-320)
                double pq[3];
                const double* nm = &A.ref->node_maps[f * 16];
                const double* nt = &A.ref->nodtria2[q * 4];
                for (int j = 0; j < 3; ++j) {
                    double s = 0.0;
                    for (int kk = 0; kk < 4; ++kk)
                        for (int tt = 0; tt < 4; ++tt) s = s + fk[j * 4 + kk] * nm[kk * 4 + tt] * nt[tt];
                    pq[j] = s;
                }
                double g[3];
                if (E2 == LYMPH_BC_DIRI) dev_dirichlet(A.did, pq, tag, g);
                else dev_neumann(A.nid, lam, mu, nv, pq, tag, g);
                s_dat[q * 3 + 0] = g[0]; s_dat[q * 3 + 1] = g[1]; s_dat[q * 3 + 2] = g[2];
            }
            __syncthreads();
            for (int it = tid; it < NQ2 * 3 * L1; it += VEC_THREADS) {
                const int q = it / (3 * L1), rr = it % (3 * L1), d = rr / L1, deg = rr % L1;
                legendre_1d(s_pt[q * 3 + d], deg, bb[2 * d], bb[2 * d + 1], &s_tab[2 * it], &s_tab[2 * it + 1]);
            }
            __syncthreads();
            for (int it = tid; it < NQ2 * NP; it += VEC_THREADS) {
                const int q = it / NP, fb = it % NP;
                const int* bl = &A.ref->blist[fb * 3];
                const double* tq = s_tab + 2 * q * 3 * L1;
                const double vx = tq[2 * bl[0]], dx = tq[2 * bl[0] + 1];
                const double vy = tq[2 * (L1 + bl[1])], dy = tq[2 * (L1 + bl[1]) + 1];
                const double vz = tq[2 * (2 * L1 + bl[2])], dz = tq[2 * (2 * L1 + bl[2]) + 1];
                s_phi[q * NP + fb] = vx * vy * vz;
                s_dphi[(q * 3 + 0) * NP + fb] = dx * vy * vz;
                s_dphi[(q * 3 + 1) * NP + fb] = vx * dy * vz;
                s_dphi[(q * 3 + 2) * NP + fb] = vx * vy * dz;
            }
            __syncthreads();
            const double sigma = A.alpha * (double)(PD * PD) / A.hk[P] * (lam + 2 * mu);
            const double n0 = nv[0], n1 = nv[1], n2 = nv[2];
            const double a0 = fabs(n0) * fabs(n0), a1 = fabs(n1) * fabs(n1), a2 = fabs(n2) * fabs(n2);
            for (int r = tid; r < ND; r += VEC_THREADS) {
                const int i = r / NP, m = r % NP;
                double rf = 0.0;
                for (int q = 0; q < NQ2; ++q) {
                    const double w = A.ref->weitria2[q];
                    const double* gd = &s_dat[q * 3];
                    const double ph = s_phi[q * NP + m];
                    if (E2 == LYMPH_BC_DIRI) {
                        const double g0 = s_dphi[(q * 3 + 0) * NP + m], g1 = s_dphi[(q * 3 + 1) * NP + m],
                                     g2 = s_dphi[(q * 3 + 2) * NP + m];
                        double tv, sv;
                        if (i == 0) {
                            tv = (lam + 2 * mu) * g0 * gd[0] * n0 + mu * g1 * gd[0] * n1 + mu * g2 * gd[0] * n2 +
                                 lam * g0 * gd[1] * n1 + mu * g1 * gd[1] * n0 + lam * g0 * gd[2] * n2 + mu * g2 * gd[2] * n0;
                            sv = ph * gd[0] * (a0 + 0.5 * a1 + 0.5 * a2) + 0.5 * ph * gd[1] * n0 * n1 + 0.5 * ph * gd[2] * n0 * n2;
                        } else if (i == 1) {
                            tv = (lam + 2 * mu) * g1 * gd[1] * n1 + mu * g0 * gd[1] * n0 + mu * g2 * gd[1] * n2 +
                                 lam * g1 * gd[0] * n0 + mu * g0 * gd[0] * n1 + lam * g1 * gd[2] * n2 + mu * g2 * gd[2] * n1;
                            sv = ph * gd[1] * (a1 + 0.5 * a0 + 0.5 * a2) + 0.5 * ph * gd[0] * n0 * n1 + 0.5 * ph * gd[2] * n1 * n2;
                        } else {
                            tv = (lam + 2 * mu) * g2 * gd[2] * n2 + mu * g0 * gd[2] * n0 + mu * g1 * gd[2] * n1 +
                                 lam * g2 * gd[0] * n0 + mu * g0 * gd[0] * n2 + lam * g2 * gd[1] * n1 + mu * g1 * gd[1] * n2;
                            sv = ph * gd[2] * (a2 + 0.5 * a0 + 0.5 * a1) + 0.5 * ph * gd[0] * n0 * n2 + 0.5 * ph * gd[1] * n1 * n2;
                        }
                        rf = rf + A.theta * w * tv * ar + sigma * w * sv * ar;
                    } else {
                        rf = rf + w * ph * gd[i] * ar;
                    }
                }
                if (rf != 0.0) s_acc[r] += rf;
            }
        }
    }
    __syncthreads();
    if (A.mode == 0) {
        for (int r = tid; r < ND; r += VEC_THREADS) A.out[(int64_t)P * ND + r] = s_acc[r];
        return;
    }
    // L2 projection: solve_LU(R^T, R) per component with the modal factor
    if (tid < 3) lane_solve_rtr(NP, A.R + (int64_t)P * NP * NP, &s_acc[tid * NP]);
    __syncthreads();
    for (int r = tid; r < ND; r += VEC_THREADS) A.out[(int64_t)P * ND + r] = s_acc[r] * A.scale;
}

// MAKE_DAMPING_FACE (assemble_element.f90:666-731) summed over the absorbing
// faces of each polyhedron that has some: one CTA per such polyhedron, the
// face's quadrature points and P's basis values in shared memory, each thread
// owning fixed entries of the ND x ND block D (row (i, m), column (j, n)):
//   D += |face| w_q (phi_m phi_n) C_ij,
//   C = c_t (t1 t1^T + t2 t2^T) + c_n n n^T = c_t (I - n n^T) + c_n n n^T,
// c_t = sqrt(rho mu), c_n = sqrt(rho (lambda + 2 mu)) of the face's
// tetrahedron.  phi_m phi_n is formed before the weight, so D is exactly
// symmetric.
template <int PD>
__global__ void __launch_bounds__(VEC_THREADS) k_damping(const int32_t* __restrict__ abs_poly,
                                                       const int32_t* __restrict__ abs_ptr,
                                                       const int32_t* __restrict__ abs_faces, const double* __restrict__ fk,
                                                       const double* __restrict__ nrm, const double* __restrict__ area,
                                                       const double* __restrict__ bbox, const int32_t* __restrict__ tet_mat,
                                                       const double* __restrict__ mat, const RefTables* __restrict__ ref,
                                                       double* __restrict__ D) {
    using Dg = Deg<PD>;
    constexpr int NP = Dg::NP, ND = Dg::ND, NQ2 = Dg::NQ2;
    __shared__ double s_phi[NQ2 * NP];
    __shared__ double s_pt[NQ2 * 3];
    const int a = blockIdx.x, tid = threadIdx.x, P = abs_poly[a];
    const double* bb = &bbox[P * 6];
    double* Da = D + (int64_t)a * ND * ND;
    for (int e = tid; e < ND * ND; e += VEC_THREADS) Da[e] = 0.0;
    for (int k = abs_ptr[a]; k < abs_ptr[a + 1]; ++k) {
        const int code = abs_faces[k], t = code >> 2, f = code & 3;
        __syncthreads();
        for (int q = tid; q < NQ2; q += VEC_THREADS) face_point(&fk[t * 12], ref, f, q, &s_pt[q * 3]);
        __syncthreads();
        for (int it = tid; it < NQ2 * NP; it += VEC_THREADS) {
            const int q = it / NP, fb = it % NP;
            double dp[3];
            basis_eval(&s_pt[q * 3], bb, &ref->blist[fb * 3], &s_phi[q * NP + fb], dp);
        }
        __syncthreads();
        const double* n = &nrm[t * 12 + f * 3];
        const int mid = tet_mat[t];
        const double rho = mat[mid * 3 + 0], lam = mat[mid * 3 + 1], mu = mat[mid * 3 + 2];
        const double ct = sqrt(rho * mu), cn = sqrt(rho * (lam + 2.0 * mu));
        const double ar = area[t * 4 + f];
        for (int e = tid; e < ND * ND; e += VEC_THREADS) {
            const int r = e / ND, cc = e - r * ND;
            const int i = r / NP, m = r - i * NP, j = cc / NP, nn = cc - j * NP;
            const double nij = n[i] * n[j];
            const double C = ct * ((i == j ? 1.0 : 0.0) - nij) + cn * nij;
            double s = 0.0;
            for (int q = 0; q < NQ2; ++q) s = s + ref->weitria2[q] * (s_phi[q * NP + m] * s_phi[q * NP + nn]);
            Da[e] += ar * C * s;
        }
    }
}

// W = M (x) I + dt/2 D for each polyhedron with absorbing faces (M: the
// rho-weighted mass matrix M_loc of the polyhedron, the same for each
// component).
__global__ void k_damping_w(int n_abs, int NP, const int32_t* __restrict__ abs_poly, const double* __restrict__ M,
                            const double* __restrict__ D, double half_dt, double* __restrict__ W) {
    const int ND = 3 * NP;
    const int64_t total = (int64_t)n_abs * ND * ND;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t a = e / ((int64_t)ND * ND);
        const int rc = (int)(e - a * ND * ND), r = rc / ND, cc = rc - r * ND;
        const int i = r / NP, m = r - i * NP, j = cc / NP, nn = cc - j * NP;
        const double mv = (i == j) ? M[(int64_t)abs_poly[a] * NP * NP + m * NP + nn] : 0.0;
        W[e] = mv + half_dt * D[e];
    }
}

// Point source: rhs[P][i*Np + m] = dir_i phi_m(x0) for the polyhedron P
// that contains x0 (one block of Np threads); the rest of rhs was zeroed by
// the caller.  The spatial part of a Ricker source f = dir delta(x - x0) R(t),
// whose time part R(t) enters through the time-function values.
__global__ void k_point_source(int Np, int P, const double* __restrict__ bbox, const RefTables* __restrict__ ref,
                               double x, double y, double z, double dx, double dy, double dz, double* rhs) {
    const int m = threadIdx.x;
    if (m >= Np) return;
    const double pt[3] = {x, y, z};
    double ph, dp[3];
    basis_eval(pt, &bbox[P * 6], &ref->blist[m * 3], &ph, dp);
    const int64_t base = (int64_t)P * 3 * Np;
    rhs[base + 0 * Np + m] = dx * ph;
    rhs[base + 1 * Np + m] = dy * ph;
    rhs[base + 2 * Np + m] = dz * ph;
}

// Double-couple source on tetrahedron t of polyhedron P (one block of Np
// threads, thread m): rhs[P][(i, m)] += sum_q w_q |J| sum_j moment(i, j)
// dphi_j(m, x_q), the body of MAKE_DOUBLE_COUPLE
// (assemble_element.f90:116-167) with the moment density
// (s n^T + n s^T) M0 / V of problem_data_and_properties.f90:317-335, in the
// reference's order (q outer, j inner).
__global__ void k_double_couple(int Np, int nq3, int t, int P, const double* __restrict__ fk,
                                const double* __restrict__ jdet, const double* __restrict__ bbox,
                                const RefTables* __restrict__ ref, const double* __restrict__ moment, double* rhs) {
    const int m = threadIdx.x;
    if (m >= Np) return;
    const double* F = fk + (int64_t)t * 12;
    const double aj = fabs(jdet[t]);
    double acc[3] = {0.0, 0.0, 0.0};
    for (int q = 0; q < nq3; ++q) {
        const double* nq = &ref->nodtet3[q * 4];
        double pt[3];
        for (int a = 0; a < 3; ++a) pt[a] = F[a * 4 + 0] * nq[0] + F[a * 4 + 1] * nq[1] + F[a * 4 + 2] * nq[2] + F[a * 4 + 3];
        double ph, dp[3];
        basis_eval(pt, &bbox[P * 6], &ref->blist[m * 3], &ph, dp);
        for (int i = 0; i < 3; ++i) {
            double reduct = 0.0;
            for (int j = 0; j < 3; ++j) reduct = reduct + moment[i * 3 + j] * dp[j];
            acc[i] = acc[i] + ref->weitet3[q] * aj * reduct;
        }
    }
    const int64_t base = (int64_t)P * 3 * Np;
    for (int i = 0; i < 3; ++i) rhs[base + i * Np + m] += acc[i];
}

template <int PD>
int launch_assemble(lymph_ctx* c, int which, void* out, int out_fp32, bool write_mass, const int64_t* list,
                    int64_t n_list, int64_t out_stride) {
    size_t smem = asm_smem<PD>();
    LYMPH_CUDA_TRY(cudaFuncSetAttribute(k_assemble<PD>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    AsmArgs A;
    A.blk_row = c->d_blk_row; A.col = c->d_col; A.bf_ptr = c->d_bf_ptr; A.bf = c->d_bf;
    A.poly_ptr = c->d_poly_ptr; A.poly_tets = c->d_poly_tets; A.tet_poly = c->d_tet_poly; A.tet_mat = c->d_tet_mat;
    A.neigh = c->d_neigh; A.mat = c->d_mat; A.fk = c->d_fk; A.jdet = c->d_jdet; A.nrm = c->d_normal; A.area = c->d_area;
    A.bbox = c->d_bbox; A.hk = c->d_hk; A.ref = c->d_ref; A.alpha = c->alpha; A.theta = c->theta;
    A.which = which; A.out_fp32 = out_fp32; A.out = out;
    A.M = write_mass ? c->d_M : nullptr; A.Mm = write_mass ? c->d_Mm : nullptr;
    A.list = list; A.out_stride = out_stride;
    const int64_t n = list ? n_list : c->n_blocks;
    const int64_t chunk = 1 << 20;
    for (int64_t b0 = 0; b0 < n; b0 += chunk) {
        A.block0 = b0;
        int64_t nb = n - b0 < chunk ? n - b0 : chunk;
        k_assemble<PD><<<(unsigned)nb, ASM_THREADS, smem, c->stream>>>(A);
        c->launches++;
        LYMPH_CUDA_TRY(cudaGetLastError());
    }
    return LYMPH_OK;
}

template <int PD>
int launch_vector(lymph_ctx* c, int mode, int fid, int did, int nid, double scale, double* out) {
    VecArgs A;
    A.poly_ptr = c->d_poly_ptr; A.poly_tets = c->d_poly_tets; A.tet_mat = c->d_tet_mat; A.neigh = c->d_neigh;
    A.fun_tag = c->d_fun_tag; A.mat = c->d_mat; A.fk = c->d_fk; A.jdet = c->d_jdet; A.nrm = c->d_normal;
    A.area = c->d_area; A.bbox = c->d_bbox; A.hk = c->d_hk; A.ref = c->d_ref; A.alpha = c->alpha; A.theta = c->theta;
    A.mode = mode; A.fid = fid; A.did = did; A.nid = nid; A.R = c->d_Rm; A.RT = c->d_RmT; A.scale = scale; A.out = out;
    using D = Deg<PD>;
    // + the 1-D factor table (NQ3 * 3 (p+1) >= NQ2 * 3 (p+1) * 2 doubles)
    size_t smem = sizeof(double) * ((size_t)D::ND + D::NQ3 * D::NP + D::NQ2 * 3 * D::NP + D::NQ3 * 3 + D::NQ3 + D::NQ2 * 3 +
                                    (size_t)D::NQ3 * 3 * (PD + 1));
    LYMPH_CUDA_TRY(cudaFuncSetAttribute(k_vector<PD>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_vector<PD><<<c->n_poly, VEC_THREADS, smem, c->stream>>>(A);
    c->launches++;
    LYMPH_CUDA_TRY(cudaGetLastError());
    return LYMPH_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
// host entry points used by abi.cu
// ---------------------------------------------------------------------------
int lymph_dev_geometry(lymph_ctx* c) {
    if (c->n_tet > 0) {
        k_geometry<<<(c->n_tet + 127) / 128, 128, 0, c->stream>>>(c->n_tet, c->d_coords, c->d_tet_vert, c->d_fk,
                                                                 c->d_jdet, c->d_normal, c->d_area, c->d_status);
        c->launches++;
        LYMPH_CUDA_TRY(cudaGetLastError());
    }
    if (c->n_poly > 0) {
        k_bbox<<<(c->n_poly + 127) / 128, 128, 0, c->stream>>>(c->n_poly, c->d_poly_ptr, c->d_poly_tets, c->d_tet_vert,
                                                              c->d_coords, c->d_bbox, c->d_hk);
        c->launches++;
        LYMPH_CUDA_TRY(cudaGetLastError());
    }
    return LYMPH_OK;
}

// Blocks list[0..n_list) (all blocks in order when list is null) into
// consecutive output slots out_stride elements apart.
int lymph_dev_assemble_list(lymph_ctx* c, int which, void* out, int out_fp32, bool write_mass, const int64_t* list,
                            int64_t n_list, int64_t out_stride) {
    switch (c->p) {
        case 1: return launch_assemble<1>(c, which, out, out_fp32, write_mass, list, n_list, out_stride);
        case 2: return launch_assemble<2>(c, which, out, out_fp32, write_mass, list, n_list, out_stride);
        case 3: return launch_assemble<3>(c, which, out, out_fp32, write_mass, list, n_list, out_stride);
        case 4: return launch_assemble<4>(c, which, out, out_fp32, write_mass, list, n_list, out_stride);
        default: lymph_set_error("degree not supported on the device"); return LYMPH_ERR_INVALID;
    }
}

// The rho-weighted and the plain mass matrix of every polyhedron (the
// self-block CTAs of k_assemble with the stiffness and face terms skipped:
// the same sums in the same order, so M and Mm have the bits a full assembly
// gives them).
int lymph_dev_mass(lymph_ctx* c, const int64_t* self_list) {
    return lymph_dev_assemble_list(c, ASM_MASS_ONLY, nullptr, 0, true, self_list, c->n_poly, 0);
}

int lymph_dev_assemble(lymph_ctx* c, int which, void* out, int out_fp32, bool write_mass) {
    return lymph_dev_assemble_list(c, which, out, out_fp32, write_mass, nullptr, 0, (int64_t)c->nd * c->nd);
}

int lymph_dev_cholesky(lymph_ctx* c) {
    const int warps_per_block = 4;
    size_t smem = sizeof(double) * warps_per_block * c->Np * c->Np;
    unsigned grid = (unsigned)((c->n_poly + warps_per_block - 1) / warps_per_block);
    k_cholesky<<<grid, 32 * warps_per_block, smem, c->stream>>>(c->n_poly, c->Np, c->d_M, c->d_R, c->d_RT, c->d_status);
    k_cholesky<<<grid, 32 * warps_per_block, smem, c->stream>>>(c->n_poly, c->Np, c->d_Mm, c->d_Rm, c->d_RmT, c->d_status);
    k_mass_inverse<<<grid, 32 * warps_per_block, 0, c->stream>>>(c->n_poly, c->Np, c->d_R, c->d_Minv);
    c->launches += 3;
    LYMPH_CUDA_TRY(cudaGetLastError());
    return LYMPH_OK;
}

// The damping blocks of the absorbing faces (once per assembly) and the
// inverses of M (x) I + dt/2 D for the context's dt: W, its Cholesky factor
// (cholesky, one warp per polyhedron) and the explicit column-major inverse
// (solve_LU per column), as for the mass matrix.
int lymph_dev_damping(lymph_ctx* c, bool assemble) {
    if (c->n_abs <= 0) return LYMPH_OK;
    const int ND = c->nd;
    if (assemble) {
        switch (c->p) {
            case 1: k_damping<1><<<c->n_abs, VEC_THREADS, 0, c->stream>>>(c->d_abs_poly, c->d_abs_ptr, c->d_abs_faces, c->d_fk, c->d_normal, c->d_area, c->d_bbox, c->d_tet_mat, c->d_mat, c->d_ref, c->d_Dabs); break;
            case 2: k_damping<2><<<c->n_abs, VEC_THREADS, 0, c->stream>>>(c->d_abs_poly, c->d_abs_ptr, c->d_abs_faces, c->d_fk, c->d_normal, c->d_area, c->d_bbox, c->d_tet_mat, c->d_mat, c->d_ref, c->d_Dabs); break;
            case 3: k_damping<3><<<c->n_abs, VEC_THREADS, 0, c->stream>>>(c->d_abs_poly, c->d_abs_ptr, c->d_abs_faces, c->d_fk, c->d_normal, c->d_area, c->d_bbox, c->d_tet_mat, c->d_mat, c->d_ref, c->d_Dabs); break;
            case 4: k_damping<4><<<c->n_abs, VEC_THREADS, 0, c->stream>>>(c->d_abs_poly, c->d_abs_ptr, c->d_abs_faces, c->d_fk, c->d_normal, c->d_area, c->d_bbox, c->d_tet_mat, c->d_mat, c->d_ref, c->d_Dabs); break;
            default: lymph_set_error("degree not supported on the device"); return LYMPH_ERR_INVALID;
        }
        c->launches++;
        LYMPH_CUDA_TRY(cudaGetLastError());
    }
    const int64_t total = (int64_t)c->n_abs * ND * ND;
    const unsigned gw = (unsigned)((total + 255) / 256 < 4096 ? (total + 255) / 256 : 4096);
    k_damping_w<<<gw, 256, 0, c->stream>>>(c->n_abs, c->Np, c->d_abs_poly, c->d_M, c->d_Dabs, 0.5 * c->dt, c->d_Wabs);
    const size_t smem = sizeof(double) * (size_t)ND * ND;  // one warp per block: its ND x ND factor
    // raise (never lower) k_cholesky's dynamic shared-memory limit: the mass
    // factorisation launches it with up to 4 Np^2 doubles per block
    const size_t lim = smem > (size_t)48 * 1024 ? smem : (size_t)48 * 1024;
    LYMPH_CUDA_TRY(cudaFuncSetAttribute(k_cholesky, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lim));
    k_cholesky<<<c->n_abs, 32, smem, c->stream>>>(c->n_abs, ND, c->d_Wabs, c->d_Rw, c->d_RwT, c->d_status);
    k_mass_inverse<<<(unsigned)((c->n_abs + 3) / 4), 128, 0, c->stream>>>(c->n_abs, ND, c->d_Rw, c->d_Winv);
    c->launches += 3;
    c->winv_dt = c->dt;
    LYMPH_CUDA_TRY(cudaGetLastError());
    return LYMPH_OK;
}

int lymph_dev_point_source(lymph_ctx* c, int P, const double x0[3], const double dir[3], double* out) {
    LYMPH_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(double) * (size_t)c->n_poly * c->nd, c->stream));
    k_point_source<<<1, 64, 0, c->stream>>>(c->Np, P, c->d_bbox, c->d_ref, x0[0], x0[1], x0[2], dir[0], dir[1], dir[2], out);
    c->launches++;
    LYMPH_CUDA_TRY(cudaGetLastError());
    return LYMPH_OK;
}

int lymph_dev_double_couple(lymph_ctx* c, int t, int P, const double moment[9], double* out) {
    double* d_m = nullptr;
    LYMPH_CUDA_TRY(cudaMalloc(&d_m, sizeof(double) * 9));
    cudaError_t e = cudaMemcpyAsync(d_m, moment, sizeof(double) * 9, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) {
        k_double_couple<<<1, 64, 0, c->stream>>>(c->Np, c->nq3, t, P, c->d_fk, c->d_jdet, c->d_bbox, c->d_ref, d_m, out);
        c->launches++;
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cudaFree(d_m);
    if (e != cudaSuccess) {
        lymph_set_error(std::string("lymph_dev_double_couple: ") + cudaGetErrorString(e));
        return LYMPH_ERR_CUDA;
    }
    return LYMPH_OK;
}

int lymph_dev_vector(lymph_ctx* c, int mode, int fid, int did, int nid, double scale, double* out) {
    switch (c->p) {
        case 1: return launch_vector<1>(c, mode, fid, did, nid, scale, out);
        case 2: return launch_vector<2>(c, mode, fid, did, nid, scale, out);
        case 3: return launch_vector<3>(c, mode, fid, did, nid, scale, out);
        case 4: return launch_vector<4>(c, mode, fid, did, nid, scale, out);
        default: lymph_set_error("degree not supported on the device"); return LYMPH_ERR_INVALID;
    }
}
