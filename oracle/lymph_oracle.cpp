// lymph_oracle.cpp -- CPU FP64 restatement of the LYMPH3D matrix-free PolyDG
// elastodynamics path (src/matrix_free.f90 and the element routines it calls).
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker the GPU library is
// compared against: only tests/, __graft_entry__.smoke() and bench.py's CPU
// baseline arm load it.  The product library never links or calls it.
//
// Parity status: UNPINNED against the reference's own numbers.  The reference
// is Fortran 90 + MPI; no Fortran compiler exists where this project is built
// or run, and the reference ships no golden vectors.  This restatement follows
// the reference's loops, formulas and evaluation order line by line (each
// function cites the file:line it restates) and is pinned instead by
// known-answer tests of the mathematics (quadrature sums, Legendre
// orthogonality, SPD mass matrices, rigid-body modes, symmetry, convergence
// rates) in tests/.
//
// Generalisation: the reference's matrix-free path indexes every array by
// tetrahedron, which is only consistent when each polyhedron is one
// tetrahedron ("mode A").  Here every per-element quantity is accumulated per
// polyhedron over its sub-tetrahedra ("mode B"); face terms are kept only on
// faces between different polyhedra or on the boundary, the face_flag rule of
// src/matrix_free.f90:290-309.  With one tetrahedron per polyhedron this is the
// reference's algorithm exactly.
//
// Build: oracle/Makefile (g++ -O2 -ffp-contract=off -fopenmp, same results on
// x86-64 and aarch64).

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>
#include <algorithm>
#include <array>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/lymph3d_gpu.h"  // lymph_mesh_desc (plain data layout only)

namespace {

const double PI = 4.0 * std::atan(1.0);        // Poly_global.f90:417
const double SQRT2 = std::sqrt(2.0);           // Poly_global.f90:416
const int BC_DIRI = -1, BC_NEUM = -2, BC_ABSO = -3;  // Poly_global.f90:420-422

thread_local std::string g_err;

// Noise-floor instrument for the tests: when non-zero, every value a data
// function returns is moved by +-g_perturb_ulps units in the last place, the
// sign drawn from a hash of the evaluation point.  It models the 1-2 ulp
// differences between two libm implementations of sin/cos.
int g_perturb_ulps = 0;

// Second instrument: when set, the operator apply of the time steps sums the
// blocks of a row and the entries of every row dot product in reverse order,
// with fused multiply-adds.
// The spread between the two orders is the algorithm's own rounding floor.
int g_reverse_sums = 0;

// Third instrument (0 = off, else the number of column slices S the CUDA step
// kernel uses at this degree): the operator apply, right-hand side, M^-1
// product and update in the CUDA step kernel's order -- row r summed as S
// column slices (columns s, s+S, ...) with two fused-multiply-add
// accumulators each (even and odd j), over the blocks in stored order, the
// slices added in order; M^-1 with two accumulators (even and odd columns);
// the contractions a*b + c of those expressions as fused multiply-adds.
int g_device_order = 0;

// Third instrument: when set, the time steps apply M^-1 as an explicit
// inverse (columns solved once with solve_LU) instead of the two triangular
// solves, the way the device kernel applies it.
int g_explicit_inverse = 0;

// Planted mistakes, for the tests that show a parity bar catches them (0 =
// none).  Only the point-by-point neighbour product (neighbour_apply_rule)
// reads it: 1 drops the penalty term, 2 flips the sign of the symmetry term,
// 3 drops the consistency term, 4 drops the last shared triangle of the pair.
int g_planted_mistake = 0;

// When 0, MAKE_MATRICES_FREE skips the A_dg blocks (the DG-norm operator): the
// timed CPU runs of the benchmark need only K, and at 46,767 polyhedra and
// p = 4 each operator holds 44 GB.  COMPUTE_ERROR_DG then reports an error.
int g_assemble_dg = 1;

double perturb(double v, const double p[3], int comp) {
    if (g_perturb_ulps == 0 || v == 0.0) return v;
    uint64_t h = 1469598103934665603ull ^ (uint64_t)comp;
    for (int k = 0; k < 3; ++k) {
        uint64_t b;
        std::memcpy(&b, &p[k], 8);
        h = (h ^ b) * 1099511628211ull;
    }
    double dir = (h >> 63) ? 1e308 : -1e308;
    for (int k = 0; k < g_perturb_ulps; ++k) v = std::nextafter(v, dir);
    return v;
}

void perturb3(double r[3], const double p[3]) {
    for (int i = 0; i < 3; ++i) r[i] = perturb(r[i], p, i);
}

// ---------------------------------------------------------------------------
// vet_mat_operations.f90
// ---------------------------------------------------------------------------

// det3, vet_mat_operations.f90:38-49 (A(i,j) stored a[i][j]).
double det3(const double a[3][3]) {
    return a[0][0] * a[1][1] * a[2][2] - a[0][0] * a[1][2] * a[2][1]
         - a[0][1] * a[1][0] * a[2][2] + a[0][1] * a[1][2] * a[2][0]
         + a[0][2] * a[1][0] * a[2][1] - a[1][1] * a[0][2] * a[2][0];
}

// cholesky, vet_mat_operations.f90:84-120: A = R^T R, R upper triangular.
// a, r are dim x dim, r(i,j) stored r[i*dim+j].  Returns false where the
// reference prints "Matrix is not positive definite!" and stops.
bool cholesky(const double* a, int dim, double* r) {
    for (int i = 0; i < dim * dim; ++i) r[i] = 0.0;
    for (int j = 0; j < dim; ++j) {
        double sum = a[j * dim + j];
        for (int k = 0; k < j; ++k) sum = sum - r[k * dim + j] * r[k * dim + j];
        if (sum <= 0.0) return false;
        r[j * dim + j] = std::sqrt(sum);
        for (int i = j + 1; i < dim; ++i) {
            sum = a[j * dim + i];
            for (int k = 0; k < j; ++k) sum = sum - r[k * dim + j] * r[k * dim + i];
            r[j * dim + i] = sum / r[j * dim + j];
        }
    }
    return true;
}

// solve_LU(R^T, R, b), vet_mat_operations.f90:123-153 with L = R^T:
// forward substitution L y = b, then back substitution R x = y.
void solve_LU_RT_R(const double* r, const double* b, int dim, double* x) {
    std::vector<double> y(dim);
    // L(i,j) = R(j,i)
    y[0] = b[0] / r[0];
    for (int i = 1; i < dim; ++i) {
        y[i] = b[i];
        for (int j = 0; j < i; ++j) y[i] = y[i] - r[j * dim + i] * y[j];
        y[i] = y[i] / r[i * dim + i];
    }
    x[dim - 1] = y[dim - 1] / r[(dim - 1) * dim + dim - 1];
    for (int i = dim - 2; i >= 0; --i) {
        x[i] = y[i];
        for (int j = i + 1; j < dim; ++j) x[i] = x[i] - r[i * dim + j] * x[j];
        x[i] = x[i] / r[i * dim + i];
    }
}

// ---------------------------------------------------------------------------
// basis_function.f90
// ---------------------------------------------------------------------------

// basis_list, basis_function.f90:12-44: monomial degree triples of total
// degree exactly p... (q1 from p down to 0, q2 from p-q1 down to 0, q3 from
// p-q1-q2 down to 0): all triples with q1+q2+q3 <= p.
void basis_list(int p, int Np, int* blist) {
    int ii = 0;
    for (int q1 = p; q1 >= 0; --q1)
        for (int q2 = p - q1; q2 >= 0; --q2)
            for (int q3 = p - q1 - q2; q3 >= 0; --q3) {
                if (ii < Np) { blist[ii * 3 + 0] = q1; blist[ii * 3 + 1] = q2; blist[ii * 3 + 2] = q3; }
                ++ii;
            }
}

// GauLeg, basis_function.f90:164-265: Newton iteration on the Legendre
// recurrence for n Gauss-Legendre nodes on (a,b); nodes come out in the
// reference's order (descending positive half, then the reflected half).
void gauleg(int a, int b, int n, double* x_gl, double* w_gl) {
    int m = (n % 2 == 0) ? (n + 1) / 2 + 1 : (n + 1) / 2;
    std::vector<double> z(m), z_old(m), errv(m), p_app(m), flip_z(m), flip_p(m);
    std::vector<double> p1(m), p2(m), p3(m);
    for (int j = 1; j <= m; ++j) z[j - 1] = std::cos(PI * ((j - 0.25) / (n + 0.5)));
    const double eps = 2.220446049250313e-16;  // epsilon(1.0d0)
    double err = eps + 1.0;
    for (int i = 0; i < m; ++i) errv[i] = err * 1.0;
    while (err > eps) {
        for (int i = 0; i < m; ++i) { p1[i] = 1.0; p2[i] = 0.0; p3[i] = 0.0; }
        for (int j = 1; j <= n; ++j) {
            for (int i = 0; i < m; ++i) {
                p3[i] = p2[i]; p2[i] = p1[i];
                p1[i] = ((2.0 * j - 1.0) / j) * z[i] * p2[i] - ((j - 1.0) / j) * p3[i];
            }
        }
        for (int i = 0; i < m; ++i) {
            p_app[i] = n * (z[i] * p1[i] - p2[i]) / (z[i] * z[i] - 1.0);
            z_old[i] = z[i];
            z[i] = z_old[i] - ((errv[i] > eps) ? (p1[i] / p_app[i]) : 0.0);
        }
        err = 0.0;
        for (int i = 0; i < m; ++i) { errv[i] = std::fabs(z[i] - z_old[i]); err = std::max(err, errv[i]); }
    }
    for (int i = 0; i < m; ++i) { flip_z[i] = z[m - 1 - i]; flip_p[i] = p_app[m - 1 - i]; }
    std::vector<double> zz, pp;
    for (int i = 0; i < m - 1; ++i) { zz.push_back(z[i]); pp.push_back(p_app[i]); }
    int start = (n % 2 == 0) ? 1 : 0;
    for (int i = start; i < m; ++i) { zz.push_back(-flip_z[i]); pp.push_back(flip_p[i]); }
    // x = (b+a)/2 - (b-a)/2 * [z(1:m-1), -flip_z(...)]
    for (int i = 0; i < n; ++i) x_gl[i] = ((b + a) / 2.0) - ((b - a) / 2.0) * zz[i];
    // z reflected WITHOUT the sign flip for the weights (basis_function.f90:243-252)
    for (int i = 0; i < n; ++i) {
        double zr = (i < m - 1) ? z[i] : flip_z[i - (m - 1) + start];
        w_gl[i] = (b - a) / ((1.0 - zr * zr) * (pp[i] * pp[i]));
    }
}

// 1D Gauss-Legendre nodes/weights hard-coded up to 7 nodes,
// basis_function.f90:77-124, GauLeg beyond.
void gl1d(int nqn, std::vector<double>& nod1, std::vector<double>& wei1) {
    nod1.assign(nqn, 0.0); wei1.assign(nqn, 0.0);
    if (nqn == 1) { nod1 = {0.0}; wei1 = {2.0}; }
    if (nqn == 2) { nod1 = {std::sqrt(1.0 / 3.0), -std::sqrt(1.0 / 3.0)}; wei1 = {1.0, 1.0}; }
    if (nqn == 3) { nod1 = {0.0, std::sqrt(3.0 / 5.0), -std::sqrt(3.0 / 5.0)}; wei1 = {8.0 / 9.0, 5.0 / 9.0, 5.0 / 9.0}; }
    if (nqn == 4) {
        nod1 = {0.3399810435848563, -0.3399810435848563, 0.8611363115940526, -0.8611363115940526};
        double s = std::sqrt(30.0);
        wei1 = {(18 + s) / 36.0, (18 + s) / 36.0, (18 - s) / 36.0, (18 - s) / 36.0};
    }
    if (nqn == 5) {
        nod1 = {0.0, 0.5384693101056831, -0.5384693101056831, 0.9061798459386640, -0.9061798459386640};
        double s = std::sqrt(70.0);
        wei1 = {128.0 / 225.0, (322 + 13 * s) / 900.0, (322 + 13 * s) / 900.0, (322 - 13 * s) / 900.0, (322 - 13 * s) / 900.0};
    }
    if (nqn == 6) {
        nod1 = {0.6612093864662645, -0.6612093864662645, 0.2386191860831969, -0.2386191860831969,
                0.9324695142031521, -0.9324695142031521};
        wei1 = {0.3607615730481386, 0.3607615730481386, 0.4679139345726910, 0.4679139345726910,
                0.1713244923791704, 0.1713244923791704};
    }
    if (nqn == 7) {
        nod1 = {0.0, 0.4058451513773972, -0.4058451513773972, 0.7415311855993945, -0.7415311855993945,
                0.9491079123427585, -0.9491079123427585};
        wei1 = {0.4179591836734694, 0.3818300505051189, 0.3818300505051189, 0.2797053914892766,
                0.2797053914892766, 0.1294849661688697, 0.1294849661688697};
    }
    if (nqn > 7) gauleg(-1, 1, nqn, nod1.data(), wei1.data());
}

struct Quadrature {
    int nq3 = 0, nq2 = 0;
    std::vector<double> nodtet3;   // [nq3][4]  (reference nodtet3(4,nq3))
    std::vector<double> weitet3;   // [nq3]
    std::vector<double> nodtria2;  // [nq2][4]  (reference nodtria2(4,nq2))
    std::vector<double> weitria2;  // [nq2]
};

// quadrature (basis_function.f90:47-161) followed by mapping_quadrature_3D /
// mapping_quadrature_2D (Poly_ref_mappings.f90:137-186).
Quadrature make_quadrature(int p) {
    Quadrature Q;
    int nqn = p + 1;
    Q.nq3 = nqn * nqn * nqn;
    Q.nq2 = nqn * nqn;
    std::vector<double> nod1, wei1;
    gl1d(nqn, nod1, wei1);
    std::vector<double> nod2(4 * Q.nq2), wei2(Q.nq2), nod3(4 * Q.nq3), wei3(Q.nq3);
    int c = 0;
    for (int i = 0; i < nqn; ++i)
        for (int j = 0; j < nqn; ++j) {
            nod2[c * 4 + 0] = nod1[i]; nod2[c * 4 + 1] = nod1[j]; wei2[c] = wei1[i] * wei1[j]; ++c;
        }
    c = 0;
    for (int i = 0; i < nqn; ++i)
        for (int j = 0; j < nqn; ++j)
            for (int k = 0; k < nqn; ++k) {
                nod3[c * 4 + 0] = nod1[i]; nod3[c * 4 + 1] = nod1[j]; nod3[c * 4 + 2] = nod1[k];
                wei3[c] = wei1[i] * wei1[j] * wei1[k]; ++c;
            }
    for (int q = 0; q < Q.nq2; ++q) { nod2[q * 4 + 2] = 1.0; nod2[q * 4 + 3] = 1.0; }
    for (int q = 0; q < Q.nq3; ++q) nod3[q * 4 + 3] = 1.0;
    // mapping_quadrature_3D: Duffy collapse of (0,1)^3 onto the reference tet.
    Q.nodtet3.assign(4 * Q.nq3, 0.0); Q.weitet3.assign(Q.nq3, 0.0);
    for (int q = 0; q < Q.nq3; ++q) {
        double a = 0.5 * nod3[q * 4 + 0] + 0.5, b = 0.5 * nod3[q * 4 + 1] + 0.5, cc = 0.5 * nod3[q * 4 + 2] + 0.5;
        double w = 0.125 * wei3[q];
        Q.nodtet3[q * 4 + 0] = a;
        Q.nodtet3[q * 4 + 1] = (1 - a) * b;
        Q.nodtet3[q * 4 + 2] = (1 - a) * (1 - b) * cc;
        Q.nodtet3[q * 4 + 3] = nod3[q * 4 + 3];
        double jd = (1 - b) * ((1 - a) * (1 - a));
        Q.weitet3[q] = std::fabs(jd) * w;
    }
    // mapping_quadrature_2D: square onto the reference triangle.
    Q.nodtria2.assign(4 * Q.nq2, 0.0); Q.weitria2.assign(Q.nq2, 0.0);
    for (int q = 0; q < Q.nq2; ++q) {
        double s = nod2[q * 4 + 0], t = nod2[q * 4 + 1];
        Q.nodtria2[q * 4 + 0] = 0.5 * (1 + s);
        Q.nodtria2[q * 4 + 1] = 0.25 * (1 - s) * (1 + t);
        Q.nodtria2[q * 4 + 2] = nod2[q * 4 + 2];
        Q.nodtria2[q * 4 + 3] = nod2[q * 4 + 3];
        double jd = 0.125 * (1 - s);
        Q.weitria2[q] = std::fabs(jd) * wei2[q];
    }
    return Q;
}

// tria2tetfaces_maps, Poly_ref_mappings.f90:79-134.  nm[k][i][j] is the
// reference's node_maps(i+1, j+1, k+1): maps (s, t, 1, 1) to (xi, eta, zeta, 1)
// on face k of the reference tetrahedron.
void tria2tetfaces_maps(double nm[4][4][4]) {
    std::memset(nm, 0, sizeof(double) * 64);
    nm[0][0][1] = 1.0; nm[0][1][0] = 1.0; nm[0][3][3] = 1.0;
    nm[1][0][0] = 1.0; nm[1][2][1] = 1.0; nm[1][3][3] = 1.0;
    nm[2][0][0] = 1.0; nm[2][1][1] = 1.0; nm[2][2][2] = 1.0; nm[2][3][3] = 1.0;
    nm[2][2][0] = -1.0; nm[2][2][1] = -1.0;
    nm[3][1][1] = 1.0; nm[3][2][0] = 1.0; nm[3][3][3] = 1.0;
}

// jacobians, Poly_ref_mappings.f90:18-75: Fk = [x2-x1, x3-x1, x4-x1 | x1].
void jacobians(const double x[4], const double y[4], const double z[4], double fk[3][4], double* jdet) {
    double mat[4][4];
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) {
            mat[i][j] = 0;
            if (j == 0) mat[i][j] = (i == 3) ? 1 : -1;
            if (j > 0 && j == i + 1) mat[i][j] = 1;
        }
    for (int j = 0; j < 4; ++j) {
        fk[0][j] = 0.0; fk[1][j] = 0.0; fk[2][j] = 0.0;
        for (int l = 0; l < 4; ++l) {
            fk[0][j] = fk[0][j] + mat[j][l] * x[l];
            fk[1][j] = fk[1][j] + mat[j][l] * y[l];
            fk[2][j] = fk[2][j] + mat[j][l] * z[l];
        }
    }
    double jac[3][3];
    for (int j = 0; j < 3; ++j)
        for (int l = 0; l < 3; ++l) jac[j][l] = fk[j][l];
    *jdet = det3(jac);
}

// LegendreP_nonnorm, basis_function.f90:268-339 (one point).
double legendre_nonnorm(double x, int p, double a, double b) {
    double hb = (b - a) / 2.0, mb = (b + a) / 2.0;
    double xp = (x - mb) / hb;
    double x2 = xp * xp, x3 = x2 * xp, x4 = x2 * x2, x5 = x4 * xp, x6 = x3 * x3, x7 = x6 * xp;
    switch (p) {
        case 0: return 1.0;
        case 1: return xp;
        case 2: return (3 * x2 - 1) / 2;
        case 3: return (5 * x3 - 3 * xp) / 2;
        case 4: return (35 * x4 - 30 * x2 + 3) / 8;
        case 5: return (63 * x5 - 70 * x3 + 15 * xp) / 8;
        case 6: return (231 * x6 - 315 * x4 + 105 * x2 - 5) / 16;
        case 7: return (429 * x7 - 693 * x5 + 315 * x3 - 35 * xp) / 16;
        default: break;
    }
    double lp_old = (429 * x7 - 693 * x5 + 315 * x3 - 35 * xp) / 16;
    double lp_oold = (231 * x6 - 315 * x4 + 105 * x2 - 5) / 16;
    double lp = 0.0;
    for (int ii = 7; ii <= p - 1; ++ii) {
        lp = 1.0 / (ii + 1.0) * ((2 * ii + 1) * xp * lp_old - ii * lp_oold);
        lp_oold = lp_old; lp_old = lp;
    }
    return lp;
}

// LegendreP, basis_function.f90:343-366: L_p / sqrt(hb).
double legendre(double x, int p, double a, double b) {
    double hb = (b - a) / 2.0;
    return legendre_nonnorm(x, p, a, b) / std::sqrt(hb);
}

// GradLegendreP, basis_function.f90:370-437: L'_p / (hb sqrt(hb)).
double grad_legendre(double x, int p, double a, double b) {
    double hb = (b - a) / 2.0, mb = (b + a) / 2.0;
    double xp = (x - mb) / hb;
    double x2 = xp * xp, x3 = x2 * xp, x4 = x2 * x2, x5 = x4 * xp, x6 = x3 * x3;
    double d = 0.0;
    switch (p) {
        case 0: d = 0.0; break;
        case 1: d = 1.0; break;
        case 2: d = 3 * xp; break;
        case 3: d = (15 * x2 - 3) / 2; break;
        case 4: d = (35 * x3 - 15 * xp) / 2; break;
        case 5: d = (315 * x4 - 210 * x2 + 15) / 8; break;
        case 6: d = (1386 * x5 - 1260 * x3 + 210 * xp - 5) / 16; break;
        case 7: d = (3003 * x6 - 3465 * x4 + 945 * x2 - 35) / 16; break;
        default: {
            for (int ii = p - 1; ii >= 0; ii -= 2) d = d + (2 * ii + 1) * legendre_nonnorm(x, ii, a, b);
        }
    }
    return d / (hb * std::sqrt(hb));
}

// Evaluation of the Np basis functions and gradients at one physical point
// with bounding box bb[3][2]; the body of the f-loop of basis
// (basis_function.f90:494-515) and basis_boundary (:586-646).
void eval_basis_point(const double pt[3], const double bb[3][2], int Np, const int* blist,
                      double* phi, double* dphi /*[3][Np]*/) {
    for (int f = 0; f < Np; ++f) {
        double vx = legendre(pt[0], blist[f * 3 + 0], bb[0][0], bb[0][1]);
        double dvx = grad_legendre(pt[0], blist[f * 3 + 0], bb[0][0], bb[0][1]);
        double vy = legendre(pt[1], blist[f * 3 + 1], bb[1][0], bb[1][1]);
        double dvy = grad_legendre(pt[1], blist[f * 3 + 1], bb[1][0], bb[1][1]);
        double vz = legendre(pt[2], blist[f * 3 + 2], bb[2][0], bb[2][1]);
        double dvz = grad_legendre(pt[2], blist[f * 3 + 2], bb[2][0], bb[2][1]);
        phi[f] = vx * vy * vz;
        dphi[0 * Np + f] = dvx * vy * vz;
        dphi[1 * Np + f] = vx * dvy * vz;
        dphi[2 * Np + f] = vx * vy * dvz;
    }
}

// ---------------------------------------------------------------------------
// problem_data_and_properties.f90 data functions
// ---------------------------------------------------------------------------
double time_function(double t) { return std::sin(SQRT2 * PI * t); }  // :14-23

void f_forcing(int id, double lambda, double mu, const double p[3], double rho, double r[3]) {
    if (id == LYMPH_F_TIME) {  // f_time :48-70
        double c = (-2.0 * rho + 3.0 * (lambda + 2.0 * mu)) * PI * PI;
        r[0] = c * std::cos(PI * p[0]) * std::sin(PI * p[1]) * std::sin(PI * p[2]);
        r[1] = c * std::sin(PI * p[0]) * std::cos(PI * p[1]) * std::sin(PI * p[2]);
        r[2] = c * std::sin(PI * p[0]) * std::sin(PI * p[1]) * std::cos(PI * p[2]);
    } else if (id == LYMPH_F_STAT) {  // f :26-45
        r[0] = 3 * PI * PI * std::cos(PI * p[0]) * std::sin(PI * p[1]) * std::sin(PI * p[2]) * (lambda + 2 * mu);
        r[1] = 3 * PI * PI * std::cos(PI * p[1]) * std::sin(PI * p[0]) * std::sin(PI * p[2]) * (lambda + 2 * mu);
        r[2] = 3 * PI * PI * std::cos(PI * p[2]) * std::sin(PI * p[0]) * std::sin(PI * p[1]) * (lambda + 2 * mu);
    } else {  // f_null :72-82
        r[0] = r[1] = r[2] = 0.0;
    }
    perturb3(r, p);
}

void u_space(const double p[3], double r[3]) {  // uex :245-254
    r[0] = std::cos(PI * p[0]) * std::sin(PI * p[1]) * std::sin(PI * p[2]);
    r[1] = std::sin(PI * p[0]) * std::cos(PI * p[1]) * std::sin(PI * p[2]);
    r[2] = std::sin(PI * p[0]) * std::sin(PI * p[1]) * std::cos(PI * p[2]);
}

void g_dirichlet(int id, const double p[3], int tag, double r[3]) {
    if (id == LYMPH_GD) {  // gd :130-154 (tags 1..3 share one formula)
        if (tag == 1 || tag == 2 || tag == 3) u_space(p, r);
        else r[0] = r[1] = r[2] = 0.0;
    } else if (id == LYMPH_GD_STAT) {  // gd_stat :106-114
        r[0] = r[1] = r[2] = 2.0;
    } else {
        r[0] = r[1] = r[2] = 0.0;
    }
    perturb3(r, p);
}

void g_neumann(int id, double lambda, double mu, const double n[3], const double p[3], int tag, double r[3]) {
    r[0] = r[1] = r[2] = 0.0;
    if (id != LYMPH_GN) return;  // gn_null / gn_stat return 0
    if (!(tag == 1 || tag == 2 || tag == 3)) return;
    double s[3][3];  // gn :186-242
    double d = -PI * std::sin(PI * p[0]) * std::sin(PI * p[1]) * std::sin(PI * p[2]) * (3.0 * lambda + 2.0 * mu);
    s[0][0] = d; s[1][1] = d; s[2][2] = d;
    s[0][1] = 2.0 * mu * PI * std::cos(PI * p[0]) * std::cos(PI * p[1]) * std::sin(PI * p[2]); s[1][0] = s[0][1];
    s[0][2] = 2.0 * mu * PI * std::cos(PI * p[0]) * std::cos(PI * p[2]) * std::sin(PI * p[1]); s[2][0] = s[0][2];
    s[1][2] = 2.0 * mu * PI * std::cos(PI * p[1]) * std::cos(PI * p[2]) * std::sin(PI * p[0]); s[2][1] = s[1][2];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) r[i] = r[i] + s[i][j] * n[j];
    perturb3(r, p);
}

void f_analytic(int id, const double p[3], double r[3]) {
    if (id == LYMPH_FUN_IC_VELOCITY) {  // ic_velocity :292-301
        r[0] = SQRT2 * PI * std::cos(PI * p[0]) * std::sin(PI * p[1]) * std::sin(PI * p[2]);
        r[1] = SQRT2 * PI * std::sin(PI * p[0]) * std::cos(PI * p[1]) * std::sin(PI * p[2]);
        r[2] = SQRT2 * PI * std::sin(PI * p[0]) * std::sin(PI * p[1]) * std::cos(PI * p[2]);
    } else if (id == LYMPH_FUN_UEX) {
        u_space(p, r);
    } else {  // ic_displacement, uex_stat: zero
        r[0] = r[1] = r[2] = 0.0;
    }
    perturb3(r, p);
}

// ---------------------------------------------------------------------------
// Oracle problem
// ---------------------------------------------------------------------------

// Vertex triples of the tetrahedron faces used for normals,
// MAKE_PARTITION_AND_MPI_FILES.f90:1087-1096 (0-based local vertex ids).
const int FACE_VERTS[4][3] = {{2, 1, 0}, {0, 1, 3}, {1, 2, 3}, {2, 0, 3}};

struct Oracle {
    // mesh
    int n_node = 0, n_tet = 0, n_poly = 0, n_mat = 0;
    std::vector<double> coords, mat;
    std::vector<int> tet_vert, tet_poly, tet_mat, neigh, fun_tag;
    // method
    int p = 1, Np = 4, nd = 12;
    double alpha = 10.0, theta = -1.0, dt = 1e-3;
    Quadrature Q;
    double nm[4][4][4];
    std::vector<int> blist;
    // geometry
    std::vector<double> fk;      // [n_tet][3][4]
    std::vector<double> jdet;    // [n_tet]
    std::vector<double> normal;  // [n_tet][4][3]
    std::vector<double> area;    // [n_tet][4]
    std::vector<double> bbox;    // [n_poly][3][2]
    std::vector<double> hk;      // [n_poly]
    std::vector<int> poly_ptr, poly_tets;  // CSR polyhedron -> tets (ascending)
    // operator
    std::vector<std::vector<int>> nbr;        // per poly: block -> column poly (block 0 = self)
    std::vector<std::vector<double>> K, A;    // per poly: [nb][nd][nd]
    std::vector<double> M, Mm, R, Rm;         // [n_poly][Np][Np]
    std::vector<double> rhs_stat, rhs_dyn;    // [n_poly][nd]
    std::vector<double> slot[4];              // [n_poly][nd]
    bool have_matrices = false;
    bool have_dg = false;      // A_dg assembled (g_assemble_dg when the matrices were made)
    // absorbing faces: per polyhedron its index among those with some (-1
    // otherwise), their damping blocks D [nd][nd] and the Cholesky factors of
    // W = M (x) I + dt/2 D (row-major, as cholesky writes them)
    std::vector<int> abs_idx;
    std::vector<std::vector<double>> Dabs, RW;
    // the same blocks summed in the device kernel's arrangement
    // (|face| C_ij sum_q w_q (phi_m phi_n)), for the device-order floor variant
    std::vector<std::vector<double>> Dabs_dev, RW_dev;
    int status = 0;
};

void geometry(Oracle& o) {
    o.fk.assign(o.n_tet * 12, 0.0); o.jdet.assign(o.n_tet, 0.0);
    o.normal.assign(o.n_tet * 12, 0.0); o.area.assign(o.n_tet * 4, 0.0);
    for (int t = 0; t < o.n_tet; ++t) {
        double x[4], y[4], z[4];
        for (int v = 0; v < 4; ++v) {
            int id = o.tet_vert[t * 4 + v];
            x[v] = o.coords[id * 3 + 0]; y[v] = o.coords[id * 3 + 1]; z[v] = o.coords[id * 3 + 2];
        }
        double fk[3][4], jd;
        jacobians(x, y, z, fk, &jd);
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 4; ++b) o.fk[t * 12 + a * 4 + b] = fk[a][b];
        o.jdet[t] = jd;
        // CREATE_NORMAL_FACE, MAKE_PARTITION_AND_MPI_FILES.f90:1429-1504
        for (int f = 0; f < 4; ++f) {
            int i1 = o.tet_vert[t * 4 + FACE_VERTS[f][0]], i2 = o.tet_vert[t * 4 + FACE_VERTS[f][1]],
                i3 = o.tet_vert[t * 4 + FACE_VERTS[f][2]];
            const double* c1 = &o.coords[i1 * 3]; const double* c2 = &o.coords[i2 * 3]; const double* c3 = &o.coords[i3 * 3];
            double Qx = c1[0] - c2[0], Qy = c1[1] - c2[1], Qz = c1[2] - c2[2];
            double Px = c3[0] - c2[0], Py = c3[1] - c2[1], Pz = c3[2] - c2[2];
            double n1 = Py * Qz - Pz * Qy, n2 = -Px * Qz + Pz * Qx, n3 = Px * Qy - Py * Qx;
            double nn = std::sqrt(n1 * n1 + n2 * n2 + n3 * n3);
            o.normal[t * 12 + f * 3 + 0] = n1 / nn;
            o.normal[t * 12 + f * 3 + 1] = n2 / nn;
            o.normal[t * 12 + f * 3 + 2] = n3 / nn;
            o.area[t * 4 + f] = nn;
        }
    }
    // polyhedron -> tets
    o.poly_ptr.assign(o.n_poly + 1, 0);
    for (int t = 0; t < o.n_tet; ++t) o.poly_ptr[o.tet_poly[t] + 1]++;
    for (int P = 0; P < o.n_poly; ++P) o.poly_ptr[P + 1] += o.poly_ptr[P];
    o.poly_tets.assign(o.n_tet, 0);
    std::vector<int> fill(o.poly_ptr.begin(), o.poly_ptr.end() - 1);
    for (int t = 0; t < o.n_tet; ++t) o.poly_tets[fill[o.tet_poly[t]]++] = t;
    // CREATE_BBOX_EL, MAKE_PARTITION_AND_MPI_FILES.f90:1510-1580
    o.bbox.assign(o.n_poly * 6, 0.0); o.hk.assign(o.n_poly, 0.0);
    for (int P = 0; P < o.n_poly; ++P) {
        std::vector<double> xv, yv, zv;
        for (int k = o.poly_ptr[P]; k < o.poly_ptr[P + 1]; ++k) {
            int t = o.poly_tets[k];
            for (int v = 0; v < 4; ++v) {
                int id = o.tet_vert[t * 4 + v];
                xv.push_back(o.coords[id * 3]); yv.push_back(o.coords[id * 3 + 1]); zv.push_back(o.coords[id * 3 + 2]);
            }
        }
        o.bbox[P * 6 + 0] = *std::min_element(xv.begin(), xv.end());
        o.bbox[P * 6 + 1] = *std::max_element(xv.begin(), xv.end());
        o.bbox[P * 6 + 2] = *std::min_element(yv.begin(), yv.end());
        o.bbox[P * 6 + 3] = *std::max_element(yv.begin(), yv.end());
        o.bbox[P * 6 + 4] = *std::min_element(zv.begin(), zv.end());
        o.bbox[P * 6 + 5] = *std::max_element(zv.begin(), zv.end());
        double h = 0.0;
        for (size_t a = 0; a < xv.size(); ++a)
            for (size_t b = a + 1; b < xv.size(); ++b) {
                double d = std::sqrt((xv[a] - xv[b]) * (xv[a] - xv[b]) + (yv[a] - yv[b]) * (yv[a] - yv[b]) +
                                     (zv[a] - zv[b]) * (zv[a] - zv[b]));
                if (d > h) h = d;
            }
        o.hk[P] = h;
    }
}

void get_bb(const Oracle& o, int P, double bb[3][2]) {
    for (int a = 0; a < 3; ++a) { bb[a][0] = o.bbox[P * 6 + 2 * a]; bb[a][1] = o.bbox[P * 6 + 2 * a + 1]; }
}

// basis, basis_function.f90:440-517: phi[q][Np], dphi[q][3][Np] at the mapped
// tetrahedron quadrature nodes, bounding box of polyhedron P.
void basis_tet(const Oracle& o, int t, int P, std::vector<double>& phi, std::vector<double>& dphi) {
    int nq3 = o.Q.nq3, Np = o.Np;
    phi.assign(nq3 * Np, 0.0); dphi.assign(nq3 * 3 * Np, 0.0);
    double bb[3][2]; get_bb(o, P, bb);
    const double* fk = &o.fk[t * 12];
    for (int q = 0; q < nq3; ++q) {
        double pt[3];
        for (int j = 0; j < 3; ++j) {
            pt[j] = 0.0;
            for (int l = 0; l < 4; ++l) pt[j] = pt[j] + fk[j * 4 + l] * o.Q.nodtet3[q * 4 + l];
        }
        eval_basis_point(pt, bb, Np, o.blist.data(), &phi[q * Np], &dphi[q * 3 * Np]);
    }
}

// Physical points of face e of tetrahedron t (basis_boundary,
// basis_function.f90:560-577): temp = Fk * node_maps(:,:,e), pt = temp * nodtria2.
void face_points(const Oracle& o, int t, int e, std::vector<double>& pts) {
    int nq2 = o.Q.nq2;
    pts.assign(nq2 * 3, 0.0);
    const double* fk = &o.fk[t * 12];
    double temp[3][4];
    for (int j = 0; j < 3; ++j)
        for (int q = 0; q < 4; ++q) {
            temp[j][q] = 0.0;
            for (int l = 0; l < 4; ++l) temp[j][q] = temp[j][q] + fk[j * 4 + l] * o.nm[e][l][q];
        }
    for (int j = 0; j < 3; ++j)
        for (int q = 0; q < nq2; ++q) {
            double s = 0.0;
            for (int l = 0; l < 4; ++l) s = s + temp[j][l] * o.Q.nodtria2[q * 4 + l];
            pts[q * 3 + j] = s;
        }
}

// basis_boundary, basis_function.f90:521-648: traces on face e of tet t for
// the E+ polyhedron P and (if internal) the E- polyhedron Qp.
void basis_boundary(const Oracle& o, int t, int e, int P, int Qp, std::vector<double>& phib /*[2][nq2][Np]*/,
                    std::vector<double>& gradb /*[2][nq2][3][Np]*/) {
    int nq2 = o.Q.nq2, Np = o.Np;
    phib.assign(2 * nq2 * Np, 0.0); gradb.assign(2 * nq2 * 3 * Np, 0.0);
    std::vector<double> pts; face_points(o, t, e, pts);
    double bb[3][2];
    get_bb(o, P, bb);
    for (int q = 0; q < nq2; ++q) eval_basis_point(&pts[q * 3], bb, Np, o.blist.data(), &phib[q * Np], &gradb[q * 3 * Np]);
    if (Qp >= 0) {
        get_bb(o, Qp, bb);
        for (int q = 0; q < nq2; ++q)
            eval_basis_point(&pts[q * 3], bb, Np, o.blist.data(), &phib[(nq2 + q) * Np], &gradb[(nq2 + q) * 3 * Np]);
    }
}

// MAKE_STIFFNESS_VOLUME (assemble_element.f90:24-77) and MAKE_MASS_VOLUME
// (:81-113).  V[i][j][m][n], mass[m][n] (the identical diagonal blocks).
void stiffness_volume(int Np, double jd, const Quadrature& Q, double lambda, double mu, const std::vector<double>& dphi,
                      std::vector<double>& V) {
    V.assign(9 * Np * Np, 0.0);
    auto D = [&](int q, int i, int m) { return dphi[(q * 3 + i) * Np + m]; };
    double temp[3][3];
    for (int q = 0; q < Q.nq3; ++q) {
        for (int m = 0; m < Np; ++m)
            for (int n = 0; n < Np; ++n) {
                temp[0][0] = (lambda + 2 * mu) * D(q, 0, m) * D(q, 0, n) + mu * D(q, 1, m) * D(q, 1, n) + mu * D(q, 2, m) * D(q, 2, n);
                temp[1][1] = (lambda + 2 * mu) * D(q, 1, m) * D(q, 1, n) + mu * D(q, 0, m) * D(q, 0, n) + mu * D(q, 2, m) * D(q, 2, n);
                temp[2][2] = (lambda + 2 * mu) * D(q, 2, m) * D(q, 2, n) + mu * D(q, 0, m) * D(q, 0, n) + mu * D(q, 1, m) * D(q, 1, n);
                for (int i = 0; i < 2; ++i)
                    for (int j = i + 1; j < 3; ++j) {
                        temp[i][j] = lambda * D(q, i, m) * D(q, j, n) + mu * D(q, j, m) * D(q, i, n);
                        temp[j][i] = lambda * D(q, j, m) * D(q, i, n) + mu * D(q, i, m) * D(q, j, n);
                    }
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j) {
                        double& v = V[((i * 3 + j) * Np + m) * Np + n];
                        v = v + Q.weitet3[q] * std::fabs(jd) * temp[i][j];
                    }
            }
    }
}

void mass_volume(int Np, double jd, const Quadrature& Q, const std::vector<double>& phi, double rho, std::vector<double>& Mv) {
    Mv.assign(Np * Np, 0.0);
    for (int q = 0; q < Q.nq3; ++q)
        for (int m = 0; m < Np; ++m)
            for (int n = 0; n < Np; ++n) {
                double& v = Mv[m * Np + n];
                v = v + rho * Q.weitet3[q] * std::fabs(jd) * phi[q * Np + m] * phi[q * Np + n];
            }
}

// MAKE_STIFFNESS_FACE, assemble_element.f90:404-661 (no absorbing branch).
// Outputs [i][j][m][n]: S_E1, I_E1, I_E2, IT_E2, S_E2.
struct FaceMats { std::vector<double> S1, I1, I2, IT2, S2; };

void stiffness_face(double alpha, int p, int Np, int E2, double hk1, double hk2, const double nrm[3], double area,
                    const Quadrature& Q, double lambda, double mu, const std::vector<double>& phib,
                    const std::vector<double>& gradb, FaceMats& F) {
    int nq2 = Q.nq2, N2 = Np * Np;
    F.S1.assign(9 * N2, 0.0); F.I1.assign(9 * N2, 0.0); F.I2.assign(9 * N2, 0.0);
    F.IT2.assign(9 * N2, 0.0); F.S2.assign(9 * N2, 0.0);
    double D_bar = lambda + 2 * mu;
    double sigma = 0.0;
    if (E2 == BC_DIRI) sigma = alpha * (p * p) / hk1 * D_bar;
    if (E2 != BC_DIRI && E2 != BC_NEUM) sigma = alpha * (p * p) / std::min(hk1, hk2) * D_bar;
    if (E2 == BC_NEUM) return;
    auto PH = [&](int s, int q, int m) { return phib[(s * nq2 + q) * Np + m]; };
    auto GR = [&](int s, int q, int i, int m) { return gradb[((s * nq2 + q) * 3 + i) * Np + m]; };
    auto at = [&](std::vector<double>& X, int i, int j, int m, int n) -> double& { return X[((i * 3 + j) * Np + m) * Np + n]; };
    const double n0 = nrm[0], n1 = nrm[1], n2 = nrm[2];
    const double c00 = std::fabs(n0) * std::fabs(n0) + 0.5 * (std::fabs(n1) * std::fabs(n1)) + 0.5 * (std::fabs(n2) * std::fabs(n2));
    const double c11 = std::fabs(n1) * std::fabs(n1) + 0.5 * (std::fabs(n0) * std::fabs(n0)) + 0.5 * (std::fabs(n2) * std::fabs(n2));
    const double c22 = std::fabs(n2) * std::fabs(n2) + 0.5 * (std::fabs(n0) * std::fabs(n0)) + 0.5 * (std::fabs(n1) * std::fabs(n1));
    double temp[3][3];
    // sigma(phi_m e_i) n . e_j phi_n with gradient g (side sg) and value v (side sv)
    auto stress_form = [&](int sg, int sv, int q, int m, int n, double T[3][3]) {
        double g0 = GR(sg, q, 0, m), g1 = GR(sg, q, 1, m), g2 = GR(sg, q, 2, m), v = PH(sv, q, n);
        T[0][0] = (lambda + 2 * mu) * g0 * v * n0 + mu * g1 * v * n1 + mu * g2 * v * n2;
        T[1][1] = (lambda + 2 * mu) * g1 * v * n1 + mu * g0 * v * n0 + mu * g2 * v * n2;
        T[2][2] = (lambda + 2 * mu) * g2 * v * n2 + mu * g1 * v * n1 + mu * g0 * v * n0;
        double g[3] = {g0, g1, g2};
        for (int i = 0; i < 2; ++i)
            for (int j = i + 1; j < 3; ++j) {
                T[i][j] = lambda * g[i] * v * nrm[j] + mu * g[j] * v * nrm[i];
                T[j][i] = lambda * g[j] * v * nrm[i] + mu * g[i] * v * nrm[j];
            }
    };
    for (int q = 0; q < nq2; ++q) {
        double w = Q.weitria2[q];
        // S_E1
        for (int m = 0; m < Np; ++m)
            for (int n = 0; n < Np; ++n) {
                double pp = PH(0, q, m) * PH(0, q, n);
                temp[0][0] = pp * c00; temp[1][1] = pp * c11; temp[2][2] = pp * c22;
                for (int i = 0; i < 2; ++i)
                    for (int j = i + 1; j < 3; ++j) {
                        temp[i][j] = 0.5 * PH(0, q, m) * PH(0, q, n) * nrm[i] * nrm[j];
                        temp[j][i] = 0.5 * PH(0, q, m) * PH(0, q, n) * nrm[i] * nrm[j];
                    }
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j) at(F.S1, i, j, m, n) = at(F.S1, i, j, m, n) + sigma * w * temp[i][j] * area;
            }
        if (E2 == BC_DIRI) {
            for (int m = 0; m < Np; ++m)
                for (int n = 0; n < Np; ++n) {
                    stress_form(0, 0, q, m, n, temp);
                    for (int i = 0; i < 3; ++i)
                        for (int j = 0; j < 3; ++j) at(F.I1, i, j, m, n) = at(F.I1, i, j, m, n) + w * area * temp[i][j];
                }
        } else if (E2 == BC_ABSO) {
            // absorbing boundary: not on the path (its call is commented out,
            // matrix_free.f90:279-287)
        } else {
            for (int m = 0; m < Np; ++m)
                for (int n = 0; n < Np; ++n) {
                    stress_form(0, 0, q, m, n, temp);
                    for (int i = 0; i < 3; ++i)
                        for (int j = 0; j < 3; ++j) at(F.I1, i, j, m, n) = at(F.I1, i, j, m, n) + 0.5 * w * area * temp[i][j];
                    stress_form(0, 1, q, m, n, temp);
                    for (int i = 0; i < 3; ++i)
                        for (int j = 0; j < 3; ++j) at(F.I2, i, j, m, n) = at(F.I2, i, j, m, n) - 0.5 * w * area * temp[i][j];
                    stress_form(1, 0, q, m, n, temp);
                    for (int i = 0; i < 3; ++i)
                        for (int j = 0; j < 3; ++j) at(F.IT2, i, j, n, m) = at(F.IT2, i, j, n, m) + 0.5 * w * area * temp[i][j];
                    double pp = PH(0, q, m) * PH(1, q, n);
                    temp[0][0] = pp * c00; temp[1][1] = pp * c11; temp[2][2] = pp * c22;
                    for (int i = 0; i < 2; ++i)
                        for (int j = i + 1; j < 3; ++j) {
                            temp[i][j] = 0.5 * PH(0, q, m) * PH(1, q, n) * nrm[i] * nrm[j];
                            temp[j][i] = 0.5 * PH(0, q, m) * PH(1, q, n) * nrm[i] * nrm[j];
                        }
                    for (int i = 0; i < 3; ++i)
                        for (int j = 0; j < 3; ++j) at(F.S2, i, j, m, n) = at(F.S2, i, j, m, n) - sigma * w * temp[i][j] * area;
                }
        }
    }
}

int block_of(Oracle& o, int P, int Qp) {
    auto& v = o.nbr[P];
    for (size_t b = 0; b < v.size(); ++b)
        if (v[b] == Qp) return (int)b;
    v.push_back(Qp);
    o.K[P].resize(v.size() * o.nd * o.nd, 0.0);
    if (o.have_dg) o.A[P].resize(v.size() * o.nd * o.nd, 0.0);
    return (int)v.size() - 1;
}

// MAKE_DAMPING_FACE (assemble_element.f90:666-731) on every absorbing face
// of a polyhedron, summed into the polyhedron's damping block D:
//   val = phi_m (t1_i b1 + t2_i b2 + n_i b3),  b = (c1 phi_n t1_j, c2 phi_n t2_j, c3 phi_n n_j),
//   D[(i,m),(j,n)] += w_q |face| val,
// over all (i, j, m, n).  The reference leaves c1 = c2 = c3 = 1 as
// placeholders, takes its two tangents straight from two face edges
// (CREATE_NORMAL_FACE, MAKE_PARTITION_AND_MPI_FILES.f90:1486-1498, not
// orthogonal to each other), loops over the upper triangle adding each term
// to both halves (so the diagonal counts twice) and writes row (i-1)*DIM + m;
// here the frame is orthonormal (t1 the first edge direction, t2 = n x t1),
// c1 = c2 = rho c_s = sqrt(rho mu) and c3 = rho c_p = sqrt(rho (lambda + 2 mu))
// (the first-order absorbing impedances of the face's tetrahedron), and every
// term is added once at row i*Np + m.  Then W = M (x) I + dt/2 D and its
// Cholesky factor.
bool make_damping(Oracle& o) {
    const int Np = o.Np, nd = o.nd, nq2 = o.Q.nq2;
    o.abs_idx.assign(o.n_poly, -1);
    o.Dabs.clear();
    o.RW.clear();
    o.Dabs_dev.clear();
    o.RW_dev.clear();
    for (int P = 0; P < o.n_poly; ++P) {
        bool any = false;
        for (int k = o.poly_ptr[P]; k < o.poly_ptr[P + 1] && !any; ++k)
            for (int f = 0; f < 4; ++f) any |= (o.neigh[o.poly_tets[k] * 4 + f] == BC_ABSO);
        if (any) {
            o.abs_idx[P] = (int)o.Dabs.size();
            o.Dabs.emplace_back((size_t)nd * nd, 0.0);
            o.RW.emplace_back((size_t)nd * nd, 0.0);
            o.Dabs_dev.emplace_back((size_t)nd * nd, 0.0);
            o.RW_dev.emplace_back((size_t)nd * nd, 0.0);
        }
    }
    bool ok = true;
#pragma omp parallel for schedule(dynamic, 1) reduction(&& : ok)
    for (int P = 0; P < o.n_poly; ++P) {
        const int a = o.abs_idx[P];
        if (a < 0) continue;
        std::vector<double>& D = o.Dabs[a];
        std::vector<double> phib, gradb;
        for (int k = o.poly_ptr[P]; k < o.poly_ptr[P + 1]; ++k) {
            const int t = o.poly_tets[k];
            const int mid = o.tet_mat[t];
            const double rho = o.mat[mid * 3 + 0], lam = o.mat[mid * 3 + 1], mu = o.mat[mid * 3 + 2];
            const double c1 = std::sqrt(rho * mu), c2 = c1, c3 = std::sqrt(rho * (lam + 2 * mu));
            for (int f = 0; f < 4; ++f) {
                if (o.neigh[t * 4 + f] != BC_ABSO) continue;
                const double* nv = &o.normal[t * 12 + f * 3];
                // first tangent: the edge from the face's second vertex to its third
                const int* fv = FACE_VERTS[f];
                double e[3], t1[3], t2[3];
                for (int d = 0; d < 3; ++d)
                    e[d] = o.coords[o.tet_vert[t * 4 + fv[2]] * 3 + d] - o.coords[o.tet_vert[t * 4 + fv[1]] * 3 + d];
                const double en = std::sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]);
                for (int d = 0; d < 3; ++d) t1[d] = e[d] / en;
                t2[0] = nv[1] * t1[2] - nv[2] * t1[1];
                t2[1] = nv[2] * t1[0] - nv[0] * t1[2];
                t2[2] = nv[0] * t1[1] - nv[1] * t1[0];
                basis_boundary(o, t, f, P, -1, phib, gradb);
                const double ar = o.area[t * 4 + f];
                for (int q = 0; q < nq2; ++q) {
                    const double w = o.Q.weitria2[q];
                    for (int i = 0; i < 3; ++i)
                        for (int j = 0; j < 3; ++j)
                            for (int m = 0; m < Np; ++m)
                                for (int n = 0; n < Np; ++n) {
                                    const double phn = phib[q * Np + n];
                                    const double b1 = c1 * phn * t1[j], b2 = c2 * phn * t2[j], b3 = c3 * phn * nv[j];
                                    const double val = phib[q * Np + m] * (t1[i] * b1 + t2[i] * b2 + nv[i] * b3);
                                    D[(size_t)(i * Np + m) * nd + j * Np + n] += w * ar * val;
                                }
                }
                // the device kernel's arrangement: C = c_t (I - n n^T) + c_n n n^T
                std::vector<double>& Dd = o.Dabs_dev[a];
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j) {
                        const double nij = nv[i] * nv[j];
                        const double C = c1 * ((i == j ? 1.0 : 0.0) - nij) + c3 * nij;
                        for (int m = 0; m < Np; ++m)
                            for (int n = 0; n < Np; ++n) {
                                double sq = 0.0;
                                for (int q = 0; q < nq2; ++q)
                                    sq = sq + o.Q.weitria2[q] * (phib[q * Np + m] * phib[q * Np + n]);
                                Dd[(size_t)(i * Np + m) * nd + j * Np + n] += ar * C * sq;
                            }
                    }
            }
        }
        std::vector<double> W((size_t)nd * nd);
        for (int v = 0; v < 2; ++v) {
            const std::vector<double>& Dv = v == 0 ? D : o.Dabs_dev[a];
            for (int r = 0; r < nd; ++r)
                for (int c = 0; c < nd; ++c) {
                    const int i = r / Np, m = r % Np, j = c / Np, n = c % Np;
                    const double mv = (i == j) ? o.M[(size_t)P * Np * Np + (size_t)m * Np + n] : 0.0;
                    W[(size_t)r * nd + c] = mv + 0.5 * o.dt * Dv[(size_t)r * nd + c];
                }
            if (!cholesky(W.data(), nd, (v == 0 ? o.RW[a] : o.RW_dev[a]).data())) ok = false;
        }
    }
    return ok;
}

// MAKE_MATRICES_FREE, matrix_free.f90:27-464, polyhedron-accumulated; then
// the Cholesky factors of the driver (Lymph3D.f90:264-271).
int make_matrices(Oracle& o) {
    int Np = o.Np, nd = o.nd, N2 = Np * Np;
    o.nbr.assign(o.n_poly, std::vector<int>());
    o.K.assign(o.n_poly, std::vector<double>());
    o.A.assign(o.n_poly, std::vector<double>());
    o.M.assign((size_t)o.n_poly * N2, 0.0); o.Mm.assign((size_t)o.n_poly * N2, 0.0);
    o.R.assign((size_t)o.n_poly * N2, 0.0); o.Rm.assign((size_t)o.n_poly * N2, 0.0);
    o.have_dg = g_assemble_dg != 0;
    const bool dg = o.have_dg;
    int bad = 0;
#pragma omp parallel for schedule(dynamic, 4) reduction(| : bad)
    for (int P = 0; P < o.n_poly; ++P) {
        o.nbr[P].push_back(P);
        o.K[P].assign(nd * nd, 0.0);
        if (dg) o.A[P].assign(nd * nd, 0.0);
        std::vector<double> phi, dphi, V, Mv, phib, gradb;
        FaceMats F;
        for (int k = o.poly_ptr[P]; k < o.poly_ptr[P + 1]; ++k) {
            int t = o.poly_tets[k];
            int mid = o.tet_mat[t];
            double rho = o.mat[mid * 3 + 0], lambda = o.mat[mid * 3 + 1], mu = o.mat[mid * 3 + 2];
            basis_tet(o, t, P, phi, dphi);
            mass_volume(Np, o.jdet[t], o.Q, phi, 1.0, Mv);
            for (int a = 0; a < N2; ++a) {
                o.Mm[(size_t)P * N2 + a] += Mv[a];
                o.M[(size_t)P * N2 + a] += Mv[a] * rho;
            }
            stiffness_volume(Np, o.jdet[t], o.Q, lambda, mu, dphi, V);
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j)
                    for (int m = 0; m < Np; ++m)
                        for (int n = 0; n < Np; ++n) {
                            double v = V[((i * 3 + j) * Np + m) * Np + n];
                            o.K[P][(i * Np + m) * nd + j * Np + n] += v;
                            if (dg) o.A[P][(i * Np + m) * nd + j * Np + n] += v;
                        }
            for (int f = 0; f < 4; ++f) {
                int E2 = o.neigh[t * 4 + f];
                int Qp = -1;
                if (E2 != BC_DIRI && E2 != BC_NEUM && E2 != BC_ABSO) {
                    Qp = o.tet_poly[E2];
                    if (Qp == P) continue;  // face_flag: same polyhedron
                }
                if (E2 == BC_NEUM || E2 == BC_ABSO) continue;  // no stiffness contribution (absorbing: damping only)
                const double* nn = &o.normal[t * 12 + f * 3];
                basis_boundary(o, t, f, P, Qp, phib, gradb);
                double hk2 = (Qp >= 0) ? o.hk[Qp] : o.hk[0];
                stiffness_face(o.alpha, o.p, Np, E2, o.hk[P], hk2, nn, o.area[t * 4 + f], o.Q, lambda, mu, phib, gradb, F);
                auto IDX = [&](int i, int j, int m, int n) { return ((i * 3 + j) * Np + m) * Np + n; };
                double* K1 = &o.K[P][0];
                double* A1 = dg ? &o.A[P][0] : nullptr;
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j)
                        for (int m = 0; m < Np; ++m)
                            for (int n = 0; n < Np; ++n) {
                                int rc = (i * Np + m) * nd + j * Np + n;
                                K1[rc] += F.S1[IDX(i, j, m, n)];
                                if (dg) A1[rc] += F.S1[IDX(i, j, m, n)];
                            }
                if (E2 == BC_DIRI) {
                    for (int i = 0; i < 3; ++i)
                        for (int j = 0; j < 3; ++j)
                            for (int m = 0; m < Np; ++m)
                                for (int n = 0; n < Np; ++n) {
                                    int rc = (i * Np + m) * nd + j * Np + n;
                                    K1[rc] = K1[rc] + o.theta * F.I1[IDX(i, j, m, n)] - F.I1[IDX(j, i, n, m)];
                                }
                } else {
                    int b = block_of(o, P, Qp);
                    K1 = &o.K[P][0];
                    double* Kb = &o.K[P][(size_t)b * nd * nd];
                    double* Ab = dg ? &o.A[P][(size_t)b * nd * nd] : nullptr;
                    for (int i = 0; i < 3; ++i)
                        for (int j = 0; j < 3; ++j)
                            for (int m = 0; m < Np; ++m)
                                for (int n = 0; n < Np; ++n) {
                                    int rc = (i * Np + m) * nd + j * Np + n;
                                    K1[rc] = K1[rc] + o.theta * F.I1[IDX(i, j, m, n)] - F.I1[IDX(j, i, n, m)];
                                    Kb[rc] = Kb[rc] + o.theta * F.I2[IDX(i, j, m, n)] + F.S2[IDX(i, j, m, n)];
                                    if (dg) Ab[rc] = Ab[rc] + F.S2[IDX(i, j, m, n)];
                                    Kb[rc] = Kb[rc] - F.IT2[IDX(i, j, m, n)];
                                }
                }
            }
        }
        if (!cholesky(&o.M[(size_t)P * N2], Np, &o.R[(size_t)P * N2])) bad |= 1;
        if (!cholesky(&o.Mm[(size_t)P * N2], Np, &o.Rm[(size_t)P * N2])) bad |= 1;
    }
    if (bad) { g_err = "oracle: mass matrix is not positive definite"; return LYMPH_EXIT_SINGULARMTX; }
    if (!make_damping(o)) { g_err = "oracle: M + dt/2 D is not positive definite"; return LYMPH_EXIT_SINGULARMTX; }
    o.have_matrices = true;
    return 0;
}

// MAKE_RHS_VOLUME (assemble_element.f90:171-237) + MAKE_RHS_FACE (:241-390)
// accumulated per polyhedron as in MAKE_RHS_FREE (matrix_free.f90:467-843).
int make_rhs(Oracle& o, int which, int fid, int did, int nid) {
    int Np = o.Np, nd = o.nd, nq3 = o.Q.nq3, nq2 = o.Q.nq2;
    std::vector<double>& rhs = (which == LYMPH_RHS_STAT) ? o.rhs_stat : o.rhs_dyn;
    rhs.assign((size_t)o.n_poly * nd, 0.0);
#pragma omp parallel for schedule(dynamic, 4)
    for (int P = 0; P < o.n_poly; ++P) {
        std::vector<double> phi, dphi, phib, gradb, pts;
        std::vector<double> rt(3 * Np), rf(3 * Np);
        for (int k = o.poly_ptr[P]; k < o.poly_ptr[P + 1]; ++k) {
            int t = o.poly_tets[k];
            int mid = o.tet_mat[t];
            double rho = o.mat[mid * 3 + 0], lambda = o.mat[mid * 3 + 1], mu = o.mat[mid * 3 + 2];
            basis_tet(o, t, P, phi, dphi);
            const double* fk = &o.fk[t * 12];
            std::fill(rt.begin(), rt.end(), 0.0);
            for (int q = 0; q < nq3; ++q)
                for (int m = 0; m < Np; ++m) {
                    double pt[3], fr[3];
                    for (int j = 0; j < 3; ++j) {
                        pt[j] = 0.0;
                        for (int kk = 0; kk < 4; ++kk) pt[j] = pt[j] + fk[j * 4 + kk] * o.Q.nodtet3[q * 4 + kk];
                    }
                    f_forcing(fid, lambda, mu, pt, rho, fr);
                    for (int i = 0; i < 3; ++i)
                        rt[i * Np + m] = rt[i * Np + m] + std::fabs(o.jdet[t]) * o.Q.weitet3[q] * fr[i] * phi[q * Np + m];
                }
            for (int a = 0; a < nd; ++a) rhs[(size_t)P * nd + a] += rt[a];
            for (int f = 0; f < 4; ++f) {
                int E2 = o.neigh[t * 4 + f];
                if (E2 != BC_DIRI && E2 != BC_NEUM) continue;  // only boundary faces are added (:809-819)
                int tag = o.fun_tag.empty() ? 1 : o.fun_tag[t * 4 + f];
                const double* nrm = &o.normal[t * 12 + f * 3];
                double ar = o.area[t * 4 + f];
                basis_boundary(o, t, f, P, -1, phib, gradb);
                face_points(o, t, f, pts);  // same points; the reference forms them as Fk*node_maps*nodtria2 per term
                double D_bar = lambda + 2 * mu;
                double sigma = o.alpha * (o.p * o.p) / o.hk[P] * D_bar;  // Dirichlet penalty (:296-298)
                std::fill(rf.begin(), rf.end(), 0.0);
                for (int q = 0; q < nq2; ++q) {
                    double w = o.Q.weitria2[q];
                    // points(j) = sum_k sum_t Fk(j,k) node_maps(k,t,e) nodtria2(t,q)
                    double pq[3];
                    for (int j = 0; j < 3; ++j) {
                        pq[j] = 0.0;
                        for (int kk = 0; kk < 4; ++kk)
                            for (int tt = 0; tt < 4; ++tt)
                                pq[j] = pq[j] + fk[j * 4 + kk] * o.nm[f][kk][tt] * o.Q.nodtria2[q * 4 + tt];
                    }
                    if (E2 == BC_DIRI) {
                        double gd[3]; g_dirichlet(did, pq, tag, gd);
                        const double n0 = nrm[0], n1 = nrm[1], n2 = nrm[2];
                        for (int m = 0; m < Np; ++m) {
                            const double* g = &gradb[(q * 3) * Np];
                            double g0 = g[0 * Np + m], g1 = g[1 * Np + m], g2 = g[2 * Np + m];
                            double ph = phib[q * Np + m];
                            double t0 = (lambda + 2 * mu) * g0 * gd[0] * n0 + mu * g1 * gd[0] * n1 + mu * g2 * gd[0] * n2 +
                                        lambda * g0 * gd[1] * n1 + mu * g1 * gd[1] * n0 + lambda * g0 * gd[2] * n2 + mu * g2 * gd[2] * n0;
                            double t1 = (lambda + 2 * mu) * g1 * gd[1] * n1 + mu * g0 * gd[1] * n0 + mu * g2 * gd[1] * n2 +
                                        lambda * g1 * gd[0] * n0 + mu * g0 * gd[0] * n1 + lambda * g1 * gd[2] * n2 + mu * g2 * gd[2] * n1;
                            double t2 = (lambda + 2 * mu) * g2 * gd[2] * n2 + mu * g0 * gd[2] * n0 + mu * g1 * gd[2] * n1 +
                                        lambda * g2 * gd[0] * n0 + mu * g0 * gd[0] * n2 + lambda * g2 * gd[1] * n1 + mu * g1 * gd[1] * n2;
                            double a0 = std::fabs(n0) * std::fabs(n0), a1 = std::fabs(n1) * std::fabs(n1), a2 = std::fabs(n2) * std::fabs(n2);
                            double s0 = ph * gd[0] * (a0 + 0.5 * a1 + 0.5 * a2) + 0.5 * ph * gd[1] * n0 * n1 + 0.5 * ph * gd[2] * n0 * n2;
                            double s1 = ph * gd[1] * (a1 + 0.5 * a0 + 0.5 * a2) + 0.5 * ph * gd[0] * n0 * n1 + 0.5 * ph * gd[2] * n1 * n2;
                            double s2 = ph * gd[2] * (a2 + 0.5 * a0 + 0.5 * a1) + 0.5 * ph * gd[0] * n0 * n2 + 0.5 * ph * gd[1] * n1 * n2;
                            double tv[3] = {t0, t1, t2}, sv[3] = {s0, s1, s2};
                            for (int i = 0; i < 3; ++i)
                                rf[i * Np + m] = rf[i * Np + m] + o.theta * w * tv[i] * ar + sigma * w * sv[i] * ar;
                        }
                    } else {
                        double gn[3]; g_neumann(nid, lambda, mu, nrm, pq, tag, gn);
                        for (int m = 0; m < Np; ++m)
                            for (int i = 0; i < 3; ++i)
                                rf[i * Np + m] = rf[i * Np + m] + w * phib[q * Np + m] * gn[i] * ar;
                    }
                }
                for (int a = 0; a < nd; ++a)
                    if (rf[a] != 0.0) rhs[(size_t)P * nd + a] += rf[a];
            }
        }
    }
    return 0;
}

// COMPUTE_MODAL_COEFFICIENTS_FREE, matrix_free.f90:847-997 (accumulated per
// polyhedron, solved with the modal mass factor once per polyhedron).
int modal_project(Oracle& o, int fun_id, std::vector<double>& out) {
    int Np = o.Np, nd = o.nd, nq3 = o.Q.nq3;
    out.assign((size_t)o.n_poly * nd, 0.0);
#pragma omp parallel for schedule(dynamic, 4)
    for (int P = 0; P < o.n_poly; ++P) {
        std::vector<double> phi, dphi, integ(nd, 0.0), v(Np), x(Np);
        for (int k = o.poly_ptr[P]; k < o.poly_ptr[P + 1]; ++k) {
            int t = o.poly_tets[k];
            basis_tet(o, t, P, phi, dphi);
            const double* fk = &o.fk[t * 12];
            for (int q = 0; q < nq3; ++q)
                for (int m = 0; m < Np; ++m) {
                    double pt[3], ev[3];
                    for (int ii = 0; ii < 3; ++ii) {
                        pt[ii] = 0.0;
                        for (int jj = 0; jj < 4; ++jj) pt[ii] = pt[ii] + fk[ii * 4 + jj] * o.Q.nodtet3[q * 4 + jj];
                    }
                    f_analytic(fun_id, pt, ev);
                    for (int i = 0; i < 3; ++i)
                        integ[i * Np + m] = integ[i * Np + m] + std::fabs(o.jdet[t]) * o.Q.weitet3[q] * ev[i] * phi[q * Np + m];
                }
        }
        for (int i = 0; i < 3; ++i) {
            for (int m = 0; m < Np; ++m) v[m] = integ[i * Np + m];
            solve_LU_RT_R(&o.Rm[(size_t)P * Np * Np], v.data(), Np, x.data());
            for (int m = 0; m < Np; ++m) out[(size_t)P * nd + i * Np + m] = x[m];
        }
    }
    return 0;
}

// Shared body of FIRST_TIME_STEP_MATRIX_FREE (matrix_free.f90:1100-1227) and
// TIME_STEP_MATRIX_FREE (:1230-1385): tmp = K u (self + neighbour blocks),
// tmp = -tmp + rhs_stat + rhs_dyn g(t), per-component solve_LU(R^T, R).
// The explicit inverse of M_P, column k = solve_LU(R, e_k).
void explicit_inverse(const Oracle& o, int P, std::vector<double>& inv) {
    const int Np = o.Np;
    inv.assign((size_t)Np * Np, 0.0);
    std::vector<double> e(Np), col(Np);
    for (int k = 0; k < Np; ++k) {
        for (int m = 0; m < Np; ++m) e[m] = (m == k) ? 1.0 : 0.0;
        solve_LU_RT_R(&o.R[(size_t)P * Np * Np], e.data(), Np, col.data());
        for (int m = 0; m < Np; ++m) inv[(size_t)m * Np + k] = col[m];
    }
}

// The CUDA step kernel's evaluation order (g_device_order = S): returns
// x = M^-1 (f - K u) for polyhedron P.
void apply_and_solve_device_order(const Oracle& o, const std::vector<double>& u, double t, int P,
                                  std::vector<double>& out) {
    const int nd = o.nd, Np = o.Np, S = g_device_order;
    const int cpt = (nd + S - 1) / S;
    const double g = time_function(t);
    const size_t nb = o.nbr[P].size();
    // the device's row order: the self block, then the neighbours by index
    std::vector<size_t> order(nb);
    for (size_t bi = 0; bi < nb; ++bi) order[bi] = bi;
    std::sort(order.begin() + 1, order.end(), [&](size_t a, size_t b) { return o.nbr[P][a] < o.nbr[P][b]; });
    std::vector<double> b(nd);
    for (int r = 0; r < nd; ++r) {
        double y = 0.0;
        for (int sl = 0; sl < S; ++sl) {
            double acc0 = 0.0, acc1 = 0.0;
            for (size_t oi = 0; oi < nb; ++oi) {
                const size_t bi = order[oi];
                const double* Kb = &o.K[P][bi * nd * nd];
                const double* uq = &u[(size_t)o.nbr[P][bi] * nd];
                for (int j = 0; j < cpt; ++j) {
                    const int c = sl + j * S;
                    if (c >= nd) continue;
                    if (j & 1) acc1 = std::fma(Kb[r * nd + c], uq[c], acc1);
                    else acc0 = std::fma(Kb[r * nd + c], uq[c], acc0);
                }
            }
            y += acc0 + acc1;
        }
        b[r] = std::fma(o.rhs_dyn[(size_t)P * nd + r], g, -y + o.rhs_stat[(size_t)P * nd + r]);
    }
    std::vector<double> inv;
    explicit_inverse(o, P, inv);
    out.assign(nd, 0.0);
    for (int i = 0; i < 3; ++i)
        for (int m = 0; m < Np; ++m) {
            double x0 = 0.0, x1 = 0.0;
            for (int c = 0; c < Np; c += 2) {
                x0 = std::fma(inv[(size_t)m * Np + c], b[i * Np + c], x0);
                if (c + 1 < Np) x1 = std::fma(inv[(size_t)m * Np + c + 1], b[i * Np + c + 1], x1);
            }
            out[i * Np + m] = x0 + x1;
        }
}

// tmp = -K u + rhs_stat + rhs_dyn g(t) for polyhedron P, the reference's
// order (blocks in stored order, each row summed forward).
void apply_rhs(const Oracle& o, const std::vector<double>& u, double t, int P, std::vector<double>& tmp) {
    const int nd = o.nd;
    tmp.assign(nd, 0.0);
    const double g = time_function(t);
    for (size_t b = 0; b < o.nbr[P].size(); ++b) {
        const double* Kb = &o.K[P][b * nd * nd];
        const double* uq = &u[(size_t)o.nbr[P][b] * nd];
        for (int r = 0; r < nd; ++r) {
            double s = 0.0;
            for (int c = 0; c < nd; ++c) s = s + Kb[r * nd + c] * uq[c];
            tmp[r] = tmp[r] + s;
        }
    }
    for (int r = 0; r < nd; ++r) tmp[r] = -tmp[r] + o.rhs_stat[(size_t)P * nd + r] + o.rhs_dyn[(size_t)P * nd + r] * g;
}

// The damped leapfrog step of a polyhedron with absorbing faces:
//   (M + dt/2 D) u^{n+1} = dt^2 (F - K u^n) + 2 M u^n - (M - dt/2 D) u^{n-1},
// solved as u^{n+1} = 2 u^n - u^{n-1} + W^-1 (dt^2 (F - K u^n) - dt D (u^n - u^{n-1})),
// W = M (x) I + dt/2 D by its Cholesky factor (solve_LU(R^T, R)).
void absorbing_step(const Oracle& o, double t, int P, double* out) {
    const int nd = o.nd, a = o.abs_idx[P];
    const std::vector<double>& un = o.slot[LYMPH_SLOT_UN];
    const std::vector<double>& u0 = o.slot[LYMPH_SLOT_U0];
    std::vector<double> tmp, b(nd), x(nd);
    apply_rhs(o, un, t, P, tmp);
    const double* D = (g_device_order ? o.Dabs_dev[a] : o.Dabs[a]).data();
    const std::vector<double>& RW = g_device_order ? o.RW_dev[a] : o.RW[a];
    const size_t base = (size_t)P * nd;
    for (int r = 0; r < nd; ++r) {
        double dv = 0.0;
        for (int c = 0; c < nd; ++c) dv = dv + D[(size_t)r * nd + c] * (un[base + c] - u0[base + c]);
        b[r] = o.dt * o.dt * tmp[r] - o.dt * dv;
    }
    if (g_explicit_inverse || g_device_order) {
        // floor variants: W^-1 as an explicit inverse (columns by solve_LU),
        // applied with fused multiply-adds, the way the device applies it
        std::vector<double> e(nd), col(nd), inv((size_t)nd * nd);
        for (int k = 0; k < nd; ++k) {
            for (int r = 0; r < nd; ++r) e[r] = (r == k) ? 1.0 : 0.0;
            solve_LU_RT_R(RW.data(), e.data(), nd, col.data());
            for (int r = 0; r < nd; ++r) inv[(size_t)r * nd + k] = col[r];
        }
        for (int r = 0; r < nd; ++r) {
            double s = 0.0;
            for (int c = 0; c < nd; ++c) s = std::fma(inv[(size_t)r * nd + c], b[c], s);
            x[r] = s;
        }
    } else {
        solve_LU_RT_R(o.RW[a].data(), b.data(), nd, x.data());
    }
    for (int r = 0; r < nd; ++r) out[r] = x[r] + 2.0 * un[base + r] - u0[base + r];
}

// The first step of a polyhedron with absorbing faces:
//   u^1 = u^0 + dt v^0 + dt^2/2 M^-1 (F - K u^0 - D v^0).
void absorbing_first_step(const Oracle& o, double t, int P, double* out) {
    const int nd = o.nd, Np = o.Np, a = o.abs_idx[P];
    const std::vector<double>& u0 = o.slot[LYMPH_SLOT_U0];
    const std::vector<double>& v0 = o.slot[LYMPH_SLOT_V0];
    std::vector<double> tmp, v(Np), x(Np);
    apply_rhs(o, u0, t, P, tmp);
    const double* D = (g_device_order ? o.Dabs_dev[a] : o.Dabs[a]).data();
    const size_t base = (size_t)P * nd;
    for (int r = 0; r < nd; ++r) {
        double dv = 0.0;
        for (int c = 0; c < nd; ++c) dv = dv + D[(size_t)r * nd + c] * v0[base + c];
        tmp[r] = tmp[r] - dv;
    }
    const double half_dt2 = 0.5 * (o.dt * o.dt);
    std::vector<double> inv;
    if (g_explicit_inverse || g_device_order) explicit_inverse(o, P, inv);
    for (int i = 0; i < 3; ++i) {
        for (int m = 0; m < Np; ++m) v[m] = tmp[i * Np + m];
        if (g_device_order) {
            // floor variant: the device's order (explicit inverse, two
            // accumulators over even and odd columns, fused multiply-adds)
            for (int m = 0; m < Np; ++m) {
                double x0 = 0.0, x1 = 0.0;
                for (int c = 0; c < Np; c += 2) {
                    x0 = std::fma(inv[(size_t)m * Np + c], v[c], x0);
                    if (c + 1 < Np) x1 = std::fma(inv[(size_t)m * Np + c + 1], v[c + 1], x1);
                }
                const size_t q = base + i * Np + m;
                out[i * Np + m] = std::fma(o.dt, v0[q], std::fma(half_dt2, x0 + x1, u0[q]));
            }
            continue;
        }
        if (g_explicit_inverse) {
            for (int m = 0; m < Np; ++m) {
                double xx = 0.0;
                for (int c = 0; c < Np; ++c) xx = std::fma(inv[(size_t)m * Np + c], v[c], xx);
                x[m] = xx;
            }
        } else {
            solve_LU_RT_R(&o.R[(size_t)P * Np * Np], v.data(), Np, x.data());
        }
        for (int m = 0; m < Np; ++m)
            out[i * Np + m] = half_dt2 * x[m] + u0[base + i * Np + m] + o.dt * v0[base + i * Np + m];
    }
}

void apply_and_solve(const Oracle& o, const std::vector<double>& u, double t, int P, std::vector<double>& out) {
    if (g_device_order) { apply_and_solve_device_order(o, u, t, P, out); return; }
    int nd = o.nd, Np = o.Np;
    std::vector<double> tmp(nd, 0.0), v(Np), x(Np);
    double g = time_function(t);
    const size_t nb = o.nbr[P].size();
    for (size_t bi = 0; bi < nb; ++bi) {
        size_t b = g_reverse_sums ? nb - 1 - bi : bi;
        int Qp = o.nbr[P][b];
        const double* Kb = &o.K[P][b * nd * nd];
        const double* uq = &u[(size_t)Qp * nd];
        for (int r = 0; r < nd; ++r) {
            double s = 0.0;  // matmul row r
            if (g_reverse_sums)  // the floor variant also contracts to FMA, as the device does
                for (int c = nd - 1; c >= 0; --c) s = std::fma(Kb[r * nd + c], uq[c], s);
            else
                for (int c = 0; c < nd; ++c) s = s + Kb[r * nd + c] * uq[c];
            tmp[r] = tmp[r] + s;
        }
    }
    for (int r = 0; r < nd; ++r) tmp[r] = -tmp[r] + o.rhs_stat[(size_t)P * nd + r] + o.rhs_dyn[(size_t)P * nd + r] * g;
    out.assign(nd, 0.0);
    if (g_explicit_inverse) {
        std::vector<double> inv;
        explicit_inverse(o, P, inv);
        for (int i = 0; i < 3; ++i)
            for (int m = 0; m < Np; ++m) {
                double x = 0.0;
                for (int c = 0; c < Np; ++c) x = std::fma(inv[(size_t)m * Np + c], tmp[i * Np + c], x);
                out[i * Np + m] = x;
            }
        return;
    }
    for (int i = 0; i < 3; ++i) {
        for (int m = 0; m < Np; ++m) v[m] = tmp[i * Np + m];
        solve_LU_RT_R(&o.R[(size_t)P * Np * Np], v.data(), Np, x.data());
        for (int m = 0; m < Np; ++m) out[i * Np + m] = x[m];
    }
}

// face_points with a caller's triangle nodes node4 = (xi, eta, 1, 1) per node.
void face_points_rule(const Oracle& o, int t, int e, int nq, const double* node4, std::vector<double>& pts) {
    pts.assign(nq * 3, 0.0);
    const double* fk = &o.fk[t * 12];
    double temp[3][4];
    for (int j = 0; j < 3; ++j)
        for (int q = 0; q < 4; ++q) {
            temp[j][q] = 0.0;
            for (int l = 0; l < 4; ++l) temp[j][q] = temp[j][q] + fk[j * 4 + l] * o.nm[e][l][q];
        }
    for (int j = 0; j < 3; ++j)
        for (int q = 0; q < nq; ++q) {
            double s = 0.0;
            for (int l = 0; l < 4; ++l) s = s + temp[j][l] * node4[q * 4 + l];
            pts[q * 3 + j] = s;
        }
}

// K_PQ u_Q point by point with a given triangle rule: nq nodes, node4 =
// (xi, eta, 1, 1) per node as in nodtria2, weights w on the reference
// triangle (summing to 1/2).
int neighbour_apply_rule(const Oracle& o, int P, int Qp, const double* uq, int nq2, const double* node4,
                         const double* wq, double* out) {
    if (P < 0 || P >= o.n_poly || Qp < 0 || Qp >= o.n_poly || P == Qp) return LYMPH_ERR_INVALID;
    const int Np = o.Np;
    for (int r = 0; r < o.nd; ++r) out[r] = 0.0;
    double bbP[3][2], bbQ[3][2];
    get_bb(o, P, bbP);
    get_bb(o, Qp, bbQ);
    std::vector<double> pts, phP(Np), dP(3 * Np), phQ(Np), dQ(3 * Np);
    int n_shared = 0, i_shared = 0;
    if (g_planted_mistake == 4)
        for (int k = o.poly_ptr[P]; k < o.poly_ptr[P + 1]; ++k)
            for (int f = 0; f < 4; ++f) {
                const int E2 = o.neigh[o.poly_tets[k] * 4 + f];
                if (E2 >= 0 && o.tet_poly[E2] == Qp) ++n_shared;
            }
    for (int k = o.poly_ptr[P]; k < o.poly_ptr[P + 1]; ++k) {
        const int t = o.poly_tets[k];
        const int mid = o.tet_mat[t];
        const double lam = o.mat[mid * 3 + 1], mu = o.mat[mid * 3 + 2];
        for (int f = 0; f < 4; ++f) {
            const int E2 = o.neigh[t * 4 + f];
            if (E2 < 0 || o.tet_poly[E2] != Qp) continue;
            if (g_planted_mistake == 4 && ++i_shared == n_shared) continue;
            const double* n = &o.normal[t * 12 + f * 3];
            const double ar = o.area[t * 4 + f];
            const double sigma = o.alpha * (o.p * o.p) / std::min(o.hk[P], o.hk[Qp]) * (lam + 2 * mu);
            const double T[3][3] = {{n[0] * n[0] + 0.5 * n[1] * n[1] + 0.5 * n[2] * n[2], 0.5 * n[0] * n[1], 0.5 * n[0] * n[2]},
                                    {0.5 * n[1] * n[0], n[1] * n[1] + 0.5 * n[0] * n[0] + 0.5 * n[2] * n[2], 0.5 * n[1] * n[2]},
                                    {0.5 * n[2] * n[0], 0.5 * n[2] * n[1], n[2] * n[2] + 0.5 * n[0] * n[0] + 0.5 * n[1] * n[1]}};
            face_points_rule(o, t, f, nq2, node4, pts);
            for (int q = 0; q < nq2; ++q) {
                const double W = wq[q] * ar;
                eval_basis_point(&pts[q * 3], bbQ, Np, o.blist.data(), phQ.data(), dQ.data());
                eval_basis_point(&pts[q * 3], bbP, Np, o.blist.data(), phP.data(), dP.data());
                double v[3] = {0, 0, 0}, D[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
                for (int j = 0; j < 3; ++j)
                    for (int b = 0; b < Np; ++b) {
                        const double c = uq[j * Np + b];
                        v[j] += phQ[b] * c;
                        for (int kk = 0; kk < 3; ++kk) D[j][kk] += dQ[kk * Np + b] * c;
                    }
                const double nv = n[0] * v[0] + n[1] * v[1] + n[2] * v[2];
                const double trD = D[0][0] + D[1][1] + D[2][2];
                for (int i = 0; i < 3; ++i) {
                    double G[3];
                    for (int kk = 0; kk < 3; ++kk)
                        G[kk] = -0.5 * o.theta * W * ((i == kk ? lam * nv : 0.0) + mu * (n[i] * v[kk] + v[i] * n[kk]));
                    const double Tv = T[i][0] * v[0] + T[i][1] * v[1] + T[i][2] * v[2];
                    const double hh = lam * (n[0] * D[0][i] + n[1] * D[1][i] + n[2] * D[2][i]) + mu * n[i] * trD +
                                      mu * (n[0] * D[i][0] + n[1] * D[i][1] + n[2] * D[i][2]);
                    const double pen = g_planted_mistake == 1 ? 0.0 : sigma * Tv;
                    const double sym = g_planted_mistake == 2 ? -0.5 * hh : 0.5 * hh;
                    const double si = -W * (pen + sym);
                    if (g_planted_mistake == 3) G[0] = G[1] = G[2] = 0.0;
                    for (int a = 0; a < Np; ++a)
                        out[i * Np + a] += dP[a] * G[0] + dP[Np + a] * G[1] + dP[2 * Np + a] * G[2] + phP[a] * si;
                }
            }
        }
    }
    return 0;
}

}  // namespace

// ===========================================================================
// C API for the tests and the CPU baseline (ctypes)
// ===========================================================================
extern "C" {

const char* oracle_last_error(void) { return g_err.c_str(); }

void oracle_set_data_perturbation(int ulps) { g_perturb_ulps = ulps; }

void oracle_set_reverse_sums(int on) { g_reverse_sums = on; }

void oracle_set_explicit_inverse(int on) { g_explicit_inverse = on; }

void oracle_set_device_order(int slices) { g_device_order = slices > 0 ? slices : 0; }

void oracle_set_planted_mistake(int kind) { g_planted_mistake = kind; }

void oracle_set_assemble_dg(int on) { g_assemble_dg = on; }

int oracle_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void oracle_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

int oracle_create(const lymph_mesh_desc* m, int degree, double alpha, double theta, double dt, void** out) {
    if (!m || !out || degree < 1 || degree > 7) { g_err = "oracle_create: bad argument"; return LYMPH_ERR_INVALID; }
    Oracle* o = new Oracle();
    o->n_node = m->n_node; o->n_tet = m->n_tet; o->n_poly = m->n_poly; o->n_mat = m->n_mat;
    o->coords.assign(m->coords, m->coords + 3 * (size_t)m->n_node);
    o->tet_vert.assign(m->tet_vert, m->tet_vert + 4 * (size_t)m->n_tet);
    o->tet_poly.assign(m->tet_poly, m->tet_poly + m->n_tet);
    o->tet_mat.assign(m->tet_mat, m->tet_mat + m->n_tet);
    o->neigh.assign(m->neigh, m->neigh + 4 * (size_t)m->n_tet);
    if (m->fun_tag) o->fun_tag.assign(m->fun_tag, m->fun_tag + 4 * (size_t)m->n_tet);
    o->mat.assign(m->mat, m->mat + 3 * (size_t)m->n_mat);
    o->p = degree; o->Np = (degree + 1) * (degree + 2) * (degree + 3) / 6; o->nd = 3 * o->Np;
    o->alpha = alpha; o->theta = theta; o->dt = dt;
    o->Q = make_quadrature(degree);
    tria2tetfaces_maps(o->nm);
    o->blist.assign(3 * o->Np, 0);
    basis_list(degree, o->Np, o->blist.data());
    geometry(*o);
    for (int k = 0; k < 4; ++k) o->slot[k].assign((size_t)o->n_poly * o->nd, 0.0);
    o->rhs_stat.assign((size_t)o->n_poly * o->nd, 0.0);
    o->rhs_dyn.assign((size_t)o->n_poly * o->nd, 0.0);
    *out = o;
    return 0;
}

int oracle_destroy(void* h) { delete (Oracle*)h; return 0; }

int oracle_make_matrices(void* h) { return make_matrices(*(Oracle*)h); }

int oracle_make_rhs(void* h, int which, int f, int d, int n) { return make_rhs(*(Oracle*)h, which, f, d, n); }

int oracle_modal_project(void* h, int fun_id, int slot, double scale) {
    Oracle& o = *(Oracle*)h;
    if (!o.have_matrices) return LYMPH_ERR_ORDER;
    std::vector<double> out;
    modal_project(o, fun_id, out);
    if (scale != 1.0)
        for (auto& v : out) v = 0.0 * 0.0 + v * scale;  // u0 = v0*0 + u0*g(t), Lymph3D.f90:465
    o.slot[slot] = out;
    return 0;
}

// FIRST_TIME_STEP_MATRIX_FREE: UN = half_dt2*tmp + U0 + dt*V0.
int oracle_first_step(void* h, double t) {
    Oracle& o = *(Oracle*)h;
    int nd = o.nd;
    double half_dt2 = 0.5 * (o.dt * o.dt);
    std::vector<double> un((size_t)o.n_poly * nd);
#pragma omp parallel for schedule(static)
    for (int P = 0; P < o.n_poly; ++P) {
        if (!o.abs_idx.empty() && o.abs_idx[P] >= 0) {
            absorbing_first_step(o, t, P, &un[(size_t)P * nd]);
            continue;
        }
        std::vector<double> x;
        apply_and_solve(o, o.slot[LYMPH_SLOT_U0], t, P, x);
        for (int r = 0; r < nd; ++r) {
            const size_t q = (size_t)P * nd + r;
            if (g_device_order)
                un[q] = std::fma(o.dt, o.slot[LYMPH_SLOT_V0][q], std::fma(half_dt2, x[r], o.slot[LYMPH_SLOT_U0][q]));
            else
                un[q] = half_dt2 * x[r] + o.slot[LYMPH_SLOT_U0][q] + o.dt * o.slot[LYMPH_SLOT_V0][q];
        }
    }
    o.slot[LYMPH_SLOT_UN] = un;
    return 0;
}

// TIME_STEP_MATRIX_FREE + driver rotation: usol = dt2*x + 2*un - u0; u0 = un; un = usol.
int oracle_step(void* h, double t) {
    Oracle& o = *(Oracle*)h;
    int nd = o.nd;
    double dt2 = o.dt * o.dt;
    std::vector<double> us((size_t)o.n_poly * nd);
#pragma omp parallel for schedule(static)
    for (int P = 0; P < o.n_poly; ++P) {
        if (!o.abs_idx.empty() && o.abs_idx[P] >= 0) {
            absorbing_step(o, t, P, &us[(size_t)P * nd]);
            continue;
        }
        std::vector<double> x;
        apply_and_solve(o, o.slot[LYMPH_SLOT_UN], t, P, x);
        for (int r = 0; r < nd; ++r) {
            const size_t q = (size_t)P * nd + r;
            if (g_device_order)
                us[q] = std::fma(dt2, x[r], 2.0 * o.slot[LYMPH_SLOT_UN][q]) - o.slot[LYMPH_SLOT_U0][q];
            else
                us[q] = dt2 * x[r] + 2.0 * o.slot[LYMPH_SLOT_UN][q] - o.slot[LYMPH_SLOT_U0][q];
        }
    }
    o.slot[LYMPH_SLOT_U0].swap(o.slot[LYMPH_SLOT_UN]);
    o.slot[LYMPH_SLOT_UN].swap(us);
    return 0;
}

// The time loop of Lymph3D.f90:389-418 (t accumulated by repeated addition).
int oracle_run_steps(void* h, double stop_time, int64_t max_steps, double* t_inout, int64_t* n_done) {
    Oracle& o = *(Oracle*)h;
    double t = *t_inout;
    int64_t n = 0;
    while (t <= stop_time && (max_steps < 0 || n < max_steps)) {
        oracle_step(h, t);
        t = t + o.dt;
        ++n;
    }
    *t_inout = t;
    if (n_done) *n_done = n;
    return 0;
}

int oracle_get_state(void* h, int slot, double* out) {
    Oracle& o = *(Oracle*)h;
    std::memcpy(out, o.slot[slot].data(), sizeof(double) * o.slot[slot].size());
    return 0;
}

int oracle_set_state(void* h, int slot, const double* in) {
    Oracle& o = *(Oracle*)h;
    std::memcpy(o.slot[slot].data(), in, sizeof(double) * o.slot[slot].size());
    return 0;
}

// COMPUTE_ERROR_L2_MATRIX_FREE, matrix_free.f90:1388-1418.
int oracle_error_l2(void* h, int s_uh, int s_uex, double* out) {
    Oracle& o = *(Oracle*)h;
    int Np = o.Np, nd = o.nd;
    double err = 0.0;
    std::vector<double> du(Np), tmp(Np);
    for (int P = 0; P < o.n_poly; ++P)
        for (int i = 0; i < 3; ++i) {
            for (int m = 0; m < Np; ++m)
                du[m] = o.slot[s_uh][(size_t)P * nd + i * Np + m] - o.slot[s_uex][(size_t)P * nd + i * Np + m];
            const double* Mm = &o.Mm[(size_t)P * Np * Np];
            for (int r = 0; r < Np; ++r) {
                double s = 0.0;
                for (int c = 0; c < Np; ++c) s = s + Mm[r * Np + c] * du[c];
                tmp[r] = s;
            }
            double e = 0.0;
            for (int m = 0; m < Np; ++m) e = e + du[m] * tmp[m];
            err = err + e;
        }
    *out = err;
    return 0;
}

// COMPUTE_ERROR_DG_MATRIX_FREE, matrix_free.f90:1421-1504.
int oracle_error_dg(void* h, int s_uh, int s_uex, double* out) {
    Oracle& o = *(Oracle*)h;
    if (!o.have_dg) { g_err = "oracle: the A_dg blocks were not assembled"; return LYMPH_ERR_ORDER; }
    int nd = o.nd;
    std::vector<double> du(o.slot[s_uh].size());
    for (size_t k = 0; k < du.size(); ++k) du[k] = o.slot[s_uh][k] - o.slot[s_uex][k];
    double err = 0.0;
    std::vector<double> tmp(nd);
    for (int P = 0; P < o.n_poly; ++P) {
        std::fill(tmp.begin(), tmp.end(), 0.0);
        for (size_t b = 0; b < o.nbr[P].size(); ++b) {
            const double* Ab = &o.A[P][b * nd * nd];
            const double* dq = &du[(size_t)o.nbr[P][b] * nd];
            for (int r = 0; r < nd; ++r) {
                double s = 0.0;
                for (int c = 0; c < nd; ++c) s = s + Ab[r * nd + c] * dq[c];
                tmp[r] = tmp[r] + s;
            }
        }
        double e = 0.0;
        for (int r = 0; r < nd; ++r) e = e + du[(size_t)P * nd + r] * tmp[r];
        err = err + e;
    }
    *out = err;
    return 0;
}

// Pattern / blocks in the same convention as lymph_get_pattern/lymph_get_blocks
// except for the neighbour order within a row (here: first appearance in the
// tet/face loop).  n_blocks_out gets the total count when row_ptr is NULL.
// det4 (vet_mat_operations.f90:52-69), cofactor expansion along row 1.
double det4(const double A[4][4]) {
    return A[0][0] * (A[1][1] * (A[2][2] * A[3][3] - A[2][3] * A[3][2]) - A[1][2] * (A[2][1] * A[3][3] - A[2][3] * A[3][1]) +
                      A[1][3] * (A[2][1] * A[3][2] - A[2][2] * A[3][1])) -
           A[0][1] * (A[1][0] * (A[2][2] * A[3][3] - A[2][3] * A[3][2]) - A[1][2] * (A[2][0] * A[3][3] - A[2][3] * A[3][0]) +
                      A[1][3] * (A[2][0] * A[3][2] - A[2][2] * A[3][0])) +
           A[0][2] * (A[1][0] * (A[2][1] * A[3][3] - A[2][3] * A[3][1]) - A[1][1] * (A[2][0] * A[3][3] - A[2][3] * A[3][0]) +
                      A[1][3] * (A[2][0] * A[3][1] - A[2][1] * A[3][0])) -
           A[0][3] * (A[1][0] * (A[2][1] * A[3][2] - A[2][2] * A[3][1]) - A[1][1] * (A[2][0] * A[3][2] - A[2][2] * A[3][0]) +
                      A[1][2] * (A[2][0] * A[3][1] - A[2][1] * A[3][0]));
}

// The double-couple load of MAKE_RHS_FREE (matrix_free.f90:602-664): volume
// (find_tet.f90:184-210), moment_density (problem_data_and_properties.f90:
// 317-335), MAKE_DOUBLE_COUPLE (assemble_element.f90:116-167), added to the
// rows of the polyhedron of tetrahedron t in RHS `which`.
int oracle_make_rhs_double_couple(void* h, int which, int t, const double* sv, const double* nv, double M0) {
    Oracle& o = *(Oracle*)h;
    if (t < 0 || t >= o.n_tet || (which != 0 && which != 1)) return LYMPH_ERR_INVALID;
    if (!o.have_matrices) return LYMPH_ERR_ORDER;
    double A[4][4];
    for (int v = 0; v < 4; ++v) {
        for (int k = 0; k < 3; ++k) A[v][k] = o.coords[(size_t)o.tet_vert[t * 4 + v] * 3 + k];
        A[v][3] = 1.0;
    }
    const double vol = std::fabs(det4(A)) / 6.0;
    double moment[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) moment[i][j] = sv[i] * nv[j] + sv[j] * nv[i];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) moment[i][j] = moment[i][j] * M0 / vol;
    const int P = o.tet_poly[t], Np = o.Np;
    std::vector<double> phi, dphi;
    basis_tet(o, t, P, phi, dphi);
    std::vector<double> couple(3 * Np, 0.0);
    const double aj = std::fabs(o.jdet[t]);
    for (int q = 0; q < o.Q.nq3; ++q)
        for (int m = 0; m < Np; ++m)
            for (int i = 0; i < 3; ++i) {
                double reduct = 0.0;
                for (int j = 0; j < 3; ++j) reduct = reduct + moment[i][j] * dphi[q * 3 * Np + j * Np + m];
                couple[i * Np + m] = couple[i * Np + m] + o.Q.weitet3[q] * aj * reduct;
            }
    std::vector<double>& rhs = which == 0 ? o.rhs_stat : o.rhs_dyn;
    if (rhs.empty()) rhs.assign((size_t)o.n_poly * o.nd, 0.0);
    for (int r = 0; r < 3 * Np; ++r) rhs[(size_t)P * o.nd + r] += couple[r];
    return 0;
}

// EXPORT_SOLUTION's evaluation loop (solution_processing.f90:62-194):
// out[t][v][k] = sum_i u(i, (k-1) Npoly + P) LegendreP_x LegendreP_y
// LegendreP_z at the v-th vertex of tetrahedron t, summed in the reference's
// order (temp = temp + u * valx * valy * valz, i = 1..Np).
int oracle_nodal_values(void* h, int slot, double* out) {
    Oracle& o = *(Oracle*)h;
    if (slot < 0 || slot > 3) return LYMPH_ERR_INVALID;
    const std::vector<double>& u = o.slot[slot];
    if (o.bbox.empty() || u.empty()) return LYMPH_ERR_ORDER;
    const int Np = o.Np, nd = o.nd;
    for (int k = 0; k < 3; ++k)
        for (int t = 0; t < o.n_tet; ++t) {
            const int P = o.tet_poly[t];
            double bb[3][2];
            get_bb(o, P, bb);
            for (int v = 0; v < 4; ++v) {
                const double* x = &o.coords[(size_t)o.tet_vert[t * 4 + v] * 3];
                double temp = 0.0;
                for (int i = 0; i < Np; ++i) {
                    const double vx = legendre(x[0], o.blist[i * 3 + 0], bb[0][0], bb[0][1]);
                    const double vy = legendre(x[1], o.blist[i * 3 + 1], bb[1][0], bb[1][1]);
                    const double vz = legendre(x[2], o.blist[i * 3 + 2], bb[2][0], bb[2][1]);
                    temp = temp + u[(size_t)P * nd + k * Np + i] * vx * vy * vz;
                }
                out[((size_t)t * 4 + v) * 3 + k] = temp;
            }
        }
    return 0;
}

// The neighbour product K_PQ u_Q evaluated point by point instead of from the
// assembled block: the contraction the matrix-free mixed path applies on the
// device (csrc/mf.cu), in FP64 with this oracle's face points, bases, normals
// and penalty (MAKE_STIFFNESS_FACE, assemble_element.f90:404-661, inserted as
// in matrix_free.f90:412-433).  Per quadrature point of a triangle of P's
// tetrahedron t shared with Q, with v = u_Q(x), D_jk = d_k u_Q,j (x):
//   out_(i,a) += sum_k d_k phi^P_a G_ik + phi^P_a s_i,
//   G_ik = -theta/2 W (lambda (n.v) delta_ik + mu (n_i v_k + v_i n_k)),
//   s_i  = -W (sigma (T v)_i + h_i / 2),
//   h_i  = lambda sum_j n_j D_ji + mu n_i tr D + mu sum_k n_k D_ik.
// Test infrastructure: it checks that rearrangement against the assembled
// block.
// The point-wise form of the neighbour product with the reference's triangle
// rule (nodtria2 / weitria2, mapping_quadrature_2D, Poly_ref_mappings.f90:137-186).
int oracle_neighbour_apply_pointwise(void* h, int P, int Qp, const double* uq, double* out) {
    const Oracle& o = *(const Oracle*)h;
    return neighbour_apply_rule(o, P, Qp, uq, o.Q.nq2, o.Q.nodtria2.data(), o.Q.weitria2.data(), out);
}

// The same with a caller's triangle rule: xyw holds (xi, eta, w) per node.
int oracle_neighbour_apply_rule(void* h, int P, int Qp, const double* uq, int nq, const double* xyw, double* out) {
    const Oracle& o = *(const Oracle*)h;
    if (nq <= 0 || !xyw) return LYMPH_ERR_INVALID;
    std::vector<double> node4(4 * (size_t)nq), w(nq);
    for (int q = 0; q < nq; ++q) {
        node4[4 * q + 0] = xyw[3 * q + 0];
        node4[4 * q + 1] = xyw[3 * q + 1];
        node4[4 * q + 2] = 1.0;
        node4[4 * q + 3] = 1.0;
        w[q] = xyw[3 * q + 2];
    }
    return neighbour_apply_rule(o, P, Qp, uq, nq, node4.data(), w.data(), out);
}

int oracle_get_pattern(void* h, int32_t* row_ptr, int32_t* col, int64_t* n_blocks_out) {
    Oracle& o = *(Oracle*)h;
    int64_t nb = 0;
    for (int P = 0; P < o.n_poly; ++P) {
        if (row_ptr) row_ptr[P] = (int32_t)nb;
        for (size_t b = 0; b < o.nbr[P].size(); ++b) {
            if (col) col[nb] = o.nbr[P][b];
            ++nb;
        }
    }
    if (row_ptr) row_ptr[o.n_poly] = (int32_t)nb;
    if (n_blocks_out) *n_blocks_out = nb;
    return 0;
}

int oracle_get_blocks(void* h, int which, double* vals) {
    Oracle& o = *(Oracle*)h;
    if (which != LYMPH_BLOCKS_K && !o.have_dg) { g_err = "oracle: the A_dg blocks were not assembled"; return LYMPH_ERR_ORDER; }
    size_t off = 0, bs = (size_t)o.nd * o.nd;
    for (int P = 0; P < o.n_poly; ++P) {
        const std::vector<double>& src = (which == LYMPH_BLOCKS_K) ? o.K[P] : o.A[P];
        std::memcpy(vals + off, src.data(), sizeof(double) * o.nbr[P].size() * bs);
        off += o.nbr[P].size() * bs;
    }
    return 0;
}

int oracle_get_mass(void* h, int which, double* vals) {
    Oracle& o = *(Oracle*)h;
    const std::vector<double>* src[4] = {&o.M, &o.Mm, &o.R, &o.Rm};
    std::memcpy(vals, src[which]->data(), sizeof(double) * src[which]->size());
    return 0;
}

int oracle_get_rhs(void* h, int which, double* vals) {
    Oracle& o = *(Oracle*)h;
    const std::vector<double>& src = (which == LYMPH_RHS_STAT) ? o.rhs_stat : o.rhs_dyn;
    std::memcpy(vals, src.data(), sizeof(double) * src.size());
    return 0;
}

int oracle_get_poly_geometry(void* h, double* bbox, double* hk) {
    Oracle& o = *(Oracle*)h;
    if (bbox) std::memcpy(bbox, o.bbox.data(), sizeof(double) * o.bbox.size());
    if (hk) std::memcpy(hk, o.hk.data(), sizeof(double) * o.hk.size());
    return 0;
}

// Reference-layout (mode A) export of K_loc / A_dg_loc as the Fortran arrays
// K_loc(ie, 1:5, 3Np, 3Np): C array [5][nd][nd][n_poly] (column-major, ie
// fastest); block f+1 is the neighbour across face f (zero on boundary faces).
int oracle_get_kloc_reference_layout(void* h, int which, double* out) {
    Oracle& o = *(Oracle*)h;
    if (o.n_poly != o.n_tet) { g_err = "reference layout needs one tet per polyhedron"; return LYMPH_ERR_INVALID; }
    if (which != LYMPH_BLOCKS_K && !o.have_dg) { g_err = "oracle: the A_dg blocks were not assembled"; return LYMPH_ERR_ORDER; }
    int nd = o.nd;
    size_t ne = o.n_poly;
    std::fill(out, out + 5 * (size_t)nd * nd * ne, 0.0);
    for (int P = 0; P < o.n_poly; ++P) {
        const std::vector<double>& src = (which == LYMPH_BLOCKS_K) ? o.K[P] : o.A[P];
        for (int slot = 0; slot < 5; ++slot) {
            int b = -1;
            if (slot == 0) b = 0;
            else {
                int E2 = o.neigh[P * 4 + slot - 1];
                if (E2 >= 0) {
                    for (size_t k = 0; k < o.nbr[P].size(); ++k) if (o.nbr[P][k] == o.tet_poly[E2]) b = (int)k;
                }
            }
            if (b < 0) continue;
            for (int r = 0; r < nd; ++r)
                for (int c = 0; c < nd; ++c)
                    out[(((size_t)c * nd + r) * 5 + slot) * ne + P] = src[(size_t)b * nd * nd + r * nd + c];
        }
    }
    return 0;
}

// Quadrature / basis access for the known-answer tests.
int oracle_quadrature(int degree, int* nq3, int* nq2, double* nodtet3, double* weitet3, double* nodtria2, double* weitria2) {
    Quadrature Q = make_quadrature(degree);
    *nq3 = Q.nq3; *nq2 = Q.nq2;
    if (nodtet3) std::memcpy(nodtet3, Q.nodtet3.data(), sizeof(double) * Q.nodtet3.size());
    if (weitet3) std::memcpy(weitet3, Q.weitet3.data(), sizeof(double) * Q.weitet3.size());
    if (nodtria2) std::memcpy(nodtria2, Q.nodtria2.data(), sizeof(double) * Q.nodtria2.size());
    if (weitria2) std::memcpy(weitria2, Q.weitria2.data(), sizeof(double) * Q.weitria2.size());
    return 0;
}

int oracle_gl1d(int n, double* x, double* w) {
    std::vector<double> a, b;
    gl1d(n, a, b);
    std::memcpy(x, a.data(), sizeof(double) * n);
    std::memcpy(w, b.data(), sizeof(double) * n);
    return 0;
}

int oracle_gauleg(int n, double* x, double* w) { gauleg(-1, 1, n, x, w); return 0; }

int oracle_basis_list(int p, int* blist) {
    int Np = (p + 1) * (p + 2) * (p + 3) / 6;
    basis_list(p, Np, blist);
    return Np;
}

int oracle_legendre(int n, const double* x, int p, double a, double b, double* val, double* der) {
    for (int i = 0; i < n; ++i) {
        if (val) val[i] = legendre(x[i], p, a, b);
        if (der) der[i] = grad_legendre(x[i], p, a, b);
    }
    return 0;
}

int oracle_cholesky(const double* a, int dim, double* r) { return cholesky(a, dim, r) ? 0 : LYMPH_EXIT_SINGULARMTX; }

int oracle_solve_lu(const double* r, const double* b, int dim, double* x) { solve_LU_RT_R(r, b, dim, x); return 0; }

double oracle_time_function(double t) { return time_function(t); }

// Independent face matching (restates FIND_NEIGHBOUR_EL,
// MAKE_PARTITION_AND_MPI_FILES.f90:2536-2580, with a sorted-key map instead of
// the O(n^2) scan): neigh[t*4+f] = neighbour tet or -1 when unmatched.
int oracle_match_faces(int n_tet, const int32_t* tet_vert, int32_t* neigh, int32_t* neigh_face) {
    static const int FV[4][3] = {{0, 1, 2}, {0, 1, 3}, {1, 2, 3}, {2, 0, 3}};
    std::map<std::array<int, 3>, std::pair<int, int>> seen;
    for (int t = 0; t < n_tet; ++t)
        for (int f = 0; f < 4; ++f) { neigh[t * 4 + f] = -1; if (neigh_face) neigh_face[t * 4 + f] = -1; }
    for (int t = 0; t < n_tet; ++t)
        for (int f = 0; f < 4; ++f) {
            std::array<int, 3> k = {tet_vert[t * 4 + FV[f][0]], tet_vert[t * 4 + FV[f][1]], tet_vert[t * 4 + FV[f][2]]};
            std::sort(k.begin(), k.end());
            auto it = seen.find(k);
            if (it == seen.end()) seen[k] = {t, f};
            else {
                int t2 = it->second.first, f2 = it->second.second;
                neigh[t * 4 + f] = t2; neigh[t2 * 4 + f2] = t;
                if (neigh_face) { neigh_face[t * 4 + f] = f2; neigh_face[t2 * 4 + f2] = f; }
                seen.erase(it);
            }
        }
    return 0;
}

}  // extern "C"
