// common.cuh -- context, error plumbing and shared device helpers of the
// GB300 PolyDG library.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>
#include <nvtx3/nvToolsExt.h>

#include "../../include/lymph3d_gpu.h"

// ---------------------------------------------------------------------------
// error plumbing
// ---------------------------------------------------------------------------
void lymph_set_error(const std::string& msg);

#define LYMPH_CUDA_TRY(expr)                                                             \
    do {                                                                                 \
        cudaError_t _e = (expr);                                                         \
        if (_e != cudaSuccess) {                                                         \
            lymph_set_error(std::string(#expr) + ": " + cudaGetErrorString(_e));         \
            return (_e == cudaErrorMemoryAllocation) ? LYMPH_ERR_OOM : LYMPH_ERR_CUDA;   \
        }                                                                                \
    } while (0)

#define LYMPH_TRY(expr)            \
    do {                           \
        int _rc = (expr);          \
        if (_rc != LYMPH_OK) return _rc; \
    } while (0)

// Device status word bits (set by kernels, read back by the host).
enum : int {
    ST_NOT_SPD = 1,      // Cholesky pivot <= 0
    ST_NONFINITE = 2,    // NaN/Inf in a state vector
    ST_BAD_INDEX = 4,    // an index failed its bounds check
    ST_DEGENERATE = 8,   // zero-volume tetrahedron / zero-area face
    ST_TIMEOUT = 16,     // a bounded wait on an asynchronous copy expired
};

constexpr int MAX_DEGREE = 4;     // device path supports p = 1..4 (Np <= 35)
constexpr int MAX_NP = 35;
constexpr int MAX_NQ3 = 125;
constexpr int MAX_NQ2 = 25;

// ---------------------------------------------------------------------------
// reference tables in device memory (one copy per context, degree-specific)
// ---------------------------------------------------------------------------
struct RefTables {
    double nodtet3[MAX_NQ3 * 4];   // [q][4]  mapped Duffy nodes (xi, eta, zeta, 1)
    double weitet3[MAX_NQ3];
    double nodtria2[MAX_NQ2 * 4];  // [q][4]  (s, t, 1, 1)
    double weitria2[MAX_NQ2];
    double node_maps[4 * 16];      // [face][row][col]
    int blist[MAX_NP * 3];         // [f][3]
};

// ---------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------
struct lymph_ctx {
    // method
    int p = 1, Np = 4, nd = 12, nq3 = 8, nq2 = 4, precision = LYMPH_FP64;
    double alpha = 10.0, theta = -1.0, dt = 1e-3;
    // sizes
    int n_node = 0, n_tet = 0, n_poly = 0, n_mat = 0;
    uint64_t mesh_hash = 0;         // FNV-1a of the mesh descriptor's arrays (checkpoints carry it)
    uint64_t uid = 0;               // unique per context in the process (caches keyed by context)
    int64_t rhs_version = 0;        // bumped whenever rhs_dyn or M^-1 change (caches of M^-1 F)
    int64_t n_blocks = 0, n_face_sides = 0, n_block_faces = 0;
    cudaStream_t stream = nullptr;
    // host copies needed for set-up logic
    std::vector<int32_t> h_row_ptr, h_col;
    // device mesh
    double* d_coords = nullptr;
    int32_t *d_tet_vert = nullptr, *d_tet_poly = nullptr, *d_tet_mat = nullptr, *d_neigh = nullptr, *d_fun_tag = nullptr;
    double* d_mat = nullptr;
    RefTables* d_ref = nullptr;
    // derived geometry
    double *d_fk = nullptr, *d_jdet = nullptr, *d_normal = nullptr, *d_area = nullptr;
    double *d_bbox = nullptr, *d_hk = nullptr;
    int32_t *d_poly_ptr = nullptr, *d_poly_tets = nullptr;
    // block pattern: row_ptr[n_poly+1], col[n_blocks], blk_row[n_blocks],
    // face lists per block bf_ptr[n_blocks+1] / bf[...] (encoded t*4+f)
    int32_t *d_row_ptr = nullptr, *d_col = nullptr, *d_blk_row = nullptr;
    int64_t* d_bf_ptr = nullptr;
    int32_t* d_bf = nullptr;
    // operator
    void* d_K = nullptr;            // [n_blocks][nd][nd] column-major per block (FP64 or FP32)
    float* d_K32 = nullptr;         // FP32 copy of FP64 blocks for the surrogate's operator apply (on demand)
    bool k32_valid = false;
    bool surrogate_apply_fp32 = false;  // lymph_surrogate_apply_fp32
    double *d_M = nullptr, *d_Mm = nullptr, *d_R = nullptr, *d_Rm = nullptr, *d_RT = nullptr, *d_RmT = nullptr;
    double* d_Minv = nullptr;       // [n_poly][Np][Np] column-major inverse of M_loc
    // absorbing faces (LYMPH_BC_ABSO): the n_abs polyhedra that have some,
    // their faces (CSR over d_abs_ptr, codes t*4+f), each polyhedron's index
    // among them (-1 for the others), the damping block D (symmetric) and the
    // column-major inverse of W = M (x) I + dt/2 D of each, [n_abs][nd][nd]
    int n_abs = 0;
    int32_t *d_abs_idx = nullptr, *d_abs_poly = nullptr, *d_abs_ptr = nullptr, *d_abs_faces = nullptr;
    double *d_Dabs = nullptr, *d_Winv = nullptr, *d_Wabs = nullptr, *d_Rw = nullptr, *d_RwT = nullptr;
    double winv_dt = 0.0;           // the dt the W inverses were made for
    // matrix-free neighbour terms (LYMPH_MIXED_MF): d_K holds the n_poly FP32
    // self blocks; d_mf_tri the FP32 geometry of every neighbour-block
    // triangle (parallel to d_bf), d_mf_poly the Legendre map of every
    // bounding box, mf_quad the triangle quadrature (xi, eta, w)
    void* d_mf_tri = nullptr;
    void* d_mf_poly = nullptr;
    void* d_mf_u32 = nullptr;       // the operator input in FP32, [n_poly][Np] x 4
    void* d_mf_range = nullptr;     // per polyhedron: its triangles' range and neighbours (mf.cu k_mf_qrec)
    float mf_quad[3 * 25] = {};
    double *d_rhs_stat = nullptr, *d_rhs_dyn = nullptr;
    // state: two rotating step buffers + V0 + UEX
    double* d_buf[2] = {nullptr, nullptr};
    int cur = 1;                    // d_buf[cur] holds UN, d_buf[cur^1] holds U0
    double *d_v0 = nullptr, *d_uex = nullptr;
    // misc
    double* d_gvals = nullptr;      // time-function values of a run
    int64_t gvals_cap = 0;
    int64_t* d_step_idx = nullptr;
    double* d_partial = nullptr;    // per-polyhedron partial sums (error norms)
    double* d_scalar = nullptr;
    double* d_layout = nullptr;     // staging of a state in the reference's (ie, k) layout (allocated on first use)
    double* d_layout2 = nullptr;    // a second staging buffer (lymph_time_step_host's u^{n-1})
    cudaStream_t stream2 = nullptr; // lymph_time_step_host: the second upload runs on its own copy engine
    cudaEvent_t ev_copy = nullptr;
    int* h_status = nullptr;        // page-locked copy of d_status (read without a second round trip)
    int* d_status = nullptr;
    bool have_matrices = false, have_rhs_stat = false, have_rhs_dyn = false;
    int64_t launches = 0;
    int64_t device_bytes = 0;
    cudaGraphExec_t graph_exec = nullptr;
    int graph_steps = 0;
    int64_t graph_launches = 0;     // kernel launches one graph launch stands for
    int graph_parity = -1;
};

// A named NVTX range over the host-side extent of a C-ABI call or a graph
// launch (visible to nsys and to ncu's --nvtx filters; no cost when no tool
// is attached).
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

double* lymph_slot_ptr(lymph_ctx* c, int slot);

// ---------------------------------------------------------------------------
// device helpers: the reference's Legendre evaluation on a bounding-box
// interval (basis_function.f90:268-437), one point, one degree.
// ---------------------------------------------------------------------------
__host__ __device__ inline double lp_nonnorm(double xp, int p) {
    double x2 = xp * xp, x3 = x2 * xp, x4 = x2 * x2, x5 = x4 * xp, x6 = x3 * x3;
    switch (p) {
        case 0: return 1.0;
        case 1: return xp;
        case 2: return (3 * x2 - 1) / 2;
        case 3: return (5 * x3 - 3 * xp) / 2;
        case 4: return (35 * x4 - 30 * x2 + 3) / 8;
        case 5: return (63 * x5 - 70 * x3 + 15 * xp) / 8;
        case 6: return (231 * x6 - 315 * x4 + 105 * x2 - 5) / 16;
        default: return 0.0;
    }
}

__host__ __device__ inline double lp_der_nonnorm(double xp, int p) {
    double x2 = xp * xp, x3 = x2 * xp, x4 = x2 * x2, x5 = x4 * xp;
    switch (p) {
        case 0: return 0.0;
        case 1: return 1.0;
        case 2: return 3 * xp;
        case 3: return (15 * x2 - 3) / 2;
        case 4: return (35 * x3 - 15 * xp) / 2;
        case 5: return (315 * x4 - 210 * x2 + 15) / 8;
        case 6: return (1386 * x5 - 1260 * x3 + 210 * xp - 5) / 16;
        default: return 0.0;
    }
}

// Value and derivative of the scaled Legendre polynomial of degree p on
// [a,b] at x: L_p(xp)/sqrt(hb) and L'_p(xp)/(hb sqrt(hb)) with
// xp = (x - mb)/hb (LegendreP / GradLegendreP).
__host__ __device__ inline void legendre_1d(double x, int p, double a, double b, double* v, double* d) {
    double hb = (b - a) / 2.0, mb = (b + a) / 2.0;
    double xp = (x - mb) / hb;
    double sh = sqrt(hb);
    *v = lp_nonnorm(xp, p) / sh;
    *d = lp_der_nonnorm(xp, p) / (hb * sh);
}

// Basis function f and its gradient at physical point pt for bounding box
// bb (xmin,xmax,ymin,ymax,zmin,zmax): phi = Lx Ly Lz, dphi = (Lx' Ly Lz,
// Lx Ly' Lz, Lx Ly Lz') (basis, basis_function.f90:508-513).
__host__ __device__ inline void basis_eval(const double pt[3], const double* bb, const int* bl, double* phi,
                                           double* dphi) {
    double vx, dx, vy, dy, vz, dz;
    legendre_1d(pt[0], bl[0], bb[0], bb[1], &vx, &dx);
    legendre_1d(pt[1], bl[1], bb[2], bb[3], &vy, &dy);
    legendre_1d(pt[2], bl[2], bb[4], bb[5], &vz, &dz);
    *phi = vx * vy * vz;
    dphi[0] = dx * vy * vz;
    dphi[1] = vx * dy * vz;
    dphi[2] = vx * vy * dz;
}

inline int np_of(int p) { return (p + 1) * (p + 2) * (p + 3) / 6; }

// ---------------------------------------------------------------------------
// the L2-norm bodies shared by the context path (step.cu) and the
// allocation-free entry point (noalloc.cu), so both give the same bits
// ---------------------------------------------------------------------------
// COMPUTE_ERROR_L2_MATRIX_FREE's body for polyhedron P
// (src/matrix_free.f90:1388-1418): sum_i du_i^T M du_i with du = uh - uex,
// M the Np x Np modal mass matrix, rows and columns in the reference's order.
__device__ __forceinline__ double l2_partial_poly(int P, int NP, const double* __restrict__ Mm,
                                                  const double* __restrict__ uh, const double* __restrict__ uex) {
    const int ND = 3 * NP;
    double err = 0.0;
    const double* M = Mm + (int64_t)P * NP * NP;
    for (int i = 0; i < 3; ++i) {
        double e = 0.0;
        for (int rr = 0; rr < NP; ++rr) {
            double t = 0.0;
            for (int c = 0; c < NP; ++c) {
                const int64_t qc = (int64_t)P * ND + i * NP + c;
                t = t + M[rr * NP + c] * (uh[qc] - uex[qc]);
            }
            const int64_t qr = (int64_t)P * ND + i * NP + rr;
            e = e + (uh[qr] - uex[qr]) * t;
        }
        err = err + e;
    }
    return err;
}

// Deterministic sum of v[0..n) by one CTA of 1024 threads: a fixed strided
// order per thread, then a fixed shared-memory tree; thread 0 writes *out.
__device__ __forceinline__ void sum_fixed_order_1024(int64_t n, const double* __restrict__ v, double* out) {
    __shared__ double red[1024];
    double s = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) s += v[i];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = red[0];
}

// ---------------------------------------------------------------------------
// FP32 basis tabulation shared by the mixed kernels (mf.cu, selftc.cu)
// ---------------------------------------------------------------------------
// The reference's basis order (basis_list, basis_function.f90:12-44): degree
// triples (x, y, z) for q1 = p..0, q2 = p-q1..0, q3 = p-q1-q2..0.
template <int PD> struct Blist {
    int d[(PD + 1) * (PD + 2) * (PD + 3) / 6][3];
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

// Legendre polynomials L_0..L_PD on [-1, 1] and their derivatives at x,
// as (L, L') pairs (Bonnet's recurrence; the reference evaluates the same
// polynomials in closed form, basis_function.f90:268-437).
template <int PD>
__device__ __forceinline__ void legendre_f32(float x, float2* out) {
    float Lv[PD + 1], Ld[PD + 1];
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
#pragma unroll
    for (int n = 0; n <= PD; ++n) out[n] = make_float2(Lv[n], Ld[n]);
}

// launch helpers (defined in abi.cu)
int lymph_sync_status(lymph_ctx* c, const char* where);
