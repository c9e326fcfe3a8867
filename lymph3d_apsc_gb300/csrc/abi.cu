// abi.cu -- implementation of the C ABI declared in include/lymph3d_gpu.h.
//
// Host responsibilities: validate and copy the flattened mesh, build the
// block pattern (which polyhedra couple through faces, which face-sides feed
// which block), the reference quadrature tables, the time-function values of
// a run, and the stream/graph orchestration.  Every floating-point operation
// on the data runs in device kernels (setup.cu, step.cu); there is no host
// compute fallback.

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <atomic>
#include <map>
#include <string>
#include <vector>

#include "common.cuh"

// kernels (setup.cu, step.cu)
int lymph_dev_geometry(lymph_ctx* c);
int lymph_dev_assemble(lymph_ctx* c, int which, void* out, int out_fp32, bool write_mass);
int lymph_dev_assemble_list(lymph_ctx* c, int which, void* out, int out_fp32, bool write_mass, const int64_t* list,
                            int64_t n_list, int64_t out_stride);
int lymph_mf_setup(lymph_ctx* c, const RefTables& R);
int lymph_dev_cholesky(lymph_ctx* c);
int lymph_dev_damping(lymph_ctx* c, bool assemble);
int lymph_dev_mass(lymph_ctx* c, const int64_t* self_list);
int lymph_dev_self_tc(lymph_ctx* c, float* out, bool block_csr);
int lymph_dev_nb_tc(lymph_ctx* c, float* out, const int64_t* list, int64_t n_list);
int lymph_dev_vector(lymph_ctx* c, int mode, int fid, int did, int nid, double scale, double* out);
int lymph_dev_step(lymph_ctx* c, bool bump);
int lymph_dev_first_step(lymph_ctx* c);
int lymph_dev_apply(lymph_ctx* c, const double* u, double* out);
int lymph_dev_ku(lymph_ctx* c, const double* u, double* out);
int lymph_dev_double_couple(lymph_ctx* c, int t, int P, const double moment[9], double* out);
int lymph_dev_power_iteration(lymph_ctx* c, double* x, double* y, double* d_ss, int iters);
int lymph_dev_point_source(lymph_ctx* c, int P, const double x0[3], const double dir[3], double* out);
int lymph_dev_bump(lymph_ctx* c);
int lymph_dev_error_dg(lymph_ctx* c, const void* blocks, const double* uh, const double* uex, double* d_out);
int lymph_dev_error_l2(lymph_ctx* c, const double* uh, const double* uex, double* d_out);
int lymph_dev_energy(lymph_ctx* c, const double* ua, const double* ub, double* d_out);

namespace {

thread_local std::string g_last_error;

const double PI = 3.14159265358979323846;

// 1D Gauss-Legendre nodes and weights in the reference's order
// (basis_function.f90:77-124).  Standard tables; the reference's order is
// kept because the tensor quadrature inherits it.
void gl_table(int nqn, std::vector<double>& x, std::vector<double>& w) {
    switch (nqn) {
        case 1: x = {0.0}; w = {2.0}; break;
        case 2: x = {std::sqrt(1.0 / 3.0), -std::sqrt(1.0 / 3.0)}; w = {1.0, 1.0}; break;
        case 3: x = {0.0, std::sqrt(3.0 / 5.0), -std::sqrt(3.0 / 5.0)}; w = {8.0 / 9.0, 5.0 / 9.0, 5.0 / 9.0}; break;
        case 4: {
            double s = std::sqrt(30.0);
            x = {0.3399810435848563, -0.3399810435848563, 0.8611363115940526, -0.8611363115940526};
            w = {(18 + s) / 36.0, (18 + s) / 36.0, (18 - s) / 36.0, (18 - s) / 36.0};
            break;
        }
        case 5: {
            double s = std::sqrt(70.0);
            x = {0.0, 0.5384693101056831, -0.5384693101056831, 0.9061798459386640, -0.9061798459386640};
            w = {128.0 / 225.0, (322 + 13 * s) / 900.0, (322 + 13 * s) / 900.0, (322 - 13 * s) / 900.0,
                 (322 - 13 * s) / 900.0};
            break;
        }
        default: x.clear(); w.clear();
    }
}

// Reference quadrature and maps for degree p: tensor Gauss-Legendre with
// p+1 points per direction (quadrature, basis_function.f90:47-161) collapsed
// onto the reference tetrahedron and triangle (mapping_quadrature_3D/2D,
// Poly_ref_mappings.f90:137-186), face maps (tria2tetfaces_maps :79-134) and
// the monomial degree list (basis_list, basis_function.f90:12-44).
bool build_ref_tables(int p, RefTables& R) {
    std::memset(&R, 0, sizeof(R));
    int nqn = p + 1;
    std::vector<double> x, w;
    gl_table(nqn, x, w);
    if ((int)x.size() != nqn) return false;
    int c = 0;
    for (int i = 0; i < nqn; ++i)
        for (int j = 0; j < nqn; ++j)
            for (int k = 0; k < nqn; ++k) {
                double a = 0.5 * x[i] + 0.5, b = 0.5 * x[j] + 0.5, cc = 0.5 * x[k] + 0.5;
                double wt = 0.125 * (w[i] * w[j] * w[k]);
                R.nodtet3[c * 4 + 0] = a;
                R.nodtet3[c * 4 + 1] = (1 - a) * b;
                R.nodtet3[c * 4 + 2] = (1 - a) * (1 - b) * cc;
                R.nodtet3[c * 4 + 3] = 1.0;
                R.weitet3[c] = std::fabs((1 - b) * ((1 - a) * (1 - a))) * wt;
                ++c;
            }
    c = 0;
    for (int i = 0; i < nqn; ++i)
        for (int j = 0; j < nqn; ++j) {
            double s = x[i], t = x[j];
            R.nodtria2[c * 4 + 0] = 0.5 * (1 + s);
            R.nodtria2[c * 4 + 1] = 0.25 * (1 - s) * (1 + t);
            R.nodtria2[c * 4 + 2] = 1.0;
            R.nodtria2[c * 4 + 3] = 1.0;
            R.weitria2[c] = std::fabs(0.125 * (1 - s)) * (w[i] * w[j]);
            ++c;
        }
    // node_maps[f][row][col]
    auto nm = [&](int f, int r, int cc) -> double& { return R.node_maps[f * 16 + r * 4 + cc]; };
    nm(0, 0, 1) = 1; nm(0, 1, 0) = 1; nm(0, 3, 3) = 1;
    nm(1, 0, 0) = 1; nm(1, 2, 1) = 1; nm(1, 3, 3) = 1;
    nm(2, 0, 0) = 1; nm(2, 1, 1) = 1; nm(2, 2, 2) = 1; nm(2, 3, 3) = 1; nm(2, 2, 0) = -1; nm(2, 2, 1) = -1;
    nm(3, 1, 1) = 1; nm(3, 2, 0) = 1; nm(3, 3, 3) = 1;
    int ii = 0;
    for (int q1 = p; q1 >= 0; --q1)
        for (int q2 = p - q1; q2 >= 0; --q2)
            for (int q3 = p - q1 - q2; q3 >= 0; --q3) {
                R.blist[ii * 3 + 0] = q1; R.blist[ii * 3 + 1] = q2; R.blist[ii * 3 + 2] = q3;
                ++ii;
            }
    return true;
}

template <typename T> int dalloc(lymph_ctx* c, T** p, size_t n) {
    *p = nullptr;
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc((void**)p, n * sizeof(T));
    if (e != cudaSuccess) {
        lymph_set_error(std::string("cudaMalloc(") + std::to_string(n * sizeof(T)) + " bytes): " + cudaGetErrorString(e));
        return LYMPH_ERR_OOM;
    }
    c->device_bytes += (int64_t)(n * sizeof(T));
    return LYMPH_OK;
}

template <typename T> int upload(lymph_ctx* c, T** p, const T* h, size_t n) {
    LYMPH_TRY(dalloc(c, p, n));
    if (n) LYMPH_CUDA_TRY(cudaMemcpyAsync(*p, h, n * sizeof(T), cudaMemcpyHostToDevice, c->stream));
    return LYMPH_OK;
}

void dfree(void* p) {
    if (p) cudaFree(p);
}

double time_function(double t) { return std::sin(std::sqrt(2.0) * PI * t); }  // problem_data_and_properties.f90:14-23

int set_g(lymph_ctx* c, double g) {
    LYMPH_CUDA_TRY(cudaMemcpyAsync(c->d_gvals, &g, sizeof(double), cudaMemcpyHostToDevice, c->stream));
    LYMPH_CUDA_TRY(cudaMemsetAsync(c->d_step_idx, 0, sizeof(int64_t), c->stream));
    return LYMPH_OK;
}

bool valid_slot(int s) { return s >= 0 && s < LYMPH_NUM_SLOTS; }

// FNV-1a (64-bit) over byte ranges: identifies the mesh a checkpoint belongs to.
struct Fnv64 {
    uint64_t h = 1469598103934665603ull;
    void add(const void* p, size_t n) {
        const unsigned char* b = (const unsigned char*)p;
        for (size_t i = 0; i < n; ++i) { h ^= b[i]; h *= 1099511628211ull; }
    }
    template <typename T> void add_value(T v) { add(&v, sizeof(v)); }
};

uint64_t mesh_hash(const lymph_mesh_desc* m) {
    Fnv64 f;
    f.add_value(m->n_node); f.add_value(m->n_tet); f.add_value(m->n_poly); f.add_value(m->n_mat);
    f.add(m->coords, sizeof(double) * 3 * (size_t)m->n_node);
    f.add(m->tet_vert, sizeof(int32_t) * 4 * (size_t)m->n_tet);
    f.add(m->tet_poly, sizeof(int32_t) * (size_t)m->n_tet);
    f.add(m->tet_mat, sizeof(int32_t) * (size_t)m->n_tet);
    f.add(m->neigh, sizeof(int32_t) * 4 * (size_t)m->n_tet);
    if (m->fun_tag) f.add(m->fun_tag, sizeof(int32_t) * 4 * (size_t)m->n_tet);
    f.add(m->mat, sizeof(double) * 3 * (size_t)m->n_mat);
    return f.h;
}

// The checkpoint file: this header, then u^{n-1} and u^n as [n_poly][3Np]
// doubles (the device layout), all in the host's byte order.
struct CheckpointHeader {
    char magic[8];          // "LYMPHCK1"
    int32_t version;        // 1
    int32_t precision;
    int32_t degree;
    int32_t reserved;
    uint64_t mesh_hash;
    int64_t n_poly, nd;
    double dt, alpha, theta;
    double t;               // the caller's time (the next step's t)
    int64_t steps;          // the caller's step count
};

// dst = src^T for a row-major rows x cols src (32 x 32 tiles through
// shared memory, so both sides are read and written in full lines).  The
// state's two layouts: [n_poly][3Np] on the device, the reference's u(ie, k)
// (column-major, element index fastest) = [3Np][n_poly] row-major on the host.
__global__ void k_transpose(const double* __restrict__ src, double* __restrict__ dst, int64_t rows, int64_t cols) {
    __shared__ double tile[32][33];
    const int64_t tiles_r = (rows + 31) / 32;   // one CTA per 32 x 32 tile, row tiles fastest
    const int64_t r0 = (int64_t)(blockIdx.x % tiles_r) * 32, c0 = (int64_t)(blockIdx.x / tiles_r) * 32;
    const int tx = threadIdx.x, ty = threadIdx.y;
    for (int j = ty; j < 32; j += 8) {
        const int64_t r = r0 + j, col = c0 + tx;
        if (r < rows && col < cols) tile[j][tx] = src[r * cols + col];
    }
    __syncthreads();
    for (int j = ty; j < 32; j += 8) {
        const int64_t col = c0 + j, r = r0 + tx;
        if (col < cols && r < rows) dst[col * rows + r] = tile[tx][j];
    }
}

int transpose(lymph_ctx* c, const double* src, double* dst, int64_t rows, int64_t cols, cudaStream_t st) {
    const int64_t tiles = ((rows + 31) / 32) * ((cols + 31) / 32);
    if (tiles <= 0) return LYMPH_OK;
    k_transpose<<<(unsigned)tiles, dim3(32, 8), 0, st>>>(src, dst, rows, cols);
    c->launches++;
    LYMPH_CUDA_TRY(cudaGetLastError());
    return LYMPH_OK;
}

int layout_buffer(lymph_ctx* c) {
    if (!c->d_layout) LYMPH_TRY(dalloc(c, &c->d_layout, (size_t)c->n_poly * c->nd));
    return LYMPH_OK;
}

}  // namespace

void lymph_set_error(const std::string& msg) { g_last_error = msg; }

double* lymph_slot_ptr(lymph_ctx* c, int slot) {
    switch (slot) {
        case LYMPH_SLOT_U0: return c->d_buf[c->cur ^ 1];
        case LYMPH_SLOT_UN: return c->d_buf[c->cur];
        case LYMPH_SLOT_V0: return c->d_v0;
        case LYMPH_SLOT_UEX: return c->d_uex;
        default: return nullptr;
    }
}

int status_rc(lymph_ctx* c, int st, const char* where);

int lymph_sync_status(lymph_ctx* c, const char* where) {
    LYMPH_CUDA_TRY(cudaStreamSynchronize(c->stream));
    int st = 0;
    LYMPH_CUDA_TRY(cudaMemcpy(&st, c->d_status, sizeof(int), cudaMemcpyDeviceToHost));
    return status_rc(c, st, where);
}

// The status word's meaning as a return code (and the word cleared).
int status_rc(lymph_ctx* c, int st, const char* where) {
    if (st == 0) return LYMPH_OK;
    LYMPH_CUDA_TRY(cudaMemset(c->d_status, 0, sizeof(int)));
    std::string w(where);
    if (st & ST_BAD_INDEX) { lymph_set_error(w + ": device index check failed"); return LYMPH_ERR_INDEX; }
    if (st & ST_NOT_SPD) { lymph_set_error(w + ": Matrix is not positive definite!"); return LYMPH_EXIT_SINGULARMTX; }
    if (st & ST_DEGENERATE) { lymph_set_error(w + ": degenerate tetrahedron or face"); return LYMPH_EXIT_SETUP; }
    if (st & ST_NONFINITE) { lymph_set_error(w + ": non-finite value in the state"); return LYMPH_EXIT_INSTAB; }
    if (st & ST_TIMEOUT) { lymph_set_error(w + ": a bounded wait on an asynchronous copy expired"); return LYMPH_ERR_TIMEOUT; }
    lymph_set_error(w + ": device status " + std::to_string(st));
    return LYMPH_ERR_CUDA;
}

extern "C" {

int lymph_version(void) { return 10000; }

const char* lymph_last_error(void) { return g_last_error.c_str(); }

int lymph_destroy(lymph_ctx* c) {
    if (!c) return LYMPH_OK;
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->graph_exec) cudaGraphExecDestroy(c->graph_exec);
    void* ptrs[] = {c->d_coords, c->d_tet_vert, c->d_tet_poly, c->d_tet_mat, c->d_neigh, c->d_fun_tag, c->d_mat,
                    c->d_ref, c->d_fk, c->d_jdet, c->d_normal, c->d_area, c->d_bbox, c->d_hk, c->d_poly_ptr,
                    c->d_poly_tets, c->d_row_ptr, c->d_col, c->d_blk_row, c->d_bf_ptr, c->d_bf, c->d_K, c->d_K32, c->d_M,
                    c->d_Mm, c->d_R, c->d_Rm, c->d_RT, c->d_RmT, c->d_Minv, c->d_rhs_stat, c->d_rhs_dyn, c->d_buf[0], c->d_buf[1],
                    c->d_v0, c->d_uex, c->d_gvals, c->d_step_idx, c->d_partial, c->d_scalar, c->d_status,
                    c->d_mf_tri, c->d_mf_poly, c->d_mf_u32, c->d_mf_range, c->d_layout};
    for (void* p : ptrs) dfree(p);
    dfree(c->d_layout2);
    void* absp[] = {c->d_abs_idx, c->d_abs_poly, c->d_abs_ptr, c->d_abs_faces, c->d_Dabs, c->d_Wabs, c->d_Rw, c->d_RwT,
                    c->d_Winv};
    for (void* p : absp) dfree(p);
    if (c->h_status) cudaFreeHost(c->h_status);
    if (c->ev_copy) cudaEventDestroy(c->ev_copy);
    if (c->stream2) cudaStreamDestroy(c->stream2);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return LYMPH_OK;
}

int lymph_create(const lymph_mesh_desc* m, const lymph_params* prm, lymph_ctx** out) {
    if (!out) { lymph_set_error("lymph_create: null output"); return LYMPH_ERR_INVALID; }
    *out = nullptr;
    if (!m || !prm || !m->coords || !m->tet_vert || !m->tet_poly || !m->tet_mat || !m->neigh || !m->mat) {
        lymph_set_error("lymph_create: null mesh array");
        return LYMPH_ERR_INVALID;
    }
    if (prm->degree < 1 || prm->degree > MAX_DEGREE) {
        lymph_set_error("lymph_create: degree must be 1..4 on the device");
        return LYMPH_ERR_INVALID;
    }
    if (prm->precision != LYMPH_FP64 && prm->precision != LYMPH_MIXED && prm->precision != LYMPH_MIXED_MF) {
        lymph_set_error("lymph_create: unknown precision");
        return LYMPH_ERR_INVALID;
    }
    if (m->n_tet <= 0 || m->n_poly <= 0 || m->n_node <= 0 || m->n_mat <= 0) {
        lymph_set_error("lymph_create: empty mesh");
        return LYMPH_EXIT_SETUP;
    }
    if (!(prm->dt > 0.0) || !std::isfinite(prm->dt)) {
        lymph_set_error("lymph_create: dt must be positive");
        return LYMPH_ERR_INVALID;
    }
    const int nt = m->n_tet, np = m->n_poly;
    // ---- validation ----
    for (int64_t i = 0; i < (int64_t)nt * 4; ++i)
        if (m->tet_vert[i] < 0 || m->tet_vert[i] >= m->n_node) { lymph_set_error("lymph_create: vertex id out of range"); return LYMPH_EXIT_SETUP; }
    std::vector<int32_t> cnt(np, 0);
    for (int t = 0; t < nt; ++t) {
        if (m->tet_poly[t] < 0 || m->tet_poly[t] >= np) { lymph_set_error("lymph_create: polyhedron id out of range"); return LYMPH_EXIT_SETUP; }
        if (m->tet_mat[t] < 0 || m->tet_mat[t] >= m->n_mat) { lymph_set_error("lymph_create: material id out of range"); return LYMPH_EXIT_SETUP; }
        cnt[m->tet_poly[t]]++;
    }
    for (int P = 0; P < np; ++P)
        if (cnt[P] == 0) { lymph_set_error("lymph_create: empty polyhedron " + std::to_string(P)); return LYMPH_EXIT_SETUP; }
    for (int t = 0; t < nt; ++t)
        for (int f = 0; f < 4; ++f) {
            int e = m->neigh[t * 4 + f];
            if (e == LYMPH_BC_DIRI || e == LYMPH_BC_NEUM || e == LYMPH_BC_ABSO) continue;
            if (e < 0 || e >= nt || e == t) { lymph_set_error("lymph_create: bad neighbour entry"); return LYMPH_EXIT_NEIGHBOUR_EL_ERROR; }
            bool back = false;
            for (int g = 0; g < 4; ++g) back |= (m->neigh[e * 4 + g] == t);
            if (!back) { lymph_set_error("lymph_create: neighbour table not symmetric"); return LYMPH_EXIT_NEIGHBOUR_EL_ERROR; }
        }
    lymph_ctx* c = new lymph_ctx();
    c->p = prm->degree; c->Np = np_of(c->p); c->nd = 3 * c->Np;
    c->nq3 = (c->p + 1) * (c->p + 1) * (c->p + 1); c->nq2 = (c->p + 1) * (c->p + 1);
    c->precision = prm->precision; c->alpha = prm->alpha; c->theta = prm->theta; c->dt = prm->dt;
    c->n_node = m->n_node; c->n_tet = nt; c->n_poly = np; c->n_mat = m->n_mat;
    c->mesh_hash = mesh_hash(m);
    {
        static std::atomic<uint64_t> next_uid{1};
        c->uid = next_uid++;
    }
    int rc = LYMPH_OK;
    auto fail = [&](int code) { lymph_destroy(c); return code; };
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
        lymph_set_error("lymph_create: no CUDA device / stream");
        delete c;
        return LYMPH_ERR_CUDA;
    }
    // ---- polyhedron -> tets CSR, block pattern, per-block face lists ----
    std::vector<int32_t> pptr(np + 1, 0), ptets(nt);
    for (int t = 0; t < nt; ++t) pptr[m->tet_poly[t] + 1]++;
    for (int P = 0; P < np; ++P) pptr[P + 1] += pptr[P];
    {
        std::vector<int32_t> fill(pptr.begin(), pptr.end() - 1);
        for (int t = 0; t < nt; ++t) ptets[fill[m->tet_poly[t]]++] = t;
    }
    std::vector<int32_t> row_ptr(np + 1, 0), col, blk_row, bf;
    std::vector<int64_t> bf_ptr(1, 0);
    std::vector<int32_t> abs_idx(np, -1), abs_poly, abs_ptr(1, 0), abs_faces;
    int64_t n_sides = 0;
    for (int P = 0; P < np; ++P) {
        std::vector<int32_t> self_faces;
        std::map<int32_t, std::vector<int32_t>> nb;
        for (int k = pptr[P]; k < pptr[P + 1]; ++k) {
            int t = ptets[k];
            for (int f = 0; f < 4; ++f) {
                int e = m->neigh[t * 4 + f];
                if (e == LYMPH_BC_ABSO) { abs_faces.push_back(t * 4 + f); continue; }  // damping only
                if (e == LYMPH_BC_NEUM) continue;
                if (e == LYMPH_BC_DIRI) { self_faces.push_back(t * 4 + f); continue; }
                int Q = m->tet_poly[e];
                if (Q == P) continue;  // face inside the polyhedron (face_flag)
                self_faces.push_back(t * 4 + f);
                nb[Q].push_back(t * 4 + f);
            }
        }
        if ((int32_t)abs_faces.size() > abs_ptr.back()) {
            abs_idx[P] = (int32_t)abs_poly.size();
            abs_poly.push_back(P);
            abs_ptr.push_back((int32_t)abs_faces.size());
        }
        n_sides += (int64_t)self_faces.size();
        row_ptr[P] = (int32_t)col.size();
        col.push_back(P); blk_row.push_back(P);
        bf.insert(bf.end(), self_faces.begin(), self_faces.end());
        bf_ptr.push_back((int64_t)bf.size());
        for (auto& kv : nb) {
            col.push_back(kv.first); blk_row.push_back(P);
            bf.insert(bf.end(), kv.second.begin(), kv.second.end());
            bf_ptr.push_back((int64_t)bf.size());
        }
    }
    row_ptr[np] = (int32_t)col.size();
    c->n_blocks = (int64_t)col.size();
    c->n_face_sides = n_sides;
    c->n_block_faces = (int64_t)bf.size();
    c->h_row_ptr = row_ptr;
    c->h_col = col;
    RefTables ref;
    if (!build_ref_tables(c->p, ref)) { lymph_set_error("lymph_create: no quadrature table"); return fail(LYMPH_ERR_INVALID); }
    std::vector<int32_t> ftag(4 * (size_t)nt, 1);
    if (m->fun_tag) std::memcpy(ftag.data(), m->fun_tag, sizeof(int32_t) * 4 * (size_t)nt);
    // ---- device copies ----
    if ((rc = upload(c, &c->d_coords, m->coords, 3 * (size_t)m->n_node))) return fail(rc);
    if ((rc = upload(c, &c->d_tet_vert, m->tet_vert, 4 * (size_t)nt))) return fail(rc);
    if ((rc = upload(c, &c->d_tet_poly, m->tet_poly, (size_t)nt))) return fail(rc);
    if ((rc = upload(c, &c->d_tet_mat, m->tet_mat, (size_t)nt))) return fail(rc);
    if ((rc = upload(c, &c->d_neigh, m->neigh, 4 * (size_t)nt))) return fail(rc);
    if ((rc = upload(c, &c->d_fun_tag, ftag.data(), 4 * (size_t)nt))) return fail(rc);
    if ((rc = upload(c, &c->d_mat, m->mat, 3 * (size_t)m->n_mat))) return fail(rc);
    if ((rc = upload(c, &c->d_ref, &ref, 1))) return fail(rc);
    if ((rc = upload(c, &c->d_poly_ptr, pptr.data(), pptr.size()))) return fail(rc);
    if ((rc = upload(c, &c->d_poly_tets, ptets.data(), ptets.size()))) return fail(rc);
    if ((rc = upload(c, &c->d_row_ptr, row_ptr.data(), row_ptr.size()))) return fail(rc);
    if ((rc = upload(c, &c->d_col, col.data(), col.size()))) return fail(rc);
    if ((rc = upload(c, &c->d_blk_row, blk_row.data(), blk_row.size()))) return fail(rc);
    if ((rc = upload(c, &c->d_bf_ptr, bf_ptr.data(), bf_ptr.size()))) return fail(rc);
    if ((rc = upload(c, &c->d_bf, bf.data(), bf.size()))) return fail(rc);
    c->n_abs = (int)abs_poly.size();
    if (c->n_abs > 0) {
        const size_t nd2 = (size_t)c->n_abs * c->nd * c->nd;
        if ((rc = upload(c, &c->d_abs_idx, abs_idx.data(), abs_idx.size()))) return fail(rc);
        if ((rc = upload(c, &c->d_abs_poly, abs_poly.data(), abs_poly.size()))) return fail(rc);
        if ((rc = upload(c, &c->d_abs_ptr, abs_ptr.data(), abs_ptr.size()))) return fail(rc);
        if ((rc = upload(c, &c->d_abs_faces, abs_faces.data(), abs_faces.size()))) return fail(rc);
        if ((rc = dalloc(c, &c->d_Dabs, nd2))) return fail(rc);
        if ((rc = dalloc(c, &c->d_Wabs, nd2))) return fail(rc);
        if ((rc = dalloc(c, &c->d_Rw, nd2))) return fail(rc);
        if ((rc = dalloc(c, &c->d_RwT, nd2))) return fail(rc);
        if ((rc = dalloc(c, &c->d_Winv, nd2))) return fail(rc);
    }
    if ((rc = dalloc(c, &c->d_fk, 12 * (size_t)nt))) return fail(rc);
    if ((rc = dalloc(c, &c->d_jdet, (size_t)nt))) return fail(rc);
    if ((rc = dalloc(c, &c->d_normal, 12 * (size_t)nt))) return fail(rc);
    if ((rc = dalloc(c, &c->d_area, 4 * (size_t)nt))) return fail(rc);
    if ((rc = dalloc(c, &c->d_bbox, 6 * (size_t)np))) return fail(rc);
    if ((rc = dalloc(c, &c->d_hk, (size_t)np))) return fail(rc);
    size_t nv = (size_t)np * c->nd;
    for (int b = 0; b < 2; ++b)
        if ((rc = dalloc(c, &c->d_buf[b], nv))) return fail(rc);
    if ((rc = dalloc(c, &c->d_v0, nv))) return fail(rc);
    if ((rc = dalloc(c, &c->d_uex, nv))) return fail(rc);
    if ((rc = dalloc(c, &c->d_rhs_stat, nv))) return fail(rc);
    if ((rc = dalloc(c, &c->d_rhs_dyn, nv))) return fail(rc);
    if ((rc = dalloc(c, &c->d_partial, (size_t)np))) return fail(rc);
    if ((rc = dalloc(c, &c->d_scalar, 4))) return fail(rc);
    if ((rc = dalloc(c, &c->d_status, 1))) return fail(rc);
    if ((rc = dalloc(c, &c->d_step_idx, 1))) return fail(rc);
    c->gvals_cap = 4096;
    if ((rc = dalloc(c, &c->d_gvals, (size_t)c->gvals_cap))) return fail(rc);
    for (double* p : {c->d_buf[0], c->d_buf[1], c->d_v0, c->d_uex, c->d_rhs_stat, c->d_rhs_dyn})
        if (cudaMemsetAsync(p, 0, nv * sizeof(double), c->stream) != cudaSuccess) return fail(LYMPH_ERR_CUDA);
    if (cudaMemsetAsync(c->d_status, 0, sizeof(int), c->stream) != cudaSuccess) return fail(LYMPH_ERR_CUDA);
    if (cudaMemsetAsync(c->d_step_idx, 0, sizeof(int64_t), c->stream) != cudaSuccess) return fail(LYMPH_ERR_CUDA);
    if ((rc = lymph_dev_geometry(c))) return fail(rc);
    if ((rc = lymph_sync_status(c, "lymph_create"))) return fail(rc);
    *out = c;
    return LYMPH_OK;
}

int lymph_sizes(const lymph_ctx* c, int32_t* Np, int32_t* n_poly, int64_t* n_blocks, int64_t* n_face_sides) {
    if (!c) return LYMPH_ERR_INVALID;
    if (Np) *Np = c->Np;
    if (n_poly) *n_poly = c->n_poly;
    if (n_blocks) *n_blocks = c->n_blocks;
    if (n_face_sides) *n_face_sides = c->n_face_sides;
    return LYMPH_OK;
}

// Matrix-free neighbour terms: the FP32 self blocks (on the tensor cores,
// one per polyhedron in consecutive slots), the FP64 mass matrices and the
// per-triangle / per-polyhedron FP32 tables.
static int make_mf_matrices(lymph_ctx* c) {
    const int np = c->n_poly, nd = c->nd;
    const size_t nK = (size_t)np * nd * nd;
    if (!c->d_K) {
        void* pK = nullptr;
        if (cudaMalloc(&pK, nK * sizeof(float)) != cudaSuccess) {
            cudaGetLastError();
            lymph_set_error("lymph_make_matrices: cannot allocate " + std::to_string(nK * sizeof(float)) +
                            " bytes of self blocks");
            return LYMPH_ERR_OOM;
        }
        c->d_K = pK;
        c->device_bytes += (int64_t)(nK * sizeof(float));
    }
    std::vector<int64_t> self(np);
    for (int P = 0; P < np; ++P) self[P] = c->h_row_ptr[P];
    int64_t* d_list = nullptr;
    LYMPH_CUDA_TRY(cudaMalloc(&d_list, sizeof(int64_t) * (size_t)np));
    int rc = cudaMemcpy(d_list, self.data(), sizeof(int64_t) * (size_t)np, cudaMemcpyHostToDevice) == cudaSuccess
                 ? LYMPH_OK : LYMPH_ERR_CUDA;
    if (rc == LYMPH_OK) rc = lymph_dev_mass(c, d_list);
    if (rc == LYMPH_OK) rc = lymph_dev_self_tc(c, (float*)c->d_K, false);
    if (rc == LYMPH_OK && cudaStreamSynchronize(c->stream) != cudaSuccess) rc = LYMPH_ERR_CUDA;
    cudaFree(d_list);
    LYMPH_TRY(rc);
    RefTables R;
    if (!build_ref_tables(c->p, R)) { lymph_set_error("lymph_make_matrices: no quadrature for this degree"); return LYMPH_ERR_INVALID; }
    return lymph_mf_setup(c, R);
}

// FP32 blocks (LYMPH_MIXED): the self and the neighbour blocks on the
// tensor cores, the mass matrices in FP64.
static int make_mixed_blocks(lymph_ctx* c) {
    const int np = c->n_poly;
    std::vector<int64_t> lists;
    lists.reserve((size_t)c->n_blocks);
    for (int P = 0; P < np; ++P) lists.push_back(c->h_row_ptr[P]);
    for (int P = 0; P < np; ++P)
        for (int64_t k = (int64_t)c->h_row_ptr[P] + 1; k < c->h_row_ptr[P + 1]; ++k) lists.push_back(k);
    const int64_t n_nb = (int64_t)lists.size() - np;
    int64_t* d_lists = nullptr;
    LYMPH_CUDA_TRY(cudaMalloc(&d_lists, sizeof(int64_t) * lists.size()));
    int rc = cudaMemcpy(d_lists, lists.data(), sizeof(int64_t) * lists.size(), cudaMemcpyHostToDevice) == cudaSuccess
                 ? LYMPH_OK : LYMPH_ERR_CUDA;
    if (rc == LYMPH_OK) rc = lymph_dev_mass(c, d_lists);
    if (rc == LYMPH_OK && n_nb > 0) rc = lymph_dev_nb_tc(c, (float*)c->d_K, d_lists + np, n_nb);
    if (rc == LYMPH_OK) rc = lymph_dev_self_tc(c, (float*)c->d_K, true);
    if (rc == LYMPH_OK && cudaStreamSynchronize(c->stream) != cudaSuccess) rc = LYMPH_ERR_CUDA;
    cudaFree(d_lists);
    return rc;
}

int lymph_make_matrices(lymph_ctx* c) {
    NvtxRange nvtx_("lymph_make_matrices");
    if (!c) return LYMPH_ERR_INVALID;
    if (c->precision == LYMPH_MIXED_MF) {
        if (!c->d_M) {
            size_t nm = (size_t)c->n_poly * c->Np * c->Np;
            LYMPH_TRY(dalloc(c, &c->d_M, nm));
            LYMPH_TRY(dalloc(c, &c->d_Mm, nm));
            LYMPH_TRY(dalloc(c, &c->d_R, nm));
            LYMPH_TRY(dalloc(c, &c->d_RT, nm));
            LYMPH_TRY(dalloc(c, &c->d_Rm, nm));
            LYMPH_TRY(dalloc(c, &c->d_RmT, nm));
            LYMPH_TRY(dalloc(c, &c->d_Minv, nm));
        }
        c->rhs_version++;
        LYMPH_TRY(make_mf_matrices(c));
        LYMPH_TRY(lymph_dev_cholesky(c));
        LYMPH_TRY(lymph_dev_damping(c, true));
        LYMPH_TRY(lymph_sync_status(c, "lymph_make_matrices"));
        c->have_matrices = true;
        return LYMPH_OK;
    }
    size_t es = (c->precision == LYMPH_MIXED) ? sizeof(float) : sizeof(double);
    size_t nK = (size_t)c->n_blocks * c->nd * c->nd;
    if (!c->d_K) {
        void* p = nullptr;
        cudaError_t e = cudaMalloc(&p, nK * es);
        if (e != cudaSuccess) {
            lymph_set_error("lymph_make_matrices: cannot allocate " + std::to_string(nK * es) + " bytes of operator blocks");
            return LYMPH_ERR_OOM;
        }
        c->d_K = p;
        c->device_bytes += (int64_t)(nK * es);
        size_t nm = (size_t)c->n_poly * c->Np * c->Np;
        LYMPH_TRY(dalloc(c, &c->d_M, nm));
        LYMPH_TRY(dalloc(c, &c->d_Mm, nm));
        LYMPH_TRY(dalloc(c, &c->d_R, nm));
        LYMPH_TRY(dalloc(c, &c->d_RT, nm));
        LYMPH_TRY(dalloc(c, &c->d_Rm, nm));
        LYMPH_TRY(dalloc(c, &c->d_RmT, nm));
        LYMPH_TRY(dalloc(c, &c->d_Minv, nm));
    }
    c->k32_valid = false;  // an FP32 copy made from earlier blocks is stale
    c->rhs_version++;      // and so is any cached M^-1 F
    if (c->precision == LYMPH_MIXED) LYMPH_TRY(make_mixed_blocks(c));
    else LYMPH_TRY(lymph_dev_assemble(c, LYMPH_BLOCKS_K, c->d_K, 0, true));
    LYMPH_TRY(lymph_dev_cholesky(c));
    LYMPH_TRY(lymph_dev_damping(c, true));
    LYMPH_TRY(lymph_sync_status(c, "lymph_make_matrices"));
    c->have_matrices = true;
    return LYMPH_OK;
}

int lymph_make_rhs(lymph_ctx* c, int which, int fid, int did, int nid) {
    NvtxRange nvtx_("lymph_make_rhs");
    if (!c || (which != LYMPH_RHS_STAT && which != LYMPH_RHS_DYN)) return LYMPH_ERR_INVALID;
    if (fid < 0 || fid > 2 || did < 0 || did > 2 || nid < 0 || nid > 2) {
        lymph_set_error("lymph_make_rhs: unknown data function id");
        return LYMPH_ERR_INVALID;
    }
    if (!c->have_matrices) { lymph_set_error("lymph_make_rhs: call lymph_make_matrices first"); return LYMPH_ERR_ORDER; }
    double* out = (which == LYMPH_RHS_STAT) ? c->d_rhs_stat : c->d_rhs_dyn;
    c->rhs_version++;
    LYMPH_TRY(lymph_dev_vector(c, 0, fid, did, nid, 1.0, out));
    LYMPH_TRY(lymph_sync_status(c, "lymph_make_rhs"));
    if (which == LYMPH_RHS_STAT) c->have_rhs_stat = true; else c->have_rhs_dyn = true;
    return LYMPH_OK;
}

int lymph_modal_project(lymph_ctx* c, int fun_id, int slot, double scale) {
    NvtxRange nvtx_("lymph_modal_project");
    if (!c || !valid_slot(slot) || fun_id < 0 || fun_id > 3) return LYMPH_ERR_INVALID;
    if (!c->have_matrices) { lymph_set_error("lymph_modal_project: call lymph_make_matrices first"); return LYMPH_ERR_ORDER; }
    LYMPH_TRY(lymph_dev_vector(c, 1, fun_id, 0, 0, scale, lymph_slot_ptr(c, slot)));
    return lymph_sync_status(c, "lymph_modal_project");
}

int lymph_first_step(lymph_ctx* c, double t) {
    NvtxRange nvtx_("lymph_first_step");
    if (!c) return LYMPH_ERR_INVALID;
    if (!c->have_matrices) { lymph_set_error("lymph_first_step: call lymph_make_matrices first"); return LYMPH_ERR_ORDER; }
    LYMPH_TRY(set_g(c, time_function(t)));
    LYMPH_TRY(lymph_dev_first_step(c));
    return lymph_sync_status(c, "lymph_first_step");
}

int lymph_step(lymph_ctx* c, double t) {
    NvtxRange nvtx_("lymph_step");
    if (!c) return LYMPH_ERR_INVALID;
    if (!c->have_matrices) { lymph_set_error("lymph_step: call lymph_make_matrices first"); return LYMPH_ERR_ORDER; }
    LYMPH_TRY(set_g(c, time_function(t)));
    LYMPH_TRY(lymph_dev_step(c, false));
    c->cur ^= 1;
    return lymph_sync_status(c, "lymph_step");
}

int lymph_time_step_host(lymph_ctx* c, double t, const double* u0, const double* un, double* usol, int layout) {
    NvtxRange nvtx_("lymph_time_step_host");
    if (!c || !u0 || !un || !usol) return LYMPH_ERR_INVALID;
    if (!c->have_matrices) { lymph_set_error("lymph_time_step_host: call lymph_make_matrices first"); return LYMPH_ERR_ORDER; }
    const size_t nv = (size_t)c->n_poly * c->nd, bytes = nv * sizeof(double);
    const bool fort = layout == LYMPH_LAYOUT_FORTRAN;
    if (!c->stream2) LYMPH_CUDA_TRY(cudaStreamCreateWithFlags(&c->stream2, cudaStreamNonBlocking));
    if (!c->ev_copy) LYMPH_CUDA_TRY(cudaEventCreateWithFlags(&c->ev_copy, cudaEventDisableTiming));
    if (!c->h_status) LYMPH_CUDA_TRY(cudaHostAlloc((void**)&c->h_status, sizeof(int), cudaHostAllocDefault));
    if (fort) {
        LYMPH_TRY(layout_buffer(c));
        if (!c->d_layout2) LYMPH_TRY(dalloc(c, &c->d_layout2, nv));
    }
    double* d_u0 = lymph_slot_ptr(c, LYMPH_SLOT_U0);
    double* d_un = lymph_slot_ptr(c, LYMPH_SLOT_UN);
    // the second stream starts after what the context stream has queued
    LYMPH_CUDA_TRY(cudaEventRecord(c->ev_copy, c->stream));
    LYMPH_CUDA_TRY(cudaStreamWaitEvent(c->stream2, c->ev_copy, 0));
    // u^{n-1} up on the second stream, u^n on the context stream: two copy engines
    LYMPH_CUDA_TRY(cudaMemcpyAsync(fort ? c->d_layout2 : d_u0, u0, bytes, cudaMemcpyHostToDevice, c->stream2));
    if (fort) LYMPH_TRY(transpose(c, c->d_layout2, d_u0, c->nd, c->n_poly, c->stream2));
    LYMPH_CUDA_TRY(cudaEventRecord(c->ev_copy, c->stream2));
    LYMPH_CUDA_TRY(cudaMemcpyAsync(fort ? c->d_layout : d_un, un, bytes, cudaMemcpyHostToDevice, c->stream));
    if (fort) LYMPH_TRY(transpose(c, c->d_layout, d_un, c->nd, c->n_poly, c->stream));
    LYMPH_CUDA_TRY(cudaStreamWaitEvent(c->stream, c->ev_copy, 0));
    // TIME_STEP_MATRIX_FREE
    LYMPH_TRY(set_g(c, time_function(t)));
    LYMPH_TRY(lymph_dev_step(c, false));
    c->cur ^= 1;
    // u^{n+1} down and the status word, then one synchronisation
    const double* d_out = lymph_slot_ptr(c, LYMPH_SLOT_UN);
    if (fort) {
        LYMPH_TRY(transpose(c, d_out, c->d_layout, c->n_poly, c->nd, c->stream));
        d_out = c->d_layout;
    }
    LYMPH_CUDA_TRY(cudaMemcpyAsync(usol, d_out, bytes, cudaMemcpyDeviceToHost, c->stream));
    LYMPH_CUDA_TRY(cudaMemcpyAsync(c->h_status, c->d_status, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    LYMPH_CUDA_TRY(cudaStreamSynchronize(c->stream));
    return status_rc(c, *c->h_status, "lymph_time_step_host");
}

int lymph_first_step_g(lymph_ctx* c, double g) {
    if (!c || !std::isfinite(g)) return LYMPH_ERR_INVALID;
    if (!c->have_matrices) { lymph_set_error("lymph_first_step_g: call lymph_make_matrices first"); return LYMPH_ERR_ORDER; }
    LYMPH_TRY(set_g(c, g));
    LYMPH_TRY(lymph_dev_first_step(c));
    return lymph_sync_status(c, "lymph_first_step_g");
}

int lymph_step_g(lymph_ctx* c, double g) {
    if (!c || !std::isfinite(g)) return LYMPH_ERR_INVALID;
    if (!c->have_matrices) { lymph_set_error("lymph_step_g: call lymph_make_matrices first"); return LYMPH_ERR_ORDER; }
    LYMPH_TRY(set_g(c, g));
    LYMPH_TRY(lymph_dev_step(c, false));
    c->cur ^= 1;
    return lymph_sync_status(c, "lymph_step_g");
}

int lymph_run_steps(lymph_ctx* c, double stop_time, int64_t max_steps, double* t_inout, int64_t* n_done,
                    float* ms_total, float* ms_kernel) {
    NvtxRange nvtx_("lymph_run_steps");
    if (!c || !t_inout) return LYMPH_ERR_INVALID;
    if (!c->have_matrices) { lymph_set_error("lymph_run_steps: call lymph_make_matrices first"); return LYMPH_ERR_ORDER; }
    // time values with the reference's accumulation (Lymph3D.f90:389-418)
    std::vector<double> g;
    double t = *t_inout;
    while (t <= stop_time && (max_steps < 0 || (int64_t)g.size() < max_steps)) {
        g.push_back(time_function(t));
        t = t + c->dt;
    }
    const int64_t n = (int64_t)g.size();
    if (n_done) *n_done = n;
    if (ms_total) *ms_total = 0.0f;
    if (ms_kernel) *ms_kernel = 0.0f;
    if (n == 0) { *t_inout = t; return LYMPH_OK; }
    if (n > c->gvals_cap) {
        dfree(c->d_gvals);
        c->device_bytes -= c->gvals_cap * (int64_t)sizeof(double);
        c->gvals_cap = n + 1024;
        LYMPH_TRY(dalloc(c, &c->d_gvals, (size_t)c->gvals_cap));
        if (c->graph_exec) { cudaGraphExecDestroy(c->graph_exec); c->graph_exec = nullptr; }
    }
    LYMPH_CUDA_TRY(cudaMemcpyAsync(c->d_gvals, g.data(), n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    LYMPH_CUDA_TRY(cudaMemsetAsync(c->d_step_idx, 0, sizeof(int64_t), c->stream));
    cudaEvent_t e0, e1;
    LYMPH_CUDA_TRY(cudaEventCreate(&e0));
    LYMPH_CUDA_TRY(cudaEventCreate(&e1));
    int rc = LYMPH_OK;
    if (ms_kernel) {
        // per-launch events around every step kernel (no graph)
        std::vector<cudaEvent_t> ev(2 * n);
        for (auto& e : ev) cudaEventCreate(&e);
        cudaEventRecord(e0, c->stream);
        for (int64_t i = 0; i < n && rc == LYMPH_OK; ++i) {
            cudaEventRecord(ev[2 * i], c->stream);
            rc = lymph_dev_step(c, false);
            cudaEventRecord(ev[2 * i + 1], c->stream);
            if (rc == LYMPH_OK) rc = lymph_dev_bump(c);
            c->cur ^= 1;
        }
        cudaEventRecord(e1, c->stream);
        cudaEventSynchronize(e1);
        float sum = 0.0f;
        for (int64_t i = 0; i < n; ++i) {
            float ms = 0.0f;
            cudaEventElapsedTime(&ms, ev[2 * i], ev[2 * i + 1]);
            sum += ms;
        }
        *ms_kernel = sum;
        for (auto& e : ev) cudaEventDestroy(e);
    } else {
        const int R = 16;  // steps per graph (even: returns to the same buffer parity)
        if (c->graph_exec && (c->graph_steps != R || c->graph_parity != c->cur)) {
            cudaGraphExecDestroy(c->graph_exec);
            c->graph_exec = nullptr;
        }
        int64_t i = 0;
        cudaEventRecord(e0, c->stream);
        if (n >= R) {
            if (!c->graph_exec) {
                cudaGraph_t graph;
                int cur0 = c->cur;
                LYMPH_CUDA_TRY(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
                int64_t l0 = c->launches;
                for (int j = 0; j < R; ++j) {
                    lymph_dev_step(c, true);
                    c->cur ^= 1;
                }
                c->graph_launches = c->launches - l0;
                c->launches = l0;
                cudaError_t ce = cudaStreamEndCapture(c->stream, &graph);
                c->cur = cur0;
                if (ce != cudaSuccess) { lymph_set_error(std::string("graph capture: ") + cudaGetErrorString(ce)); return LYMPH_ERR_CUDA; }
                ce = cudaGraphInstantiate(&c->graph_exec, graph, 0);
                cudaGraphDestroy(graph);
                if (ce != cudaSuccess) { lymph_set_error(std::string("graph instantiate: ") + cudaGetErrorString(ce)); return LYMPH_ERR_CUDA; }
                c->graph_steps = R;
                c->graph_parity = cur0;
            }
            // the graph holds the buffer pointers of parity cur0; R is even, so
            // the parity is the same after every launch
            for (; i + R <= n; i += R) {
                NvtxRange nvtx_step("16 leapfrog steps (graph)");
                LYMPH_CUDA_TRY(cudaGraphLaunch(c->graph_exec, c->stream));
                c->launches += c->graph_launches;
            }
        }
        for (; i < n; ++i) {
            LYMPH_TRY(lymph_dev_step(c, true));
            c->cur ^= 1;
        }
        cudaEventRecord(e1, c->stream);
    }
    cudaEventSynchronize(e1);
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms_total) *ms_total = ms;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *t_inout = t;
    LYMPH_TRY(rc);
    return lymph_sync_status(c, "lymph_run_steps");
}

int lymph_get_state(lymph_ctx* c, int slot, double* host, int layout) {
    if (!c || !host || !valid_slot(slot)) return LYMPH_ERR_INVALID;
    size_t nv = (size_t)c->n_poly * c->nd;
    const double* src = lymph_slot_ptr(c, slot);
    if (layout == LYMPH_LAYOUT_FORTRAN) {
        // transposed on the device, then one direct copy
        LYMPH_TRY(layout_buffer(c));
        LYMPH_TRY(transpose(c, src, c->d_layout, c->n_poly, c->nd, c->stream));
        src = c->d_layout;
    }
    // a page-locked caller buffer moves by DMA
    LYMPH_CUDA_TRY(cudaMemcpyAsync(host, src, nv * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    LYMPH_CUDA_TRY(cudaStreamSynchronize(c->stream));
    return LYMPH_OK;
}

int lymph_set_state(lymph_ctx* c, int slot, const double* host, int layout) {
    if (!c || !host || !valid_slot(slot)) return LYMPH_ERR_INVALID;
    size_t nv = (size_t)c->n_poly * c->nd;
    double* dst = lymph_slot_ptr(c, slot);
    if (layout != LYMPH_LAYOUT_FORTRAN) {
        LYMPH_CUDA_TRY(cudaMemcpyAsync(dst, host, nv * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    } else {
        LYMPH_TRY(layout_buffer(c));
        LYMPH_CUDA_TRY(cudaMemcpyAsync(c->d_layout, host, nv * sizeof(double), cudaMemcpyHostToDevice, c->stream));
        LYMPH_TRY(transpose(c, c->d_layout, dst, c->nd, c->n_poly, c->stream));
    }
    LYMPH_CUDA_TRY(cudaStreamSynchronize(c->stream));
    return LYMPH_OK;
}

int lymph_checkpoint_save(lymph_ctx* c, const char* path, double t, int64_t steps) {
    if (!c || !path) return LYMPH_ERR_INVALID;
    CheckpointHeader h;
    std::memset(&h, 0, sizeof(h));
    std::memcpy(h.magic, "LYMPHCK1", 8);
    h.version = 1;
    h.precision = c->precision;
    h.degree = c->p;
    h.mesh_hash = c->mesh_hash;
    h.n_poly = c->n_poly;
    h.nd = c->nd;
    h.dt = c->dt; h.alpha = c->alpha; h.theta = c->theta;
    h.t = t;
    h.steps = steps;
    const size_t nv = (size_t)c->n_poly * c->nd;
    std::vector<double> u(2 * nv);
    LYMPH_CUDA_TRY(cudaMemcpyAsync(u.data(), lymph_slot_ptr(c, LYMPH_SLOT_U0), nv * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    LYMPH_CUDA_TRY(cudaMemcpyAsync(u.data() + nv, lymph_slot_ptr(c, LYMPH_SLOT_UN), nv * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    LYMPH_CUDA_TRY(cudaStreamSynchronize(c->stream));
    const std::string tmp = std::string(path) + ".tmp";
    FILE* f = std::fopen(tmp.c_str(), "wb");
    if (!f) { lymph_set_error(std::string("lymph_checkpoint_save: cannot write ") + tmp); return LYMPH_ERR_INVALID; }
    const bool ok = std::fwrite(&h, sizeof(h), 1, f) == 1 && std::fwrite(u.data(), sizeof(double), 2 * nv, f) == 2 * nv;
    const bool closed = std::fclose(f) == 0;
    if (!ok || !closed || std::rename(tmp.c_str(), path) != 0) {
        std::remove(tmp.c_str());
        lymph_set_error(std::string("lymph_checkpoint_save: write failed: ") + path);
        return LYMPH_ERR_INVALID;
    }
    return LYMPH_OK;
}

int lymph_checkpoint_load(lymph_ctx* c, const char* path, double* t, int64_t* steps) {
    if (!c || !path) return LYMPH_ERR_INVALID;
    FILE* f = std::fopen(path, "rb");
    if (!f) { lymph_set_error(std::string("lymph_checkpoint_load: cannot read ") + path); return LYMPH_ERR_INVALID; }
    CheckpointHeader h;
    const size_t nv = (size_t)c->n_poly * c->nd;
    std::vector<double> u;
    auto bad = [&](const std::string& why) {
        std::fclose(f);
        lymph_set_error("lymph_checkpoint_load: " + why);
        return LYMPH_ERR_INVALID;
    };
    if (std::fread(&h, sizeof(h), 1, f) != 1 || std::memcmp(h.magic, "LYMPHCK1", 8) != 0 || h.version != 1)
        return bad("not a checkpoint of this library");
    if (h.mesh_hash != c->mesh_hash || h.n_poly != c->n_poly) return bad("written for another mesh");
    if (h.degree != c->p || h.nd != c->nd) return bad("written for another degree");
    if (h.precision != c->precision) return bad("written for another precision mode");
    if (h.dt != c->dt || h.alpha != c->alpha || h.theta != c->theta) return bad("written with another dt, alpha or theta");
    u.resize(2 * nv);
    if (std::fread(u.data(), sizeof(double), 2 * nv, f) != 2 * nv) return bad("truncated file");
    std::fclose(f);
    LYMPH_CUDA_TRY(cudaMemcpyAsync(lymph_slot_ptr(c, LYMPH_SLOT_U0), u.data(), nv * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    LYMPH_CUDA_TRY(cudaMemcpyAsync(lymph_slot_ptr(c, LYMPH_SLOT_UN), u.data() + nv, nv * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    LYMPH_CUDA_TRY(cudaStreamSynchronize(c->stream));
    if (t) *t = h.t;
    if (steps) *steps = h.steps;
    return LYMPH_OK;
}

int lymph_copy_state(lymph_ctx* c, int dst, int src) {
    if (!c || !valid_slot(dst) || !valid_slot(src)) return LYMPH_ERR_INVALID;
    if (dst == src) return LYMPH_OK;
    LYMPH_CUDA_TRY(cudaMemcpyAsync(lymph_slot_ptr(c, dst), lymph_slot_ptr(c, src), sizeof(double) * (size_t)c->n_poly * c->nd,
                                   cudaMemcpyDeviceToDevice, c->stream));
    LYMPH_CUDA_TRY(cudaStreamSynchronize(c->stream));
    return LYMPH_OK;
}

int lymph_error_l2(lymph_ctx* c, int s_uh, int s_uex, double* sumsq) {
    if (!c || !sumsq || !valid_slot(s_uh) || !valid_slot(s_uex)) return LYMPH_ERR_INVALID;
    if (!c->have_matrices) { lymph_set_error("lymph_error_l2: call lymph_make_matrices first"); return LYMPH_ERR_ORDER; }
    LYMPH_TRY(lymph_dev_error_l2(c, lymph_slot_ptr(c, s_uh), lymph_slot_ptr(c, s_uex), c->d_scalar));
    LYMPH_CUDA_TRY(cudaMemcpyAsync(sumsq, c->d_scalar, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    return lymph_sync_status(c, "lymph_error_l2");
}

int lymph_error_dg(lymph_ctx* c, int s_uh, int s_uex, double* sumsq) {
    if (!c || !sumsq || !valid_slot(s_uh) || !valid_slot(s_uex)) return LYMPH_ERR_INVALID;
    if (!c->have_matrices) { lymph_set_error("lymph_error_dg: call lymph_make_matrices first"); return LYMPH_ERR_ORDER; }
    size_t nK = (size_t)c->n_blocks * c->nd * c->nd;
    double* A = nullptr;
    if (cudaMalloc(&A, nK * sizeof(double)) != cudaSuccess) {
        lymph_set_error("lymph_error_dg: cannot allocate the A_dg blocks");
        return LYMPH_ERR_OOM;
    }
    int rc = lymph_dev_assemble(c, LYMPH_BLOCKS_ADG, A, 0, false);
    if (rc == LYMPH_OK) rc = lymph_dev_error_dg(c, A, lymph_slot_ptr(c, s_uh), lymph_slot_ptr(c, s_uex), c->d_scalar);
    if (rc == LYMPH_OK && cudaMemcpyAsync(sumsq, c->d_scalar, sizeof(double), cudaMemcpyDeviceToHost, c->stream) != cudaSuccess)
        rc = LYMPH_ERR_CUDA;
    cudaStreamSynchronize(c->stream);
    cudaFree(A);
    LYMPH_TRY(rc);
    return lymph_sync_status(c, "lymph_error_dg");
}

int lymph_energy(lymph_ctx* c, int slot_a, int slot_b, double* energy) {
    if (!c || !energy || !valid_slot(slot_a) || !valid_slot(slot_b)) return LYMPH_ERR_INVALID;
    if (!c->have_matrices) { lymph_set_error("lymph_energy: call lymph_make_matrices first"); return LYMPH_ERR_ORDER; }
    LYMPH_TRY(lymph_dev_energy(c, lymph_slot_ptr(c, slot_a), lymph_slot_ptr(c, slot_b), c->d_scalar));
    double t[2];
    LYMPH_CUDA_TRY(cudaMemcpyAsync(t, c->d_scalar, sizeof(t), cudaMemcpyDeviceToHost, c->stream));
    LYMPH_TRY(lymph_sync_status(c, "lymph_energy"));
    *energy = 0.5 * t[0] / (c->dt * c->dt) + 0.5 * t[1];
    return LYMPH_OK;
}

int lymph_apply_operator(lymph_ctx* c, const double* u, double* ku) {
    if (!c || !u || !ku) return LYMPH_ERR_INVALID;
    if (!c->have_matrices) { lymph_set_error("lymph_apply_operator: call lymph_make_matrices first"); return LYMPH_ERR_ORDER; }
    const size_t nv = (size_t)c->n_poly * c->nd;
    double *du = nullptr, *dk = nullptr;
    if (cudaMalloc(&du, nv * sizeof(double)) != cudaSuccess || cudaMalloc(&dk, nv * sizeof(double)) != cudaSuccess) {
        if (du) cudaFree(du);
        cudaGetLastError();
        lymph_set_error("lymph_apply_operator: out of memory");
        return LYMPH_ERR_OOM;
    }
    int rc = LYMPH_OK;
    if (cudaMemcpyAsync(du, u, nv * sizeof(double), cudaMemcpyHostToDevice, c->stream) != cudaSuccess) rc = LYMPH_ERR_CUDA;
    if (rc == LYMPH_OK) rc = lymph_dev_ku(c, du, dk);
    if (rc == LYMPH_OK && cudaMemcpyAsync(ku, dk, nv * sizeof(double), cudaMemcpyDeviceToHost, c->stream) != cudaSuccess)
        rc = LYMPH_ERR_CUDA;
    cudaStreamSynchronize(c->stream);
    cudaFree(du);
    cudaFree(dk);
    LYMPH_TRY(rc);
    return lymph_sync_status(c, "lymph_apply_operator");
}

int lymph_compute_error_l2_free(lymph_ctx* c, int s_uh, int s_uex, double* sumsq) { return lymph_error_l2(c, s_uh, s_uex, sumsq); }
int lymph_compute_error_dg_free(lymph_ctx* c, int s_uh, int s_uex, double* sumsq) { return lymph_error_dg(c, s_uh, s_uex, sumsq); }

int lymph_get_pattern(lymph_ctx* c, int32_t* row_ptr, int32_t* col) {
    if (!c) return LYMPH_ERR_INVALID;
    if (row_ptr) std::memcpy(row_ptr, c->h_row_ptr.data(), sizeof(int32_t) * c->h_row_ptr.size());
    if (col) std::memcpy(col, c->h_col.data(), sizeof(int32_t) * c->h_col.size());
    return LYMPH_OK;
}

int lymph_get_blocks(lymph_ctx* c, int which, double* vals) {
    if (!c || !vals || (which != LYMPH_BLOCKS_K && which != LYMPH_BLOCKS_ADG)) return LYMPH_ERR_INVALID;
    if (!c->have_matrices) { lymph_set_error("lymph_get_blocks: call lymph_make_matrices first"); return LYMPH_ERR_ORDER; }
    const int nd = c->nd;
    size_t nK = (size_t)c->n_blocks * nd * nd;
    std::vector<double> tmp(nK);
    if (which == LYMPH_BLOCKS_K && c->precision == LYMPH_MIXED_MF) {
        // the operator the matrix-free path evaluates: the FP64 assembly of
        // every block (the neighbour blocks are not stored in this mode)
        double* A = nullptr;
        if (cudaMalloc(&A, nK * sizeof(double)) != cudaSuccess) { lymph_set_error("lymph_get_blocks: out of memory"); return LYMPH_ERR_OOM; }
        int rc = lymph_dev_assemble(c, LYMPH_BLOCKS_K, A, 0, false);
        if (rc == LYMPH_OK && cudaStreamSynchronize(c->stream) != cudaSuccess) rc = LYMPH_ERR_CUDA;
        if (rc == LYMPH_OK && cudaMemcpy(tmp.data(), A, nK * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess) rc = LYMPH_ERR_CUDA;
        cudaFree(A);
        LYMPH_TRY(rc);
    } else if (which == LYMPH_BLOCKS_K && c->precision == LYMPH_MIXED) {
        std::vector<float> tf(nK);
        LYMPH_CUDA_TRY(cudaMemcpy(tf.data(), c->d_K, nK * sizeof(float), cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < nK; ++i) tmp[i] = tf[i];
    } else if (which == LYMPH_BLOCKS_K) {
        LYMPH_CUDA_TRY(cudaMemcpy(tmp.data(), c->d_K, nK * sizeof(double), cudaMemcpyDeviceToHost));
    } else {
        double* A = nullptr;
        if (cudaMalloc(&A, nK * sizeof(double)) != cudaSuccess) { lymph_set_error("lymph_get_blocks: out of memory"); return LYMPH_ERR_OOM; }
        int rc = lymph_dev_assemble(c, LYMPH_BLOCKS_ADG, A, 0, false);
        if (rc == LYMPH_OK && cudaStreamSynchronize(c->stream) != cudaSuccess) rc = LYMPH_ERR_CUDA;
        if (rc == LYMPH_OK && cudaMemcpy(tmp.data(), A, nK * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess) rc = LYMPH_ERR_CUDA;
        cudaFree(A);
        LYMPH_TRY(rc);
    }
    // device blocks are column-major; return row-major
    for (int64_t b = 0; b < c->n_blocks; ++b)
        for (int r = 0; r < nd; ++r)
            for (int cc = 0; cc < nd; ++cc) vals[((size_t)b * nd + r) * nd + cc] = tmp[((size_t)b * nd + cc) * nd + r];
    return lymph_sync_status(c, "lymph_get_blocks");
}

int lymph_get_self_blocks(lymph_ctx* c, double* vals) {
    if (!c || !vals) return LYMPH_ERR_INVALID;
    if (!c->have_matrices) { lymph_set_error("lymph_get_self_blocks: call lymph_make_matrices first"); return LYMPH_ERR_ORDER; }
    const int nd = c->nd;
    const size_t nb = (size_t)nd * nd;
    std::vector<double> tmp(nb);
    std::vector<float> tf(nb);
    for (int P = 0; P < c->n_poly; ++P) {
        // MIXED_MF stores the self blocks alone, one per polyhedron; the
        // block-CSR modes store each row's self block first
        const size_t slot = c->precision == LYMPH_MIXED_MF ? (size_t)P : (size_t)c->h_row_ptr[P];
        if (c->precision == LYMPH_FP64) {
            LYMPH_CUDA_TRY(cudaMemcpy(tmp.data(), (const double*)c->d_K + slot * nb, nb * sizeof(double),
                                      cudaMemcpyDeviceToHost));
        } else {
            LYMPH_CUDA_TRY(cudaMemcpy(tf.data(), (const float*)c->d_K + slot * nb, nb * sizeof(float),
                                      cudaMemcpyDeviceToHost));
            for (size_t i = 0; i < nb; ++i) tmp[i] = tf[i];
        }
        for (int r = 0; r < nd; ++r)
            for (int cc = 0; cc < nd; ++cc) vals[((size_t)P * nd + r) * nd + cc] = tmp[(size_t)cc * nd + r];
    }
    return lymph_sync_status(c, "lymph_get_self_blocks");
}

int lymph_get_mass(lymph_ctx* c, int which, double* vals) {
    if (!c || !vals || which < 0 || which > 4) return LYMPH_ERR_INVALID;
    if (!c->have_matrices) { lymph_set_error("lymph_get_mass: call lymph_make_matrices first"); return LYMPH_ERR_ORDER; }
    const double* src[5] = {c->d_M, c->d_Mm, c->d_R, c->d_Rm, c->d_Minv};
    const size_t nm = (size_t)c->n_poly * c->Np * c->Np;
    LYMPH_CUDA_TRY(cudaMemcpy(vals, src[which], sizeof(double) * nm, cudaMemcpyDeviceToHost));
    if (which == 4) {  // stored column-major per polyhedron
        const int Np = c->Np;
        std::vector<double> t(Np * Np);
        for (int P = 0; P < c->n_poly; ++P) {
            double* b = vals + (size_t)P * Np * Np;
            for (int i = 0; i < Np * Np; ++i) t[(i % Np) * Np + i / Np] = b[i];
            std::memcpy(b, t.data(), sizeof(double) * Np * Np);
        }
    }
    return LYMPH_OK;
}

int lymph_get_rhs(lymph_ctx* c, int which, double* vals) {
    if (!c || !vals || (which != LYMPH_RHS_STAT && which != LYMPH_RHS_DYN)) return LYMPH_ERR_INVALID;
    LYMPH_CUDA_TRY(cudaMemcpy(vals, which == LYMPH_RHS_STAT ? c->d_rhs_stat : c->d_rhs_dyn,
                              sizeof(double) * (size_t)c->n_poly * c->nd, cudaMemcpyDeviceToHost));
    return LYMPH_OK;
}

int lymph_get_poly_geometry(lymph_ctx* c, double* bbox, double* hk) {
    if (!c) return LYMPH_ERR_INVALID;
    if (bbox) LYMPH_CUDA_TRY(cudaMemcpy(bbox, c->d_bbox, sizeof(double) * 6 * (size_t)c->n_poly, cudaMemcpyDeviceToHost));
    if (hk) LYMPH_CUDA_TRY(cudaMemcpy(hk, c->d_hk, sizeof(double) * (size_t)c->n_poly, cudaMemcpyDeviceToHost));
    return LYMPH_OK;
}

int lymph_make_rhs_point(lymph_ctx* c, int which, int32_t tet, const double* x0, const double* dir) {
    if (!c || !x0 || !dir || (which != LYMPH_RHS_STAT && which != LYMPH_RHS_DYN)) return LYMPH_ERR_INVALID;
    if (tet < 0 || tet >= c->n_tet) { lymph_set_error("lymph_make_rhs_point: tetrahedron out of range"); return LYMPH_ERR_INVALID; }
    if (!c->have_matrices) { lymph_set_error("lymph_make_rhs_point: call lymph_make_matrices first"); return LYMPH_ERR_ORDER; }
    int32_t P = 0;
    LYMPH_CUDA_TRY(cudaMemcpy(&P, c->d_tet_poly + tet, sizeof(int32_t), cudaMemcpyDeviceToHost));
    double* out = (which == LYMPH_RHS_STAT) ? c->d_rhs_stat : c->d_rhs_dyn;
    c->rhs_version++;
    LYMPH_TRY(lymph_dev_point_source(c, P, x0, dir, out));
    LYMPH_TRY(lymph_sync_status(c, "lymph_make_rhs_point"));
    if (which == LYMPH_RHS_STAT) c->have_rhs_stat = true; else c->have_rhs_dyn = true;
    return LYMPH_OK;
}

// Double-couple seismic source (matrix_free.f90:602-664): adds to RHS
// `which` the moment-tensor load of tetrahedron `tet` with strike vector s,
// fault normal n and moment magnitude M0, moment density
// (s n^T + n s^T) M0 / V, V the tetrahedron's volume (find_tet.f90:184-210).
int lymph_make_rhs_double_couple(lymph_ctx* c, int which, int32_t tet, const double* s, const double* n, double M0) {
    if (!c || !s || !n || (which != LYMPH_RHS_STAT && which != LYMPH_RHS_DYN) || !std::isfinite(M0))
        return LYMPH_ERR_INVALID;
    if (tet < 0 || tet >= c->n_tet) {
        lymph_set_error("lymph_make_rhs_double_couple: tetrahedron out of range");
        return LYMPH_ERR_INVALID;
    }
    if (!c->have_matrices) {
        lymph_set_error("lymph_make_rhs_double_couple: call lymph_make_matrices first");
        return LYMPH_ERR_ORDER;
    }
    int32_t P = 0, tv[4];
    LYMPH_CUDA_TRY(cudaMemcpy(&P, c->d_tet_poly + tet, sizeof(int32_t), cudaMemcpyDeviceToHost));
    LYMPH_CUDA_TRY(cudaMemcpy(tv, c->d_tet_vert + (size_t)tet * 4, sizeof(tv), cudaMemcpyDeviceToHost));
    double X[4][3];
    for (int v = 0; v < 4; ++v)
        LYMPH_CUDA_TRY(cudaMemcpy(X[v], c->d_coords + (size_t)tv[v] * 3, sizeof(double) * 3, cudaMemcpyDeviceToHost));
    // volume = |det [x_v 1]| / 6 (find_tet.f90:208), expanded along the ones column
    double a[3][3];
    for (int r = 0; r < 3; ++r)
        for (int k = 0; k < 3; ++k) a[r][k] = X[r + 1][k] - X[0][k];
    const double det = a[0][0] * (a[1][1] * a[2][2] - a[1][2] * a[2][1]) - a[0][1] * (a[1][0] * a[2][2] - a[1][2] * a[2][0]) +
                       a[0][2] * (a[1][0] * a[2][1] - a[1][1] * a[2][0]);
    const double vol = std::fabs(det) / 6.0;
    if (!(vol > 0.0)) {
        lymph_set_error("lymph_make_rhs_double_couple: degenerate tetrahedron");
        return LYMPH_EXIT_ELEM_ORIENT;
    }
    double moment[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) moment[i * 3 + j] = (s[i] * n[j] + s[j] * n[i]) * M0 / vol;
    double* out = (which == LYMPH_RHS_STAT) ? c->d_rhs_stat : c->d_rhs_dyn;
    c->rhs_version++;
    LYMPH_TRY(lymph_dev_double_couple(c, tet, P, moment, out));
    LYMPH_TRY(lymph_sync_status(c, "lymph_make_rhs_double_couple"));
    if (which == LYMPH_RHS_STAT) c->have_rhs_stat = true; else c->have_rhs_dyn = true;
    return LYMPH_OK;
}

int lymph_set_dt(lymph_ctx* c, double dt) {
    if (!c || !(dt > 0.0) || !std::isfinite(dt)) return LYMPH_ERR_INVALID;
    c->dt = dt;
    if (c->graph_exec) { cudaGraphExecDestroy(c->graph_exec); c->graph_exec = nullptr; }
    if (c->n_abs > 0 && c->have_matrices && c->winv_dt != dt) {
        // the absorbing polyhedra's M (x) I + dt/2 D depends on dt
        LYMPH_TRY(lymph_dev_damping(c, false));
        return lymph_sync_status(c, "lymph_set_dt");
    }
    return LYMPH_OK;
}

int lymph_get_dt(const lymph_ctx* c, double* dt) {
    if (!c || !dt) return LYMPH_ERR_INVALID;
    *dt = c->dt;
    return LYMPH_OK;
}

int lymph_max_eigenvalue(lymph_ctx* c, int32_t iters, double* lam) {
    if (!c || !lam || iters < 1) return LYMPH_ERR_INVALID;
    if (!c->have_matrices) { lymph_set_error("lymph_max_eigenvalue: call lymph_make_matrices first"); return LYMPH_ERR_ORDER; }
    const size_t nv = (size_t)c->n_poly * c->nd;
    std::vector<double> x(nv);
    uint64_t st = 0x243F6A8885A308D3ull;  // fixed pseudo-random start vector
    for (size_t i = 0; i < nv; ++i) {
        st = st * 6364136223846793005ull + 1442695040888963407ull;
        x[i] = ((double)(st >> 11) / 9007199254740992.0) - 0.5;
    }
    double *dx = nullptr, *dy = nullptr;
    if (cudaMalloc(&dx, nv * sizeof(double)) != cudaSuccess || cudaMalloc(&dy, nv * sizeof(double)) != cudaSuccess) {
        if (dx) cudaFree(dx);
        lymph_set_error("lymph_max_eigenvalue: out of memory");
        return LYMPH_ERR_OOM;
    }
    int rc = LYMPH_OK;
    if (cudaMemcpyAsync(dx, x.data(), nv * sizeof(double), cudaMemcpyHostToDevice, c->stream) != cudaSuccess) rc = LYMPH_ERR_CUDA;
    if (rc == LYMPH_OK) rc = lymph_dev_power_iteration(c, dx, dy, c->d_scalar, iters);
    double ss = 0.0;
    if (rc == LYMPH_OK && cudaMemcpyAsync(&ss, c->d_scalar, sizeof(double), cudaMemcpyDeviceToHost, c->stream) != cudaSuccess)
        rc = LYMPH_ERR_CUDA;
    cudaStreamSynchronize(c->stream);
    cudaFree(dx);
    cudaFree(dy);
    LYMPH_TRY(rc);
    *lam = std::sqrt(ss);  // |M^-1 K x| with |x| = 1
    return lymph_sync_status(c, "lymph_max_eigenvalue");
}

int lymph_launch_count(const lymph_ctx* c, int64_t* count) {
    if (!c || !count) return LYMPH_ERR_INVALID;
    *count = c->launches;
    return LYMPH_OK;
}

int lymph_device_bytes(const lymph_ctx* c, int64_t* bytes) {
    if (!c || !bytes) return LYMPH_ERR_INVALID;
    *bytes = c->device_bytes;
    return LYMPH_OK;
}

}  // extern "C"
