// export.cu -- nodal values of the modal solution at the tetrahedra's
// vertices: the evaluation half of EXPORT_SOLUTION
// (src/solution_processing.f90:62-194); the file writers (VTK / VTU / PVD,
// export_file_formats.f90) are host code in lymph3d_apsc_gb300/export.py.
//
// u_nod[t][v][k] = sum_i u[P][k*Np + i] L_bx(i)(x_v) L_by(i)(y_v) L_bz(i)(z_v)
// with P the polyhedron of tetrahedron t, L the bounding-box-scaled Legendre
// polynomials of the basis and (x_v, y_v, z_v) the v-th vertex of t: the
// reference's u_nod_vet(k, ivert, ie) in the same memory order (k fastest).

#include "common.cuh"

namespace {

// One thread per (tetrahedron, vertex); the basis list comes from the
// reference tables, the bounding box from the polyhedron geometry.
__global__ void k_nodal_values(int n_tet, int Np, const double* __restrict__ X, const int32_t* __restrict__ tv,
                               const int32_t* __restrict__ tp, const double* __restrict__ bbox,
                               const RefTables* __restrict__ ref, const double* __restrict__ u, double* out) {
    const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q >= (int64_t)n_tet * 4) return;
    const int64_t t = q / 4;
    const int v = (int)(q % 4);
    const int P = tp[t];
    const double* xv = X + (int64_t)tv[t * 4 + v] * 3;
    const double pt[3] = {xv[0], xv[1], xv[2]};
    const double* bb = bbox + (int64_t)P * 6;
    const double* uP = u + (int64_t)P * 3 * Np;
    double acc[3] = {0.0, 0.0, 0.0};
    for (int i = 0; i < Np; ++i) {
        double phi, dphi[3];
        basis_eval(pt, bb, ref->blist + 3 * i, &phi, dphi);
        acc[0] += uP[i] * phi;
        acc[1] += uP[Np + i] * phi;
        acc[2] += uP[2 * Np + i] * phi;
    }
    out[q * 3 + 0] = acc[0];
    out[q * 3 + 1] = acc[1];
    out[q * 3 + 2] = acc[2];
}

}  // namespace


extern "C" {

// Nodal values of the field in `slot` at the four vertices of every
// tetrahedron: out (host) [n_tet][4][3], the layout of the reference's
// u_nod_vet(DIM, 4, num_elem_loc).  Replaces the evaluation loop of
// EXPORT_SOLUTION (solution_processing.f90:62-194).
int lymph_nodal_values(lymph_ctx* c, int slot, double* out) {
    if (!c || !out || slot < 0 || slot > 3) return LYMPH_ERR_INVALID;
    if (!c->have_matrices) {
        lymph_set_error("lymph_nodal_values: call lymph_make_matrices first (it builds the bounding boxes)");
        return LYMPH_ERR_ORDER;
    }
    const size_t bytes = sizeof(double) * (size_t)c->n_tet * 12;
    double* d_out = nullptr;
    if (cudaMalloc(&d_out, bytes) != cudaSuccess) {
        lymph_set_error("lymph_nodal_values: out of memory");
        return LYMPH_ERR_OOM;
    }
    const int64_t n = (int64_t)c->n_tet * 4;
    k_nodal_values<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(c->n_tet, c->Np, c->d_coords, c->d_tet_vert,
                                                                      c->d_tet_poly, c->d_bbox, c->d_ref,
                                                                      lymph_slot_ptr(c, slot), d_out);
    c->launches++;
    cudaError_t e = cudaMemcpyAsync(out, d_out, bytes, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cudaFree(d_out);
    if (e != cudaSuccess) {
        lymph_set_error(std::string("lymph_nodal_values: ") + cudaGetErrorString(e));
        return LYMPH_ERR_CUDA;
    }
    return lymph_sync_status(c, "lymph_nodal_values");
}

}  // extern "C"
