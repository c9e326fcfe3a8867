// step.cu -- the per-step hot kernel and the error norms.
//
// One CTA per polyhedron P fuses what TIME_STEP_MATRIX_FREE
// (src/matrix_free.f90:1230-1385) does for one element:
//   1. y = sum_b K_{P,col(b)} u_{col(b)}     (self + neighbour blocks; the
//      neighbour coefficients the reference receives by MPI_EXCHANGE_DOF are
//      gathered from global memory, L2-resident)
//   2. tmp = -y + F_stat + F_dyn g(t)
//   3. x = M^-1 tmp per component: the value of the reference's
//      solve_LU(R^T, R, tmp) (vet_mat_operations.f90:123-153), applied as a
//      dense FP64 product with the inverse built once from the same factor
//   4. u^{n+1} = dt^2 x + 2 u^n - u^{n-1}    (written over u^{n-1} in place)
// Blocks are stored column-major so that thread r (row r) reads
// K[c][r] for consecutive r: coalesced, streamed once per step with an
// evict-first hint so the state vectors stay in L2.  Threads are laid out as
// S column slices x ND rows, S chosen per degree so that ND*S fills whole
// warps; the S partial sums of a row are combined in a fixed order.

#include "step_body.cuh"

namespace {

using namespace stepk;

// One CTA per polyhedron.
template <int PD, typename KT, int MODE>
__global__ void __launch_bounds__(Shape<PD>::T, Shape<PD>::MINB) k_step(StepArgs A) {
    __shared__ __align__(16) char smem[SmemSize<PD, KT>::bytes];
    step_poly<PD, KT, MODE>(A, blockIdx.x, smem);
}

__global__ void k_bump(int64_t* idx) { *idx += 1; }

// COMPUTE_ERROR_L2_MATRIX_FREE body per polyhedron: sum_i du_i^T M du_i.
__global__ void k_l2_partial(int n_poly, int NP, const double* __restrict__ Mm, const double* __restrict__ uh,
                             const double* __restrict__ uex, double* partial) {
    const int P = blockIdx.x * blockDim.x + threadIdx.x;
    if (P >= n_poly) return;
    partial[P] = l2_partial_poly(P, NP, Mm, uh, uex);
}

// Deterministic sum of n values (one CTA of 1024 threads).
__global__ void __launch_bounds__(1024) k_sum(int64_t n, const double* __restrict__ v, double* out) {
    sum_fixed_order_1024(n, v, out);
}

// Sum of squares of v into *out (one CTA, fixed order).
__global__ void k_sumsq(int64_t n, const double* __restrict__ v, double* out) {
    __shared__ double red[1024];
    double s = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) s += v[i] * v[i];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = red[0];
}

// x = y / sqrt(*ss)
__global__ void k_normalize(int64_t n, const double* __restrict__ y, const double* __restrict__ ss, double* x) {
    const double inv = 1.0 / sqrt(*ss);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i] = y[i] * inv;
}

template <int PD, typename KT, int MODE>
int launch_step_t(lymph_ctx* c, const StepArgs& A) {
    k_step<PD, KT, MODE><<<c->n_poly, Shape<PD>::T, 0, c->stream>>>(A);
    c->launches++;
    return LYMPH_OK;
}

template <typename KT, int MODE>
int launch_step_p(lymph_ctx* c, const StepArgs& A) {
    switch (c->p) {
        case 1: return launch_step_t<1, KT, MODE>(c, A);
        case 2: return launch_step_t<2, KT, MODE>(c, A);
        case 3: return launch_step_t<3, KT, MODE>(c, A);
        case 4: return launch_step_t<4, KT, MODE>(c, A);
        default: lymph_set_error("degree not supported on the device"); return LYMPH_ERR_INVALID;
    }
}

template <int MODE>
int launch_step_mode(lymph_ctx* c, const StepArgs& A, bool fp32) {
    return fp32 ? launch_step_p<float, MODE>(c, A) : launch_step_p<double, MODE>(c, A);
}

}  // namespace

int lymph_dev_mf(lymph_ctx* c, int mode, const stepk::StepArgs& A);

namespace {

// The operator pass of a step mode in the context's precision: the fused
// block-CSR kernel (FP64 or FP32 blocks) or the matrix-free neighbour kernel.
template <int MODE>
int launch_ctx(lymph_ctx* c, const StepArgs& A) {
    if (c->precision == LYMPH_MIXED_MF) return lymph_dev_mf(c, MODE, A);
    return launch_step_mode<MODE>(c, A, c->precision == LYMPH_MIXED);
}

StepArgs base_args(lymph_ctx* c) {
    StepArgs A;
    A.row_ptr = c->d_row_ptr; A.col = c->d_col; A.K = c->d_K; A.Minv = c->d_Minv;
    A.rhs_stat = c->d_rhs_stat; A.rhs_dyn = c->d_rhs_dyn; A.gvals = c->d_gvals; A.step_idx = c->d_step_idx;
    A.u0 = nullptr; A.un = nullptr; A.out = nullptr; A.partial = c->d_partial; A.dt = c->dt; A.status = c->d_status;
    A.n_poly = c->n_poly;
    A.abs_idx = c->n_abs > 0 ? c->d_abs_idx : nullptr;
    A.Dabs = c->d_Dabs;
    A.Winv = c->d_Winv;
    return A;
}

}  // namespace

// One leapfrog step on the context stream (no rotation): reads U0/UN buffers,
// writes u^{n+1} over U0.  The caller flips c->cur afterwards.
int lymph_dev_step(lymph_ctx* c, bool bump) {
    StepArgs A = base_args(c);
    A.u0 = c->d_buf[c->cur ^ 1];
    A.un = c->d_buf[c->cur];
    A.out = c->d_buf[c->cur ^ 1];
    LYMPH_TRY(launch_ctx<MODE_STEP>(c, A));
    if (bump) {
        k_bump<<<1, 1, 0, c->stream>>>(c->d_step_idx);
        c->launches++;
    }
    return LYMPH_OK;
}

int lymph_dev_bump(lymph_ctx* c) {
    k_bump<<<1, 1, 0, c->stream>>>(c->d_step_idx);
    c->launches++;
    return LYMPH_OK;
}

// out = M^-1 K u (u read from `u`), for the power iteration of the CFL bound.
int lymph_dev_apply(lymph_ctx* c, const double* u, double* out) {
    StepArgs A = base_args(c);
    A.un = u;
    A.u0 = u;
    A.out = out;
    return launch_ctx<MODE_APPLY>(c, A);
}

// out = K u in the context's precision (the operator apply of
// TIME_STEP_MATRIX_FREE before the mass-matrix solve).
int lymph_dev_ku(lymph_ctx* c, const double* u, double* out) {
    StepArgs A = base_args(c);
    A.un = u;
    A.u0 = u;
    A.out = out;
    return launch_ctx<MODE_KU>(c, A);
}

// out = M^-1 K u with the FP32 copy K32 of an FP64 context's blocks (the
// surrogate's predictor term, whose own error is far above FP32 rounding).
int lymph_dev_apply_fp32(lymph_ctx* c, const float* K32, const double* u, double* out) {
    StepArgs A = base_args(c);
    A.K = K32;
    A.un = u;
    A.u0 = u;
    A.out = out;
    return launch_step_p<float, MODE_APPLY>(c, A);
}

// dst[i] = (float)src[i]
__global__ void k_blocks_to_f32(int64_t n, const double* __restrict__ src, float* dst) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        dst[i] = (float)src[i];
}

// The FP32 copy of an FP64 context's blocks, made on first use (null when the
// context is FP32 already or the copy does not fit in device memory).
const float* lymph_dev_blocks_f32(lymph_ctx* c) {
    if (c->precision != LYMPH_FP64 || !c->have_matrices) return nullptr;
    const int64_t nK = c->n_blocks * (int64_t)c->nd * c->nd;
    if (!c->d_K32) {
        if (cudaMalloc(&c->d_K32, sizeof(float) * (size_t)nK) != cudaSuccess) {
            cudaGetLastError();  // clear the allocation failure: the caller falls back to the FP64 blocks
            c->d_K32 = nullptr;
            return nullptr;
        }
        c->device_bytes += (int64_t)sizeof(float) * nK;
        c->k32_valid = false;
    }
    if (!c->k32_valid) {
        k_blocks_to_f32<<<4096, 256, 0, c->stream>>>(nK, (const double*)c->d_K, c->d_K32);
        c->launches++;
        c->k32_valid = true;
    }
    return c->d_K32;
}

// `iters` power iterations x <- M^-1 K x / |M^-1 K x| entirely on the
// device; x must hold a nonzero start vector, y is scratch; *d_ss receives
// |M^-1 K x|^2 of the last iteration (x normalised before it).
int lymph_dev_power_iteration(lymph_ctx* c, double* x, double* y, double* d_ss, int iters) {
    const int64_t n = (int64_t)c->n_poly * c->nd;
    k_sumsq<<<1, 1024, 0, c->stream>>>(n, x, d_ss);
    k_normalize<<<1024, 256, 0, c->stream>>>(n, x, d_ss, x);
    c->launches += 2;
    for (int it = 0; it < iters; ++it) {
        LYMPH_TRY(lymph_dev_apply(c, x, y));
        k_sumsq<<<1, 1024, 0, c->stream>>>(n, y, d_ss);
        c->launches++;
        if (it + 1 < iters) {
            k_normalize<<<1024, 256, 0, c->stream>>>(n, y, d_ss, x);
            c->launches++;
        }
    }
    LYMPH_CUDA_TRY(cudaGetLastError());
    return LYMPH_OK;
}

int lymph_dev_first_step(lymph_ctx* c) {
    StepArgs A = base_args(c);
    A.u0 = c->d_buf[c->cur ^ 1];
    A.un = c->d_v0;
    A.out = c->d_buf[c->cur];
    return launch_ctx<MODE_FIRST>(c, A);
}

// du . (A du) per polyhedron with FP64 A_dg blocks in `blocks`, then the sum.
int lymph_dev_error_dg(lymph_ctx* c, const void* blocks, const double* uh, const double* uex, double* d_out) {
    StepArgs A = base_args(c);
    A.K = blocks;
    A.u0 = uh;
    A.un = uex;
    LYMPH_TRY(launch_step_mode<MODE_DG>(c, A, false));
    k_sum<<<1, 1024, 0, c->stream>>>(c->n_poly, c->d_partial, d_out);
    c->launches++;
    LYMPH_CUDA_TRY(cudaGetLastError());
    return LYMPH_OK;
}

// Leapfrog energy terms: d_out[0] = |ub - ua|^2_M (rho-weighted mass),
// d_out[1] = ub . K ua.
int lymph_dev_energy(lymph_ctx* c, const double* ua, const double* ub, double* d_out) {
    k_l2_partial<<<(c->n_poly + 127) / 128, 128, 0, c->stream>>>(c->n_poly, c->Np, c->d_M, ub, ua, c->d_partial);
    k_sum<<<1, 1024, 0, c->stream>>>(c->n_poly, c->d_partial, d_out);
    StepArgs A = base_args(c);
    A.u0 = ua;
    A.un = ub;
    LYMPH_TRY(launch_ctx<MODE_BILIN>(c, A));
    k_sum<<<1, 1024, 0, c->stream>>>(c->n_poly, c->d_partial, d_out + 1);
    c->launches += 3;
    LYMPH_CUDA_TRY(cudaGetLastError());
    return LYMPH_OK;
}

int lymph_dev_error_l2(lymph_ctx* c, const double* uh, const double* uex, double* d_out) {
    k_l2_partial<<<(c->n_poly + 127) / 128, 128, 0, c->stream>>>(c->n_poly, c->Np, c->d_Mm, uh, uex, c->d_partial);
    k_sum<<<1, 1024, 0, c->stream>>>(c->n_poly, c->d_partial, d_out);
    c->launches += 2;
    LYMPH_CUDA_TRY(cudaGetLastError());
    return LYMPH_OK;
}
