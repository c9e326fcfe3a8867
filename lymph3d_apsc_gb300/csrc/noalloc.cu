// noalloc.cu -- an L2-error entry point that allocates no device memory.
//
// lymph_error_l2 keeps its per-polyhedron partial sums in buffers the
// context allocated with cudaMalloc.  Some callers cannot allocate device
// memory at the time they need the norm: a driver that hands all device
// memory to its own pool up front, a process running under a device-memory
// cap that is already reached, or code that must not trigger the implicit
// synchronisation a cudaMalloc/cudaFree may cause in the middle of a time
// loop.  lymph_error_l2_noalloc serves them: the caller passes device
// pointers to its own inputs and a host pointer for the result, and the
// partial sums live in one file-scope device array of fixed size that the
// module carries from load to exit on every GPU that loads the library.

#include <mutex>

#include "common.cuh"

namespace {

// Largest number of polyhedra one call accepts; the scratch is that many
// partial sums plus the total (2 MiB + 8 bytes per device).
constexpr int NOALLOC_MAX_POLY = 262144;

static __device__ __align__(256) double g_l2_scratch[NOALLOC_MAX_POLY + 1];

// Device address of g_l2_scratch per device.  In host code the symbol is
// only a host-side stand-in, so the address is looked up once per device
// (with that device current) and cached.
std::mutex g_scratch_mu;
double* g_scratch_dev[128] = {};

int scratch_address(double** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        lymph_set_error(std::string("lymph_error_l2_noalloc: cudaGetDevice: ") + cudaGetErrorString(e));
        return LYMPH_ERR_CUDA;
    }
    if (dev < 0 || dev >= 128) {
        lymph_set_error("lymph_error_l2_noalloc: device index out of range");
        return LYMPH_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_dev[dev]) {
        double* p = nullptr;
        e = cudaGetSymbolAddress((void**)&p, g_l2_scratch);
        if (e != cudaSuccess || p == nullptr) {
            lymph_set_error(std::string("lymph_error_l2_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            return LYMPH_ERR_CUDA;
        }
        g_scratch_dev[dev] = p;
    }
    *out = g_scratch_dev[dev];
    return LYMPH_OK;
}

// The context path's arithmetic (the same device functions, common.cuh):
// per polyhedron sum_i du_i^T M du_i (COMPUTE_ERROR_L2_MATRIX_FREE's body),
// then the fixed-order sum.
__global__ void k_l2_partial_noalloc(int n_poly, int NP, const double* __restrict__ Mm, const double* __restrict__ uh,
                                     const double* __restrict__ uex, double* partial) {
    const int P = blockIdx.x * blockDim.x + threadIdx.x;
    if (P >= n_poly) return;
    partial[P] = l2_partial_poly(P, NP, Mm, uh, uex);
}

__global__ void __launch_bounds__(1024) k_sum_noalloc(int64_t n, const double* __restrict__ v, double* out) {
    sum_fixed_order_1024(n, v, out);
}

}  // namespace

extern "C" int lymph_error_l2_noalloc(const double* d_mass_modal, const double* d_uh, const double* d_uex,
                                      int32_t n_poly, int32_t Np, double* sumsq) {
    if (!d_mass_modal || !d_uh || !d_uex || !sumsq) {
        lymph_set_error("lymph_error_l2_noalloc: null pointer");
        return LYMPH_ERR_INVALID;
    }
    if (n_poly <= 0 || n_poly > NOALLOC_MAX_POLY) {
        lymph_set_error("lymph_error_l2_noalloc: n_poly must be 1.." + std::to_string(NOALLOC_MAX_POLY) +
                        " (the size of the static scratch array); got " + std::to_string(n_poly));
        return LYMPH_ERR_INVALID;
    }
    if (Np != 4 && Np != 10 && Np != 20 && Np != 35) {
        lymph_set_error("lymph_error_l2_noalloc: Np must be 4, 10, 20 or 35 (degree 1..4)");
        return LYMPH_ERR_INVALID;
    }
    double* scratch = nullptr;
    LYMPH_TRY(scratch_address(&scratch));
    // every partial is overwritten and the total is written once, so nothing
    // left over from an earlier call is read
    k_l2_partial_noalloc<<<(n_poly + 127) / 128, 128>>>(n_poly, Np, d_mass_modal, d_uh, d_uex, scratch);
    LYMPH_CUDA_TRY(cudaGetLastError());
    k_sum_noalloc<<<1, 1024>>>(n_poly, scratch, scratch + NOALLOC_MAX_POLY);
    LYMPH_CUDA_TRY(cudaGetLastError());
    LYMPH_CUDA_TRY(cudaMemcpy(sumsq, scratch + NOALLOC_MAX_POLY, sizeof(double), cudaMemcpyDeviceToHost));
    return LYMPH_OK;
}
