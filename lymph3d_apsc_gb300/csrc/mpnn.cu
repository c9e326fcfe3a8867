// mpnn.cu -- the learned surrogate's network: forward, backward and Adam in
// hand-written CUDA (no counterpart in the reference).
//
// Per polyhedron (node) i, with face-area weights w_ij (rows sum to 1) and
// aggregated shared-face geometry g_i = sum_j w_ij e_ij:
//     h = relu(x W0 + b0)
//     L times:  m = relu(h Wm + bm);  a = W m;  h += relu([h a g] Wu + bu)
//     y = h Wo + bo
// Optional gated head (lymph_mpnn_set_gate): y holds per-node coefficients
// alpha[j][b][i] (j < 2 outputs, b < B basis vectors, i < 3 components) and
// the effective output is  yg[j][i*Np + m] = sum_b alpha[j][b][i] x[b*nd + i*Np + m]
// (nd = 3 Np): a learned per-node combination of the first B feature blocks.
// Weight matrices are kept as FP32 masters for Adam and as BF16 copies that
// every GEMM reads; activations and accumulation are FP32.  The forward GEMMs
// run on the tcgen05 tensor cores (umma_gemm.cuh: the activations split into
// TF32 hi and lo parts, the BF16 weights exact in TF32, FP32 accumulation in
// tensor memory) whenever the shapes suit it, else on the FP32 SIMT kernel
// k_gemm, which also runs the backward.  The concatenation [h a g] is never
// formed: the tensor-core GEMM reads it as three K segments, the SIMT path as
// three GEMMs on row slices of Wu accumulating into one output.  Aggregation
// is a CSR gather (fixed order); its adjoint uses the transposed CSR, so
// training is deterministic.

#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "common.cuh"
#include "umma_gemm.cuh"
#include "umma_ws.cuh"

int lymph_dev_apply(lymph_ctx* c, const double* u, double* out);  // out = M^-1 K u (step.cu)
int lymph_dev_apply_fp32(lymph_ctx* c, const float* K32, const double* u, double* out);
const float* lymph_dev_blocks_f32(lymph_ctx* c);

namespace {

// ---------------------------------------------------------------------------
// GEMM: C[M x N] (op) = op(A)[M x K] * op(B)[K x N] (+ bias), FP32 accumulate.
// op(A)[m,k] = TA ? A[k*lda + m] : A[m*lda + k]; op(B)[k,n] = TB ? B[n*ldb + k]
// : B[k*ldb + n].  64 x 64 tiles, 256 threads, 4 x 4 outputs per thread.
// ---------------------------------------------------------------------------
// EPI_STORE: C = v; EPI_ADD: C += v; EPI_RELU: Z = v, C = relu(v);
// EPI_ADD_RELU: Z = v, C += relu(v); EPI_ACC_RELU_ADD: v += Z, Z = v, C += relu(v)
// (v = the product plus the bias, Z the pre-activation buffer, same layout as C).
enum { EPI_STORE = 0, EPI_ADD = 1, EPI_RELU = 2, EPI_ADD_RELU = 3, EPI_ACC_RELU_ADD = 4 };

__device__ __forceinline__ float to_f(float v) { return v; }
__device__ __forceinline__ float to_f(__nv_bfloat16 v) { return __bfloat162float(v); }

template <bool TA, bool TB, typename BT>
__global__ void __launch_bounds__(256) k_gemm(int M, int N, int K, const float* __restrict__ A, int lda,
                                              const BT* __restrict__ B, int ldb, float* C, int ldc,
                                              const float* __restrict__ bias, float* Zpre, int epi) {
    constexpr int TM = 64, TN = 64, TK = 16;
    __shared__ float As[TK][TM + 1];
    __shared__ float Bs[TK][TN + 1];
    const int tid = threadIdx.x;
    const int m0 = blockIdx.y * TM, n0 = blockIdx.x * TN;
    const int tr = tid / 16, tc = tid % 16;  // 16 x 16 threads, 4 x 4 each
    float acc[4][4] = {};
    for (int k0 = 0; k0 < K; k0 += TK) {
        for (int i = tid; i < TM * TK; i += 256) {
            const int mm = i % TM, kk = i / TM;
            const int m = m0 + mm, k = k0 + kk;
            float v = 0.0f;
            if (m < M && k < K) v = TA ? A[(int64_t)k * lda + m] : A[(int64_t)m * lda + k];
            As[kk][mm] = v;
        }
        for (int i = tid; i < TN * TK; i += 256) {
            const int nn = i % TN, kk = i / TN;
            const int n = n0 + nn, k = k0 + kk;
            float v = 0.0f;
            if (n < N && k < K) v = to_f(TB ? B[(int64_t)n * ldb + k] : B[(int64_t)k * ldb + n]);
            Bs[kk][nn] = v;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < TK; ++kk) {
            float a[4], b[4];
#pragma unroll
            for (int r = 0; r < 4; ++r) a[r] = As[kk][tr + 16 * r];
#pragma unroll
            for (int c = 0; c < 4; ++c) b[c] = Bs[kk][tc + 16 * c];
#pragma unroll
            for (int r = 0; r < 4; ++r)
#pragma unroll
                for (int c = 0; c < 4; ++c) acc[r][c] += a[r] * b[c];
        }
        __syncthreads();
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const int m = m0 + tr + 16 * r;
        if (m >= M) continue;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const int n = n0 + tc + 16 * c;
            if (n >= N) continue;
            float v = acc[r][c] + (bias ? bias[n] : 0.0f);
            float* dst = C + (int64_t)m * ldc + n;
            if (epi == EPI_STORE) *dst = v;
            else if (epi == EPI_ADD) *dst += v;
            else {
                if (epi == EPI_ACC_RELU_ADD) v += Zpre[(int64_t)m * ldc + n];
                if (Zpre) Zpre[(int64_t)m * ldc + n] = v;
                const float rv = v > 0.0f ? v : 0.0f;
                if (epi == EPI_RELU) *dst = rv;
                else *dst += rv;
            }
        }
    }
}

// out[i, :] = sum_{k in row i} val[k] * in[idx[k], :]   (width columns)
__global__ void k_aggregate(int n, int width, const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                            const float* __restrict__ val, const float* __restrict__ in, float* out) {
    const int i = blockIdx.x;
    if (i >= n) return;
    for (int c = threadIdx.x; c < width; c += blockDim.x) {
        float s = 0.0f;
        for (int k = ptr[i]; k < ptr[i + 1]; ++k) s += val[k] * in[(int64_t)idx[k] * width + c];
        out[(int64_t)i * width + c] = s;
    }
}

// The same with one warp per node and 16-byte loads (width a multiple of 4):
// each neighbour row is read as one coalesced segment; the sum over the
// neighbours runs in the CSR order, as in k_aggregate.
__global__ void __launch_bounds__(256) k_aggregate_v4(int n, int width, const int32_t* __restrict__ ptr,
                                                      const int32_t* __restrict__ idx, const float* __restrict__ val,
                                                      const float* __restrict__ in, float* out) {
    const int i = blockIdx.x * 8 + threadIdx.x / 32, lane = threadIdx.x % 32;
    if (i >= n) return;
    const int k0 = ptr[i], k1 = ptr[i + 1];
    for (int c = 4 * lane; c < width; c += 128) {
        float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
        for (int k = k0; k < k1; ++k) {
            const float w = val[k];
            const float4 v = *(const float4*)(in + (int64_t)idx[k] * width + c);
            s.x += w * v.x; s.y += w * v.y; s.z += w * v.z; s.w += w * v.w;
        }
        *(float4*)(out + (int64_t)i * width + c) = s;
    }
}

// dz = dy * (z > 0)
__global__ void k_relu_back(int64_t n, const float* __restrict__ dy, const float* __restrict__ z, float* dz) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        dz[i] = z[i] > 0.0f ? dy[i] : 0.0f;
}

// column sums of dz [M x N] into db (bias gradient), one thread per column
__global__ void k_colsum(int M, int N, const float* __restrict__ dz, float* db, int accumulate) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    float s = 0.0f;
    for (int m = 0; m < M; ++m) s += dz[(int64_t)m * N + n];
    db[n] = accumulate ? db[n] + s : s;
}

// loss = mean (y - t)^2 (partials per block, then host sum), dy = 2 (y - t) / n
__global__ void k_mse(int64_t n, const float* __restrict__ y, const float* __restrict__ t, float* dy, double* partial) {
    __shared__ double red[256];
    double s = 0.0;
    const float inv = 2.0f / (float)n;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float d = y[i] - t[i];
        s += (double)d * d;
        dy[i] = inv * d;
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

// Adam on FP32 masters; weight matrices are re-rounded to their BF16 copies.
__global__ void k_adam(int64_t n, float* p, const float* __restrict__ g, float* m, float* v, __nv_bfloat16* pb,
                       float lr, float b1, float b2, float eps, float c1, float c2) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.0f - b1) * gi;
        const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float pi = p[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
        p[i] = pi;
        if (pb) pb[i] = __float2bfloat16_rn(pi);
    }
}

__global__ void k_to_bf16(int64_t n, const float* __restrict__ a, __nv_bfloat16* b) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = __float2bfloat16_rn(a[i]);
}

// Gated head: yg[P][j*nd + c] = sum_b y[P][(j*B + b)*3 + i] x[P][b*nd + c],
// i = c / Np (the displacement component of DOF c).
__global__ void k_gate(int N, int nd, int B, int F, const float* __restrict__ y, const float* __restrict__ x,
                       float* yg) {
    const int Np = nd / 3, O = 2 * B * 3;
    const int64_t tot = (int64_t)N * 2 * nd;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < tot; q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t P = q / (2 * nd);
        const int r = (int)(q % (2 * nd)), j = r / nd, c = r % nd, i = c / Np;
        float v = 0.0f;
        for (int b = 0; b < B; ++b) v += y[P * O + (j * B + b) * 3 + i] * x[P * F + b * nd + c];
        yg[q] = v;
    }
}

// Its adjoint: dy[P][(j*B + b)*3 + i] = sum_m dyg[P][j*nd + i*Np + m] x[P][b*nd + i*Np + m]
__global__ void k_gate_back(int N, int nd, int B, int F, const float* __restrict__ dyg, const float* __restrict__ x,
                            float* dy) {
    const int Np = nd / 3, O = 2 * B * 3;
    const int64_t tot = (int64_t)N * O;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < tot; q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t P = q / O;
        const int o = (int)(q % O), i = o % 3, jb = o / 3, j = jb / B, b = jb % B;
        const float* g = dyg + P * 2 * nd + j * nd + i * Np;
        const float* xv = x + P * F + b * nd + i * Np;
        float s = 0.0f;
        for (int m = 0; m < Np; ++m) s += g[m] * xv[m];
        dy[q] = s;
    }
}

}  // namespace

// ---------------------------------------------------------------------------
// network object
// ---------------------------------------------------------------------------
struct lymph_mpnn {
    int F = 0, H = 0, O = 0, L = 0, G = 0;
    cudaStream_t stream = nullptr;
    // parameter offsets inside one FP32 buffer; matrices also have BF16 copies
    struct P { int64_t off, rows, cols; bool matrix; };
    std::vector<P> par;  // order: W0 b0 (Wm bm Wu bu)*L Wo bo
    int64_t n_par = 0;
    float *d_p = nullptr, *d_g = nullptr, *d_m = nullptr, *d_v = nullptr;
    __nv_bfloat16* d_pb = nullptr;
    int64_t adam_t = 0;
    // activations for the current graph size
    int n_cap = 0;
    float *d_x = nullptr, *d_z0 = nullptr, *d_y = nullptr, *d_t = nullptr, *d_dy = nullptr, *d_gf = nullptr;
    // gated head: gate_nd DOFs per node, gate_B basis blocks (0: plain head)
    int gate_nd = 0, gate_B = 0;
    float *d_yg = nullptr, *d_dyg = nullptr;
    std::vector<float*> d_h, d_zm, d_m_, d_a, d_zu;  // per layer
    float *d_dh = nullptr, *d_dz = nullptr, *d_dtmp = nullptr, *d_dm = nullptr;
    double* d_partial = nullptr;
    // surrogate-block scratch (first and second differences, sums of squares)
    int64_t nv_cap = 0;
    double *d_d1 = nullptr, *d_d2 = nullptr, *d_ss = nullptr;
    double* d_u3 = nullptr;  // the predicted u^{n+K}, checked after the closing plain step
    double* d_minvf = nullptr;        // M^-1 rhs_dyn of the context minvf_uid at its rhs_version minvf_ver
    uint64_t minvf_uid = 0;
    int64_t minvf_ver = -1;
    double* d_a1 = nullptr;  // dt^2 M^-1 (K d1 - gdiff F) (a feature)
    double* d_sig = nullptr;  // per-polyhedron scales [n_poly][4] of the last features
    const lymph_ctx* have_u3 = nullptr;      // context of the last prediction
    const lymph_ctx* judge_saved = nullptr;  // context whose pair the judge keeps
    // graph (CSR weights, and transposed)
    int n_nodes = 0;
    int32_t *d_wp = nullptr, *d_wi = nullptr, *d_tp = nullptr, *d_ti = nullptr;
    float *d_wv = nullptr, *d_tv = nullptr;
    int64_t launches = 0;
    // tensor-core forward: per weight matrix W [K][N] (BF16), an FP32 copy of
    // W^T padded to Npad = round16(N) rows (the K-major B operand)
    float* d_wt = nullptr;
    std::vector<int64_t> wt_off;  // per entry of par (matrices only), -1 otherwise
    bool wt_dirty = true;
    bool use_umma = true;         // LYMPH_MPNN_SIMT=1 selects the SIMT GEMMs for the forward too
    bool use_ws = true;           // LYMPH_UMMA_WS=0 selects the cp.async tensor-core kernel over the TMA one
    int* d_status = nullptr;      // bit 0: a tensor-core wait ran out
};

namespace {

int64_t pidx(const lymph_mpnn* n, const char* what, int l) {
    // index into n->par
    if (!strcmp(what, "W0")) return 0;
    if (!strcmp(what, "b0")) return 1;
    if (!strcmp(what, "Wm")) return 2 + 4 * l;
    if (!strcmp(what, "bm")) return 3 + 4 * l;
    if (!strcmp(what, "Wu")) return 4 + 4 * l;
    if (!strcmp(what, "bu")) return 5 + 4 * l;
    if (!strcmp(what, "Wo")) return 2 + 4 * n->L;
    return 3 + 4 * n->L;  // bo
}

float* P_(lymph_mpnn* n, const char* w, int l = 0) { return n->d_p + n->par[pidx(n, w, l)].off; }
float* G_(lymph_mpnn* n, const char* w, int l = 0) { return n->d_g + n->par[pidx(n, w, l)].off; }
const __nv_bfloat16* B_(lymph_mpnn* n, const char* w, int l = 0) { return n->d_pb + n->par[pidx(n, w, l)].off; }

int round16(int x) { return (x + 15) / 16 * 16; }

// Bt[n][k] = W[k][n] for n < N, 0 for N <= n < Npad
__global__ void k_transpose_w(int K, int N, int Npad, const __nv_bfloat16* __restrict__ W, float* Bt) {
    const int64_t tot = (int64_t)Npad * K;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < tot; i += (int64_t)gridDim.x * blockDim.x) {
        const int n = (int)(i / K), k = (int)(i % K);
        Bt[i] = n < N ? __bfloat162float(W[(int64_t)k * N + n]) : 0.0f;
    }
}

// Refreshes the transposed FP32 weight copies after the BF16 weights changed.
void refresh_wt(lymph_mpnn* n) {
    if (!n->wt_dirty) return;
    for (size_t i = 0; i < n->par.size(); ++i) {
        if (n->wt_off[i] < 0) continue;
        const auto& P = n->par[i];
        const int K = (int)P.rows, N = (int)P.cols;
        k_transpose_w<<<256, 256, 0, n->stream>>>(K, N, round16(N), n->d_pb + P.off, n->d_wt + n->wt_off[i]);
        n->launches++;
    }
    n->wt_dirty = false;
}

// Can the tensor-core kernel take this GEMM?  (N <= 256, every K and leading
// dimension a multiple of 4 for its 16-byte loads.)
bool umma_ok(const lymph_mpnn* n, int N, std::initializer_list<int> dims) {
    if (!n->use_umma || N > 256 || N <= 0) return false;
    for (int d : dims)
        if (d % 4) return false;
    return true;
}

using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// cuTensorMapEncodeTiled from the driver (looked up once; null when absent)
EncodeTiled encode_tiled() {
    static EncodeTiled fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiled)p;
    }
    return fn;
}

// A 2-D FP32 tensor map [rows][cols] (row stride ld floats), box 32 x box_rows,
// 128-byte swizzle, zero fill outside the tensor.
bool make_map(CUtensorMap* m, const float* base, int cols, int rows, int ld, int box_rows) {
    EncodeTiled enc = encode_tiled();
    if (!enc) return false;
    const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)ld * 4};
    const cuuint32_t box[2] = {(cuuint32_t)umma::BK, (cuuint32_t)box_rows};
    const cuuint32_t es[2] = {1, 1};
    return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void*)base, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// C = sum_s A_s W_s (+ bias) with the epilogue, on the tensor cores; the
// weight matrix is parameter `pi`, whose rows are the concatenated K of the
// segments.  The warp-specialised TMA kernel runs when its tensor maps can
// be made (and LYMPH_UMMA_WS is not 0), else the cp.async kernel.
void umma_gemm(lymph_mpnn* n, int pi, int M, const umma::Seg* segs, int nseg, const float* bias, float* C, int ldc,
               float* Z, const float* R, int epi) {
    const auto& P = n->par[pi];
    const int N = (int)P.cols, Npad = round16(N), Ktot = (int)P.rows;
    const float* Bt = n->d_wt + n->wt_off[pi];
    if (n->use_ws) {
        umma::WsArgs w;
        std::memset(&w, 0, sizeof(w));
        bool ok = make_map(&w.mapB, Bt, Ktot, Npad, Ktot, Npad < umma::WS_BN ? Npad : umma::WS_BN);
        for (int s = 0; s < nseg && ok; ++s) {
            ok = make_map(&w.mapA[s], segs[s].A, segs[s].K, M, segs[s].lda, umma::BM);
            w.segK[s] = segs[s].K;
        }
        if (ok) {
            w.nseg = nseg; w.M = M; w.N = N; w.Npad = Npad; w.Ktot = Ktot;
            w.bias = bias; w.C = C; w.ldc = ldc; w.Z = Z; w.R = R; w.epi = epi; w.status = n->d_status;
            static bool attr = false;
            if (!attr) {
                cudaFuncSetAttribute(umma::k_umma_gemm_ws, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)umma::WS_SMEM);
                attr = true;
            }
            const dim3 grid((M + umma::BM - 1) / umma::BM, (Npad + umma::WS_BN - 1) / umma::WS_BN);
            umma::k_umma_gemm_ws<<<grid, umma::WS_THREADS, umma::WS_SMEM, n->stream>>>(w);
            n->launches++;
            return;
        }
    }
    umma::Args a;
    for (int s = 0; s < nseg; ++s) a.seg[s] = segs[s];
    a.nseg = nseg;
    a.M = M;
    a.N = N;
    a.Npad = Npad;
    a.Bt = Bt;
    a.Ktot = Ktot;
    a.bias = bias;
    a.C = C;
    a.ldc = ldc;
    a.Z = Z;
    a.R = R;
    a.epi = epi;
    a.status = n->d_status;
    static bool attr_set = false;
    if (!attr_set) {
        cudaFuncSetAttribute(umma::k_umma_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)umma::SMEM_ALLOC);
        attr_set = true;
    }
    const dim3 grid((M + umma::BM - 1) / umma::BM, (a.Npad + umma::BN - 1) / umma::BN);
    umma::k_umma_gemm<<<grid, umma::THREADS, umma::SMEM_ALLOC, n->stream>>>(a);
    n->launches++;
}

int read_status(lymph_mpnn* n, const char* who) {
    int st = 0;
    LYMPH_CUDA_TRY(cudaMemcpyAsync(&st, n->d_status, sizeof(int), cudaMemcpyDeviceToHost, n->stream));
    LYMPH_CUDA_TRY(cudaStreamSynchronize(n->stream));
    if (st) {
        cudaMemsetAsync(n->d_status, 0, sizeof(int), n->stream);
        lymph_set_error(std::string(who) + ": a tensor-core wait ran out (the kernel returned without its result)");
        return LYMPH_ERR_TIMEOUT;
    }
    return LYMPH_OK;
}

template <bool TA, bool TB, typename BT>
void gemm(lymph_mpnn* n, int M, int N, int K, const float* A, int lda, const BT* B, int ldb, float* C, int ldc,
          const float* bias, float* Z, int epi) {
    if (M <= 0 || N <= 0) return;
    dim3 grid((N + 63) / 64, (M + 63) / 64);
    k_gemm<TA, TB, BT><<<grid, 256, 0, n->stream>>>(M, N, K, A, lda, B, ldb, C, ldc, bias, Z, epi);
    n->launches++;
}

void aggregate(lymph_mpnn* n, bool transposed, int width, const float* in, float* out) {
    const int32_t* p = transposed ? n->d_tp : n->d_wp;
    const int32_t* ix = transposed ? n->d_ti : n->d_wi;
    const float* v = transposed ? n->d_tv : n->d_wv;
    if (width % 4 == 0)  // rows of 16-byte multiples from cudaMalloc'd buffers: 16-byte aligned
        k_aggregate_v4<<<(n->n_nodes + 7) / 8, 256, 0, n->stream>>>(n->n_nodes, width, p, ix, v, in, out);
    else
        k_aggregate<<<n->n_nodes, 128, 0, n->stream>>>(n->n_nodes, width, p, ix, v, in, out);
    n->launches++;
}

int ensure_capacity(lymph_mpnn* n, int N) {
    if (N <= n->n_cap) return LYMPH_OK;
    auto fr = [](float*& p) { if (p) cudaFree(p); p = nullptr; };
    fr(n->d_x); fr(n->d_z0); fr(n->d_y); fr(n->d_t); fr(n->d_dy); fr(n->d_gf); fr(n->d_yg); fr(n->d_dyg);
    fr(n->d_dh); fr(n->d_dz); fr(n->d_dtmp); fr(n->d_dm);
    for (auto* v : {&n->d_h, &n->d_zm, &n->d_m_, &n->d_a, &n->d_zu})
        for (auto& p : *v) fr(p);
    const int H = n->H;
    auto al = [&](float*& p, int64_t cnt) { return cudaMalloc(&p, sizeof(float) * (size_t)cnt) == cudaSuccess; };
    const int64_t Ot = n->gate_B ? 2 * n->gate_nd : n->O;  // width of the effective output and target
    bool ok = al(n->d_x, (int64_t)N * n->F) && al(n->d_z0, (int64_t)N * H) && al(n->d_y, (int64_t)N * n->O) &&
              al(n->d_t, (int64_t)N * Ot) && al(n->d_dy, (int64_t)N * n->O) && al(n->d_gf, (int64_t)N * n->G) &&
              (!n->gate_B || (al(n->d_yg, (int64_t)N * Ot) && al(n->d_dyg, (int64_t)N * Ot))) &&
              al(n->d_dh, (int64_t)N * H) && al(n->d_dz, (int64_t)N * H) && al(n->d_dtmp, (int64_t)N * H) &&
              al(n->d_dm, (int64_t)N * H);
    n->d_h.assign(n->L + 1, nullptr);
    n->d_zm.assign(n->L, nullptr);
    n->d_m_.assign(n->L, nullptr);
    n->d_a.assign(n->L, nullptr);
    n->d_zu.assign(n->L, nullptr);
    for (int l = 0; l <= n->L && ok; ++l) ok = al(n->d_h[l], (int64_t)N * H);
    for (int l = 0; l < n->L && ok; ++l)
        ok = al(n->d_zm[l], (int64_t)N * H) && al(n->d_m_[l], (int64_t)N * H) && al(n->d_a[l], (int64_t)N * H) &&
             al(n->d_zu[l], (int64_t)N * H);
    if (!ok) {
        lymph_set_error("lymph_mpnn: cannot allocate activations");
        return LYMPH_ERR_OOM;
    }
    n->n_cap = N;
    return LYMPH_OK;
}

// forward on the current graph; x in d_x, g in d_gf, output in d_y.
// keep_z: also store the pre-activations z0 / zm / zu the backward pass
// reads; inference (forward, predict) leaves them out on the tensor-core
// path, one N x H store per GEMM fewer.
void forward(lymph_mpnn* n, bool keep_z = true) {
    const int N = n->n_nodes, H = n->H, F = n->F, G = n->G, O = n->O;
    const bool tc = umma_ok(n, H, {F, H, G}) && umma_ok(n, O, {H});
    if (tc) {
        // tensor cores: h0 = relu(x W0 + b0); per layer m = relu(h Wm + bm),
        // a = W m, h1 = h + relu([h a g] Wu + bu); y = h Wo + bo
        refresh_wt(n);
        umma::Seg s0[1] = {{n->d_x, F, F}};
        umma_gemm(n, (int)pidx(n, "W0", 0), N, s0, 1, P_(n, "b0"), n->d_h[0], H, keep_z ? n->d_z0 : nullptr,
                  nullptr, umma::EPI_RELU);
        for (int l = 0; l < n->L; ++l) {
            float* h = n->d_h[l];
            umma::Seg sm[1] = {{h, H, H}};
            umma_gemm(n, (int)pidx(n, "Wm", l), N, sm, 1, P_(n, "bm", l), n->d_m_[l], H,
                      keep_z ? n->d_zm[l] : nullptr, nullptr, umma::EPI_RELU);
            aggregate(n, false, H, n->d_m_[l], n->d_a[l]);
            umma::Seg su[3] = {{h, H, H}, {n->d_a[l], H, H}, {n->d_gf, G, G}};
            umma_gemm(n, (int)pidx(n, "Wu", l), N, su, 3, P_(n, "bu", l), n->d_h[l + 1], H,
                      keep_z ? n->d_zu[l] : nullptr, h, umma::EPI_RES_RELU);
        }
        umma::Seg so[1] = {{n->d_h[n->L], H, H}};
        umma_gemm(n, (int)pidx(n, "Wo", 0), N, so, 1, P_(n, "bo"), n->d_y, O, nullptr, nullptr, umma::EPI_STORE);
    } else {
        gemm<false, false, __nv_bfloat16>(n, N, H, F, n->d_x, F, B_(n, "W0"), H, n->d_h[0], H, P_(n, "b0"), n->d_z0,
                                          EPI_RELU);
        for (int l = 0; l < n->L; ++l) {
            float* h = n->d_h[l];
            float* h1 = n->d_h[l + 1];
            cudaMemcpyAsync(h1, h, sizeof(float) * (size_t)N * H, cudaMemcpyDeviceToDevice, n->stream);
            gemm<false, false, __nv_bfloat16>(n, N, H, H, h, H, B_(n, "Wm", l), H, n->d_m_[l], H, P_(n, "bm", l),
                                              n->d_zm[l], EPI_RELU);
            aggregate(n, false, H, n->d_m_[l], n->d_a[l]);
            const __nv_bfloat16* Wu = B_(n, "Wu", l);
            // zu = h Wu[0:H] + a Wu[H:2H] + g Wu[2H:] + bu ; h1 = h + relu(zu)
            gemm<false, false, __nv_bfloat16>(n, N, H, H, h, H, Wu, H, n->d_zu[l], H, P_(n, "bu", l), nullptr,
                                              EPI_STORE);
            gemm<false, false, __nv_bfloat16>(n, N, H, H, n->d_a[l], H, Wu + (int64_t)H * H, H, n->d_zu[l], H,
                                              nullptr, nullptr, EPI_ADD);
            // last slice: finishes zu and adds relu(zu) into h1 in its epilogue
            gemm<false, false, __nv_bfloat16>(n, N, H, G, n->d_gf, G, Wu + (int64_t)2 * H * H, H, h1, H, nullptr,
                                              n->d_zu[l], EPI_ACC_RELU_ADD);
        }
        gemm<false, false, __nv_bfloat16>(n, N, O, H, n->d_h[n->L], H, B_(n, "Wo"), O, n->d_y, O, P_(n, "bo"),
                                          nullptr, EPI_STORE);
    }
    if (n->gate_B) {
        const int64_t tot = (int64_t)N * 2 * n->gate_nd;
        k_gate<<<(int)std::min<int64_t>((tot + 255) / 256, 4096), 256, 0, n->stream>>>(N, n->gate_nd, n->gate_B, n->F,
                                                                                       n->d_y, n->d_x, n->d_yg);
        n->launches++;
    }
}

// effective output (what predictions and the loss use)
const float* eff_out(const lymph_mpnn* n) { return n->gate_B ? n->d_yg : n->d_y; }
int64_t eff_width(const lymph_mpnn* n) { return n->gate_B ? 2 * n->gate_nd : n->O; }

// backward from d_dy; gradients into d_g
void backward(lymph_mpnn* n) {
    const int N = n->n_nodes, H = n->H, F = n->F, G = n->G, O = n->O;
    // Wo, bo
    gemm<true, false, float>(n, H, O, N, n->d_h[n->L], H, n->d_dy, O, G_(n, "Wo"), O, nullptr, nullptr, EPI_STORE);
    k_colsum<<<(O + 127) / 128, 128, 0, n->stream>>>(N, O, n->d_dy, G_(n, "bo"), 0);
    n->launches++;
    // dh = dy Wo^T
    gemm<false, true, __nv_bfloat16>(n, N, H, O, n->d_dy, O, B_(n, "Wo"), O, n->d_dh, H, nullptr, nullptr, EPI_STORE);
    for (int l = n->L - 1; l >= 0; --l) {
        float* h = n->d_h[l];
        const __nv_bfloat16* Wu = B_(n, "Wu", l);
        float* gWu = G_(n, "Wu", l);
        // dzu = dh * (zu > 0)
        k_relu_back<<<256, 256, 0, n->stream>>>((int64_t)N * H, n->d_dh, n->d_zu[l], n->d_dz);
        n->launches++;
        // dWu slices, dbu
        gemm<true, false, float>(n, H, H, N, h, H, n->d_dz, H, gWu, H, nullptr, nullptr, EPI_STORE);
        gemm<true, false, float>(n, H, H, N, n->d_a[l], H, n->d_dz, H, gWu + (int64_t)H * H, H, nullptr, nullptr,
                                 EPI_STORE);
        gemm<true, false, float>(n, G, H, N, n->d_gf, G, n->d_dz, H, gWu + (int64_t)2 * H * H, H, nullptr, nullptr,
                                 EPI_STORE);
        k_colsum<<<(H + 127) / 128, 128, 0, n->stream>>>(N, H, n->d_dz, G_(n, "bu", l), 0);
        n->launches++;
        // dh (residual path) += dzu Wu[0:H]^T ; da = dzu Wu[H:2H]^T
        gemm<false, true, __nv_bfloat16>(n, N, H, H, n->d_dz, H, Wu, H, n->d_dh, H, nullptr, nullptr, EPI_ADD);
        gemm<false, true, __nv_bfloat16>(n, N, H, H, n->d_dz, H, Wu + (int64_t)H * H, H, n->d_dtmp, H, nullptr,
                                         nullptr, EPI_STORE);
        // dm = W^T da ; dzm = dm * (zm > 0)
        aggregate(n, true, H, n->d_dtmp, n->d_dm);
        k_relu_back<<<256, 256, 0, n->stream>>>((int64_t)N * H, n->d_dm, n->d_zm[l], n->d_dz);
        n->launches++;
        gemm<true, false, float>(n, H, H, N, h, H, n->d_dz, H, G_(n, "Wm", l), H, nullptr, nullptr, EPI_STORE);
        k_colsum<<<(H + 127) / 128, 128, 0, n->stream>>>(N, H, n->d_dz, G_(n, "bm", l), 0);
        n->launches++;
        gemm<false, true, __nv_bfloat16>(n, N, H, H, n->d_dz, H, B_(n, "Wm", l), H, n->d_dh, H, nullptr, nullptr,
                                         EPI_ADD);
    }
    // dz0 = dh * (z0 > 0); dW0 = x^T dz0; db0
    k_relu_back<<<256, 256, 0, n->stream>>>((int64_t)N * H, n->d_dh, n->d_z0, n->d_dz);
    n->launches++;
    gemm<true, false, float>(n, F, H, N, n->d_x, F, n->d_dz, H, G_(n, "W0"), H, nullptr, nullptr, EPI_STORE);
    k_colsum<<<(H + 127) / 128, 128, 0, n->stream>>>(N, H, n->d_dz, G_(n, "b0"), 0);
    n->launches++;
}

int set_graph(lymph_mpnn* n, int n_nodes, const int32_t* wp, const int32_t* wi, const float* wv, const float* gfeat) {
    if (n_nodes <= 0 || !wp || !wi || !wv || !gfeat) return LYMPH_ERR_INVALID;
    LYMPH_TRY(ensure_capacity(n, n_nodes));
    const int nnz = wp[n_nodes];
    for (int i = 0; i < nnz; ++i)
        if (wi[i] < 0 || wi[i] >= n_nodes) { lymph_set_error("lymph_mpnn: graph index out of range"); return LYMPH_ERR_INVALID; }
    // transposed CSR
    std::vector<int32_t> tp(n_nodes + 1, 0), ti(nnz);
    std::vector<float> tv(nnz);
    for (int k = 0; k < nnz; ++k) tp[wi[k] + 1]++;
    for (int i = 0; i < n_nodes; ++i) tp[i + 1] += tp[i];
    std::vector<int32_t> fill(tp.begin(), tp.end() - 1);
    for (int i = 0; i < n_nodes; ++i)
        for (int k = wp[i]; k < wp[i + 1]; ++k) {
            const int j = wi[k];
            ti[fill[j]] = i;
            tv[fill[j]] = wv[k];
            fill[j]++;
        }
    for (auto* p : {&n->d_wp, &n->d_wi, &n->d_tp, &n->d_ti})
        if (*p) { cudaFree(*p); *p = nullptr; }
    for (auto* p : {&n->d_wv, &n->d_tv})
        if (*p) { cudaFree(*p); *p = nullptr; }
    size_t ni = sizeof(int32_t), nf = sizeof(float);
    if (cudaMalloc(&n->d_wp, ni * (n_nodes + 1)) != cudaSuccess || cudaMalloc(&n->d_tp, ni * (n_nodes + 1)) != cudaSuccess ||
        cudaMalloc(&n->d_wi, ni * (nnz + 1)) != cudaSuccess || cudaMalloc(&n->d_ti, ni * (nnz + 1)) != cudaSuccess ||
        cudaMalloc(&n->d_wv, nf * (nnz + 1)) != cudaSuccess || cudaMalloc(&n->d_tv, nf * (nnz + 1)) != cudaSuccess) {
        lymph_set_error("lymph_mpnn: cannot allocate the graph");
        return LYMPH_ERR_OOM;
    }
    LYMPH_CUDA_TRY(cudaMemcpyAsync(n->d_wp, wp, ni * (n_nodes + 1), cudaMemcpyHostToDevice, n->stream));
    LYMPH_CUDA_TRY(cudaMemcpyAsync(n->d_wi, wi, ni * nnz, cudaMemcpyHostToDevice, n->stream));
    LYMPH_CUDA_TRY(cudaMemcpyAsync(n->d_wv, wv, nf * nnz, cudaMemcpyHostToDevice, n->stream));
    LYMPH_CUDA_TRY(cudaMemcpyAsync(n->d_tp, tp.data(), ni * (n_nodes + 1), cudaMemcpyHostToDevice, n->stream));
    LYMPH_CUDA_TRY(cudaMemcpyAsync(n->d_ti, ti.data(), ni * nnz, cudaMemcpyHostToDevice, n->stream));
    LYMPH_CUDA_TRY(cudaMemcpyAsync(n->d_tv, tv.data(), nf * nnz, cudaMemcpyHostToDevice, n->stream));
    LYMPH_CUDA_TRY(cudaMemcpyAsync(n->d_gf, gfeat, nf * (size_t)n_nodes * n->G, cudaMemcpyHostToDevice, n->stream));
    LYMPH_CUDA_TRY(cudaStreamSynchronize(n->stream));  // host vectors die at return
    n->n_nodes = n_nodes;
    return LYMPH_OK;
}

}  // namespace

namespace {

constexpr int SS_BLOCKS = 304;  // 2 x 152 SMs

// d1 = u1 - u0, d2 = u1 - 2 u0 + um elementwise, and per-CTA partial sums of
// squares of u1, d1, d2 into part[3 * blockIdx.x + 0..2] (fixed order).
__global__ void __launch_bounds__(256) k_diffs_sumsq(int64_t n, const double* __restrict__ um,
                                                     const double* __restrict__ u0, const double* __restrict__ u1,
                                                     double* d1, double* d2, double* part) {
    __shared__ double red[3][256];
    double s0 = 0.0, s1 = 0.0, s2 = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double a = u1[i], b = u0[i];
        const double x = a - b, y = (a - 2.0 * b) + um[i];
        d1[i] = x;
        d2[i] = y;
        s0 += a * a;
        s1 += x * x;
        s2 += y * y;
    }
    red[0][threadIdx.x] = s0;
    red[1][threadIdx.x] = s1;
    red[2][threadIdx.x] = s2;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w)
            for (int j = 0; j < 3; ++j) red[j][threadIdx.x] += red[j][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x < 3) part[3 * blockIdx.x + threadIdx.x] = red[threadIdx.x][0];
}

// out[j] = sum over CTAs of part[3 c + j], j = 0..2 (one warp per j, fixed order)
__global__ void k_sum3(int nblk, const double* __restrict__ part, double* out) {
    const int j = threadIdx.x / 32, lane = threadIdx.x % 32;
    if (j >= 3) return;
    double s = 0.0;
    for (int c = lane; c < nblk; c += 32) s += part[3 * c + j];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) out[j] = s;
}

// Node features of the surrogate (one row per polyhedron, F columns), all
// normalised per polyhedron so that they do not depend on the mesh's size:
// [u1/r1, d1/r2, d2/r3, a1/r4, log10(r2/r1), log10(r3/r2), log10(r4/r3),
//  lambda, mu, rho, 0...] with a1 = dt^2 M^-1 (K d1 - gdiff F)
// (the third difference to leading order, up to sign), r_b = the
// polyhedron's RMS of vector b plus 1e-3 x its mesh-wide RMS s_b (a floor
// where the field is quiet).  sig[P][b] = r_b (the per-polyhedron scales of
// the correction).
constexpr int FEAT_WARPS = 8;  // one warp per polyhedron, 8 per CTA

// A positive double v as m 2^e with m in [1, 2) (m as a float, e an int);
// v below the smallest normal double gives m = 0.  Integer and FP32 work only.
__device__ __forceinline__ float split_pow2(double v, int* e) {
    const long long bits = __double_as_longlong(v);
    const int ex = (int)((bits >> 52) & 0x7ff);
    if (ex == 0) { *e = 0; return 0.0f; }
    *e = ex - 1023;
    const float hi = __int_as_float(0x3f800000 | (int)((bits >> 29) & 0x7fffff));  // mantissa rounded down to 23 bits
    return hi;
}
// 2^e as a double (e in the normal range)
__device__ __forceinline__ double pow2d(int e) { return __longlong_as_double((long long)(e + 1023) << 52); }

// sqrt(v) for a double v >= 0 to FP32 accuracy, over the whole double range,
// without FP64 arithmetic: the exponent halved exactly, the mantissa's root in FP32
__device__ __forceinline__ double sqrt_fp32acc(double v) {
    int e;
    float m = split_pow2(v, &e);
    if (m == 0.0f) return 0.0;
    if (e & 1) { m *= 2.0f; e -= 1; }
    return (double)sqrtf(m) * pow2d(e / 2);
}

// The node features, a warp per polyhedron.  The GB300's FP64 pipe retires
// one warp instruction per 64 cycles on each SM quarter however few lanes
// are active, so the per-polyhedron scalar math (square roots, reciprocals,
// logarithms) runs on split exponents and FP32 mantissas, lane-parallel: the
// sums of squares are FP64, the scales carry FP32 rounding over the full
// double range (the states of a quiet start are far below FP32's).
__global__ void __launch_bounds__(32 * FEAT_WARPS) k_features(
    int n_poly, int nd, int F, const double* __restrict__ u1, const double* __restrict__ d1,
    const double* __restrict__ d2, const double* __restrict__ a1, const double* __restrict__ ss, double inv_nd,
    double inv_nall, const int32_t* __restrict__ pptr, const int32_t* __restrict__ ptets,
    const int32_t* __restrict__ tmat, const double* __restrict__ mat, float* x, double* sig) {
    const int P = blockIdx.x * FEAT_WARPS + (int)(threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (P >= n_poly) return;
    const int64_t q = (int64_t)P * nd;
    const double* vec[4] = {u1, d1, d2, a1};
    double mine = 0.0;  // lane b (< 4): vector b's sum of squares
#pragma unroll
    for (int b = 0; b < 4; ++b) {
        double v = 0.0;
        for (int c = lane; c < nd; c += 32) {
            const double w = vec[b][q + c];
            v += w * w;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == b) mine = v;
    }
    const int bl = lane & 3;
    // r_b = RMS of the polyhedron's vector b + 1e-3 x its mesh-wide RMS (+ a floor)
    const double rl = sqrt_fp32acc(mine * inv_nd) + 1e-3 * sqrt_fp32acc(ss[bl] * inv_nall) + 1e-300;
    int er;
    const float mr = split_pow2(rl, &er);
    const double invl = (double)(1.0f / mr) * pow2d(-er);       // 1 / r_b
    const float lgl = ((float)er + log2f(mr)) * 0.30102999566f;  // log10 r_b
    if (lane < 4) sig[(int64_t)P * 4 + lane] = rl;
    float* row = x + (int64_t)P * F;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
        const double inv = __shfl_sync(0xffffffffu, invl, b);
        for (int c = lane; c < nd; c += 32) row[b * nd + c] = (float)(vec[b][q + c] * inv);
    }
    const float lg_next = __shfl_down_sync(0xffffffffu, lgl, 1);
    const int c = 4 * nd + lane;
    if (c < F) {
        float v = 0.0f;
        if (lane < 3) v = lg_next - lgl;  // log10(r_{b+1} / r_b)
        else if (lane < 6) v = (float)mat[tmat[ptets[pptr[P]]] * 3 + (lane - 2) % 3];
        row[c] = v;
    }
    for (int cc = c + 32; cc < F; cc += 32) row[cc] = 0.0f;
}

// y[q] = sum_c Minv_P[m, c] rhs[P, i, c] for q = (P, i, m): M^-1 applied to
// the source's right-hand side (Minv column-major per polyhedron).
__global__ void k_minv_rhs(int n_poly, int Np, const double* __restrict__ Minv, const double* __restrict__ rhs,
                           double* y) {
    const int64_t nv = (int64_t)n_poly * 3 * Np;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < nv; q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t P = q / (3 * Np);
        const int r = (int)(q % (3 * Np)), i = r / Np, m = r % Np;
        const double* Mi = Minv + P * Np * Np + m;
        const double* b = rhs + P * 3 * Np + i * Np;
        double x = 0.0;
        for (int c = 0; c < Np; ++c) x += Mi[(int64_t)c * Np] * b[c];
        y[q] = x;
    }
}

// a1 = dt^2 (a1 - gdiff * MinvF): dt^2 M^-1 (K d1 - gdiff F), minus the
// third difference of the leapfrog to leading order
__global__ void k_accel_combine(int64_t n, double dt2, double gdiff, const double* __restrict__ minvf, double* a1) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        a1[i] = dt2 * (a1[i] - gdiff * minvf[i]);
}

// Per-CTA partial sums of squares of one vector (into part[3 blk])
__global__ void __launch_bounds__(256) k_one_sumsq(int64_t n, const double* __restrict__ a, double* part) {
    __shared__ double red[256];
    double s0 = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        s0 += a[i] * a[i];
    red[threadIdx.x] = s0;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[3 * blockIdx.x] = red[0];
        part[3 * blockIdx.x + 1] = 0.0;
        part[3 * blockIdx.x + 2] = 0.0;
    }
}

// Predicted states u^{n+1+k} = u1 + k d1 + k(k+1)/2 d2 - k(k+1)(k+2)/6 a1
//                             + sc (y3 phi3(k) + y4 phi4(k)),
// a1 = dt^2 M^-1 (K d1 - gdiff F) (the third difference, up to sign, to
// leading order), phi3(k) = k(k+1)(k+2)/K^3, phi4(k) = phi3(k) (k+3)/K (the
// Newton basis of the remaining cubic and quartic error terms),
// sc = (r4^2/r3) K^4/24 per polyhedron (r: its scales from k_features;
// r4/r3 ~ omega dt: coefficients of order one); y = [y3 | y4] per row.
// Written for k = K-3 (out_a), K-2 (out_b), K-1 (out_c).
__global__ void k_predict(int64_t n, int nd, int K, const double* __restrict__ u1, const double* __restrict__ d1,
                          const double* __restrict__ d2, const double* __restrict__ a1,
                          const double* __restrict__ sig, const float* __restrict__ y, int use_net,
                          double* out_a, double* out_b, double* out_c) {
    // the extrapolation in FP64 with its coefficients formed once per thread;
    // the network's correction (FP32 coefficients y, FP32 scale) in FP32
    const double Kd = (double)K;
    double ck[3], ck2[3], ck3[3];
    float cp3[3], cp4[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        const double k = Kd - 3.0 + j;
        const double c3 = k * (k + 1.0) * (k + 2.0);
        ck[j] = k;
        ck2[j] = 0.5 * k * (k + 1.0);
        ck3[j] = c3 / 6.0;
        cp3[j] = (float)(c3 / (Kd * Kd * Kd));
        cp4[j] = (float)(c3 / (Kd * Kd * Kd) * (k + 3.0) / Kd);
    }
    const float k4 = (float)(Kd * Kd * Kd * Kd / 24.0);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t P = i / nd, c = i - P * nd;
        float y3 = 0.0f, y4 = 0.0f;
        if (use_net) {
            const float r3 = (float)sig[P * 4 + 2], r4 = (float)sig[P * 4 + 3];
            const float sc = (r4 * r4 / r3) * k4;
            y3 = sc * y[P * 2 * nd + c];
            y4 = sc * y[P * 2 * nd + nd + c];
        }
        const double vu = u1[i], vd1 = d1[i], vd2 = d2[i], va = a1[i];
        double* outs[3] = {out_a, out_b, out_c};
#pragma unroll
        for (int j = 0; j < 3; ++j)
            outs[j][i] = vu + ck[j] * vd1 + ck2[j] * vd2 - ck3[j] * va + (double)(y3 * cp3[j] + y4 * cp4[j]);
    }
}

// Per-CTA partial sums of |a - b|^2 and |a|^2 (into part[3 blk + 0, 1]).
__global__ void __launch_bounds__(256) k_dist_sumsq(int64_t n, const double* __restrict__ a,
                                                    const double* __restrict__ b, double* part) {
    __shared__ double red[2][256];
    double s0 = 0.0, s1 = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double x = a[i] - b[i], y = a[i];
        s0 += x * x;
        s1 += y * y;
    }
    red[0][threadIdx.x] = s0;
    red[1][threadIdx.x] = s1;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) {
            red[0][threadIdx.x] += red[0][threadIdx.x + w];
            red[1][threadIdx.x] += red[1][threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x < 2) part[3 * blockIdx.x + threadIdx.x] = red[threadIdx.x][0];
    if (threadIdx.x == 2) part[3 * blockIdx.x + 2] = 0.0;
}

}  // namespace

extern "C" {

int lymph_mpnn_create(int32_t F, int32_t H, int32_t O, int32_t L, int32_t G, lymph_mpnn** out) {
    if (!out || F <= 0 || H <= 0 || O <= 0 || L < 0 || L > 8 || G <= 0) return LYMPH_ERR_INVALID;
    lymph_mpnn* n = new lymph_mpnn();
    n->F = F; n->H = H; n->O = O; n->L = L; n->G = G;
    auto add = [&](int64_t r, int64_t c, bool mat) {
        n->par.push_back({n->n_par, r, c, mat});
        n->n_par += r * c;
    };
    add(F, H, true); add(1, H, false);
    for (int l = 0; l < L; ++l) { add(H, H, true); add(1, H, false); add(2 * H + G, H, true); add(1, H, false); }
    add(H, O, true); add(1, O, false);
    int64_t n_wt = 0;
    for (const auto& P : n->par) {
        n->wt_off.push_back(P.matrix ? n_wt : -1);
        if (P.matrix) n_wt += (int64_t)round16((int)P.cols) * P.rows;
    }
    const char* simt = std::getenv("LYMPH_MPNN_SIMT");
    n->use_umma = !(simt && simt[0] == '1');
    const char* ws = std::getenv("LYMPH_UMMA_WS");
    n->use_ws = !(ws && ws[0] == '0');
    if (cudaStreamCreateWithFlags(&n->stream, cudaStreamNonBlocking) != cudaSuccess) { delete n; lymph_set_error("lymph_mpnn_create: stream"); return LYMPH_ERR_CUDA; }
    size_t b = sizeof(float) * (size_t)n->n_par;
    if (cudaMalloc(&n->d_p, b) != cudaSuccess || cudaMalloc(&n->d_g, b) != cudaSuccess || cudaMalloc(&n->d_m, b) != cudaSuccess ||
        cudaMalloc(&n->d_v, b) != cudaSuccess || cudaMalloc(&n->d_pb, sizeof(__nv_bfloat16) * (size_t)n->n_par) != cudaSuccess ||
        cudaMalloc(&n->d_partial, sizeof(double) * 1024) != cudaSuccess ||
        cudaMalloc(&n->d_wt, sizeof(float) * (size_t)n_wt) != cudaSuccess || cudaMalloc(&n->d_status, sizeof(int)) != cudaSuccess) {
        lymph_mpnn_destroy(n);
        lymph_set_error("lymph_mpnn_create: out of memory");
        return LYMPH_ERR_OOM;
    }
    cudaMemsetAsync(n->d_p, 0, b, n->stream);
    cudaMemsetAsync(n->d_g, 0, b, n->stream);
    cudaMemsetAsync(n->d_m, 0, b, n->stream);
    cudaMemsetAsync(n->d_v, 0, b, n->stream);
    cudaMemsetAsync(n->d_status, 0, sizeof(int), n->stream);
    *out = n;
    return LYMPH_OK;
}

int lymph_mpnn_destroy(lymph_mpnn* n) {
    if (!n) return LYMPH_OK;
    if (n->stream) cudaStreamSynchronize(n->stream);
    for (void* p : {(void*)n->d_p, (void*)n->d_g, (void*)n->d_m, (void*)n->d_v, (void*)n->d_pb, (void*)n->d_partial,
                    (void*)n->d_wt, (void*)n->d_status,
                    (void*)n->d_d1, (void*)n->d_d2, (void*)n->d_ss, (void*)n->d_u3, (void*)n->d_a1, (void*)n->d_sig,
                    (void*)n->d_minvf,
                    (void*)n->d_x, (void*)n->d_z0, (void*)n->d_y, (void*)n->d_t, (void*)n->d_dy, (void*)n->d_gf,
                    (void*)n->d_yg, (void*)n->d_dyg,
                    (void*)n->d_dh, (void*)n->d_dz, (void*)n->d_dtmp, (void*)n->d_dm, (void*)n->d_wp, (void*)n->d_wi,
                    (void*)n->d_tp, (void*)n->d_ti, (void*)n->d_wv, (void*)n->d_tv})
        if (p) cudaFree(p);
    for (auto* v : {&n->d_h, &n->d_zm, &n->d_m_, &n->d_a, &n->d_zu})
        for (float* p : *v)
            if (p) cudaFree(p);
    if (n->stream) cudaStreamDestroy(n->stream);
    delete n;
    return LYMPH_OK;
}

int64_t lymph_mpnn_num_params(const lymph_mpnn* n) { return n ? n->n_par : -1; }

// params: FP32 host array of lymph_mpnn_num_params values in the order
// W0 b0 (Wm bm Wu bu) x L Wo bo, each matrix row-major [rows x cols].
int lymph_mpnn_set_params(lymph_mpnn* n, const float* params) {
    if (!n || !params) return LYMPH_ERR_INVALID;
    LYMPH_CUDA_TRY(cudaMemcpyAsync(n->d_p, params, sizeof(float) * (size_t)n->n_par, cudaMemcpyHostToDevice, n->stream));
    k_to_bf16<<<256, 256, 0, n->stream>>>(n->n_par, n->d_p, n->d_pb);
    n->wt_dirty = true;
    LYMPH_CUDA_TRY(cudaMemsetAsync(n->d_m, 0, sizeof(float) * (size_t)n->n_par, n->stream));
    LYMPH_CUDA_TRY(cudaMemsetAsync(n->d_v, 0, sizeof(float) * (size_t)n->n_par, n->stream));
    n->adam_t = 0;
    n->launches++;
    LYMPH_CUDA_TRY(cudaStreamSynchronize(n->stream));
    return LYMPH_OK;
}

int lymph_mpnn_get_params(lymph_mpnn* n, float* params, float* grads) {
    if (!n) return LYMPH_ERR_INVALID;
    if (params) LYMPH_CUDA_TRY(cudaMemcpyAsync(params, n->d_p, sizeof(float) * (size_t)n->n_par, cudaMemcpyDeviceToHost, n->stream));
    if (grads) LYMPH_CUDA_TRY(cudaMemcpyAsync(grads, n->d_g, sizeof(float) * (size_t)n->n_par, cudaMemcpyDeviceToHost, n->stream));
    LYMPH_CUDA_TRY(cudaStreamSynchronize(n->stream));
    return LYMPH_OK;
}

// Graph of one mesh: CSR rows of face-area weights (w_ptr[n+1], w_idx, w_val)
// and the aggregated edge geometry g [n][G].
int lymph_mpnn_set_graph(lymph_mpnn* n, int32_t n_nodes, const int32_t* w_ptr, const int32_t* w_idx,
                         const float* w_val, const float* g) {
    if (!n) return LYMPH_ERR_INVALID;
    return set_graph(n, n_nodes, w_ptr, w_idx, w_val, g);
}

// y = f(x) for the current graph; x host [n][F], y host [n][O].
int lymph_mpnn_forward(lymph_mpnn* n, const float* x, float* y) {
    if (!n || !x || !y || n->n_nodes <= 0) return LYMPH_ERR_INVALID;
    LYMPH_CUDA_TRY(cudaMemcpyAsync(n->d_x, x, sizeof(float) * (size_t)n->n_nodes * n->F, cudaMemcpyHostToDevice, n->stream));
    forward(n, false);
    LYMPH_CUDA_TRY(cudaGetLastError());
    LYMPH_CUDA_TRY(cudaMemcpyAsync(y, eff_out(n), sizeof(float) * (size_t)n->n_nodes * eff_width(n),
                                   cudaMemcpyDeviceToHost, n->stream));
    LYMPH_CUDA_TRY(cudaStreamSynchronize(n->stream));
    return read_status(n, "lymph_mpnn_forward");
}

// Forward, MSE loss against target, backward: gradients stay on the device
// (read them with lymph_mpnn_get_params).  loss may be NULL.
int lymph_mpnn_loss_grad(lymph_mpnn* n, const float* x, const float* target, double* loss) {
    if (!n || !x || !target || n->n_nodes <= 0) return LYMPH_ERR_INVALID;
    const int64_t ny = (int64_t)n->n_nodes * eff_width(n);
    LYMPH_CUDA_TRY(cudaMemcpyAsync(n->d_x, x, sizeof(float) * (size_t)n->n_nodes * n->F, cudaMemcpyHostToDevice, n->stream));
    LYMPH_CUDA_TRY(cudaMemcpyAsync(n->d_t, target, sizeof(float) * (size_t)ny, cudaMemcpyHostToDevice, n->stream));
    forward(n);
    const int nb = 120;
    if (n->gate_B) {
        k_mse<<<nb, 256, 0, n->stream>>>(ny, n->d_yg, n->d_t, n->d_dyg, n->d_partial);
        const int64_t tot = (int64_t)n->n_nodes * n->O;
        k_gate_back<<<(int)std::min<int64_t>((tot + 255) / 256, 4096), 256, 0, n->stream>>>(
            n->n_nodes, n->gate_nd, n->gate_B, n->F, n->d_dyg, n->d_x, n->d_dy);
        n->launches += 2;
    } else {
        k_mse<<<nb, 256, 0, n->stream>>>(ny, n->d_y, n->d_t, n->d_dy, n->d_partial);
        n->launches++;
    }
    backward(n);
    LYMPH_CUDA_TRY(cudaGetLastError());
    double part[nb];
    LYMPH_CUDA_TRY(cudaMemcpyAsync(part, n->d_partial, sizeof(double) * nb, cudaMemcpyDeviceToHost, n->stream));
    LYMPH_CUDA_TRY(cudaStreamSynchronize(n->stream));
    if (loss) {
        double s = 0.0;
        for (int i = 0; i < nb; ++i) s += part[i];
        *loss = s / (double)ny;
    }
    return read_status(n, "lymph_mpnn_loss_grad");
}

// Switches the output head to the gated form over the first B feature blocks
// of nd DOFs each (nd = 3 Np): O must be 2 * B * 3 and F >= B * nd.  The
// effective output (forward, loss target) then has 2 * nd columns.
int lymph_mpnn_set_gate(lymph_mpnn* n, int32_t nd, int32_t B) {
    if (!n || nd <= 0 || nd % 3 || B <= 0 || n->O != 2 * B * 3 || n->F < B * nd) {
        lymph_set_error("lymph_mpnn_set_gate: need nd % 3 == 0, O == 6 B and F >= B nd");
        return LYMPH_ERR_INVALID;
    }
    n->gate_nd = nd;
    n->gate_B = B;
    const int N = n->n_cap;
    n->n_cap = 0;  // re-size the activations for the new output width
    if (N > 0) LYMPH_TRY(ensure_capacity(n, N));
    return LYMPH_OK;
}

// Device time of the inference forward (as lymph_mpnn_forward and the
// surrogate's predict run it) on the features already on the device (from
// the last lymph_mpnn_forward / _loss_grad): `reps` forwards between two CUDA
// events on the network's stream; *ms = the average.
int lymph_mpnn_time_forward(lymph_mpnn* n, int32_t reps, double* ms) {
    if (!n || reps < 1 || !ms || n->n_nodes <= 0) return LYMPH_ERR_INVALID;
    cudaEvent_t e0, e1;
    LYMPH_CUDA_TRY(cudaEventCreate(&e0));
    LYMPH_CUDA_TRY(cudaEventCreate(&e1));
    forward(n, false);  // weight copies refreshed outside the timed region
    cudaEventRecord(e0, n->stream);
    for (int r = 0; r < reps; ++r) forward(n, false);
    cudaEventRecord(e1, n->stream);
    cudaError_t e = cudaEventSynchronize(e1);
    float t = 0.0f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) {
        lymph_set_error(std::string("lymph_mpnn_time_forward: ") + cudaGetErrorString(e));
        return LYMPH_ERR_CUDA;
    }
    *ms = (double)t / reps;
    return read_status(n, "lymph_mpnn_time_forward");
}

// 1 when the forward GEMMs of this network run on the tensor cores.
int lymph_mpnn_uses_tensor_cores(const lymph_mpnn* n) {
    return n && umma_ok(n, n->H, {n->F, n->H, n->G}) && umma_ok(n, n->O, {n->H}) ? 1 : 0;
}

// One Adam step with the gradients of the last lymph_mpnn_loss_grad.
int lymph_mpnn_adam(lymph_mpnn* n, float lr, float beta1, float beta2, float eps) {
    if (!n) return LYMPH_ERR_INVALID;
    n->adam_t++;
    const float c1 = 1.0f - powf(beta1, (float)n->adam_t), c2 = 1.0f - powf(beta2, (float)n->adam_t);
    k_adam<<<1024, 256, 0, n->stream>>>(n->n_par, n->d_p, n->d_g, n->d_m, n->d_v, n->d_pb, lr, beta1, beta2, eps, c1, c2);
    n->wt_dirty = true;
    n->launches++;
    LYMPH_CUDA_TRY(cudaGetLastError());
    LYMPH_CUDA_TRY(cudaStreamSynchronize(n->stream));
    return LYMPH_OK;
}

int lymph_mpnn_launch_count(const lymph_mpnn* n, int64_t* count) {
    if (!n || !count) return LYMPH_ERR_INVALID;
    *count = n->launches;
    return LYMPH_OK;
}

}  // extern "C"

namespace {

// Shared front of a surrogate block on a context with V0 = u^{n-1},
// U0 = u^n, UN = u^{n+1}: d1, d2, a1 = dt^2 M^-1 (K d1 - gdiff F_dyn) and
// their sums of squares (ss[0..3]: u1, d1, d2, a1) into the network's
// scratch; with_features also the feature rows in d_x.  gdiff is the source
// time function's increment g(t_{n+1}) - g(t_n).
int surrogate_front(lymph_ctx* c, lymph_mpnn* n, bool with_features, double gdiff, const char* who) {
    const int nd = c->nd;
    if (with_features && (n->F < 4 * nd + 6 || eff_width(n) != 2 * nd || (n->gate_B && n->gate_nd != nd))) {
        lymph_set_error(std::string(who) + ": network shape does not match the problem (F >= 4*3Np+6, output 2*3Np)");
        return LYMPH_ERR_INVALID;
    }
    if (with_features && n->n_nodes != c->n_poly) {
        lymph_set_error(std::string(who) + ": set the network's graph for this mesh first");
        return LYMPH_ERR_ORDER;
    }
    if (!c->have_matrices) {
        lymph_set_error(std::string(who) + ": call lymph_make_matrices first");
        return LYMPH_ERR_ORDER;
    }
    const int64_t nv = (int64_t)c->n_poly * nd;
    if (nv > n->nv_cap) {  // scratch grows once per (network, largest mesh) and is kept
        for (double** p : {&n->d_d1, &n->d_d2, &n->d_ss, &n->d_u3, &n->d_a1, &n->d_sig, &n->d_minvf})
            if (*p) { cudaFree(*p); *p = nullptr; }
        n->nv_cap = 0;
        n->minvf_uid = 0;
        if (cudaMalloc(&n->d_sig, sizeof(double) * 4 * (size_t)c->n_poly) != cudaSuccess ||
            cudaMalloc(&n->d_d1, sizeof(double) * nv) != cudaSuccess ||
            cudaMalloc(&n->d_d2, sizeof(double) * nv) != cudaSuccess ||
            cudaMalloc(&n->d_u3, sizeof(double) * nv) != cudaSuccess ||
            cudaMalloc(&n->d_a1, sizeof(double) * nv) != cudaSuccess ||
            cudaMalloc(&n->d_minvf, sizeof(double) * nv) != cudaSuccess ||
            cudaMalloc(&n->d_ss, sizeof(double) * (6 * SS_BLOCKS + 6)) != cudaSuccess) {
            lymph_set_error(std::string(who) + ": out of memory");
            return LYMPH_ERR_OOM;
        }
        n->nv_cap = nv;
    }
    cudaStream_t st = c->stream;
    // the network's own work is ordered before this block; its forward then
    // runs on the context's stream, so the block needs no host round trip
    LYMPH_CUDA_TRY(cudaStreamSynchronize(n->stream));
    double *ss = n->d_ss, *part = n->d_ss + 6;
    k_diffs_sumsq<<<SS_BLOCKS, 256, 0, st>>>(nv, c->d_v0, lymph_slot_ptr(c, LYMPH_SLOT_U0),
                                             lymph_slot_ptr(c, LYMPH_SLOT_UN), n->d_d1, n->d_d2, part);
    k_sum3<<<1, 96, 0, st>>>(SS_BLOCKS, part, ss);
    c->launches += 2;
    // the predictor term, optionally with an FP32 copy of the blocks
    // (lymph_surrogate_apply_fp32): half the bytes streamed and no FP64 pipe,
    // at the price of FP32 rounding in a1 (~1e-5 relative after M^-1)
    const float* k32 = c->surrogate_apply_fp32 ? lymph_dev_blocks_f32(c) : nullptr;
    if (k32) LYMPH_TRY(lymph_dev_apply_fp32(c, k32, n->d_d1, n->d_a1));
    else LYMPH_TRY(lymph_dev_apply(c, n->d_d1, n->d_a1));
    // M^-1 F changes only with the source's right-hand side or the mass
    // matrices: computed once per (context, right-hand side) and kept
    if (n->minvf_uid != c->uid || n->minvf_ver != c->rhs_version) {
        k_minv_rhs<<<1024, 256, 0, st>>>(c->n_poly, c->Np, c->d_Minv, c->d_rhs_dyn, n->d_minvf);
        c->launches++;
        n->minvf_uid = c->uid;
        n->minvf_ver = c->rhs_version;
    }
    k_accel_combine<<<1024, 256, 0, st>>>(nv, c->dt * c->dt, gdiff, n->d_minvf, n->d_a1);
    k_one_sumsq<<<SS_BLOCKS, 256, 0, st>>>(nv, n->d_a1, part);
    k_sum3<<<1, 96, 0, st>>>(SS_BLOCKS, part, ss + 3);  // ss[3] (ss[4], ss[5] get zeros)
    c->launches += 3;
    if (with_features) {
        const unsigned blocks = (unsigned)((c->n_poly + FEAT_WARPS - 1) / FEAT_WARPS);
        k_features<<<blocks, 32 * FEAT_WARPS, 0, st>>>(c->n_poly, nd, n->F, lymph_slot_ptr(c, LYMPH_SLOT_UN),
                                                      n->d_d1, n->d_d2, n->d_a1, ss, 1.0 / nd, 1.0 / (double)nv,
                                                      c->d_poly_ptr,
                                                      c->d_poly_tets, c->d_tet_mat, c->d_mat, n->d_x, n->d_sig);
        c->launches++;
    }
    LYMPH_CUDA_TRY(cudaGetLastError());
    return LYMPH_OK;
}

int read_scales(lymph_ctx* c, lymph_mpnn* n, double* scales, int count) {
    double t[4];
    LYMPH_CUDA_TRY(cudaMemcpyAsync(t, n->d_ss, sizeof(double) * count, cudaMemcpyDeviceToHost, c->stream));
    LYMPH_CUDA_TRY(cudaStreamSynchronize(c->stream));
    const double nv = (double)c->n_poly * c->nd;
    for (int i = 0; i < count; ++i) scales[i] = std::sqrt(t[i] / nv);
    return LYMPH_OK;
}

}  // namespace

extern "C" {

// Selects the blocks of the surrogate's operator apply (the a1 term): on = 1
// uses an FP32 copy of an FP64 context's blocks (made on first use, 4 bytes
// per block entry of device memory; the FP64 blocks when it does not fit),
// on = 0 (the default) the context's own blocks.
int lymph_surrogate_apply_fp32(lymph_ctx* c, int32_t on) {
    if (!c) return LYMPH_ERR_INVALID;
    c->surrogate_apply_fp32 = on != 0;
    return LYMPH_OK;
}

// The features of a block, built on the device exactly as
// lymph_surrogate_predict builds them, copied to x (host, n_poly x F
// floats); scales (nullable, 4 doubles) receives the mesh-wide RMS s1..s4,
// a1 (nullable, n_poly x 3Np doubles) the operator term and sig (nullable,
// n_poly x 4 doubles) the per-polyhedron scales.  Used to make training
// samples from solver runs.
int lymph_surrogate_features(lymph_ctx* c, lymph_mpnn* n, double gdiff, float* x, double* scales, double* a1,
                             double* sig) {
    if (!c || !n || !x) return LYMPH_ERR_INVALID;
    LYMPH_TRY(surrogate_front(c, n, true, gdiff, "lymph_surrogate_features"));
    LYMPH_CUDA_TRY(cudaMemcpyAsync(x, n->d_x, sizeof(float) * (size_t)c->n_poly * n->F, cudaMemcpyDeviceToHost,
                                   c->stream));
    if (a1)
        LYMPH_CUDA_TRY(cudaMemcpyAsync(a1, n->d_a1, sizeof(double) * (size_t)c->n_poly * c->nd,
                                       cudaMemcpyDeviceToHost, c->stream));
    if (sig)
        LYMPH_CUDA_TRY(cudaMemcpyAsync(sig, n->d_sig, sizeof(double) * 4 * (size_t)c->n_poly, cudaMemcpyDeviceToHost,
                                       c->stream));
    if (scales) LYMPH_TRY(read_scales(c, n, scales, 4));
    return lymph_sync_status(c, "lymph_surrogate_features");
}

// One surrogate block on a context whose slots hold V0 = u^{n-1},
// U0 = u^n, UN = u^{n+1}: builds the features on the device, runs the
// network (use_net = 0: the extrapolation alone), saves u^n into V0 and
// u^{n+1} into UEX (for a fallback), and writes the predicted u^{n+K-2},
// u^{n+K-1} into U0, UN and u^{n+K} into the network's scratch.  scales
// (nullable, 4 doubles) receives the RMS of u1, d1, d2, a1.
int lymph_surrogate_predict(lymph_ctx* c, lymph_mpnn* n, int32_t K, int32_t use_net, double gdiff, double* scales) {
    if (!c || !n || K < 4) return LYMPH_ERR_INVALID;
    LYMPH_TRY(surrogate_front(c, n, use_net != 0, gdiff, "lymph_surrogate_predict"));
    const int nd = c->nd;
    const int64_t nv = (int64_t)c->n_poly * nd;
    cudaStream_t st = c->stream;
    double* u0 = lymph_slot_ptr(c, LYMPH_SLOT_U0);
    double* u1 = lymph_slot_ptr(c, LYMPH_SLOT_UN);
    if (use_net) {
        cudaStream_t own = n->stream;
        n->stream = st;
        const int64_t before = n->launches;
        forward(n, false);
        c->launches += n->launches - before;
        n->stream = own;
    }
    // keep u^n, u^{n+1} for a fallback, then overwrite U0/UN with the prediction
    LYMPH_CUDA_TRY(cudaMemcpyAsync(c->d_v0, u0, sizeof(double) * nv, cudaMemcpyDeviceToDevice, st));
    LYMPH_CUDA_TRY(cudaMemcpyAsync(c->d_uex, u1, sizeof(double) * nv, cudaMemcpyDeviceToDevice, st));
    k_predict<<<1024, 256, 0, st>>>(nv, nd, K, c->d_uex, n->d_d1, n->d_d2, n->d_a1, n->d_sig, eff_out(n), use_net,
                                    u0, u1, n->d_u3);
    c->launches++;
    LYMPH_CUDA_TRY(cudaGetLastError());
    if (scales) LYMPH_TRY(read_scales(c, n, scales, 4));
    n->have_u3 = c;
    LYMPH_TRY(lymph_sync_status(c, "lymph_surrogate_predict"));
    return use_net ? read_status(n, "lymph_surrogate_predict") : LYMPH_OK;
}

// After the closing plain step of a block (U0 = the predicted u^{n+K-1},
// UN = the stepped u^{n+K}): residual = |UN - u3| / |UN| with u3 the
// predicted u^{n+K}: how far one step of the true dynamics moves away from
// the prediction, relative to the state.
int lymph_surrogate_residual(lymph_ctx* c, lymph_mpnn* n, double* residual) {
    if (!c || !n || !residual) return LYMPH_ERR_INVALID;
    if (n->have_u3 != c || n->nv_cap < (int64_t)c->n_poly * c->nd) {
        lymph_set_error("lymph_surrogate_residual: call lymph_surrogate_predict on this context first");
        return LYMPH_ERR_ORDER;
    }
    const int64_t nv = (int64_t)c->n_poly * c->nd;
    cudaStream_t st = c->stream;
    k_dist_sumsq<<<SS_BLOCKS, 256, 0, st>>>(nv, lymph_slot_ptr(c, LYMPH_SLOT_UN), n->d_u3, n->d_ss + 6);
    k_sum3<<<1, 96, 0, st>>>(SS_BLOCKS, n->d_ss + 6, n->d_ss + 3);
    c->launches += 2;
    double t[3];
    LYMPH_CUDA_TRY(cudaMemcpyAsync(t, n->d_ss + 3, sizeof(t), cudaMemcpyDeviceToHost, st));
    LYMPH_TRY(lymph_sync_status(c, "lymph_surrogate_residual"));
    *residual = t[1] > 0.0 ? std::sqrt(t[0] / t[1]) : (t[0] > 0.0 ? INFINITY : 0.0);
    return LYMPH_OK;
}

// The judge of a block, on the device.  phase 0: keep the current pair
// (U0, UN) in the network's scratch (after the closing step, before the
// plain redo).  phase 1: rel = |(U0, UN) - kept pair| / |(U0, UN)| (after
// the plain redo).  The scratch is the one lymph_surrogate_predict uses, so
// phase 1 must come before the next prediction.
int lymph_surrogate_judge(lymph_ctx* c, lymph_mpnn* n, int32_t phase, double* rel) {
    if (!c || !n || (phase != 0 && phase != 1) || (phase == 1 && !rel)) return LYMPH_ERR_INVALID;
    const int64_t nv = (int64_t)c->n_poly * c->nd;
    if (n->have_u3 != c || n->nv_cap < nv) {
        lymph_set_error("lymph_surrogate_judge: call lymph_surrogate_predict on this context first");
        return LYMPH_ERR_ORDER;
    }
    cudaStream_t st = c->stream;
    double* a = lymph_slot_ptr(c, LYMPH_SLOT_U0);
    double* b = lymph_slot_ptr(c, LYMPH_SLOT_UN);
    if (phase == 0) {
        LYMPH_CUDA_TRY(cudaMemcpyAsync(n->d_d1, a, sizeof(double) * nv, cudaMemcpyDeviceToDevice, st));
        LYMPH_CUDA_TRY(cudaMemcpyAsync(n->d_d2, b, sizeof(double) * nv, cudaMemcpyDeviceToDevice, st));
        n->judge_saved = c;
        return lymph_sync_status(c, "lymph_surrogate_judge");
    }
    if (n->judge_saved != c) {
        lymph_set_error("lymph_surrogate_judge: phase 0 first");
        return LYMPH_ERR_ORDER;
    }
    n->judge_saved = nullptr;
    k_dist_sumsq<<<SS_BLOCKS, 256, 0, st>>>(nv, a, n->d_d1, n->d_ss + 6);
    k_sum3<<<1, 96, 0, st>>>(SS_BLOCKS, n->d_ss + 6, n->d_ss + 3);
    k_dist_sumsq<<<SS_BLOCKS, 256, 0, st>>>(nv, b, n->d_d2, n->d_ss + 6 + 3 * SS_BLOCKS);
    k_sum3<<<1, 96, 0, st>>>(SS_BLOCKS, n->d_ss + 6 + 3 * SS_BLOCKS, n->d_ss);
    c->launches += 4;
    double t[6];
    LYMPH_CUDA_TRY(cudaMemcpyAsync(t, n->d_ss, sizeof(t), cudaMemcpyDeviceToHost, st));
    LYMPH_TRY(lymph_sync_status(c, "lymph_surrogate_judge"));
    const double num = t[3] + t[0], den = t[4] + t[1];
    *rel = den > 0.0 ? std::sqrt(num / den) : 0.0;
    return LYMPH_OK;
}

}  // extern "C"
