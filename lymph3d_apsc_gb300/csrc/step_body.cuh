// step_body.cuh -- the per-polyhedron body of the time step, shared by the
// single-problem kernel (step.cu) and the multi-problem persistent kernel
// (batch.cu).
#pragma once

#include "common.cuh"

namespace stepk {

template <int P> struct Deg {
    static constexpr int NP = (P + 1) * (P + 2) * (P + 3) / 6;
    static constexpr int ND = 3 * NP;
};

// Thread shape per degree: S column slices x ND rows (ND*S fills whole warps
// but for a few lanes), and the CTAs per SM the launch bounds ask for.
template <int P> struct Shape {
    static constexpr int ND = Deg<P>::ND;
    static constexpr int S = P == 1 ? 8 : (P == 2 ? 8 : (P == 3 ? 4 : 3));
    static constexpr int T = ((ND * S + 31) / 32) * 32;       // 96, 256, 256, 320
    static constexpr int MINB = P == 1 ? 16 : (P == 4 ? 4 : 6);
};

constexpr int NBB = 16;   // neighbour blocks staged in shared memory at once

// MODE_APPLY: out = M^-1 K u (power iteration for the CFL bound)
// MODE_BILIN: partial[P] = un_P . (K u0)_P (the bilinear form of the leapfrog energy)
// MODE_KU:    out = K u (the operator apply alone, before M^-1)
enum { MODE_STEP = 0, MODE_FIRST = 1, MODE_DG = 2, MODE_APPLY = 3, MODE_BILIN = 4, MODE_KU = 5 };

struct StepArgs {
    const int32_t* row_ptr;
    const int32_t* col;
    const void* K;             // [n_blocks][ND][ND] column-major (double or float)
    const double* Minv;        // [n_poly][NP][NP] column-major inverse of M_loc
    const double* rhs_stat;
    const double* rhs_dyn;
    const double* gvals;       // time-function values
    const int64_t* step_idx;   // index into gvals (device counter)
    const double* u0;          // u^{n-1} (MODE_STEP), u^0 (MODE_FIRST), u_h (MODE_DG)
    const double* un;          // u^n (MODE_STEP, MODE_APPLY), v^0 (MODE_FIRST), u_ex (MODE_DG)
    double* out;               // u^{n+1} (MODE_STEP: may alias u0), u^1 (MODE_FIRST), M^-1 K u (MODE_APPLY),
                               // K u (MODE_KU)
    double* partial;           // MODE_DG: per-polyhedron du . (A du)
    const int32_t* abs_idx;    // per polyhedron its index among those with absorbing faces, -1 for the
                               // others; null when the mesh has no absorbing face
    const double* Dabs;        // [n_abs][ND][ND] damping blocks (symmetric)
    const double* Winv;        // [n_abs][ND][ND] column-major inverse of M (x) I + dt/2 D
    double dt;
    int* status;
    int n_poly;
};

__device__ __forceinline__ double ld_stream(const double* p) { return __ldcs(p); }
__device__ __forceinline__ float ld_stream(const float* p) { return __ldcs(p); }

// Shared-memory layout of one polyhedron's step: the gathered coefficients
// and the row partial sums in the accumulation type, then the FP64 right-hand
// side at an offset rounded up to 16 bytes (with FP32 blocks and odd ND the
// raw offset is not 8-byte aligned).
template <int PD, typename KT, int S_ = Shape<PD>::S> struct SmemSize {
    static constexpr int ND = Deg<PD>::ND, S = S_;
    static constexpr size_t b_offset = ((sizeof(KT) * (size_t)(NBB * ND + S * ND)) + 15) & ~(size_t)15;
    static constexpr size_t bytes = b_offset + sizeof(double) * ND;
};

// The end of one polyhedron's step once thread tid < ND holds y = (K u)_tid
// of row tid in FP64: the right-hand side, the mass-matrix inverse and the
// leapfrog update (or the bilinear/DG partial sum).  The mass-matrix inverse is
// applied in FP64 as a dense Np x Np product per component (precomputed from
// the Cholesky factor), which replaces the reference's two triangular solves
// per component with a parallel product of the same value.  s_b holds ND
// doubles, 16-byte aligned.  Every thread of the CTA must call this (it
// synchronises).
template <int PD, int MODE>
__device__ __forceinline__ void finish_poly(const StepArgs& A, int P, double y, double* s_b) {
    constexpr int NP = Deg<PD>::NP, ND = Deg<PD>::ND;
    const int tid = threadIdx.x;
    if (MODE == MODE_DG || MODE == MODE_BILIN) {
        if (tid < ND) s_b[tid] = y;
        __syncthreads();
        if (tid == 0) {
            double e = 0.0;
            for (int rr = 0; rr < ND; ++rr) {
                const int64_t q = (int64_t)P * ND + rr;
                e = e + (MODE == MODE_DG ? (A.u0[q] - A.un[q]) : A.un[q]) * s_b[rr];
            }
            A.partial[P] = e;
        }
        return;
    }
    if (MODE == MODE_KU) {
        if (tid < ND) {
            if (!isfinite(y)) atomicOr(A.status, ST_NONFINITE);
            A.out[(int64_t)P * ND + tid] = y;
        }
        return;
    }
    if (tid < ND) {
        const int64_t q = (int64_t)P * ND + tid;
        if (MODE == MODE_APPLY) {
            s_b[tid] = y;
        } else {
            const double g = A.gvals[*A.step_idx];
            s_b[tid] = -y + A.rhs_stat[q] + A.rhs_dyn[q] * g;
        }
    }
    __syncthreads();
    // polyhedra with absorbing faces (the index is the same for the whole CTA)
    const int ai = (MODE == MODE_STEP || MODE == MODE_FIRST) && A.abs_idx ? A.abs_idx[P] : -1;
    if (ai >= 0) {
        const double* Db = A.Dabs + (int64_t)ai * ND * ND;
        const int64_t base = (int64_t)P * ND;
        double dv = 0.0;
        if (tid < ND) {
            // MODE_STEP: D (u^n - u^{n-1}); MODE_FIRST: D v^0 (v^0 is in un)
#pragma unroll 1
            for (int c = 0; c < ND; ++c) {
                const double w = (MODE == MODE_STEP) ? A.un[base + c] - A.u0[base + c] : A.un[base + c];
                dv += Db[(int64_t)c * ND + tid] * w;
            }
        }
        double bn = 0.0;
        if (tid < ND) bn = (MODE == MODE_STEP) ? A.dt * A.dt * s_b[tid] - A.dt * dv : s_b[tid] - dv;
        __syncthreads();
        if (tid < ND) s_b[tid] = bn;
        __syncthreads();
        if (MODE == MODE_STEP) {
            // u^{n+1} = 2 u^n - u^{n-1} + W^-1 (dt^2 (F - K u^n) - dt D (u^n - u^{n-1}))
            if (tid < ND) {
                const double* Wi = A.Winv + (int64_t)ai * ND * ND + tid;
                double x0 = 0.0, x1 = 0.0;
#pragma unroll 1
                for (int c = 0; c < ND; c += 2) {
                    x0 += Wi[(int64_t)c * ND] * s_b[c];
                    if (c + 1 < ND) x1 += Wi[(int64_t)(c + 1) * ND] * s_b[c + 1];
                }
                const int64_t q = base + tid;
                const double v = (x0 + x1) + 2.0 * A.un[q] - A.u0[q];
                if (!isfinite(v)) atomicOr(A.status, ST_NONFINITE);
                A.out[q] = v;
            }
            return;
        }
        // MODE_FIRST continues with M^-1 (F - K u^0 - D v^0) below
    }
    if (tid < ND) {
        const int i = tid / NP, m = tid % NP;
        const double* Mi = A.Minv + (int64_t)P * NP * NP + m;
        const double* bi = s_b + i * NP;
        double x0 = 0.0, x1 = 0.0;
#pragma unroll
        for (int c = 0; c < NP; c += 2) {
            x0 += Mi[c * NP] * bi[c];
            if (c + 1 < NP) x1 += Mi[(c + 1) * NP] * bi[c + 1];
        }
        const double x = x0 + x1;
        const int64_t q = (int64_t)P * ND + tid;
        double v;
        if (MODE == MODE_STEP) {
            const double dt2 = A.dt * A.dt;
            v = dt2 * x + 2.0 * A.un[q] - A.u0[q];
        } else if (MODE == MODE_FIRST) {
            const double half_dt2 = 0.5 * (A.dt * A.dt);
            v = half_dt2 * x + A.u0[q] + A.dt * A.un[q];
        } else {
            v = x;
        }
        if (!isfinite(v)) atomicOr(A.status, ST_NONFINITE);
        A.out[q] = v;
    }
}

// The block row of polyhedron P is one contiguous column-major
// [ND x nb*ND] matrix (its blocks are adjacent in memory), multiplied by the
// gathered coefficients of the column polyhedra, then finish_poly.  S_ is
// the number of column slices (the tile shape; the CTA needs ND * S_ threads).
// Every thread of the CTA must call this (it synchronises); threads beyond the
// degree's shape only help with the gather.
template <int PD, typename KT, int MODE, int S_ = Shape<PD>::S>
__device__ __forceinline__ void step_poly(const StepArgs& A, int P, char* smem) {
    constexpr int NP = Deg<PD>::NP, ND = Deg<PD>::ND, S = S_;
    constexpr int CPT = (ND + S - 1) / S;
    using AT = KT;  // FP64 blocks accumulate in FP64, FP32 blocks in FP32
    AT* s_u = (AT*)smem;
    AT* s_red = s_u + NBB * ND;
    double* s_b = (double*)(smem + SmemSize<PD, KT, S>::b_offset);
    static_assert(SmemSize<PD, KT, S>::b_offset % 16 == 0, "FP64 rhs must be 16-byte aligned");
    const int nthr = blockDim.x;
    const int tid = threadIdx.x;
    const int r = tid % ND, s = tid / ND;
    const bool act = tid < ND * S;
    const int rb = A.row_ptr[P], re = A.row_ptr[P + 1];
    const KT* Kbase = (const KT*)A.K;

    AT acc0 = 0, acc1 = 0;
    for (int b0 = rb; b0 < re; b0 += NBB) {
        const int nb = (re - b0) < NBB ? (re - b0) : NBB;
        __syncthreads();
        for (int i = tid; i < nb * ND; i += nthr) {
            const int bb = i / ND, c = i % ND;
            const int64_t q = (int64_t)A.col[b0 + bb] * ND + c;
            double v;
            if (MODE == MODE_STEP || MODE == MODE_APPLY || MODE == MODE_KU) v = A.un[q];
            else if (MODE == MODE_FIRST || MODE == MODE_BILIN) v = A.u0[q];
            else v = A.u0[q] - A.un[q];
            s_u[i] = (AT)v;
        }
        __syncthreads();
        if (act) {
            for (int bb = 0; bb < nb; ++bb) {
                const KT* Kb = Kbase + (int64_t)(b0 + bb) * ND * ND + r;
                const AT* ub = s_u + bb * ND;
                KT kv[CPT];
#pragma unroll
                for (int j = 0; j < CPT; ++j) {
                    const int c = s + j * S;
                    kv[j] = (c < ND) ? ld_stream(Kb + (int64_t)c * ND) : (KT)0;
                }
#pragma unroll
                for (int j = 0; j < CPT; ++j) {
                    const int c = s + j * S;
                    if (c < ND) {
                        if (j & 1) acc1 += (AT)kv[j] * ub[c];
                        else acc0 += (AT)kv[j] * ub[c];
                    }
                }
            }
        }
    }
    if (act) s_red[s * ND + r] = acc0 + acc1;
    __syncthreads();
    double y = 0.0;
    if (tid < ND)
        for (int ss = 0; ss < S; ++ss) y += (double)s_red[ss * ND + tid];
    finish_poly<PD, MODE>(A, P, y, s_b);
}

}  // namespace stepk
