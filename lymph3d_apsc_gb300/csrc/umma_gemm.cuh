// umma_gemm.cuh -- the surrogate network's forward GEMMs on the 5th-generation
// tensor cores (tcgen05), FP32-accurate:
//
//   C[M x N] (epilogue)= sum_s A_s[M x K_s] . B_s[K_s x N] + bias
//
// A (activations, FP32 row-major, K contiguous) is split per element into
// hi = the value with its low 13 mantissa bits cleared (exact in TF32) and
// lo = value - hi (exact in FP32); the weights B are BF16 values held as FP32
// (exact in TF32), transposed to [Npad][Ktot] so both operands are K-major.
// Each k-step issues two kind::tf32 MMAs, A_hi.B and A_lo.B, into one FP32
// accumulator in tensor memory: the product is FP32-accurate (the lo part
// keeps 10 of its 13 bits), not TF32-rounded.
//
// One CTA of 128 threads computes a 128-row x 128-column tile (N <= 256
// takes one or two column tiles); two CTAs share an SM, so one CTA's loads
// overlap the other's MMAs and epilogue.  Operand tiles of 32 K-elements
// (128 bytes per row) stream in with asynchronous 16-byte copies (cp.async)
// one tile ahead through two stages, eight threads per 128-byte row (so the
// global reads are coalesced), straight into the 128-byte-swizzled K-major
// layout the MMA reads: row r at r * 128, its 16-byte chunk c at
// (c ^ (r % 8)) * 16, 8-row atoms of 1 KB (the swizzle also keeps the
// shared-memory writes conflict-free); each thread then splits the A chunks
// it copied, in place, into the hi and lo tiles.  Thread 0 issues the MMAs of a
// tile and commits them to its stage's mbarrier, which the copies into that
// stage two tiles later wait on.  The
// epilogue reads the accumulator with tcgen05.ld (warp w owns TMEM lanes
// 32w..32w+31 = tile rows, 32 columns at a time), transposes each 32 x 32
// block through shared memory and stores 16-byte row segments (bias, ReLU,
// pre-activation, residual), so global stores are coalesced.
// Every wait is bounded (2 s of %globaltimer); on expiry the kernel sets
// *status, waits (bounded) for its MMAs in flight, frees its tensor memory
// and returns.
#pragma once

#include <cstdint>

#include "tc_prims.cuh"

namespace umma {

constexpr int BM = 128;       // rows per CTA (the MMA's M)
constexpr int BK = 32;        // K-elements per stage (4 MMAs of K = 8)
constexpr int THREADS = 128;  // 4 warps: one per 32 TMEM lanes
constexpr int STAGES = 2;
constexpr int BN = 128;       // columns per CTA

enum { EPI_STORE = 0, EPI_RELU = 1, EPI_RES_RELU = 2 };

struct Seg {
    const float* A;  // [M][lda] row-major
    int lda;         // multiple of 4
    int K;           // multiple of 4
};

struct Args {
    Seg seg[3];
    int nseg;
    int M, N, Npad;     // Npad: multiple of 16, N <= Npad <= 256
    const float* Bt;    // [Npad][Ktot], rows n >= N zero
    int Ktot;
    const float* bias;  // [N] or null
    float* C;           // [M][ldc]
    int ldc;            // multiple of 4
    float* Z;           // pre-activation out ([M][ldc]) or null
    const float* R;     // residual in ([M][ldc]) for EPI_RES_RELU
    int epi;
    int* status;        // bit 0: a wait ran out
};

// shared memory: STAGES x (A_hi, A_lo, B) operand stages (the epilogue
// reuses the first), then the barriers
constexpr size_t TILE_A = (size_t)BM * BK * 4;                // 16 KB
constexpr size_t STAGE_MAX = 2 * TILE_A + (size_t)BN * BK * 4; // 48 KB
constexpr size_t BAR_OFF = STAGES * STAGE_MAX;
constexpr int EPI_LD = 36;  // floats per staged row (16-byte aligned rows)
constexpr size_t SMEM_ALLOC = BAR_OFF + 64 + 1024;  // + room to align the base to the 1 KB swizzle atom
static_assert(BAR_OFF + 64 <= SMEM_ALLOC, "shared-memory layout exceeds the allocation");
static_assert((size_t)(THREADS / 32) * 32 * EPI_LD * 4 <= STAGE_MAX, "epilogue staging exceeds a stage");


// 16-byte asynchronous copy global -> shared; zero-fills when !valid (no
// bytes are read then, and src is the segment's base, a valid address).
__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src, bool valid) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(valid ? 16 : 0) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N> __device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// The segment, its K offset and the tile start of flat k-tile kt.
__device__ __forceinline__ void tile_of(const Args& a, int kt, int& s, int& koff, int& k0) {
    koff = 0;
    for (s = 0; s < a.nseg; ++s) {
        const int nt = (a.seg[s].K + BK - 1) / BK;
        if (kt < nt) { k0 = kt * BK; return; }
        kt -= nt;
        koff += a.seg[s].K;
    }
    s = a.nseg - 1;
    k0 = 0;
}

// Issues the asynchronous copies of flat k-tile kt into an operand stage:
// A into its hi tile (split in place later), B into its B tile.  Thread t
// copies chunk t % 8 of rows t / 8 + 16 q.
__device__ __forceinline__ void issue_tile(const Args& a, int kt, int m0, int n0, int nloc, uint32_t stage) {
    const uint32_t raw = stage, bst = stage + 2 * (uint32_t)TILE_A;
    int s, koff, k0;
    tile_of(a, kt, s, koff, k0);
    const Seg& g = a.seg[s];
    const int t = threadIdx.x, c = t % 8, k = k0 + 4 * c;
#pragma unroll
    for (int q = 0; q < BM / 16; ++q) {
        const int r = t / 8 + 16 * q, gm = m0 + r;
        const bool v = gm < a.M && k < g.K;
        cp_async16(raw + sw128(r, c), v ? (const void*)(g.A + (int64_t)gm * g.lda + k) : (const void*)g.A, v);
    }
    for (int r = t / 8; r < nloc; r += THREADS / 8) {
        const bool v = k < g.K;
        cp_async16(bst + sw128(r, c), v ? (const void*)(a.Bt + (int64_t)(n0 + r) * a.Ktot + koff + k) : (const void*)a.Bt,
                   v);
    }
}

// Splits the A chunks this thread copied, in place: hi tile <- hi, lo tile <- lo.
__device__ __forceinline__ void split_tile(char* st) {
    const int t = threadIdx.x, c = t % 8;
    char* ahi = st;
    char* alo = st + TILE_A;
#pragma unroll
    for (int q = 0; q < BM / 16; ++q) {
        const uint32_t o = sw128(t / 8 + 16 * q, c);
        const float4 v = *(const float4*)(ahi + o);
        float4 h, l;
        h.x = __uint_as_float(__float_as_uint(v.x) & 0xFFFFE000u); l.x = v.x - h.x;
        h.y = __uint_as_float(__float_as_uint(v.y) & 0xFFFFE000u); l.y = v.y - h.y;
        h.z = __uint_as_float(__float_as_uint(v.z) & 0xFFFFE000u); l.z = v.z - h.z;
        h.w = __uint_as_float(__float_as_uint(v.w) & 0xFFFFE000u); l.w = v.w - h.w;
        *(float4*)(ahi + o) = h;
        *(float4*)(alo + o) = l;
    }
}

__global__ void __launch_bounds__(THREADS, 2) k_umma_gemm(Args a) {
    extern __shared__ __align__(1024) char smem_raw[];
    // the swizzle pattern is a function of the address: align the stages to 1 KB
    char* smem = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
    const int n0 = blockIdx.y * BN;
    const int npad = (a.Npad - n0) < BN ? (a.Npad - n0) : BN;  // this CTA's columns (a multiple of 16)
    uint64_t* bars = (uint64_t*)(smem + BAR_OFF);
    uint32_t* tmem_slot = (uint32_t*)(bars + STAGES);
    __shared__ int s_ok;
    const int t = threadIdx.x, warp = t / 32, lane = t % 32;
    const int m0 = blockIdx.x * BM;
    uint32_t ncols = 32;
    while ((int)ncols < npad) ncols <<= 1;
    int T = 0;
    for (int s = 0; s < a.nseg; ++s) T += (a.seg[s].K + BK - 1) / BK;

    if (t == 0) {
        for (int s = 0; s < STAGES; ++s) mbar_init(smem_u32(&bars[s]), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(ncols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;
    const uint32_t idesc = idesc_tf32(BM, npad);
    const uint32_t sbase = smem_u32(smem);

    bool ok = true;
    for (int p = 0; p < STAGES - 1 && p < T; ++p) {
        issue_tile(a, p, m0, n0, npad, sbase + (uint32_t)(p * STAGE_MAX));
        cp_async_commit();
    }
    int kt = 0;
    for (; kt < T; ++kt) {
        const int st = kt % STAGES;
        const int ahead = kt + STAGES - 1;  // the tile whose copies this iteration issues
        if (ahead < T) {
            if (kt >= 1) {
                // its stage was read by the MMAs of tile kt-1: thread 0 waits
                // for them, the CTA barrier orders the new copies after them
                // and carries one verdict to all threads
                if (t == 0)
                    s_ok = mbar_wait(smem_u32(&bars[(kt - 1) % STAGES]), (uint32_t)(((kt - 1) / STAGES) & 1)) ? 1 : 0;
                __syncthreads();
                if (!s_ok) {
                    ok = false;
                    break;
                }
            }
            issue_tile(a, ahead, m0, n0, npad, sbase + (uint32_t)((ahead % STAGES) * STAGE_MAX));
            cp_async_commit();
            cp_async_wait<STAGES - 1>();  // this thread's copies of tile kt have landed
        } else if (kt + 1 < T) {
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        char* sp = smem + st * STAGE_MAX;
        split_tile(sp);  // the chunks this thread copied (its own copies have landed)
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (t == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t ahi = smem_u32(sp), alo = ahi + (uint32_t)TILE_A, bsm = ahi + 2 * (uint32_t)TILE_A;
#pragma unroll
            for (int j = 0; j < BK / 8; ++j) {  // k-step j: bytes 32 j .. 32 j + 31 of every row
                const uint64_t db = sdesc_sw128(bsm + 32 * j);
                mma_tf32(tmem, sdesc_sw128(ahi + 32 * j), db, idesc, (kt > 0 || j > 0) ? 1u : 0u);
                mma_tf32(tmem, sdesc_sw128(alo + 32 * j), db, idesc, 1u);
            }
            mma_commit(smem_u32(&bars[st]));
        }
    }
    cp_async_wait<0>();  // no copy may still be landing when the epilogue reuses a stage
    // the last commit covers every MMA issued before it
    const int last = kt - 1;
    if (t == 0) {
        bool done = true;
        if (last >= 0) done = mbar_wait(smem_u32(&bars[last % STAGES]), (uint32_t)((last / STAGES) & 1));
        if (!done || !ok) atomicOr(a.status, 1);
        s_ok = (done && ok) ? 1 : 0;
    }
    __syncthreads();
    ok = s_ok != 0;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

    if (ok && last >= 0) {
        // warp w: tile rows 32w..32w+31; 32 x 32 blocks through shared memory
        float* stg = (float*)smem + warp * 32 * EPI_LD;
        // 16-byte stores need N, ldc multiples of 4 and 16-byte aligned rows and bias
        const bool vec = (a.N % 4 == 0) && (a.ldc % 4 == 0) && ((uintptr_t)a.C % 16 == 0) &&
                         (!a.Z || (uintptr_t)a.Z % 16 == 0) && (!a.R || (uintptr_t)a.R % 16 == 0) &&
                         (!a.bias || (uintptr_t)a.bias % 16 == 0);
        const int nl = (a.N - n0) < npad ? (a.N - n0) : npad;  // valid columns of this tile
        for (int c0 = 0; c0 < nl; c0 += 32) {
            uint32_t r[32];
            tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, r);
#pragma unroll
            for (int q = 0; q < 8; ++q)
                *(float4*)(stg + lane * EPI_LD + 4 * q) = make_float4(
                    __uint_as_float(r[4 * q]), __uint_as_float(r[4 * q + 1]), __uint_as_float(r[4 * q + 2]),
                    __uint_as_float(r[4 * q + 3]));
            __syncwarp();
            if (vec) {
                // lane: row i*4 + lane/8 of the block, columns 4 (lane % 8) .. +3
                const int cq = lane % 8, col = n0 + c0 + 4 * cq;
                const bool cv = col < a.N;
                const float4 b = (cv && a.bias) ? *(const float4*)(a.bias + col) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll 2
                for (int i = 0; i < 8; ++i) {
                    const int rr = 4 * i + lane / 8, row = m0 + warp * 32 + rr;
                    if (!cv || row >= a.M) continue;
                    float4 x = *(const float4*)(stg + rr * EPI_LD + 4 * cq);
                    x.x += b.x; x.y += b.y; x.z += b.z; x.w += b.w;
                    const int64_t o = (int64_t)row * a.ldc + col;
                    if (a.epi == EPI_STORE) {
                        *(float4*)(a.C + o) = x;
                    } else {
                        if (a.Z) *(float4*)(a.Z + o) = x;
                        float4 y = make_float4(fmaxf(x.x, 0.f), fmaxf(x.y, 0.f), fmaxf(x.z, 0.f), fmaxf(x.w, 0.f));
                        if (a.epi == EPI_RES_RELU) {
                            const float4 rv = *(const float4*)(a.R + o);
                            y.x += rv.x; y.y += rv.y; y.z += rv.z; y.w += rv.w;
                        }
                        *(float4*)(a.C + o) = y;
                    }
                }
            } else {
                const int col = n0 + c0 + lane;
                const bool cv = col < a.N;
                const float b = (cv && a.bias) ? a.bias[col] : 0.0f;
                for (int i = 0; i < 32; ++i) {
                    const int row = m0 + warp * 32 + i;
                    if (!cv || row >= a.M) continue;
                    const float x = stg[i * EPI_LD + lane] + b;
                    const int64_t o = (int64_t)row * a.ldc + col;
                    if (a.epi == EPI_STORE) {
                        a.C[o] = x;
                    } else {
                        if (a.Z) a.Z[o] = x;
                        const float rl = x > 0.0f ? x : 0.0f;
                        a.C[o] = (a.epi == EPI_RES_RELU) ? a.R[o] + rl : rl;
                    }
                }
            }
            __syncwarp();
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols));
}

}  // namespace umma
