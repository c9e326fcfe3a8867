// umma_ws.cuh -- the warp-specialised, TMA-fed version of the network's
// forward GEMM (same arithmetic as k_umma_gemm in umma_gemm.cuh: kind::tf32
// MMAs of the activations' hi and lo parts against BF16-exact weights, FP32
// accumulation in tensor memory, bias / ReLU / residual epilogue).
//
// One CTA computes a 128-row x min(N, 256)-column tile with 2 + WS_SPLIT_WARPS
// warps:
//   warp 0      producer: one thread issues the TMA loads
//               (cp.async.bulk.tensor.2d, 128-byte swizzle) of the A and B
//               tiles of each 32-wide k-step into a 3-stage ring, arming the
//               stage's "full" mbarrier with the bytes expected;
//   warps 2..   split (WS_SPLIT_WARPS = 16 warps: the pass sets the pace of
//               the ring, 4 warps took 0.73 ms per forward, 16 take 0.57):
//               wait for "full", write the lo part of the raw A tile (the
//               value minus the value with its low 13 mantissa bits cleared)
//               into the lo tile — an elementwise pass, blind to the swizzle;
//               the raw tile itself serves as hi, since kind::tf32 ignores
//               those 13 bits — fence the generic writes for the tensor core
//               and arrive on "split";
//               afterwards the epilogue in groups of 4 warps on interleaved
//               32-column blocks (warp w reads TMEM lanes 32 (w % 4) .. +31,
//               transposed through shared memory into coalesced 16-byte row
//               stores);
//   warp 1      MMA: allocates the tensor memory, one thread waits for
//               "split" and issues the 8 MMAs of the k-step, committing them
//               to the stage's "empty" mbarrier (which frees the stage for
//               the producer) and, after the last k-step, to "acc".
// TMA writes the 128-byte-swizzled K-major layout the MMA descriptors name
// (row r at r * 128 bytes, 16-byte chunk c at (c ^ (r % 8)) * 16, 1 KB
// atoms), and fills rows and columns outside the tensors with zeros.  Every
// wait is bounded (2 s of %globaltimer) and gives up at once when another
// warp has given up: the kernel then sets *status, waits (bounded) for the
// work it has in flight, frees its tensor memory and returns.
#pragma once

#include <cuda.h>

#include "umma_gemm.cuh"

namespace umma {

constexpr int WS_STAGES = 3;
constexpr int WS_SPLIT_WARPS = 16;                  // split / epilogue warps (2 ..), a multiple of 4
constexpr int WS_SPLIT = 32 * WS_SPLIT_WARPS;
constexpr int WS_THREADS = 64 + WS_SPLIT;
constexpr int WS_BN = 256;
constexpr size_t WS_TILE_A = (size_t)BM * BK * 4;                      // 16 KB
constexpr size_t WS_STAGE = 2 * WS_TILE_A + (size_t)WS_BN * BK * 4;     // 64 KB
constexpr size_t WS_BAR_OFF = WS_STAGES * WS_STAGE;
constexpr size_t WS_SMEM = WS_BAR_OFF + 256 + 1024;  // + barriers, + room to align to 1 KB
static_assert((size_t)WS_SPLIT_WARPS * 32 * EPI_LD * 4 <= WS_BAR_OFF, "epilogue staging exceeds the stages");
static_assert(WS_SPLIT_WARPS % 4 == 0, "whole groups of 4 warps (one per TMEM lane quarter)");

struct alignas(64) WsArgs {
    CUtensorMap mapA[3];  // per K segment: [M][K_s] FP32, box 32 x 128, 128-byte swizzle
    CUtensorMap mapB;     // [Npad][Ktot] FP32, box 32 x min(Npad, 256), 128-byte swizzle
    int segK[3];
    int nseg;
    int M, N, Npad, Ktot;
    const float* bias;
    float* C;
    int ldc;
    float* Z;
    const float* R;
    int epi;
    int* status;
};

// Bounded wait that also gives up when *abort is set by another warp.
__device__ __forceinline__ bool mbar_wait_ab(uint32_t bar, uint32_t parity, volatile int* abort) {
    const unsigned long long t0 = now_ns();
    while (!mbar_try_wait(bar, parity)) {
        if (*abort) return false;
        if (now_ns() - t0 > WAIT_NS) {
            *abort = 1;
            return false;
        }
    }
    return true;
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(dst), "l"((uint64_t)map), "r"(x), "r"(y), "r"(bar)
        : "memory");
}

__global__ void __launch_bounds__(WS_THREADS, 1) k_umma_gemm_ws(const __grid_constant__ WsArgs a) {
    extern __shared__ __align__(1024) char smem_raw[];
    char* smem = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
    uint64_t* full = (uint64_t*)(smem + WS_BAR_OFF);
    uint64_t* split = full + WS_STAGES;
    uint64_t* empty = split + WS_STAGES;
    uint64_t* acc = empty + WS_STAGES;
    uint32_t* tmem_slot = (uint32_t*)(acc + 1);
    __shared__ int s_abort;
    __shared__ int s_issued[WS_STAGES];  // per stage the last k-step whose TMA loads were issued (-1: none)
    const int t = threadIdx.x, warp = t / 32, lane = t % 32;
    const int m0 = blockIdx.x * BM, n0 = blockIdx.y * WS_BN;
    const int nb = (a.Npad - n0) < WS_BN ? (a.Npad - n0) : WS_BN;  // this CTA's columns (multiple of 16)
    uint32_t ncols = 32;
    while ((int)ncols < nb) ncols <<= 1;
    int T = 0;
    for (int s = 0; s < a.nseg; ++s) T += (a.segK[s] + BK - 1) / BK;
    const uint32_t sbase = smem_u32(smem);

    if (t == 0) {
        s_abort = 0;
        for (int s = 0; s < WS_STAGES; ++s) s_issued[s] = -1;
        for (int s = 0; s < WS_STAGES; ++s) {
            mbar_init(smem_u32(&full[s]), 1);
            mbar_init(smem_u32(&split[s]), WS_SPLIT);
            mbar_init(smem_u32(&empty[s]), 1);
        }
        mbar_init(smem_u32(acc), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(ncols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;
    volatile int* abort = &s_abort;

    if (warp == 0) {
        // ---- producer ----
        if (lane == 0) {
            const uint32_t bytes = (uint32_t)(BM * BK * 4 + nb * BK * 4);
            int kt = 0, koff = 0;
            for (int sg = 0; sg < a.nseg && !*abort; ++sg) {
                for (int k0 = 0; k0 < a.segK[sg]; k0 += BK, ++kt) {
                    const int st = kt % WS_STAGES;
                    if (!mbar_wait_ab(smem_u32(&empty[st]), (uint32_t)(((kt / WS_STAGES) & 1) ^ 1), abort)) break;
                    const uint32_t sp = sbase + (uint32_t)(st * WS_STAGE);
                    mbar_expect_tx(smem_u32(&full[st]), bytes);
                    tma_load_2d(sp, &a.mapA[sg], k0, m0, smem_u32(&full[st]));
                    tma_load_2d(sp + 2 * (uint32_t)WS_TILE_A, &a.mapB, koff + k0, n0, smem_u32(&full[st]));
                    ((volatile int*)s_issued)[st] = kt;
                }
                koff += a.segK[sg];
            }
        }
    } else if (warp == 1) {
        // ---- MMA issuer ----
        if (lane == 0) {
            const uint32_t idesc = idesc_tf32(BM, nb);
            int kt = 0;
            for (; kt < T; ++kt) {
                const int st = kt % WS_STAGES;
                if (!mbar_wait_ab(smem_u32(&split[st]), (uint32_t)((kt / WS_STAGES) & 1), abort)) break;
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t ahi = sbase + (uint32_t)(st * WS_STAGE), alo = ahi + (uint32_t)WS_TILE_A,
                               bsm = ahi + 2 * (uint32_t)WS_TILE_A;
#pragma unroll
                for (int j = 0; j < BK / 8; ++j) {
                    const uint64_t db = sdesc_sw128(bsm + 32 * j);
                    mma_tf32(tmem, sdesc_sw128(ahi + 32 * j), db, idesc, (kt > 0 || j > 0) ? 1u : 0u);
                    mma_tf32(tmem, sdesc_sw128(alo + 32 * j), db, idesc, 1u);
                }
                mma_commit(smem_u32(&empty[st]));
            }
            mma_commit(smem_u32(acc));  // completes when every MMA issued above has
        }
    } else {
        // ---- split, then epilogue (warps 2..: WS_SPLIT threads) ----
        const int u = t - 64;
        for (int kt = 0; kt < T; ++kt) {
            const int st = kt % WS_STAGES;
            if (!mbar_wait_ab(smem_u32(&full[st]), (uint32_t)((kt / WS_STAGES) & 1), abort)) break;
            const float4* hi = (const float4*)(smem + st * WS_STAGE);
            float4* lo = (float4*)(smem + st * WS_STAGE + WS_TILE_A);
            // kind::tf32 reads an FP32 operand's upper 19 bits and ignores the
            // low 13 mantissa bits (checked on the device: the raw tile and
            // the tile with those bits cleared give the same bits), so the
            // raw tile is the hi part as it stands; only lo is written
#pragma unroll 4
            for (int i = u; i < BM * BK / 4; i += WS_SPLIT) {
                const float4 v = hi[i];
                float4 l;
                l.x = v.x - __uint_as_float(__float_as_uint(v.x) & 0xFFFFE000u);
                l.y = v.y - __uint_as_float(__float_as_uint(v.y) & 0xFFFFE000u);
                l.z = v.z - __uint_as_float(__float_as_uint(v.z) & 0xFFFFE000u);
                l.w = v.w - __uint_as_float(__float_as_uint(v.w) & 0xFFFFE000u);
                lo[i] = l;
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            mbar_arrive(smem_u32(&split[st]));
        }
        const bool done = T > 0 && mbar_wait_ab(smem_u32(acc), 0u, abort);
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        if (done) {
            const int q4 = warp % 4;  // the TMEM lane quarter this warp may read
            float* stg = (float*)smem + (warp - 2) * 32 * EPI_LD;
            const int grp = (warp - 2) / 4;  // groups of 4 warps take interleaved 32-column blocks
            const bool vec = (a.N % 4 == 0) && (a.ldc % 4 == 0) && ((uintptr_t)a.C % 16 == 0) &&
                             (!a.Z || (uintptr_t)a.Z % 16 == 0) && (!a.R || (uintptr_t)a.R % 16 == 0) &&
                             (!a.bias || (uintptr_t)a.bias % 16 == 0);
            const int nl = (a.N - n0) < nb ? (a.N - n0) : nb;
            for (int c0 = 32 * grp; c0 < nl; c0 += 32 * (WS_SPLIT_WARPS / 4)) {
                uint32_t r[32];
                tmem_ld32(tmem + ((uint32_t)(q4 * 32) << 16) + (uint32_t)c0, r);
#pragma unroll
                for (int q = 0; q < 8; ++q)
                    *(float4*)(stg + lane * EPI_LD + 4 * q) = make_float4(
                        __uint_as_float(r[4 * q]), __uint_as_float(r[4 * q + 1]), __uint_as_float(r[4 * q + 2]),
                        __uint_as_float(r[4 * q + 3]));
                __syncwarp();
                if (vec) {
                    const int cq = lane % 8, col = n0 + c0 + 4 * cq;
                    const bool cv = col < a.N;
                    const float4 b = (cv && a.bias) ? *(const float4*)(a.bias + col) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll 2
                    for (int i = 0; i < 8; ++i) {
                        const int rr = 4 * i + lane / 8, row = m0 + q4 * 32 + rr;
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
                        const int row = m0 + q4 * 32 + i;
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
    }
    // teardown: after an abort, let the work in flight finish (bounded) before
    // the tensor memory and the shared memory go away: the MMAs (the "acc"
    // commit, issued after the MMA loop however it ended) and the last TMA
    // loads of every stage (no later load was issued on a stage, so the
    // phase of its last one is the one still pending, if any)
    __syncthreads();
    if (t == 0 && *abort) {
        atomicOr(a.status, 1);
        mbar_wait(smem_u32(acc), 0u);
        for (int s = 0; s < WS_STAGES; ++s) {
            const int kt = ((volatile int*)s_issued)[s];
            if (kt >= 0) mbar_wait(smem_u32(&full[s]), (uint32_t)((kt / WS_STAGES) & 1));
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 1) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols));
}

}  // namespace umma
