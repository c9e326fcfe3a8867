// umma_ps.cuh -- the persistent version of the network's forward GEMM
// (same arithmetic as k_umma_gemm_ws: kind::tf32 MMAs of the activations' hi
// and lo parts against BF16-exact weights, FP32 accumulation in tensor
// memory, bias / ReLU / residual epilogue).
//
// One CTA per SM walks the 128-row x min(Npad, 256)-column tiles
// blockIdx.x, blockIdx.x + gridDim.x, ... with 10 warps:
//   warp 0      producer: TMA loads (cp.async.bulk.tensor.2d, 128-byte
//               swizzle) of every k-step of every tile into a 3-stage ring;
//   warps 2..5  split: the raw A tile of each stage into hi and lo parts;
//   warp 1      MMA: two accumulators in tensor memory, used by alternate
//               tiles; before a tile it waits until the epilogue has drained
//               the accumulator it reuses ("acc_empty"), after the tile's
//               last k-step it commits to "acc_full";
//   warps 6..9  epilogue: wait for "acc_full", read the accumulator (warp w
//               owns TMEM lanes 32 (w % 4) .. +31), store through their own
//               shared-memory slots, release the accumulator.
// So the epilogue of tile i runs while the MMAs of tile i + 1 stream, and the
// stage ring never drains between tiles.  Every wait is bounded (2 s of
// %globaltimer) and gives up at once when another warp has given up; the
// kernel then sets *status, lets the MMAs and copies in flight finish
// (bounded) and frees its tensor memory.
#pragma once

#include "umma_ws.cuh"

namespace umma {

constexpr int PS_STAGES = 3;
constexpr int PS_THREADS = 320;
constexpr size_t PS_STAGE = WS_STAGE;                            // A hi, A lo, B: 64 KB
constexpr size_t PS_EPI_OFF = PS_STAGES * PS_STAGE;
constexpr size_t PS_EPI = (size_t)4 * 32 * EPI_LD * 4;           // epilogue slots of warps 6..9
constexpr size_t PS_BAR_OFF = PS_EPI_OFF + PS_EPI;
constexpr size_t PS_SMEM = PS_BAR_OFF + 256 + 1024;             // + barriers, + room to align to 1 KB
static_assert(PS_SMEM <= 227 * 1024, "shared memory per CTA");

__global__ void __launch_bounds__(PS_THREADS, 1) k_umma_gemm_ps(const __grid_constant__ WsArgs a) {
    extern __shared__ __align__(1024) char smem_raw[];
    char* smem = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
    uint64_t* full = (uint64_t*)(smem + PS_BAR_OFF);
    uint64_t* split = full + PS_STAGES;
    uint64_t* empty = split + PS_STAGES;
    uint64_t* acc_full = empty + PS_STAGES;   // [2]
    uint64_t* acc_empty = acc_full + 2;       // [2]
    uint64_t* drain = acc_empty + 2;
    uint32_t* tmem_slot = (uint32_t*)(drain + 1);
    __shared__ int s_abort;
    __shared__ int s_issued;  // k-steps the producer has issued (for the teardown after an abort)
    const int t = threadIdx.x, warp = t / 32, lane = t % 32;
    const int n_mt = (a.M + BM - 1) / BM, n_nt = (a.Npad + WS_BN - 1) / WS_BN;
    const int n_tiles = n_mt * n_nt;
    const int my_tiles = (int)blockIdx.x < n_tiles ? (n_tiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    const int wmax = a.Npad < WS_BN ? a.Npad : WS_BN;  // widest tile (columns, multiple of 16)
    uint32_t acc_cols = 32;
    while ((int)acc_cols < wmax) acc_cols <<= 1;   // <= 256: two accumulators fit the 512 columns
    int T = 0;
    for (int s = 0; s < a.nseg; ++s) T += (a.segK[s] + BK - 1) / BK;
    const uint32_t sbase = smem_u32(smem);

    if (t == 0) {
        s_abort = 0;
        s_issued = 0;
        for (int s = 0; s < PS_STAGES; ++s) {
            mbar_init(smem_u32(&full[s]), 1);
            mbar_init(smem_u32(&split[s]), 128);
            mbar_init(smem_u32(&empty[s]), 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(smem_u32(&acc_full[b]), 1);
            mbar_init(smem_u32(&acc_empty[b]), 128);
        }
        mbar_init(smem_u32(drain), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(2 * acc_cols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;
    volatile int* abort = &s_abort;

    auto tile_origin = [&](int li, int& m0, int& n0, int& nb) {
        const int tile = (int)blockIdx.x + li * (int)gridDim.x;
        m0 = (tile % n_mt) * BM;
        n0 = (tile / n_mt) * WS_BN;
        nb = (a.Npad - n0) < WS_BN ? (a.Npad - n0) : WS_BN;
    };

    if (warp == 0) {
        // ---- producer ----
        if (lane == 0) {
            int g = 0;  // k-steps issued so far (all tiles)
            for (int li = 0; li < my_tiles && !*abort; ++li) {
                int m0, n0, nb;
                tile_origin(li, m0, n0, nb);
                // the B box is wmax rows wide whatever the tile's width (rows
                // past Npad arrive zero-filled and count as transferred)
                const uint32_t bytes = (uint32_t)(BM * BK * 4 + wmax * BK * 4);
                int koff = 0;
                bool ok = true;
                for (int sg = 0; sg < a.nseg && ok; ++sg) {
                    for (int k0 = 0; k0 < a.segK[sg]; k0 += BK, ++g) {
                        const int st = g % PS_STAGES;
                        if (!mbar_wait_ab(smem_u32(&empty[st]), (uint32_t)(((g / PS_STAGES) & 1) ^ 1), abort)) {
                            ok = false;
                            break;
                        }
                        const uint32_t sp = sbase + (uint32_t)(st * PS_STAGE);
                        mbar_expect_tx(smem_u32(&full[st]), bytes);
                        tma_load_2d(sp, &a.mapA[sg], k0, m0, smem_u32(&full[st]));
                        tma_load_2d(sp + 2 * (uint32_t)WS_TILE_A, &a.mapB, koff + k0, n0, smem_u32(&full[st]));
                        *(volatile int*)&s_issued = g + 1;
                    }
                    koff += a.segK[sg];
                }
            }
        }
    } else if (warp == 1) {
        // ---- MMA issuer ----
        if (lane == 0) {
            int g = 0;
            for (int li = 0; li < my_tiles && !*abort; ++li) {
                int m0, n0, nb;
                tile_origin(li, m0, n0, nb);
                const int b = li & 1;
                if (!mbar_wait_ab(smem_u32(&acc_empty[b]), (uint32_t)(((li >> 1) & 1) ^ 1), abort)) break;
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t d = tmem + (uint32_t)b * acc_cols;
                const uint32_t idesc = idesc_tf32(BM, nb);
                bool ok = true;
                for (int kt = 0; kt < T; ++kt, ++g) {
                    const int st = g % PS_STAGES;
                    if (!mbar_wait_ab(smem_u32(&split[st]), (uint32_t)((g / PS_STAGES) & 1), abort)) {
                        ok = false;
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const uint32_t ahi = sbase + (uint32_t)(st * PS_STAGE), alo = ahi + (uint32_t)WS_TILE_A,
                                   bsm = ahi + 2 * (uint32_t)WS_TILE_A;
#pragma unroll
                    for (int j = 0; j < BK / 8; ++j) {
                        const uint64_t db = sdesc_sw128(bsm + 32 * j);
                        mma_tf32(d, sdesc_sw128(ahi + 32 * j), db, idesc, (kt > 0 || j > 0) ? 1u : 0u);
                        mma_tf32(d, sdesc_sw128(alo + 32 * j), db, idesc, 1u);
                    }
                    mma_commit(smem_u32(&empty[st]));
                }
                if (!ok) break;
                mma_commit(smem_u32(&acc_full[b]));
            }
            // every MMA issued above completes before the tensor memory is freed
            mma_commit(smem_u32(drain));
            mbar_wait(smem_u32(drain), 0u);
        }
    } else if (warp < 6) {
        // ---- split (warps 2..5: 128 threads) ----
        const int u = t - 64;
        const int steps = my_tiles * T;
        for (int g = 0; g < steps; ++g) {
            const int st = g % PS_STAGES;
            if (!mbar_wait_ab(smem_u32(&full[st]), (uint32_t)((g / PS_STAGES) & 1), abort)) break;
            float4* hi = (float4*)(smem + st * PS_STAGE);
            float4* lo = (float4*)(smem + st * PS_STAGE + WS_TILE_A);
#pragma unroll 4
            for (int i = u; i < BM * BK / 4; i += 128) {
                const float4 v = hi[i];
                float4 h, l;
                h.x = __uint_as_float(__float_as_uint(v.x) & 0xFFFFE000u); l.x = v.x - h.x;
                h.y = __uint_as_float(__float_as_uint(v.y) & 0xFFFFE000u); l.y = v.y - h.y;
                h.z = __uint_as_float(__float_as_uint(v.z) & 0xFFFFE000u); l.z = v.z - h.z;
                h.w = __uint_as_float(__float_as_uint(v.w) & 0xFFFFE000u); l.w = v.w - h.w;
                hi[i] = h;
                lo[i] = l;
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            mbar_arrive(smem_u32(&split[st]));
        }
    } else {
        // ---- epilogue (warps 6..9: 128 threads) ----
        const int q4 = warp % 4;  // the TMEM lane quarter this warp may read
        float* stg = (float*)(smem + PS_EPI_OFF) + (warp - 6) * 32 * EPI_LD;
        for (int li = 0; li < my_tiles; ++li) {
            int m0, n0, nb;
            tile_origin(li, m0, n0, nb);
            const int b = li & 1;
            if (T == 0 || !mbar_wait_ab(smem_u32(&acc_full[b]), (uint32_t)((li >> 1) & 1), abort)) break;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            ws_epilogue(a, tmem + (uint32_t)b * acc_cols, q4, lane, stg, m0, n0, nb);
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            mbar_arrive(smem_u32(&acc_empty[b]));
        }
    }
    // teardown: after an abort, let the copies in flight (the last PS_STAGES
    // k-steps issued) land, each wait bounded, before the shared memory goes
    // away
    __syncthreads();
    if (t == 0 && *abort) {
        atomicOr(a.status, 1);
        const int gi = s_issued;
        for (int g = gi > PS_STAGES ? gi - PS_STAGES : 0; g < gi; ++g)
            mbar_wait(smem_u32(&full[g % PS_STAGES]), (uint32_t)((g / PS_STAGES) & 1));
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 1) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * acc_cols));
}

}  // namespace umma
