// Staging of pull-table tiles into shared memory with the tensor copy engine
// (TMA, cp.async.bulk.tensor) and one mbarrier per buffer.
//
// A staged step kernel is persistent and every warp runs its own pipeline, with
// no block-wide barrier: warp w of block b walks the 32-slot sub-tiles
// s = b*NW + w, s + gridDim.x*NW, ...  While it computes sub-tile k it has
// already asked the copy engine for the table rows of sub-tile k+1 (one 2-D
// tensor copy: 32 slots x the Q-1 rows, 128 bytes of each row) into the other
// of two shared-memory buffers.  A thread therefore finds its gather indices in
// shared memory instead of first waiting on an HBM load of them, and the table
// costs the warp one copy instruction per 32 slots instead of Q-1 loads per
// thread.  At any moment the warps of the grid work on a contiguous window of
// sub-tiles, as the blocks of an ordinary launch do.
//
// Every wait on a copy is bounded by kWaitCycles SM clock cycles (about 0.13 s
// at 2 GHz; a sub-tile arrives in microseconds).  A warp whose wait runs out
// computes nothing more, sets kFlagWaitTimeout in the handle's device flag
// word (bclbm_reduce reports it as BCLBM_ERR_CUDA), waits (bounded again) for
// the copies it has in flight, and returns; the other warps are not held up.
#pragma once

#include <cuda.h>  // CUtensorMap

#include <cstdint>

namespace bclbm {
namespace stage {

constexpr long long kWaitCycles = 1ll << 28;
constexpr int kFlagWaitTimeout = 2;  // bit in DevParams::fx_overflow (bit 0: fixed-point range)
constexpr int kSub = 32;             // slots per sub-tile (one per lane)

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// makes the initialised barriers visible to the copy engine
__device__ __forceinline__ void fence_barrier_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// orders the warp's earlier shared-memory reads (made visible to this thread by
// the warp's vote) before the next tensor copy into the same buffer
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// one arrival that also announces the bytes the phase waits for
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// 2-D tensor copy global -> shared of the box at (x, y) of the map
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// waits for the phase of the given parity, at most kWaitCycles; false if it ran out
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
    if (mbar_try_wait(bar, parity)) return true;
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity))
        if (clock64() - t0 > kWaitCycles) return false;
    return true;
}

// Per warp: two buffers of NR table rows x 32 slots (each buffer a multiple of
// 128 bytes, so every buffer starts 128-byte aligned), and their barriers.
template <int NR, int NW>
struct WarpStage {
    alignas(128) int32_t tab[NW][2][NR][kSub];
    alignas(8) uint64_t bar[NW][2];
};

// The sub-tile loop of a staged kernel.  map describes the table [NR][pad] int32
// (box kSub x NR).  body(i, rows, lane) computes slot i; it is called for every
// slot i < nf of every sub-tile this warp owns, with rows[q][lane] the staged
// table entry of row q for that slot.
template <int NR, int NW, class Body>
__device__ __forceinline__ void staged_warps(WarpStage<NR, NW>& st, const CUtensorMap* map, int nf, int* flag,
                                             Body&& body) {
    constexpr uint32_t kBytes = NR * kSub * 4;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int nsub = (nf + kSub - 1) / kSub;
    const int stride = static_cast<int>(gridDim.x) * NW;
    int sub = static_cast<int>(blockIdx.x) * NW + w;
    if (sub >= nsub) return;  // no block-wide barrier follows: a warp may leave on its own
    uint64_t* bar = st.bar[w];
    if (lane == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_barrier_init();
        mbar_arrive_expect_tx(&bar[0], kBytes);
        tma_load_2d(&st.tab[w][0][0][0], map, sub * kSub, 0, &bar[0]);
    }
    __syncwarp();
    int k = 0;
    bool timed_out = false;
    for (; sub < nsub; sub += stride, ++k) {
        const int b = k & 1;
        const int next = sub + stride;
        if (lane == 0 && next < nsub) {
            fence_proxy_async_smem();
            mbar_arrive_expect_tx(&bar[b ^ 1], kBytes);
            tma_load_2d(&st.tab[w][b ^ 1][0][0], map, next * kSub, 0, &bar[b ^ 1]);
        }
        const bool ok = mbar_wait_bounded(&bar[b], static_cast<uint32_t>(k >> 1) & 1u);
        const int i = sub * kSub + lane;
        if (ok && i < nf) body(i, st.tab[w][b], lane);
        if (__any_sync(0xffffffffu, !ok)) {
            timed_out = true;
            break;
        }
    }
    if (timed_out && lane == 0) {
        if (flag) atomicOr(flag, kFlagWaitTimeout);
        // copies still in flight: this sub-tile's and, if it was asked for, the next one's
        const int b = k & 1;
        mbar_wait_bounded(&bar[b], static_cast<uint32_t>(k >> 1) & 1u);
        if (sub + stride < nsub) mbar_wait_bounded(&bar[b ^ 1], static_cast<uint32_t>((k + 1) >> 1) & 1u);
    }
}

}  // namespace stage
}  // namespace bclbm
