// Restructured FP64 kernels (FMA), FP32-arithmetic kernels for the shifted
// storage formats, the download gather and the deterministic FP64 reductions.
#include <algorithm>
#include <mutex>
#include <type_traits>
#include <unordered_map>

#include "bclbm_launch.h"

namespace bclbm {

std::atomic<int64_t>& launch_counter() {
    static std::atomic<int64_t> n{0};
    return n;
}

// the fixed-point copy of the flux controller's force; |F| >= 8 is out of range
__device__ void set_forcex(DevParams* params) {
    int ovf = 0;
    params->forcex[0] = fx::from_f64(params->force[0], ovf);
    if (ovf) params->fx_overflow |= 1;
}

__global__ void k_flux_force(const double* sum, double inv_n, double mom_x, DevParams* params) {
    // meanfcXGlobal /= numNodesGlobal; bodyForce.x = 2 * (setMomX - meanfcXGlobal)
    // (src/twophase/main_TWOPHASE.cpp:301-308)
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        params->force[0] = 2 * (mom_x - sum[0] * inv_n);
        params->forcef[0] = static_cast<float>(params->force[0]);
        set_forcex(params);
    }
}

__global__ void k_rk_fix(const double* sum, double n, double rho_ref, double mom_x, int flux, int fix,
                         DevParams* params) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        if (flux) {
            params->force[0] = 2 * (mom_x - sum[0] / n);
            params->forcef[0] = static_cast<float>(params->force[0]);
            set_forcex(params);
        }
        if (fix) {
            // totals now: n rho_ref + sum[1] and sum[2]; the deficit spread over the nodes.
            // fix == 2 (one pass per step): the sums are of the state this step's collision
            // still corrects by the correction in place, so the next one takes the rest
            double dt = (params->mass_target[0] - (n * rho_ref + sum[1])) / n;
            double dc = (params->mass_target[1] - sum[2]) / n;
            if (fix == 2) {
                dt -= params->mass_fix[0];
                dc -= params->mass_fix[1];
            }
            params->mass_fix[0] = dt;
            params->mass_fix[1] = dc;
            params->mass_fixf[0] = static_cast<float>(dt);
            params->mass_fixf[1] = static_cast<float>(dc);
        }
    }
}

namespace {

// Persistent grid of a staged kernel (bclbm_stage.cuh): the blocks that fit on
// the device at once (resident blocks per SM x SMs), at most one per tile.
// BCLBM_STAGED_CARVEOUT picks the shared-memory carveout: 0 the driver's
// choice, 1 the maximum, 2 just what the resident blocks need (the rest stays
// L1 cache for the gathers and spills).  Looked up once per kernel.
#ifndef BCLBM_STAGED_CARVEOUT
#define BCLBM_STAGED_CARVEOUT 2
#endif
int staged_grid(const void* kernel, int nf) {
    static std::mutex mu;
    static std::unordered_map<const void*, int> per_device;
    int resident = 0;
    {
        std::lock_guard<std::mutex> lock(mu);
        auto it = per_device.find(kernel);
        if (it == per_device.end()) {
            int dev = 0, sms = 0, per_sm = 0, smem_sm = 0;
            cudaGetDevice(&dev);
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
            if (BCLBM_STAGED_CARVEOUT >= 1)
                cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                                     cudaSharedmemCarveoutMaxShared);
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kBlock, 0);
            if (BCLBM_STAGED_CARVEOUT == 2 && per_sm > 0 && smem_sm > 0) {
                cudaFuncAttributes fa;
                if (cudaFuncGetAttributes(&fa, kernel) == cudaSuccess) {
                    const size_t need = static_cast<size_t>(per_sm) * (fa.sharedSizeBytes + 1024);
                    const int pct = static_cast<int>(std::min<size_t>(100, (need * 100 + smem_sm - 1) / smem_sm));
                    cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, pct);
                }
            }
            it = per_device.emplace(kernel, std::max(1, sms * per_sm)).first;
        }
        resident = it->second;
    }
    return std::max(1, std::min(grid_for(nf), resident));
}

template <int Q, class S>
cudaError_t single_fast_qs(bool trt, bool local, const StepArgs& a, const CUtensorMap* pull_map, cudaStream_t s) {
    const int g = grid_for(a.L.nf);
    // the staged kernel serves the native-FP64 step only (see k_single_staged); the
    // shifted formats take two slots per thread after the first step (k_single_pair)
    constexpr bool kStaged = std::is_same<S, double>::value;
    if constexpr (!kStaged) {
        if (!local) {
            const int gp = ((a.L.nf + 1) / 2 + BCLBM_PAIR_BLOCK - 1) / BCLBM_PAIR_BLOCK;
            if (trt) k_single_pair<Q, S, true><<<gp, BCLBM_PAIR_BLOCK, 0, s>>>(a);
            else k_single_pair<Q, S, false><<<gp, BCLBM_PAIR_BLOCK, 0, s>>>(a);
            launch_counter()++;
            return cudaGetLastError();
        }
    }
    if (local || !pull_map || !kStaged) {
        if (trt) {
            if (local) k_single<Q, S, 1, true, true><<<g, kBlock, 0, s>>>(a);
            else k_single<Q, S, 1, true, false><<<g, kBlock, 0, s>>>(a);
        } else {
            if (local) k_single<Q, S, 1, false, true><<<g, kBlock, 0, s>>>(a);
            else k_single<Q, S, 1, false, false><<<g, kBlock, 0, s>>>(a);
        }
    } else if constexpr (kStaged) {
        if (trt) {
            const void* k = reinterpret_cast<const void*>(&k_single_staged<Q, S, true>);
            k_single_staged<Q, S, true><<<staged_grid(k, a.L.nf), kBlock, 0, s>>>(a, *pull_map);
        } else {
            const void* k = reinterpret_cast<const void*>(&k_single_staged<Q, S, false>);
            k_single_staged<Q, S, false><<<staged_grid(k, a.L.nf), kBlock, 0, s>>>(a, *pull_map);
        }
    }
    launch_counter()++;
    return cudaGetLastError();
}

template <int Q>
cudaError_t single_fixed_q(bool trt, bool local, const StepArgs& a, cudaStream_t s) {
    const int g = (a.L.nf + BCLBM_FX_BLOCK - 1) / BCLBM_FX_BLOCK;
    if (trt) {
        if (local) k_single_fixed<Q, true, true><<<g, BCLBM_FX_BLOCK, 0, s>>>(a);
        else k_single_fixed<Q, true, false><<<g, BCLBM_FX_BLOCK, 0, s>>>(a);
    } else {
        if (local) k_single_fixed<Q, false, true><<<g, BCLBM_FX_BLOCK, 0, s>>>(a);
        else k_single_fixed<Q, false, false><<<g, BCLBM_FX_BLOCK, 0, s>>>(a);
    }
    launch_counter()++;
    return cudaGetLastError();
}

template <int Q>
cudaError_t single_fast_q(int precision, bool trt, bool local, const StepArgs& a, const CUtensorMap* pull_map,
                          cudaStream_t s) {
    switch (precision) {
        case kF64: return single_fast_qs<Q, double>(trt, local, a, pull_map, s);
        case kF32: return single_fast_qs<Q, float>(trt, local, a, pull_map, s);
        case kF16: return single_fast_qs<Q, __half>(trt, local, a, pull_map, s);
        case kBF16: return single_fast_qs<Q, __nv_bfloat16>(trt, local, a, pull_map, s);
    }
    return cudaErrorInvalidValue;
}

template <int Q, class S>
cudaError_t rk_shift_qs(bool local, bool flux, const StepArgs& a, cudaStream_t s, bool density) {
    const int g = grid_for(a.L.nf);
    if (density) {
        if (local) {
            if (flux) k_rk_density<Q, S, true, true><<<g, kBlock, 0, s>>>(a);
            else k_rk_density<Q, S, true, false><<<g, kBlock, 0, s>>>(a);
        } else {
            if (flux) k_rk_density<Q, S, false, true><<<g, kBlock, 0, s>>>(a);
            else k_rk_density<Q, S, false, false><<<g, kBlock, 0, s>>>(a);
        }
    } else {
        const int gc = (a.L.nf + BCLBM_RK_COLL_BLOCK - 1) / BCLBM_RK_COLL_BLOCK;
        if (local) k_rk_collide_shift<Q, S, true><<<gc, BCLBM_RK_COLL_BLOCK, 0, s>>>(a);
        else k_rk_collide_shift<Q, S, false><<<gc, BCLBM_RK_COLL_BLOCK, 0, s>>>(a);
    }
    launch_counter()++;
    return cudaGetLastError();
}

template <int Q>
cudaError_t rk_fx_q(bool local, bool flux, const StepArgs& a, cudaStream_t s, bool density) {
    const int g = grid_for(a.L.nf);
    if (density) {
        if (local) {
            if (flux) k_rk_density<Q, int64_t, true, true><<<g, kBlock, 0, s>>>(a);
            else k_rk_density<Q, int64_t, true, false><<<g, kBlock, 0, s>>>(a);
        } else {
            if (flux) k_rk_density<Q, int64_t, false, true><<<g, kBlock, 0, s>>>(a);
            else k_rk_density<Q, int64_t, false, false><<<g, kBlock, 0, s>>>(a);
        }
    } else {
        const int gc = (a.L.nf + BCLBM_RK_FX_BLOCK - 1) / BCLBM_RK_FX_BLOCK;
        if (local) k_rk_collide_fx<Q, true><<<gc, BCLBM_RK_FX_BLOCK, 0, s>>>(a);
        else k_rk_collide_fx<Q, false><<<gc, BCLBM_RK_FX_BLOCK, 0, s>>>(a);
    }
    launch_counter()++;
    return cudaGetLastError();
}

template <int Q>
cudaError_t rk_shift_q(int precision, bool local, bool flux, const StepArgs& a, cudaStream_t s, bool density) {
    switch (precision) {
        case kF32: return rk_shift_qs<Q, float>(local, flux, a, s, density);
        case kF16: return rk_shift_qs<Q, __half>(local, flux, a, s, density);
        case kBF16: return rk_shift_qs<Q, __nv_bfloat16>(local, flux, a, s, density);
    }
    return cudaErrorInvalidValue;
}

template <int Q, class S>
cudaError_t gather_qs(int nfields, bool local, const StepArgs& a, const int32_t* sb, double* out, cudaStream_t s) {
    const int g = grid_for(a.L.nf);
    if (nfields == 1) {
        if (local) k_gather<Q, S, 1, true><<<g, kBlock, 0, s>>>(a, sb, out);
        else k_gather<Q, S, 1, false><<<g, kBlock, 0, s>>>(a, sb, out);
    } else {
        if (local) k_gather<Q, S, 2, true><<<g, kBlock, 0, s>>>(a, sb, out);
        else k_gather<Q, S, 2, false><<<g, kBlock, 0, s>>>(a, sb, out);
    }
    launch_counter()++;
    return cudaGetLastError();
}

template <int Q, class S>
cudaError_t moments_qs(int nfields, bool local, const StepArgs& a, cudaStream_t s) {
    const int g = grid_for(a.L.nf);
    if (nfields == 1) {
        if (local) k_moments<Q, S, 1, true><<<g, kBlock, 0, s>>>(a);
        else k_moments<Q, S, 1, false><<<g, kBlock, 0, s>>>(a);
    } else {
        if (local) k_moments<Q, S, 2, true><<<g, kBlock, 0, s>>>(a);
        else k_moments<Q, S, 2, false><<<g, kBlock, 0, s>>>(a);
    }
    launch_counter()++;
    return cudaGetLastError();
}

#define BCLBM_BY_PRECISION(FN, Q, ...)                                   \
    switch (precision) {                                                 \
        case kF64: return FN<Q, double>(__VA_ARGS__);                    \
        case kF32: return FN<Q, float>(__VA_ARGS__);                     \
        case kF16: return FN<Q, __half>(__VA_ARGS__);                    \
        case kBF16: return FN<Q, __nv_bfloat16>(__VA_ARGS__);            \
        case kFX: return FN<Q, int64_t>(__VA_ARGS__);                    \
    }                                                                    \
    return cudaErrorInvalidValue;

template <int Q>
cudaError_t gather_q(int precision, int nfields, bool local, const StepArgs& a, const int32_t* sb, double* out,
                     cudaStream_t s) {
    BCLBM_BY_PRECISION(gather_qs, Q, nfields, local, a, sb, out, s)
}

template <int Q>
cudaError_t moments_q(int precision, int nfields, bool local, const StepArgs& a, cudaStream_t s) {
    BCLBM_BY_PRECISION(moments_qs, Q, nfields, local, a, s)
}

}  // namespace

cudaError_t launch_single_fast(int Q, int precision, bool trt, bool local, const StepArgs& a,
                               const CUtensorMap* pull_map, cudaStream_t s) {
    return Q == 9 ? single_fast_q<9>(precision, trt, local, a, pull_map, s)
                  : single_fast_q<19>(precision, trt, local, a, pull_map, s);
}

cudaError_t launch_rk_fx(int Q, bool local, bool sums, const StepArgs& a, cudaStream_t s, bool density) {
    return Q == 9 ? rk_fx_q<9>(local, sums, a, s, density) : rk_fx_q<19>(local, sums, a, s, density);
}

cudaError_t launch_single_fixed(int Q, bool trt, bool local, const StepArgs& a, cudaStream_t s) {
    return Q == 9 ? single_fixed_q<9>(trt, local, a, s) : single_fixed_q<19>(trt, local, a, s);
}

cudaError_t launch_rk_shift(int Q, int precision, bool local, bool flux, const StepArgs& a, cudaStream_t s,
                            bool density) {
    return Q == 9 ? rk_shift_q<9>(precision, local, flux, a, s, density)
                  : rk_shift_q<19>(precision, local, flux, a, s, density);
}

template <int Q, class S>
cudaError_t rk_fused_qs(bool sums, const StepArgs& a, cudaStream_t s) {
    const int g = grid_for(a.L.nf);
    if (sums) k_rk_fused_shift<Q, S, true><<<g, kBlock, 0, s>>>(a);
    else k_rk_fused_shift<Q, S, false><<<g, kBlock, 0, s>>>(a);
    launch_counter()++;
    return cudaGetLastError();
}

template <int Q>
cudaError_t rk_fused_q(int precision, bool sums, const StepArgs& a, cudaStream_t s) {
    switch (precision) {
        case kF32: return rk_fused_qs<Q, float>(sums, a, s);
        case kF16: return rk_fused_qs<Q, __half>(sums, a, s);
        case kBF16: return rk_fused_qs<Q, __nv_bfloat16>(sums, a, s);
    }
    return cudaErrorInvalidValue;
}

cudaError_t launch_rk_fused(int Q, int precision, bool sums, const StepArgs& a, cudaStream_t s) {
    return Q == 9 ? rk_fused_q<9>(precision, sums, a, s) : rk_fused_q<19>(precision, sums, a, s);
}

cudaError_t launch_flux_force(const double* sum, double inv_n, double mom_x, DevParams* params, cudaStream_t s) {
    k_flux_force<<<1, 32, 0, s>>>(sum, inv_n, mom_x, params);
    launch_counter()++;
    return cudaGetLastError();
}

cudaError_t launch_rk_collide_f64_fma(int Q, bool local, const StepArgs& a, cudaStream_t s) {
    const int g = grid_for(a.L.nf);
    if (Q == 9) {
        if (local) k_rk_collide_f64<9, true, true><<<g, kBlock, 0, s>>>(a);
        else k_rk_collide_f64<9, false, true><<<g, kBlock, 0, s>>>(a);
    } else {
        if (local) k_rk_collide_f64<19, true, true><<<g, kBlock, 0, s>>>(a);
        else k_rk_collide_f64<19, false, true><<<g, kBlock, 0, s>>>(a);
    }
    launch_counter()++;
    return cudaGetLastError();
}

cudaError_t launch_rk_fix(const double* sum, double n, double rho_ref, double mom_x, bool flux, int fix,
                          DevParams* params, cudaStream_t s) {
    k_rk_fix<<<1, 32, 0, s>>>(sum, n, rho_ref, mom_x, flux ? 1 : 0, fix, params);
    launch_counter()++;
    return cudaGetLastError();
}

cudaError_t launch_gather(int Q, int precision, int nfields, bool local, const StepArgs& a, const int32_t* slot_bulk,
                          double* out, cudaStream_t s) {
    return Q == 9 ? gather_q<9>(precision, nfields, local, a, slot_bulk, out, s)
                  : gather_q<19>(precision, nfields, local, a, slot_bulk, out, s);
}

cudaError_t launch_moments(int Q, int precision, int nfields, bool local, const StepArgs& a, cudaStream_t s) {
    return Q == 9 ? moments_q<9>(precision, nfields, local, a, s) : moments_q<19>(precision, nfields, local, a, s);
}

cudaError_t launch_reduce_final(int nv, const double* partials, int nblocks, double* out, bool max_last,
                                cudaStream_t s) {
    if (nv == 1) k_reduce_final<1><<<1, kFinalThreads, 0, s>>>(partials, nblocks, out, max_last ? 1 : 0);
    else if (nv == 3) k_reduce_final<3><<<1, kFinalThreads, 0, s>>>(partials, nblocks, out, max_last ? 1 : 0);
    else if (nv == 6) k_reduce_final<6><<<1, kFinalThreads, 0, s>>>(partials, nblocks, out, max_last ? 1 : 0);
    else return cudaErrorInvalidValue;
    launch_counter()++;
    return cudaGetLastError();
}


// cuTensorMapEncodeTiled through the runtime's driver entry point (the library
// links the runtime only).
cudaError_t encode_table_map(const int32_t* table, int pad, int rows, CUtensorMap* out) {
    using EncodeFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
    static EncodeFn encode = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            encode = reinterpret_cast<EncodeFn>(fn);
    });
    if (!encode) return cudaErrorNotSupported;
    if (!table || pad % 64 != 0 || rows < 1 || rows > 256) return cudaErrorInvalidValue;
    const cuuint64_t dims[2] = {static_cast<cuuint64_t>(pad), static_cast<cuuint64_t>(rows)};
    const cuuint64_t strides[1] = {static_cast<cuuint64_t>(pad) * sizeof(int32_t)};
    const cuuint32_t box[2] = {static_cast<cuuint32_t>(stage::kSub), static_cast<cuuint32_t>(rows)};
    const cuuint32_t elem[2] = {1, 1};
    const CUresult r = encode(out, CU_TENSOR_MAP_DATA_TYPE_INT32, 2, const_cast<int32_t*>(table), dims, strides, box,
                              elem, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

}  // namespace bclbm
