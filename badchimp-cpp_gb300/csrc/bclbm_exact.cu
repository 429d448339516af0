// FP64 kernels that evaluate every expression in the reference's order.
// This translation unit is compiled with -fmad=false: no multiply-add is
// contracted, so each rounding happens where the reference's x86-64 build
// (which has no FMA) rounds, and results are bit-identical to the reference.
#include "bclbm_launch.h"

namespace bclbm {

namespace {

template <int Q>
cudaError_t single_exact_q(bool trt, bool local, const StepArgs& a, cudaStream_t s) {
    const int g = grid_for(a.L.nf);
    if (trt) {
        if (local) k_single<Q, double, 0, true, true><<<g, kBlock, 0, s>>>(a);
        else k_single<Q, double, 0, true, false><<<g, kBlock, 0, s>>>(a);
    } else {
        if (local) k_single<Q, double, 0, false, true><<<g, kBlock, 0, s>>>(a);
        else k_single<Q, double, 0, false, false><<<g, kBlock, 0, s>>>(a);
    }
    launch_counter()++;
    return cudaGetLastError();
}

template <int Q>
cudaError_t rk_f64_q(bool local, bool flux, const StepArgs& a, cudaStream_t s, bool density) {
    const int g = grid_for(a.L.nf);
    if (density) {
        if (local) {
            if (flux) k_rk_density<Q, double, true, true><<<g, kBlock, 0, s>>>(a);
            else k_rk_density<Q, double, true, false><<<g, kBlock, 0, s>>>(a);
        } else {
            if (flux) k_rk_density<Q, double, false, true><<<g, kBlock, 0, s>>>(a);
            else k_rk_density<Q, double, false, false><<<g, kBlock, 0, s>>>(a);
        }
    } else {
        if (local) k_rk_collide_f64<Q, true, false><<<g, kBlock, 0, s>>>(a);
        else k_rk_collide_f64<Q, false, false><<<g, kBlock, 0, s>>>(a);
    }
    launch_counter()++;
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_single_exact(int Q, bool trt, bool local, const StepArgs& a, cudaStream_t s) {
    return Q == 9 ? single_exact_q<9>(trt, local, a, s) : single_exact_q<19>(trt, local, a, s);
}

cudaError_t launch_rk_f64(int Q, bool local, bool flux, const StepArgs& a, cudaStream_t s, bool density) {
    return Q == 9 ? rk_f64_q<9>(local, flux, a, s, density) : rk_f64_q<19>(local, flux, a, s, density);
}

}  // namespace bclbm
