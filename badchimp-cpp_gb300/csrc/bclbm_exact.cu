// FP64 kernels that evaluate every expression in the reference's order.
// This translation unit is compiled with -fmad=false: no multiply-add is
// contracted, so each rounding happens where the reference's x86-64 build
// (which has no FMA) rounds, and results are bit-identical to the reference.
#include "bclbm_launch.h"
#include "bclbm_links.h"

namespace bclbm {

__global__ void k_links_flux(LinksArgs A) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const size_t pad = static_cast<size_t>(A.s.L.nf_pad);
    double s[2] = {0.0, 0.0};
    for (int k = 0; k < A.nflux; ++k) {
        const int i = A.flux_slot[k];
        s[A.flux_phase[k]] += A.s.vel_out[2 * pad + i] * A.s.rho_out[i];  // massFluxLocal[phase] += vel_z * rho
    }
    A.flux_out[0] = 0.5 * s[0];
    A.flux_out[1] = 0.5 * s[1];
}

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

cudaError_t launch_links_mass_exact(bool local, const LinksArgs& A, cudaStream_t s) {
    if (local) k_links_mass<true, true><<<grid_for(A.nlabeled), kBlock, 0, s>>>(A);
    else k_links_mass<true, false><<<grid_for(A.nlabeled), kBlock, 0, s>>>(A);
    launch_counter()++;
    return cudaGetLastError();
}

cudaError_t launch_links_label_sum_exact(const LinksArgs& A, cudaStream_t s) {
    k_links_label_sum<true><<<(A.nlab + kBlock - 1) / kBlock, kBlock, 0, s>>>(A);
    launch_counter()++;
    return cudaGetLastError();
}

cudaError_t launch_links_collide_exact(bool local, const LinksArgs& A, cudaStream_t s) {
    const int n = A.s.L.nf;
    if (local) k_links_collide<true, true><<<grid_for(n), kBlock, 0, s>>>(A);
    else k_links_collide<true, false><<<grid_for(n), kBlock, 0, s>>>(A);
    launch_counter()++;
    return cudaGetLastError();
}

cudaError_t launch_links_gather_exact(bool local, const LinksArgs& A, const int32_t* slot_bulk, double* out,
                                      cudaStream_t s) {
    const int g = grid_for(A.s.L.nf);
    if (local) k_links_gather<true, true><<<g, kBlock, 0, s>>>(A, slot_bulk, out);
    else k_links_gather<true, false><<<g, kBlock, 0, s>>>(A, slot_bulk, out);
    launch_counter()++;
    return cudaGetLastError();
}

cudaError_t launch_links_moments_exact(bool local, const LinksArgs& A, cudaStream_t s) {
    const int g = grid_for(A.s.L.nf);
    if (local) k_links_moments<true, true><<<g, kBlock, 0, s>>>(A);
    else k_links_moments<true, false><<<g, kBlock, 0, s>>>(A);
    launch_counter()++;
    return cudaGetLastError();
}

cudaError_t launch_links_flux(const LinksArgs& A, cudaStream_t s) {
    k_links_flux<<<1, 32, 0, s>>>(A);
    launch_counter()++;
    return cudaGetLastError();
}

cudaError_t launch_single_exact(int Q, bool trt, bool local, const StepArgs& a, cudaStream_t s) {
    return Q == 9 ? single_exact_q<9>(trt, local, a, s) : single_exact_q<19>(trt, local, a, s);
}

cudaError_t launch_rk_f64(int Q, bool local, bool flux, const StepArgs& a, cudaStream_t s, bool density) {
    return Q == 9 ? rk_f64_q<9>(local, flux, a, s, density) : rk_f64_q<19>(local, flux, a, s, density);
}

}  // namespace bclbm
