// Kernel templates of the std_one_phase time step (src/std_one_phase/main.cpp:
// 470-575, D3Q19, FP64): BGK with the Guo force scaled per node by the force
// attribute, a mass source per interior domain (calcDeltaOmegaQ,
// src/lbsolver/LBcollision.h:80-98) and the link-based boundaries of the node
// tags, applied after streaming in the reference:
//   solid-fluid     f(q_rev, n) = f(q, wall)                           main.cpp:138-151
//   pressure-fluid  f(q_rev, n) = -f(q, ghost) + 2 w rho_w (1 + (9 cu^2 - 3 u^2)/2)
//                   (anti-bounce-back, u = the node's velocity)        main.cpp:154-173
//   fluid-fluid     the two populations that cross the phase link swap
//                   (the velocity correction is multiplied by 0)       main.cpp:176-203
// In pull form the three rules are resolved into the pull table at create: a
// bounce-back entry reads the node's own post-collision value in the reversed
// direction; an anti-bounce-back entry is stored as ~element (negative) and
// combines that value with the node's velocity of the previous step, which the
// collision keeps per pressure-boundary node in u_store.
//
// Every kernel takes EXACT: true only in the -fmad=false translation unit
// (the reference's rounding, bit-identical), false in the contracting one.
#pragma once

#include "bclbm_kernels.cuh"

namespace bclbm {

constexpr uint32_t kLinkLabelMask = 0xFFFFFFu;  // interior-domain label
constexpr uint32_t kLinkAdd = 1u << 24;         // the node takes its domain's mass source
constexpr uint32_t kLinkPress = 1u << 25;       // the node has anti-bounce-back links (u_store entry)

struct LinksArgs {
    StepArgs s;
    const uint32_t* info;       // [nf] label | kLinkAdd | kLinkPress
    const int32_t* pidx;        // [nf] u_store index of a pressure-boundary node, else -1
    const int32_t* force_on;    // [nf] force attribute
    double* ustore;             // [3][npress] velocity of the last step
    int npress;
    double rho_w;               // pressure-boundary density
    const int32_t* lab_slot;    // [nlabeled] slots of the labelled bulk nodes, by label, in bulk order
    const int32_t* lab_start;   // [nlab + 2] label l owns lab_slot[lab_start[l] .. lab_start[l + 1])
    double* lab_val;            // [nlabeled] 1 - rho of this step
    const double* lab_g;        // [nlab + 1] 0.9 * 2 / (number of source nodes of the label)
    double* lab_q;              // [nlab + 1] the label's source of this step
    int nlab, nlabeled;
    const int32_t* flux_slot;   // [nflux] bulk pressure-boundary nodes in node order
    const int32_t* flux_phase;  // [nflux] their fluid phase (0 or 1)
    int nflux;
    double* flux_out;           // [2]
    float f_rho_w;              // shifted storage: rho_w and 2 (rho_w - rho_ref) in FP32
    float f_dw;
};

// the populations that stream into slot i: plain pulls, bounce-back, and the
// anti-bounce-back of the pressure boundary with the node's velocity u
template <bool EXACT, bool LOCAL>
__device__ __forceinline__ void load_links(const double* __restrict__ g, const LatticeView& L, int i, const double* u,
                                           double rho_w, double* f) {
    constexpr int Q = 19, R = Lat<Q>::REST;
    const size_t pad = static_cast<size_t>(L.nf_pad);
    if constexpr (LOCAL) {
#pragma unroll
        for (int q = 0; q < Q; ++q) f[q] = g[static_cast<size_t>(q) * pad + i];
        return;
    }
    double u2 = 0.0;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        if (q == R) {
            f[q] = g[static_cast<size_t>(R) * pad + i];
            continue;
        }
        const int e = __ldg(L.pull + static_cast<size_t>(q) * pad + i);
        if (e >= 0) {
            f[q] = g[e];
        } else {
            // applyPressureFluidBoundary, qUnknown = q, qKnown = rev(q)
            const int k = Lat<Q>::rev(q);
            const double fk = g[~e];
            u2 = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];  // DXQY::dot
            const double cu = Lat<Q>::cx(k) * u[0] + Lat<Q>::cy(k) * u[1] + Lat<Q>::cz(k) * u[2];  // cDotRef
            const double w = Lat<Q>::w(k);
            f[q] = -fk + 2 * w * rho_w * (1 + 0.5 * (9.0 * cu * cu - 3.0 * u2));
        }
    }
}

template <bool LOCAL>
__device__ __forceinline__ void links_velocity(const LinksArgs& A, int i, uint32_t inf, double* u) {
    u[0] = u[1] = u[2] = 0.0;
    if (!LOCAL && (inf & kLinkPress)) {
        const int p = __ldg(A.pidx + i);
#pragma unroll
        for (int d = 0; d < 3; ++d) u[d] = A.ustore[static_cast<size_t>(d) * A.npress + p];
    }
}

// the node loop of src/std_one_phase/main.cpp:496-539 for one node
template <bool EXACT>
__device__ __forceinline__ void collide_links(double* f, const LinksArgs& A, int i, uint32_t inf, double& rho_o,
                                              double* vel_o) {
    constexpr int Q = 19;
    const StepArgs& a = A.s;
    double rho = 0.0;  // calcRho
#pragma unroll
    for (int q = 0; q < Q; ++q) rho += f[q];
    // qMassConservation = 0.9*2*scale[label]*massChange[label]*addMassSource[node]
    const double qm = (inf & kLinkAdd) ? A.lab_q[inf & kLinkLabelMask] : 0.0;
    rho += 0.5 * qm;
    const double fo = static_cast<double>(__ldg(A.force_on + i));
    double F[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) F[d] = a.params->force[d] * fo;  // bodyForce(0, 0) * forceOn(0, node)
    double j[3], vel[3];
    qsumc_ref<Q>(f, j);
#pragma unroll
    for (int d = 0; d < 3; ++d) vel[d] = (j[d] + 0.5 * F[d]) / rho;  // calcVel
    rho_o = rho;
#pragma unroll
    for (int d = 0; d < 3; ++d) vel_o[d] = vel[d];
    const double u2 = dot_ref<Q>(vel, vel);
    double cu[Q], cF[Q];
    cdotall_ref<Q>(vel, cu);
    const double uF = dot_ref<Q>(vel, F);
    cdotall_ref<Q>(F, cF);
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const double w = Lat<Q>::w(q);
        // calcOmegaBGK (LBcollision.h:43), calcDeltaOmegaF (:210), calcDeltaOmegaQ (:95)
        const double om = -a.tau_inv * (f[q] - rho * w * (1.0 + 3.0 * cu[q] + 4.5 * (cu[q] * cu[q] - C2 * u2)));
        const double dF = w * a.tf * (3.0 * cF[q] + 9.0 * (cF[q] * cu[q] - C2 * uF));
        const double dQ = a.tf * qm * w * (1.0 + 3.0 * cu[q] + 4.5 * (cu[q] * cu[q] - C2 * u2));
        f[q] = f[q] + om + dF + dQ;
    }
}

// mass pass (main.cpp:474-481): 1 - rho of every labelled bulk node
template <bool EXACT, bool LOCAL>
__global__ void __launch_bounds__(kBlock) k_links_mass(LinksArgs A) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= A.nlabeled) return;
    const int i = __ldg(A.lab_slot + k);
    const uint32_t inf = __ldg(A.info + i);
    double u[3], f[19];
    links_velocity<LOCAL>(A, i, inf, u);
    load_links<EXACT, LOCAL>(static_cast<const double*>(A.s.src), A.s.L, i, u, A.rho_w, f);
    double rho = 0.0;
#pragma unroll
    for (int q = 0; q < 19; ++q) rho += f[q];
    A.lab_val[k] = 1.0 - rho;
}

// per-label sums of the mass pass and the sources they give.  EXACT: one thread
// per label adds its nodes in bulk order, as the reference's serial loop does;
// otherwise one warp per label, strided partial sums and a fixed shuffle tree
// (deterministic).
template <bool EXACT>
__global__ void k_links_label_sum(LinksArgs A) {
    if constexpr (EXACT) {
        const int l = blockIdx.x * blockDim.x + threadIdx.x + 1;
        if (l > A.nlab) return;
        double s = 0.0;
        for (int k = A.lab_start[l]; k < A.lab_start[l + 1]; ++k) s += A.lab_val[k];
        A.lab_q[l] = A.lab_g[l] * s;
    } else {
        const int l = (blockIdx.x * blockDim.x + threadIdx.x) / 32 + 1;
        const int lane = threadIdx.x & 31;
        if (l > A.nlab) return;
        double s = 0.0;
        for (int k = A.lab_start[l] + lane; k < A.lab_start[l + 1]; k += 32) s += A.lab_val[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) A.lab_q[l] = A.lab_g[l] * s;
    }
}

template <bool EXACT, bool LOCAL>
__global__ void __launch_bounds__(kBlock) k_links_collide(LinksArgs A) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.s.L.nf) return;
    const uint32_t inf = __ldg(A.info + i);
    double u[3], f[19], rho, vel[3];
    links_velocity<LOCAL>(A, i, inf, u);
    load_links<EXACT, LOCAL>(static_cast<const double*>(A.s.src), A.s.L, i, u, A.rho_w, f);
    collide_links<EXACT>(f, A, i, inf, rho, vel);
    const size_t pad = static_cast<size_t>(A.s.L.nf_pad);
    double* out = static_cast<double*>(A.s.dst);
#pragma unroll
    for (int q = 0; q < 19; ++q) out[static_cast<size_t>(q) * pad + i] = f[q];
    if (inf & kLinkPress) {
        const int p = __ldg(A.pidx + i);
#pragma unroll
        for (int d = 0; d < 3; ++d) A.ustore[static_cast<size_t>(d) * A.npress + p] = vel[d];
    }
    if (A.s.rho_out) {
        A.s.rho_out[i] = rho;
#pragma unroll
        for (int d = 0; d < 3; ++d) A.s.vel_out[static_cast<size_t>(d) * pad + i] = vel[d];
    }
}

// the reference's f (after streaming and the boundaries) in AoS bulk order
template <bool EXACT, bool LOCAL>
__global__ void __launch_bounds__(kBlock) k_links_gather(LinksArgs A, const int32_t* __restrict__ slot_bulk,
                                                         double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.s.L.nf) return;
    const uint32_t inf = __ldg(A.info + i);
    double u[3], f[19];
    links_velocity<LOCAL>(A, i, inf, u);
    load_links<EXACT, LOCAL>(static_cast<const double*>(A.s.src), A.s.L, i, u, A.rho_w, f);
    const size_t b = static_cast<size_t>(slot_bulk[i]);
#pragma unroll
    for (int q = 0; q < 19; ++q) out[b * 19 + q] = f[q];
}

// per-block sums of [mass, 0, fc_x, fc_y, fc_z, max|f|] of the reference's f
template <bool EXACT, bool LOCAL>
__global__ void __launch_bounds__(kBlock) k_links_moments(LinksArgs A) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double vals[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    if (i < A.s.L.nf) {
        const uint32_t inf = __ldg(A.info + i);
        double u[3], f[19];
        links_velocity<LOCAL>(A, i, inf, u);
        load_links<EXACT, LOCAL>(static_cast<const double*>(A.s.src), A.s.L, i, u, A.rho_w, f);
        double j[3], mx = 0.0;
        qsumc_ref<19>(f, j);
#pragma unroll
        for (int q = 0; q < 19; ++q) {
            vals[0] += f[q];
            const double af = fabs(f[q]);
            mx = (af != af || isinf(af)) ? CUDART_INF : fmax(mx, af);
        }
        vals[2] = j[0];
        vals[3] = j[1];
        vals[4] = j[2];
        vals[5] = mx;
    }
    block_reduce_store<6>(vals, A.s.partials, true);
}

// ---------------------------------------------------------------------------
// Shifted storage (F32 / F16 / BF16) with FP32 arithmetic on the deviations
// d_q = f_q - w_q rho_ref; the stored value is d_q * scale / w_q.
// ---------------------------------------------------------------------------
template <class S, bool LOCAL>
__device__ __forceinline__ void load_links_shift(const S* __restrict__ g, const LinksArgs& A, int i, const float* u,
                                                 float* fd) {
    constexpr int Q = 19, R = Lat<Q>::REST;
    const LatticeView& L = A.s.L;
    const size_t pad = static_cast<size_t>(L.nf_pad);
    const float is = A.s.f_inv_scale;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const float wq = static_cast<float>(Lat<Q>::w(q));
        if (LOCAL || q == R) {
            fd[q] = Store<S>::val(g[static_cast<size_t>(q) * pad + i]) * (wq * is);
            continue;
        }
        const int e = __ldg(L.pull + static_cast<size_t>(q) * pad + i);
        if (e >= 0) {
            fd[q] = Store<S>::val(g[e]) * (wq * is);  // reversed directions have the same weight
        } else {
            // f = -f_k + 2 w rho_w (1 + (9 cu^2 - 3 u^2)/2)  ->  d = -d_k + w (2 (rho_w - rho_ref) + rho_w (9 cu^2 - 3 u^2))
            const int k = Lat<Q>::rev(q);
            const float dk = Store<S>::val(g[~e]) * (wq * is);
            const float u2 = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
            const float cu = Lat<Q>::cx(k) * u[0] + Lat<Q>::cy(k) * u[1] + Lat<Q>::cz(k) * u[2];
            fd[q] = -dk + wq * (A.f_dw + A.f_rho_w * (9.0f * cu * cu - 3.0f * u2));
        }
    }
}

template <bool LOCAL>
__device__ __forceinline__ void links_velocity_f(const LinksArgs& A, int i, uint32_t inf, float* u) {
    u[0] = u[1] = u[2] = 0.0f;
    if (!LOCAL && (inf & kLinkPress)) {
        const int p = __ldg(A.pidx + i);
#pragma unroll
        for (int d = 0; d < 3; ++d) u[d] = static_cast<float>(A.ustore[static_cast<size_t>(d) * A.npress + p]);
    }
}

// the collision of collide_links on deviations: feq - w rho_ref = w (drho + rho (3 cu + 4.5 cu^2 - 1.5 u^2))
__device__ __forceinline__ void collide_links_shift(float* fd, const LinksArgs& A, int i, uint32_t inf, float& drho_o,
                                                    float* vel_o) {
    constexpr int Q = 19;
    const StepArgs& a = A.s;
    float dr = 0.0f;
#pragma unroll
    for (int q = 0; q < Q; ++q) dr += fd[q];
    const float qs = (inf & kLinkAdd) ? static_cast<float>(A.lab_q[inf & kLinkLabelMask]) : 0.0f;
    dr += 0.5f * qs;
    const float rho = a.f_rho_ref + dr;
    const float fo = static_cast<float>(__ldg(A.force_on + i));
    float F[3], j[3] = {0.0f, 0.0f, 0.0f}, vel[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) F[d] = a.params->forcef[d] * fo;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        j[0] += Lat<Q>::cx(q) * fd[q];
        j[1] += Lat<Q>::cy(q) * fd[q];
        j[2] += Lat<Q>::cz(q) * fd[q];
    }
    const float irho = 1.0f / rho;
#pragma unroll
    for (int d = 0; d < 3; ++d) vel[d] = (j[d] + 0.5f * F[d]) * irho;
    drho_o = dr;
#pragma unroll
    for (int d = 0; d < 3; ++d) vel_o[d] = vel[d];
    const float u2 = vel[0] * vel[0] + vel[1] * vel[1] + vel[2] * vel[2];
    const float uF = vel[0] * F[0] + vel[1] * F[1] + vel[2] * F[2];
    const float oms = a.f_tau_inv, tf = a.f_tf;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const float w = static_cast<float>(Lat<Q>::w(q));
        const float cu = Lat<Q>::cx(q) * vel[0] + Lat<Q>::cy(q) * vel[1] + Lat<Q>::cz(q) * vel[2];
        const float cF = Lat<Q>::cx(q) * F[0] + Lat<Q>::cy(q) * F[1] + Lat<Q>::cz(q) * F[2];
        const float sh = 3.0f * cu + 4.5f * cu * cu - 1.5f * u2;
        const float eq = w * (dr + rho * sh);
        const float dF = w * tf * (3.0f * cF + 9.0f * cF * cu - 3.0f * uF);
        const float dQ = tf * qs * w * (1.0f + sh);
        fd[q] = fd[q] - oms * (fd[q] - eq) + dF + dQ;
    }
}

template <class S, bool LOCAL>
__global__ void __launch_bounds__(kBlock) k_links_mass_shift(LinksArgs A) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= A.nlabeled) return;
    const int i = __ldg(A.lab_slot + k);
    const uint32_t inf = __ldg(A.info + i);
    float u[3], fd[19];
    links_velocity_f<LOCAL>(A, i, inf, u);
    load_links_shift<S, LOCAL>(static_cast<const S*>(A.s.src), A, i, u, fd);
    float dr = 0.0f;
#pragma unroll
    for (int q = 0; q < 19; ++q) dr += fd[q];
    A.lab_val[k] = (1.0 - A.s.rho_ref) - static_cast<double>(dr);
}

// resident blocks per SM asked of the register allocator for the shifted step (192^3
// tagged pack, F32 / F16 MLUPS: 3 blocks 15.7k / 17.1k, 4: 17.6k / 18.7k, 5: 18.3k / 20.4k,
// 6: 17.4k / 18.7k)
#ifndef BCLBM_LINKS_MINB
#define BCLBM_LINKS_MINB 5
#endif

template <class S, bool LOCAL>
__global__ void __launch_bounds__(kBlock, BCLBM_LINKS_MINB) k_links_collide_shift(LinksArgs A) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.s.L.nf) return;
    const uint32_t inf = __ldg(A.info + i);
    float u[3], fd[19], dr, vel[3];
    links_velocity_f<LOCAL>(A, i, inf, u);
    load_links_shift<S, LOCAL>(static_cast<const S*>(A.s.src), A, i, u, fd);
    collide_links_shift(fd, A, i, inf, dr, vel);
    const size_t pad = static_cast<size_t>(A.s.L.nf_pad);
    S* out = static_cast<S*>(A.s.dst);
    const float sc = A.s.f_scale;
#pragma unroll
    for (int q = 0; q < 19; ++q)
        Store<S>::store(out + static_cast<size_t>(q) * pad + i, fd[q] * (sc / static_cast<float>(Lat<19>::w(q))));
    if (inf & kLinkPress) {
        const int p = __ldg(A.pidx + i);
#pragma unroll
        for (int d = 0; d < 3; ++d) A.ustore[static_cast<size_t>(d) * A.npress + p] = vel[d];
    }
    if (A.s.rho_out) {
        A.s.rho_out[i] = A.s.rho_ref + static_cast<double>(dr);
#pragma unroll
        for (int d = 0; d < 3; ++d) A.s.vel_out[static_cast<size_t>(d) * pad + i] = vel[d];
    }
}

template <class S, bool LOCAL>
__global__ void __launch_bounds__(kBlock) k_links_gather_shift(LinksArgs A, const int32_t* __restrict__ slot_bulk,
                                                               double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.s.L.nf) return;
    const uint32_t inf = __ldg(A.info + i);
    float u[3], fd[19];
    links_velocity_f<LOCAL>(A, i, inf, u);
    load_links_shift<S, LOCAL>(static_cast<const S*>(A.s.src), A, i, u, fd);
    const size_t b = static_cast<size_t>(slot_bulk[i]);
#pragma unroll
    for (int q = 0; q < 19; ++q) out[b * 19 + q] = Lat<19>::w(q) * A.s.rho_ref + static_cast<double>(fd[q]);
}

template <class S, bool LOCAL>
__global__ void __launch_bounds__(kBlock) k_links_moments_shift(LinksArgs A) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double vals[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    if (i < A.s.L.nf) {
        const uint32_t inf = __ldg(A.info + i);
        float u[3], fd[19];
        links_velocity_f<LOCAL>(A, i, inf, u);
        load_links_shift<S, LOCAL>(static_cast<const S*>(A.s.src), A, i, u, fd);
        double mx = 0.0, dr = 0.0;
#pragma unroll
        for (int q = 0; q < 19; ++q) {
            const double d = static_cast<double>(fd[q]);
            dr += d;
            vals[2] += Lat<19>::cx(q) * d;
            vals[3] += Lat<19>::cy(q) * d;
            vals[4] += Lat<19>::cz(q) * d;
            const double af = fabs(Lat<19>::w(q) * A.s.rho_ref + d);
            mx = (af != af || isinf(af)) ? CUDART_INF : fmax(mx, af);
        }
        vals[0] = A.s.rho_ref + dr;
        vals[5] = mx;
    }
    block_reduce_store<6>(vals, A.s.partials, true);
}

// the mass flux of the write step (main.cpp:552-562): 0.5 sum of rho u_z over
// the pressure-boundary nodes of each phase, in node order
__global__ void k_links_flux(LinksArgs A);

}  // namespace bclbm
