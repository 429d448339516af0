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
    double* ustore;             // [3][npress] velocity of the last step (FP64; the shifted formats keep
                                // FP32 values in it: their kernels alone read it)
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
    int64_t x_wrho[3];          // fixed-point step: w rho_w by weight class (rest, axis, diagonal)
};

// FP64 value of a stored population: FP64 storage holds f itself; the default
// FP64 step (collide in fixed point) keeps its state in the collision's int64
// format (Store<int64_t>), as the std_case step does
__device__ __forceinline__ double as_f64(double v) { return v; }
__device__ __forceinline__ double as_f64(int64_t v) { return fx::store_f64(v); }

// applyPressureFluidBoundary (main.cpp:154-173), qUnknown = q, qKnown = rev(q):
// the anti-bounce-back population from the known one and the node's velocity
__device__ __forceinline__ double anti_bounce_back(int q, double fk, const double* u, double rho_w) {
    constexpr int Q = 19;
    const int k = Lat<Q>::rev(q);
    const double u2 = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];  // DXQY::dot
    const double cu = Lat<Q>::cx(k) * u[0] + Lat<Q>::cy(k) * u[1] + Lat<Q>::cz(k) * u[2];  // cDotRef
    const double w = Lat<Q>::w(k);
    return -fk + 2 * w * rho_w * (1 + 0.5 * (9.0 * cu * cu - 3.0 * u2));
}

// the populations that stream into slot i: plain pulls, bounce-back, and the
// anti-bounce-back of the pressure boundary with the node's velocity u
template <bool EXACT, bool LOCAL, class G = double>
__device__ __forceinline__ void load_links(const G* __restrict__ g, const LatticeView& L, int i, const double* u,
                                           double rho_w, double* f) {
    constexpr int Q = 19, R = Lat<Q>::REST;
    const size_t pad = static_cast<size_t>(L.nf_pad);
    if constexpr (LOCAL) {
#pragma unroll
        for (int q = 0; q < Q; ++q) f[q] = as_f64(g[static_cast<size_t>(q) * pad + i]);
        return;
    }
    // table entries, then the gathers (an anti-bounce-back entry ~e reads element e), then the
    // anti-bounce-back terms, so that the loads are in flight together
    int e[Q - 1];
#pragma unroll
    for (int q = 0; q < Q - 1; ++q) e[q] = __ldg(L.pull + static_cast<size_t>(q) * pad + i);
#pragma unroll
    for (int q = 0; q < Q - 1; ++q) f[q] = as_f64(g[e[q] >= 0 ? e[q] : ~e[q]]);
    f[R] = as_f64(g[static_cast<size_t>(R) * pad + i]);
#pragma unroll
    for (int q = 0; q < Q - 1; ++q)
        if (e[q] < 0) f[q] = anti_bounce_back(q, f[q], u, rho_w);
}

// load_links of the int64 state without conversions, the anti-bounce-back entries
// (pressure-boundary nodes only) in fixed point from the node's velocity u and
// xw = w rho_w by weight class
template <bool LOCAL>
__device__ __forceinline__ void load_links_fx(const int64_t* __restrict__ g, const LatticeView& L, int i,
                                              const double* u, const int64_t* xw, int64_t* X, unsigned& emax) {
    constexpr int Q = 19, R = Lat<Q>::REST;
    const size_t pad = static_cast<size_t>(L.nf_pad);
    if constexpr (LOCAL) {
#pragma unroll
        for (int q = 0; q < Q; ++q) X[q] = g[static_cast<size_t>(q) * pad + i];
        return;
    }
    int e[Q - 1];
#pragma unroll
    for (int q = 0; q < Q - 1; ++q) e[q] = ld_table(L.pull + static_cast<size_t>(q) * pad + i);
#pragma unroll
    for (int q = 0; q < Q - 1; ++q) X[q] = ld_pop(g + (e[q] >= 0 ? e[q] : ~e[q]));
    X[R] = ld_pop(g + static_cast<size_t>(R) * pad + i);
    // the pressure boundary's links (FP64) behind one branch per node: predicated per
    // direction, their conversions would occupy the FP64 pipe in every warp
    unsigned neg = 0;
#pragma unroll
    for (int q = 0; q < Q - 1; ++q) neg |= (static_cast<unsigned>(e[q]) >> 31) << q;
    if (__builtin_expect(neg != 0, 0)) {
        // anti_bounce_back in fixed point, -f_k + 2 w rho_w + w rho_w (9 (c.u)^2 - 3 u^2): the
        // pressure-boundary nodes sit in nearly every warp (each column of the grid starts and
        // ends with one), so their terms stay off the FP64 pipe but for the velocity's conversion
        int64_t ux[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) ux[d] = fx::load_f64_hw(u[d], emax);
        const int64_t u2 = fx::mul_ss(ux[0], ux[0]) + fx::mul_ss(ux[1], ux[1]) + fx::mul_ss(ux[2], ux[2]);
#pragma unroll
        for (int q = 0; q < Q - 1; ++q)
            if (neg & (1u << q)) {
                const int k = Lat<Q>::rev(q);
                const int64_t cu = Lat<Q>::cx(k) * ux[0] + Lat<Q>::cy(k) * ux[1] + Lat<Q>::cz(k) * ux[2];
                const int64_t wr = xw[Lat<Q>::wclass(k)];
                X[q] = 2 * wr - X[q] + fx::mul_ss(9 * fx::mul_ss(cu, cu) - 3 * u2, wr);
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
template <bool EXACT, bool LOCAL, class G = double>
__global__ void __launch_bounds__(kBlock) k_links_mass(LinksArgs A) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= A.nlabeled) return;
    const int i = __ldg(A.lab_slot + k);
    const uint32_t inf = __ldg(A.info + i);
    double u[3], f[19];
    links_velocity<LOCAL>(A, i, inf, u);
    load_links<EXACT, LOCAL, G>(static_cast<const G*>(A.s.src), A.s.L, i, u, A.rho_w, f);
    double rho = 0.0;
#pragma unroll
    for (int q = 0; q < 19; ++q) rho += f[q];
    A.lab_val[k] = 1.0 - rho;
}

// the mass pass of the int64 state: the node's populations summed exactly, one
// conversion of 1 - rho
template <bool LOCAL>
__global__ void __launch_bounds__(kBlock) k_links_mass_fx(LinksArgs A) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= A.nlabeled) return;
    const int i = __ldg(A.lab_slot + k);
    const uint32_t inf = __ldg(A.info + i);
    double u[3];
    links_velocity<LOCAL>(A, i, inf, u);
    unsigned emax = 0;
    int64_t X[19];
    load_links_fx<LOCAL>(static_cast<const int64_t*>(A.s.src), A.s.L, i, u, A.x_wrho, X, emax);
    int64_t rho = 0;
#pragma unroll
    for (int q = 0; q < 19; ++q) rho += X[q];
    A.lab_val[k] = fx::store_f64(fx::ONE - rho);
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
#pragma unroll 8
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

// k_links_collide with the collision in 64-bit fixed point (bclbm_fixed.cuh,
// collide_to with the node's force attribute and mass source), the state kept
// in the collision's int64 format between steps (no conversion per population;
// the anti-bounce-back terms of the pressure-boundary nodes are formed in FP64).
// The default BCLBM_F64 arithmetic of the std_one_phase step: GB300's FP64 pipe
// caps the FP64 forms of the collision at about a tenth of the HBM bandwidth.
template <bool LOCAL>
// resident blocks per SM asked of the register allocator by the fixed-point links step
#ifndef BCLBM_LINKS_FX_MINB
#define BCLBM_LINKS_FX_MINB 3
#endif
#ifndef BCLBM_LINKS_FX_BLOCK
#define BCLBM_LINKS_FX_BLOCK 256
#endif
__global__ void __launch_bounds__(BCLBM_LINKS_FX_BLOCK, BCLBM_LINKS_FX_MINB) k_links_collide_fixed(LinksArgs A) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.s.L.nf) return;
    const uint32_t inf = __ldg(A.info + i);
    double u[3];
    links_velocity<LOCAL>(A, i, inf, u);
    unsigned emax = 0;
    int64_t X[19];
    load_links_fx<LOCAL>(static_cast<const int64_t*>(A.s.src), A.s.L, i, u, A.x_wrho, X, emax);
    int64_t qm = 0;
    if (inf & kLinkAdd) qm = fx::load_f64_hw(A.lab_q[inf & kLinkLabelMask], emax);
    int ovf = emax >= fx::kLoadEmaxLimit ? 1 : 0;
    const int fo = __ldg(A.force_on + i);
    const size_t pad = static_cast<size_t>(A.s.L.nf_pad);
    int64_t* out = static_cast<int64_t*>(A.s.dst) + i;
    int64_t rho, uf[3];
    fx::collide_to<19, false, true>(
        X, A.s.fxk, rho, uf, ovf, [out, pad](int q, int64_t v) { out[static_cast<size_t>(q) * pad] = v; }, fo, qm);
    // FP64 velocities only where they are kept: pressure-boundary nodes and macro downloads
    if (inf & kLinkPress) {
        const int p = __ldg(A.pidx + i);
#pragma unroll
        for (int d = 0; d < 3; ++d) A.ustore[static_cast<size_t>(d) * A.npress + p] = fx::store_f64(uf[d]);
    }
    if (A.s.rho_out) {
        A.s.rho_out[i] = fx::store_f64(rho);
#pragma unroll
        for (int d = 0; d < 3; ++d) A.s.vel_out[static_cast<size_t>(d) * pad + i] = fx::store_f64(uf[d]);
    }
    if (ovf) atomicOr(A.s.fx_flag, 1);
}

// the reference's f (after streaming and the boundaries) in AoS bulk order
template <bool EXACT, bool LOCAL, class G = double>
__global__ void __launch_bounds__(kBlock) k_links_gather(LinksArgs A, const int32_t* __restrict__ slot_bulk,
                                                         double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.s.L.nf) return;
    const uint32_t inf = __ldg(A.info + i);
    double u[3], f[19];
    links_velocity<LOCAL>(A, i, inf, u);
    load_links<EXACT, LOCAL, G>(static_cast<const G*>(A.s.src), A.s.L, i, u, A.rho_w, f);
    const size_t b = static_cast<size_t>(slot_bulk[i]);
#pragma unroll
    for (int q = 0; q < 19; ++q) out[b * 19 + q] = f[q];
}

// per-block sums of [mass, 0, fc_x, fc_y, fc_z, max|f|] of the reference's f
template <bool EXACT, bool LOCAL, class G = double>
__global__ void __launch_bounds__(kBlock) k_links_moments(LinksArgs A) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double vals[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    if (i < A.s.L.nf) {
        const uint32_t inf = __ldg(A.info + i);
        double u[3], f[19];
        links_velocity<LOCAL>(A, i, inf, u);
        load_links<EXACT, LOCAL, G>(static_cast<const G*>(A.s.src), A.s.L, i, u, A.rho_w, f);
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
    if constexpr (LOCAL) {
#pragma unroll
        for (int q = 0; q < Q; ++q)
            fd[q] = Store<S>::val(g[static_cast<size_t>(q) * pad + i]) * (static_cast<float>(Lat<Q>::w(q)) * is);
        return;
    }
    // all table entries, then all gathers (an anti-bounce-back entry ~e reads element e), then the
    // anti-bounce-back terms: no branch between the loads, so they are all in flight together
    int e[Q - 1];
    typename Store<S>::T raw[Q];
#pragma unroll
    for (int q = 0; q < Q - 1; ++q) e[q] = __ldg(L.pull + static_cast<size_t>(q) * pad + i);
#pragma unroll
    for (int q = 0; q < Q - 1; ++q) raw[q] = g[e[q] >= 0 ? e[q] : ~e[q]];
    raw[R] = g[static_cast<size_t>(R) * pad + i];
    const float u2 = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const float wq = static_cast<float>(Lat<Q>::w(q));  // reversed directions have the same weight
        float v = Store<S>::val(raw[q]) * (wq * is);
        if (q != R && e[q < R ? q : 0] < 0) {
            // f = -f_k + 2 w rho_w (1 + (9 cu^2 - 3 u^2)/2)  ->  d = -d_k + w (2 (rho_w - rho_ref) + rho_w (9 cu^2 - 3 u^2))
            const int k = Lat<Q>::rev(q);
            const float cu = Lat<Q>::cx(k) * u[0] + Lat<Q>::cy(k) * u[1] + Lat<Q>::cz(k) * u[2];
            v = -v + wq * (A.f_dw + A.f_rho_w * (9.0f * cu * cu - 3.0f * u2));
        }
        fd[q] = v;
    }
}

template <bool LOCAL>
__device__ __forceinline__ void links_velocity_f(const LinksArgs& A, int i, uint32_t inf, float* u) {
    u[0] = u[1] = u[2] = 0.0f;
    if (!LOCAL && (inf & kLinkPress)) {
        const int p = __ldg(A.pidx + i);
#pragma unroll
        for (int d = 0; d < 3; ++d) u[d] = reinterpret_cast<const float*>(A.ustore)[static_cast<size_t>(d) * A.npress + p];
    }
}

// the collision of collide_links on deviations, regrouped by direction pairs
// (k, k + 9): with drho' = sum d + q/2, rho = rho_ref + drho', G = oms rho + tsf q,
//   X = w (G (4.5 cu^2 - 1.5 u^2) + oms drho' + tsf q + tsf (9 cF cu - 3 uF))
//   Y = 3 w (G cu + tsf cF)
//   d*_k = (1 - oms) d_k + X + Y,   d*_{k+9} = (1 - oms) d_{k+9} + X - Y
// which is calcOmegaBGK + calcDeltaOmegaF + calcDeltaOmegaQ of the node loop.
__device__ __forceinline__ void collide_links_shift(float* fd, const LinksArgs& A, int i, uint32_t inf, float& drho_o,
                                                    float* vel_o) {
    constexpr int Q = 19, NP = Lat<Q>::NP, R = Lat<Q>::REST;
    const StepArgs& a = A.s;
    float p[NP], m[NP];
#pragma unroll
    for (int k = 0; k < NP; ++k) {
        p[k] = fd[k] + fd[k + NP];
        m[k] = fd[k] - fd[k + NP];
    }
    float dr = fd[R];
#pragma unroll
    for (int k = 0; k < NP; ++k) dr += p[k];
    float j[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
    for (int k = 0; k < NP; ++k) {
        if (Lat<Q>::cx(k) > 0) j[0] += m[k];
        if (Lat<Q>::cx(k) < 0) j[0] -= m[k];
        if (Lat<Q>::cy(k) > 0) j[1] += m[k];
        if (Lat<Q>::cy(k) < 0) j[1] -= m[k];
        if (Lat<Q>::cz(k) > 0) j[2] += m[k];
        if (Lat<Q>::cz(k) < 0) j[2] -= m[k];
    }
    const float qs = (inf & kLinkAdd) ? static_cast<float>(A.lab_q[inf & kLinkLabelMask]) : 0.0f;
    dr += 0.5f * qs;
    const float rho = a.f_rho_ref + dr;
    const float fo = static_cast<float>(__ldg(A.force_on + i));
    float F[3], u[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) F[d] = a.params->forcef[d] * fo;
    const float irho = 1.0f / rho;
#pragma unroll
    for (int d = 0; d < 3; ++d) u[d] = (j[d] + 0.5f * F[d]) * irho;
    drho_o = dr;
#pragma unroll
    for (int d = 0; d < 3; ++d) vel_o[d] = u[d];
    const float u2 = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
    const float uF = u[0] * F[0] + u[1] * F[1] + u[2] * F[2];
    const float oms = a.f_tau_inv, tsf = a.f_tf;
    const float G = oms * rho + tsf * qs;
    const float base = -1.5f * u2;
    const float K0 = oms * dr + tsf * qs - 3.0f * tsf * uF;
    const float keep = 1.0f - oms;
#pragma unroll
    for (int k = 0; k < NP; ++k) {
        const float w = static_cast<float>(Lat<Q>::w(k));
        const float cu = Lat<Q>::cx(k) * u[0] + Lat<Q>::cy(k) * u[1] + Lat<Q>::cz(k) * u[2];
        const float cF = Lat<Q>::cx(k) * F[0] + Lat<Q>::cy(k) * F[1] + Lat<Q>::cz(k) * F[2];
        const float X = w * (G * (4.5f * cu * cu + base) + (9.0f * tsf * cF) * cu + K0);
        const float Y = 3.0f * w * (G * cu + tsf * cF);
        const float fq = fd[k], fr = fd[k + NP];
        fd[k] = keep * fq + (X + Y);
        fd[k + NP] = keep * fr + (X - Y);
    }
    fd[R] = keep * fd[R] + static_cast<float>(Lat<Q>::w(R)) * (G * base + K0);
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
// 6: 17.4k / 18.7k; after the later changes 4: 20.9k / 24.0k, 5: 20.4k / 24.9k, 6: 17.6k /
// 21.5k): 5 for the 2-byte formats, 4 for FP32
#ifndef BCLBM_LINKS_MINB
#define BCLBM_LINKS_MINB 5
#endif
template <class S>
constexpr int links_min_blocks() {
    return sizeof(S) == 2 ? BCLBM_LINKS_MINB : 4;
}

template <class S, bool LOCAL>
__global__ void __launch_bounds__(kBlock, links_min_blocks<S>()) k_links_collide_shift(LinksArgs A) {
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
    if (inf & kLinkPress) {  // FP32 values (no conversion on the FP64 pipe in the many warps with one)
        const int p = __ldg(A.pidx + i);
#pragma unroll
        for (int d = 0; d < 3; ++d) reinterpret_cast<float*>(A.ustore)[static_cast<size_t>(d) * A.npress + p] = vel[d];
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
