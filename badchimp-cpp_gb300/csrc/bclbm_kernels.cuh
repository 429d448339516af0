// Kernel templates of the bclbm time step.  Included by bclbm_exact.cu
// (compiled with -fmad=false; the FP64 kernels that follow the reference's
// expression order) and by bclbm_kernels.cu (everything else).
//
// One thread owns one fluid slot.  A step kernel pulls the Q populations that
// stream into its slot (bounce-back fused, see bclbm_device.cuh), computes the
// moments, collides, and writes the post-collision populations to its own
// slot of the other buffer: reads are gathers along the neighbour table,
// writes are fully coalesced rows.  The device state is therefore the
// post-collision field G of the last step; the reference's f (post-stream,
// post-bounce-back) is one pull of G away and is produced by k_gather on
// download.  The first step after create reads the uploaded f directly
// (LOCAL = true).
#pragma once

#include <math_constants.h>
#include <type_traits>

#include "bclbm_device.cuh"
#include "bclbm_fixed.cuh"
#include "bclbm_stage.cuh"

namespace bclbm {

constexpr int kBlock = 256;
constexpr double C2 = 1.0 / 3.0;  // DXQY::c2 = 1.0 / c2Inv

struct DevParams {
    double force[3];
    float forcef[3];  // the same force rounded to FP32, for the FP32-arithmetic kernels
    int64_t forcex[3];  // and in 64-bit fixed point, for the fixed-point two-phase kernel
    int fx_overflow;  // set by the fixed-point kernel when a value left its range
    // two-phase shifted storage: the conserved totals sum f0 + f1 and sum f0 - f1
    // (set at create) and the uniform per-node correction the collision adds this
    // step to put the totals back (mass-drift correction)
    double mass_target[2];
    double mass_fix[2];
    float mass_fixf[2];
};

struct StepArgs {
    LatticeView L;
    const void* src;        // state read by this step (G, or f when LOCAL)
    void* dst;              // post-collision output
    double* rho_out;        // [nfields][nf_pad] when MACROS
    double* vel_out;        // [D][nf_pad] when MACROS
    double* cg;             // RK, F64: colour of [nf fluid | ns solids | ghost]
    float* cgf;             // RK, shifted formats: the same colour field in FP32
    float* cgf_out;         // RK, one pass per step: the colour field this step writes
    int64_t* cgx;           // RK, int64 fixed-point state: the colour field in fixed point
                            // (the buffer of cg, which that step does not use)
    const DevParams* params;
    double tau, tau_anti;   // single phase: relaxation times; RK: unused
    double tau_inv, tf;     // exact single phase: 1/tau, 1 - 0.5/tau (host-computed like the reference)
    double tauA_inv, taf;   // exact TRT: 1/tau_anti, 1 - 0.5/tau_anti
    double nu0inv, nu1inv;  // RK
    double sigma, beta;     // RK
    double rho_ref;         // shifted storage reference density
    double scale, inv_scale;// shifted storage scale
    double* partials;       // per-block partial sums (flux controller)
    int n_bulk;             // RK flux controller divisor
    // FP32 copies of the parameters above, rounded on the host, for the FP32-arithmetic
    // kernels (a double -> float conversion in every thread runs on the FP64 pipe)
    float f_tau_inv, f_tauA_inv, f_tf, f_taf, f_rho_ref, f_scale, f_inv_scale, f_nu0inv, f_nu1inv, f_sigma, f_beta;
    int* fx_flag;           // &params->fx_overflow
    fx::Consts fxk;         // constants of the fixed-point collision
    fx::RkConsts fxr;       // constants of the fixed-point two-phase collision
};

// ---------------------------------------------------------------------------
// Reference-order helpers (exact mode).  Each mirrors one reference function
// term by term; C++ evaluates a + b - c as (a + b) - c, as the reference does.
// ---------------------------------------------------------------------------
template <int Q>
__device__ __forceinline__ void qsumc_ref(const double* d, double* r) {  // qSumC
    if constexpr (Q == 9) {  // LBd2q9.h:170-177
        r[0] = +d[0] + d[1] - d[3] - d[4] - d[5] + d[7];
        r[1] = +d[1] + d[2] + d[3] - d[5] - d[6] - d[7];
    } else {  // LBd3q19.h:182-190
        r[0] = +d[0] + d[3] + d[4] + d[5] + d[6] - d[9] - d[12] - d[13] - d[14] - d[15];
        r[1] = +d[1] + d[3] - d[4] + d[7] + d[8] - d[10] - d[12] + d[13] - d[16] - d[17];
        r[2] = +d[2] + d[5] - d[6] + d[7] - d[8] - d[11] - d[14] + d[15] - d[16] + d[17];
    }
}

template <int Q>
__device__ __forceinline__ void cdotall_ref(const double* v, double* r) {  // cDotAll
    if constexpr (Q == 9) {  // LBd2q9.h:128-142
        r[0] = +v[0];
        r[1] = +v[0] + v[1];
        r[2] = +v[1];
        r[3] = -v[0] + v[1];
        r[4] = -v[0];
        r[5] = -v[0] - v[1];
        r[6] = -v[1];
        r[7] = +v[0] - v[1];
        r[8] = 0.0;
    } else {  // LBd3q19.h:129-153
        r[0] = +v[0];
        r[1] = +v[1];
        r[2] = +v[2];
        r[3] = +v[0] + v[1];
        r[4] = +v[0] - v[1];
        r[5] = +v[0] + v[2];
        r[6] = +v[0] - v[2];
        r[7] = +v[1] + v[2];
        r[8] = +v[1] - v[2];
        r[9] = -v[0];
        r[10] = -v[1];
        r[11] = -v[2];
        r[12] = -v[0] - v[1];
        r[13] = -v[0] + v[1];
        r[14] = -v[0] - v[2];
        r[15] = -v[0] + v[2];
        r[16] = -v[1] - v[2];
        r[17] = -v[1] + v[2];
        r[18] = 0.0;
    }
}

template <int Q>
__device__ __forceinline__ double dot_ref(const double* a, const double* b) {  // DXQY::dot
    if constexpr (Q == 9) return a[0] * b[0] + a[1] * b[1];
    else return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

template <int Q>
__device__ __forceinline__ void grad_ref(const double* s, double* r) {  // DXQY::grad
    constexpr double a = Lat<Q>::w1c2inv, b = Lat<Q>::w2c2inv;
    if constexpr (Q == 9) {  // LBd2q9.h:144-151
        r[0] = +a * (+s[0] - s[4]) + b * (+s[1] - s[3] - s[5] + s[7]);
        r[1] = +a * (+s[2] - s[6]) + b * (+s[1] + s[3] - s[5] - s[7]);
    } else {  // LBd3q19.h:155-163
        r[0] = +a * (+s[0] - s[9]) + b * (+s[3] + s[4] + s[5] + s[6] - s[12] - s[13] - s[14] - s[15]);
        r[1] = +a * (+s[1] - s[10]) + b * (+s[3] - s[4] + s[7] + s[8] - s[12] + s[13] - s[16] - s[17]);
        r[2] = +a * (+s[2] - s[11]) + b * (+s[5] - s[6] + s[7] - s[8] - s[14] + s[15] - s[16] + s[17]);
    }
}

__device__ __forceinline__ double cnorm_ref(int wclass) {  // DXQY::cNorm (SQRT2, LBglobal.h:11)
    return wclass == 1 ? 1.0 : 1.4142135623730950488;
}

// ---------------------------------------------------------------------------
// Population access
// ---------------------------------------------------------------------------
// Loads of the pull table and of the gathered populations.  BCLBM_L2_HINT asks
// the L2 to fetch the surrounding 128 (1) or 256 (2) bytes with each miss: a
// warp reads 64-256 contiguous bytes of a table row or of a population row,
// and the warps on the next slots read the bytes after them.
#ifndef BCLBM_L2_HINT
#define BCLBM_L2_HINT 2
#endif
__device__ __forceinline__ int32_t ld_table(const int32_t* p) {
#if BCLBM_L2_HINT == 2
    int32_t v;
    asm("ld.global.nc.L2::256B.b32 %0, [%1];" : "=r"(v) : "l"(p));
    return v;
#elif BCLBM_L2_HINT == 1
    int32_t v;
    asm("ld.global.nc.L2::128B.b32 %0, [%1];" : "=r"(v) : "l"(p));
    return v;
#else
    return __ldg(p);
#endif
}

template <class T>
__device__ __forceinline__ T ld_pop(const T* p) {
#if BCLBM_L2_HINT >= 1
#if BCLBM_L2_HINT == 2
#define BCLBM_L2Q ".L2::256B"
#else
#define BCLBM_L2Q ".L2::128B"
#endif
    if constexpr (sizeof(T) == 2) {
        unsigned short v;
        asm("ld.global" BCLBM_L2Q ".b16 %0, [%1];" : "=h"(v) : "l"(p));
        T r;
        __builtin_memcpy(&r, &v, 2);
        return r;
    } else if constexpr (sizeof(T) == 4) {
        unsigned v;
        asm("ld.global" BCLBM_L2Q ".b32 %0, [%1];" : "=r"(v) : "l"(p));
        T r;
        __builtin_memcpy(&r, &v, 4);
        return r;
    } else {
        unsigned long long v;
        asm("ld.global" BCLBM_L2Q ".b64 %0, [%1];" : "=l"(v) : "l"(p));
        T r;
        __builtin_memcpy(&r, &v, 8);
        return r;
    }
#undef BCLBM_L2Q
#else
    return *p;
#endif
}

// PULL: single-phase instances read the resolved pull table, two-phase
// instances the extended neighbour table (which the colour gradient needs too).
template <int Q, class S, bool LOCAL, bool PULL = false>
__device__ __forceinline__ void load_field(const S* __restrict__ g, const LatticeView& L, int i,
                                           typename Store<S>::T* v) {
    constexpr int R = Lat<Q>::REST;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        if (q == R || LOCAL) {
            v[q] = g[static_cast<size_t>(q) * L.nf_pad + i];
        } else if (PULL) {
            v[q] = ld_pop(g + ld_table(L.pull + static_cast<size_t>(q) * L.nf_pad + i));
        } else {
            const int y = __ldg(L.nbr + static_cast<size_t>(Lat<Q>::rev(q)) * L.nf_pad + i);
            v[q] = pull_raw<Q, S>(g, L, q, y, i);
        }
    }
}

// The same pull with the table entries already staged in shared memory:
// rows[q][t] is the pull-table entry of direction q for this thread's slot.
template <int Q, class S, int TILE>
__device__ __forceinline__ void load_field_staged(const S* __restrict__ g, const LatticeView& L, int i,
                                                  const int32_t (*rows)[TILE], int t, typename Store<S>::T* v) {
    constexpr int R = Lat<Q>::REST;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        if (q == R) v[q] = g[static_cast<size_t>(q) * L.nf_pad + i];
        else v[q] = g[rows[q][t]];
    }
}

// Converts raw stored values to the compute representation: f itself (F64),
// or the deviation f - w rho_ref (shifted formats).
template <int Q, class S, class C>
__device__ __forceinline__ void decode(const typename Store<S>::T* v, C* f, C inv_scale) {
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        if constexpr (Store<S>::shifted) f[q] = static_cast<C>(Store<S>::val(v[q])) * (static_cast<C>(Lat<Q>::w(q)) * inv_scale);
        else f[q] = static_cast<C>(v[q]);
    }
}

template <int Q, class S, class C>
__device__ __forceinline__ void encode_store(S* __restrict__ out, size_t nf_pad, int i, const C* f, C scale) {
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        if constexpr (Store<S>::shifted) Store<S>::store(out + q * nf_pad + i, static_cast<float>(f[q] * (scale / static_cast<C>(Lat<Q>::w(q)))));
        else out[q * nf_pad + i] = static_cast<double>(f[q]);
    }
}

// ---------------------------------------------------------------------------
// Single-phase collision, exact reference order (std_case/main.cpp:112-133)
// ---------------------------------------------------------------------------
template <int Q, bool TRT>
__device__ __forceinline__ void collide_exact(double* f, const double* F, const StepArgs& a, double& rho_o,
                                              double* vel_o) {
    constexpr int D = Lat<Q>::D;
    double rho = 0.0;  // calcRho -> qSum
#pragma unroll
    for (int q = 0; q < Q; ++q) rho += f[q];
    double j[D], vel[D];
    qsumc_ref<Q>(f, j);
#pragma unroll
    for (int d = 0; d < D; ++d) vel[d] = (j[d] + 0.5 * F[d]) / rho;  // calcVel (LBmacroscopic.h:85)
    rho_o = rho;
#pragma unroll
    for (int d = 0; d < D; ++d) vel_o[d] = vel[d];
    const double u2 = dot_ref<Q>(vel, vel);
    double cu[Q], cF[Q];
    cdotall_ref<Q>(vel, cu);
    const double uF = dot_ref<Q>(vel, F);
    cdotall_ref<Q>(F, cF);
    double post[Q];
    if constexpr (!TRT) {
#pragma unroll
        for (int q = 0; q < Q; ++q) {  // calcOmegaBGK (LBcollision.h:43), calcDeltaOmegaF (:210)
            const double w = Lat<Q>::w(q);
            const double om = -a.tau_inv * (f[q] - rho * w * (1.0 + 3.0 * cu[q] + 4.5 * (cu[q] * cu[q] - C2 * u2)));
            const double dF = w * a.tf * (3.0 * cF[q] + 9.0 * (cF[q] * cu[q] - C2 * uF));
            post[q] = f[q] + om + dF;
        }
    } else {
#pragma unroll
        for (int q = 0; q < Q; ++q) {  // calcOmegaBGKTRT (LBcollision.h:68-72), calcDeltaOmegaFTRT (:233)
            const double w = Lat<Q>::w(q);
            const int r = Lat<Q>::rev(q);
            const double fs = 0.5 * (f[q] + f[r]);
            const double fa = 0.5 * (f[q] - f[r]);
            const double om = -a.tau_inv * (fs - rho * w * (1.0 + 4.5 * (cu[q] * cu[q] - C2 * u2))) -
                              a.tauA_inv * (fa - rho * w * 3.0 * cu[q]);
            const double dF = w * 1.0 * (a.taf * 3.0 * cF[q] + a.tf * 9.0 * (cF[q] * cu[q] - C2 * uF));
            post[q] = f[q] + om + dF;
        }
    }
#pragma unroll
    for (int q = 0; q < Q; ++q) f[q] = post[q];
}

// ---------------------------------------------------------------------------
// Single-phase collision, restructured (FMA) in compute type C.
// SHIFT: f holds deviations f - w rho_ref.  BGK is TRT with equal rates.
// post_q  = al f_q + be f_rq + X + Y,  post_rq = al f_rq + be f_q + X - Y
// X = oms w (rho (1 + 4.5 cu^2 - 1.5 u^2) [shifted: rho' + rho(4.5cu^2 - 1.5u^2)]) + w tsf (9 cF cu - 3 uF)
// Y = oma 3 w rho cu + 3 w taf cF
// al = 1 - (oms + oma)/2, be = (oma - oms)/2; the sums are the reference's
// calcOmegaBGK(TRT) + calcDeltaOmegaF(TRT) regrouped by direction pairs.
// ---------------------------------------------------------------------------
template <int Q, class C, bool TRT, bool SHIFT>
__device__ __forceinline__ void collide_fast(C* f, const C* F, C oms, C oma, C tsf, C taf, C rho_ref, C& rho_o,
                                             C* vel_o) {
    constexpr int D = Lat<Q>::D, NP = Lat<Q>::NP, R = Lat<Q>::REST;
    C p[NP], m[NP];
#pragma unroll
    for (int k = 0; k < NP; ++k) {
        p[k] = f[k] + f[k + NP];
        m[k] = f[k] - f[k + NP];
    }
    C rs = f[R];
#pragma unroll
    for (int k = 0; k < NP; ++k) rs += p[k];
    C j[3] = {C(0), C(0), C(0)};
#pragma unroll
    for (int k = 0; k < NP; ++k) {
        if (Lat<Q>::cx(k) > 0) j[0] += m[k];
        if (Lat<Q>::cx(k) < 0) j[0] -= m[k];
        if (Lat<Q>::cy(k) > 0) j[1] += m[k];
        if (Lat<Q>::cy(k) < 0) j[1] -= m[k];
        if (D == 3 && Lat<Q>::cz(k) > 0) j[2] += m[k];
        if (D == 3 && Lat<Q>::cz(k) < 0) j[2] -= m[k];
    }
    const C rho = SHIFT ? rho_ref + rs : rs;  // rs is rho' when shifted
    const C inv = C(1) / rho;
    C u[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) u[d] = (d < D) ? (j[d] + C(0.5) * F[d]) * inv : C(0);
    rho_o = rho;
#pragma unroll
    for (int d = 0; d < D; ++d) vel_o[d] = u[d];
    const C u2 = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
    const C uF = u[0] * F[0] + u[1] * F[1] + u[2] * F[2];
    const C base = SHIFT ? C(-1.5) * u2 : C(1) - C(1.5) * u2;
    const C al = C(1) - C(0.5) * (oms + oma);
    const C be = C(0.5) * (oma - oms);
    // per weight class constants (0 rest, 1 axis, 2 diagonal)
    C Aw[3], Bw[3], Kw[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const C w = static_cast<C>(c == 0 ? Lat<Q>::w(R) : (c == 1 ? Lat<Q>::w(0) : Lat<Q>::w(NP - 1)));
        Aw[c] = oms * rho * w;
        Bw[c] = C(3) * oma * rho * w;
        Kw[c] = C(-3) * w * tsf * uF + (SHIFT ? oms * w * rs : C(0));
    }
#pragma unroll
    for (int k = 0; k < NP; ++k) {
        const int c = Lat<Q>::wclass(k);
        const C w = static_cast<C>(Lat<Q>::w(k));
        const C cu = Lat<Q>::cx(k) * u[0] + Lat<Q>::cy(k) * u[1] + Lat<Q>::cz(k) * u[2];
        const C cF = Lat<Q>::cx(k) * F[0] + Lat<Q>::cy(k) * F[1] + Lat<Q>::cz(k) * F[2];
        const C X = Aw[c] * (C(4.5) * cu * cu + base) + ((C(9) * w * tsf * cF) * cu + Kw[c]);
        const C Y = Bw[c] * cu + C(3) * w * taf * cF;
        const C fq = f[k], fr = f[k + NP];
        if constexpr (TRT) {
            f[k] = al * fq + (be * fr + (X + Y));
            f[k + NP] = al * fr + (be * fq + (X - Y));
        } else {
            f[k] = al * fq + (X + Y);
            f[k + NP] = al * fr + (X - Y);
        }
    }
    f[R] = (C(1) - oms) * f[R] + (Aw[0] * base + Kw[0]);
}

// ---------------------------------------------------------------------------
// k_single: one single-phase time step.
// MODE 0: exact reference order (F64, instantiated in the -fmad=false unit)
// MODE 1: restructured, compute in double (F64) or float (shifted formats)
// ---------------------------------------------------------------------------
// One single-phase update of slot i from its pulled raw values v.
template <int Q, class S, int MODE, bool TRT>
__device__ __forceinline__ void single_node_values(const StepArgs& a, int i, typename Store<S>::T* v) {
    const bool MACROS = a.rho_out != nullptr;
    constexpr int D = Lat<Q>::D;
    S* out = static_cast<S*>(a.dst);
    if constexpr (MODE == 0) {
        double f[Q], F[3], rho, vel[3];
#pragma unroll
        for (int q = 0; q < Q; ++q) f[q] = v[q];
        F[0] = a.params->force[0];
        F[1] = a.params->force[1];
        F[2] = a.params->force[2];
        collide_exact<Q, TRT>(f, F, a, rho, vel);
        if (MACROS) {
            a.rho_out[i] = rho;
#pragma unroll
            for (int d = 0; d < D; ++d) a.vel_out[static_cast<size_t>(d) * a.L.nf_pad + i] = vel[d];
        }
#pragma unroll
        for (int q = 0; q < Q; ++q) out[static_cast<size_t>(q) * a.L.nf_pad + i] = f[q];
    } else {
        constexpr bool F64 = std::is_same<S, double>::value;
        using C = typename std::conditional<F64, double, float>::type;
        C f[Q], F[3], rho, vel[3];
        C oms, oma, tsf, taf, rho_ref, scale, inv_scale;
        if constexpr (F64) {
            F[0] = a.params->force[0];
            F[1] = a.params->force[1];
            F[2] = a.params->force[2];
            oms = a.tau_inv;
            oma = TRT ? a.tauA_inv : a.tau_inv;
            tsf = a.tf;
            taf = TRT ? a.taf : a.tf;
            rho_ref = a.rho_ref;
            scale = a.scale;
            inv_scale = a.inv_scale;
        } else {
            F[0] = a.params->forcef[0];
            F[1] = a.params->forcef[1];
            F[2] = a.params->forcef[2];
            oms = a.f_tau_inv;
            oma = TRT ? a.f_tauA_inv : a.f_tau_inv;
            tsf = a.f_tf;
            taf = TRT ? a.f_taf : a.f_tf;
            rho_ref = a.f_rho_ref;
            scale = a.f_scale;
            inv_scale = a.f_inv_scale;
        }
        decode<Q, S, C>(v, f, inv_scale);
        collide_fast<Q, C, TRT, Store<S>::shifted>(f, F, oms, oma, tsf, taf, rho_ref, rho, vel);
        if (MACROS) {
            a.rho_out[i] = static_cast<double>(rho);
#pragma unroll
            for (int d = 0; d < D; ++d) a.vel_out[static_cast<size_t>(d) * a.L.nf_pad + i] = static_cast<double>(vel[d]);
        }
        encode_store<Q, S, C>(out, a.L.nf_pad, i, f, scale);
    }
}


template <int Q, class S, int MODE, bool TRT, bool LOCAL>
__device__ __forceinline__ void single_node(const StepArgs& a, int i) {
    using T = typename Store<S>::T;
    T v[Q];
    load_field<Q, S, LOCAL, true>(static_cast<const S*>(a.src), a.L, i, v);
    single_node_values<Q, S, MODE, TRT>(a, i, v);
}

// resident blocks per SM asked of the register allocator: the shifted formats
// are HBM-latency bound, and 5 blocks (51 registers, no spills) keep more loads in
// flight than the 4 the allocator picks by itself (FP16 256^3: 38.2 -> 39.6 GLUPS)
template <class S>
constexpr int single_min_blocks() {
    return std::is_same<S, double>::value ? 1 : 5;
}

template <int Q, class S, int MODE, bool TRT, bool LOCAL>
__global__ void __launch_bounds__(kBlock, single_min_blocks<S>()) k_single(StepArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < a.L.nf) single_node<Q, S, MODE, TRT, LOCAL>(a, i);
}

// k_single on a persistent grid with the pull table staged through shared memory
// by the tensor copy engine (bclbm_stage.cuh; pull_map describes L.pull as
// [Q-1][nf_pad] int32): the steps after the first of the native-FP64 (FMA)
// kernel.  At one resident block per SM (146 registers) that kernel cannot hide
// the table -> gather latency chain with other warps, and staging the table one
// sub-tile ahead is measured faster; the shifted-storage and fixed-point kernels
// keep 24-40 warps per SM, hide it already, and measured slower staged (the
// pipeline's loop state, shared-memory reads and wait cost more than it saves).
template <int Q, class S, bool TRT>
__global__ void __launch_bounds__(kBlock, 1) k_single_staged(StepArgs a, const __grid_constant__ CUtensorMap pull_map) {
    __shared__ stage::WarpStage<Q - 1, kBlock / 32> st;
    stage::staged_warps<Q - 1, kBlock / 32>(st, &pull_map, a.L.nf, a.fx_flag,
                                            [&](int i, const int32_t(*rows)[stage::kSub], int lane) {
                                                typename Store<S>::T v[Q];
                                                load_field_staged<Q, S, stage::kSub>(static_cast<const S*>(a.src),
                                                                                     a.L, i, rows, lane, v);
                                                single_node_values<Q, S, 1, TRT>(a, i, v);
                                            });
}

// ---------------------------------------------------------------------------
// k_single_fixed: one single-phase step on F64 storage with 64-bit fixed-point
// arithmetic (bclbm_fixed.cuh).  BCLBM_FX_BLOCK threads per block and at least
// BCLBM_FX_MINB resident blocks per SM asked of the register allocator: 80
// registers, 24 warps per SM.  Blocks of 256 at 3 per SM measured 14,420
// MLUPS at 256^3, of 128 at 6-7 14,600, of 64 at 12 or 14 14,650 (the same
// warps in smaller blocks: finer placement of the work over the SMs), of 32 at
// 28 14,130.  (Earlier: 3 blocks of 256 at 80 registers beat the 2 blocks of
// the unbounded 115-132 registers, 8,925 -> 9,410 MLUPS.)
// ---------------------------------------------------------------------------
#ifndef BCLBM_FX_MINB
#define BCLBM_FX_MINB 12
#endif
// threads per block of k_single_fixed (the kernel uses no shared memory)
#ifndef BCLBM_FX_BLOCK
#define BCLBM_FX_BLOCK 64
#endif

// one update of slot i from its pulled values X (the int64 state of Store<int64_t>)
template <int Q, bool TRT>
__device__ __forceinline__ void fixed_node_values(const StepArgs& a, int i, int64_t* X) {
    constexpr int D = Lat<Q>::D;
    int ovf = 0;
    int64_t rho, u[3];
    int64_t* out = static_cast<int64_t*>(a.dst) + i;
    const size_t pad = static_cast<size_t>(a.L.nf_pad);
    fx::collide_to<Q, TRT>(X, a.fxk, rho, u, ovf, [out, pad](int q, int64_t v) { out[static_cast<size_t>(q) * pad] = v; });
    if (a.rho_out != nullptr) {
        a.rho_out[i] = fx::store_f64(rho);
#pragma unroll
        for (int d = 0; d < D; ++d) a.vel_out[static_cast<size_t>(d) * a.L.nf_pad + i] = fx::store_f64(u[d]);
    }
    if (ovf) atomicOr(a.fx_flag, 1);
}

template <int Q, bool TRT, bool LOCAL>
__device__ __forceinline__ void fixed_node(const StepArgs& a, int i) {
    int64_t X[Q];
    load_field<Q, int64_t, LOCAL, true>(static_cast<const int64_t*>(a.src), a.L, i, X);
    fixed_node_values<Q, TRT>(a, i, X);
}

template <int Q, bool TRT, bool LOCAL>
__global__ void __launch_bounds__(BCLBM_FX_BLOCK, BCLBM_FX_MINB) k_single_fixed(StepArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < a.L.nf) fixed_node<Q, TRT, LOCAL>(a, i);
}

// ---------------------------------------------------------------------------
// Deterministic block reduction of NV doubles (fixed shuffle tree + fixed
// warp order); thread 0 writes partials[blockIdx.x * NV + k].
// ---------------------------------------------------------------------------
template <int NV>
__device__ __forceinline__ void block_reduce_store(double* vals, double* partials, bool max_last, int slot = -1) {
    __shared__ double sh[kBlock / 32][NV];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        double v = vals[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const double t = __shfl_down_sync(0xffffffffu, v, o);
            v = (max_last && k == NV - 1) ? fmax(v, t) : v + t;
        }
        if (lane == 0) sh[warp][k] = v;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            double s = sh[0][k];
            for (int w = 1; w < kBlock / 32; ++w) s = (max_last && k == NV - 1) ? fmax(s, sh[w][k]) : s + sh[w][k];
            partials[static_cast<size_t>(slot < 0 ? static_cast<int>(blockIdx.x) : slot) * NV + k] = s;
        }
    }
}

// The same tree in FP32 (for the per-step sums of the FP32-arithmetic two-phase
// kernels, where FP64 shuffle trees would cost more than the pass itself; the
// block sums go on in FP64).  Deterministic.
template <int NV>
__device__ __forceinline__ void block_reduce_store_f32(float* vals, double* partials) {
    __shared__ float shf[kBlock / 32][NV];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        float v = vals[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) shf[warp][k] = v;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            float s = shf[0][k];
            for (int w = 1; w < kBlock / 32; ++w) s += shf[w][k];
            partials[static_cast<size_t>(blockIdx.x) * NV + k] = static_cast<double>(s);
        }
    }
}

// The block's sums of NV values per thread held in shared memory as sh[NV][kBlock]
// (written by each thread, read after the barrier): warp k adds row k, lane l the
// entries l, l + 32, ... in order, then a shuffle tree.  Deterministic.
template <int NV>
__device__ __forceinline__ void block_sums_from_shared(const float* sh, double* partials) {
    static_assert(NV <= kBlock / 32, "one warp per value");
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (warp < NV) {
        float v = sh[warp * kBlock + lane];
#pragma unroll
        for (int m = 1; m < kBlock / 32; ++m) v += sh[warp * kBlock + m * 32 + lane];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) partials[static_cast<size_t>(blockIdx.x) * NV + warp] = static_cast<double>(v);
    }
}

// Final sum of nrows rows of NV partials by one block of kFinalThreads threads,
// in a fixed order: thread t takes rows t, t + kFinalThreads, ... (loads issued
// four at a time, added in row order), then a fixed pairwise tree over the
// threads.  With max_last the last value is a max instead of a sum.
constexpr int kFinalThreads = 512;

template <int NV>
__device__ __forceinline__ void final_sum(const double* __restrict__ p, int nrows, double* out, bool max_last) {
    __shared__ double sh[NV][kFinalThreads];
    const int t = threadIdx.x;
    double acc[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) acc[k] = 0.0;
    auto add = [&](int k, double v) { acc[k] = (max_last && k == NV - 1) ? fmax(acc[k], v) : acc[k] + v; };
    int b = t;
    for (; b + 3 * kFinalThreads < nrows; b += 4 * kFinalThreads) {
        double v[4][NV];
#pragma unroll
        for (int r = 0; r < 4; ++r)
#pragma unroll
            for (int k = 0; k < NV; ++k) v[r][k] = p[static_cast<size_t>(b + r * kFinalThreads) * NV + k];
#pragma unroll
        for (int r = 0; r < 4; ++r)
#pragma unroll
            for (int k = 0; k < NV; ++k) add(k, v[r][k]);
    }
    for (; b < nrows; b += kFinalThreads)
#pragma unroll
        for (int k = 0; k < NV; ++k) add(k, p[static_cast<size_t>(b) * NV + k]);
#pragma unroll
    for (int k = 0; k < NV; ++k) sh[k][t] = acc[k];
    __syncthreads();
    for (int st = kFinalThreads / 2; st > 0; st >>= 1) {
        if (t < st)
#pragma unroll
            for (int k = 0; k < NV; ++k)
                sh[k][t] = (max_last && k == NV - 1) ? fmax(sh[k][t], sh[k][t + st]) : sh[k][t] + sh[k][t + st];
        __syncthreads();
    }
    if (t < NV) out[t] = sh[t][0];
}

// Sums nblocks rows of NV partials with one block of kFinalThreads; result to out[NV].
template <int NV>
__global__ void __launch_bounds__(kFinalThreads) k_reduce_final(const double* __restrict__ partials, int nblocks,
                                                               double* out, int max_last) {
    final_sum<NV>(partials, nblocks, out, max_last != 0);
}

// ---------------------------------------------------------------------------
// Two-phase (Rothman-Keller) storage.
// F64: field 0 = f0, field 1 = f1 (the reference's two LbField fields).
// Shifted formats: field 0 = total deviation ft - w rho_ref, field 1 = the
// colour difference (f0 - f1); both weight-normalised and scaled.  f0 and f1
// are (ft +- (f0 - f1)) / 2.  The total carries the flow with the FP16 mantissa
// spent on the velocity signal; the colour difference is bounded by w.
// The two fields of an element are stored side by side, [Q][nf_pad][2]: both
// stream from the same upstream element, so a pull is one vector load of the
// pair (4 bytes in FP16/BF16, 8 in FP32, 16 in FP64) and a store one vector
// store, half the memory instructions of two separate fields.
// ---------------------------------------------------------------------------
template <class S>
struct Pair;
template <>
struct Pair<double> {
    using V = double2;
};
template <>
struct Pair<float> {
    using V = float2;
};
template <>
struct Pair<__half> {
    using V = __half2;
};
template <>
struct Pair<__nv_bfloat16> {
    using V = __nv_bfloat162;
};
template <>
struct Pair<int64_t> {
    using V = longlong2;
};

// Two FP32 values rounded to nearest into one stored pair: for the 2-byte formats
// one packed conversion (cvt.rn.f16x2.f32 / cvt.rn.bf16x2.f32), the same bits as
// two separate round-to-nearest conversions.
template <class S>
__device__ __forceinline__ typename Pair<S>::V pack2(float a, float b);
template <>
__device__ __forceinline__ float2 pack2<float>(float a, float b) {
    return make_float2(a, b);
}
template <>
__device__ __forceinline__ __half2 pack2<__half>(float a, float b) {
    return __floats2half2_rn(a, b);
}
template <>
__device__ __forceinline__ __nv_bfloat162 pack2<__nv_bfloat16>(float a, float b) {
    return __floats2bfloat162_rn(a, b);
}

template <class S>
__device__ __forceinline__ void store_pair(S* out, size_t elem, S a, S b) {
    typename Pair<S>::V v;
    v.x = a;
    v.y = b;
    reinterpret_cast<typename Pair<S>::V*>(out)[elem] = v;
}

// both fields of the Q populations that stream into slot i (extended neighbour table)
template <int Q, class S, bool LOCAL>
__device__ __forceinline__ void load_field2(const S* __restrict__ g, const LatticeView& L, int i,
                                            typename Store<S>::T* v0, typename Store<S>::T* v1) {
    constexpr int R = Lat<Q>::REST;
    using V = typename Pair<S>::V;
    const V* gp = reinterpret_cast<const V*>(g);
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        elem_t e;
        if (q == R || LOCAL) {
            e = static_cast<elem_t>(q) * static_cast<elem_t>(L.nf_pad) + static_cast<elem_t>(i);
        } else {
            const int y = ld_table(L.nbr + static_cast<size_t>(Lat<Q>::rev(q)) * L.nf_pad + i);
            e = pull_elem<Q>(L, q, y, i);
        }
        const V p = gp[e];
        v0[q] = static_cast<typename Store<S>::T>(p.x);
        v1[q] = static_cast<typename Store<S>::T>(p.y);
    }
}

// load_field2 from the table entries e[q] = nbr[q][i] already in registers (the
// colour gradient reads the same entries: the pull along c_q takes e[rev q])
template <int Q, class S, bool LOCAL>
__device__ __forceinline__ void load_field2_e(const S* __restrict__ g, const LatticeView& L, int i, const int* e,
                                              typename Store<S>::T* v0, typename Store<S>::T* v1) {
    constexpr int R = Lat<Q>::REST;
    using V = typename Pair<S>::V;
    const V* gp = reinterpret_cast<const V*>(g);
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const elem_t el = (q == R || LOCAL)
                              ? static_cast<elem_t>(q) * static_cast<elem_t>(L.nf_pad) + static_cast<elem_t>(i)
                              : pull_elem<Q>(L, q, e[Lat<Q>::rev(q)], i);
        const V p = gp[el];
        v0[q] = static_cast<typename Store<S>::T>(p.x);
        v1[q] = static_cast<typename Store<S>::T>(p.y);
    }
}

template <int Q, class S, bool LOCAL>
__device__ __forceinline__ void load_rk(const S* __restrict__ g, const LatticeView& L, int i, double* f0,
                                        double* f1, double rho_ref, double inv_scale) {
    using T = typename Store<S>::T;
    T v0[Q], v1[Q];
    load_field2<Q, S, LOCAL>(g, L, i, v0, v1);
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        if constexpr (Store<S>::shifted) {
            const double w = Lat<Q>::w(q);
            const double ft = w * (rho_ref + static_cast<double>(Store<S>::val(v0[q])) * inv_scale);
            const double dc = w * (static_cast<double>(Store<S>::val(v1[q])) * inv_scale);
            f0[q] = 0.5 * (ft + dc);
            f1[q] = 0.5 * (ft - dc);
        } else if constexpr (std::is_same<S, int64_t>::value) {  // int64 fixed-point state
            f0[q] = fx::store_f64(v0[q]);
            f1[q] = fx::store_f64(v1[q]);
        } else {
            f0[q] = v0[q];
            f1[q] = v1[q];
        }
    }
}

// ---------------------------------------------------------------------------
// k_single_pair: the single-phase step on the shifted formats with two adjacent
// slots per thread (2t, 2t + 1): the table is read as one int2 per direction,
// the rest population as one pair and the results stored as one pair per
// direction (half2 / bfloat162 / float2), about a third fewer memory
// instructions per node than one slot per thread.  The steps after the first.
// A thread whose second slot is padding (nf odd) computes it from element 0
// (the padding rows of the pull table are 0) and stores it into the padding.
// ---------------------------------------------------------------------------
// resident blocks per SM asked of the register allocator (256^3, ms per step, one slot
// per thread / two at 2, 3, 4 blocks: FP16 0.1699 / 0.1797, 0.1579, 0.1556; FP32
// 0.2212 / 0.2256, 0.2194, 0.2231)
#ifndef BCLBM_PAIR_BLOCK
#define BCLBM_PAIR_BLOCK 256
#endif
template <class S>
constexpr int pair_min_blocks() {
    return (sizeof(S) == 2 ? 4 : 3) * (256 / BCLBM_PAIR_BLOCK);
}

template <int Q, class S, bool TRT>
__global__ void __launch_bounds__(BCLBM_PAIR_BLOCK, pair_min_blocks<S>()) k_single_pair(StepArgs a) {
    constexpr int D = Lat<Q>::D, R = Lat<Q>::REST;
    const int i = 2 * (blockIdx.x * blockDim.x + threadIdx.x);
    if (i >= a.L.nf) return;
    using T = typename Store<S>::T;
    using V = typename Pair<S>::V;
    const S* __restrict__ g = static_cast<const S*>(a.src);
    const size_t pad = static_cast<size_t>(a.L.nf_pad);
    T va[Q], vb[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        if (q == R) {
            const V p = *reinterpret_cast<const V*>(g + static_cast<size_t>(R) * pad + i);
            va[q] = p.x;
            vb[q] = p.y;
        } else {
            const int2 e = __ldg(reinterpret_cast<const int2*>(a.L.pull + static_cast<size_t>(q) * pad + i));
            va[q] = ld_pop(g + e.x);
            vb[q] = ld_pop(g + e.y);
        }
    }
    const float F[3] = {a.params->forcef[0], a.params->forcef[1], a.params->forcef[2]};
    const float oms = a.f_tau_inv, oma = TRT ? a.f_tauA_inv : a.f_tau_inv;
    const float tsf = a.f_tf, taf = TRT ? a.f_taf : a.f_tf;
    float fa[Q], fb[Q], rhoa, rhob, vela[3], velb[3];
    decode<Q, S, float>(va, fa, a.f_inv_scale);
    decode<Q, S, float>(vb, fb, a.f_inv_scale);
    collide_fast<Q, float, TRT, true>(fa, F, oms, oma, tsf, taf, a.f_rho_ref, rhoa, vela);
    collide_fast<Q, float, TRT, true>(fb, F, oms, oma, tsf, taf, a.f_rho_ref, rhob, velb);
    if (a.rho_out != nullptr) {
        a.rho_out[i] = rhoa;
        a.rho_out[i + 1] = rhob;
#pragma unroll
        for (int d = 0; d < D; ++d) {
            a.vel_out[static_cast<size_t>(d) * pad + i] = vela[d];
            a.vel_out[static_cast<size_t>(d) * pad + i + 1] = velb[d];
        }
    }
    S* out = static_cast<S*>(a.dst);
    const float scale = a.f_scale;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const float s = scale / static_cast<float>(Lat<Q>::w(q));
        *reinterpret_cast<V*>(out + static_cast<size_t>(q) * pad + i) = pack2<S>(fa[q] * s, fb[q] * s);
    }
}

// PASS 1 (main_TWOPHASE.cpp:238-246): densities, colour field; SUMS writes the
// per-block sums of qSumC(f0 + f1)[0] for the flux controller (:292-298) and,
// for shifted storage, of the node totals sum_q (f0 + f1) - rho_ref and
// sum_q (f0 - f1) for the mass-drift correction.
// resident blocks per SM asked of the register allocator by the shifted two-phase passes
// (192^3 pack, F16 / F32 MLUPS: no hint 7,935 / 7,026 (4 and 3 blocks); 4 + 4: 8,532 / 7,810;
// 5 + 4: 8,170 / 7,503; 6 + 4: 7,754 / 7,055; 5 + 3: 8,225 / 6,882)
#ifndef BCLBM_RK_DENS_MINB
#define BCLBM_RK_DENS_MINB 4
#endif
#ifndef BCLBM_RK_COLL_MINB
#define BCLBM_RK_COLL_MINB 4
#endif

// the int64 fixed-point state's density pass (exact integer sums, one FP64 division):
// unbounded registers measured best (192^3, ms per pass: 0.173 against 0.191 at 4 and
// 0.267 at 5 resident blocks); its collide pass at 2 blocks (0.773 ms against 0.835 at 3
// and 1.065 at 1)
#ifndef BCLBM_RK_FX_DENS_MINB
#define BCLBM_RK_FX_DENS_MINB 1
#endif
template <class S>
constexpr int rk_density_min_blocks() {
    return Store<S>::shifted ? BCLBM_RK_DENS_MINB : (std::is_same<S, int64_t>::value ? BCLBM_RK_FX_DENS_MINB : 1);
}

template <int Q, class S, bool LOCAL, bool SUMS>
__global__ void __launch_bounds__(kBlock, rk_density_min_blocks<S>()) k_rk_density(StepArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double fx = 0.0;
    float fxf = 0.f, mt = 0.f, mc = 0.f;
    if (i < a.L.nf) {
        using T = typename Store<S>::T;
        const S* g = static_cast<const S*>(a.src);
        if constexpr (std::is_same<S, int64_t>::value) {
            // int64 fixed-point state: exact sums, the colour formed in FP64 as the
            // reference forms it (this pass is bound by its loads) and kept in fixed
            // point for the gradient of the collision pass; |colour| >= 2 is out of
            // that pass's range
            T v0[Q], v1[Q];
            load_field2<Q, S, LOCAL>(g, a.L, i, v0, v1);
            int64_t r0 = 0, r1 = 0, jx = 0;
#pragma unroll
            for (int q = 0; q < Q; ++q) {
                r0 += v0[q];
                r1 += v1[q];
                if (SUMS) jx += Lat<Q>::cx(q) * (v0[q] + v1[q]);
            }
            unsigned emax = 0;
            a.cgx[i] = fx::load_f64_hw(fx::store_f64(r0 - r1) / fx::store_f64(r0 + r1), emax);
            if (emax >= (1024u << 20)) atomicOr(a.fx_flag, 1);
            if (SUMS) fx = fx::store_f64(jx);
        } else if constexpr (!Store<S>::shifted) {
            T v0[Q], v1[Q];
            load_field2<Q, S, LOCAL>(g, a.L, i, v0, v1);
            double r0 = 0.0, r1 = 0.0;
#pragma unroll
            for (int q = 0; q < Q; ++q) r0 += v0[q];
#pragma unroll
            for (int q = 0; q < Q; ++q) r1 += v1[q];
            a.cg[i] = (r0 - r1) / (r0 + r1);
            if (SUMS) {
                double ft[Q], j[3];
#pragma unroll
                for (int q = 0; q < Q; ++q) ft[q] = v0[q] + v1[q];
                qsumc_ref<Q>(ft, j);
                fx = j[0];
            }
        } else {
            T v0[Q], v1[Q];
            load_field2<Q, S, LOCAL>(g, a.L, i, v0, v1);
            float rs = 0.f, dr = 0.f, jx = 0.f;
            const float isc = a.f_inv_scale;
#pragma unroll
            for (int q = 0; q < Q; ++q) {
                const float w = static_cast<float>(Lat<Q>::w(q));
                const float t = Store<S>::val(v0[q]) * (w * isc);
                rs += t;
                dr += Store<S>::val(v1[q]) * (w * isc);
                jx += Lat<Q>::cx(q) * t;
            }
            const float rho = a.f_rho_ref + rs;
            a.cgf[i] = dr / rho;
            fxf = jx;
            mt = rs;
            mc = dr;
        }
    }
    if constexpr (SUMS) {
        if constexpr (Store<S>::shifted) {
            float vals[3] = {fxf, mt, mc};
            block_reduce_store_f32<3>(vals, a.partials);
        } else {
            double vals[3] = {fx, 0.0, 0.0};
            block_reduce_store<3>(vals, a.partials, false);
        }
    }
}

// After the PASS 1 sums (sum[0] flux, sum[1] total deviation, sum[2] colour
// difference, over n fluid nodes): the flux controller's force and the
// mass-drift correction of this step.
__global__ void k_rk_fix(const double* sum, double n, double rho_ref, double mom_x, int flux, int fix,
                         DevParams* params);

// Flux controller (main_TWOPHASE.cpp:301-308): force_x = 2 (mom_x - mean).
__global__ void k_flux_force(const double* sum, double inv_n, double mom_x, DevParams* params);

// PASS 2 (main_TWOPHASE.cpp:312-376): RK collision, perturbation and
// recolouring of F64 populations, in the reference's expression order.  FMA
// tells the instantiations apart: false in the -fmad=false unit (rounding as the
// reference), true in the contracting unit (BCLBM_FLAG_FP64_FMA).
template <int Q, bool LOCAL, bool FMA>
__global__ void __launch_bounds__(kBlock) k_rk_collide_f64(StepArgs a) {
    const bool MACROS = a.rho_out != nullptr;
    constexpr int D = Lat<Q>::D, R = Lat<Q>::REST;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.L.nf) return;
    double f0[Q], f1[Q];
    load_rk<Q, double, LOCAL>(static_cast<const double*>(a.src), a.L, i, f0, f1, a.rho_ref, a.inv_scale);
    // colour at the downstream neighbours (grad, LButilities.h:12-22)
    double sc[Q];
#pragma unroll
    for (int q = 0; q < Q - 1; ++q) sc[q] = a.cg[__ldg(a.L.nbr + static_cast<size_t>(q) * a.L.nf_pad + i)];
    sc[R] = a.cg[i];
    const double F[3] = {a.params->force[0], a.params->force[1], a.params->force[2]};
    double ft[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) ft[q] = f0[q] + f1[q];
    double rho0 = 0.0, rho1 = 0.0;  // pass-1 densities, recomputed from the same populations
#pragma unroll
    for (int q = 0; q < Q; ++q) rho0 += f0[q];
#pragma unroll
    for (int q = 0; q < Q; ++q) rho1 += f1[q];
    const double rho = rho0 + rho1;
    double j[3] = {0.0, 0.0, 0.0}, vel[3] = {0.0, 0.0, 0.0};
    qsumc_ref<Q>(ft, j);
    // FMA: the divisions by the same value become one reciprocal and products
    // (an IEEE FP64 division is a dozen FP64-pipe instructions on this part);
    // the reference-order kernel keeps every division
    const double inv_rho = FMA ? 1.0 / rho : 0.0;
#pragma unroll
    for (int d = 0; d < D; ++d) vel[d] = FMA ? (j[d] + 0.5 * F[d]) * inv_rho : (j[d] + 0.5 * F[d]) / rho;
    const double q0 = 0.0, q1 = 0.0;  // mass sources are zero (main_TWOPHASE.cpp:132-136)
    rho0 += 0.5 * q0;
    rho1 += 0.5 * q1;
    const double tau = 3.0 * rho / (rho0 * a.nu0inv + rho1 * a.nu1inv) + 0.5;
    const double uu = dot_ref<Q>(vel, vel);
    double cu[Q], cF[Q];
    cdotall_ref<Q>(vel, cu);
    const double tau_inv = 1.0 / tau;
    const double uF = dot_ref<Q>(vel, F);
    cdotall_ref<Q>(F, cF);
    const double tf = FMA ? 1 - 0.5 * tau_inv : (1 - 0.5 / tau);
    double G[3] = {0.0, 0.0, 0.0};
    grad_ref<Q>(sc, G);
    const double cgn = sqrt(dot_ref<Q>(G, G));
    const double gs = 1.0 / (cgn + static_cast<double>(cgn < 2.220446049250313080847e-16));
#pragma unroll
    for (int d = 0; d < D; ++d) G[d] *= gs;
    double cn[Q];
    cdotall_ref<Q>(G, cn);
    // calcDeltaOmegaST (LBcollision2phase.h:11), calcDeltaOmegaRC (LBcollision2phase.h:74)
    const double af = FMA ? 1.125 * cgn * a.sigma * tau_inv : 1.125 * cgn * a.sigma / tau;
    const double rfb = FMA ? a.beta * rho0 * rho1 * inv_rho : a.beta * rho0 * rho1 / rho;
    const double c0 = FMA ? rho0 * inv_rho : (rho0 / rho);
    const double c1 = FMA ? rho1 * inv_rho : (rho1 / rho);
    if (MACROS) {
        a.rho_out[i] = rho0;
        a.rho_out[static_cast<size_t>(a.L.nf_pad) + i] = rho1;
#pragma unroll
        for (int d = 0; d < D; ++d) a.vel_out[static_cast<size_t>(d) * a.L.nf_pad + i] = vel[d];
    }
    double* out = static_cast<double*>(a.dst);
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const double w = Lat<Q>::w(q);
        const double om = -tau_inv * (ft[q] - rho * w * (1.0 + 3.0 * cu[q] + 4.5 * (cu[q] * cu[q] - C2 * uu)));
        const double dF = w * tf * (3.0 * cF[q] + 9.0 * (cF[q] * cu[q] - C2 * uF));
        const double e = (1.0 + 3.0 * cu[q] + 4.5 * (cu[q] * cu[q] - C2 * uu));
        const double dQ0 = tf * q0 * w * e;
        const double dQ1 = tf * q1 * w * e;
        const double dST = (q == R) ? -af * Lat<Q>::B(q) : af * (w * cn[q] * cn[q] - Lat<Q>::B(q));
        const double dRC = (q == R)  ? 0.0
                           : FMA     ? rfb * w * cn[q] * (Lat<Q>::wclass(q) == 1 ? 1.0 : 0.70710678118654752440)
                                     : rfb * w * cn[q] / cnorm_ref(Lat<Q>::wclass(q));
        store_pair(out, static_cast<size_t>(q) * a.L.nf_pad + i, c0 * (ft[q] + om + dF + dST) + dRC + dQ0,
                   c1 * (ft[q] + om + dF + dST) - dRC + dQ1);
    }
}

// PASS 2 for the shifted formats, FP32 arithmetic on (total deviation ft',
// colour difference dc).  With X_q the reference's
// fTot + omegaBGK + deltaOmegaF + deltaOmegaST, the two outputs
// c0 X + RC and c1 X - RC become  ft'_post = X - w rho_ref  and
// dc_post = (c0 - c1) X + 2 RC.
// FUSED (BCLBM_FLAG_LAGGED_COLOUR): PASS 1 and PASS 2 in one: the neighbours'
// colours come from the previous step's field (a.cgf), the node's own colour goes
// to this step's (a.cgf_out), and sums (when not null) receives the PASS 1 sums of
// the node (flux, total deviation, colour difference) at sums[0], sums[kBlock],
// sums[2 kBlock]: a shared-memory column, written as soon as they are known
// (192^3, MLUPS with the sums in registers to the end / in shared memory: FP16
// 16,291 / 16,615, BF16 16,095 / 16,457, FP32 13,230 / 13,813).
template <int Q, class S, bool LOCAL, bool FUSED>
__device__ __forceinline__ void rk_collide_shift_node(const StepArgs& a, int i, float* sums) {
    const bool MACROS = a.rho_out != nullptr;
    constexpr int D = Lat<Q>::D, R = Lat<Q>::REST;
    using T = typename Store<S>::T;
    const S* g = static_cast<const S*>(a.src);
    int e[Q - 1];  // each table entry once, for the pull and the colour gradient
#pragma unroll
    for (int q = 0; q < Q - 1; ++q) e[q] = ld_table(a.L.nbr + static_cast<size_t>(q) * a.L.nf_pad + i);
    T v0[Q], v1[Q];
    load_field2_e<Q, S, LOCAL>(g, a.L, i, e, v0, v1);
    float sc[Q];
#pragma unroll
    for (int q = 0; q < Q - 1; ++q) sc[q] = a.cgf[e[q]];
    sc[R] = 0.f;
    const float isc = a.f_inv_scale;
    float ft[Q], dc[Q];
    float rs = 0.f, dr = 0.f, j[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const float ws = static_cast<float>(Lat<Q>::w(q)) * isc;
        ft[q] = Store<S>::val(v0[q]) * ws;
        dc[q] = Store<S>::val(v1[q]) * ws;
        rs += ft[q];
        dr += dc[q];
        j[0] += Lat<Q>::cx(q) * ft[q];
        j[1] += Lat<Q>::cy(q) * ft[q];
        j[2] += Lat<Q>::cz(q) * ft[q];
    }
    if constexpr (FUSED) {
        // to shared memory at once (stride kBlock), so they hold no registers below
        if (sums != nullptr) {
            sums[0] = j[0];
            sums[kBlock] = rs;
            sums[2 * kBlock] = dr;
        }
    }
    const float F[3] = {a.params->forcef[0], a.params->forcef[1], a.params->forcef[2]};
    const float rho_ref = a.f_rho_ref;
    const float rho = rho_ref + rs;
    const float inv = 1.f / rho;
    const float rho0 = 0.5f * (rho + dr), rho1 = 0.5f * (rho - dr);
    float u[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) u[d] = (d < D) ? (j[d] + 0.5f * F[d]) * inv : 0.f;
    const float om = 1.f / (3.f * rho / (rho0 * a.f_nu0inv + rho1 * a.f_nu1inv) + 0.5f);
    const float tf = 1.f - 0.5f * om;
    const float uu = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
    const float uF = u[0] * F[0] + u[1] * F[1] + u[2] * F[2];
    float G[3] = {0.f, 0.f, 0.f};
    {
        constexpr float ga = static_cast<float>(Lat<Q>::w1c2inv), gb = static_cast<float>(Lat<Q>::w2c2inv);
#pragma unroll
        for (int q = 0; q < Q - 1; ++q) {
            const float wq = Lat<Q>::wclass(q) == 1 ? ga : gb;
            G[0] += (wq * Lat<Q>::cx(q)) * sc[q];
            G[1] += (wq * Lat<Q>::cy(q)) * sc[q];
            G[2] += (wq * Lat<Q>::cz(q)) * sc[q];
        }
    }
    const float cgn = sqrtf(G[0] * G[0] + G[1] * G[1] + G[2] * G[2]);
    const float gs = 1.f / (cgn + (cgn < 1.1920929e-07f ? 1.f : 0.f));
    const float af = 1.125f * cgn * a.f_sigma * om;
    const float rfb = a.f_beta * rho0 * rho1 * inv;
    const float dcf = dr * inv;  // c0 - c1
    const float sc_out = a.f_scale;
    // mass-drift correction: + w_q delta to every population of the node
    const float fix_t = a.params->mass_fixf[0] * sc_out, fix_c = a.params->mass_fixf[1] * sc_out;
    S* out = static_cast<S*>(a.dst);
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const float w = static_cast<float>(Lat<Q>::w(q));
        const float cu = Lat<Q>::cx(q) * u[0] + Lat<Q>::cy(q) * u[1] + Lat<Q>::cz(q) * u[2];
        const float cF = Lat<Q>::cx(q) * F[0] + Lat<Q>::cy(q) * F[1] + Lat<Q>::cz(q) * F[2];
        const float cn = (Lat<Q>::cx(q) * G[0] + Lat<Q>::cy(q) * G[1] + Lat<Q>::cz(q) * G[2]) * gs;
        // deviation of the equilibrium from w rho_ref
        const float feq = w * (rs + rho * (3.f * cu + 4.5f * cu * cu - 1.5f * uu));
        const float dST = (q == R) ? -af * static_cast<float>(Lat<Q>::B(q))
                                   : af * (w * cn * cn - static_cast<float>(Lat<Q>::B(q)));
        const float Xd = ft[q] - om * (ft[q] - feq) + w * tf * (3.f * cF + 9.f * cF * cu - 3.f * uF) + dST;
        const float dRC = (q == R) ? 0.f : rfb * w * cn * (Lat<Q>::wclass(q) == 1 ? 1.f : 0.70710678118654752f);
        const float X = Xd + w * rho_ref;
        const float s = sc_out / w;
        reinterpret_cast<typename Pair<S>::V*>(out)[static_cast<size_t>(q) * a.L.nf_pad + i] =
            pack2<S>(Xd * s + fix_t, (dcf * X + 2.f * dRC) * s + fix_c);
    }
    if (MACROS) {
        a.rho_out[i] = rho0;
        a.rho_out[static_cast<size_t>(a.L.nf_pad) + i] = rho1;
#pragma unroll
        for (int d = 0; d < D; ++d) a.vel_out[static_cast<size_t>(d) * a.L.nf_pad + i] = u[d];
    }
    if constexpr (FUSED) {
        a.cgf_out[i] = dcf;
    }
}

// FP32 storage takes 3 resident blocks per SM (192^3: 8,908 -> 9,284 MLUPS against 4;
// FP16 11,615 at 4, 11,078 at 3, 10,738 at 5)
// threads per block (192^3, MLUPS at 256 / 128 / 64 with the same resident warps:
// FP16 11,914 / 11,894 / 11,825, BF16 12,096 / 11,807 / 11,710, FP32 9,521 / 9,588 / 9,586)
#ifndef BCLBM_RK_COLL_BLOCK
#define BCLBM_RK_COLL_BLOCK 256
#endif
template <class S>
constexpr int rk_collide_min_blocks() {
    return (sizeof(S) == 2 ? BCLBM_RK_COLL_MINB : 3) * (256 / BCLBM_RK_COLL_BLOCK);
}

template <int Q, class S, bool LOCAL>
__global__ void __launch_bounds__(BCLBM_RK_COLL_BLOCK, rk_collide_min_blocks<S>()) k_rk_collide_shift(StepArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.L.nf) return;
    rk_collide_shift_node<Q, S, LOCAL, false>(a, i, nullptr);
}

// One pass per step (BCLBM_FLAG_LAGGED_COLOUR), after a step of both passes; SUMS
// writes the per-block sums that k_rk_fix turns into the next step's force and
// mass correction.
// resident blocks per SM asked of the register allocator (192^3, MLUPS at 3 / 4 / 5
// blocks: FP16 14,750 / 15,413 / 13,436, FP32 12,974 / 12,474 / 10,659)
// (FP32 after the shared-memory sums and 32-bit element numbers: 13,835 at 3, 12,990 at 4)
#ifndef BCLBM_RK_FUSED_MINB_F32
#define BCLBM_RK_FUSED_MINB_F32 3
#endif
template <class S>
constexpr int fused_min_blocks() {
    return sizeof(S) == 2 ? 4 : BCLBM_RK_FUSED_MINB_F32;
}
template <int Q, class S, bool SUMS>
__global__ void __launch_bounds__(kBlock, fused_min_blocks<S>()) k_rk_fused_shift(StepArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if constexpr (SUMS) {
        // the node's flux, total deviation and colour difference, [3][kBlock]
        __shared__ float sh[3 * kBlock];
        float* mine = sh + threadIdx.x;
        if (i < a.L.nf) {
            rk_collide_shift_node<Q, S, false, true>(a, i, mine);
        } else {
            mine[0] = mine[kBlock] = mine[2 * kBlock] = 0.f;
        }
        block_sums_from_shared<3>(sh, a.partials);
    } else {
        if (i < a.L.nf) rk_collide_shift_node<Q, S, false, true>(a, i, nullptr);
    }
}

// PASS 2 of the default FP64 two-phase step, on the int64 fixed-point state
// (main_TWOPHASE.cpp:312-376, the expressions of k_rk_collide_f64 regrouped by
// direction pairs).  Every term is a 64-bit fixed-point product: the FP64 pipe
// issues one warp instruction per 16 cycles, so the per-node scalars stay off
// it too.
//   colour gradient: the exact integer sum of the fixed-point colours
//     (DXQY::grad with the weights' common factor 1/12 taken out);
//   |G| and G / |G|: the gradient scaled by a power of two to [1/2, 1), an FP32
//     reciprocal square root and two Newton steps in fixed point, and the
//     reference's |G| < eps case (G / (|G| + 1) = G to 2^-104);
//   c0 = rho0 / rho: 1/rho times rho0 and one correction by its residual;
//   recolouring amplitude beta rho0 rho1 / rho = beta c0 rho1;
//   relaxation rate oms = Dn / (3 rho + Dn / 2): a per-handle constant when the
//     two viscosities are equal, else formed in FP64 from the exact densities.
// With ft = f0 + f1, P / M the pair sums and j = sum ft c + F/2 (exact):
//   X_q = (1 - oms) ft_q + oms feq_q + dF_q + dST_q,
//   out0 = c0 X_q + dRC_q,  out1 = X_q - out0   (c1 = 1 - c0),
// where oms feq_q = oms w (rho - 1.5 j.u) + 4.5 oms w (c.j)(c.u) +- 3 oms w (c.j).
#ifndef BCLBM_RK_FX_MINB
#define BCLBM_RK_FX_MINB 2
#endif
#ifndef BCLBM_RK_FX_BLOCK
#define BCLBM_RK_FX_BLOCK 256
#endif
template <int Q, bool LOCAL>
__global__ void __launch_bounds__(BCLBM_RK_FX_BLOCK, BCLBM_RK_FX_MINB) k_rk_collide_fx(StepArgs a) {
    const bool MACROS = a.rho_out != nullptr;
    constexpr int D = Lat<Q>::D, R = Lat<Q>::REST, NP = Lat<Q>::NP;
    constexpr int SH1 = Q == 19 ? 1 : 2;  // w_axis / w_diag
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.L.nf) return;
    const size_t pad = static_cast<size_t>(a.L.nf_pad);
    int e[Q - 1];  // each table entry once, for the pull and the colour gradient
#pragma unroll
    for (int q = 0; q < Q - 1; ++q) e[q] = ld_table(a.L.nbr + static_cast<size_t>(q) * pad + i);
    int64_t X0[Q], X1[Q];
    load_field2_e<Q, int64_t, LOCAL>(static_cast<const int64_t*>(a.src), a.L, i, e, X0, X1);
    // colour at the downstream neighbours (grad, LButilities.h:12-22), a quarter
    // of it so that the gradient sums stay inside the range (|colour| < 2)
    int64_t sc[Q - 1];
#pragma unroll
    for (int q = 0; q < Q - 1; ++q) sc[q] = a.cgx[e[q]] >> 2;
    int ovf = 0;
    int64_t rho0 = 0, rho1 = 0, ft[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        rho0 += X0[q];
        rho1 += X1[q];
        ft[q] = X0[q] + X1[q];
    }
    const int64_t rho = rho0 + rho1;
    {
        int t = 0;  // sum_q |ft_q| below 8 (see fx::collide_to)
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            const int h = static_cast<int>(ft[q] >> 56);
            t += h < 0 ? -h : h;
        }
        if (t > 108) ovf = 1;
    }
    // the body force (the flux controller may change it every step)
    int64_t Ff[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) Ff[d] = a.params->forcex[d];
    int64_t j[3] = {0, 0, 0};
#pragma unroll
    for (int k = 0; k < NP; ++k) {
        const int64_t Mk = ft[k] - ft[k + NP];
        if (Lat<Q>::cx(k) > 0) j[0] += Mk;
        if (Lat<Q>::cx(k) < 0) j[0] -= Mk;
        if (Lat<Q>::cy(k) > 0) j[1] += Mk;
        if (Lat<Q>::cy(k) < 0) j[1] -= Mk;
        if (D == 3 && Lat<Q>::cz(k) > 0) j[2] += Mk;
        if (D == 3 && Lat<Q>::cz(k) < 0) j[2] -= Mk;
    }
#pragma unroll
    for (int d = 0; d < D; ++d) j[d] += Ff[d] >> 1;
    // 1 / rho: FP32 estimate, one Newton step in fixed point
    const float rf = static_cast<float>(rho) * 8.67361737988403547e-19f;  // 2^-60
    if (!(rf > 0.15f)) ovf = 1;
    int64_t inv = static_cast<int64_t>(__frcp_rn(rf) * 1.152921504606846976e18f);
    inv = fx::mul_uu(inv, 2 * fx::ONE - fx::mul_uu(rho, inv));
    int64_t u[3] = {0, 0, 0};
#pragma unroll
    for (int d = 0; d < D; ++d) u[d] = fx::mul_su(j[d], inv);
    const fx::RkConsts& K = a.fxr;
    // colour fraction and recolouring amplitude
    int64_t c0 = fx::mul_su(rho0, inv);
    c0 += fx::mul_su(rho0 - fx::mul_su(c0, rho), inv);
    const int64_t rfb = fx::mul_ss(fx::mul_ss(c0, rho1), K.beta);
    // colour gradient G = T / 3, T = sum_q (36 w_q) c_q sc_q
    int64_t T[3] = {0, 0, 0};
#pragma unroll
    for (int q = 0; q < Q - 1; ++q) {
        const int m = Lat<Q>::wclass(q) == 1 ? (Q == 19 ? 2 : 4) : 1;
        if (Lat<Q>::cx(q) != 0) T[0] += (Lat<Q>::cx(q) * m) * sc[q];
        if (Lat<Q>::cy(q) != 0) T[1] += (Lat<Q>::cy(q) * m) * sc[q];
        if (D == 3 && Lat<Q>::cz(q) != 0) T[2] += (Lat<Q>::cz(q) * m) * sc[q];
    }
    // |G| and n = G / |G| (the reference's gs = 1 / (|G| + (|G| < eps)))
    int64_t n[3] = {0, 0, 0}, cgn = 0;
    fx::unit_normal<D>(T, K.third, n, cgn);
    // relaxation rate and the products that carry it
    int64_t oms, omsw2, k45, K3, tf3w2, sto;
    if (K.uniform) {
        oms = K.oms;
        omsw2 = K.oms_w2;
        k45 = K.oms_k45;
        K3 = K.oms_k3;
        tf3w2 = K.tf3w2;
        sto = K.st_oms;
    } else {
        const double r0d = fx::store_f64(rho0), r1d = fx::store_f64(rho1), rd = fx::store_f64(rho);
        const double Dn = r0d * a.nu0inv + r1d * a.nu1inv;
        unsigned emax = 0;
        oms = fx::load_f64_hw(Dn / (3.0 * rd + 0.5 * Dn), emax);  // 1 / tau, tau = 3 rho / Dn + 0.5
        if (emax >= fx::kLoadEmaxLimit) ovf = 1;
        omsw2 = fx::mul_su(oms, K.w2);
        k45 = fx::mul_su(oms, K.w2_45);
        K3 = fx::mul_su(oms, K.w2_3);
        tf3w2 = fx::mul_su(fx::ONE - (oms >> 1), K.w2_3);
        sto = fx::mul_ss(oms, K.st);
    }
    const int64_t af = fx::mul_su(sto, cgn);  // 9/8 sigma oms |G|
    // the multipliers in [0, 1) in k form (fx::mul_sk): |1 - oms| / 2 (its sign applied to the
    // products: zero at tau = 1, as the reference's), oms w2, 4.5 oms w2, 3 oms w2, 3 w2 tf
    const int64_t hom = (fx::ONE - oms) >> 1;
    const bool hneg = hom < 0;
    const uint64_t hom_k = fx::kform(hneg ? -hom : hom), omsw2_k = fx::kform(omsw2), k45_k = fx::kform(k45),
                   K3_k = fx::kform(K3), tf3w2_k = fx::kform(tf3w2);
    int64_t ju = fx::mul_ss(j[0], u[0]) + fx::mul_ss(j[1], u[1]);
    if (D == 3) ju += fx::mul_ss(j[2], u[2]);
    const int64_t AB2 = fx::mul_sk(rho - (ju + (ju >> 1)), omsw2_k);  // oms w2 (rho - 1.5 j.u)
    int64_t u45[3] = {0, 0, 0};
#pragma unroll
    for (int d = 0; d < D; ++d) u45[d] = fx::mul_sk(u[d], k45_k);
    // force terms: -3 w2 tf u.F, and 3 w2 tf F_d (ka3 of a direction = c . g3, kf9 = 3 c . g3)
    int64_t uF = 0, g3[3] = {0, 0, 0};
#pragma unroll
    for (int d = 0; d < D; ++d)
        if (Ff[d] != 0) {
            uF += fx::mul_ss(u[d], Ff[d]);
            g3[d] = fx::mul_sk(Ff[d], tf3w2_k);
        }
    const int64_t K2 = -fx::mul_sk(uF, tf3w2_k);
    // surface tension af (w cn^2 - B) and recolouring rfb w cn / |c|
    const int64_t afw2 = fx::mul_ss(af, K.w2);
    const int64_t afB1 = fx::mul_ss(af, K.B[1]), afB2 = fx::mul_ss(af, K.B[2]), afB0 = fx::mul_ss(af, K.B[0]);
    const int64_t rfb1 = fx::mul_sk(rfb, K.w1_k), rfb2 = fx::mul_sk(rfb, K.w2s_k);
    // the colour split out0 = c0 X + dRC, out1 = X - out0 through the smaller fraction
    // m = min(c0, 1 - c0) in [0, 1/2] (a k-form multiplier; the other colour by difference)
    const bool sw = c0 > (fx::ONE >> 1);
    int64_t cm = sw ? fx::ONE - c0 : c0;
    cm = cm < 0 ? 0 : cm;
    const uint64_t cm_k = fx::kform(cm);
    auto by_class = [](int64_t v2, int c) -> int64_t {
        return c == 2 ? v2 : (c == 1 ? (v2 << SH1) : (Q == 19 ? (v2 << 3) + (v2 << 2) : (v2 << 4)));
    };
    int64_t* out = static_cast<int64_t*>(a.dst);
#pragma unroll
    for (int k = 0; k < NP; ++k) {
        const int c = Lat<Q>::wclass(k);
        const int cx = Lat<Q>::cx(k), cy = Lat<Q>::cy(k), cz = Lat<Q>::cz(k);
        const int64_t cj = cx * j[0] + cy * j[1] + cz * j[2];
        const int64_t cu45 = cx * u45[0] + cy * u45[1] + cz * u45[2];
        const int64_t cn = cx * n[0] + cy * n[1] + cz * n[2];
        const int64_t acn = cn < 0 ? -cn : cn;
        const int64_t cn2 = fx::mul_uu(acn, acn);
        const int64_t P = ft[k] + ft[k + NP], M = ft[k] - ft[k + NP];
        const int64_t sP = fx::mul_sk(P, hom_k), sM = fx::mul_sk(M, hom_k);
        int64_t Sv = (hneg ? -sP : sP) + by_class(AB2 + fx::mul_ss(cj, cu45) + K2 + fx::mul_su(afw2, cn2), c) -
                     (c == 1 ? afB1 : afB2);
        const int64_t ka3 = by_class(cx * g3[0] + cy * g3[1] + cz * g3[2], c);
        if (ka3 != 0) {  // 9 w tf (c.F)(c.u) for the directions with c.F != 0 (uniform over the grid)
            const int64_t cu = cx * u[0] + cy * u[1] + cz * u[2];
            Sv += fx::mul_ss(3 * ka3, cu);
        }
        const int64_t Av = (hneg ? -sM : sM) + by_class(fx::mul_sk(cj, K3_k), c) + ka3;
        const int64_t Xk = Sv + Av, Xr = Sv - Av;
        const int64_t dRC = fx::mul_ss(cn, c == 1 ? rfb1 : rfb2);
        const int64_t pk = fx::mul_sk(Xk, cm_k), pr = fx::mul_sk(Xr, cm_k);
        const int64_t o0k = (sw ? Xk - pk : pk) + dRC, o0r = (sw ? Xr - pr : pr) - dRC;
        store_pair(out, static_cast<size_t>(k) * pad + i, o0k, Xk - o0k);
        store_pair(out, static_cast<size_t>(k + NP) * pad + i, o0r, Xr - o0r);
    }
    {
        const int64_t XR = ft[R] - fx::mul_su(ft[R], oms) + by_class(AB2 + K2, 0) - afB0;
        const int64_t pR = fx::mul_sk(XR, cm_k);
        const int64_t o0 = sw ? XR - pR : pR;
        store_pair(out, static_cast<size_t>(R) * pad + i, o0, XR - o0);
    }
    if (MACROS) {
        a.rho_out[i] = fx::store_f64(rho0);
        a.rho_out[pad + i] = fx::store_f64(rho1);
#pragma unroll
        for (int d = 0; d < D; ++d) a.vel_out[static_cast<size_t>(d) * pad + i] = fx::store_f64(u[d]);
    }
    if (ovf) atomicOr(a.fx_flag, 1);
}

// ---------------------------------------------------------------------------
// k_gather: the reference's f (one pull of G, or the state itself when LOCAL),
// decoded to FP64 and written in reference AoS order [bulk index][field][q].
// ---------------------------------------------------------------------------
template <int Q, class S, int NF, bool LOCAL>
__global__ void __launch_bounds__(kBlock) k_gather(StepArgs a, const int32_t* __restrict__ slot_bulk,
                                                   double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.L.nf) return;
    const size_t b = static_cast<size_t>(slot_bulk[i]);
    const S* g = static_cast<const S*>(a.src);
    if constexpr (NF == 1) {
        using T = typename Store<S>::T;
        T v[Q];
        load_field<Q, S, LOCAL, true>(g, a.L, i, v);
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            double f;
            if constexpr (Store<S>::shifted)
                f = Lat<Q>::w(q) * (a.rho_ref + static_cast<double>(Store<S>::val(v[q])) * a.inv_scale);
            else
                f = Store<S>::val(v[q]);
            out[b * Q + q] = f;
        }
    } else {
        double f0[Q], f1[Q];
        load_rk<Q, S, LOCAL>(g, a.L, i, f0, f1, a.rho_ref, a.inv_scale);
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            out[b * 2 * Q + q] = f0[q];
            out[b * 2 * Q + Q + q] = f1[q];
        }
    }
}

// k_moments: per-block FP64 sums over the reference's f of
// [mass0, mass1, fc_x, fc_y, fc_z, max|f|(last)]; a NaN or Inf population turns
// max|f| into +Inf.  The single-field path works on direction pairs
// (P = f_q + f_rq, M = f_q - f_rq): mass = f_rest + sum P, fc = sum c M, about
// 40 FP64 operations per node.  For the shifted formats the sums are taken over
// the stored deviations (exact in FP64) and scaled by w_q / scale afterwards, per
// weight class; max |f| and the finite check are done on the integer / FP32 side.
template <int Q, class S, int NF, bool LOCAL>
__device__ __forceinline__ void moments_node(const StepArgs& a, int i, double* vals) {
    constexpr int D = Lat<Q>::D, NP = Lat<Q>::NP, R = Lat<Q>::REST;
    {
        const S* g = static_cast<const S*>(a.src);
        if constexpr (NF == 1) {
            using T = typename Store<S>::T;
            T v[Q];
            load_field<Q, S, LOCAL, true>(g, a.L, i, v);
            double x[Q];
            float mx = 0.f;
            bool bad = false;
#pragma unroll
            for (int q = 0; q < Q; ++q) {
                if constexpr (Store<S>::shifted) {
                    const float fv = Store<S>::val(v[q]);
                    x[q] = static_cast<double>(fv);
                    const float fq = static_cast<float>(Lat<Q>::w(q)) * (a.f_rho_ref + fv * a.f_inv_scale);
                    bad |= !(fabsf(fq) < CUDART_INF_F);
                    mx = fmaxf(mx, fabsf(fq));
                } else {
                    x[q] = Store<S>::val(v[q]);
                }
            }
            // sums per weight class of P (mass) and signed sums of M (momentum)
            double pc[3] = {0.0, 0.0, 0.0}, jc[3][3] = {{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}};
#pragma unroll
            for (int k = 0; k < NP; ++k) {
                const int c = Store<S>::shifted ? Lat<Q>::wclass(k) : 1;
                const double P = x[k] + x[k + NP], M = x[k] - x[k + NP];
                pc[c] += P;
                if (Lat<Q>::cx(k) > 0) jc[c][0] += M;
                if (Lat<Q>::cx(k) < 0) jc[c][0] -= M;
                if (Lat<Q>::cy(k) > 0) jc[c][1] += M;
                if (Lat<Q>::cy(k) < 0) jc[c][1] -= M;
                if (D == 3 && Lat<Q>::cz(k) > 0) jc[c][2] += M;
                if (D == 3 && Lat<Q>::cz(k) < 0) jc[c][2] -= M;
            }
            if constexpr (Store<S>::shifted) {
                // f_q = w_q (rho_ref + d_q / scale): sum_q w_q = 1, sum_q w_q c_q = 0
                const double w1 = Lat<Q>::w(0), w2 = Lat<Q>::w(NP - 1), w0 = Lat<Q>::w(R);
                vals[0] = a.rho_ref + a.inv_scale * (w0 * x[R] + w1 * pc[1] + w2 * pc[2]);
#pragma unroll
                for (int d = 0; d < 3; ++d) vals[2 + d] = a.inv_scale * (w1 * jc[1][d] + w2 * jc[2][d]);
                vals[5] = bad ? CUDART_INF : static_cast<double>(mx);
            } else {
                vals[0] = x[R] + pc[1];
#pragma unroll
                for (int d = 0; d < 3; ++d) vals[2 + d] = jc[1][d];
                // max |f| and the finite check on the bit patterns: for non-negative
                // doubles the integer order is the value order; exponent 0x7FF is Inf/NaN
                unsigned long long mb = 0;
#pragma unroll
                for (int q = 0; q < Q; ++q) {
                    const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(x[q])) &
                                                 0x7FFFFFFFFFFFFFFFull;
                    mb = b > mb ? b : mb;
                }
                vals[5] = mb >= 0x7FF0000000000000ull ? CUDART_INF : __longlong_as_double(static_cast<long long>(mb));
            }
        } else {
            double f0[Q], f1[Q];
            load_rk<Q, S, LOCAL>(g, a.L, i, f0, f1, a.rho_ref, a.inv_scale);
            double mx = 0.0;
#pragma unroll
            for (int q = 0; q < Q; ++q) {
                const double ft = f0[q] + f1[q];
                vals[0] += f0[q];
                vals[1] += f1[q];
                vals[2] += Lat<Q>::cx(q) * ft;
                vals[3] += Lat<Q>::cy(q) * ft;
                vals[4] += Lat<Q>::cz(q) * ft;
                const double af = fmax(fabs(f0[q]), fabs(f1[q]));
                mx = (af != af || isinf(af)) ? CUDART_INF : fmax(mx, af);
            }
            vals[5] = mx;
        }
    }
}

template <int Q, class S, int NF, bool LOCAL>
__global__ void __launch_bounds__(kBlock) k_moments(StepArgs a) {
    constexpr int NV = 6;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double vals[NV] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    if (i < a.L.nf) moments_node<Q, S, NF, LOCAL>(a, i, vals);
    block_reduce_store<NV>(vals, a.partials, true);
}

}  // namespace bclbm
