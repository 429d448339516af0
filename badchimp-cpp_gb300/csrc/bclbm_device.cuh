// Device-side building blocks shared by the bclbm kernels.
//
// Lattices follow the reference's lattice templates exactly: velocity order,
// weights, reverse directions and rest direction last
// (src/lbsolver/LBd2q9.h:14-40, src/lbsolver/LBd3q19.h:14-40).
//
// HBM layout (one lattice instance):
//   pops   [nfields][Q][nf_pad]   structure of arrays, one row per direction;
//                                 row stride nf_pad is a multiple of 64 slots
//   nbr    [Q-1][nf_pad] int32    extended neighbour table in device numbering:
//                                 nbr[q][i] is the node reached from slot i along c_q;
//                                 values < nf are fluid slots, nf .. nf+ns-1 stored
//                                 boundary solids, nf+ns the ghost node 0
//   ghost_src[Q]                  slot whose reverse population a link from the
//                                 ghost node reads (see stream map below)
//
// Pull streaming with fused half-way bounce-back.  The reference pushes the
// post-collision populations G along c_q (LbField::propagateTo,
// src/lbsolver/LBfield.h:350-357) and then, for every fluid node whose
// upstream neighbour is solid, copies back the value that was pushed into the
// solid (HalfWayBounceBack::apply, src/lbsolver/LBhalfwaybb.h:49-62).  In pull
// form the population arriving at slot i along c_q is
//     y = nbr[rev q][i]
//     y fluid       -> G[q][y]
//     y stored solid-> G[rev q][i]            (bounce-back off the wall)
//     y ghost       -> G[rev q][ghost_src[rev q]]
// The last case reproduces the reference exactly: every node whose neighbour
// along c_p is node 0 pushes into the single slot (p, node 0); the last of
// them in bulk order wins and every bounce-back through node 0 reads that
// value.
#pragma once

#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_fp16.h>

namespace bclbm {

// ---- lattice constants -------------------------------------------------------
template <int Q>
struct Lat;

template <>
struct Lat<9> {
    static constexpr int Q = 9, D = 2, NP = 4, REST = 8;
    __host__ __device__ static constexpr int cx(int q) {
        return q == 0 ? 1 : q == 1 ? 1 : q == 2 ? 0 : q == 3 ? -1 : q == 4 ? -1 : q == 5 ? -1 : q == 6 ? 0 : q == 7 ? 1 : 0;
    }
    __host__ __device__ static constexpr int cy(int q) {
        return q == 0 ? 0 : q == 1 ? 1 : q == 2 ? 1 : q == 3 ? 1 : q == 4 ? 0 : q == 5 ? -1 : q == 6 ? -1 : q == 7 ? -1 : 0;
    }
    __host__ __device__ static constexpr int cz(int) { return 0; }
    __host__ __device__ static constexpr int rev(int q) { return q == 8 ? 8 : (q + 4) % 8; }
    // weight class: 0 rest, 1 axis, 2 diagonal
    __host__ __device__ static constexpr int wclass(int q) { return q == 8 ? 0 : (q % 2 == 0 ? 1 : 2); }
    __host__ __device__ static constexpr double w(int q) {
        return wclass(q) == 0 ? 16.0 / 36.0 : wclass(q) == 1 ? 4.0 / 36.0 : 1.0 / 36.0;
    }
    __host__ __device__ static constexpr double B(int q) {
        return wclass(q) == 0 ? -16.0 / 108.0 : wclass(q) == 1 ? 8.0 / 108.0 : 5.0 / 108.0;
    }
    static constexpr double w1c2inv = (4.0 / 36.0) * 3.0;
    static constexpr double w2c2inv = (1.0 / 36.0) * 3.0;
};

template <>
struct Lat<19> {
    static constexpr int Q = 19, D = 3, NP = 9, REST = 18;
    __host__ __device__ static constexpr int cx(int q) {
        return (q == 0 || q == 3 || q == 4 || q == 5 || q == 6) ? 1 : (q == 9 || q == 12 || q == 13 || q == 14 || q == 15) ? -1 : 0;
    }
    __host__ __device__ static constexpr int cy(int q) {
        return (q == 1 || q == 3 || q == 7 || q == 8 || q == 13) ? 1 : (q == 4 || q == 10 || q == 12 || q == 16 || q == 17) ? -1 : 0;
    }
    __host__ __device__ static constexpr int cz(int q) {
        return (q == 2 || q == 5 || q == 7 || q == 15 || q == 17) ? 1 : (q == 6 || q == 8 || q == 11 || q == 14 || q == 16) ? -1 : 0;
    }
    __host__ __device__ static constexpr int rev(int q) { return q == 18 ? 18 : (q + 9) % 18; }
    __host__ __device__ static constexpr int wclass(int q) { return q == 18 ? 0 : ((q % 9) < 3 ? 1 : 2); }
    __host__ __device__ static constexpr double w(int q) {
        return wclass(q) == 0 ? 12.0 / 36.0 : wclass(q) == 1 ? 2.0 / 36.0 : 1.0 / 36.0;
    }
    __host__ __device__ static constexpr double B(int q) {
        return wclass(q) == 0 ? -12.0 / 54.0 : wclass(q) == 1 ? 1.0 / 54.0 : 2.0 / 54.0;
    }
    static constexpr double w1c2inv = (2.0 / 36.0) * 3.0;
    static constexpr double w2c2inv = (1.0 / 36.0) * 3.0;
};

// ---- storage codecs -----------------------------------------------------------
// F64 stores f itself.  The reduced formats store the shifted, weight-normalised
// deviation d_q = (f_q - w_q rho_ref) / w_q * scale, so the stored numbers are
// O(rho' + 3 c.u) instead of O(w_q): FP16 keeps its 11-bit mantissa on the part
// that carries the flow, and the constant w_q rho_ref is never rounded.
template <class S>
struct Store;

template <>
struct Store<double> {
    using T = double;
    static constexpr bool shifted = false;
    __device__ static double val(double v) { return v; }
    __device__ static void store(double* p, double v) { *p = v; }
};
template <>
struct Store<float> {
    using T = float;
    static constexpr bool shifted = true;
    __device__ static float val(float v) { return v; }
    __device__ static void store(float* p, float v) { *p = v; }
};
template <>
struct Store<__half> {
    using T = __half;
    static constexpr bool shifted = true;
    __device__ static float val(__half v) { return __half2float(v); }
    __device__ static void store(__half* p, float v) { *p = __float2half_rn(v); }
};
template <>
struct Store<__nv_bfloat16> {
    using T = __nv_bfloat16;
    static constexpr bool shifted = true;
    __device__ static float val(__nv_bfloat16 v) { return __bfloat162float(v); }
    __device__ static void store(__nv_bfloat16* p, float v) { *p = __float2bfloat16_rn(v); }
};

// Parameters of one lattice instance as the kernels see them.
struct LatticeView {
    int nf;          // fluid (bulk) slots
    int nf_pad;      // row stride of pops / nbr
    int ns;          // stored solid nodes; nbr value nf+ns is the ghost node
    const int32_t* nbr;   // extended neighbour table (two-phase instances)
    const int32_t* pull;  // single-phase instances: [Q-1][nf_pad] element index (row * nf_pad + slot)
                          // of the post-collision value that streams into slot i along c_q, with
                          // the bounce-back and ghost cases of pull_raw resolved at set-up
    int32_t ghost_src[19];
};

// Element index (row * nf_pad + slot) of the population arriving at slot i along
// c_q from extended neighbour y, in post-collision storage.  32-bit arithmetic
// (bclbm_create keeps Q nf_pad <= INT32_MAX), so that the address is one wide
// multiply-add and the index one register (192^3 two-phase, MLUPS with 64-bit /
// 32-bit indices: one pass FP16 16,557 / 17,460, BF16 16,418 / 17,179; two
// passes BF16 11,293 / 12,109; FP64 and FP32 unchanged).
using elem_t = uint32_t;
template <int Q>
__device__ __forceinline__ elem_t pull_elem(const LatticeView& L, int q, int y, int i) {
    const int rq = Lat<Q>::rev(q);
    int slot, row;
    if (y < L.nf) {
        slot = y;
        row = q;
    } else {
        row = rq;
        slot = (y == L.nf + L.ns) ? L.ghost_src[rq] : i;
    }
    return static_cast<elem_t>(row) * static_cast<elem_t>(L.nf_pad) + static_cast<elem_t>(slot);
}

// Population arriving at slot i along c_q, read from post-collision storage g
// (one field: rows g + q*nf_pad).  Returns the raw stored value.
template <int Q, class S>
__device__ __forceinline__ typename Store<S>::T pull_raw(const S* __restrict__ g, const LatticeView& L, int q, int y,
                                                          int i) {
    const int rq = Lat<Q>::rev(q);
    int slot, row;
    if (y < L.nf) {
        slot = y;
        row = q;
    } else {
        row = rq;
        slot = (y == L.nf + L.ns) ? L.ghost_src[rq] : i;
    }
    return g[static_cast<elem_t>(row) * static_cast<elem_t>(L.nf_pad) + static_cast<elem_t>(slot)];
}

}  // namespace bclbm
