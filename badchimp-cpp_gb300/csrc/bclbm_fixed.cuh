// 64-bit fixed-point arithmetic for the FP64-storage collision.
//
// GB300 executes FP64 at about 1/64 of its FP32 rate, so an FP64 BGK/TRT
// collision (~200 FP64 instructions per node update) saturates the FP64 pipe
// at ~15 % of HBM bandwidth.  The integer pipes have the throughput.  Values
// are held as int64 with FB = 60 fractional bits (range |x| < 8, resolution
// 2^-60 = 8.7e-19).  LB populations of a fluid with rho ~ 1 are O(w_q) > 0.02,
// so the resolution is finer than an FP64 ulp of any population (>= 3.5e-18),
// sums of populations are exact, and each product is rounded to nearest once.
// Results are rounded back to FP64.  Values of magnitude >= 8 cannot be held:
// they saturate and raise a flag the host reads (bclbm_reduce).
//
// Everything here is __host__ __device__ so that the arithmetic can be tested
// on the CPU against 128-bit integer references.
#pragma once

#include <cstdint>

#include "bclbm_device.cuh"

#ifndef __CUDACC__
#define __host__
#define __device__
#define __forceinline__ inline
#endif

namespace bclbm {
namespace fx {

constexpr int FB = 60;
constexpr int64_t ONE = int64_t(1) << FB;

__host__ __device__ __forceinline__ uint64_t bits_of(double d) {
#ifdef __CUDA_ARCH__
    return static_cast<uint64_t>(__double_as_longlong(d));
#else
    uint64_t b;
    __builtin_memcpy(&b, &d, 8);
    return b;
#endif
}

__host__ __device__ __forceinline__ double double_of(uint64_t b) {
#ifdef __CUDA_ARCH__
    return __longlong_as_double(static_cast<long long>(b));
#else
    double d;
    __builtin_memcpy(&d, &b, 8);
    return d;
#endif
}

__host__ __device__ __forceinline__ int clz64(uint64_t a) {
#ifdef __CUDA_ARCH__
    return __clzll(static_cast<long long>(a));
#else
    return a ? __builtin_clzll(a) : 64;
#endif
}

// high 64 bits of the signed 128-bit product
__host__ __device__ __forceinline__ int64_t mulhi(int64_t a, int64_t b) {
#ifdef __CUDA_ARCH__
    return __mul64hi(static_cast<long long>(a), static_cast<long long>(b));
#else
    return static_cast<int64_t>((static_cast<__int128>(a) * static_cast<__int128>(b)) >> 64);
#endif
}

// a * b / 2^FB, rounded to nearest (ties toward +inf), through __mul64hi
__host__ __device__ __forceinline__ int64_t mul(int64_t a, int64_t b) {
    const uint64_t lo = static_cast<uint64_t>(a) * static_cast<uint64_t>(b);
    int64_t hi = mulhi(a, b);
    const uint64_t lo2 = lo + (uint64_t(1) << (FB - 1));
    hi += (lo2 < lo) ? 1 : 0;
    return static_cast<int64_t>((static_cast<uint64_t>(hi) << (64 - FB)) | (lo2 >> FB));
}

// The kernel's products, by operand signs (uu: both >= 0, su: b >= 0, ss).
// All equal mul() bit for bit.
// hi:lo of the unsigned 128-bit product a b + 2^59 (the rounding constant),
// from four 32 x 32 -> 64 partial products that share their carries (the
// device's form; callable on the host so that it can be checked there).
__host__ __device__ __forceinline__ void umul128_round_pieces(uint64_t a, uint64_t b, uint64_t& hi, uint32_t& lo_hi) {
    const uint32_t a0 = static_cast<uint32_t>(a), a1 = static_cast<uint32_t>(a >> 32);
    const uint32_t b0 = static_cast<uint32_t>(b), b1 = static_cast<uint32_t>(b >> 32);
    const uint64_t p00 = static_cast<uint64_t>(a0) * b0;
    // + 2^27 at weight 2^32 is the rounding constant 2^59; the sum stays below 2^64
    const uint64_t p01 = static_cast<uint64_t>(a0) * b1 + ((p00 >> 32) + (uint64_t(1) << 27));
    const uint64_t p10 = static_cast<uint64_t>(a1) * b0 + static_cast<uint32_t>(p01);
    hi = static_cast<uint64_t>(a1) * b1 + (p01 >> 32) + (p10 >> 32);
    lo_hi = static_cast<uint32_t>(p10);  // bits [32, 64) of the low word
}

__host__ __device__ __forceinline__ void umul128_round(uint64_t a, uint64_t b, uint64_t& hi, uint32_t& lo_hi) {
#ifdef __CUDA_ARCH__
    umul128_round_pieces(a, b, hi, lo_hi);
#else
    const unsigned __int128 p = static_cast<unsigned __int128>(a) * b + (static_cast<unsigned __int128>(1) << (FB - 1));
    hi = static_cast<uint64_t>(p >> 64);
    lo_hi = static_cast<uint32_t>(static_cast<uint64_t>(p) >> 32);
#endif
}

// High word of the unsigned 128-bit product a b + 2^63, in the same pieces
// (+ 2^31 at weight 2^32; the sum stays below 2^64).
__host__ __device__ __forceinline__ uint64_t umulhi_r63_pieces(uint64_t a, uint64_t b) {
    const uint32_t a0 = static_cast<uint32_t>(a), a1 = static_cast<uint32_t>(a >> 32);
    const uint32_t b0 = static_cast<uint32_t>(b), b1 = static_cast<uint32_t>(b >> 32);
    const uint64_t p00 = static_cast<uint64_t>(a0) * b0;
    const uint64_t p01 = static_cast<uint64_t>(a0) * b1 + ((p00 >> 32) + (uint64_t(1) << 31));
    const uint64_t p10 = static_cast<uint64_t>(a1) * b0 + static_cast<uint32_t>(p01);
    return static_cast<uint64_t>(a1) * b1 + (p01 >> 32) + (p10 >> 32);
}

__host__ __device__ __forceinline__ uint64_t umulhi_r63(uint64_t a, uint64_t b) {
#ifdef __CUDA_ARCH__
    return umulhi_r63_pieces(a, b);
#else
    const unsigned __int128 p = static_cast<unsigned __int128>(a) * b + (static_cast<unsigned __int128>(1) << 63);
    return static_cast<uint64_t>(p >> 64);
#endif
}

// bits [60, 124) of the 128-bit product
__host__ __device__ __forceinline__ int64_t combine(uint64_t hi, uint32_t lo_hi) {
    return static_cast<int64_t>((hi << (64 - FB)) | (lo_hi >> (FB - 32)));
}

// Products with a constant 0 <= b < 1 held in k form, bk = b 2^4 (b in units of
// 2^-FB): the rounded product a b 2^-FB is then the high word of a bk + 2^63,
// with no shift to join two words.  For a signed a, a + 2^63 (a with its sign
// bit flipped) is unsigned and (a + 2^63) bk 2^-64 = a bk 2^-64 + bk / 2 with
// bk / 2 an integer, so the sign costs one constant subtraction.  Both equal
// mul_su(a, b) bit for bit.
__host__ __device__ __forceinline__ uint64_t kform(int64_t b) { return static_cast<uint64_t>(b) << 4; }

__host__ __device__ __forceinline__ int64_t mul_uk(int64_t a, uint64_t bk) {  // a >= 0
    return static_cast<int64_t>(umulhi_r63(static_cast<uint64_t>(a), bk));
}

__host__ __device__ __forceinline__ int64_t mul_sk(int64_t a, uint64_t bk) {
    return static_cast<int64_t>(umulhi_r63(static_cast<uint64_t>(a) ^ (uint64_t(1) << 63), bk) - (bk >> 1));
}

// a b / 2^FB rounded to nearest, for a, b >= 0
__host__ __device__ __forceinline__ int64_t mul_uu(int64_t a, int64_t b) {
    uint64_t hi;
    uint32_t lh;
    umul128_round(static_cast<uint64_t>(a), static_cast<uint64_t>(b), hi, lh);
    return combine(hi, lh);
}

// a signed, b >= 0: the two's-complement pattern of a is a + 2^64 when a < 0, so
// the signed product's high word is the unsigned one minus b
__host__ __device__ __forceinline__ int64_t mul_su(int64_t a, int64_t b) {
    uint64_t hi;
    uint32_t lh;
    umul128_round(static_cast<uint64_t>(a), static_cast<uint64_t>(b), hi, lh);
    hi -= static_cast<uint64_t>(a >> 63) & static_cast<uint64_t>(b);
    return combine(hi, lh);
}

// both signed
__host__ __device__ __forceinline__ int64_t mul_ss(int64_t a, int64_t b) {
    uint64_t hi;
    uint32_t lh;
    umul128_round(static_cast<uint64_t>(a), static_cast<uint64_t>(b), hi, lh);
    hi -= (static_cast<uint64_t>(a >> 63) & static_cast<uint64_t>(b)) + (static_cast<uint64_t>(b >> 63) & static_cast<uint64_t>(a));
    return combine(hi, lh);
}

// FP64 -> fixed, rounded to nearest; |d| >= 8 saturates and sets ovf.
__host__ __device__ __forceinline__ int64_t from_f64(double d, int& ovf) {
    const uint64_t b = bits_of(d);
    const int e = static_cast<int>((b >> 52) & 0x7FF);
    const uint64_t m = (b & 0xFFFFFFFFFFFFFull) | (uint64_t(1) << 52);
    const int sh = e - 1075 + FB;  // d = m 2^(e - 1075)
    uint64_t mag;
    if (e == 0) {
        mag = 0;  // zero or subnormal
    } else if (sh >= 0) {
        if (sh > 10 || e == 0x7FF) {
            ovf = 1;
            mag = uint64_t(7) << FB;
        } else {
            mag = m << sh;
        }
    } else if (sh > -64) {
        mag = (m + (uint64_t(1) << (-sh - 1))) >> (-sh);
    } else {
        mag = 0;
    }
    return (b >> 63) ? -static_cast<int64_t>(mag) : static_cast<int64_t>(mag);
}

// fixed -> FP64, rounded to nearest (ties away from zero)
__host__ __device__ __forceinline__ double to_f64(int64_t x) {
    if (x == 0) return 0.0;
    const uint64_t s = static_cast<uint64_t>(x) >> 63;
    const uint64_t a = s ? static_cast<uint64_t>(-x) : static_cast<uint64_t>(x);
    const int lz = clz64(a);
    const uint64_t n = a << lz;
    uint64_t m = (n >> 11) + ((n >> 10) & 1);
    int e = 63 - lz - FB + 1023;
    if (m >> 53) {
        m >>= 1;
        e += 1;
    }
    return double_of((s << 63) | (static_cast<uint64_t>(e) << 52) | (m & 0xFFFFFFFFFFFFFull));
}

// Conversions used by the kernel (BCLBM_FX_CONV):
//   0  from_f64 / to_f64 above (generic integer code)
//   1  integer code specialised for the common exponent ranges, funnel shifts
//   2  hardware F2I.S64.F64 / I2F.F64.S64, the 2^60 scaling done as an
//      integer add to the exponent field
#ifndef BCLBM_FX_CONV
#define BCLBM_FX_CONV 2
#endif
// the store side can use its own choice (default: the same)
#ifndef BCLBM_FX_CONV_STORE
#define BCLBM_FX_CONV_STORE BCLBM_FX_CONV
#endif

__host__ __device__ __forceinline__ int64_t load_f64(double d, int& ovf) {
#if BCLBM_FX_CONV == 2 && defined(__CUDA_ARCH__)
    const long long b = __double_as_longlong(d);
    // 2^60 d: exponent + 60 (d = 0 stays 0; |d| >= 8 saturates in the conversion and
    // is caught by the range guard of collide())
    const long long bs = ((b & 0x7FF0000000000000ll) == 0) ? 0ll : b + (60ll << 52);
    const long long r = __double2ll_rn(__longlong_as_double(bs));
    if (((b >> 52) & 0x7FF) >= 1026) ovf = 1;
    return r;
#elif BCLBM_FX_CONV == 1 && defined(__CUDA_ARCH__)
    const unsigned hi = static_cast<unsigned>(__double2hiint(d));
    const unsigned lo = static_cast<unsigned>(__double2loint(d));
    const int e = static_cast<int>((hi >> 20) & 0x7FF);
    const int sh = e - 1075 + FB;
    if (sh >= 0 && sh <= 10) {  // |d| in [2^-10, 8)
        const unsigned mhi = (hi & 0xFFFFFu) | 0x100000u;
        const unsigned rhi = __funnelshift_l(lo, mhi, sh);
        const unsigned rlo = lo << sh;
        int64_t r = static_cast<int64_t>((static_cast<uint64_t>(rhi) << 32) | rlo);
        const int64_t sm = static_cast<int64_t>(static_cast<int>(hi) >> 31);  // 0 or -1
        return (r ^ sm) - sm;
    }
    return from_f64(d, ovf);
#else
    return from_f64(d, ovf);
#endif
}

#ifdef __CUDACC__
// The kernel's load: hardware F2I of 2^60 d, the scaling an add to the exponent
// field of the high word.  Zero and subnormal inputs become values below 2^-900,
// which convert to 0.  The largest exponent field seen goes to emax: >= 1026
// (|d| >= 8, Inf, NaN) is out of range, and is also where the add can wrap.
__device__ __forceinline__ int64_t load_f64_hw(double d, unsigned& emax) {
    const unsigned hi = static_cast<unsigned>(__double2hiint(d));
    emax = max(emax, hi & 0x7FF00000u);
    return __double2ll_rn(__hiloint2double(static_cast<int>(hi + (60u << 20)), __double2loint(d)));
}
constexpr unsigned kLoadEmaxLimit = 1026u << 20;
#endif

__host__ __device__ __forceinline__ double store_f64(int64_t x) {
#if BCLBM_FX_CONV_STORE == 2 && defined(__CUDA_ARCH__)
    // 2^-60 of the hardware I2F result: exponent - 60 on the high word.  Nonzero
    // results have exponent >= 963 or the sign bit set, so the unsigned max leaves
    // them alone and maps 0 to 0.
    const double r = __ll2double_rn(x);
    const unsigned hi = static_cast<unsigned>(__double2hiint(r));
    return __hiloint2double(static_cast<int>(max(hi, 60u << 20) - (60u << 20)), __double2loint(r));
#elif BCLBM_FX_CONV_STORE == 1 && defined(__CUDA_ARCH__)
    const int64_t sm = x >> 63;
    const uint64_t a = static_cast<uint64_t>((x ^ sm) - sm);
    const unsigned ahi = static_cast<unsigned>(a >> 32), alo = static_cast<unsigned>(a);
    if (ahi != 0) {  // |x| >= 2^32
        const int lz = __clz(static_cast<int>(ahi));
        const unsigned nhi = __funnelshift_l(alo, ahi, lz);
        const unsigned nlo = alo << lz;
        uint64_t m = ((static_cast<uint64_t>(nhi) << 32 | nlo) >> 11) + ((nlo >> 10) & 1u);
        const unsigned e = static_cast<unsigned>(63 - lz - FB + 1023) + static_cast<unsigned>(m >> 53);
        const uint64_t bits = (static_cast<uint64_t>(sm) & 0x8000000000000000ull) |
                              (static_cast<uint64_t>(e) << 52) | (m & 0xFFFFFFFFFFFFFull);
        return __longlong_as_double(static_cast<long long>(bits));
    }
    return to_f64(x);
#else
    return to_f64(x);
#endif
}

#ifdef __CUDACC__
}  // namespace fx

// Fixed-point storage of the FP64 populations (the default BCLBM_F64 step keeps its
// state in the collision's own int64 format: no conversion per step; downloads
// and reductions convert to FP64).
template <>
struct Store<int64_t> {
    using T = int64_t;
    static constexpr bool shifted = false;
    __device__ static double val(int64_t v) { return fx::store_f64(v); }
};

namespace fx {
#endif

// Host-side conversion of a parameter (no overflow expected).
inline int64_t param(double d) {
    int ovf = 0;
    return from_f64(d, ovf);
}

// Per-handle constants of the fixed-point BGK/TRT collision (collide_to).  All
// multiplying constants are positive, so their products with a signed value
// take the cheaper signed x unsigned form.
struct Consts {
    int64_t homs, homa;   // oms / 2, oma / 2 (pairs: f_q - homs P - homa M)
    int64_t oms;          // rest direction: f_R - oms f_R
    int64_t oms_w2;       // oms w_diag
    int64_t k45;          // 4.5 oms w_diag
    int64_t oma3_w2;      // 3 oma w_diag
    int64_t tsf3_w2;      // 3 w_diag tsf
    int64_t tso;          // tsf / oms (the mass source's share of the equilibrium density)
    int64_t kf9[19];      // 9 w_q tsf (c_q . F)
    int64_t ka3[19];      // 3 w_q taf (c_q . F)
    int64_t force[3];     // F
    int64_t half_force[3];  // F / 2
    // the multipliers in [0, 1) in k form (kform): homs, homa, oms_w2, k45, oma3_w2, tsf3_w2
    uint64_t homs_k, homa_k, oms_w2_k, k45_k, oma3_w2_k, tsf3_w2_k;
};

// The constants for relaxation times tau (symmetric) and tau_anti (TRT; BGK
// uses tau for both) and body force F, computed in FP64 as the reference
// computes 1/tau and 1 - 0.5/tau (src/lbsolver/LBcollision.h:27-75, 194-236),
// then converted to fixed point.
template <int Q>
inline Consts make_consts(bool trt, double tau, double tau_anti, const double* F) {
    using L = Lat<Q>;
    Consts K;
    __builtin_memset(&K, 0, sizeof(K));
    const double oms = 1.0 / tau, oma = trt ? 1.0 / tau_anti : oms;
    const double tsf = 1 - 0.5 / tau, taf = trt ? 1 - 0.5 / tau_anti : tsf;
    const double w2 = L::w(L::NP - 1);  // the diagonal (smallest) weight
    K.homs = param(0.5 * oms);
    K.homa = param(0.5 * oma);
    K.oms = param(oms);
    K.oms_w2 = param(oms * w2);
    K.k45 = param(4.5 * oms * w2);
    K.oma3_w2 = param(3.0 * oma * w2);
    K.tsf3_w2 = param(3.0 * w2 * tsf);
    K.tso = param(tsf / oms);
    for (int q = 0; q < Q; ++q) {
        const double cF = L::cx(q) * F[0] + L::cy(q) * F[1] + L::cz(q) * F[2];
        K.kf9[q] = param(9.0 * L::w(q) * tsf * cF);
        K.ka3[q] = param(3.0 * L::w(q) * taf * cF);
    }
    for (int d = 0; d < 3; ++d) {
        K.force[d] = param(F[d]);
        K.half_force[d] = param(0.5 * F[d]);
    }
    // tau, tau_anti > 0.5 (checked at create) puts these in [0, 1)
    K.homs_k = kform(K.homs);
    K.homa_k = kform(K.homa);
    K.oms_w2_k = kform(K.oms_w2);
    K.k45_k = kform(K.k45);
    K.oma3_w2_k = kform(K.oma3_w2);
    K.tsf3_w2_k = kform(K.tsf3_w2);
    return K;
}

// The colour gradient's norm and direction for the two-phase collision, from the
// integer gradient T (G = T / 3, |T_d| < 6): cgn = |G| and n = G / |G| in fixed
// point, or n = G where |G| < 2^-52 (the reference's gs = 1 / (|G| + (|G| < eps))
// gives G / (|G| + 1), equal to G to 2^-104).  T is scaled by a power of two so that
// its largest component t_d is in [1/2, 1); x = |t|^2 in [1/4, 3); y = 1/sqrt(x) from
// an FP32 estimate and two Newton steps y (3 - x y^2) / 2 in fixed point; n = t y and
// |G| = x y / 3 scaled back.  third = 1/3 in fixed point.
__host__ __device__ __forceinline__ float rsqrt_estimate(float x) {
#ifdef __CUDA_ARCH__
    return rsqrtf(x);
#else
    return 1.0f / __builtin_sqrtf(x);
#endif
}

template <int D>
__host__ __device__ __forceinline__ void unit_normal(const int64_t* T, int64_t third, int64_t* n, int64_t& cgn) {
    auto mag = [](int64_t v) { return static_cast<uint64_t>(v < 0 ? -v : v); };
    uint64_t mx = mag(T[0]) > mag(T[1]) ? mag(T[0]) : mag(T[1]);
    if (D == 3 && mag(T[2]) > mx) mx = mag(T[2]);
    n[0] = n[1] = n[2] = 0;
    cgn = 0;
    if (mx == 0) return;
    const int sh = clz64(mx) - 4;  // mx < 2^63: sh >= -3
    int64_t t[3] = {0, 0, 0};
    for (int d = 0; d < D; ++d) t[d] = sh >= 0 ? static_cast<int64_t>(static_cast<uint64_t>(T[d]) << sh) : (T[d] >> -sh);
    int64_t x = mul_ss(t[0], t[0]) + mul_ss(t[1], t[1]);
    if (D == 3) x += mul_ss(t[2], t[2]);
    const float xf = static_cast<float>(static_cast<int>(x >> 32)) * 3.7252902984619140625e-9f;  // 2^-28
    const float ys = rsqrt_estimate(xf) * 536870912.0f;                                       // 2^29
    int64_t y = static_cast<int64_t>(static_cast<int>(ys + 0.5f)) << 31;
    for (int it = 0; it < 2; ++it) y = mul_uu(y, 3 * ONE - mul_uu(x, mul_uu(y, y))) >> 1;
    const int64_t r3 = mul_uu(mul_uu(x, y), third);  // |t| / 3
    cgn = sh >= 0 ? r3 >> sh : static_cast<int64_t>(static_cast<uint64_t>(r3) << -sh);
    if (cgn >= 256) {  // |G| >= 2^-52
        for (int d = 0; d < D; ++d) n[d] = mul_su(t[d], y);
    } else {
        for (int d = 0; d < D; ++d) n[d] = mul_su(T[d], third);
    }
}

// Constants of the two-phase (Rothman-Keller) collision in fixed point: the
// lattice weights and B coefficients by weight class (0 rest, 1 axis, 2 diagonal).
struct RkConsts {
    int64_t w1, w2;      // w_axis, w_diag
    int64_t w2_3, w2_45; // 3 w_diag, 4.5 w_diag
    int64_t w2s;         // w_diag / sqrt(2) (recolouring of the diagonal links, |c| = sqrt 2)
    int64_t B[3];        // calcDeltaOmegaST's B_q by class
    int64_t beta;        // recolouring parameter
    int64_t st;          // 9/8 sigma: the surface-tension amplitude is 9/8 sigma oms |grad|
    int64_t third;       // 1/3
    // Equal kinematic viscosities make the relaxation rate a constant,
    // oms = nu^-1 / (3 + nu^-1 / 2) (Dn = nu^-1 rho at every node), and with it
    // the products below; otherwise the kernel forms them per node.
    int uniform;
    int64_t oms, oms_w2, oms_k45, oms_k3, tf3w2, st_oms;
    uint64_t w1_k, w2s_k;  // w_axis, w_diag / sqrt(2) in k form
};

template <int Q>
inline RkConsts make_rk_consts(double nu0inv, double nu1inv, double sigma, double beta) {
    using L = Lat<Q>;
    RkConsts K;
    const double w1 = L::w(0), w2 = L::w(L::NP - 1);
    K.w1 = param(w1);
    K.w2 = param(w2);
    K.w2_3 = param(3.0 * w2);
    K.w2_45 = param(4.5 * w2);
    K.w2s = param(w2 * 0.70710678118654752440);
    K.B[0] = param(L::B(L::REST));
    K.B[1] = param(L::B(0));
    K.B[2] = param(L::B(L::NP - 1));
    K.beta = param(beta);
    K.st = param(1.125 * sigma);
    K.third = param(1.0 / 3.0);
    K.uniform = nu0inv == nu1inv;
    const double oms = K.uniform ? nu0inv / (3.0 + 0.5 * nu0inv) : 0.0;
    K.oms = param(oms);
    K.oms_w2 = param(oms * w2);
    K.oms_k45 = param(oms * 4.5 * w2);
    K.oms_k3 = param(oms * 3.0 * w2);
    K.tf3w2 = param((1.0 - 0.5 * oms) * 3.0 * w2);
    K.st_oms = param(1.125 * sigma * oms);
    K.w1_k = kform(K.w1);
    K.w2s_k = kform(K.w2s);
    return K;
}

// One BGK (TRT = false) or TRT collision in fixed point: the regrouping by
// direction pairs of calcOmegaBGK(TRT) + calcDeltaOmegaF(TRT)
// (src/lbsolver/LBcollision.h:27-75, 194-236).  With P = f_q + f_rq,
// M = f_q - f_rq and j = rho u = sum_q f c_q + F/2 (exact in fixed point):
//   post_q  = f_q  - (oms/2) P - (oma/2) M + X + Y
//   post_rq = f_rq - (oms/2) P + (oma/2) M + X - Y
//   X = oms w (rho - 1.5 j.u) + 4.5 oms w (c.j)(c.u) + 9 w tsf (c.F)(c.u) - 3 w tsf u.F
//   Y = 3 oma w (c.j) + 3 w taf (c.F)
//   post_rest = f_R - oms f_R + oms w0 (rho - 1.5 j.u) - 3 w0 tsf u.F
// (rho (c.u)^2 = (c.j)(c.u) and rho u^2 = j.u, so no product involves rho).
// F holds the node's Q populations on entry; each post-collision population is
// handed to sink(q, value) as soon as it is known (pairs in order, the rest
// direction last), so a kernel can store it and free its registers while the
// remaining pairs are computed.  rho and u receive the moments.  ovf is set
// when the node's values do not fit the fixed-point range: the sum of |f_q|
// must stay below 8 (it bounds rho and every momentum component) and rho above
// 0.15 (1 / rho below 8).
//
// Weight classes: w_rest : w_axis : w_diag = 12 : 2 : 1 (D3Q19) and 16 : 4 : 1
// (D2Q9), so the class products are exact multiples of the diagonal one.
//
// SRC = true adds the two terms of the std_one_phase node loop
// (src/std_one_phase/main.cpp:496-539): the body force is the handle's force
// times the node's integer force attribute fo, and qm is the node's mass
// source (calcDeltaOmegaQ, src/lbsolver/LBcollision.h:80-98): rho = sum f +
// qm/2, and the equilibrium weight oms rho + tsf qm = oms rho_e with
// rho_e = rho + (tsf/oms) qm, so j_e = rho_e u takes the place of j in X and Y.
template <int Q, bool TRT, bool SRC = false, class Sink>
__host__ __device__ __forceinline__ void collide_to(int64_t* F, const Consts& K, int64_t& rho_o, int64_t* u_o,
                                                    int& ovf, Sink&& sink, int fo = 1, int64_t qm = 0) {
    constexpr int D = Lat<Q>::D, NP = Lat<Q>::NP, R = Lat<Q>::REST;
    constexpr int SH1 = Q == 19 ? 1 : 2;  // w_axis / w_diag = 2 or 4
    {
        // sum_q |f_q| / 2^56 <= t + Q; t <= 108 keeps sum |f_q| below 127 * 2^56 < 8 * 2^60
        int t = 0;
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            const int h = static_cast<int>(F[q] >> 56);
            t += h < 0 ? -h : h;
        }
        if (t > 108) ovf = 1;
    }
    int64_t rho = F[R];
    if (SRC) rho += qm >> 1;
    int64_t J[3] = {0, 0, 0};
#pragma unroll
    for (int k = 0; k < NP; ++k) {
        const int64_t Pk = F[k] + F[k + NP], Mk = F[k] - F[k + NP];
        rho += Pk;
        if (Lat<Q>::cx(k) > 0) J[0] += Mk;
        if (Lat<Q>::cx(k) < 0) J[0] -= Mk;
        if (Lat<Q>::cy(k) > 0) J[1] += Mk;
        if (Lat<Q>::cy(k) < 0) J[1] -= Mk;
        if (D == 3 && Lat<Q>::cz(k) > 0) J[2] += Mk;
        if (D == 3 && Lat<Q>::cz(k) < 0) J[2] -= Mk;
    }
    // 1 / rho: FP32 estimate (24 bits), one Newton step in fixed point (48 bits):
    // u = j / rho is O(1e-2) or less, so its absolute error stays below 2^-60
    const float rf = static_cast<float>(rho) * 8.67361737988403547e-19f;  // 2^-60
    if (!(rf > 0.15f)) ovf = 1;
#ifdef __CUDA_ARCH__
    const float ri = __frcp_rn(rf);
#else
    const float ri = 1.0f / rf;
#endif
    int64_t inv = static_cast<int64_t>(ri * 1.152921504606846976e18f);  // 2^60
    inv = mul_uu(inv, 2 * ONE - mul_uu(rho, inv));
    int64_t j[3], u[3], u45[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        j[d] = (d < D) ? J[d] + (SRC ? K.half_force[d] * fo : K.half_force[d]) : 0;
        u[d] = (d < D) ? mul_su(j[d], inv) : 0;
        u45[d] = (d < D) ? mul_sk(u[d], K.k45_k) : 0;
    }
    rho_o = rho;
#pragma unroll
    for (int d = 0; d < D; ++d) u_o[d] = u[d];
    int64_t rho_e = rho;
    if (SRC && qm != 0) {
        // j_e = j + (tsf/oms) qm u, rho_e = rho + (tsf/oms) qm
        const int64_t s = mul_ss(qm, K.tso);
        rho_e += s;
#pragma unroll
        for (int d = 0; d < D; ++d) j[d] += mul_ss(u[d], s);
    }
    int64_t ju = mul_ss(j[0], u[0]) + mul_ss(j[1], u[1]);
    if (D == 3) ju += mul_ss(j[2], u[2]);
    // u.F over the force's nonzero components (the branches are uniform)
    int64_t uF = 0;
#pragma unroll
    for (int d = 0; d < D; ++d)
        if (K.force[d] != 0) uF += mul_ss(u[d], K.force[d]);
    if (SRC) uF *= fo;
    const int64_t AB2 = mul_sk(rho_e - (ju + (ju >> 1)), K.oms_w2_k);  // oms w2 (rho_e - 1.5 j.u)
    const int64_t K2 = -mul_sk(uF, K.tsf3_w2_k);                      // -3 w2 tsf u.F
    // class c values (rest 0, axis 1, diagonal 2) by the exact weight ratios
    auto by_class = [](int64_t v2, int c) -> int64_t {
        return c == 2 ? v2 : (c == 1 ? (v2 << SH1) : (Q == 19 ? (v2 << 3) + (v2 << 2) : (v2 << 4)));
    };
    const uint64_t homa_k = TRT ? K.homa_k : K.homs_k;
#pragma unroll
    for (int k = 0; k < NP; ++k) {
        const int c = Lat<Q>::wclass(k);
        const int64_t cj = Lat<Q>::cx(k) * j[0] + Lat<Q>::cy(k) * j[1] + Lat<Q>::cz(k) * j[2];
        const int64_t cu45 = Lat<Q>::cx(k) * u45[0] + Lat<Q>::cy(k) * u45[1] + Lat<Q>::cz(k) * u45[2];
        int64_t X = by_class(AB2 + mul_ss(cj, cu45) + K2, c);
        // the force term vanishes for directions normal to the force (uniform branch)
        if (K.kf9[k] != 0) {
            const int64_t cu = Lat<Q>::cx(k) * u[0] + Lat<Q>::cy(k) * u[1] + Lat<Q>::cz(k) * u[2];
            X += SRC ? mul_ss(K.kf9[k], cu) * fo : mul_ss(K.kf9[k], cu);
        }
        const int64_t Y = by_class(mul_sk(cj, K.oma3_w2_k), c) + (SRC ? K.ka3[k] * fo : K.ka3[k]);
        const int64_t P = F[k] + F[k + NP], M = F[k] - F[k + NP];
        const int64_t sp = mul_sk(P, K.homs_k), sm = mul_sk(M, homa_k);
        sink(k, F[k] - sp - sm + X + Y);
        sink(k + NP, F[k + NP] - sp + sm + X - Y);
    }
    sink(R, F[R] - mul_su(F[R], K.oms) + by_class(AB2 + K2, 0));
}

// collide_to with the results written back into F
template <int Q, bool TRT>
__host__ __device__ __forceinline__ void collide(int64_t* F, const Consts& K, int64_t& rho_o, int64_t* u_o,
                                                 int& ovf) {
    collide_to<Q, TRT>(F, K, rho_o, u_o, ovf, [F](int q, int64_t v) { F[q] = v; });
}

}  // namespace fx
}  // namespace bclbm
