// Test harness: runs the fixed-point collision of csrc/bclbm_fixed.cuh on the
// CPU (host branch of its __host__ __device__ functions, 128-bit integer
// multiplies), with the state kept in int64 between steps as the device keeps
// it, so that its arithmetic can be checked against the reference fixtures
// without a GPU.  Built by tests/test_fixed_point.py with nvcc as
// host-only code; never part of the library.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "bclbm_fixed.cuh"

using namespace bclbm;

namespace {

template <int Q>
fx::Consts make_consts(bool trt, double tau, double tau_anti, const double* F) {
    return fx::make_consts<Q>(trt, tau, tau_anti, F);
}

template <int Q, bool TRT>
int run(int n_nodes, const int32_t* neigh, const int16_t* types, int n_bulk, const int32_t* bulk, int steps,
        double tau, double tau_anti, const double* F, double* f, double* rho_out, double* vel_out) {
    using L = Lat<Q>;
    const fx::Consts K = make_consts<Q>(TRT, tau, tau_anti, F);
    // ghost sources: last bulk node whose neighbour along c_p is node 0
    int gsrc[19] = {0};
    for (int p = 0; p < Q - 1; ++p)
        for (int b = n_bulk - 1; b >= 0; --b)
            if (neigh[static_cast<size_t>(bulk[b]) * Q + p] == 0) {
                gsrc[p] = bulk[b];
                break;
            }
    // the state between steps stays in the collision's int64 format, as on the device
    std::vector<int64_t> G(static_cast<size_t>(n_nodes) * Q, 0), G2(G.size(), 0);
    int ovf = 0;
    auto pulled = [&](size_t x, int q) -> int64_t {
        if (q == L::REST) return G[x * Q + q];
        const int rq = L::rev(q);
        const int y = neigh[x * Q + rq];
        if (y != 0 && types[y] > 1) return G[static_cast<size_t>(y) * Q + q];
        if (y == 0) return G[static_cast<size_t>(gsrc[rq]) * Q + rq];
        return G[x * Q + rq];
    };
    for (int s = 0; s < steps; ++s) {
        for (int b = 0; b < n_bulk; ++b) {
            const size_t x = static_cast<size_t>(bulk[b]);
            int64_t Fx[Q];
            for (int q = 0; q < Q; ++q) Fx[q] = s == 0 ? fx::from_f64(f[x * Q + q], ovf) : pulled(x, q);
            int64_t rho, u[3];
            fx::collide<Q, TRT>(Fx, K, rho, u, ovf);
            rho_out[x] = fx::to_f64(rho);
            for (int d = 0; d < L::D; ++d) vel_out[x * L::D + d] = fx::to_f64(u[d]);
            for (int q = 0; q < Q; ++q) G2[x * Q + q] = Fx[q];
        }
        G.swap(G2);
    }
    // the reference's f after the last step: one pull of G
    for (int b = 0; b < n_bulk; ++b) {
        const size_t x = static_cast<size_t>(bulk[b]);
        for (int q = 0; q < Q; ++q) f[x * Q + q] = fx::to_f64(pulled(x, q));
    }
    return ovf;
}

}  // namespace

extern "C" int fx_collide_ovf(double scale) {
    // one D3Q19 rest-state node at rho = scale: does the collision flag it?
    const double F0[3] = {0.0, 0.0, 0.0};
    const fx::Consts K = fx::make_consts<19>(false, 0.8, 0.8, F0);
    int ovf = 0;
    int64_t F[19];
    for (int q = 0; q < 19; ++q) F[q] = fx::from_f64(Lat<19>::w(q) * scale, ovf);
    int64_t rho, u[3];
    fx::collide<19, false>(F, K, rho, u, ovf);
    return ovf;
}

extern "C" {

int fx_run(int nq, int trt, int n_nodes, const int32_t* neigh, const int16_t* types, int n_bulk, const int32_t* bulk,
           int steps, double tau, double tau_anti, const double* F, double* f, double* rho, double* vel) {
    if (nq == 9) return trt ? run<9, true>(n_nodes, neigh, types, n_bulk, bulk, steps, tau, tau_anti, F, f, rho, vel)
                            : run<9, false>(n_nodes, neigh, types, n_bulk, bulk, steps, tau, tau_anti, F, f, rho, vel);
    return trt ? run<19, true>(n_nodes, neigh, types, n_bulk, bulk, steps, tau, tau_anti, F, f, rho, vel)
               : run<19, false>(n_nodes, neigh, types, n_bulk, bulk, steps, tau, tau_anti, F, f, rho, vel);
}

// elementwise checks of the primitives; returns the number of failures
int fx_primitives(const double* a, const double* b, int n) {
    int bad = 0;
    for (int i = 0; i < n; ++i) {
        int ovf = 0;
        const int64_t xa = fx::from_f64(a[i], ovf), xb = fx::from_f64(b[i], ovf);
        // conversion: exact integer reference by long double (64-bit mantissa)
        const long double ra = std::nearbyintl(static_cast<long double>(a[i]) * 1152921504606846976.0L);
        if (std::fabs(static_cast<long double>(xa) - ra) > 1.0L) ++bad;
        // round trip back to FP64: within half an ulp of FP64 and of the fixed resolution
        const double back = fx::to_f64(xa);
        const double tol = std::fabs(a[i]) * 1.2e-16 + 8.7e-19;
        if (std::fabs(back - a[i]) > tol) ++bad;
        // product: 128-bit reference, rounded to nearest
        const __int128 p = static_cast<__int128>(xa) * static_cast<__int128>(xb);
        const int64_t ref = static_cast<int64_t>((p + (static_cast<__int128>(1) << 59)) >> 60);
        if (fx::mul(xa, xb) != ref) ++bad;
        if (fx::mul_ss(xa, xb) != ref) ++bad;
        if (xb >= 0 && fx::mul_su(xa, xb) != ref) ++bad;
        if (xa >= 0 && xb >= 0 && fx::mul_uu(xa, xb) != ref) ++bad;
        // the device's 32-bit-piece forms against 128-bit products
        const uint64_t ua = static_cast<uint64_t>(xa), ub = static_cast<uint64_t>(xb);
        const unsigned __int128 up = static_cast<unsigned __int128>(ua) * ub;
        uint64_t hi;
        uint32_t lh;
        fx::umul128_round_pieces(ua, ub, hi, lh);
        const unsigned __int128 r59 = up + (static_cast<unsigned __int128>(1) << 59);
        if (hi != static_cast<uint64_t>(r59 >> 64) || lh != static_cast<uint32_t>(static_cast<uint64_t>(r59) >> 32)) ++bad;
        const unsigned __int128 r63 = up + (static_cast<unsigned __int128>(1) << 63);
        if (fx::umulhi_r63_pieces(ua, ub) != static_cast<uint64_t>(r63 >> 64)) ++bad;
        // k-form products for multipliers in [0, 1): equal to mul_su
        if (xb >= 0 && xb < fx::ONE) {
            const uint64_t bk = fx::kform(xb);
            if (fx::mul_sk(xa, bk) != ref) ++bad;
            if (static_cast<int64_t>(fx::umulhi_r63_pieces(ua ^ (uint64_t(1) << 63), bk) - (bk >> 1)) != ref) ++bad;
            if (xa >= 0 && fx::mul_uk(xa, bk) != ref) ++bad;
        }
    }
    return bad;
}

// fx::unit_normal against long-double norms over n integer gradients T with
// |T_d| < 6 (in fixed point) spread over 60 binary orders of magnitude (every 7th in
// two dimensions); worst[0] = max |n_d - T_d / |T||, worst[1] = max ||G| - |T| / 3|,
// worst[2] = max over |G| < 2^-52 of |n_d - T_d / 3|
void fx_unit_normal_check(int n, unsigned seed, double* worst) {
    uint64_t st = 0x9E3779B97F4A7C15ull ^ seed;
    auto next = [&st]() {  // splitmix64
        uint64_t z = (st += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    };
    const int64_t third = fx::param(1.0 / 3.0);
    const long double one = static_cast<long double>(fx::ONE);
    worst[0] = worst[1] = worst[2] = 0.0;
    for (int k = 0; k < n; ++k) {
        const int scale = static_cast<int>(next() % 61);
        int64_t T[3];
        for (int d = 0; d < 3; ++d) {
            int64_t v = static_cast<int64_t>(next() % (uint64_t(6) << 60)) >> scale;
            if (next() & 1) v = -v;
            T[d] = v;
        }
        const bool two = k % 7 == 0;
        if (two) T[2] = 0;
        int64_t nv[3], cgn;
        if (two) fx::unit_normal<2>(T, third, nv, cgn);
        else fx::unit_normal<3>(T, third, nv, cgn);
        long double t2 = 0;
        for (int d = 0; d < 3; ++d) t2 += (static_cast<long double>(T[d]) / one) * (static_cast<long double>(T[d]) / one);
        const long double tn = std::sqrt(t2);
        if (tn == 0) continue;
        const double eg = static_cast<double>(std::fabs(static_cast<long double>(cgn) / one - tn / 3));
        if (eg > worst[1]) worst[1] = eg;
        for (int d = 0; d < 3; ++d) {
            const long double nd = static_cast<long double>(nv[d]) / one;
            if (tn / 3 >= 2.220446049250313e-16L) {
                const double e = static_cast<double>(std::fabs(nd - (static_cast<long double>(T[d]) / one) / tn));
                if (e > worst[0]) worst[0] = e;
            } else {
                const double e = static_cast<double>(std::fabs(nd - static_cast<long double>(T[d]) / one / 3));
                if (e > worst[2]) worst[2] = e;
            }
        }
    }
}

}  // extern "C"
