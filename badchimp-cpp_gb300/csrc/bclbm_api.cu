// The C ABI of include/bclbm.h: set-up of the device lattice from the
// reference's Grid/Nodes/LbField arrays, the step loop, downloads in the
// reference's layout, and FP64 reductions.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <climits>
#include <cstddef>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include "bclbm.h"
#include "bclbm_internal.h"
#include "bclbm_host.h"
#include "bclbm_launch.h"
#include "bclbm_links.h"
#include "bclbm_trace.h"

using namespace bclbm;
using bclbm::host::FirstBad;
using bclbm::host::parallel_for;


namespace {

// The library's stream-ordered memory pool of each device.  Its release threshold
// is unlimited: device memory that bclbm_destroy frees stays mapped in the pool,
// and the next bclbm_create on the device takes it without mapping new pages
// (mapping several GB costs tens of ms; with the default pool, any device-wide
// synchronisation of the caller's gives freed memory back).  bclbm_trim returns
// it.  The caller's own stream-ordered allocations (the device's default pool)
// are not affected.
constexpr int kMaxPoolDevices = 64;
std::mutex g_pool_mutex;
cudaMemPool_t g_pool[kMaxPoolDevices] = {};

cudaError_t library_pool(cudaMemPool_t* out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxPoolDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_pool_mutex);
    if (!g_pool[dev]) {
        cudaMemPoolProps props;
        std::memset(&props, 0, sizeof(props));
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        cudaMemPool_t pool = nullptr;
        e = cudaMemPoolCreate(&pool, &props);
        if (e != cudaSuccess) return e;
        uint64_t threshold = UINT64_MAX;
        e = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &threshold);
        if (e != cudaSuccess) {
            cudaMemPoolDestroy(pool);
            return e;
        }
        g_pool[dev] = pool;
    }
    *out = g_pool[dev];
    return cudaSuccess;
}

// cudaMallocAsync from the library's pool of the current device
cudaError_t pool_malloc(void** p, size_t bytes, cudaStream_t s) {
    cudaMemPool_t pool = nullptr;
    const cudaError_t e = library_pool(&pool);
    if (e != cudaSuccess) return e;
    return cudaMallocFromPoolAsync(p, bytes, pool, s);
}

// The caller's large host arrays page-locked for the length of one copy.  On the
// Grace host the device reads pageable memory through the host's page tables, and
// a range whose translations it has not walked yet copies at ~20-25 GB/s (1 GiB:
// 42-51 ms in a process that had just built its arrays) instead of ~190; locking
// the range costs 2-6 ms per GiB and the copy then runs at the link's rate.  A
// range that cannot be locked (already registered, a mapping the driver refuses)
// is copied as it is.  unlock() only after the copies that use the range have
// completed.
struct HostLock {
    void* p = nullptr;
    void lock(const void* ptr, size_t bytes) {
        if (p || !ptr || bytes < (size_t(64) << 20)) return;
        if (cudaHostRegister(const_cast<void*>(ptr), bytes, cudaHostRegisterDefault) == cudaSuccess)
            p = const_cast<void*>(ptr);
        else
            cudaGetLastError();  // the copy falls back to the pageable path
    }
    void unlock() {
        if (p) cudaHostUnregister(p);
        cudaGetLastError();
        p = nullptr;
    }
    // still locked on an error path: a copy may be in flight
    ~HostLock() {
        if (p) {
            cudaDeviceSynchronize();
            unlock();
        }
    }
};

size_t store_bytes(int precision) {
    switch (precision) {
        case BCLBM_F64: return 8;
        case BCLBM_F32: return 4;
        default: return 2;
    }
}

int fail(bclbm_handle* h, int code, const std::string& msg) {
    if (h) h->last_error = msg;
    return code;
}

#define CUDA_TRY(h, expr)                                                                           \
    do {                                                                                            \
        cudaError_t e_ = (expr);                                                                    \
        if (e_ != cudaSuccess) {                                                                    \
            return fail((h), e_ == cudaErrorMemoryAllocation ? BCLBM_ERR_NOMEM : BCLBM_ERR_CUDA,      \
                        std::string(#expr) + ": " + cudaGetErrorString(e_));                          \
        }                                                                                           \
    } while (0)

int rev_dir(int Q, int q) {
    if (Q == 9) return q == 8 ? 8 : (q + 4) % 8;
    return q == 18 ? 18 : (q + 9) % 18;
}

uint64_t spread_bits(uint64_t v, int dims) {
    uint64_t out = 0;
    for (int b = 0; b < 21; ++b)
        if (v & (1ull << b)) out |= 1ull << (b * dims);
    return out;
}

// Everything derived from the descriptor on the host (shared by create and footprint).
struct Plan {
    int nf = 0, nf_pad = 0, ns = 0, nfields = 1;
    std::vector<int32_t> slot_node, slot_bulk, solid_node, ext_of_node;
};

// full: also the stream-map checks (rest neighbour, symmetry), unless device_links:
// bclbm_create then runs them on the device (k_check_links) from the uploaded rows
// The descriptor's own fields (no table is read).
int validate_descriptor(const bclbm_desc* d, std::string& err) {
    if (!d) { err = "null descriptor"; return BCLBM_ERR_INVALID; }
    const int Q = d->lattice_q;
    if (Q != 9 && Q != 19) { err = "lattice_q must be 9 or 19"; return BCLBM_ERR_INVALID; }
    if (d->n_nodes < 2 || !d->neigh || !d->types || !d->bulk || d->n_bulk < 1) {
        err = "n_nodes, neigh, types, n_bulk and bulk are required";
        return BCLBM_ERR_INVALID;
    }
    if (d->collision < BCLBM_BGK || d->collision > BCLBM_LINKS) { err = "unknown collision"; return BCLBM_ERR_INVALID; }
    if (d->collision == BCLBM_LINKS && Q != 19) {
        err = "BCLBM_LINKS (the std_one_phase step) is D3Q19";
        return BCLBM_ERR_UNSUPPORTED;
    }
    if (d->collision == BCLBM_LINKS && (!d->tags || !d->labels)) {
        err = "BCLBM_LINKS needs the tags and labels attributes";
        return BCLBM_ERR_INVALID;
    }
    if (d->precision < BCLBM_F64 || d->precision > BCLBM_BF16) { err = "unknown precision"; return BCLBM_ERR_INVALID; }
    if ((d->flags & BCLBM_FLAG_EXACT) && d->precision != BCLBM_F64) {
        err = "BCLBM_FLAG_EXACT needs BCLBM_F64";
        return BCLBM_ERR_INVALID;
    }
    if ((d->flags & BCLBM_FLAG_SFC_ORDER) && !d->pos) { err = "BCLBM_FLAG_SFC_ORDER needs pos"; return BCLBM_ERR_INVALID; }
    if (d->n_bulk >= d->n_nodes) { err = "n_bulk must be smaller than n_nodes"; return BCLBM_ERR_INVALID; }
    if (static_cast<int64_t>(Q) * ((static_cast<int64_t>(d->n_bulk) + 63) / 64 * 64) > INT32_MAX) {
        // element numbers (row * nf_pad + slot) are 32-bit in the pull table and the two-phase pull
        err = "Q times n_bulk (rounded up to a multiple of 64) exceeds the int32 element numbers "
              "(D3Q19: 113 M fluid nodes per instance)";
        return BCLBM_ERR_UNSUPPORTED;
    }
    const bool fixed = d->precision == BCLBM_F64 && !(d->flags & (BCLBM_FLAG_EXACT | BCLBM_FLAG_FP64_FMA));
    if ((d->flags & BCLBM_FLAG_LAGGED_COLOUR) && !(d->collision == BCLBM_RK && d->precision != BCLBM_F64)) {
        err = "BCLBM_FLAG_LAGGED_COLOUR needs BCLBM_RK with shifted storage (F32, F16 or BF16)";
        return BCLBM_ERR_INVALID;
    }
    if ((d->flags & BCLBM_FLAG_LAGGED_COLOUR) && d->flux_control) {
        // with its sums one step late, the controller force = 2 (target - mean) would overshoot
        err = "BCLBM_FLAG_LAGGED_COLOUR takes a constant body force (flux_control 0)";
        return BCLBM_ERR_INVALID;
    }
    if (fixed && d->collision != BCLBM_RK && !(d->tau[0] > 0.5 && (d->collision != BCLBM_TRT || d->tau[1] > 0.5))) {
        // the fixed-point collision holds oms / 2, oma / 2 and 1 - 0.5 / tau as constants in [0, 1)
        err = "the fixed-point FP64 step needs tau > 0.5 (and tau_anti > 0.5 for TRT; "
              "BCLBM_FLAG_FP64_FMA or BCLBM_FLAG_EXACT take any value)";
        return BCLBM_ERR_INVALID;
    }
    if (fixed && d->collision == BCLBM_RK && !(std::fabs(d->sigma) < 3.5 && std::fabs(d->beta) < 4.0)) {
        // 9/8 sigma and beta are fixed-point constants of the default FP64 two-phase step
        err = "the fixed-point FP64 two-phase step needs |sigma| < 3.5 and |beta| < 4 "
              "(BCLBM_FLAG_FP64_FMA or BCLBM_FLAG_EXACT take any value)";
        return BCLBM_ERR_INVALID;
    }
    return BCLBM_OK;
}

int validate_and_plan(const bclbm_desc* d, Plan& p, std::string& err, bool full, bool device_links = false) {
    const int vrc = validate_descriptor(d, err);
    if (vrc) return vrc;
    const int Q = d->lattice_q;
    const int N = d->n_nodes;
    const int nb = d->n_bulk;
    p.nfields = d->collision == BCLBM_RK ? 2 : 1;
    const int32_t* nbr = d->neigh;
    const int16_t* ty = d->types;
    {
        FirstBad bad;
        parallel_for(static_cast<size_t>(N) * Q, [&](size_t b0, size_t b1) {
            for (size_t k = b0; k < b1; ++k)
                if (nbr[k] < 0 || nbr[k] >= N) {
                    bad.set(static_cast<int64_t>(k));
                    return;
                }
        });
        if (bad.any()) {
            err = "neighbour id out of range at entry " + std::to_string(bad.get());
            return BCLBM_ERR_TABLE;
        }
    }
    std::vector<int32_t> slot_of(N, -1);
    {
        FirstBad bad;
        parallel_for(static_cast<size_t>(nb), [&](size_t b0, size_t b1) {
            for (size_t b = b0; b < b1; ++b) {
                const int n = d->bulk[b];
                int c = 0;
                if (n < 1 || n >= N) c = 1;
                else if (b > 0 && n <= d->bulk[b - 1]) c = 2;
                else if (ty[n] != 2 && ty[n] != 3) c = 3;
                if (c) {
                    bad.set(static_cast<int64_t>(b));
                    return;
                }
                slot_of[n] = static_cast<int32_t>(b);  // provisional: bulk index
            }
        });
        if (bad.any()) {
            const int64_t b = bad.get();
            const int n = d->bulk[b];
            if (n < 1 || n >= N) { err = "bulk node out of range"; return BCLBM_ERR_INVALID; }
            if (b > 0 && n <= d->bulk[b - 1]) { err = "bulk list must be increasing"; return BCLBM_ERR_INVALID; }
            err = "bulk node " + std::to_string(n) + " is not own-rank fluid";
            return BCLBM_ERR_TABLE;
        }
    }
    {
        FirstBad bad;
        parallel_for(static_cast<size_t>(N), [&](size_t n0, size_t n1) {
            for (size_t n = std::max<size_t>(n0, 1); n < n1; ++n)
                if (ty[n] > 1 && slot_of[n] < 0) {
                    bad.set(static_cast<int64_t>(n));
                    return;
                }
        });
        if (bad.any()) {
            err = "fluid node " + std::to_string(bad.get()) + " missing from the bulk list";
            return BCLBM_ERR_TABLE;
        }
    }
    // device order
    std::vector<int32_t> order(nb);
    std::iota(order.begin(), order.end(), 0);
    if (d->flags & BCLBM_FLAG_SFC_ORDER) {
        const int nd = Q == 9 ? 2 : 3;
        std::vector<uint64_t> code(nb);
        parallel_for(static_cast<size_t>(nb), [&](size_t b0, size_t b1) {
            for (size_t b = b0; b < b1; ++b) {
                const int n = d->bulk[b];
                uint64_t c = 0;
                for (int k = 0; k < nd; ++k) {
                    const int64_t v = static_cast<int64_t>(d->pos[static_cast<size_t>(n) * nd + k]) + 1;
                    c |= spread_bits(static_cast<uint64_t>(std::max<int64_t>(v, 0)), nd) << (nd - 1 - k);
                }
                code[b] = c;
            }
        });
        std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) { return code[a] < code[b]; });
    }
    p.nf = nb;
    p.nf_pad = (nb + 63) / 64 * 64;
    p.slot_node.resize(nb);
    p.slot_bulk.resize(nb);
    parallel_for(static_cast<size_t>(nb), [&](size_t s0, size_t s1) {
        for (size_t s = s0; s < s1; ++s) {
            p.slot_bulk[s] = order[s];
            p.slot_node[s] = d->bulk[order[s]];
            slot_of[d->bulk[order[s]]] = static_cast<int32_t>(s);
        }
    });
    // extended numbering: fluid slots, then (two-phase only) the referenced solids in
    // node order, then the ghost; single-phase instances only need the fluid slots
    p.ext_of_node.assign(N, -1);
    parallel_for(static_cast<size_t>(N), [&](size_t n0, size_t n1) {
        for (size_t n = std::max<size_t>(n0, 1); n < n1; ++n)
            if (slot_of[n] >= 0) p.ext_of_node[n] = slot_of[n];
    });
    p.solid_node.clear();
    if (d->collision == BCLBM_RK) {
        std::vector<char> used(N, 0);
        for (int b = 0; b < nb; ++b) {
            const size_t n = static_cast<size_t>(d->bulk[b]);
            for (int q = 0; q < Q; ++q) used[nbr[n * Q + q]] = 1;
        }
        for (int n = 1; n < N; ++n)
            if (used[n] && ty[n] < 2) {
                p.ext_of_node[n] = nb + static_cast<int>(p.solid_node.size());
                p.solid_node.push_back(n);
            }
    }
    p.ns = static_cast<int>(p.solid_node.size());
    p.ext_of_node[0] = nb + p.ns;
    if (!full || device_links) return BCLBM_OK;
    // the reference streams rest populations to neighbor(rest, n); it must be n itself.
    // Pull equivalence: the fluid upstream neighbour pushes into this node, and this
    // node's fluid downstream neighbour pulls from it (a one-to-one stream map).
    const int R = Q - 1;
    FirstBad bad_rest, bad_sym;
    parallel_for(static_cast<size_t>(nb), [&](size_t b0, size_t b1) {
        for (size_t b = b0; b < b1; ++b) {
            const size_t n = static_cast<size_t>(d->bulk[b]);
            if (nbr[n * Q + R] != static_cast<int32_t>(n)) {
                bad_rest.set(static_cast<int64_t>(b));
                return;
            }
            // y = neighbor(rev q, n) fluid must have neighbor(q, y) = n; over all q this
            // also covers the downstream side (t = neighbor(q, n) with neighbor(rev q, t) = n)
            for (int q = 0; q < R; ++q) {
                const int y = nbr[n * Q + rev_dir(Q, q)];
                if (y != 0 && ty[y] > 1 && nbr[static_cast<size_t>(y) * Q + q] != static_cast<int32_t>(n)) {
                    bad_sym.set(static_cast<int64_t>(b) * 32 + q);
                    return;
                }
            }
        }
    });
    if (bad_rest.any()) {
        err = "rest-direction neighbour of node " + std::to_string(d->bulk[bad_rest.get()]) + " is not the node itself";
        return BCLBM_ERR_TABLE;
    }
    if (bad_sym.any()) {
        const int64_t v = bad_sym.get();
        err = "neighbour table not symmetric at node " + std::to_string(d->bulk[v / 32]) + " direction " +
              std::to_string(v % 32);
        return BCLBM_ERR_TABLE;
    }
    return BCLBM_OK;
}

// The plan of the common case, checked on the host only as far as the host must:
// a single-phase descriptor whose bulk list is the contiguous, increasing run
// bulk[0] .. bulk[0] + n_bulk - 1 (vtklb.py numbers the fluid nodes first), kept in
// reference order.  Slot s then holds node bulk[0] + s, and bclbm_create runs every
// table check (neighbour ids in range, node types against the bulk list, rest
// neighbour, one-to-one stream map) on the device over the uploaded rows.  Returns
// -1 when the bulk list is not such a run.
int validate_affine(const bclbm_desc* d, Plan& p) {
    if (!d || !d->bulk || d->n_bulk < 1 || d->n_nodes < 2) return -1;
    const int N = d->n_nodes, nb = d->n_bulk;
    const int64_t b0 = d->bulk[0];
    if (b0 < 1 || b0 + nb > N) return -1;
    FirstBad bad;
    parallel_for(static_cast<size_t>(nb), [&](size_t k0, size_t k1) {
        for (size_t k = k0; k < k1; ++k)
            if (d->bulk[k] != b0 + static_cast<int64_t>(k)) {
                bad.set(static_cast<int64_t>(k));
                return;
            }
    });
    if (bad.any()) return -1;
    p.nfields = 1;
    p.nf = nb;
    p.nf_pad = (nb + 63) / 64 * 64;
    p.ns = 0;
    return BCLBM_OK;
}

size_t footprint_bytes(const bclbm_desc* d, const Plan& p) {
    const int Q = d->lattice_q, D = Q == 9 ? 2 : 3;
    const size_t pad = static_cast<size_t>(p.nf_pad);
    size_t b = 2 * static_cast<size_t>(p.nfields) * Q * pad * store_bytes(d->precision);  // two population buffers
    b += static_cast<size_t>(Q - 1) * pad * 4;                                             // neighbour table
    b += (static_cast<size_t>(p.nfields) + D) * pad * 8;                                   // macros
    b += pad * 4;                                                                          // slot -> bulk
    if (d->collision == BCLBM_RK)                                                           // colour field
        b += (static_cast<size_t>(p.nf) + p.ns + 1) * (d->precision == BCLBM_F64 ? 8 : 12);
    if (d->flags & BCLBM_FLAG_LAGGED_COLOUR) b += (static_cast<size_t>(p.nf) + p.ns + 1) * 4;  // its second copy
    b += (static_cast<size_t>(grid_for(p.nf)) * 6 + 64) * 8;                               // reduction partials
    if (d->collision == BCLBM_LINKS) b += pad * 12 + pad * 8;  // info, u_store index, force; labelled-node lists
    return b;
}

template <int Q>
fx::Consts fixed_consts_q(const bclbm_handle* h) {
    return fx::make_consts<Q>(h->trt, h->tau[0], h->tau[1], h->force);
}

fx::Consts fixed_consts(const bclbm_handle* h) { return h->q == 9 ? fixed_consts_q<9>(h) : fixed_consts_q<19>(h); }

}  // namespace

StepArgs bclbm::handle_args(const bclbm_handle* h) {
    StepArgs a;
    std::memset(&a, 0, sizeof(a));
    a.L.nf = h->nf;
    a.L.nf_pad = h->nf_pad;
    a.L.ns = h->ns;
    a.L.nbr = h->collision == BCLBM_RK ? h->d_nbr : nullptr;
    a.L.pull = h->collision == BCLBM_RK ? nullptr : h->d_nbr;
    for (int q = 0; q < 19; ++q) a.L.ghost_src[q] = h->ghost_src[q];
    a.cg = h->d_cg;
    a.cgf = h->d_cgf;
    a.cgf_out = h->d_cgf2;
    a.cgx = h->fx_storage ? reinterpret_cast<int64_t*>(h->d_cg) : nullptr;
    a.params = h->d_params;
    a.tau = h->tau[0];
    a.tau_anti = h->tau[1];
    // the reference computes 1.0 / tau and (1 - 0.5 / tau) inside its collision functions
    a.tau_inv = 1.0 / h->tau[0];
    a.tf = (1 - 0.5 / h->tau[0]);
    a.tauA_inv = 1.0 / h->tau[1];
    a.taf = (1 - 0.5 / h->tau[1]);
    const double c2 = 1.0 / 3.0;
    a.nu0inv = 1.0 / (c2 * (h->tau[0] - 0.5));
    a.nu1inv = 1.0 / (c2 * (h->tau[1] - 0.5));
    a.sigma = h->sigma;
    a.beta = h->beta;
    a.rho_ref = h->rho_ref;
    a.scale = h->scale;
    a.inv_scale = 1.0 / h->scale;
    a.partials = h->d_partials;
    a.n_bulk = h->nf;
    a.f_tau_inv = static_cast<float>(a.tau_inv);
    a.f_tauA_inv = static_cast<float>(a.tauA_inv);
    a.f_tf = static_cast<float>(a.tf);
    a.f_taf = static_cast<float>(a.taf);
    a.f_rho_ref = static_cast<float>(a.rho_ref);
    a.f_scale = static_cast<float>(a.scale);
    a.f_inv_scale = static_cast<float>(a.inv_scale);
    a.f_nu0inv = static_cast<float>(a.nu0inv);
    a.f_nu1inv = static_cast<float>(a.nu1inv);
    a.f_sigma = static_cast<float>(a.sigma);
    a.f_beta = static_cast<float>(a.beta);
    a.fx_flag = h->d_params ? &h->d_params->fx_overflow : nullptr;
    a.fxk = fixed_consts(h);
    a.fxr = h->q == 9 ? fx::make_rk_consts<9>(a.nu0inv, a.nu1inv, a.sigma, a.beta)
                      : fx::make_rk_consts<19>(a.nu0inv, a.nu1inv, a.sigma, a.beta);
    return a;
}

namespace {

StepArgs make_args(const bclbm_handle* h) { return handle_args(h); }

LinksArgs links_args(const bclbm_handle* h, const StepArgs& a) {
    LinksArgs A;
    std::memset(&A, 0, sizeof(A));
    A.s = a;
    A.info = h->d_info;
    A.pidx = h->d_pidx;
    A.force_on = h->d_force_on;
    A.ustore = h->d_ustore;
    A.npress = h->npress;
    A.rho_w = h->rho_w;
    A.lab_slot = h->d_lab_slot;
    A.lab_start = h->d_lab_start;
    A.lab_val = h->d_lab_val;
    A.lab_g = h->d_lab_g;
    A.lab_q = h->d_lab_q;
    A.nlab = h->nlab;
    A.nlabeled = h->nlabeled;
    A.flux_slot = h->d_flux_slot;
    A.flux_phase = h->d_flux_phase;
    A.nflux = h->nflux;
    A.flux_out = h->d_flux_out;
    A.f_rho_w = static_cast<float>(h->rho_w);
    A.f_dw = static_cast<float>(2.0 * (h->rho_w - h->rho_ref));
    for (int c = 0; c < 3; ++c) A.x_wrho[c] = fx::param((c == 0 ? 12.0 : c == 1 ? 2.0 : 1.0) / 36.0 * h->rho_w);
    return A;
}

// FP64 populations -> the int64 fixed-point storage of the default F64 step (the
// conversion the step itself used to make on every load); out-of-range values
// raise the fixed-point overflow flag
__global__ void k_encode_fx(const double* __restrict__ f, int64_t* __restrict__ out, size_t n, int* flag) {
    const size_t k = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (k >= n) return;
    unsigned emax = 0;
    out[k] = fx::load_f64_hw(f[k], emax);
    if (emax >= fx::kLoadEmaxLimit) atomicOr(flag, 1);
}

__global__ void k_encode(const double* __restrict__ f, void* out, int nf, int nf_pad, int Q, int nfields,
                         int precision, double rho_ref, double scale) {
    // f: FP64 [Q][nf_pad][nfields] reference populations -> storage format (same layout)
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nf) return;
    for (int q = 0; q < Q; ++q) {
        const double w = Q == 9 ? (q == 8 ? 16.0 / 36.0 : (q % 2 == 0 ? 4.0 / 36.0 : 1.0 / 36.0))
                                : (q == 18 ? 12.0 / 36.0 : ((q % 9) < 3 ? 2.0 / 36.0 : 1.0 / 36.0));
        const size_t k = (static_cast<size_t>(q) * nf_pad + i) * nfields;
        double v0, v1 = 0.0;
        if (nfields == 1) {
            v0 = (f[k] - w * rho_ref) / w * scale;
        } else {
            v0 = (f[k] + f[k + 1] - w * rho_ref) / w * scale;
            v1 = (f[k] - f[k + 1]) / w * scale;
        }
        switch (precision) {
            case BCLBM_F32:
                static_cast<float*>(out)[k] = static_cast<float>(v0);
                if (nfields == 2) static_cast<float*>(out)[k + 1] = static_cast<float>(v1);
                break;
            case BCLBM_F16:
                static_cast<__half*>(out)[k] = __double2half(v0);
                if (nfields == 2) static_cast<__half*>(out)[k + 1] = __double2half(v1);
                break;
            case BCLBM_BF16:
                static_cast<__nv_bfloat16*>(out)[k] = __double2bfloat16(v0);
                if (nfields == 2) static_cast<__nv_bfloat16*>(out)[k + 1] = __double2bfloat16(v1);
                break;
        }
    }
}

struct GhostSrc {
    int32_t v[19];
};

// The resolved pull table of a single-phase instance, built on the device from the
// reference's neighbour rows of the bulk nodes (rows [n_bulk][Q], uploaded as they
// are): for slot s and direction q the element (row x stride + slot) that streams
// into s along c_q -- the upstream fluid slot, the node's own reversed value
// (bounce-back) or the last bulk node's push into node 0.
__global__ void k_build_pull(const int32_t* __restrict__ rows, const int32_t* __restrict__ slot_bulk,
                             const int16_t* __restrict__ types, const int32_t* __restrict__ ext_of_node,
                             GhostSrc ghost, int32_t* __restrict__ tab, int nf, int nf_pad, int Q) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nf) return;
    const int32_t* row = rows + static_cast<size_t>(slot_bulk[s]) * Q;
    const int R = Q - 1;
    for (int q = 0; q < R; ++q) {
        const int rq = Q == 9 ? (q + 4) % 8 : (q + 9) % 18;
        const int y = row[rq];
        int64_t e;
        if (y != 0 && types[y] > 1) e = static_cast<int64_t>(q) * nf_pad + ext_of_node[y];
        else if (y == 0) e = static_cast<int64_t>(rq) * nf_pad + ghost.v[rq];
        else e = static_cast<int64_t>(rq) * nf_pad + s;
        tab[static_cast<size_t>(q) * nf_pad + s] = static_cast<int32_t>(e);
    }
}

// The stream-map checks of validate_and_plan on the device, for a contiguous bulk
// list (rows [n_bulk][Q] of nodes b0 .. b0 + n_bulk - 1): the rest neighbour of each
// fluid node is the node itself, and a fluid upstream neighbour y = neighbor(rev q, n)
// has neighbor(q, y) = n.  bad[0] / bad[1]: the smallest failing bulk index.
__global__ void k_check_links(const int32_t* __restrict__ rows, const int16_t* __restrict__ types, int b0, int nf,
                              int Q, int* bad) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nf) return;
    const int n = b0 + b, R = Q - 1;
    const int32_t* row = rows + static_cast<size_t>(b) * Q;
    if (row[R] != n) {
        atomicMin(bad, b);
        return;
    }
    for (int q = 0; q < R; ++q) {
        const int rq = Q == 9 ? (q + 4) % 8 : (q + 9) % 18;
        const int y = row[rq];
        if (y != 0 && types[y] > 1 && rows[static_cast<size_t>(y - b0) * Q + q] != n) {
            atomicMin(bad + 1, b);
            return;
        }
    }
}

// The table checks of an affine handle (bulk list = nodes b0 .. b0 + nf - 1) on the
// device, one thread per node and per bulk row; every access is bounds-checked
// before it indexes anything.  bad[2]: smallest bulk index whose node is not
// fluid (type 2 or 3); bad[3]: smallest fluid node outside the bulk list;
// bad[4]: smallest bulk index with a neighbour id out of [0, n_nodes).  ghost[p]:
// largest bulk index whose neighbour along c_p is node 0 (the ghost source).
// Also writes slot_bulk[s] = s.
__global__ void k_prepare_affine(const int32_t* __restrict__ rows, const int16_t* __restrict__ types, int n_nodes,
                                 int b0, int nf, int Q, int* bad, int* ghost, int32_t* slot_bulk) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 1 && t < n_nodes) {
        const int ty = types[t];
        const bool inside = t >= b0 && t - b0 < nf;
        if (inside && ty != 2 && ty != 3) atomicMin(bad + 2, t - b0);
        if (!inside && ty > 1) atomicMin(bad + 3, t);
    }
    if (t < nf) {
        slot_bulk[t] = t;
        const int32_t* row = rows + static_cast<size_t>(t) * Q;
        for (int q = 0; q < Q; ++q) {
            const int y = row[q];
            if (y < 0 || y >= n_nodes) atomicMin(bad + 4, t);
            else if (y == 0 && q < Q - 1) atomicMax(ghost + q, t);
        }
    }
}

// k_check_links for an affine handle: a node y is fluid exactly when b0 <= y <
// b0 + nf (k_prepare_affine checks the types against that), so no node type is
// read and no row outside the uploaded bulk rows is indexed.  bad[0] / bad[1]:
// smallest bulk index with a wrong rest neighbour / an asymmetric link.
__global__ void k_check_links_affine(const int32_t* __restrict__ rows, int b0, int nf, int Q, int* bad) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nf) return;
    const int n = b0 + b, R = Q - 1;
    const int32_t* row = rows + static_cast<size_t>(b) * Q;
    if (row[R] != n) {
        atomicMin(bad, b);
        return;
    }
    for (int q = 0; q < R; ++q) {
        const int rq = Q == 9 ? (q + 4) % 8 : (q + 9) % 18;
        const int y = row[rq];
        if (y >= b0 && y - b0 < nf && rows[static_cast<size_t>(y - b0) * Q + q] != n) {
            atomicMin(bad + 1, b);
            return;
        }
    }
}

// k_build_pull for an affine handle: upstream fluid y is slot y - b0; node 0 gives
// the ghost source (device array from k_prepare_affine); anything else is a wall
// (bounce-back of the node's own reversed value).  An out-of-range id (reported
// by k_prepare_affine) is treated as a wall and never dereferenced.
__global__ void k_build_pull_affine(const int32_t* __restrict__ rows, const int* __restrict__ ghost,
                                    int32_t* __restrict__ tab, int b0, int nf, int nf_pad, int Q) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nf) return;
    const int32_t* row = rows + static_cast<size_t>(s) * Q;
    const int R = Q - 1;
    for (int q = 0; q < R; ++q) {
        const int rq = Q == 9 ? (q + 4) % 8 : (q + 9) % 18;
        const int y = row[rq];
        int64_t e;
        if (y >= b0 && y - b0 < nf) e = static_cast<int64_t>(q) * nf_pad + (y - b0);
        else if (y == 0) e = static_cast<int64_t>(rq) * nf_pad + max(ghost[rq], 0);
        else e = static_cast<int64_t>(rq) * nf_pad + s;
        tab[static_cast<size_t>(q) * nf_pad + s] = static_cast<int32_t>(e);
    }
}

// The initial populations straight from the reference's AoS rows of the bulk nodes
// (aos [n_bulk][nfields][Q], uploaded as they are) into the storage format, slot
// by slot: the transpose runs on the device instead of the host.
__global__ void k_upload_aos(const double* __restrict__ aos, const int32_t* __restrict__ slot_bulk, void* out,
                             int nf, int nf_pad, int Q, int nfields, int mode, int precision, double rho_ref,
                             double scale, int* flag) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nf) return;
    const size_t es = static_cast<size_t>(nfields) * Q;
    const double* row = aos + static_cast<size_t>(slot_bulk[i]) * es;
    unsigned emax = 0;
    for (int q = 0; q < Q; ++q) {
        // storage layout [Q][nf_pad][nfields]
        const size_t k = (static_cast<size_t>(q) * nf_pad + i) * nfields;
        if (mode == 0) {  // FP64 storage
            for (int f = 0; f < nfields; ++f) static_cast<double*>(out)[k + f] = row[f * Q + q];
            continue;
        }
        if (mode == 1) {  // int64 fixed point
            for (int f = 0; f < nfields; ++f) static_cast<int64_t*>(out)[k + f] = fx::load_f64_hw(row[f * Q + q], emax);
            continue;
        }
        const double w = Q == 9 ? (q == 8 ? 16.0 / 36.0 : (q % 2 == 0 ? 4.0 / 36.0 : 1.0 / 36.0))
                                : (q == 18 ? 12.0 / 36.0 : ((q % 9) < 3 ? 2.0 / 36.0 : 1.0 / 36.0));
        double v0, v1 = 0.0;
        if (nfields == 1) {
            v0 = (row[q] - w * rho_ref) / w * scale;
        } else {
            v0 = (row[q] + row[Q + q] - w * rho_ref) / w * scale;
            v1 = (row[q] - row[Q + q]) / w * scale;
        }
        switch (precision) {
            case BCLBM_F32:
                static_cast<float*>(out)[k] = static_cast<float>(v0);
                if (nfields == 2) static_cast<float*>(out)[k + 1] = static_cast<float>(v1);
                break;
            case BCLBM_F16:
                static_cast<__half*>(out)[k] = __double2half(v0);
                if (nfields == 2) static_cast<__half*>(out)[k + 1] = __double2half(v1);
                break;
            case BCLBM_BF16:
                static_cast<__nv_bfloat16*>(out)[k] = __double2bfloat16(v0);
                if (nfields == 2) static_cast<__nv_bfloat16*>(out)[k + 1] = __double2bfloat16(v1);
                break;
        }
    }
    if (mode == 1 && emax >= fx::kLoadEmaxLimit) atomicOr(flag, 1);
}

// rho [nfields][pad] and vel [nd][pad] of the last step (slot order) -> the reference's
// node-major rows of the bulk nodes: rho [n_bulk][nfields] then vel [n_bulk][nd]
__global__ void k_macros_aos(const double* __restrict__ rho, const double* __restrict__ vel,
                             const int32_t* __restrict__ slot_bulk, double* __restrict__ out, int nf, int nf_pad,
                             int nfields, int nd) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nf) return;
    const size_t b = static_cast<size_t>(slot_bulk[s]);
    for (int k = 0; k < nfields; ++k) out[b * nfields + k] = rho[static_cast<size_t>(k) * nf_pad + s];
    double* ov = out + static_cast<size_t>(nf) * nfields;
    for (int d = 0; d < nd; ++d) ov[b * nd + d] = vel[static_cast<size_t>(d) * nf_pad + s];
}

// The handle's device buffers are stream-ordered allocations on its own stream
// (cudaMallocAsync / cudaFreeAsync): creating or destroying a handle does not
// synchronise the device, which matters when a batch creates and retires handles
// while other instances step (cudaFree synchronises, even for a null pointer).
void free_dev(bclbm_handle* h, void* p) {
    if (h->stream) cudaFreeAsync(p, h->stream);
    else cudaFree(p);
}

void free_all(bclbm_handle* h) {
    if (h->pops[0]) free_dev(h, h->pops[0]);
    if (h->pops[1]) free_dev(h, h->pops[1]);
    if (h->d_nbr) free_dev(h, h->d_nbr);
    if (h->d_slot_bulk) free_dev(h, h->d_slot_bulk);
    if (h->d_rho) free_dev(h, h->d_rho);
    if (h->d_vel) free_dev(h, h->d_vel);
    if (h->d_cg) free_dev(h, h->d_cg);
    if (h->d_cgf) free_dev(h, h->d_cgf);
    if (h->d_cgf2) free_dev(h, h->d_cgf2);
    if (h->d_params) free_dev(h, h->d_params);
    if (h->d_partials) free_dev(h, h->d_partials);
    if (h->d_red) free_dev(h, h->d_red);
    if (h->d_gather) free_dev(h, h->d_gather);
    if (h->d_info) free_dev(h, h->d_info);
    if (h->d_pidx) free_dev(h, h->d_pidx);
    if (h->d_force_on) free_dev(h, h->d_force_on);
    if (h->d_ustore) free_dev(h, h->d_ustore);
    if (h->d_lab_slot) free_dev(h, h->d_lab_slot);
    if (h->d_lab_start) free_dev(h, h->d_lab_start);
    if (h->d_lab_val) free_dev(h, h->d_lab_val);
    if (h->d_lab_g) free_dev(h, h->d_lab_g);
    if (h->d_lab_q) free_dev(h, h->d_lab_q);
    if (h->d_flux_slot) free_dev(h, h->d_flux_slot);
    if (h->d_flux_phase) free_dev(h, h->d_flux_phase);
    if (h->d_flux_out) free_dev(h, h->d_flux_out);
    if (h->stage) cudaFreeHost(h->stage);
    if (h->stage_cgf) cudaFreeHost(h->stage_cgf);
    if (h->stage_event) cudaEventDestroy(h->stage_event);
    if (h->stream) cudaStreamDestroy(h->stream);
}

int run_gather(bclbm_handle* h) {
    const size_t n = static_cast<size_t>(h->nf) * h->nfields * h->q;
    if (!h->d_gather) CUDA_TRY(h, pool_malloc(reinterpret_cast<void**>(&h->d_gather), n * sizeof(double), h->stream));
    StepArgs a = make_args(h);
    a.src = h->pops[h->cur];
    if (h->collision == BCLBM_LINKS) {
        CUDA_TRY(h, launch_links_gather(h->precision, h->exact, h->fx_storage, !h->state_post, links_args(h, a), h->d_slot_bulk,
                                        h->d_gather, h->stream));
        return BCLBM_OK;
    }
    CUDA_TRY(h, launch_gather(h->q, h->fx_storage ? kFX : h->precision, h->nfields, !h->state_post, a, h->d_slot_bulk,
                              h->d_gather,
                              h->stream));
    return BCLBM_OK;
}

}  // namespace

extern "C" {

const char* bclbm_error(int status) {
    switch (status) {
        case BCLBM_OK: return "ok";
        case BCLBM_ERR_INVALID: return "invalid argument";
        case BCLBM_ERR_TABLE: return "inconsistent neighbour table or node types";
        case BCLBM_ERR_NOMEM: return "out of memory";
        case BCLBM_ERR_CUDA: return "CUDA error";
        case BCLBM_ERR_UNSUPPORTED: return "unsupported combination";
        case BCLBM_ERR_NONFINITE: return "non-finite populations";
        case BCLBM_ERR_BUDGET: return "request exceeds the HBM budget";
        case BCLBM_ERR_NOCUDA: return "no CUDA device";
        default: return "unknown status";
    }
}

const char* bclbm_last_error(const bclbm_handle* h) { return h ? h->last_error.c_str() : ""; }

int64_t bclbm_launch_count(void) { return launch_counter().load(); }

int bclbm_footprint(const bclbm_desc* desc, size_t* bytes) {
    // sizes only (admission control is called often): the bulk count fixes every
    // buffer of a single-phase instance; two-phase instances also hold the colour of
    // the solids their fluid nodes see.  bclbm_create validates the tables.
    if (!bytes || !desc) return BCLBM_ERR_INVALID;
    const int Q = desc->lattice_q;
    if ((Q != 9 && Q != 19) || desc->n_nodes < 2 || desc->n_bulk < 1 || desc->n_bulk >= desc->n_nodes ||
        desc->collision < BCLBM_BGK || desc->collision > BCLBM_LINKS || desc->precision < BCLBM_F64 ||
        desc->precision > BCLBM_BF16)
        return BCLBM_ERR_INVALID;
    Plan p;
    p.nf = desc->n_bulk;
    p.nf_pad = (p.nf + 63) / 64 * 64;
    p.nfields = desc->collision == BCLBM_RK ? 2 : 1;
    if (desc->collision == BCLBM_RK) {
        if (!desc->neigh || !desc->types || !desc->bulk) return BCLBM_ERR_INVALID;
        const int N = desc->n_nodes;
        std::vector<uint8_t> used(N, 0);
        FirstBad bad;
        parallel_for(static_cast<size_t>(p.nf), [&](size_t b0, size_t b1) {
            for (size_t b = b0; b < b1; ++b) {
                const int n = desc->bulk[b];
                if (n < 1 || n >= N) {
                    bad.set(static_cast<int64_t>(b));
                    return;
                }
                for (int q = 0; q < Q; ++q) {
                    const int y = desc->neigh[static_cast<size_t>(n) * Q + q];
                    if (y < 0 || y >= N) {
                        bad.set(static_cast<int64_t>(b));
                        return;
                    }
                    if (y != 0 && desc->types[y] < 2) __atomic_store_n(&used[y], static_cast<uint8_t>(1), __ATOMIC_RELAXED);
                }
            }
        });
        if (bad.any()) return BCLBM_ERR_TABLE;
        int64_t ns = 0;
        for (int n = 1; n < N; ++n) ns += used[n];
        p.ns = static_cast<int>(ns);
    }
    *bytes = footprint_bytes(desc, p);
    return BCLBM_OK;
}

int bclbm_create(const bclbm_desc* d, bclbm_handle** out) {
    BCLBM_TRACE("bclbm_create");
    if (!out) return BCLBM_ERR_INVALID;
    *out = nullptr;
    Plan p;
    std::string err;
    int ndev = 0;
    const bool have_gpu = cudaGetDeviceCount(&ndev) == cudaSuccess && ndev > 0;
    // single-phase with a contiguous bulk list on a machine with a GPU: the table is
    // resolved and the stream map checked on the device (k_build_pull, k_check_links)
    const bool device_links = have_gpu && d && d->bulk && d->n_bulk > 0 && d->collision != BCLBM_RK &&
                              d->collision != BCLBM_LINKS &&
                              static_cast<int64_t>(d->bulk[d->n_bulk - 1]) - d->bulk[0] + 1 == d->n_bulk;
    // the common case: the bulk list is one run in reference order; its tables are
    // checked and resolved on the device and the node <-> slot maps are implicit
    const bool affine = device_links && !(d->flags & BCLBM_FLAG_SFC_ORDER) && validate_affine(d, p) == BCLBM_OK;
    int rc = affine ? validate_descriptor(d, err) : validate_and_plan(d, p, err, true, device_links);
    if (rc) {
        std::fprintf(stderr, "bclbm_create: %s\n", err.c_str());
        return rc;
    }
    if (!d->f_init) return BCLBM_ERR_INVALID;
    if (d->collision == BCLBM_RK && !d->rho_init) return BCLBM_ERR_INVALID;
    if (!have_gpu) return BCLBM_ERR_NOCUDA;
    bclbm_handle* h = new (std::nothrow) bclbm_handle();
    if (!h) return BCLBM_ERR_NOMEM;
    h->q = d->lattice_q;
    h->nd = h->q == 9 ? 2 : 3;
    h->nfields = p.nfields;
    h->collision = d->collision;
    h->precision = d->precision;
    h->flags = d->flags;
    h->exact = (d->flags & BCLBM_FLAG_EXACT) != 0;
    h->trt = d->collision == BCLBM_TRT;
    h->fma64 = (d->flags & BCLBM_FLAG_FP64_FMA) != 0;
    h->fx_storage = d->precision == BCLBM_F64 && !h->exact && !h->fma64;
    h->lagged = (d->flags & BCLBM_FLAG_LAGGED_COLOUR) != 0;
    h->rho_w = d->rho_w != 0.0 ? d->rho_w : 1.0;
    h->flux = d->collision == BCLBM_RK && d->flux_control != 0;
    h->mass_fix = d->collision == BCLBM_RK && d->precision != BCLBM_F64 && !(d->flags & BCLBM_FLAG_NO_MASS_FIX);
    h->n_nodes = d->n_nodes;
    h->footprint = footprint_bytes(d, p);
    h->nf = p.nf;
    h->nf_pad = p.nf_pad;
    h->ns = p.ns;
    h->tau[0] = d->tau[0];
    h->tau[1] = d->collision == BCLBM_BGK ? d->tau[0] : d->tau[1];
    h->sigma = d->sigma;
    h->beta = d->beta;
    h->mom_x = d->mom_x;
    h->rho_ref = d->rho_ref > 0 ? d->rho_ref : 1.0;
    h->scale = d->store_scale > 0 ? d->store_scale : (d->precision == BCLBM_F16 ? 4096.0 : 1.0);
    for (int k = 0; k < 3; ++k) h->force[k] = d->force[k];
    h->affine = affine;
    h->bulk0 = d->bulk[0];
    if (!affine) {
        h->slot_node = std::move(p.slot_node);
        h->slot_bulk = std::move(p.slot_bulk);
        h->bulk.assign(d->bulk, d->bulk + d->n_bulk);
        h->solid_node = std::move(p.solid_node);
    }
    h->bulk_contiguous = static_cast<int64_t>(d->bulk[d->n_bulk - 1]) - d->bulk[0] + 1 == d->n_bulk;
    cudaGetDevice(&h->device);

    const int Q = h->q, D = h->nd, R = Q - 1;
    const size_t pad = static_cast<size_t>(h->nf_pad);
    auto cleanup = [&](int code) {
        free_all(h);
        delete h;
        return code;
    };
#define CREATE_TRY(expr)                                                                \
    do {                                                                                \
        cudaError_t e_ = (expr);                                                        \
        if (e_ != cudaSuccess) {                                                        \
            std::fprintf(stderr, "bclbm_create: %s: %s\n", #expr, cudaGetErrorString(e_)); \
            return cleanup(e_ == cudaErrorMemoryAllocation ? BCLBM_ERR_NOMEM : BCLBM_ERR_CUDA); \
        }                                                                               \
    } while (0)

    // ghost sources: last bulk node (bulk order) whose neighbour along c_p is node 0
    // (an affine handle finds them on the device, k_prepare_affine)
    for (int pdir = 0; pdir < 19; ++pdir) h->ghost_src[pdir] = 0;
    if (!affine) {
        std::vector<int32_t> slot_of_bulk(h->nf);
        parallel_for(static_cast<size_t>(h->nf), [&](size_t s0, size_t s1) {
            for (size_t s = s0; s < s1; ++s) slot_of_bulk[h->slot_bulk[s]] = static_cast<int32_t>(s);
        });
        std::atomic<int> last[19];
        for (auto& x : last) x.store(-1);
        parallel_for(static_cast<size_t>(h->nf), [&](size_t b0, size_t b1) {
            int loc[19];
            for (int k = 0; k < 19; ++k) loc[k] = -1;
            for (size_t b = b0; b < b1; ++b) {
                const int32_t* row = d->neigh + static_cast<size_t>(d->bulk[b]) * Q;
                for (int pdir = 0; pdir < R; ++pdir)
                    if (row[pdir] == 0) loc[pdir] = static_cast<int>(b);
            }
            for (int pdir = 0; pdir < R; ++pdir) {
                int cur = last[pdir].load();
                while (loc[pdir] > cur && !last[pdir].compare_exchange_weak(cur, loc[pdir])) {
                }
            }
        });
        for (int pdir = 0; pdir < R; ++pdir)
            if (last[pdir].load() >= 0) h->ghost_src[pdir] = slot_of_bulk[last[pdir].load()];
    }
    std::vector<int32_t> tab;
    bool device_table = false;
    LinksPlan lp;
    if (h->collision == BCLBM_LINKS) {
        std::string lerr;
        if (static_cast<size_t>(Q) * pad > static_cast<size_t>(INT32_MAX)) {
            std::fprintf(stderr, "bclbm_create: %d fluid nodes exceed the int32 pull table\n", h->nf);
            free_all(h);
            delete h;
            return BCLBM_ERR_UNSUPPORTED;
        }
        const int lrc = links_plan(d, h->slot_node, h->ghost_src, pad, lp, tab, lerr);
        if (lrc != BCLBM_OK) {
            std::fprintf(stderr, "bclbm_create: %s\n", lerr.c_str());
            free_all(h);
            delete h;
            return lrc;
        }
        h->npress = lp.npress;
        h->nlab = lp.nlab;
        h->nlabeled = static_cast<int>(lp.lab_slot.size());
        h->nflux = static_cast<int>(lp.flux_slot.size());
        h->force_on_sum = lp.force_on_sum;
    } else if (h->collision == BCLBM_RK) {
        // extended neighbour table in device numbering (pull + colour gradient)
        tab.assign(static_cast<size_t>(R) * pad, static_cast<int32_t>(h->nf + h->ns));
        parallel_for(static_cast<size_t>(h->nf), [&](size_t s0, size_t s1) {
            for (size_t s = s0; s < s1; ++s) {
                const size_t n = static_cast<size_t>(h->slot_node[s]);
                for (int q = 0; q < R; ++q) tab[static_cast<size_t>(q) * pad + s] = p.ext_of_node[d->neigh[n * Q + q]];
            }
        });
    } else {
        // resolved pull table: element index (row * pad + slot) of the post-collision
        // value that streams into slot s along c_q (fluid upstream, wall, or ghost)
        if (static_cast<size_t>(Q) * pad > static_cast<size_t>(INT32_MAX)) {
            std::fprintf(stderr, "bclbm_create: %d fluid nodes exceed the int32 pull table\n", h->nf);
            free_all(h);
            delete h;
            return BCLBM_ERR_UNSUPPORTED;
        }
        if (device_links) {
            device_table = true;  // built by k_build_pull once the buffers exist
        } else {
            tab.assign(static_cast<size_t>(R) * pad, 0);
            parallel_for(static_cast<size_t>(h->nf), [&](size_t s0, size_t s1) {
                for (size_t s = s0; s < s1; ++s) {
                    const size_t n = static_cast<size_t>(h->slot_node[s]);
                    for (int q = 0; q < R; ++q) {
                        const int rq = rev_dir(Q, q);
                        const int y = d->neigh[n * Q + rq];
                        int64_t e;
                        if (y != 0 && d->types[y] > 1) e = static_cast<int64_t>(q) * pad + p.ext_of_node[y];
                        else if (y == 0) e = static_cast<int64_t>(rq) * pad + h->ghost_src[rq];
                        else e = static_cast<int64_t>(rq) * pad + static_cast<int64_t>(s);
                        tab[static_cast<size_t>(q) * pad + s] = static_cast<int32_t>(e);
                    }
                }
            });
        }
    }
    CREATE_TRY(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    const size_t sb = store_bytes(h->precision);
    const size_t pop_bytes = static_cast<size_t>(h->nfields) * Q * pad * sb;
    CREATE_TRY(pool_malloc(reinterpret_cast<void**>(&h->pops[0]), pop_bytes, h->stream));
    CREATE_TRY(pool_malloc(reinterpret_cast<void**>(&h->pops[1]), pop_bytes, h->stream));
    const size_t ntab = device_table ? static_cast<size_t>(R) * pad : tab.size();
    CREATE_TRY(pool_malloc(reinterpret_cast<void**>(&h->d_nbr), ntab * sizeof(int32_t), h->stream));
    if ((h->collision == BCLBM_BGK || h->collision == BCLBM_TRT) && ntab == static_cast<size_t>(R) * pad) {
        // the native-FP64 steps after the first stage the pull table through shared
        // memory with the tensor copy engine; without the driver's encoder they read it
        // directly
        h->pull_map_ok = encode_table_map(h->d_nbr, static_cast<int>(pad), R, &h->pull_map) == cudaSuccess;
    }
    CREATE_TRY(pool_malloc(reinterpret_cast<void**>(&h->d_slot_bulk), pad * sizeof(int32_t), h->stream));
    CREATE_TRY(pool_malloc(reinterpret_cast<void**>(&h->d_rho), static_cast<size_t>(h->nfields) * pad * sizeof(double), h->stream));
    CREATE_TRY(pool_malloc(reinterpret_cast<void**>(&h->d_vel), static_cast<size_t>(D) * pad * sizeof(double), h->stream));
    CREATE_TRY(pool_malloc(reinterpret_cast<void**>(&h->d_params), sizeof(DevParams), h->stream));
    CREATE_TRY(pool_malloc(reinterpret_cast<void**>(&h->d_partials), (static_cast<size_t>(grid_for(h->nf)) * 6 + 64) * sizeof(double), h->stream));
    CREATE_TRY(pool_malloc(reinterpret_cast<void**>(&h->d_red), 16 * sizeof(double), h->stream));
    // the step parameters: body force, and for shifted two-phase storage the conserved
    // totals of the uploaded state
    auto build_params = [&]() {
        DevParams prm;
        std::memset(&prm, 0, sizeof(prm));
        for (int k = 0; k < 3; ++k) {
            prm.force[k] = h->force[k];
            prm.forcef[k] = static_cast<float>(h->force[k]);
            prm.forcex[k] = fx::param(h->force[k]);
        }
        if (h->mass_fix) {
            // the conserved totals of the uploaded state, sum over bulk nodes of
            // sum_q (f0 + f1) and sum_q (f0 - f1), in FP64 (fixed order per chunk)
            const size_t nb = static_cast<size_t>(d->n_bulk), Qs = static_cast<size_t>(h->q);
            std::vector<double> pt(64, 0.0), pc(64, 0.0);
            parallel_for(64, [&](size_t c0, size_t c1) {
                for (size_t c = c0; c < c1; ++c)
                    for (size_t b = nb * c / 64; b < nb * (c + 1) / 64; ++b) {
                        const double* fb = d->f_init + static_cast<size_t>(d->bulk[b]) * 2 * Qs;
                        for (size_t q = 0; q < Qs; ++q) {
                            pt[c] += fb[q] + fb[Qs + q];
                            pc[c] += fb[q] - fb[Qs + q];
                        }
                    }
            }, 1);
            for (int c = 0; c < 64; ++c) {
                prm.mass_target[0] += pt[c];
                prm.mass_target[1] += pc[c];
            }
        }
        return prm;
    };
    // The common case, a contiguous bulk list whose table is checked on the device: the
    // populations go up on a second stream while the neighbour rows are copied and checked,
    // and are converted after the checks; one synchronisation covers both.  The conversion
    // reads slot i = bulk index i (k_prepare_affine writes that map whatever the checks
    // find), so it stays in bounds when a check fails; DevParams goes up first, so that
    // the conversion's range flag is not overwritten.
    const bool early_pops = affine && h->bulk_contiguous && device_table;
    cudaStream_t side = nullptr;
    cudaEvent_t ev_alloc = nullptr, ev_copied = nullptr;
    double* early_tmp = nullptr;
    HostLock lock_f, lock_rows;
    // releases the second stream's objects (their pending work completes first) and,
    // stream-ordered, the staging buffer
    auto end_side = [&]() {
        if (early_tmp) cudaFreeAsync(early_tmp, h->stream);
        if (side) cudaStreamDestroy(side);
        if (ev_alloc) cudaEventDestroy(ev_alloc);
        if (ev_copied) cudaEventDestroy(ev_copied);
        early_tmp = nullptr;
        side = nullptr;
        ev_alloc = ev_copied = nullptr;
    };
    if (early_pops) {
        const DevParams prm = build_params();
        const size_t naos = static_cast<size_t>(h->nf) * h->nfields * Q;
        cudaError_t e = cudaMemcpyAsync(h->d_params, &prm, sizeof(prm), cudaMemcpyHostToDevice, h->stream);
        if (e == cudaSuccess) e = pool_malloc(reinterpret_cast<void**>(&early_tmp), naos * sizeof(double), h->stream);
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev_alloc, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev_copied, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventRecord(ev_alloc, h->stream);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(side, ev_alloc, 0);
        if (e == cudaSuccess) {
            const double* src = d->f_init + static_cast<size_t>(h->bulk0) * h->nfields * Q;
            lock_f.lock(src, naos * sizeof(double));
            e = cudaMemcpyAsync(early_tmp, src, naos * sizeof(double), cudaMemcpyHostToDevice, side);
        }
        if (e == cudaSuccess) e = cudaEventRecord(ev_copied, side);
        if (e != cudaSuccess) {
            if (side) cudaStreamSynchronize(side);
            lock_f.unlock();
            end_side();
        }
        CREATE_TRY(e);
    }
    if (!affine)
        CREATE_TRY(cudaMemcpyAsync(h->d_slot_bulk, h->slot_bulk.data(), h->nf * sizeof(int32_t),
                                   cudaMemcpyHostToDevice, h->stream));
    if (!device_table) {
        HostLock lk;
        lk.lock(tab.data(), tab.size() * sizeof(int32_t));
        CREATE_TRY(cudaMemcpyAsync(h->d_nbr, tab.data(), tab.size() * sizeof(int32_t), cudaMemcpyHostToDevice,
                                   h->stream));
        CREATE_TRY(cudaStreamSynchronize(h->stream));
        lk.unlock();
    } else {
        // the bulk nodes' neighbour rows and the node types go up as they are (and, for
        // a plan with explicit maps, the node -> slot map); the table is checked and
        // resolved on the device
        const size_t nrow = static_cast<size_t>(h->nf) * Q;
        int32_t* rows = nullptr;
        int16_t* dty = nullptr;
        int32_t* dext = nullptr;
        int* dbad = nullptr;  // [5] error slots, then [19] ghost sources
        cudaError_t e = pool_malloc(reinterpret_cast<void**>(&rows), nrow * sizeof(int32_t), h->stream);
        if (e == cudaSuccess) e = pool_malloc(reinterpret_cast<void**>(&dty), static_cast<size_t>(d->n_nodes) * sizeof(int16_t), h->stream);
        if (e == cudaSuccess && !affine)
            e = pool_malloc(reinterpret_cast<void**>(&dext), static_cast<size_t>(d->n_nodes) * sizeof(int32_t), h->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(h->d_nbr, 0, ntab * sizeof(int32_t), h->stream);
        if (e == cudaSuccess) {
            lock_rows.lock(d->neigh + static_cast<size_t>(h->bulk0) * Q, nrow * sizeof(int32_t));
            e = cudaMemcpyAsync(rows, d->neigh + static_cast<size_t>(h->bulk0) * Q, nrow * sizeof(int32_t),
                                cudaMemcpyHostToDevice, h->stream);
        }
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(dty, d->types, static_cast<size_t>(d->n_nodes) * sizeof(int16_t),
                                cudaMemcpyHostToDevice, h->stream);
        if (e == cudaSuccess && !affine)
            e = cudaMemcpyAsync(dext, p.ext_of_node.data(), static_cast<size_t>(d->n_nodes) * sizeof(int32_t),
                                cudaMemcpyHostToDevice, h->stream);
        int init[24];
        for (int k = 0; k < 5; ++k) init[k] = INT32_MAX;
        for (int k = 5; k < 24; ++k) init[k] = -1;
        int bad[24];
        std::memcpy(bad, init, sizeof(bad));
        if (e == cudaSuccess) e = pool_malloc(reinterpret_cast<void**>(&dbad), sizeof(init), h->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(dbad, init, sizeof(init), cudaMemcpyHostToDevice, h->stream);
        if (e == cudaSuccess) {
            if (affine) {
                k_prepare_affine<<<grid_for(std::max(d->n_nodes, h->nf)), kBlock, 0, h->stream>>>(
                    rows, dty, d->n_nodes, h->bulk0, h->nf, Q, dbad, dbad + 5, h->d_slot_bulk);
                k_check_links_affine<<<grid_for(h->nf), kBlock, 0, h->stream>>>(rows, h->bulk0, h->nf, Q, dbad);
                k_build_pull_affine<<<grid_for(h->nf), kBlock, 0, h->stream>>>(rows, dbad + 5, h->d_nbr, h->bulk0,
                                                                                h->nf, h->nf_pad, Q);
                launch_counter() += 3;
                if (early_pops) {  // the populations, once their copy on the second stream is done
                    e = cudaStreamWaitEvent(h->stream, ev_copied, 0);
                    if (e == cudaSuccess)
                        e = cudaMemsetAsync(h->pops[0], 0, static_cast<size_t>(h->nfields) * Q * pad *
                                                               store_bytes(h->precision), h->stream);
                    if (e == cudaSuccess) {
                        const int mode = h->fx_storage ? 1 : (h->precision == BCLBM_F64 ? 0 : 2);
                        k_upload_aos<<<grid_for(h->nf), kBlock, 0, h->stream>>>(
                            early_tmp, h->d_slot_bulk, h->pops[0], h->nf, h->nf_pad, Q, h->nfields, mode,
                            h->precision, h->rho_ref, h->scale, &h->d_params->fx_overflow);
                        launch_counter()++;
                    }
                }
            } else {
                k_check_links<<<grid_for(h->nf), kBlock, 0, h->stream>>>(rows, dty, h->bulk0, h->nf, Q, dbad);
                GhostSrc g;
                for (int k = 0; k < 19; ++k) g.v[k] = h->ghost_src[k];
                k_build_pull<<<grid_for(h->nf), kBlock, 0, h->stream>>>(rows, h->d_slot_bulk, dty, dext, g, h->d_nbr,
                                                                        h->nf, h->nf_pad, Q);
                launch_counter() += 2;
            }
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaGetLastError();
        end_side();
        if (e == cudaSuccess) e = cudaMemcpyAsync(bad, dbad, sizeof(bad), cudaMemcpyDeviceToHost, h->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
        else cudaStreamSynchronize(h->stream);  // the copies from the locked ranges are done either way
        lock_rows.unlock();
        lock_f.unlock();
        // stream-ordered frees: no device-wide synchronisation while other handles run
        if (rows) cudaFreeAsync(rows, h->stream);
        if (dty) cudaFreeAsync(dty, h->stream);
        if (dext) cudaFreeAsync(dext, h->stream);
        if (dbad) cudaFreeAsync(dbad, h->stream);
        CREATE_TRY(e);
        // reported in the host's order of checks: ids in range, bulk list, missing
        // fluid nodes, rest neighbour, stream-map symmetry
        const int32_t* nb_rows = d->neigh + static_cast<size_t>(h->bulk0) * Q;
        if (bad[4] != INT32_MAX) {
            int qd = 0;
            for (int q = 0; q < Q; ++q) {
                const int y = nb_rows[static_cast<size_t>(bad[4]) * Q + q];
                if (y < 0 || y >= d->n_nodes) {
                    qd = q;
                    break;
                }
            }
            std::fprintf(stderr, "bclbm_create: neighbour id out of range at entry %lld\n",
                         static_cast<long long>(h->bulk0 + bad[4]) * Q + qd);
            return cleanup(BCLBM_ERR_TABLE);
        }
        if (bad[2] != INT32_MAX) {
            std::fprintf(stderr, "bclbm_create: bulk node %d is not own-rank fluid\n", h->bulk0 + bad[2]);
            return cleanup(BCLBM_ERR_TABLE);
        }
        if (bad[3] != INT32_MAX) {
            std::fprintf(stderr, "bclbm_create: fluid node %d missing from the bulk list\n", bad[3]);
            return cleanup(BCLBM_ERR_TABLE);
        }
        if (bad[0] != INT32_MAX) {
            std::fprintf(stderr, "bclbm_create: rest-direction neighbour of node %d is not the node itself\n",
                         h->bulk0 + bad[0]);
            return cleanup(BCLBM_ERR_TABLE);
        }
        if (bad[1] != INT32_MAX) {
            const int n = h->bulk0 + bad[1];
            int qd = 0;
            for (int q = 0; q < Q - 1; ++q) {
                const int y = nb_rows[static_cast<size_t>(bad[1]) * Q + rev_dir(Q, q)];
                if (y >= h->bulk0 && y - h->bulk0 < h->nf && d->neigh[static_cast<size_t>(y) * Q + q] != n) {
                    qd = q;
                    break;
                }
            }
            std::fprintf(stderr, "bclbm_create: neighbour table not symmetric at node %d direction %d\n", n, qd);
            return cleanup(BCLBM_ERR_TABLE);
        }
        if (affine)
            for (int k = 0; k < R; ++k) h->ghost_src[k] = std::max(bad[5 + k], 0);
    }
    if (!early_pops) {
        const DevParams prm = build_params();
        CREATE_TRY(cudaMemcpyAsync(h->d_params, &prm, sizeof(prm), cudaMemcpyHostToDevice, h->stream));
    }
    if (h->collision == BCLBM_LINKS) {
        auto up = [&](auto** dst, const auto& v, size_t n_min) -> cudaError_t {
            using E = typename std::remove_reference<decltype(v)>::type::value_type;
            const size_t n = std::max(v.size(), n_min);
            cudaError_t e = pool_malloc(reinterpret_cast<void**>(dst), n * sizeof(E), h->stream);
            if (e == cudaSuccess && !v.empty())
                e = cudaMemcpyAsync(*dst, v.data(), v.size() * sizeof(E), cudaMemcpyHostToDevice, h->stream);
            return e;
        };
        CREATE_TRY(up(&h->d_info, lp.info, 1));
        CREATE_TRY(up(&h->d_pidx, lp.pidx, 1));
        CREATE_TRY(up(&h->d_force_on, lp.force_on, 1));
        CREATE_TRY(up(&h->d_lab_slot, lp.lab_slot, 1));
        CREATE_TRY(up(&h->d_lab_start, lp.lab_start, 2));
        CREATE_TRY(up(&h->d_lab_g, lp.lab_g, 1));
        CREATE_TRY(up(&h->d_flux_slot, lp.flux_slot, 1));
        CREATE_TRY(up(&h->d_flux_phase, lp.flux_phase, 1));
        CREATE_TRY(pool_malloc(reinterpret_cast<void**>(&h->d_ustore), std::max<size_t>(3 * static_cast<size_t>(h->npress), 1) * sizeof(double), h->stream));
        CREATE_TRY(pool_malloc(reinterpret_cast<void**>(&h->d_lab_val), std::max<size_t>(lp.lab_slot.size(), 1) * sizeof(double), h->stream));
        CREATE_TRY(pool_malloc(reinterpret_cast<void**>(&h->d_lab_q), (static_cast<size_t>(h->nlab) + 1) * sizeof(double), h->stream));
        CREATE_TRY(cudaMemsetAsync(h->d_lab_q, 0, (static_cast<size_t>(h->nlab) + 1) * sizeof(double), h->stream));
        CREATE_TRY(pool_malloc(reinterpret_cast<void**>(&h->d_flux_out), 2 * sizeof(double), h->stream));
        CREATE_TRY(cudaStreamSynchronize(h->stream));  // the host vectors go out of scope
    }

    // colour field: fluid slots (written every step), stored solids (fixed), ghost (0)
    if (h->collision == BCLBM_RK) {
        const size_t ncg = static_cast<size_t>(h->nf) + h->ns + 1;
        CREATE_TRY(pool_malloc(reinterpret_cast<void**>(&h->d_cg), ncg * sizeof(double), h->stream));
        std::vector<double> cg(ncg, 0.0);
        h->solid_cg.assign(h->ns, 0.0);
        for (int k = 0; k < h->ns; ++k) {
            const int n = h->solid_node[k];
            if (d->types[n] == 1) {  // findSolidBndNodes (main_TWOPHASE.cpp:280-284)
                const double r0 = d->rho_init[static_cast<size_t>(n) * 2], r1 = d->rho_init[static_cast<size_t>(n) * 2 + 1];
                h->solid_cg[k] = (r0 - r1) / (r0 + r1);
            }
            cg[static_cast<size_t>(h->nf) + k] = h->solid_cg[k];
        }
        if (h->fx_storage) {
            // the fixed-point step keeps the colour field in fixed point (|colour| < 2)
            for (size_t k = h->nf; k < ncg; ++k) {
                if (!(std::fabs(cg[k]) < 2.0)) {
                    std::fprintf(stderr, "bclbm_create: a boundary solid's colour %g is outside (-2, 2)\n", cg[k]);
                    return cleanup(BCLBM_ERR_INVALID);
                }
                const int64_t v = fx::param(cg[k]);
                std::memcpy(&cg[k], &v, sizeof(v));
            }
        }
        CREATE_TRY(cudaMemcpyAsync(h->d_cg, cg.data(), ncg * sizeof(double), cudaMemcpyHostToDevice, h->stream));
        if (h->precision != BCLBM_F64) {
            std::vector<float> cgf(cg.begin(), cg.end());
            CREATE_TRY(pool_malloc(reinterpret_cast<void**>(&h->d_cgf), ncg * sizeof(float), h->stream));
            CREATE_TRY(cudaMemcpyAsync(h->d_cgf, cgf.data(), ncg * sizeof(float), cudaMemcpyHostToDevice, h->stream));
            if (h->lagged) {  // the second field carries the same boundary solids and ghost
                CREATE_TRY(pool_malloc(reinterpret_cast<void**>(&h->d_cgf2), ncg * sizeof(float), h->stream));
                CREATE_TRY(cudaMemcpyAsync(h->d_cgf2, cgf.data(), ncg * sizeof(float), cudaMemcpyHostToDevice,
                                           h->stream));
            }
        }
        CREATE_TRY(cudaStreamSynchronize(h->stream));
    }

    // initial populations: reference AoS -> storage format.  The bulk nodes' rows are
    // one contiguous block in the common case (vtklb.py numbers the fluid nodes first):
    // upload it as it is and transpose on the device; otherwise transpose on the host.
    if (early_pops) {
        // uploaded and converted with the table checks
    } else if (h->bulk_contiguous) {
        const int es = h->nfields * Q;
        const size_t naos = static_cast<size_t>(h->nf) * es;
        const int mode = h->fx_storage ? 1 : (h->precision == BCLBM_F64 ? 0 : 2);
        double* tmp = nullptr;
        CREATE_TRY(pool_malloc(reinterpret_cast<void**>(&tmp), naos * sizeof(double), h->stream));
        cudaError_t e = cudaMemsetAsync(h->pops[0], 0, static_cast<size_t>(h->nfields) * Q * pad * store_bytes(h->precision),
                                        h->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(tmp, d->f_init + static_cast<size_t>(h->bulk0) * es, naos * sizeof(double),
                                cudaMemcpyHostToDevice, h->stream);
        if (e == cudaSuccess) {
            k_upload_aos<<<grid_for(h->nf), kBlock, 0, h->stream>>>(tmp, h->d_slot_bulk, h->pops[0], h->nf, h->nf_pad, Q,
                                                                    h->nfields, mode, h->precision, h->rho_ref,
                                                                    h->scale, &h->d_params->fx_overflow);
            launch_counter()++;
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
        cudaFreeAsync(tmp, h->stream);
        CREATE_TRY(e);
    } else {
        const size_t nsoa = static_cast<size_t>(h->nfields) * Q * pad;
        std::vector<double> soa(nsoa, 0.0);
        const int es = h->nfields * Q;
        parallel_for(static_cast<size_t>(h->nf), [&](size_t s0, size_t s1) {
            for (size_t s = s0; s < s1; ++s) {
                const size_t n = static_cast<size_t>(h->slot_node[s]);
                for (int k = 0; k < h->nfields; ++k)
                    for (int q = 0; q < Q; ++q)
                        soa[(static_cast<size_t>(q) * pad + s) * h->nfields + k] =
                            d->f_init[n * es + static_cast<size_t>(k) * Q + q];
            }
        });
        HostLock lk;
        lk.lock(soa.data(), nsoa * sizeof(double));
        if (h->precision == BCLBM_F64 && !h->fx_storage) {
            CREATE_TRY(cudaMemcpyAsync(h->pops[0], soa.data(), nsoa * sizeof(double), cudaMemcpyHostToDevice, h->stream));
            CREATE_TRY(cudaStreamSynchronize(h->stream));
        } else if (h->fx_storage) {
            double* tmp = nullptr;
            CREATE_TRY(pool_malloc(reinterpret_cast<void**>(&tmp), nsoa * sizeof(double), h->stream));
            cudaError_t e = cudaMemcpyAsync(tmp, soa.data(), nsoa * sizeof(double), cudaMemcpyHostToDevice, h->stream);
            if (e == cudaSuccess) {
                k_encode_fx<<<static_cast<unsigned>((nsoa + kBlock - 1) / kBlock), kBlock, 0, h->stream>>>(
                    tmp, static_cast<int64_t*>(h->pops[0]), nsoa, &h->d_params->fx_overflow);
                launch_counter()++;
                e = cudaGetLastError();
            }
            if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
            cudaFreeAsync(tmp, h->stream);
            CREATE_TRY(e);
        } else {
            double* tmp = nullptr;
            CREATE_TRY(pool_malloc(reinterpret_cast<void**>(&tmp), nsoa * sizeof(double), h->stream));
            cudaError_t e = cudaMemcpyAsync(tmp, soa.data(), nsoa * sizeof(double), cudaMemcpyHostToDevice, h->stream);
            if (e == cudaSuccess) {
                k_encode<<<grid_for(h->nf), kBlock, 0, h->stream>>>(tmp, h->pops[0], h->nf, h->nf_pad, Q, h->nfields,
                                                                    h->precision, h->rho_ref, h->scale);
                launch_counter()++;
                e = cudaGetLastError();
            }
            if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
            cudaFreeAsync(tmp, h->stream);
            CREATE_TRY(e);
        }
        lk.unlock();  // every branch above ends with the stream synchronised
    }
#undef CREATE_TRY
    h->cur = 0;
    h->state_post = false;
    *out = h;
    return BCLBM_OK;
}

}  // extern "C"

namespace {

// The step loop.  ev (optional) receives, per step, the events around the
// density pass (RK) and around the main step kernel: ev[4 s + 0..3].
int step_impl(bclbm_handle* h, int nsteps, cudaEvent_t* ev) {
    BCLBM_TRACE("bclbm_step");
    if (!h || nsteps < 0) return BCLBM_ERR_INVALID;
    if (nsteps == 0) return BCLBM_OK;
    CUDA_TRY(h, cudaSetDevice(h->device));
    StepArgs a = make_args(h);
    for (int s = 0; s < nsteps; ++s) {
        const bool local = !h->state_post;
        const bool macros = (s == nsteps - 1);
        a.src = h->pops[h->cur];
        a.dst = h->pops[1 - h->cur];
        a.rho_out = macros ? h->d_rho : nullptr;
        a.vel_out = macros ? h->d_vel : nullptr;
        if (h->collision == BCLBM_LINKS) {
            if (ev) CUDA_TRY(h, cudaEventRecord(ev[4 * s + 2], h->stream));
            CUDA_TRY(h, launch_links_step(h->precision, h->exact, h->fx_storage, local, links_args(h, a), h->stream));
            if (ev) CUDA_TRY(h, cudaEventRecord(ev[4 * s + 3], h->stream));
        } else if (h->collision != BCLBM_RK) {
            if (ev) CUDA_TRY(h, cudaEventRecord(ev[4 * s + 2], h->stream));
            const CUtensorMap* pm = h->pull_map_ok ? &h->pull_map : nullptr;
            if (h->exact) CUDA_TRY(h, launch_single_exact(h->q, h->trt, local, a, h->stream));
            else if (h->precision == BCLBM_F64 && !h->fma64)
                CUDA_TRY(h, launch_single_fixed(h->q, h->trt, local, a, h->stream));
            else CUDA_TRY(h, launch_single_fast(h->q, h->precision, h->trt, local, a, pm, h->stream));
            if (ev) CUDA_TRY(h, cudaEventRecord(ev[4 * s + 3], h->stream));
        } else if (h->lagged && !local) {
            // one pass; its sums give the force and mass correction of the next step
            const bool sums = h->flux || h->mass_fix;
            if (ev) CUDA_TRY(h, cudaEventRecord(ev[4 * s + 0], h->stream));
            if (ev) CUDA_TRY(h, cudaEventRecord(ev[4 * s + 1], h->stream));
            if (ev) CUDA_TRY(h, cudaEventRecord(ev[4 * s + 2], h->stream));
            a.cgf = h->d_cgf;
            a.cgf_out = h->d_cgf2;
            CUDA_TRY(h, launch_rk_fused(h->q, h->precision, sums, a, h->stream));
            if (sums) {
                CUDA_TRY(h, launch_reduce_final(3, h->d_partials, grid_for(h->nf), h->d_red, false, h->stream));
                CUDA_TRY(h, launch_rk_fix(h->d_red, static_cast<double>(h->nf), h->rho_ref, h->mom_x, h->flux,
                                          h->mass_fix ? 2 : 0, h->d_params, h->stream));
            }
            std::swap(h->d_cgf, h->d_cgf2);
            if (ev) CUDA_TRY(h, cudaEventRecord(ev[4 * s + 3], h->stream));
        } else {
            StepArgs ad = a;
            ad.rho_out = nullptr;
            if (ev) CUDA_TRY(h, cudaEventRecord(ev[4 * s + 0], h->stream));
            const bool sums = h->flux || h->mass_fix;
            if (h->fx_storage) CUDA_TRY(h, launch_rk_fx(h->q, local, sums, ad, h->stream, true));
            else if (h->precision == BCLBM_F64) CUDA_TRY(h, launch_rk_f64(h->q, local, sums, ad, h->stream, true));
            else CUDA_TRY(h, launch_rk_shift(h->q, h->precision, local, sums, ad, h->stream, true));
            if (sums) {
                CUDA_TRY(h, launch_reduce_final(3, h->d_partials, grid_for(h->nf), h->d_red, false, h->stream));
                CUDA_TRY(h, launch_rk_fix(h->d_red, static_cast<double>(h->nf), h->rho_ref, h->mom_x, h->flux,
                                          h->mass_fix ? 1 : 0, h->d_params, h->stream));
            }
            if (ev) CUDA_TRY(h, cudaEventRecord(ev[4 * s + 1], h->stream));
            if (ev) CUDA_TRY(h, cudaEventRecord(ev[4 * s + 2], h->stream));
            if (h->fx_storage) CUDA_TRY(h, launch_rk_fx(h->q, local, false, a, h->stream, false));
            else if (h->precision == BCLBM_F64 && !h->exact) CUDA_TRY(h, launch_rk_collide_f64_fma(h->q, local, a, h->stream));
            else if (h->precision == BCLBM_F64) CUDA_TRY(h, launch_rk_f64(h->q, local, false, a, h->stream, false));
            else CUDA_TRY(h, launch_rk_shift(h->q, h->precision, local, false, a, h->stream, false));
            if (ev) CUDA_TRY(h, cudaEventRecord(ev[4 * s + 3], h->stream));
        }
        h->cur = 1 - h->cur;
        h->state_post = true;
    }
    h->macros_valid = true;
    h->steps_done += nsteps;
    return BCLBM_OK;
}

}  // namespace

extern "C" {

int bclbm_step(bclbm_handle* h, int nsteps) { return step_impl(h, nsteps, nullptr); }

int bclbm_step_timed(bclbm_handle* h, int nsteps, bclbm_timing* out) {
    if (!h || !out || nsteps < 1) return BCLBM_ERR_INVALID;
    CUDA_TRY(h, cudaSetDevice(h->device));
    std::vector<cudaEvent_t> ev(4 * static_cast<size_t>(nsteps) + 2, nullptr);
    int rc = BCLBM_OK;
    for (auto& e : ev)
        if (cudaEventCreate(&e) != cudaSuccess) rc = fail(h, BCLBM_ERR_CUDA, "cudaEventCreate failed");
    const int64_t l0 = launch_counter().load();
    if (rc == BCLBM_OK && cudaEventRecord(ev[0], h->stream) != cudaSuccess) rc = fail(h, BCLBM_ERR_CUDA, "event");
    if (rc == BCLBM_OK) rc = step_impl(h, nsteps, ev.data() + 2);
    if (rc == BCLBM_OK && cudaEventRecord(ev[1], h->stream) != cudaSuccess) rc = fail(h, BCLBM_ERR_CUDA, "event");
    if (rc == BCLBM_OK && cudaEventSynchronize(ev[1]) != cudaSuccess) rc = fail(h, BCLBM_ERR_CUDA, "sync");
    if (rc == BCLBM_OK) {
        std::memset(out, 0, sizeof(*out));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ev[0], ev[1]);
        out->total_ms = ms;
        for (int s = 0; s < nsteps; ++s) {
            cudaEvent_t* e = ev.data() + 2 + 4 * static_cast<size_t>(s);
            if (cudaEventElapsedTime(&ms, e[2], e[3]) == cudaSuccess) out->step_kernel_ms += ms;
            if (h->collision == BCLBM_RK && cudaEventElapsedTime(&ms, e[0], e[1]) == cudaSuccess) out->density_ms += ms;
        }
        out->launches = launch_counter().load() - l0;
        out->nsteps = nsteps;
    }
    for (auto& e : ev)
        if (e) cudaEventDestroy(e);
    return rc;
}

int bclbm_sync(bclbm_handle* h) {
    if (!h) return BCLBM_ERR_INVALID;
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    return BCLBM_OK;
}

int bclbm_download_f(bclbm_handle* h, double* f) {
    BCLBM_TRACE("bclbm_download_f");
    if (!h || !f) return BCLBM_ERR_INVALID;
    CUDA_TRY(h, cudaSetDevice(h->device));
    int rc = run_gather(h);
    if (rc) return rc;
    const int es = h->nfields * h->q;
    const size_t n = static_cast<size_t>(h->nf) * es;
    if (h->bulk_contiguous) {
        HostLock lk;
        lk.lock(f + static_cast<size_t>(h->bulk0) * es, n * sizeof(double));
        cudaError_t e = cudaMemcpyAsync(f + static_cast<size_t>(h->bulk0) * es, h->d_gather, n * sizeof(double),
                                        cudaMemcpyDeviceToHost, h->stream);
        const cudaError_t es2 = cudaStreamSynchronize(h->stream);
        lk.unlock();
        if (e == cudaSuccess) e = es2;
        CUDA_TRY(h, e);
    } else {
        std::vector<double> tmp(n);
        CUDA_TRY(h, cudaMemcpyAsync(tmp.data(), h->d_gather, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
        CUDA_TRY(h, cudaStreamSynchronize(h->stream));
        parallel_for(static_cast<size_t>(h->nf), [&](size_t b0, size_t b1) {
            for (size_t b = b0; b < b1; ++b)
                std::memcpy(f + static_cast<size_t>(h->bulk[b]) * es, tmp.data() + b * es, es * sizeof(double));
        });
    }
    return BCLBM_OK;
}

int bclbm_macros_begin(bclbm_handle* h) {
    if (!h) return BCLBM_ERR_INVALID;
    if (!h->macros_valid) return fail(h, BCLBM_ERR_INVALID, "no step has run yet");
    if (h->stage_pending) return fail(h, BCLBM_ERR_INVALID, "a macro download is pending: collect it first");
    CUDA_TRY(h, cudaSetDevice(h->device));
    const size_t pad = static_cast<size_t>(h->nf_pad);
    const size_t nr = static_cast<size_t>(h->nfields) * pad, nv = static_cast<size_t>(h->nd) * pad;
    const bool rk = h->collision == BCLBM_RK;
    if (!h->stage) {
        // pinned, so the copies run asynchronously to the host
        CUDA_TRY(h, cudaMallocHost(&h->stage, (nr + nv + (rk ? static_cast<size_t>(h->nf) : 0)) * sizeof(double)));
        if (rk && h->d_cgf) CUDA_TRY(h, cudaMallocHost(&h->stage_cgf, static_cast<size_t>(h->nf) * sizeof(float)));
        CUDA_TRY(h, cudaEventCreateWithFlags(&h->stage_event, cudaEventDisableTiming));
    }
    CUDA_TRY(h, cudaMemcpyAsync(h->stage, h->d_rho, nr * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(h, cudaMemcpyAsync(h->stage + nr, h->d_vel, nv * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    if (rk) {
        if (h->d_cgf)
            CUDA_TRY(h, cudaMemcpyAsync(h->stage_cgf, h->d_cgf, h->nf * sizeof(float), cudaMemcpyDeviceToHost,
                                        h->stream));
        else
            CUDA_TRY(h, cudaMemcpyAsync(h->stage + nr + nv, h->d_cg, h->nf * sizeof(double), cudaMemcpyDeviceToHost,
                                        h->stream));
    }
    CUDA_TRY(h, cudaEventRecord(h->stage_event, h->stream));
    h->stage_pending = true;
    return BCLBM_OK;
}

int bclbm_macros_collect(bclbm_handle* h, double* rho, double* vel, double* cg) {
    if (!h) return BCLBM_ERR_INVALID;
    if (!h->stage_pending) return fail(h, BCLBM_ERR_INVALID, "no macro download to collect");
    CUDA_TRY(h, cudaSetDevice(h->device));
    h->stage_pending = false;
    CUDA_TRY(h, cudaEventSynchronize(h->stage_event));
    const size_t pad = static_cast<size_t>(h->nf_pad);
    const double* r = h->stage;
    const double* v = h->stage + static_cast<size_t>(h->nfields) * pad;
    const double* c = v + static_cast<size_t>(h->nd) * pad;
    const bool rk = h->collision == BCLBM_RK;
    parallel_for(static_cast<size_t>(h->nf), [&](size_t s0, size_t s1) {
        for (size_t s = s0; s < s1; ++s) {
            const size_t n = static_cast<size_t>(slot_node_of(h, s));
            if (rho)
                for (int k = 0; k < h->nfields; ++k) rho[n * h->nfields + k] = r[k * pad + s];
            if (vel)
                for (int dd = 0; dd < h->nd; ++dd) vel[n * h->nd + dd] = v[dd * pad + s];
            if (cg && rk) {
                if (h->stage_cgf) {
                    cg[n] = static_cast<double>(h->stage_cgf[s]);
                } else if (h->fx_storage) {
                    int64_t v;
                    std::memcpy(&v, &c[s], sizeof(v));
                    cg[n] = fx::to_f64(v);
                } else {
                    cg[n] = c[s];
                }
            }
        }
    });
    if (cg && rk)
        for (int k = 0; k < h->ns; ++k) cg[h->solid_node[k]] = h->solid_cg[k];
    return BCLBM_OK;
}

int bclbm_download_macros(bclbm_handle* h, double* rho, double* vel, double* cg) {
    BCLBM_TRACE("bclbm_download_macros");
    if (h && h->collision != BCLBM_RK && h->bulk_contiguous && h->macros_valid && !h->stage_pending && rho && vel) {
        // synchronous download: reorder on the device and copy the two blocks of bulk rows
        // straight into the caller's arrays (no pinned staging, no host scatter)
        CUDA_TRY(h, cudaSetDevice(h->device));
        const size_t n = static_cast<size_t>(h->nf) * h->nfields * h->q;
        if (!h->d_gather) CUDA_TRY(h, pool_malloc(reinterpret_cast<void**>(&h->d_gather), n * sizeof(double), h->stream));
        k_macros_aos<<<grid_for(h->nf), kBlock, 0, h->stream>>>(h->d_rho, h->d_vel, h->d_slot_bulk, h->d_gather, h->nf,
                                                                h->nf_pad, h->nfields, h->nd);
        launch_counter()++;
        CUDA_TRY(h, cudaGetLastError());
        const size_t b0 = static_cast<size_t>(h->bulk0), nr = static_cast<size_t>(h->nf) * h->nfields;
        CUDA_TRY(h, cudaMemcpyAsync(rho + b0 * h->nfields, h->d_gather, nr * sizeof(double), cudaMemcpyDeviceToHost,
                                    h->stream));
        CUDA_TRY(h, cudaMemcpyAsync(vel + b0 * h->nd, h->d_gather + nr, static_cast<size_t>(h->nf) * h->nd * sizeof(double),
                                    cudaMemcpyDeviceToHost, h->stream));
        CUDA_TRY(h, cudaStreamSynchronize(h->stream));
        return BCLBM_OK;
    }
    const int rc = bclbm_macros_begin(h);
    return rc ? rc : bclbm_macros_collect(h, rho, vel, cg);
}

int bclbm_reduce(bclbm_handle* h, bclbm_stats* out) {
    BCLBM_TRACE("bclbm_reduce");
    if (!h || !out) return BCLBM_ERR_INVALID;
    CUDA_TRY(h, cudaSetDevice(h->device));
    StepArgs a = make_args(h);
    a.src = h->pops[h->cur];
    if (h->collision == BCLBM_LINKS)
        CUDA_TRY(h, launch_links_moments(h->precision, h->exact, h->fx_storage, !h->state_post, links_args(h, a), h->stream));
    else
        CUDA_TRY(h, launch_moments(h->q, h->fx_storage ? kFX : h->precision, h->nfields, !h->state_post, a, h->stream));
    CUDA_TRY(h, launch_reduce_final(6, h->d_partials, grid_for(h->nf), h->d_red, true, h->stream));
    double red[6];
    DevParams prm;
    CUDA_TRY(h, cudaMemcpyAsync(red, h->d_red, sizeof(red), cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(h, cudaMemcpyAsync(&prm, h->d_params, sizeof(prm), cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    std::memset(out, 0, sizeof(*out));
    out->mass[0] = red[0];
    out->mass[1] = red[1];
    for (int k = 0; k < 3; ++k) {
        out->flux_fc[k] = red[2 + k];
        out->momentum[k] = red[2 + k] + 0.5 * prm.force[k] *
                                            (h->collision == BCLBM_LINKS ? h->force_on_sum : static_cast<double>(h->nf));
    }
    out->saturation = h->collision == BCLBM_RK ? red[0] / (red[0] + red[1]) : 0.0;
    out->max_abs_f = red[5];
    out->n_bulk = h->nf;
    out->steps_done = h->steps_done;
    out->nonfinite = std::isfinite(red[5]) && std::isfinite(red[0]) && std::isfinite(red[1]) ? 0 : 1;
    if (prm.fx_overflow & stage::kFlagWaitTimeout)
        return fail(h, BCLBM_ERR_CUDA, "a step kernel's bounded wait for a staged table tile ran out");
    if (prm.fx_overflow) {
        out->nonfinite = 1;
        return fail(h, BCLBM_ERR_NONFINITE, "a node left the fixed-point range (sum |f| < 8, rho > 0.15)");
    }
    return out->nonfinite ? fail(h, BCLBM_ERR_NONFINITE, "NaN or Inf in the populations") : BCLBM_OK;
}

int bclbm_set_force(bclbm_handle* h, const double force[3]) {
    if (!h || !force) return BCLBM_ERR_INVALID;
    CUDA_TRY(h, cudaSetDevice(h->device));
    DevParams prm;
    for (int k = 0; k < 3; ++k) {
        prm.force[k] = h->force[k] = force[k];
        prm.forcef[k] = static_cast<float>(force[k]);
        prm.forcex[k] = fx::param(force[k]);
    }
    CUDA_TRY(h, cudaMemcpyAsync(h->d_params, &prm, offsetof(DevParams, fx_overflow), cudaMemcpyHostToDevice,
                                h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    return BCLBM_OK;
}

int bclbm_pressure_flux(bclbm_handle* h, double q[2]) {
    BCLBM_TRACE("bclbm_pressure_flux");
    if (!h || !q) return BCLBM_ERR_INVALID;
    if (h->collision != BCLBM_LINKS) return fail(h, BCLBM_ERR_INVALID, "the mass flux is a BCLBM_LINKS output");
    if (!h->macros_valid) return fail(h, BCLBM_ERR_INVALID, "no step has run yet");
    CUDA_TRY(h, cudaSetDevice(h->device));
    StepArgs a = make_args(h);
    a.rho_out = h->d_rho;
    a.vel_out = h->d_vel;
    CUDA_TRY(h, launch_links_flux(links_args(h, a), h->stream));
    CUDA_TRY(h, cudaMemcpyAsync(q, h->d_flux_out, 2 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    return BCLBM_OK;
}

int bclbm_node_perm(bclbm_handle* h, int32_t* out) {
    if (!h || !out) return BCLBM_ERR_INVALID;
    if (h->affine) {
        parallel_for(static_cast<size_t>(h->nf), [&](size_t s0, size_t s1) {
            for (size_t s = s0; s < s1; ++s) out[s] = h->bulk0 + static_cast<int32_t>(s);
        });
    } else {
        std::memcpy(out, h->slot_node.data(), h->slot_node.size() * sizeof(int32_t));
    }
    return BCLBM_OK;
}

int bclbm_trim(void) {
    std::lock_guard<std::mutex> lock(g_pool_mutex);
    for (int dev = 0; dev < kMaxPoolDevices; ++dev) {
        if (!g_pool[dev]) continue;
        int cur = 0;
        if (cudaGetDevice(&cur) != cudaSuccess) return BCLBM_ERR_CUDA;
        if (cudaSetDevice(dev) != cudaSuccess) return BCLBM_ERR_CUDA;
        // memory of live handles stays; what destroyed handles left in the pool goes
        const cudaError_t e = cudaDeviceSynchronize();
        const cudaError_t t = cudaMemPoolTrimTo(g_pool[dev], 0);
        cudaSetDevice(cur);
        if (e != cudaSuccess || t != cudaSuccess) return BCLBM_ERR_CUDA;
    }
    return BCLBM_OK;
}

void bclbm_destroy(bclbm_handle* h) {
    if (!h) return;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    free_all(h);
    delete h;
}

}  // extern "C"
