// The std_one_phase step (BCLBM_LINKS): host-side resolution of the node tags
// into the pull table, the interior-domain lists, and the launchers of the
// contracting (FMA) kernel instances; the exact instances are in
// bclbm_exact.cu.
#include <algorithm>
#include <string>
#include <vector>

#include "bclbm_host.h"
#include "bclbm_launch.h"
#include "bclbm_links.h"

namespace bclbm {

using host::FirstBad;
using host::parallel_for;

namespace {

constexpr int kQ = 19, kR = 18;

inline int tag_of(const int32_t* tags, int n) { return n == 0 ? -1 : tags[n]; }  // Nodes: nodeTag_ starts at -1

}  // namespace

// The link rules of src/std_one_phase/main.cpp:24-129, per fluid slot s (node n)
// and incoming direction q, with y = neighbor(rev q, n) the node that pushes
// into (q, n) and k = rev q the direction of the push from n to y:
//   solid-fluid     n has bit 8 and tag(y) & 3 == 0          -> f*(k, n)
//   pressure-fluid  n has bit 16 and tag(y) & 3 == 3         -> anti-bounce-back of f(k, y) after
//                   streaming: f*(k, n), or for y = 0 (tag -1) the last bulk node's push into node 0
//   fluid-fluid     n phase 1 with bit 4 and y phase 2, or
//                   n phase 2 and y phase 1 with bit 4      -> f*(k, n)
//   otherwise y must be a fluid slot                        -> f*(q, y)
int links_plan(const bclbm_desc* d, const std::vector<int32_t>& slot_node, const int32_t* ghost_src, size_t pad,
               LinksPlan& P, std::vector<int32_t>& tab, std::string& err) {
    const int N = d->n_nodes, nf = static_cast<int>(slot_node.size());
    const int32_t* T = d->tags;
    const int32_t* lab = d->labels;
    if (d->lattice_q != kQ) {
        err = "the std_one_phase step is D3Q19";
        return BCLBM_ERR_UNSUPPORTED;
    }
    if (!T || !lab) {
        err = "BCLBM_LINKS needs tags and labels";
        return BCLBM_ERR_INVALID;
    }
    std::vector<int32_t> slot_of(N, -1);
    for (int s = 0; s < nf; ++s) slot_of[slot_node[s]] = s;
    // interior domains (main.cpp:318-358): label maximum, source nodes per label
    int64_t lmax = 0;
    for (int n = 1; n < N; ++n) {
        if (lab[n] < 0) {
            err = "negative interior-domain label at node " + std::to_string(n);
            return BCLBM_ERR_INVALID;
        }
        lmax = std::max<int64_t>(lmax, lab[n]);
    }
    if (lmax > static_cast<int64_t>(kLinkLabelMask)) {
        err = "more than 2^24 - 1 interior domains";
        return BCLBM_ERR_UNSUPPORTED;
    }
    const int L = static_cast<int>(lmax);
    std::vector<double> count(static_cast<size_t>(L) + 1, 0.0);
    std::vector<char> add(N, 0);
    for (int n = 1; n < N; ++n)
        if (lab[n] > 0 && tag_of(T, n) < 3) {
            count[lab[n]] += 1;
            add[n] = 1;
        }
    P.lab_g.assign(static_cast<size_t>(L) + 1, 0.0);
    for (int l = 1; l <= L; ++l) {
        if (count[l] == 0.0) {
            err = "interior domain " + std::to_string(l) + " has no interior nodes";
            return BCLBM_ERR_INVALID;
        }
        const double scale = 1.0 / count[l];
        P.lab_g[l] = 0.9 * 2 * scale;
    }
    P.nlab = L;
    // labelled bulk nodes grouped by label, each group in bulk order
    P.lab_start.assign(static_cast<size_t>(L) + 2, 0);
    for (int b = 0; b < d->n_bulk; ++b) {
        const int l = lab[d->bulk[b]];
        if (l > 0) ++P.lab_start[l + 1];
    }
    for (int l = 1; l <= L; ++l) P.lab_start[l + 1] += P.lab_start[l];
    P.lab_slot.assign(static_cast<size_t>(P.lab_start[L + 1]), 0);
    {
        std::vector<int32_t> fill(P.lab_start.begin(), P.lab_start.end());
        for (int b = 0; b < d->n_bulk; ++b) {
            const int n = d->bulk[b], l = lab[n];
            if (l > 0) P.lab_slot[fill[l]++] = slot_of[n];
        }
    }
    // the resolved pull table
    tab.assign(static_cast<size_t>(kR) * pad, 0);
    std::vector<char> press(nf, 0);
    FirstBad bad;
    parallel_for(static_cast<size_t>(nf), [&](size_t s0, size_t s1) {
        for (size_t s = s0; s < s1; ++s) {
            const int n = slot_node[s], tn = tag_of(T, n);
            for (int q = 0; q < kR; ++q) {
                const int k = Lat<kQ>::rev(q);
                const int y = d->neigh[static_cast<size_t>(n) * kQ + k];
                const int ty = tag_of(T, y);
                const int64_t own = static_cast<int64_t>(k) * pad + static_cast<int64_t>(s);
                int64_t e;
                if (((tn >> 3) & 1) && (ty & 3) == 0) {
                    e = own;
                } else if (((tn >> 4) & 1) && (ty & 3) == 3) {
                    const int64_t base = y == 0 ? static_cast<int64_t>(k) * pad + ghost_src[k] : own;
                    e = ~base;
                    press[s] = 1;
                } else if (((tn & 3) == 1 && ((tn >> 2) & 1) && (ty & 3) == 2) ||
                           ((tn & 3) == 2 && (ty & 3) == 1 && ((ty >> 2) & 1))) {
                    e = own;
                } else if (y != 0 && slot_of[y] >= 0) {
                    e = static_cast<int64_t>(q) * pad + slot_of[y];
                } else {
                    bad.set(static_cast<int64_t>(s) * 32 + q);
                    return;
                }
                tab[static_cast<size_t>(q) * pad + s] = static_cast<int32_t>(e);
            }
        }
    });
    if (bad.any()) {
        const int s = static_cast<int>(bad.get() / 32), q = static_cast<int>(bad.get() % 32);
        const int n = slot_node[s], y = d->neigh[static_cast<size_t>(n) * kQ + Lat<kQ>::rev(q)];
        err = "node " + std::to_string(n) + " (tag " + std::to_string(tag_of(T, n)) + ") has no boundary rule for " +
              "its link to node " + std::to_string(y) + " (tag " + std::to_string(tag_of(T, y)) +
              "): the reference would stream a stale population there";
        return BCLBM_ERR_TABLE;
    }
    // per-slot info, force indicator, velocity store of the pressure-boundary nodes
    P.info.assign(nf, 0u);
    P.pidx.assign(nf, -1);
    P.force_on.assign(nf, 1);
    P.npress = 0;
    P.force_on_sum = 0.0;
    for (int s = 0; s < nf; ++s) {
        const int n = slot_node[s];
        uint32_t v = static_cast<uint32_t>(lab[n]);
        if (add[n]) v |= kLinkAdd;
        if (press[s]) {
            v |= kLinkPress;
            P.pidx[s] = P.npress++;
        }
        P.info[s] = v;
        if (d->force_on) P.force_on[s] = d->force_on[n];
    }
    for (int b = 0; b < d->n_bulk; ++b) P.force_on_sum += static_cast<double>(d->force_on ? d->force_on[d->bulk[b]] : 1);
    // the write step's mass flux: nodes with bit 16 in node order (main.cpp:80-92, 550-562)
    P.flux_slot.clear();
    P.flux_phase.clear();
    for (int n = 1; n < N; ++n)
        if ((tag_of(T, n) >> 4) & 1) {
            const int ph = (tag_of(T, n) & 3) - 1;
            if (ph != 0 && ph != 1) {
                err = "pressure-boundary node " + std::to_string(n) + " is not in fluid phase 1 or 2";
                return BCLBM_ERR_INVALID;
            }
            if (slot_of[n] >= 0) {  // others keep rho = 1, u = 0 in the reference: they add 0
                P.flux_slot.push_back(slot_of[n]);
                P.flux_phase.push_back(ph);
            }
        }
    return BCLBM_OK;
}

namespace {

// the three parts of a step for one arithmetic (exact FP64, FMA FP64, shifted S)
struct StepParts {
    cudaError_t (*mass)(bool, const LinksArgs&, cudaStream_t);
    cudaError_t (*sum)(const LinksArgs&, cudaStream_t);
    cudaError_t (*collide)(bool, const LinksArgs&, cudaStream_t);
};

cudaError_t sum_fast(const LinksArgs& A, cudaStream_t s) {
    k_links_label_sum<false><<<(A.nlab * 32 + kBlock - 1) / kBlock, kBlock, 0, s>>>(A);
    launch_counter()++;
    return cudaGetLastError();
}

cudaError_t mass_fma(bool local, const LinksArgs& A, cudaStream_t s) {
    if (local) k_links_mass<false, true><<<grid_for(A.nlabeled), kBlock, 0, s>>>(A);
    else k_links_mass<false, false><<<grid_for(A.nlabeled), kBlock, 0, s>>>(A);
    launch_counter()++;
    return cudaGetLastError();
}

cudaError_t collide_fma(bool local, const LinksArgs& A, cudaStream_t s) {
    const int n = A.s.L.nf;
    if (local) k_links_collide<false, true><<<grid_for(n), kBlock, 0, s>>>(A);
    else k_links_collide<false, false><<<grid_for(n), kBlock, 0, s>>>(A);
    launch_counter()++;
    return cudaGetLastError();
}

cudaError_t mass_fixed(bool local, const LinksArgs& A, cudaStream_t s) {
    if (local) k_links_mass_fx<true><<<grid_for(A.nlabeled), kBlock, 0, s>>>(A);
    else k_links_mass_fx<false><<<grid_for(A.nlabeled), kBlock, 0, s>>>(A);
    launch_counter()++;
    return cudaGetLastError();
}

cudaError_t collide_fixed(bool local, const LinksArgs& A, cudaStream_t s) {
    const int g = (A.s.L.nf + BCLBM_LINKS_FX_BLOCK - 1) / BCLBM_LINKS_FX_BLOCK;
    if (local) k_links_collide_fixed<true><<<g, BCLBM_LINKS_FX_BLOCK, 0, s>>>(A);
    else k_links_collide_fixed<false><<<g, BCLBM_LINKS_FX_BLOCK, 0, s>>>(A);
    launch_counter()++;
    return cudaGetLastError();
}

template <class S>
cudaError_t mass_shift(bool local, const LinksArgs& A, cudaStream_t s) {
    if (local) k_links_mass_shift<S, true><<<grid_for(A.nlabeled), kBlock, 0, s>>>(A);
    else k_links_mass_shift<S, false><<<grid_for(A.nlabeled), kBlock, 0, s>>>(A);
    launch_counter()++;
    return cudaGetLastError();
}

template <class S>
cudaError_t collide_shift(bool local, const LinksArgs& A, cudaStream_t s) {
    const int n = A.s.L.nf;
    if (local) k_links_collide_shift<S, true><<<grid_for(n), kBlock, 0, s>>>(A);
    else k_links_collide_shift<S, false><<<grid_for(n), kBlock, 0, s>>>(A);
    launch_counter()++;
    return cudaGetLastError();
}

template <class S>
cudaError_t shift_s(int what, bool local, const LinksArgs& A, const int32_t* slot_bulk, double* out, cudaStream_t s) {
    const int g = grid_for(A.s.L.nf);
    if (what == 1) {
        if (local) k_links_gather_shift<S, true><<<g, kBlock, 0, s>>>(A, slot_bulk, out);
        else k_links_gather_shift<S, false><<<g, kBlock, 0, s>>>(A, slot_bulk, out);
    } else {
        if (local) k_links_moments_shift<S, true><<<g, kBlock, 0, s>>>(A);
        else k_links_moments_shift<S, false><<<g, kBlock, 0, s>>>(A);
    }
    launch_counter()++;
    return cudaGetLastError();
}

cudaError_t shift(int precision, int what, bool local, const LinksArgs& A, const int32_t* slot_bulk, double* out,
                  cudaStream_t s) {
    switch (precision) {
        case kF32: return shift_s<float>(what, local, A, slot_bulk, out, s);
        case kF16: return shift_s<__half>(what, local, A, slot_bulk, out, s);
        case kBF16: return shift_s<__nv_bfloat16>(what, local, A, slot_bulk, out, s);
    }
    return cudaErrorInvalidValue;
}

bool parts_for(int precision, bool exact, bool fixed, StepParts& P) {
    switch (precision) {
        case kF64:
            if (exact) P = StepParts{launch_links_mass_exact, launch_links_label_sum_exact, launch_links_collide_exact};
            else if (fixed) P = StepParts{mass_fixed, sum_fast, collide_fixed};
            else P = StepParts{mass_fma, sum_fast, collide_fma};
            return true;
        case kF32: P = StepParts{mass_shift<float>, sum_fast, collide_shift<float>}; return true;
        case kF16: P = StepParts{mass_shift<__half>, sum_fast, collide_shift<__half>}; return true;
        case kBF16:
            P = StepParts{mass_shift<__nv_bfloat16>, sum_fast, collide_shift<__nv_bfloat16>};
            return true;
    }
    return false;
}

}  // namespace

cudaError_t launch_links_step(int precision, bool exact, bool fixed, bool local, const LinksArgs& A, cudaStream_t s) {
    StepParts P;
    if (!parts_for(precision, exact, fixed, P)) return cudaErrorInvalidValue;
    cudaError_t e;
    if (A.nlabeled > 0) {
        if ((e = P.mass(local, A, s)) != cudaSuccess) return e;
        if ((e = P.sum(A, s)) != cudaSuccess) return e;
    }
    return P.collide(local, A, s);
}

cudaError_t launch_links_gather(int precision, bool exact, bool fixed, bool local, const LinksArgs& A,
                                const int32_t* slot_bulk, double* out, cudaStream_t s) {
    if (precision != kF64) return shift(precision, 1, local, A, slot_bulk, out, s);
    if (exact) return launch_links_gather_exact(local, A, slot_bulk, out, s);
    const int g = grid_for(A.s.L.nf);
    if (fixed) {
        if (local) k_links_gather<false, true, int64_t><<<g, kBlock, 0, s>>>(A, slot_bulk, out);
        else k_links_gather<false, false, int64_t><<<g, kBlock, 0, s>>>(A, slot_bulk, out);
    } else {
        if (local) k_links_gather<false, true><<<g, kBlock, 0, s>>>(A, slot_bulk, out);
        else k_links_gather<false, false><<<g, kBlock, 0, s>>>(A, slot_bulk, out);
    }
    launch_counter()++;
    return cudaGetLastError();
}

cudaError_t launch_links_moments(int precision, bool exact, bool fixed, bool local, const LinksArgs& A,
                                 cudaStream_t s) {
    if (precision != kF64) return shift(precision, 2, local, A, nullptr, nullptr, s);
    if (exact) return launch_links_moments_exact(local, A, s);
    const int g = grid_for(A.s.L.nf);
    if (fixed) {
        if (local) k_links_moments<false, true, int64_t><<<g, kBlock, 0, s>>>(A);
        else k_links_moments<false, false, int64_t><<<g, kBlock, 0, s>>>(A);
    } else {
        if (local) k_links_moments<false, true><<<g, kBlock, 0, s>>>(A);
        else k_links_moments<false, false><<<g, kBlock, 0, s>>>(A);
    }
    launch_counter()++;
    return cudaGetLastError();
}

}  // namespace bclbm
