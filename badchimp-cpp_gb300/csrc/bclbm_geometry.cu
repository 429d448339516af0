// Host-side lattice builder: a voxel mask to the node numbering, neighbour
// table, positions and node types that the reference's Grid and Nodes hold
// after reading a .vtklb file.  The numbering rules are those of the
// single-rank case of PythonScripts/vtklb.py (setup_processor_labels and
// write_neighbors_fast, vtklb.py:6-45, 84-114, 182-218) and of
// Nodes::setupNodeType (src/lbsolver/LBnodes.h:141-209):
//   - node 0 is the ghost node;
//   - fluid voxels are numbered 1..nf in C order of the interior;
//   - then every solid that is a lattice neighbour of a fluid node, in C order
//     of the array padded by a one-voxel rim (a periodic rim voxel copies the
//     opposite interior layer and is a node of its own);
//   - a neighbour outside the padded array, or at an unlisted voxel, is node 0,
//     except that a rim voxel holding fluid maps to the fluid node it copies.
// Work is split over the host cores by contiguous ranges; every output is the
// same whatever the thread count.
#include <cstdint>
#include <cstring>
#include <new>
#include <vector>

#include "bclbm.h"
#include "bclbm_device.cuh"
#include "bclbm_host.h"
#include "bclbm_lattice.h"

using bclbm::host::parallel_for;


namespace {

template <int Q>
int build(int nd, const int32_t* shape, const int8_t* mask, uint32_t periodic, bclbm_lattice* L) {
    using Lt = bclbm::Lat<Q>;
    int64_t ps[3] = {1, 1, 1};  // padded shape, C order
    for (int d = 0; d < nd; ++d) ps[d] = static_cast<int64_t>(shape[d]) + 2;
    const int64_t st[3] = {nd == 3 ? ps[1] * ps[2] : ps[1], nd == 3 ? ps[2] : 1, 1};
    const int64_t total = nd == 3 ? ps[0] * ps[1] * ps[2] : ps[0] * ps[1];
    int64_t off[Q];
    for (int q = 0; q < Q; ++q) {
        const int c[3] = {Lt::cx(q), Lt::cy(q), Lt::cz(q)};
        off[q] = 0;
        for (int d = 0; d < nd; ++d) off[q] += c[d] * st[d];
    }
    auto coord = [&](int64_t p, int64_t* x) {
        for (int d = 0; d < nd; ++d) {
            x[d] = p / st[d];
            p -= x[d] * st[d];
        }
    };
    auto interior = [&](const int64_t* x) {
        for (int d = 0; d < nd; ++d)
            if (x[d] < 1 || x[d] > ps[d] - 2) return false;
        return true;
    };
    // P: -1 outside, else the mask value (periodic rims copy the opposite layer);
    // idx: node number of each padded voxel (0 = none)
    std::vector<int8_t> P(total, -1);
    std::vector<int32_t> idx(total, 0);
    parallel_for(static_cast<size_t>(total), [&](size_t b, size_t e) {
        int64_t x[3];
        for (size_t p = b; p < e; ++p) {
            coord(static_cast<int64_t>(p), x);
            if (!interior(x)) continue;
            int64_t m = 0;
            int64_t ms = 1;
            for (int d = nd - 1; d >= 0; --d) {
                m += (x[d] - 1) * ms;
                ms *= shape[d];
            }
            P[p] = mask[m];
        }
    });
    // fluid labels in C order: per-chunk counts, then an exclusive scan
    const size_t nchunk = 256;
    std::vector<int64_t> cnt(nchunk + 1, 0);
    auto chunk_lo = [&](size_t c) { return static_cast<int64_t>(static_cast<size_t>(total) * c / nchunk); };
    parallel_for(nchunk, [&](size_t c0, size_t c1) {
        for (size_t c = c0; c < c1; ++c) {
            int64_t n = 0;
            for (int64_t p = chunk_lo(c); p < chunk_lo(c + 1); ++p) n += P[p] == 1;
            cnt[c + 1] = n;
        }
    }, 1);
    for (size_t c = 0; c < nchunk; ++c) cnt[c + 1] += cnt[c];
    const int64_t nf = cnt[nchunk];
    if (nf + 1 > INT32_MAX) return BCLBM_ERR_UNSUPPORTED;
    parallel_for(nchunk, [&](size_t c0, size_t c1) {
        for (size_t c = c0; c < c1; ++c) {
            int32_t lab = static_cast<int32_t>(cnt[c]) + 1;
            for (int64_t p = chunk_lo(c); p < chunk_lo(c + 1); ++p)
                if (P[p] == 1) idx[p] = lab++;
        }
    }, 1);
    // periodic rims: copy mask and labels of the opposite interior layer, axis by
    // axis in x, y, z order (later axes copy the rims earlier axes filled)
    for (int d = 0; d < nd; ++d) {
        if (!(periodic & (1u << d))) continue;
        const int64_t n_planes = total / ps[d];
        parallel_for(static_cast<size_t>(n_planes), [&](size_t b, size_t e) {
            for (size_t k = b; k < e; ++k) {
                // k enumerates the voxels of one hyperplane normal to axis d
                const int64_t hi = static_cast<int64_t>(k) / st[d], lo = static_cast<int64_t>(k) % st[d];
                const int64_t base = hi * st[d] * ps[d] + lo;
                const int64_t r0 = base, r1 = base + (ps[d] - 1) * st[d];
                const int64_t s0 = base + (ps[d] - 2) * st[d], s1 = base + st[d];
                P[r0] = P[s0];
                idx[r0] = idx[s0];
                P[r1] = P[s1];
                idx[r1] = idx[s1];
            }
        });
    }
    // fluid voxel positions in label order
    std::vector<int64_t> fpos(nf);
    parallel_for(nchunk, [&](size_t c0, size_t c1) {
        int64_t x[3];
        for (size_t c = c0; c < c1; ++c) {
            int64_t k = cnt[c];
            for (int64_t p = chunk_lo(c); p < chunk_lo(c + 1); ++p) {
                if (P[p] != 1) continue;
                coord(p, x);
                if (interior(x)) fpos[k++] = p;
            }
        }
    }, 1);
    // solids adjacent to fluid: mark, then number in C order of the padded array
    std::vector<uint8_t> added(total, 0);
    parallel_for(static_cast<size_t>(nf), [&](size_t b, size_t e) {
        for (size_t k = b; k < e; ++k)
            for (int q = 0; q < Q; ++q) {
                const int64_t p = fpos[k] + off[q];
                if (P[p] == 0) __atomic_store_n(&added[p], static_cast<uint8_t>(1), __ATOMIC_RELAXED);
            }
    });
    std::vector<int64_t> scnt(nchunk + 1, 0);
    parallel_for(nchunk, [&](size_t c0, size_t c1) {
        for (size_t c = c0; c < c1; ++c) {
            int64_t n = 0;
            for (int64_t p = chunk_lo(c); p < chunk_lo(c + 1); ++p) n += added[p];
            scnt[c + 1] = n;
        }
    }, 1);
    for (size_t c = 0; c < nchunk; ++c) scnt[c + 1] += scnt[c];
    const int64_t ns = scnt[nchunk];
    if (1 + nf + ns > INT32_MAX) return BCLBM_ERR_UNSUPPORTED;
    std::vector<int64_t> spos(ns);
    parallel_for(nchunk, [&](size_t c0, size_t c1) {
        for (size_t c = c0; c < c1; ++c) {
            int64_t k = scnt[c];
            for (int64_t p = chunk_lo(c); p < chunk_lo(c + 1); ++p)
                if (added[p]) {
                    spos[k] = p;
                    idx[p] = static_cast<int32_t>(nf + 1 + k);
                    ++k;
                }
        }
    }, 1);
    const int64_t n_nodes = 1 + nf + ns;
    L->q = Q;
    L->nd = nd;
    L->nf = nf;
    L->ns = ns;
    L->neigh.assign(static_cast<size_t>(n_nodes) * Q, 0);
    L->pos.assign(static_cast<size_t>(n_nodes) * nd, -1);
    L->types.assign(static_cast<size_t>(n_nodes), 0);
    int32_t* nb = L->neigh.data();
    parallel_for(static_cast<size_t>(nf + ns), [&](size_t b, size_t e) {
        int64_t x[3];
        for (size_t k = b; k < e; ++k) {
            const bool fl = static_cast<int64_t>(k) < nf;
            const int64_t p = fl ? fpos[k] : spos[k - nf];
            const size_t node = k + 1;
            coord(p, x);
            for (int d = 0; d < nd; ++d) L->pos[node * nd + d] = static_cast<int32_t>(x[d] - 1);
            for (int q = 0; q < Q; ++q) {
                const int c[3] = {Lt::cx(q), Lt::cy(q), Lt::cz(q)};
                bool ok = true;
                for (int d = 0; d < nd; ++d) {
                    const int64_t y = x[d] + c[d];
                    ok &= y >= 0 && y < ps[d];
                }
                nb[node * Q + q] = ok ? idx[p + off[q]] : 0;
            }
        }
    });
    // node types (Nodes::setupNodeType): fluids 2 with a non-fluid neighbour
    // (node 0 counts as solid) else 3; solids 1 with a fluid neighbour else 0
    int16_t* ty = L->types.data();
    ty[0] = -1;
    parallel_for(static_cast<size_t>(nf + ns), [&](size_t b, size_t e) {
        for (size_t k = b; k < e; ++k) {
            const size_t node = k + 1;
            const bool fl = static_cast<int64_t>(node) <= nf;
            bool any_fluid = false, any_solid = false;
            for (int q = 0; q < Q; ++q) {
                const int32_t y = nb[node * Q + q];
                const bool yf = y >= 1 && y <= nf;
                any_fluid |= yf;
                any_solid |= !yf;
            }
            ty[node] = fl ? (any_solid ? 2 : 3) : (any_fluid ? 1 : 0);
        }
    });
    return BCLBM_OK;
}

}  // namespace

extern "C" {

int bclbm_lattice_build(int32_t lattice_q, int32_t nd, const int32_t* shape, const int8_t* mask,
                        uint32_t periodic, bclbm_lattice** out) {
    if (!out) return BCLBM_ERR_INVALID;
    *out = nullptr;
    if (!shape || !mask || (lattice_q == 9 && nd != 2) || (lattice_q == 19 && nd != 3) ||
        (lattice_q != 9 && lattice_q != 19))
        return BCLBM_ERR_INVALID;
    int64_t vox = 1;
    for (int d = 0; d < nd; ++d) {
        if (shape[d] < 1) return BCLBM_ERR_INVALID;
        vox *= static_cast<int64_t>(shape[d]) + 2;
    }
    if (vox > (int64_t(1) << 40)) return BCLBM_ERR_UNSUPPORTED;
    {
        int64_t n = 1;
        for (int d = 0; d < nd; ++d) n *= shape[d];
        for (int64_t i = 0; i < n; ++i)
            if (mask[i] != 0 && mask[i] != 1) return BCLBM_ERR_INVALID;
    }
    bclbm_lattice* L = new (std::nothrow) bclbm_lattice();
    if (!L) return BCLBM_ERR_NOMEM;
    int rc;
    try {
        rc = lattice_q == 9 ? build<9>(nd, shape, mask, periodic, L) : build<19>(nd, shape, mask, periodic, L);
    } catch (const std::bad_alloc&) {
        rc = BCLBM_ERR_NOMEM;
    }
    if (rc) {
        delete L;
        return rc;
    }
    *out = L;
    return BCLBM_OK;
}

int bclbm_lattice_info(const bclbm_lattice* L, int64_t* n_nodes, int64_t* n_fluid, int64_t* n_solid) {
    if (!L) return BCLBM_ERR_INVALID;
    if (n_nodes) *n_nodes = 1 + L->nf + L->ns;
    if (n_fluid) *n_fluid = L->nf;
    if (n_solid) *n_solid = L->ns;
    return BCLBM_OK;
}

int bclbm_lattice_export(const bclbm_lattice* L, int32_t* neigh, int16_t* types, int32_t* pos) {
    if (!L) return BCLBM_ERR_INVALID;
    if (neigh) std::memcpy(neigh, L->neigh.data(), L->neigh.size() * sizeof(int32_t));
    if (types) std::memcpy(types, L->types.data(), L->types.size() * sizeof(int16_t));
    if (pos) std::memcpy(pos, L->pos.data(), L->pos.size() * sizeof(int32_t));
    return BCLBM_OK;
}

void bclbm_lattice_free(bclbm_lattice* L) { delete L; }

}  // extern "C"
