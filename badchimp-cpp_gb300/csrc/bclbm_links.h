// The std_one_phase step (BCLBM_LINKS): host plan and launchers.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "bclbm.h"
#include "bclbm_links.cuh"

namespace bclbm {

// what bclbm_create derives from the node attributes of a BCLBM_LINKS descriptor
struct LinksPlan {
    std::vector<uint32_t> info;        // [nf] label | kLinkAdd | kLinkPress
    std::vector<int32_t> pidx;         // [nf] u_store index or -1
    std::vector<int32_t> force_on;     // [nf]
    std::vector<int32_t> lab_slot;     // labelled bulk nodes by label, bulk order
    std::vector<int32_t> lab_start;    // [nlab + 2]
    std::vector<double> lab_g;         // [nlab + 1] 0.9 * 2 / (source nodes of the label)
    std::vector<int32_t> flux_slot;    // bulk pressure-boundary nodes, node order
    std::vector<int32_t> flux_phase;
    int npress = 0, nlab = 0;
    double force_on_sum = 0.0;         // sum of the force attribute over the bulk nodes
};

// resolves the tags into the pull table tab [18][pad] (see bclbm_links.cu)
int links_plan(const bclbm_desc* d, const std::vector<int32_t>& slot_node, const int32_t* ghost_src, size_t pad,
               LinksPlan& P, std::vector<int32_t>& tab, std::string& err);

// bclbm_exact.cu (-fmad=false): the reference's rounding
cudaError_t launch_links_mass_exact(bool local, const LinksArgs& A, cudaStream_t s);
cudaError_t launch_links_label_sum_exact(const LinksArgs& A, cudaStream_t s);
cudaError_t launch_links_collide_exact(bool local, const LinksArgs& A, cudaStream_t s);
cudaError_t launch_links_gather_exact(bool local, const LinksArgs& A, const int32_t* slot_bulk, double* out,
                                      cudaStream_t s);
cudaError_t launch_links_moments_exact(bool local, const LinksArgs& A, cudaStream_t s);
// the write step's mass flux from the last step's moments (always exact)
cudaError_t launch_links_flux(const LinksArgs& A, cudaStream_t s);

// bclbm_links.cu: F64 exact or contracting instances, or the shifted storage formats
// (precision BCLBM_F32 / F16 / BF16, FP32 arithmetic)
// One step: with interior domains the mass pass and the domain sums, then the collision.  (Running
// the mass pass and the labelled nodes on a second stream beside the other nodes was measured slower:
// 192^3 F32 135 -> 151 us per step, F16 unchanged.)
// F64 arithmetic: exact (the reference's rounding), else 64-bit fixed point (fixed) or FP64 with FMA
cudaError_t launch_links_step(int precision, bool exact, bool fixed, bool local, const LinksArgs& A, cudaStream_t s);
// fixed: the FP64 state is held as int64 fixed point (the default FP64 step)
cudaError_t launch_links_gather(int precision, bool exact, bool fixed, bool local, const LinksArgs& A,
                                const int32_t* slot_bulk, double* out, cudaStream_t s);
cudaError_t launch_links_moments(int precision, bool exact, bool fixed, bool local, const LinksArgs& A,
                                 cudaStream_t s);

}  // namespace bclbm
