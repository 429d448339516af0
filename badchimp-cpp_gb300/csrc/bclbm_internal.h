// Internal to the library: the handle's state, shared by the C ABI
// (bclbm_api.cu) and the multi-instance batch (bclbm_batch.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "bclbm.h"
#include "bclbm_kernels.cuh"

struct bclbm_handle {
    int q = 0, nd = 0, nfields = 1, collision = 0, precision = 0;
    uint32_t flags = 0;
    bool exact = false, trt = false, flux = false, fma64 = false;
    bool mass_fix = false;  // two-phase shifted storage: per-step mass-drift correction
    bool fx_storage = false;  // default F64 step: populations held as int64 fixed point
    int n_nodes = 0, nf = 0, nf_pad = 0, ns = 0;
    double tau[2] = {1.0, 1.0};
    double sigma = 0.0, beta = 0.0, mom_x = 0.0, rho_ref = 1.0, scale = 1.0;
    double force[3] = {0.0, 0.0, 0.0};
    std::vector<int32_t> slot_node;   // device slot -> reference node number
    std::vector<int32_t> slot_bulk;   // device slot -> index in the bulk list
    std::vector<int32_t> bulk;        // the bulk list
    std::vector<int32_t> solid_node;  // extended solid index -> reference node number
    std::vector<double> solid_cg;     // RK colour of the stored solids
    bool bulk_contiguous = false;
    // affine numbering: the bulk list is nodes bulk0 .. bulk0 + nf - 1 in reference
    // order, so slot s holds node bulk0 + s and slot_node / slot_bulk / bulk stay empty
    bool affine = false;
    int32_t bulk0 = 0;
    int device = 0;
    cudaStream_t stream = nullptr;
    void* pops[2] = {nullptr, nullptr};
    int cur = 0;
    bool state_post = false;          // pops[cur] holds post-collision populations
    bool macros_valid = false;
    int32_t* d_nbr = nullptr;
    // single-phase pull table as a tensor map (the staged step kernels); valid when pull_map_ok
    CUtensorMap pull_map;
    bool pull_map_ok = false;
    int32_t* d_slot_bulk = nullptr;
    double* d_rho = nullptr;
    double* d_vel = nullptr;
    double* d_cg = nullptr;
    float* d_cgf = nullptr;
    float* d_cgf2 = nullptr;  // BCLBM_FLAG_LAGGED_COLOUR: the colour field the next step writes
    bool lagged = false;
    bclbm::DevParams* d_params = nullptr;
    double* d_partials = nullptr;
    double* d_red = nullptr;
    double* d_gather = nullptr;
    int32_t ghost_src[19] = {0};
    int64_t steps_done = 0;
    size_t footprint = 0;             // device bytes (bclbm_footprint of the descriptor)
    // asynchronous macro download: pinned staging of rho, vel (slot order) and the
    // colour, and the event recorded after the copies
    double* stage = nullptr;
    float* stage_cgf = nullptr;
    cudaEvent_t stage_event = nullptr;
    bool stage_pending = false;
    bool stage_cg = false;
    // the std_one_phase step (BCLBM_LINKS): per-slot info / u_store index / force
    // attribute, the velocity store of the pressure-boundary nodes, the interior
    // domains' node lists, sums and sources, and the mass-flux node list
    uint32_t* d_info = nullptr;
    int32_t* d_pidx = nullptr;
    int32_t* d_force_on = nullptr;
    double* d_ustore = nullptr;
    int32_t* d_lab_slot = nullptr;
    int32_t* d_lab_start = nullptr;
    double* d_lab_val = nullptr;
    double* d_lab_g = nullptr;
    double* d_lab_q = nullptr;
    int32_t* d_flux_slot = nullptr;
    int32_t* d_flux_phase = nullptr;
    double* d_flux_out = nullptr;
    int npress = 0, nlab = 0, nlabeled = 0, nflux = 0;
    double rho_w = 1.0, force_on_sum = 0.0;
    std::string last_error;
};

namespace bclbm {
// kernel arguments of a handle's current configuration (src/dst left for the caller)
StepArgs handle_args(const bclbm_handle* h);
// reference node number of device slot s
inline int32_t slot_node_of(const bclbm_handle* h, size_t s) {
    return h->affine ? h->bulk0 + static_cast<int32_t>(s) : h->slot_node[s];
}
}  // namespace bclbm
