// The host-side lattice object of the C ABI (bclbm_lattice_build,
// bclbm_lattice_read_vtklb): the arrays the reference's Grid and Nodes hold for
// one rank, plus the scalar attributes of a .vtklb file.
#pragma once

#include <cstdint>
#include <map>
#include <string>
#include <vector>

struct bclbm_lattice {
    int q = 0, nd = 0;
    int64_t nf = 0, ns = 0;
    std::vector<int32_t> neigh;  // [n_nodes * q]
    std::vector<int16_t> types;  // [n_nodes]
    std::vector<int32_t> pos;    // [n_nodes * nd], -1 for node 0
    std::vector<int32_t> global_dims;                     // .vtklb GLOBAL_DIMENSIONS
    std::map<std::string, std::vector<double>> attributes;  // .vtklb SCALARS, [n_nodes], 0 at node 0
    std::string error;
};
