/*
 * bclbm_lbsolver.hpp: C++ adaptor between the reference's lbsolver objects and
 * the C ABI of bclbm.h.  Header only; include it after the reference's
 * LBSOLVER.h (it names Grid, Nodes, LbField, ScalarField and VectorField).
 *
 * The reference has no plugin interface: its main files run the per-node loops
 * themselves.  The adaptor replaces, in those loops, everything between the
 * start of an iteration and the output step with one call:
 *
 *   src/std_case/main.cpp:109-146
 *     for (int i = 0; i <= nIterations; i++) {
 *         step.run(1);                        // node loop, swapData, communicate, bounce-back
 *         if ((i % nItrWrite) == 0) {
 *             step.download_macros(rho, vel);  // what the node loop stored in rho / vel
 *             output.write(i);
 *         }
 *     }
 *   with   bclbm::LbStep<LT> step(grid, nodes, bulkNodes, f,
 *                                 bclbm::SinglePhase{tau, {Fx, Fy, Fz}});
 *
 *   src/twophase/main_TWOPHASE.cpp:236-393 likewise, with
 *          bclbm::LbStep<LT> step(grid, nodes, bulkNodes, f, rho,
 *                                 bclbm::TwoPhase{tau0, tau1, sigma, beta, {Fx, Fy, Fz}});
 *   and step.download_macros(rho, vel, cgField) before output.write(i).
 *
 * The tables are read through the reference's accessors (Grid::neighbor,
 * Grid::pos, Nodes::getType: src/lbsolver/LBgrid.h:97-112, LBnodes.h:72) and the
 * fields through their element references (LBfield.h:59, 170, 298), once, at
 * construction.  The device keeps its own copies; downloads write back in the
 * reference's layout and numbering.
 *
 * Errors follow the reference's convention (print and exit(1), as in
 * src/lbsolver/LBvtk.h:230-233); define BCLBM_ADAPTOR_THROW before including this
 * header to get a std::runtime_error instead.
 */
#ifndef BCLBM_LBSOLVER_HPP
#define BCLBM_LBSOLVER_HPP

#include <array>
#include <cstdint>
#include <functional>
#include <cstdlib>
#include <iostream>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "bclbm.h"

namespace bclbm {

/* std_case: BGK (tau_anti = 0) or TRT with the antisymmetric time tau_anti;
 * force = bodyForce(0, 0) of the main file. */
struct SinglePhase {
    double tau;
    std::array<double, 3> force;
    double tau_anti = 0.0;
    int32_t precision = BCLBM_F64;
    uint32_t flags = 0;
    double store_scale = 0.0;
};

/* twophase: fluid.tau[0], fluid.tau[1], fluid.sigma, fluid.beta and the body
 * force; flux_control = 1 keeps the flux controller of main_TWOPHASE.cpp:292-308
 * with target mom_x. */
struct TwoPhase {
    double tau0, tau1, sigma, beta;
    std::array<double, 3> force;
    int32_t flux_control = 0;
    double mom_x = 0.0;
    int32_t precision = BCLBM_F64;
    uint32_t flags = 0;
    double store_scale = 0.0;
};

/* std_one_phase: relaxation time, body force and the pressure-boundary density
 * (main.cpp:537 passes 1.0); flags BCLBM_FLAG_EXACT for the reference's rounding. */
struct OnePhaseLinks {
    double tau;
    std::array<double, 3> force;
    double rho_w = 1.0;
    uint32_t flags = 0;
};

[[noreturn]] inline void adaptor_fail(const std::string& what) {
#ifdef BCLBM_ADAPTOR_THROW
    throw std::runtime_error(what);
#else
    std::cout << what << std::endl;
    std::exit(1);
#endif
}

inline void adaptor_check(int rc, const bclbm_handle* h, const char* call) {
    if (rc == BCLBM_OK) return;
    std::string msg = std::string("bclbm: ") + call + " failed: " + bclbm_error(rc);
    if (h) {
        const std::string detail = bclbm_last_error(h);
        if (!detail.empty()) msg += " (" + detail + ")";
    }
    adaptor_fail(msg);
}

/* The reference's Grid/Nodes arrays in the layout bclbm_desc takes. */
template <typename DXQY>
struct LbTables {
    std::vector<int32_t> neigh;  // [N*Q]
    std::vector<int16_t> types;  // [N]
    std::vector<int32_t> pos;    // [N*nD]
    std::vector<int32_t> bulk;   // [n_bulk]

    template <class GridT, class NodesT>
    LbTables(const GridT& grid, const NodesT& nodes, const std::vector<int>& bulkNodes) {
        const int N = grid.size();
        neigh.resize(static_cast<size_t>(N) * DXQY::nQ);
        types.resize(static_cast<size_t>(N));
        for (int n = 0; n < N; ++n) {
            for (int q = 0; q < DXQY::nQ; ++q) neigh[static_cast<size_t>(n) * DXQY::nQ + q] = grid.neighbor(q, n);
            types[static_cast<size_t>(n)] = static_cast<int16_t>(nodes.getType(n));
        }
        const std::vector<int>& p = grid.pos();
        pos.assign(p.begin(), p.end());
        bulk.assign(bulkNodes.begin(), bulkNodes.end());
    }
};

template <typename DXQY>
class LbStep {
public:
    /* std_case */
    template <class GridT, class NodesT>
    LbStep(const GridT& grid, const NodesT& nodes, const std::vector<int>& bulkNodes, const LbField<DXQY>& f,
           const SinglePhase& p)
        : tab_(grid, nodes, bulkNodes), nfields_(1) {
        if (f.num_fields() != 1) adaptor_fail("bclbm: the std_case LbField has one field");
        bclbm_desc d = base_desc(grid.size());
        d.collision = p.tau_anti > 0.0 ? BCLBM_TRT : BCLBM_BGK;
        d.precision = p.precision;
        d.flags = p.flags;
        d.tau[0] = p.tau;
        d.tau[1] = p.tau_anti > 0.0 ? p.tau_anti : p.tau;
        for (int k = 0; k < 3; ++k) d.force[k] = p.force[k];
        d.store_scale = p.store_scale;
        d.f_init = &f(0, 0, 0);
        create(d);
    }

    /* twophase: rho holds the two phase densities (ScalarField(2, N)); only the
     * solid boundary entries (the wettability densities) are read */
    template <class GridT, class NodesT>
    LbStep(const GridT& grid, const NodesT& nodes, const std::vector<int>& bulkNodes, const LbField<DXQY>& f,
           const ScalarField& rho, const TwoPhase& p)
        : tab_(grid, nodes, bulkNodes), nfields_(2) {
        if (f.num_fields() != 2 || rho.num_fields() != 2)
            adaptor_fail("bclbm: the twophase LbField and ScalarField have two fields");
        bclbm_desc d = base_desc(grid.size());
        d.collision = BCLBM_RK;
        d.precision = p.precision;
        d.flags = p.flags;
        d.tau[0] = p.tau0;
        d.tau[1] = p.tau1;
        d.sigma = p.sigma;
        d.beta = p.beta;
        d.flux_control = p.flux_control;
        d.mom_x = p.mom_x;
        for (int k = 0; k < 3; ++k) d.force[k] = p.force[k];
        d.store_scale = p.store_scale;
        d.f_init = &f(0, 0, 0);
        d.rho_init = &rho(0, 0);
        create(d);
    }

    /* std_one_phase (src/std_one_phase/main.cpp:239-575): the node tags are read
     * through Nodes::getTag, the interior-domain labels and the force indicator
     * as main.cpp:284-305 stores them */
    template <class GridT, class NodesT>
    LbStep(const GridT& grid, const NodesT& nodes, const std::vector<int>& bulkNodes, const LbField<DXQY>& f,
           const std::vector<int>& interiorDomainsLabel, const ScalarField& forceOn, const OnePhaseLinks& p)
        : tab_(grid, nodes, bulkNodes), nfields_(1) {
        const int N = grid.size();
        if (f.num_fields() != 1 || static_cast<int>(interiorDomainsLabel.size()) != N)
            adaptor_fail("bclbm: std_one_phase takes one LbField field and a label per node");
        std::vector<int32_t> tags(static_cast<size_t>(N), -1), labels(interiorDomainsLabel.begin(),
                                                                      interiorDomainsLabel.end()),
            force(static_cast<size_t>(N), 0);
        for (int n = 1; n < N; ++n) {
            tags[static_cast<size_t>(n)] = nodes.getTag(n);
            force[static_cast<size_t>(n)] = static_cast<int32_t>(forceOn(0, n));
        }
        bclbm_desc d = base_desc(N);
        d.collision = BCLBM_LINKS;
        d.precision = BCLBM_F64;
        d.flags = p.flags;
        d.tau[0] = d.tau[1] = p.tau;
        for (int k = 0; k < 3; ++k) d.force[k] = p.force[k];
        d.f_init = &f(0, 0, 0);
        d.tags = tags.data();
        d.labels = labels.data();
        d.force_on = force.data();
        d.rho_w = p.rho_w;
        create(d);
    }

    /* std_one_phase: the write step's q1, q2 (main.cpp:548-562) of the last step */
    std::array<double, 2> pressure_flux() const {
        std::array<double, 2> q{};
        adaptor_check(bclbm_pressure_flux(h_, q.data()), h_, "bclbm_pressure_flux");
        return q;
    }

    LbStep(const LbStep&) = delete;
    LbStep& operator=(const LbStep&) = delete;
    ~LbStep() { bclbm_destroy(h_); }

    /* nsteps iterations of the main-file loop body (asynchronous) */
    void run(int nsteps) { adaptor_check(bclbm_step(h_, nsteps), h_, "bclbm_step"); }

    /* f after the last iteration (the bulk rows of the reference's LbField) */
    void download(LbField<DXQY>& f) const { adaptor_check(bclbm_download_f(h_, &f(0, 0, 0)), h_, "bclbm_download_f"); }

    /* rho / vel as the last iteration's node loop stored them */
    void download_macros(ScalarField& rho, VectorField<DXQY>& vel) const {
        adaptor_check(bclbm_download_macros(h_, &rho(0, 0), &vel(0, 0, 0), nullptr), h_, "bclbm_download_macros");
    }
    /* twophase: also the colour field cgField */
    void download_macros(ScalarField& rho, VectorField<DXQY>& vel, ScalarField& cg) const {
        adaptor_check(bclbm_download_macros(h_, &rho(0, 0), &vel(0, 0, 0), &cg(0, 0)), h_, "bclbm_download_macros");
    }

    /* the same download in two halves: begin after the step to be written, run the
     * next steps, collect before Output::write (the host writes while the GPU steps) */
    void macros_begin() { adaptor_check(bclbm_macros_begin(h_), h_, "bclbm_macros_begin"); }
    void macros_collect(ScalarField& rho, VectorField<DXQY>& vel) const {
        adaptor_check(bclbm_macros_collect(h_, &rho(0, 0), &vel(0, 0, 0), nullptr), h_, "bclbm_macros_collect");
    }
    void macros_collect(ScalarField& rho, VectorField<DXQY>& vel, ScalarField& cg) const {
        adaptor_check(bclbm_macros_collect(h_, &rho(0, 0), &vel(0, 0, 0), &cg(0, 0)), h_, "bclbm_macros_collect");
    }

    /* FP64 sums: mass per field, momentum, flux-controller sum, saturation */
    bclbm_stats stats() const {
        bclbm_stats s;
        adaptor_check(bclbm_reduce(h_, &s), h_, "bclbm_reduce");
        return s;
    }

    void set_force(const std::array<double, 3>& F) {
        adaptor_check(bclbm_set_force(h_, F.data()), h_, "bclbm_set_force");
    }

    bclbm_handle* handle() const { return h_; }
    const LbTables<DXQY>& tables() const { return tab_; }

private:
    bclbm_desc base_desc(int n_nodes) const {
        bclbm_desc d{};
        d.lattice_q = DXQY::nQ;
        d.n_nodes = n_nodes;
        d.neigh = tab_.neigh.data();
        d.types = tab_.types.data();
        d.n_bulk = static_cast<int32_t>(tab_.bulk.size());
        d.bulk = tab_.bulk.data();
        d.pos = tab_.pos.data();
        d.rho_ref = 1.0;
        return d;
    }

    void create(const bclbm_desc& d) { adaptor_check(bclbm_create(&d, &h_), nullptr, "bclbm_create"); }

    LbTables<DXQY> tab_;
    int nfields_;
    bclbm_handle* h_ = nullptr;
};

/* The output step: Output<LT, T, FMT> of src/io/Output.h:26-177 written by the
 * library's VTU writer (bclbm_output_*, bclbm.h).  Same constructors and calls
 * as the reference's class, the same files byte for byte; write_async returns
 * once the values are read and writes the files on a background thread, so
 *
 *   step.download_macros(rho, vel);
 *   output.write_async(i);        // the host writes while
 *   step.run(nItrWrite);          // the GPU steps
 *
 * overlaps the file write with the next steps.  FMT: 0 binary (VTK::BINARY, the
 * reference's default), 1 ASCII. */
template <typename DXQY, typename T = double, int FMT = 0>
class Output {
public:
    /* Output(grid, nodes, dir, rank, nproc) (Output.h:51-54) */
    template <class GridT>
    Output(const GridT& grid, const std::vector<int>& nodes, const std::string& dir, int rank, int nproc)
        : nodes_(nodes.begin(), nodes.end()) {
        const std::vector<int> p = grid.pos(nodes);
        create(std::vector<int32_t>(p.begin(), p.end()), nodes_.data(), dir, rank, nproc);
    }
    /* Output(pos, dir, rank, nproc) (Output.h:44-47): plain vectors only */
    Output(const std::vector<int>& pos, const std::string& dir, int rank, int nproc) {
        create(std::vector<int32_t>(pos.begin(), pos.end()), nullptr, dir, rank, nproc);
    }
    /* Output(pos, dir, rank, nproc, varname, var) (Output.h:35-41) */
    Output(const std::vector<int>& pos, const std::string& dir, int rank, int nproc, const std::string& varname,
           const std::vector<T>& var)
        : Output(pos, dir, rank, nproc) {
        add_file(varname);
        add_vector(varname, var);
    }
    Output(const Output&) = delete;
    Output& operator=(const Output&) = delete;
    ~Output() { bclbm_output_destroy(o_); }

    void add_file(const std::string& name) { check(bclbm_output_add_file(o_, name.c_str()), "bclbm_output_add_file"); }

    void add_scalar_variables(const std::vector<std::string>& names,
                              const std::vector<std::reference_wrapper<const ScalarField>>& fields) {
        add_fields(names, fields);
    }
    void add_vector_variables(const std::vector<std::string>& names,
                              const std::vector<std::reference_wrapper<const VectorField<DXQY>>>& fields) {
        add_fields(names, fields);
    }
    template <typename F>
    void add_variable(const std::string& name, const F& field) {
        add_field(name, field, -1);
    }
    /* one variable per field, named explicitly (Output.h:111-126) */
    template <typename F>
    void add_variable_with_names(const std::vector<std::string>& names, const F& field) {
        if (static_cast<int>(names.size()) != field.num_fields())
            adaptor_fail("bclbm: add_variable_with_names: size of names-vector does not match number of fields");
        for (int i = 0; i < field.num_fields(); ++i) add_field(names[static_cast<size_t>(i)], field, i);
    }
    /* plain vectors (Output.h:137-142) */
    void add_variables(const std::vector<std::string>& names,
                       const std::vector<std::reference_wrapper<std::vector<T>>>& vectors) {
        for (size_t i = 0; i < names.size() && i < vectors.size(); ++i) add_vector(names[i], vectors[i].get());
    }

    void write(double t = 0.0) { check(bclbm_output_write(o_, t), "bclbm_output_write"); }
    void write_async(double t = 0.0) { check(bclbm_output_write_async(o_, t), "bclbm_output_write_async"); }
    void wait() { check(bclbm_output_wait(o_), "bclbm_output_wait"); }

private:
    static constexpr int32_t type_code() {
        return std::is_same<T, double>::value ? BCLBM_VTU_FLOAT64
                                              : (std::is_same<T, float>::value ? BCLBM_VTU_FLOAT32 : BCLBM_VTU_INT32);
    }
    static_assert(std::is_same<T, double>::value || std::is_same<T, float>::value || std::is_same<T, int>::value,
                  "the writer writes double, float or int");

    void create(const std::vector<int32_t>& pos, const int32_t* nodes, const std::string& dir, int rank, int nproc) {
        const int64_t n = static_cast<int64_t>(pos.size() / DXQY::nD);
        const int rc = bclbm_output_create(DXQY::nD, n, pos.data(), nodes, dir.c_str(), rank, nproc, type_code(), FMT,
                                           &o_);
        if (rc != BCLBM_OK) adaptor_fail(std::string("bclbm: bclbm_output_create failed: ") + bclbm_error(rc));
    }
    void check(int rc, const char* call) const {
        if (rc == BCLBM_OK) return;
        std::string msg = std::string("bclbm: ") + call + " failed: " + bclbm_error(rc);
        const std::string detail = bclbm_output_last_error(o_);
        if (!detail.empty()) msg += " (" + detail + ")";
        adaptor_fail(msg);
    }
    template <typename F>
    void add_fields(const std::vector<std::string>& names, const std::vector<std::reference_wrapper<const F>>& fields) {
        for (size_t i = 0; i < names.size() && i < fields.size(); ++i) add_field(names[i], fields[i].get(), -1);
    }
    template <typename F>
    void add_field(const std::string& name, const F& field, int field_no) {
        check(bclbm_output_add_field(o_, name.c_str(), &field.data()[0], field.num_fields(), field.dim(), field_no),
              "bclbm_output_add_field");
    }
    void add_vector(const std::string& name, const std::vector<T>& v) {
        check(bclbm_output_add_array(o_, name.c_str(), v.data(), type_code(), static_cast<int64_t>(v.size())),
              "bclbm_output_add_array");
    }

    std::vector<int32_t> nodes_;
    bclbm_output* o_ = nullptr;
};

}  // namespace bclbm

#endif
