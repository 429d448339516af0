// Compile-and-run check of include/bclbm_lbsolver.hpp against the reference's
// own lbsolver objects (built by tests/test_adaptor.py with the reference
// headers and the single-rank mpi.h stub of oracle/mpi_stub; test only).
//
//   adaptor_check <vtklb> <outdir>
// reads the .vtklb file into the reference's LBvtk / Grid / Nodes, writes the
// adaptor's tables (neigh.i32, types.i16, pos.i32, bulk.i32) into outdir,
// writes the same fields with the reference's Output<LT> and with
// bclbm::Output<LT> into outdir/ref_out and outdir/our_out, then builds an
// LbStep from the tables and runs 3 steps; prints "status <text>" with the
// adaptor's error message, or "ran <sum of f>" when a GPU ran the steps.
#include "IO.h"
#include "LBSOLVER.h"

#define BCLBM_ADAPTOR_THROW
#include "bclbm_lbsolver.hpp"

#include <cstdio>
#include <fstream>
#include <string>

#ifndef BCLBM_LT
#define BCLBM_LT D3Q19
#endif
#define LT BCLBM_LT

template <typename T>
static void dump(const std::string& path, const std::vector<T>& v) {
    std::ofstream ofs(path, std::ios::binary);
    ofs.write(reinterpret_cast<const char*>(v.data()), static_cast<std::streamsize>(v.size() * sizeof(T)));
}

int main(int argc, char** argv) {
    if (argc < 3) return 2;
    MPI_Init(NULL, NULL);
    LBvtk<LT> vtklb(argv[1]);
    Grid<LT> grid(vtklb);
    Nodes<LT> nodes(vtklb, grid);
    BndMpi<LT> mpiBoundary(vtklb, nodes, grid);
    std::vector<int> bulkNodes = findBulkNodes(nodes);
    const std::string out(argv[2]);
    bclbm::LbTables<LT> tab(grid, nodes, bulkNodes);
    dump(out + "/neigh.i32", tab.neigh);
    dump(out + "/types.i16", tab.types);
    dump(out + "/pos.i32", tab.pos);
    dump(out + "/bulk.i32", tab.bulk);
    {
        ScalarField rho(2, grid.size());
        VectorField<LT> vel(1, grid.size());
        for (int n = 0; n < grid.size(); ++n) {
            rho(0, n) = 1.0 + 1e-3 * n;
            rho(1, n) = 0.5 - 1e-4 * n;
            for (int d = 0; d < LT::nD; ++d) vel(0, d, n) = 1e-5 * (n % 17) - 2e-5 * d;
        }
        auto geo = nodes.geo(grid, vtklb);
        Output<LT> ro(grid, bulkNodes, out + "/ref_out", 0, 1);
        ro.add_file("lb_run");
        ro.add_scalar_variables({"rho"}, {rho});
        ro.add_vector_variables({"vel"}, {vel});
        ro.add_file("named");
        ro.add_variable_with_names({"red", "blue"}, rho);
        Output<LT, int> rg(grid.pos(), out + "/ref_out", 0, 1, "geo", geo);
        bclbm::Output<LT> bo(grid, bulkNodes, out + "/our_out", 0, 1);
        bo.add_file("lb_run");
        bo.add_scalar_variables({"rho"}, {rho});
        bo.add_vector_variables({"vel"}, {vel});
        bo.add_file("named");
        bo.add_variable_with_names({"red", "blue"}, rho);
        bclbm::Output<LT, int> bg(grid.pos(), out + "/our_out", 0, 1, "geo", geo);
        ro.write(0);
        rg.write();
        bo.write(0);
        bg.write();
        for (int n = 0; n < grid.size(); ++n) rho(0, n) *= 3.0;
        ro.write(500);
        bo.write_async(500);
        bo.wait();
    }
    LbField<LT> f(1, grid.size());
    for (auto n : bulkNodes)
        for (int q = 0; q < LT::nQ; ++q) f(0, q, n) = LT::w[q] * 1.0;
    try {
        bclbm::LbStep<LT> step(grid, nodes, bulkNodes, f, bclbm::SinglePhase{0.8, {1e-5, 0.0, 0.0}});
        step.run(3);
        step.download(f);
        ScalarField rho(1, grid.size());
        VectorField<LT> vel(1, grid.size());
        step.download_macros(rho, vel);
        double s = 0.0;
        for (auto n : bulkNodes)
            for (int q = 0; q < LT::nQ; ++q) s += f(0, q, n);
        std::printf("ran %.17g\n", s);
    } catch (const std::runtime_error& e) {
        std::printf("status %s\n", e.what());
    }
    // the std_one_phase constructor (node tags from Nodes::getTag; none are set here,
    // so every tag is the -1 Nodes starts with)
    try {
        ScalarField forceOn(1, grid.size());
        std::vector<int> labels(grid.size(), 0);
        bclbm::LbStep<LT> links(grid, nodes, bulkNodes, f, labels, forceOn, bclbm::OnePhaseLinks{0.8, {0.0, 0.0, 1e-5}});
        links.run(2);
        const auto q = links.pressure_flux();
        std::printf("links ran %.17g\n", q[0]);
    } catch (const std::runtime_error& e) {
        std::printf("links status %s\n", e.what());
    }
    MPI_Finalize();
    return 0;
}
