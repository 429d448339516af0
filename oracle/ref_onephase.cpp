// Oracle driver for the std_one_phase step, around the UNMODIFIED reference.
//
// Test infrastructure only, built into oracle/_ref/ like ref_driver.cpp.  The
// reference's src/std_one_phase/main.cpp is compiled in as it is, with its
// main() renamed, so that its own link finders and boundary functions
// (findSolidFluidLinks, findPressureFluidLinks, findFluidFluidLinks,
// applySolidFluidBoundary, applyPressureFluidBoundary, applyFluidFluidBoundary,
// main.cpp:24-203) do the boundary work.  The set-up and the time loop of its
// main() (main.cpp:239-575: attributes, interior-domain mass sources, the node
// loop, swap, boundaries, the write step's mass flux) are restated below with
// the reference's own lbsolver calls, reading a .vtklb file given on the
// command line instead of the hard-coded input paths, with the output files
// replaced by dumps:
//
//   ref_onephase <vtklb> <outdir> steps=<n> tau=<t> fx=.. fy=.. fz=..
//     writes <outdir>/f, rho, vel (LbField/ScalarField/VectorField::writeToFile)
//     and <outdir>/flux.txt (q1 q2 of the last step, %.17g)
#define main bclbm_std_one_phase_main_unused
#include "std_one_phase/main.cpp"
#undef main

#include <cstdio>
#include <map>
#include <string>

namespace {

std::map<std::string, double> parse_kv(int argc, char** argv, int first) {
    std::map<std::string, double> kv;
    for (int i = first; i < argc; ++i) {
        std::string a(argv[i]);
        auto eq = a.find('=');
        if (eq == std::string::npos) {
            std::fprintf(stderr, "bad argument %s\n", argv[i]);
            std::exit(2);
        }
        kv[a.substr(0, eq)] = std::atof(a.substr(eq + 1).c_str());
    }
    return kv;
}

double get(const std::map<std::string, double>& kv, const char* k, double dflt) {
    auto it = kv.find(k);
    return it == kv.end() ? dflt : it->second;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 3) {
        std::fprintf(stderr, "usage: %s <file.vtklb> <outdir> [key=value ...]\n", argv[0]);
        return 2;
    }
    MPI_Init(NULL, NULL);
    int nProcs;
    MPI_Comm_size(MPI_COMM_WORLD, &nProcs);
    int myRank;
    MPI_Comm_rank(MPI_COMM_WORLD, &myRank);
    const std::string out(argv[2]);
    auto kv = parse_kv(argc, argv, 3);
    const int nIterations = static_cast<int>(get(kv, "steps", 1));
    const lbBase_t tau = get(kv, "tau", 1.0);
    VectorField<LT> bodyForce(1, 1, std::vector<lbBase_t>{get(kv, "fx", 0.0), get(kv, "fy", 0.0), get(kv, "fz", 0.0)});

    LBvtk<LT> vtklb(argv[1]);
    Grid<LT> grid(vtklb);
    Nodes<LT> nodes(vtklb, grid);
    BndMpi<LT> mpiBoundary(vtklb, nodes, grid);
    std::vector<int> bulkNodes = findBulkNodes(nodes);

    // attributes (main.cpp:256-313)
    vtklb.toAttribute("nodetags");
    for (int n = vtklb.beginNodeNo(); n < vtklb.endNodeNo(); ++n) nodes.setTag(vtklb.getScalarAttribute<int>(), n);
    ScalarField forceOn(1, grid.size());
    vtklb.toAttribute("force");
    for (int n = vtklb.beginNodeNo(); n < vtklb.endNodeNo(); ++n) forceOn(0, n) = vtklb.getScalarAttribute<int>();
    std::vector<int> interiorDomainsLabel(grid.size(), 0);
    std::vector<lbBase_t> addMassSource(grid.size(), 0.0);
    vtklb.toAttribute("interior_domains");
    int localDomainLabelMax = 0;
    for (int n = vtklb.beginNodeNo(); n < vtklb.endNodeNo(); ++n) {
        int val = vtklb.getScalarAttribute<int>();
        interiorDomainsLabel[n] = val;
        if (nodes.isMyRank(n))
            if (val > localDomainLabelMax) localDomainLabelMax = val;
    }
    VectorField<LT> normals(1, grid.size());
    const char* nname[3] = {"normal_x", "normal_y", "normal_z"};
    for (int d = 0; d < 3; ++d) {
        vtklb.toAttribute(nname[d]);
        for (int n = vtklb.beginNodeNo(); n < vtklb.endNodeNo(); ++n) normals(0, d, n) = vtklb.getScalarAttribute<lbBase_t>();
    }

    // interior-domain mass sources (main.cpp:318-358)
    int globalDomainLabelMax;
    MPI_Allreduce(&localDomainLabelMax, &globalDomainLabelMax, 1, MPI_INT, MPI_MAX, MPI_COMM_WORLD);
    std::vector<lbBase_t> massSourceScaleFactor(globalDomainLabelMax + 1, 0);
    std::vector<lbBase_t> massChangeLocal(globalDomainLabelMax + 1, 0);
    std::vector<lbBase_t> massChange(globalDomainLabelMax + 1, 0);
    {
        std::vector<lbBase_t> tmp(globalDomainLabelMax + 1, 0.0);
        for (int n = 1; n < grid.size(); ++n) {
            if (nodes.isMyRank(n)) {
                int label = interiorDomainsLabel[n];
                int tag = nodes.getTag(n);
                if ((label > 0) && (tag < 3)) {
                    tmp[label] += 1;
                    addMassSource[n] = 1.0;
                }
            }
        }
        MPI_Allreduce(tmp.data(), massSourceScaleFactor.data(), globalDomainLabelMax + 1, MPI_DOUBLE, MPI_SUM,
                      MPI_COMM_WORLD);
        for (int i = 1; i < globalDomainLabelMax + 1; ++i) {
            if (massSourceScaleFactor[i] == 0.0) {
                std::cout << "ERROR: Interior domain " << i << " has no interior nodes!" << std::endl;
                exit(1);
            }
            massSourceScaleFactor[i] = 1.0 / massSourceScaleFactor[i];
        }
    }
    auto pressureFluidNodes = findPressureFluidNodes(nodes, grid);

    // fields (main.cpp:414-468)
    ScalarField rho(1, grid.size());
    for (int n = vtklb.beginNodeNo(); n < vtklb.endNodeNo(); ++n) rho(0, n) = 1.0;
    VectorField<LT> vel(1, grid.size());
    for (auto nodeNo : bulkNodes) vel.set(0, nodeNo) = 0;
    auto solidFluidLinks = findSolidFluidLinks(nodes, grid);
    auto pressureFluidLinks = findPressureFluidLinks(nodes, grid);
    auto fluidFluidLinks = findFluidFluidLinks(nodes, grid);
    LbField<LT> f(1, grid.size());
    LbField<LT> fTmp(1, grid.size());
    for (auto nodeNo : bulkNodes) {
        auto u2 = LT::dot(vel(0, nodeNo), vel(0, nodeNo));
        auto cu = LT::cDotAll(vel(0, nodeNo));
        f.set(0, nodeNo) = calcfeq<LT>(rho(0, nodeNo), u2, cu);
        fTmp.set(0, nodeNo) = 0;
    }

    // main loop (main.cpp:480-575; the output files are left out)
    std::vector<lbBase_t> massFluxGlobal(2, 0.0);
    for (int i = 0; i < nIterations; i++) {
        std::fill(massChangeLocal.begin(), massChangeLocal.end(), 0.0);
        for (auto nodeNo : bulkNodes) {
            const std::valarray<lbBase_t> fNode = f(0, nodeNo);
            const lbBase_t rhoNode = calcRho<LT>(fNode);
            int label = interiorDomainsLabel[nodeNo];
            massChangeLocal[label] += 1.0 - rhoNode;
        }
        MPI_Allreduce(massChangeLocal.data(), massChange.data(), massChange.size(), MPI_DOUBLE, MPI_SUM,
                      MPI_COMM_WORLD);
        std::fill(massChangeLocal.begin(), massChangeLocal.end(), 0.0);
        for (auto nodeNo : bulkNodes) {
            const std::valarray<lbBase_t> fNode = f(0, nodeNo);
            lbBase_t rhoNode = calcRho<LT>(fNode);
            int label = interiorDomainsLabel[nodeNo];
            lbBase_t qMassConservation = 0.9 * 2 * massSourceScaleFactor[label] * massChange[label] * addMassSource[nodeNo];
            rhoNode += 0.5 * qMassConservation;
            massChangeLocal[label] += 1.0 - rhoNode;
            const std::valarray<lbBase_t> forceNode = bodyForce(0, 0) * forceOn(0, nodeNo);
            const auto velNode = calcVel<LT>(fNode, rhoNode, forceNode);
            rho(0, nodeNo) = rhoNode;
            vel.set(0, nodeNo) = velNode;
            const lbBase_t u2 = LT::dot(velNode, velNode);
            const std::valarray<lbBase_t> cu = LT::cDotAll(velNode);
            const std::valarray<lbBase_t> omegaBGK = calcOmegaBGK<LT>(fNode, tau, rhoNode, u2, cu);
            const lbBase_t uF = LT::dot(velNode, forceNode);
            const std::valarray<lbBase_t> cF = LT::cDotAll(forceNode);
            const std::valarray<lbBase_t> deltaOmegaF = calcDeltaOmegaF<LT>(tau, cu, uF, cF);
            const std::valarray<lbBase_t> deltaOmegaQ0 = calcDeltaOmegaQ<LT>(tau, cu, u2, qMassConservation);
            fTmp.propagateTo(0, nodeNo, fNode + omegaBGK + deltaOmegaF + deltaOmegaQ0, grid);
        }
        f.swapData(fTmp);
        mpiBoundary.communicateLbField(f, grid);
        mpiBoundary.communciateVectorField_TEST(vel);
        applySolidFluidBoundary(f, solidFluidLinks);
        applyPressureFluidBoundary(f, vel, 1.0, pressureFluidLinks);
        applyFluidFluidBoundary(f, vel, normals, fluidFluidLinks, nodes);
        // the write step's mass flux (main.cpp:548-562)
        std::vector<lbBase_t> massFluxLocal(2, 0.0);
        for (auto n : pressureFluidNodes) {
            int fluidPhase = (nodes.getTag(n) & 3) - 1;
            if ((fluidPhase != 0) && (fluidPhase != 1)) {
                std::cout << "Fluid phase = " << fluidPhase << " in write mass flux" << std::endl;
                MPI_Finalize();
                exit(1);
            }
            massFluxLocal[fluidPhase] += vel(0, 2, n) * rho(0, n);
        }
        MPI_Allreduce(massFluxLocal.data(), massFluxGlobal.data(), 2, MPI_DOUBLE, MPI_SUM, MPI_COMM_WORLD);
    }
    f.writeToFile(out + "/f");
    rho.writeToFile(out + "/rho");
    vel.writeToFile(out + "/vel");
    if (FILE* fp = std::fopen((out + "/flux.txt").c_str(), "w")) {
        std::fprintf(fp, "%.17g %.17g\n", 0.5 * massFluxGlobal[0], 0.5 * massFluxGlobal[1]);
        std::fclose(fp);
    }
    std::printf("onephase: %d steps on %zu fluid nodes, %zu solid, %zu pressure, %zu fluid-fluid links, %d domains\n",
                nIterations, bulkNodes.size(), solidFluidLinks.size(), pressureFluidLinks.size(), fluidFluidLinks.size(),
                globalDomainLabelMax);
    MPI_Finalize();
    return 0;
}
