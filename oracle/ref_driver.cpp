// Oracle driver around the UNMODIFIED reference lbsolver headers.
//
// Test infrastructure only.  This file is compiled against the reference
// sources where they lie (src/LBSOLVER.h, src/IO.h) together with the
// single-rank mpi.h stub in oracle/mpi_stub, and is built into oracle/_ref/.
// It runs the reference's own per-node loops so that its outputs are the
// reference's outputs, and dumps them in the reference's binary formats
// (LbField/ScalarField/VectorField::writeToFile, src/lbsolver/LBfield.h:102-138,
// 233-248, 378-393) plus raw dumps of the setup tables.
//
// Modes
//   tables   <vtklb> <out>           neighbour table, node types, bulk list and
//                                    half-way bounce-back link classes
//   single   <vtklb> <out> k=v ...   the std_case loop (src/std_case/main.cpp:109-146)
//                                    with BGK (calcOmegaBGK + calcDeltaOmegaF) or,
//                                    with trt=1, calcOmegaBGKTRT + calcDeltaOmegaFTRT(phi=1)
//   twophase <vtklb> <out> k=v ...   the twophase loop (src/twophase/main_TWOPHASE.cpp:236-393);
//                                    momx=<target> keeps the reference flux controller
//                                    (:292-308), otherwise the body force stays constant
//   vtu      <vtklb> <out> nfields=k     the output step (src/io/Output.h:26-177): rho [N*k] and
//                                    vel [N*k*nD] read from <out>/fields.bin are written by
//                                    Output<LT> (Float64, binary; two files, two writes, rho
//                                    doubled in between), Output<LT, float>, Output<LT, double,
//                                    VTK::ASCII> and the geo file of main_TWOPHASE.cpp:222-224,
//                                    into <out>/f64, <out>/f32, <out>/ascii and <out>/geo
//
// The lattice is chosen at compile time with -DBCLBM_LT=D2Q9|D3Q19, as the
// reference mains do with '#define LT' (src/std_case/main.cpp:14-15).

#include "LBSOLVER.h"
#include "IO.h"

#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <map>
#include <string>
#include <vector>

#ifndef BCLBM_LT
#define BCLBM_LT D2Q9
#endif
#define LT BCLBM_LT

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

template <typename T>
void dump_raw(const std::string& path, const std::vector<T>& v) {
    std::ofstream ofs(path, std::ios::binary);
    ofs.write(reinterpret_cast<const char*>(v.data()), static_cast<std::streamsize>(v.size() * sizeof(T)));
}

int run_tables(LBvtk<LT>& vtklb, const std::string& out) {
    Grid<LT> grid(vtklb);
    Nodes<LT> nodes(vtklb, grid);
    BndMpi<LT> mpiBoundary(vtklb, nodes, grid);
    std::vector<int> bulk = findBulkNodes(nodes);
    std::vector<int> fluidBnd = findFluidBndNodes(nodes);
    std::vector<int> solidBnd = findSolidBndNodes(nodes);

    const int N = grid.size();
    std::vector<int> neigh(static_cast<size_t>(N) * LT::nQ);
    std::vector<short> types(N);
    std::vector<int> pos(static_cast<size_t>(N) * LT::nD);
    for (int n = 0; n < N; ++n) {
        for (int q = 0; q < LT::nQ; ++q) neigh[static_cast<size_t>(n) * LT::nQ + q] = grid.neighbor(q, n);
        types[n] = static_cast<short>(nodes.getType(n));
        for (int d = 0; d < LT::nD; ++d) pos[static_cast<size_t>(n) * LT::nD + d] = grid.pos(n, d);
    }
    dump_raw(out + "/neigh.i32", neigh);
    dump_raw(out + "/types.i16", types);
    dump_raw(out + "/pos.i32", pos);
    dump_raw(out + "/bulk.i32", bulk);
    dump_raw(out + "/fluidbnd.i32", fluidBnd);
    dump_raw(out + "/solidbnd.i32", solidBnd);

    // Link classes of the std_case boundary (fluid boundary nodes) and of the
    // twophase boundary (all bulk nodes): per node [node, nBeta, nGamma, nDelta,
    // link list of nDirPairs entries].
    for (int which = 0; which < 2; ++which) {
        const std::vector<int>& list = which == 0 ? fluidBnd : bulk;
        HalfWayBounceBack<LT> bb(list, nodes, grid);
        std::vector<int> rec;
        for (int b = 0; b < bb.size(); ++b) {
            rec.push_back(bb.nodeNo(b));
            rec.push_back(bb.nBeta(b));
            rec.push_back(bb.nGamma(b));
            rec.push_back(bb.nDelta(b));
            for (int v : bb.beta(b)) rec.push_back(v);
            for (int v : bb.gamma(b)) rec.push_back(v);
            for (int v : bb.delta(b)) rec.push_back(v);
        }
        dump_raw(out + (which == 0 ? "/links_fluidbnd.i32" : "/links_bulk.i32"), rec);
    }
    std::printf("tables: N=%d Nf=%zu Nfb=%zu Nsb=%zu\n", N, bulk.size(), fluidBnd.size(), solidBnd.size());
    return 0;
}

// std_case loop, src/std_case/main.cpp:47-146 (VTU output replaced by a final dump).
int run_single(LBvtk<LT>& vtklb, const std::string& out, const std::map<std::string, double>& kv) {
    Grid<LT> grid(vtklb);
    Nodes<LT> nodes(vtklb, grid);
    BndMpi<LT> mpiBoundary(vtklb, nodes, grid);
    std::vector<int> bulkNodes = findBulkNodes(nodes);

    const int nSteps = static_cast<int>(get(kv, "steps", 1));
    const bool trt = get(kv, "trt", 0) != 0;
    const lbBase_t tau = get(kv, "tau", 1.0);
    const lbBase_t tauAnti = get(kv, "tau_anti", 1.0);
    std::vector<lbBase_t> bf = {get(kv, "fx", 0.0), get(kv, "fy", 0.0)};
    if (LT::nD == 3) bf.push_back(get(kv, "fz", 0.0));
    VectorField<LT> bodyForce(1, 1, bf);

    ScalarField rho(1, grid.size());
    vtklb.toAttribute("init_rho");
    for (int n = vtklb.beginNodeNo(); n < vtklb.endNodeNo(); ++n) rho(0, n) = vtklb.getScalarAttribute<lbBase_t>();
    VectorField<LT> vel(1, grid.size());
    for (auto nodeNo : bulkNodes)
        for (int d = 0; d < LT::nD; ++d) vel(0, d, nodeNo) = 0.0;

    HalfWayBounceBack<LT> bounceBackBnd(findFluidBndNodes(nodes), nodes, grid);

    LbField<LT> f(1, grid.size());
    LbField<LT> fTmp(1, grid.size());
    for (auto nodeNo : bulkNodes)
        for (int q = 0; q < LT::nQ; ++q) f(0, q, nodeNo) = LT::w[q] * rho(0, nodeNo);

    for (int i = 0; i < nSteps; i++) {
        for (auto nodeNo : bulkNodes) {
            const std::valarray<lbBase_t> fNode = f(0, nodeNo);
            const lbBase_t rhoNode = calcRho<LT>(fNode);
            const auto velNode = calcVel<LT>(fNode, rhoNode, bodyForce(0, 0));
            rho(0, nodeNo) = rhoNode;
            vel.set(0, nodeNo) = velNode;
            const lbBase_t u2 = LT::dot(velNode, velNode);
            const std::valarray<lbBase_t> cu = LT::cDotAll(velNode);
            const lbBase_t uF = LT::dot(velNode, bodyForce(0, 0));
            const std::valarray<lbBase_t> cF = LT::cDotAll(bodyForce(0, 0));
            if (!trt) {
                const std::valarray<lbBase_t> omegaBGK = calcOmegaBGK<LT>(fNode, tau, rhoNode, u2, cu);
                const std::valarray<lbBase_t> deltaOmegaF = calcDeltaOmegaF<LT>(tau, cu, uF, cF);
                fTmp.propagateTo(0, nodeNo, fNode + omegaBGK + deltaOmegaF, grid);
            } else {
                const std::valarray<lbBase_t> omegaTRT = calcOmegaBGKTRT<LT>(fNode, tau, tauAnti, rhoNode, u2, cu);
                const std::valarray<lbBase_t> deltaOmegaF = calcDeltaOmegaFTRT<LT>(tau, tauAnti, 1.0, cu, uF, cF);
                fTmp.propagateTo(0, nodeNo, fNode + omegaTRT + deltaOmegaF, grid);
            }
        }
        f.swapData(fTmp);
        mpiBoundary.communicateLbField(0, f, grid);
        bounceBackBnd.apply(f, grid);
    }
    f.writeToFile(out + "/f");
    rho.writeToFile(out + "/rho");
    vel.writeToFile(out + "/vel");
    std::printf("single: %d steps on %zu fluid nodes\n", nSteps, bulkNodes.size());
    return 0;
}

// twophase loop, src/twophase/main_TWOPHASE.cpp:79-393 with the mass source Q = 0
// (as in the reference, where Q is zero-initialised and never set) and the
// VTU/force.dat output replaced by a final dump.
int run_twophase(LBvtk<LT>& vtklb, const std::string& out, const std::map<std::string, double>& kv) {
    Grid<LT> grid(vtklb);
    Nodes<LT> nodes(vtklb, grid);
    BndMpi<LT> mpiBoundary(vtklb, nodes, grid);
    HalfWayBounceBack<LT> bbBnd(findBulkNodes(nodes), nodes, grid);
    std::vector<int> solidBnd = findSolidBndNodes(nodes);
    std::vector<int> bulkNodes = findBulkNodes(nodes);

    const int nSteps = static_cast<int>(get(kv, "steps", 1));
    std::vector<lbBase_t> bf = {get(kv, "fx", 0.0), get(kv, "fy", 0.0)};
    if (LT::nD == 3) bf.push_back(get(kv, "fz", 0.0));
    VectorField<LT> bodyForce(1, 1, bf);
    const bool fluxControl = kv.count("momx") != 0;
    const lbBase_t setMomX = get(kv, "momx", 0.0);
    const lbBase_t sigma = get(kv, "sigma", 0.0);
    const lbBase_t beta = get(kv, "beta", 0.0);
    const lbBase_t nu0Inv = 1.0 / (LT::c2 * (get(kv, "tau0", 1.0) - 0.5));
    const lbBase_t nu1Inv = 1.0 / (LT::c2 * (get(kv, "tau1", 1.0) - 0.5));

    ScalarField Q(2, grid.size());
    for (int n = 0; n < Q.size(); ++n) { Q(0, n) = 0.0; Q(1, n) = 0.0; }
    LbField<LT> f(2, grid.size());
    LbField<LT> fTmp(2, grid.size());
    ScalarField rho(2, grid.size());
    VectorField<LT> vel(1, grid.size());
    ScalarField cgField(1, grid.size());

    vtklb.toAttribute("rho0");
    for (int nodeNo = vtklb.beginNodeNo(); nodeNo < vtklb.endNodeNo(); ++nodeNo) {
        float val = vtklb.getScalar<float>();
        rho(0, nodeNo) = val;
        for (int d = 0; d < LT::nD; ++d) vel(0, d, nodeNo) = 0.0;
    }
    vtklb.toAttribute("rho1");
    for (int nodeNo = vtklb.beginNodeNo(); nodeNo < vtklb.endNodeNo(); ++nodeNo) {
        float val = vtklb.getScalar<float>();
        rho(1, nodeNo) = val;
    }
    vtklb.toAttribute("wettability");
    for (int nodeNo = vtklb.beginNodeNo(); nodeNo < vtklb.endNodeNo(); ++nodeNo) {
        float val = vtklb.getScalar<float>();
        if (nodes.isSolidBoundary(nodeNo)) {
            rho(0, nodeNo) = val;
            rho(1, nodeNo) = 1 - val;
        }
    }
    int numNodesGlobal = static_cast<int>(bulkNodes.size());
    initiateLbField(0, 0, 0, bulkNodes, rho, vel, f);
    initiateLbField(1, 1, 0, bulkNodes, rho, vel, f);

    std::vector<lbBase_t> forceLog;
    for (int i = 0; i < nSteps; i++) {
        for (auto nodeNo : bulkNodes) {
            lbBase_t rho0Node = rho(0, nodeNo) = calcRho<LT>(f(0, nodeNo));
            lbBase_t rho1Node = rho(1, nodeNo) = calcRho<LT>(f(1, nodeNo));
            cgField(0, nodeNo) = (rho0Node - rho1Node) / (rho0Node + rho1Node);
        }
        for (auto nodeNo : solidBnd) {
            const lbBase_t rho0Node = rho(0, nodeNo);
            const lbBase_t rho1Node = rho(1, nodeNo);
            cgField(0, nodeNo) = (rho0Node - rho1Node) / (rho0Node + rho1Node);
        }
        mpiBoundary.communciateScalarField(cgField);

        if (fluxControl) {
            lbBase_t meanfcX = 0.0;
            for (auto nodeNo : bulkNodes) {
                std::valarray<lbBase_t> fTot = f(0, nodeNo) + f(1, nodeNo);
                std::valarray<lbBase_t> sumfc = LT::qSumC(fTot);
                meanfcX += sumfc[0];
            }
            lbBase_t meanfcXGlobal = meanfcX;
            meanfcXGlobal /= numNodesGlobal;
            bodyForce(0, 0, 0) = 2 * (setMomX - meanfcXGlobal);
        }
        forceLog.push_back(bodyForce(0, 0, 0));

        for (auto nodeNo : bulkNodes) {
            std::valarray<lbBase_t> fTot = f(0, nodeNo) + f(1, nodeNo);
            lbBase_t rho0Node = rho(0, nodeNo);
            lbBase_t rho1Node = rho(1, nodeNo);
            lbBase_t rhoNode = rho0Node + rho1Node;
            std::valarray<lbBase_t> forceNode = bodyForce(0, 0);
            std::valarray<lbBase_t> velNode = calcVel<LT>(fTot, rhoNode, forceNode);
            vel.set(0, nodeNo) = velNode;
            lbBase_t q0Node = Q(0, nodeNo);
            lbBase_t q1Node = Q(1, nodeNo);
            rho(0, nodeNo) = rho0Node += 0.5 * q0Node;
            rho(1, nodeNo) = rho1Node += 0.5 * q1Node;
            lbBase_t tau = LT::c2Inv * rhoNode / (rho0Node * nu0Inv + rho1Node * nu1Inv) + 0.5;
            lbBase_t uu = LT::dot(velNode, velNode);
            std::valarray<lbBase_t> cu = LT::cDotAll(velNode);
            std::valarray<lbBase_t> omegaBGK = calcOmegaBGK<LT>(fTot, tau, rhoNode, uu, cu);
            lbBase_t uF = LT::dot(velNode, forceNode);
            std::valarray<lbBase_t> cF = LT::cDotAll(forceNode);
            std::valarray<lbBase_t> deltaOmegaF = calcDeltaOmegaF<LT>(tau, cu, uF, cF);
            std::valarray<lbBase_t> deltaOmegaQ0 = calcDeltaOmegaQ<LT>(tau, cu, uu, q0Node);
            std::valarray<lbBase_t> deltaOmegaQ1 = calcDeltaOmegaQ<LT>(tau, cu, uu, q1Node);
            std::valarray<lbBase_t> colorGradNode = grad(cgField, 0, nodeNo, grid);
            lbBase_t CGNorm = vecNorm<LT>(colorGradNode);
            colorGradNode *= 1.0 / (CGNorm + (CGNorm < lbBaseEps));
            std::valarray<lbBase_t> cCGNorm = LT::cDotAll(colorGradNode);
            std::valarray<lbBase_t> deltaOmegaST = calcDeltaOmegaST<LT>(tau, sigma, CGNorm, cCGNorm);
            std::valarray<lbBase_t> deltaOmegaRC = calcDeltaOmegaRC<LT>(beta, rho0Node, rho1Node, rhoNode, cCGNorm);
            lbBase_t c0 = (rho0Node / rhoNode);
            lbBase_t c1 = (rho1Node / rhoNode);
            for (int q = 0; q < LT::nQ; ++q) {
                fTmp(0, q, grid.neighbor(q, nodeNo)) = c0 * (fTot[q] + omegaBGK[q] + deltaOmegaF[q] + deltaOmegaST[q]) + deltaOmegaRC[q] + deltaOmegaQ0[q];
                fTmp(1, q, grid.neighbor(q, nodeNo)) = c1 * (fTot[q] + omegaBGK[q] + deltaOmegaF[q] + deltaOmegaST[q]) - deltaOmegaRC[q] + deltaOmegaQ1[q];
            }
        }
        f.swapData(fTmp);
        mpiBoundary.communicateLbField(0, f, grid);
        mpiBoundary.communicateLbField(1, f, grid);
        bbBnd.apply(0, f, grid);
        bbBnd.apply(1, f, grid);
    }
    f.writeToFile(out + "/f");
    rho.writeToFile(out + "/rho");
    vel.writeToFile(out + "/vel");
    cgField.writeToFile(out + "/cg");
    dump_raw(out + "/force.f64", forceLog);
    std::printf("twophase: %d steps on %zu fluid nodes\n", nSteps, bulkNodes.size());
    return 0;
}

}  // namespace

// The output step of the reference mains (src/std_case/main.cpp:101-104, 151;
// src/twophase/main_TWOPHASE.cpp:217-224), on fields read from <out>/fields.bin.
int run_vtu(LBvtk<LT>& vtklb, const std::string& out, const std::map<std::string, double>& kv) {
    Grid<LT> grid(vtklb);
    Nodes<LT> nodes(vtklb, grid);
    BndMpi<LT> mpiBoundary(vtklb, nodes, grid);
    std::vector<int> bulkNodes = findBulkNodes(nodes);
    const int nF = static_cast<int>(get(kv, "nfields", 1));
    ScalarField rho(nF, grid.size());
    VectorField<LT> vel(nF, grid.size());
    {
        std::ifstream ifs(out + "/fields.bin", std::ios::binary);
        ifs.read(reinterpret_cast<char*>(&rho(0, 0)), static_cast<std::streamsize>(sizeof(double)) * nF * grid.size());
        ifs.read(reinterpret_cast<char*>(&vel(0, 0, 0)),
                 static_cast<std::streamsize>(sizeof(double)) * nF * LT::nD * grid.size());
        if (!ifs) {
            std::fprintf(stderr, "cannot read %s/fields.bin\n", out.c_str());
            return 1;
        }
    }
    Output<LT> o64(grid, bulkNodes, out + "/f64", 0, 1);
    o64.add_file("lb_run");
    o64.add_scalar_variables({"rho"}, {rho});
    o64.add_vector_variables({"vel"}, {vel});
    o64.add_file("second");
    o64.add_scalar_variables({"rho"}, {rho});
    o64.write(0);
    for (int n = 0; n < grid.size(); ++n)
        for (int i = 0; i < nF; ++i) rho(i, n) *= 2.0;
    o64.write(1000);

    Output<LT, float> o32(grid, bulkNodes, out + "/f32", 0, 1);
    o32.add_file("lb_f32");
    o32.add_vector_variables({"vel"}, {vel});
    o32.add_scalar_variables({"rho"}, {rho});
    o32.write(0.5);

    Output<LT, double, VTK::ASCII> oa(grid, bulkNodes, out + "/ascii", 0, 1);
    oa.add_file("lb_ascii");
    oa.add_scalar_variables({"rho"}, {rho});
    oa.add_vector_variables({"vel"}, {vel});
    oa.write(2);

    auto geo = nodes.geo(grid, vtklb);
    Output<LT, int> geoout(grid.pos(), out + "/geo", 0, 1, "geo", geo);
    geoout.write();
    std::printf("vtu: N=%d Nb=%zu nF=%d\n", grid.size(), bulkNodes.size(), nF);
    return 0;
}

int main(int argc, char** argv) {
    if (argc < 4) {
        std::fprintf(stderr, "usage: %s tables|single|twophase|vtu <file.vtklb> <outdir> [key=value ...]\n", argv[0]);
        return 2;
    }
    MPI_Init(NULL, NULL);
    std::string mode(argv[1]);
    LBvtk<LT> vtklb(argv[2]);
    std::string out(argv[3]);
    auto kv = parse_kv(argc, argv, 4);
    int rc = 2;
    if (mode == "tables") rc = run_tables(vtklb, out);
    else if (mode == "single") rc = run_single(vtklb, out, kv);
    else if (mode == "twophase") rc = run_twophase(vtklb, out, kv);
    else if (mode == "vtu") rc = run_vtu(vtklb, out, kv);
    else std::fprintf(stderr, "unknown mode %s\n", mode.c_str());
    MPI_Finalize();
    return rc;
}
