// A compiled C++ caller of include/bclbm.h and nothing else (no reference
// headers, no Python): the shape of the reference's std_case main loop
// (src/std_case/main.cpp:109-157) with the node loops replaced by bclbm_step
// and the output step by bclbm_download_macros.
//
//   abi_caller <dir> <flags>
//
// <dir>/meta.txt   "q n_nodes n_bulk nsteps write_every tau fx fy fz"
// <dir>/neigh.i32  [N*Q]  Grid neighbour table, reference numbering
// <dir>/types.i16  [N]    Nodes types
// <dir>/bulk.i32   [n_bulk]
// <dir>/f.f64      [N*Q]  LbField data at the start
// writes <dir>/out_<flags>_{f,rho,vel}.f64 (reference layout) and prints one
// line "ok <steps> <sum rho>" on success, "fail <where> <status> <text>" else.
#include <bclbm.h>

#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

namespace {

template <class T>
bool read_all(const std::string& path, std::vector<T>& v, size_t n) {
    v.resize(n);
    FILE* fp = std::fopen(path.c_str(), "rb");
    if (!fp) return false;
    const size_t got = std::fread(v.data(), sizeof(T), n, fp);
    std::fclose(fp);
    return got == n;
}

template <class T>
bool write_all(const std::string& path, const std::vector<T>& v) {
    FILE* fp = std::fopen(path.c_str(), "wb");
    if (!fp) return false;
    const size_t put = std::fwrite(v.data(), sizeof(T), v.size(), fp);
    std::fclose(fp);
    return put == v.size();
}

int fail(const char* where, int status, const bclbm_handle* h) {
    std::printf("fail %s %d %s %s\n", where, status, bclbm_error(status), h ? bclbm_last_error(h) : "");
    return 1;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc != 3) {
        std::fprintf(stderr, "usage: abi_caller <dir> <flags>\n");
        return 2;
    }
    const std::string dir = argv[1];
    const unsigned flags = static_cast<unsigned>(std::strtoul(argv[2], nullptr, 10));
    int q = 0, n_nodes = 0, n_bulk = 0, nsteps = 0, write_every = 0;
    double tau = 0, fx = 0, fy = 0, fz = 0;
    FILE* mf = std::fopen((dir + "/meta.txt").c_str(), "r");
    if (!mf || std::fscanf(mf, "%d %d %d %d %d %lf %lf %lf %lf", &q, &n_nodes, &n_bulk, &nsteps, &write_every, &tau,
                           &fx, &fy, &fz) != 9) {
        std::printf("fail meta 0\n");
        return 1;
    }
    std::fclose(mf);
    const int nd = q == 9 ? 2 : 3;
    std::vector<int32_t> neigh, bulk;
    std::vector<int16_t> types;
    std::vector<double> f;
    if (!read_all(dir + "/neigh.i32", neigh, static_cast<size_t>(n_nodes) * q) ||
        !read_all(dir + "/types.i16", types, n_nodes) || !read_all(dir + "/bulk.i32", bulk, n_bulk) ||
        !read_all(dir + "/f.f64", f, static_cast<size_t>(n_nodes) * q)) {
        std::printf("fail read 0\n");
        return 1;
    }

    // the descriptor from the arrays the reference's objects hold after set-up
    bclbm_desc d = {};
    d.lattice_q = q;
    d.n_nodes = n_nodes;
    d.neigh = neigh.data();
    d.types = types.data();
    d.n_bulk = n_bulk;
    d.bulk = bulk.data();
    d.collision = BCLBM_BGK;
    d.precision = BCLBM_F64;
    d.flags = flags;
    d.tau[0] = d.tau[1] = tau;
    d.force[0] = fx;
    d.force[1] = fy;
    d.force[2] = fz;
    d.f_init = f.data();

    bclbm_handle* h = nullptr;
    int rc = bclbm_create(&d, &h);
    if (rc != BCLBM_OK) return fail("create", rc, nullptr);

    // ScalarField rho(1, N), VectorField vel(1, N) of the reference loop
    std::vector<double> rho(n_nodes, 0.0), vel(static_cast<size_t>(n_nodes) * nd, 0.0);
    for (int i = 0; i < nsteps; ++i) {
        rc = bclbm_step(h, 1);  // the node loop, swapData, communicate, bounce-back
        if (rc != BCLBM_OK) return fail("step", rc, h);
        if (write_every > 0 && (i + 1) % write_every == 0) {  // an output step
            rc = bclbm_download_macros(h, rho.data(), vel.data(), nullptr);
            if (rc != BCLBM_OK) return fail("download_macros", rc, h);
        }
    }
    rc = bclbm_download_macros(h, rho.data(), vel.data(), nullptr);
    if (rc != BCLBM_OK) return fail("download_macros", rc, h);
    std::vector<double> fout(f.size(), 0.0);
    rc = bclbm_download_f(h, fout.data());
    if (rc != BCLBM_OK) return fail("download_f", rc, h);
    bclbm_stats st;
    rc = bclbm_reduce(h, &st);
    if (rc != BCLBM_OK) return fail("reduce", rc, h);
    bclbm_destroy(h);

    const std::string tag = dir + "/out_" + std::to_string(flags) + "_";
    if (!write_all(tag + "f.f64", fout) || !write_all(tag + "rho.f64", rho) || !write_all(tag + "vel.f64", vel)) {
        std::printf("fail write 0\n");
        return 1;
    }
    std::printf("ok %lld %.17g\n", static_cast<long long>(st.steps_done), st.mass[0]);
    return 0;
}
