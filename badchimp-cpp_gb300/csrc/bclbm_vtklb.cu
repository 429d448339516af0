// Reader of the reference's .vtklb geometry files (the files PythonScripts/vtklb.py
// writes and src/lbsolver/LBvtk.h reads), producing the arrays that Grid and
// Nodes hold after reading them (LBgrid.h:127-148, LBnodes.h:112-209), for one
// rank.  Host code.  The file is read into memory and parsed in one pass with
// 64-bit offsets, so files past 2 GiB read (LBvtk.h keeps positions in int).
//
// Sections, in file order (LBvtk.h:221-662):
//   header line, title line, ASCII | BINARY (both text, as LBvtk reads them)
//   DATASET UNSTRUCTURED_LB_GRID
//   [NUM_DIMENSIONS nd]  GLOBAL_DIMENSIONS d0 .. d(nd-1)  [USE_ZERO_GHOST_NODE]
//   POINTS n type          then nd integers per point
//   LATTICE nq type        then nq basis vectors (file basis order)
//   NEIGHBORS type         then nq neighbour numbers per point, file basis order
//   PARALLEL_COMPUTING r   then PROCESSOR blocks (other ranks; none at one rank)
//   POINT_DATA n           then SCALARS name type + n values, repeated
//   [POINT_DATA_SUBSET     SCALARS size name type + size lines, repeated]
// With USE_ZERO_GHOST_NODE point k is node k + 1 and node 0 is the ghost.
#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

#include <cerrno>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <map>
#include <new>
#include <string>
#include <vector>

#include "bclbm.h"
#include "bclbm_device.cuh"
#include "bclbm_lattice.h"

namespace {

struct Cursor {
    const char* p;
    const char* end;
    bool ok = true;

    void skip_space() {
        while (p < end && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r')) ++p;
    }
    std::string word() {
        skip_space();
        const char* b = p;
        while (p < end && !(*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r')) ++p;
        if (b == p) ok = false;
        return std::string(b, p);
    }
    void rest_of_line() {
        while (p < end && *p != '\n') ++p;
        if (p < end) ++p;
    }
    long long integer() {
        skip_space();
        char* e = nullptr;
        const long long v = std::strtoll(p, &e, 10);
        if (e == p) ok = false;
        p = e;
        return v;
    }
    double real() {
        skip_space();
        char* e = nullptr;
        const double v = std::strtod(p, &e);
        if (e == p) ok = false;
        p = e;
        return v;
    }
    // the next word without consuming it
    std::string peek() {
        const char* save = p;
        std::string w = word();
        p = save;
        ok = true;
        return w;
    }
};

template <int Q>
int basis_index(const int* c, int nd) {
    using L = bclbm::Lat<Q>;
    for (int q = 0; q < Q; ++q) {
        const int v[3] = {L::cx(q), L::cy(q), L::cz(q)};
        bool same = true;
        for (int d = 0; d < nd; ++d) same &= v[d] == c[d];
        if (same) return q;
    }
    return -1;
}

int parse(Cursor& c, int Q, bclbm_lattice* L, std::string& err) {
    c.rest_of_line();  // header
    c.rest_of_line();  // title
    // ASCII or BINARY: LBvtk reads both as text (its ascii_ flag is set and never
    // used, LBvtk.h:277-289); anything else is an error there
    const std::string kind = c.word();
    if (kind != "ASCII" && kind != "BINARY") {
        err = "files data type must be ASCII or BINARY";
        return BCLBM_ERR_INVALID;
    }
    c.rest_of_line();
    if (c.word() != "DATASET" || c.word() != "UNSTRUCTURED_LB_GRID") {
        err = "expected DATASET UNSTRUCTURED_LB_GRID";
        return BCLBM_ERR_INVALID;
    }
    c.rest_of_line();
    int nd = 3;
    if (c.peek() == "NUM_DIMENSIONS") {
        c.word();
        nd = static_cast<int>(c.integer());
        c.rest_of_line();
    }
    if (nd != (Q == 9 ? 2 : 3)) {
        err = "NUM_DIMENSIONS does not match the lattice";
        return BCLBM_ERR_INVALID;
    }
    if (c.word() != "GLOBAL_DIMENSIONS") {
        err = "expected GLOBAL_DIMENSIONS";
        return BCLBM_ERR_INVALID;
    }
    for (int d = 0; d < nd; ++d) L->global_dims.push_back(static_cast<int32_t>(c.integer()));
    c.rest_of_line();
    bool zero_ghost = false;
    if (c.peek() == "USE_ZERO_GHOST_NODE") {
        zero_ghost = true;
        c.word();
        c.rest_of_line();
    }
    if (c.word() != "POINTS") {
        err = "expected POINTS";
        return BCLBM_ERR_INVALID;
    }
    const long long np = c.integer();
    c.rest_of_line();
    if (np < 1 || np + 1 > INT32_MAX) {
        err = "bad number of points";
        return BCLBM_ERR_INVALID;
    }
    const int64_t begin = zero_ghost ? 1 : 0, N = zero_ghost ? np + 1 : np;
    L->q = Q;
    L->nd = nd;
    L->pos.assign(static_cast<size_t>(N) * nd, -1);
    for (int64_t n = begin; n < N; ++n)
        for (int d = 0; d < nd; ++d) L->pos[static_cast<size_t>(n) * nd + d] = static_cast<int32_t>(c.integer());
    c.rest_of_line();
    if (c.word() != "LATTICE") {
        err = "expected LATTICE";
        return BCLBM_ERR_INVALID;
    }
    if (c.integer() != Q) {
        err = "LATTICE has another number of basis vectors";
        return BCLBM_ERR_INVALID;
    }
    c.rest_of_line();
    std::vector<int> f2p(Q, -1);
    std::vector<bool> seen(Q, false);
    for (int q = 0; q < Q; ++q) {
        int v[3] = {0, 0, 0};
        for (int d = 0; d < nd; ++d) v[d] = static_cast<int>(c.integer());
        f2p[q] = Q == 9 ? basis_index<9>(v, nd) : basis_index<19>(v, nd);
        if (f2p[q] < 0 || seen[f2p[q]]) {
            err = "LATTICE basis is not the lattice's";
            return BCLBM_ERR_INVALID;
        }
        seen[f2p[q]] = true;
    }
    c.rest_of_line();
    if (c.word() != "NEIGHBORS") {
        err = "expected NEIGHBORS";
        return BCLBM_ERR_INVALID;
    }
    c.rest_of_line();
    L->neigh.assign(static_cast<size_t>(N) * Q, 0);
    for (int64_t n = begin; n < N; ++n)
        for (int q = 0; q < Q; ++q) {
            const long long y = c.integer();
            if (y < 0 || y >= N) c.ok = false;
            L->neigh[static_cast<size_t>(n) * Q + f2p[q]] = static_cast<int32_t>(y);
        }
    if (!c.ok) {
        err = "bad NEIGHBORS entry";
        return BCLBM_ERR_TABLE;
    }
    c.rest_of_line();
    if (c.word() != "PARALLEL_COMPUTING") {
        err = "expected PARALLEL_COMPUTING";
        return BCLBM_ERR_INVALID;
    }
    c.rest_of_line();
    if (c.peek() == "PROCESSOR") {
        err = "the file shares nodes with other ranks (one rank is read)";
        return BCLBM_ERR_UNSUPPORTED;
    }
    if (c.word() != "POINT_DATA") {
        err = "expected POINT_DATA";
        return BCLBM_ERR_INVALID;
    }
    if (c.integer() != np) {
        err = "POINT_DATA size differs from POINTS";
        return BCLBM_ERR_INVALID;
    }
    c.rest_of_line();
    while (c.ok && c.peek() == "SCALARS") {
        c.word();
        const std::string name = c.word();
        c.rest_of_line();
        std::vector<double> v(static_cast<size_t>(N), 0.0);
        for (int64_t n = begin; n < N; ++n) v[static_cast<size_t>(n)] = c.real();
        c.rest_of_line();
        L->attributes[name] = std::move(v);
    }
    if (!c.ok) {
        err = "bad SCALARS block";
        return BCLBM_ERR_INVALID;
    }
    // POINT_DATA_SUBSET blocks are not needed by the lattice and are left unread
    // node types (Nodes::setupNodeType): the nodetype attribute marks solids (0)
    // and fluids (other values); solids with a fluid neighbour are 1, else 0;
    // fluids with a solid neighbour (node 0 counts as solid) are 2, else 3
    auto it = L->attributes.find("nodetype");
    if (it == L->attributes.end()) {
        err = "no nodetype attribute";
        return BCLBM_ERR_INVALID;
    }
    const std::vector<double>& nt = it->second;
    std::vector<char> fluid(static_cast<size_t>(N), 0);
    for (int64_t n = 1; n < N; ++n) fluid[static_cast<size_t>(n)] = nt[static_cast<size_t>(n)] != 0.0;
    L->types.assign(static_cast<size_t>(N), 0);
    L->types[0] = -1;
    int64_t nf = 0;
    for (int64_t n = 1; n < N; ++n) {
        bool any_fluid = false, any_solid = false;
        for (int q = 0; q < Q; ++q) {
            const bool f = fluid[static_cast<size_t>(L->neigh[static_cast<size_t>(n) * Q + q])] != 0;
            any_fluid |= f;
            any_solid |= !f;
        }
        if (fluid[static_cast<size_t>(n)]) {
            L->types[static_cast<size_t>(n)] = any_solid ? 2 : 3;
            ++nf;
        } else {
            L->types[static_cast<size_t>(n)] = any_fluid ? 1 : 0;
        }
    }
    L->nf = nf;
    L->ns = N - 1 - nf;
    return BCLBM_OK;
}

}  // namespace

extern "C" {

int bclbm_lattice_read_vtklb(const char* path, int32_t lattice_q, bclbm_lattice** out) {
    if (!out || !path || (lattice_q != 9 && lattice_q != 19)) return BCLBM_ERR_INVALID;
    *out = nullptr;
    // the whole file in memory with a terminating NUL (the number parsers stop there)
    const int fd = open(path, O_RDONLY);
    if (fd < 0) return BCLBM_ERR_INVALID;
    struct stat sb;
    if (fstat(fd, &sb) != 0 || sb.st_size <= 0) {
        close(fd);
        return BCLBM_ERR_INVALID;
    }
    const size_t size = static_cast<size_t>(sb.st_size);
    std::vector<char> buf;
    try {
        buf.resize(size + 1, '\0');
    } catch (const std::bad_alloc&) {
        close(fd);
        return BCLBM_ERR_NOMEM;
    }
    size_t got = 0;
    while (got < size) {
        const ssize_t r = read(fd, buf.data() + got, size - got);
        if (r <= 0) break;
        got += static_cast<size_t>(r);
    }
    close(fd);
    if (got != size) return BCLBM_ERR_INVALID;
    bclbm_lattice* L = new (std::nothrow) bclbm_lattice();
    int rc = BCLBM_ERR_NOMEM;
    if (L) {
        Cursor c{buf.data(), buf.data() + size};
        std::string err;
        try {
            rc = parse(c, lattice_q, L, err);
        } catch (const std::bad_alloc&) {
            rc = BCLBM_ERR_NOMEM;
        }
        L->error = err;
    }
    if (rc != BCLBM_OK) {
        delete L;
        return rc;
    }
    *out = L;
    return BCLBM_OK;
}

int bclbm_lattice_attribute(const bclbm_lattice* L, const char* name, double* out) {
    if (!L || !name) return BCLBM_ERR_INVALID;
    auto it = L->attributes.find(name);
    if (it == L->attributes.end()) return BCLBM_ERR_INVALID;
    if (out) std::memcpy(out, it->second.data(), it->second.size() * sizeof(double));
    return BCLBM_OK;
}

}  // extern "C"
