// VTU/PVTU writer of the reference's output step: Output<LT, T, FMT, voxel>
// (src/io/Output.h:26-177) over VTK::Output (src/io/VTK.h:1421-1550).  Host code.
//
// The files are byte-identical to the reference's for the same node positions,
// variables and write sequence (the PVTU "Created" comment carries the local
// time, as there):
//   <dir>/<name>_<nwrite:7>.pvtu           VTK.h:1207-1356, the MPI piece path
//   <dir>/vtu/<rank:4>_<name>_<nwrite:7>.vtu VTK.h:1081-1200
// Mesh (VTK.h:395-555): one voxel (3-D) or pixel (2-D) per written node, its
// corners numbered in order of first appearance; points are Float32 corner
// coordinates shifted by -0.5.  Binary data is "appended" raw with a 32-bit byte
// count before each array.  Where the appended data passes 2^31 bytes (the
// reference's int offsets overflow there) the file is written with
// header_type="UInt64" and 64-bit counts instead, which VTK readers accept
// (BCLBM_VTU_BINARY64 asks for that form at any size).
//
// What differs is the work per write: the mesh and its appended blocks are
// built once at creation; each write gathers every variable into one buffer
// with all host cores and writes each array with one call (the reference
// writes non-contiguous variables one value at a time).  bclbm_output_write_async
// takes the values at the call and writes on a background thread, so a caller
// that downloads the moments and returns to stepping overlaps the file write
// with the GPU's steps.
#include <sys/stat.h>
#include <sys/types.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <system_error>
#include <thread>
#include <vector>

#include "bclbm.h"
#include "bclbm_host.h"
#include "bclbm_trace.h"

namespace {

using bclbm::host::parallel_for;

constexpr int64_t kInt32Max = 2147483647;

int value_size(int32_t t) { return t == BCLBM_VTU_FLOAT64 ? 8 : 4; }

const char* type_name(int32_t t) {
    return t == BCLBM_VTU_FLOAT64 ? "Float64" : (t == BCLBM_VTU_FLOAT32 ? "Float32" : "Int32");
}

// the ostream default formatting of the reference's ASCII path (%g, 6 digits)
void put_ascii(std::string& s, double v, bool integer) {
    char b[40];
    int n;
    if (integer) n = std::snprintf(b, sizeof b, "%d ", static_cast<int>(v));
    else if (std::fabs(v) < 1e-20) n = std::snprintf(b, sizeof b, "0 ");  // Data::min_value_ (VTK.h:646)
    else n = std::snprintf(b, sizeof b, "%g ", v);
    s.append(b, static_cast<size_t>(n));
}

// One array of the file: what it reads and how (VTK::Data, VTK.h:634-777)
struct Var {
    std::string name;
    int32_t out_type = BCLBM_VTU_FLOAT64;
    const void* src = nullptr;
    int32_t src_type = BCLBM_VTU_FLOAT64;
    bool field = false;         // Output::add_variable__ indexing (Output.h:156-173)
    int32_t n_fields = 1, field_no = 0;
    int32_t dim = 1;            // components read per cell (1, 2 or 3)
    int32_t dim_out = 1;        // written per cell: 2-D vectors get a zero third component
    int64_t length = 0;         // values written
    int64_t offset = -1;        // appended-data offset (binary)

    double at(int64_t j, const int32_t* nodes) const {
        int64_t s;
        if (field) {
            const int64_t c = j / dim_out, d = j % dim_out;
            if (d >= dim) return 0.0;
            s = (static_cast<int64_t>(nodes[c]) * n_fields + field_no) * dim + d;
        } else if (dim == 2) {
            const int64_t c = j / 3, d = j % 3;
            if (d >= 2) return 0.0;
            s = c * 2 + d;
        } else {
            s = j;
        }
        switch (src_type) {
            case BCLBM_VTU_FLOAT64: return static_cast<const double*>(src)[s];
            case BCLBM_VTU_FLOAT32: return static_cast<const float*>(src)[s];
            default: return static_cast<const int32_t*>(src)[s];
        }
    }
    // the same element without the double round trip (int32 to int32, float to float)
    template <class T>
    T value(int64_t j, const int32_t* nodes) const {
        if (!field && dim != 2 && src_type == out_type) return static_cast<const T*>(src)[j];
        return static_cast<T>(at(j, nodes));
    }
};

struct File {
    std::string name;
    std::vector<Var> vars;
    int nwrite = 0;
    int64_t offset = 0;  // VTU_file::offset_: the end of the appended data
};

struct Block {  // one appended array: count + values, or its ASCII text
    std::vector<char> bytes;
};

}  // namespace

struct bclbm_output {
    int32_t nd = 3, value_type = BCLBM_VTU_FLOAT64, format = BCLBM_VTU_BINARY, rank = 0, nproc = 1;
    int64_t n_cells = 0, n_points = 0;
    std::vector<int32_t> nodes;  // node numbers of the cells (field indexing), may be empty
    std::string dir, vtu_dir;    // "<dir>/" and "<dir>/vtu/"
    // mesh arrays (VTK::Grid, VTK.h:854-920)
    std::vector<float> points;
    std::vector<int32_t> conn, offsets, types;
    int64_t grid_bytes = 0;  // Grid::offset(): the appended bytes of the four mesh arrays
    std::vector<File> files;
    // the mesh's appended blocks (or ASCII texts), built on first write
    std::vector<Block> grid_blocks;
    bool wide = false;        // header_type UInt64
    bool force_wide = false;  // BCLBM_VTU_BINARY64: UInt64 counts whatever the size
    std::thread writer;
    int async_status = BCLBM_OK;
    std::string error;
    std::mutex mu;
};

namespace {

void make_dir(const std::string& d) {
    struct stat st;
    if (stat(d.c_str(), &st) == -1) mkdir(d.c_str(), 0700);
}

// VTK::Mesh::set_size/get_stride/calc_points_and_conn (VTK.h:464-553)
int build_mesh(bclbm_output* o, const int32_t* pos) {
    const int D = o->nd;
    const int nc = D == 3 ? 8 : 4;
    static const int corner3[8][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {1, 1, 0},
                                      {0, 0, 1}, {1, 0, 1}, {0, 1, 1}, {1, 1, 1}};
    static const int corner2[4][2] = {{0, 0}, {1, 0}, {0, 1}, {1, 1}};
    int64_t mn[3] = {999999, 999999, 999999}, mx[3] = {-1, -1, -1};
    const int64_t N = o->n_cells;
    for (int64_t n = 0; n < N; ++n)
        for (int i = 0; i < D; ++i) {
            const int64_t v = pos[n * D + i];
            if (v > mx[i]) mx[i] = v;
            if (v < mn[i]) mn[i] = v;
        }
    int64_t stride[3] = {1, 1, 1};
    for (int i = 1; i < D; ++i) stride[i] = stride[i - 1] * ((mx[i - 1] - mn[i - 1] + 1) + 1);
    auto corner = [&](int64_t n, int p, int i) -> int64_t {
        return pos[n * D + i] + (D == 3 ? corner3[p][i] : corner2[p][i]);
    };
    auto corner_index = [&](int64_t n, int p) -> int64_t {
        int64_t idx = 0;
        for (int i = 0; i < D; ++i) idx += corner(n, p, i) * stride[i];
        return idx;
    };
    // the range of the corner indices (all cores), then the numbering of the
    // corners in order of first appearance (one pass, in cell order)
    int64_t imin = INT64_MAX, imax = INT64_MIN;
    std::mutex m;
    parallel_for(static_cast<size_t>(N), [&](size_t b, size_t e) {
        int64_t lo = INT64_MAX, hi = INT64_MIN;
        for (size_t n = b; n < e; ++n)
            for (int p = 0; p < nc; ++p) {
                const int64_t idx = corner_index(static_cast<int64_t>(n), p);
                lo = idx < lo ? idx : lo;
                hi = idx > hi ? idx : hi;
            }
        std::lock_guard<std::mutex> g(m);
        imin = lo < imin ? lo : imin;
        imax = hi > imax ? hi : imax;
    });
    if (imax - imin + 1 > (int64_t(1) << 32)) return BCLBM_ERR_UNSUPPORTED;
    std::vector<int32_t> number(static_cast<size_t>(imax - imin + 1), -1);
    o->conn.resize(static_cast<size_t>(N * nc));
    o->points.clear();
    o->points.reserve(static_cast<size_t>(N) * 3 * (D == 3 ? 2 : 1) + 64);
    int64_t npts = 0;
    for (int64_t n = 0; n < N; ++n)
        for (int p = 0; p < nc; ++p) {
            int32_t& num = number[static_cast<size_t>(corner_index(n, p) - imin)];
            if (num < 0) {
                if (npts >= kInt32Max) return BCLBM_ERR_UNSUPPORTED;
                num = static_cast<int32_t>(npts++);
                for (int d = 0; d < 3; ++d)  // Float32 corner minus 0.5, padded to three coordinates
                    o->points.push_back(
                        d < D ? static_cast<float>(static_cast<double>(static_cast<float>(corner(n, p, d))) - 0.5)
                              : 0.0f);
            }
            o->conn[static_cast<size_t>(n * nc + p)] = num;
        }
    o->n_points = npts;
    o->offsets.resize(static_cast<size_t>(N));
    o->types.assign(static_cast<size_t>(N), D == 3 ? 11 : 8);
    for (int64_t n = 0; n < N; ++n) o->offsets[static_cast<size_t>(n)] = static_cast<int32_t>((n + 1) * nc);
    return BCLBM_OK;
}

std::string data_array(const std::string& name, const char* type, int dim, int format, int64_t offset) {
    // DataArray tags (VTK.h:563-625): Name, type, NumberOfComponents, format, offset
    std::string s = "<DataArray Name=\"" + name + "\" type=\"" + type + "\" NumberOfComponents=\"" +
                    std::to_string(dim) + "\" format=\"" + (format == BCLBM_VTU_BINARY ? "appended" : "ascii") + "\" ";
    if (format == BCLBM_VTU_BINARY) s += "offset=\"" + std::to_string(offset) + "\" ";
    s += "> ";
    return s;
}

template <class T>
void put_block(std::vector<char>& out, size_t at, const T* v, int64_t n, bool wide) {
    const uint64_t nb = static_cast<uint64_t>(n) * sizeof(T);
    if (wide) std::memcpy(out.data() + at, &nb, 8);
    else {
        const uint32_t nb32 = static_cast<uint32_t>(nb);
        std::memcpy(out.data() + at, &nb32, 4);
    }
    std::memcpy(out.data() + at + (wide ? 8 : 4), v, nb);
}

template <class T>
std::vector<char> binary_block(const std::vector<T>& v, bool wide) {
    std::vector<char> b((wide ? 8 : 4) + v.size() * sizeof(T));
    put_block(b, 0, v.data(), static_cast<int64_t>(v.size()), wide);
    return b;
}

template <class T>
std::vector<char> ascii_block(const std::vector<T>& v, bool integer) {
    std::string s;
    s.reserve(v.size() * 8);
    for (const T& x : v) put_ascii(s, static_cast<double>(x), integer);
    return std::vector<char>(s.begin(), s.end());
}

void build_grid_blocks(bclbm_output* o) {
    o->grid_blocks.clear();
    if (o->format == BCLBM_VTU_BINARY) {
        o->grid_blocks.push_back({binary_block(o->points, o->wide)});
        o->grid_blocks.push_back({binary_block(o->conn, o->wide)});
        o->grid_blocks.push_back({binary_block(o->offsets, o->wide)});
        o->grid_blocks.push_back({binary_block(o->types, o->wide)});
    } else {
        o->grid_blocks.push_back({ascii_block(o->points, false)});
        o->grid_blocks.push_back({ascii_block(o->conn, true)});
        o->grid_blocks.push_back({ascii_block(o->offsets, true)});
        o->grid_blocks.push_back({ascii_block(o->types, true)});
    }
}

// the appended offsets of the mesh arrays and of every file's variables
// (Grid::update_offset, Outfile::update_offset: VTK.h:885-893, 1391-1394)
void layout(bclbm_output* o) {
    const int64_t hdr = o->wide ? 8 : 4;
    o->grid_bytes = 0;
    if (o->format != BCLBM_VTU_BINARY) return;
    const int64_t nc = o->nd == 3 ? 8 : 4;
    o->grid_bytes = (o->n_points * 3 * 4 + hdr) + (o->n_cells * nc * 4 + hdr) + 2 * (o->n_cells * 4 + hdr);
    for (File& f : o->files) {
        int64_t off = o->grid_bytes;
        for (Var& v : f.vars) {
            v.offset = off;
            off += v.length * value_size(v.out_type) + hdr;
        }
        f.offset = off;
    }
}

// switches to 64-bit counts where the reference's 32-bit offsets would overflow
void relayout(bclbm_output* o) {
    o->wide = o->force_wide;
    layout(o);
    bool big = o->grid_bytes > kInt32Max;
    for (const File& f : o->files) big |= f.offset > kInt32Max;
    if (big && !o->wide) {
        o->wide = true;
        layout(o);
    }
    o->grid_blocks.clear();
}

// the values of one variable as written (binary block or ASCII text)
std::vector<char> gather(const bclbm_output* o, const Var& v) {
    const int32_t* nodes = o->nodes.empty() ? nullptr : o->nodes.data();
    if (o->format == BCLBM_VTU_BINARY) {
        const int sz = value_size(v.out_type), hdr = o->wide ? 8 : 4;
        std::vector<char> b(static_cast<size_t>(hdr + v.length * sz));
        const uint64_t nb = static_cast<uint64_t>(v.length) * sz;
        if (o->wide) std::memcpy(b.data(), &nb, 8);
        else {
            const uint32_t nb32 = static_cast<uint32_t>(nb);
            std::memcpy(b.data(), &nb32, 4);
        }
        char* base = b.data() + hdr;
        parallel_for(static_cast<size_t>(v.length), [&](size_t s, size_t e) {
            if (v.out_type == BCLBM_VTU_FLOAT64) {
                double* d = reinterpret_cast<double*>(base);
                for (size_t j = s; j < e; ++j) d[j] = v.value<double>(static_cast<int64_t>(j), nodes);
            } else if (v.out_type == BCLBM_VTU_FLOAT32) {
                float* d = reinterpret_cast<float*>(base);
                for (size_t j = s; j < e; ++j) d[j] = v.value<float>(static_cast<int64_t>(j), nodes);
            } else {
                int32_t* d = reinterpret_cast<int32_t*>(base);
                for (size_t j = s; j < e; ++j) d[j] = v.value<int32_t>(static_cast<int64_t>(j), nodes);
            }
        });
        return b;
    }
    std::string s;
    s.reserve(static_cast<size_t>(v.length) * 8);
    const bool integer = v.out_type == BCLBM_VTU_INT32;
    for (int64_t j = 0; j < v.length; ++j) {
        double x;
        if (v.out_type == BCLBM_VTU_FLOAT64) x = v.value<double>(j, nodes);
        else if (v.out_type == BCLBM_VTU_FLOAT32) x = v.value<float>(j, nodes);
        else x = v.value<int32_t>(j, nodes);
        put_ascii(s, x, integer);
    }
    return std::vector<char>(s.begin(), s.end());
}

std::string timestring() {  // PVTU_file::timestring (VTK.h:1248-1257)
    const time_t t = time(nullptr);
    struct tm tm;
    localtime_r(&t, &tm);
    char b[64];
    std::snprintf(b, sizeof b, "%02d.%02d.%02d %02d:%02d:%02d", tm.tm_mday, tm.tm_mon + 1, tm.tm_year + 1900,
                  tm.tm_hour, tm.tm_min, tm.tm_sec);
    return b;
}

bool put(FILE* fp, const void* p, size_t n) { return n == 0 || std::fwrite(p, 1, n, fp) == n; }
bool put(FILE* fp, const std::string& s) { return put(fp, s.data(), s.size()); }

// VTU_file::write (VTK.h:1095-1104) and PVTU_file::write (:1226-1244) of one file
int write_file(const bclbm_output* o, const File& f, int nwrite, double time, const std::vector<std::vector<char>>& vals,
               std::string& err) {
    char num[64];
    std::snprintf(num, sizeof num, "%04d_%s_%07d.vtu", o->rank, f.name.c_str(), nwrite);
    const std::string vtu_name = num;
    {
        FILE* fp = std::fopen((o->vtu_dir + vtu_name).c_str(), "wb");
        if (!fp) {
            err = "cannot open " + o->vtu_dir + vtu_name;
            return BCLBM_ERR_INVALID;
        }
        const int fmt = o->format;
        const int64_t hdr = o->wide ? 8 : 4;
        std::string h = "<?xml version=\"1.0\"?>\n<VTKFile type=\"UnstructuredGrid\" version=\"0.1\" byte_order=\"LittleEndian\"";
        if (o->wide) h += " header_type=\"UInt64\"";
        h += ">\n  <UnstructuredGrid>\n    <Piece NumberOfPoints=\"" + std::to_string(o->n_points) +
             "\" NumberOfCells=\"" + std::to_string(o->n_cells) + "\">\n      <Points>\n";
        bool ok = true;
        const char* gnames[4] = {"points", "connectivity", "offsets", "types"};
        const char* gtypes[4] = {"Float32", "Int32", "Int32", "Int32"};
        int64_t goff = 0;
        for (int k = 0; k < 4; ++k) {
            if (k == 1) h += "      </Points>\n      <Cells>\n";
            h += "        " + data_array(gnames[k], gtypes[k], k == 0 ? 3 : 1, fmt, goff);
            if (fmt != BCLBM_VTU_BINARY) {
                ok &= put(fp, h);
                ok &= put(fp, o->grid_blocks[k].bytes.data(), o->grid_blocks[k].bytes.size());
                h.clear();
            }
            h += "</DataArray>\n";
            goff += static_cast<int64_t>(o->grid_blocks[k].bytes.size());
        }
        h += "      </Cells>\n";
        // CellData Scalars/Vectors name lists (Variables::update_names, VTK.h:970-980)
        std::string scal, vect;
        for (const Var& v : f.vars) {
            std::string& l = v.dim_out > 1 ? vect : scal;
            if (!l.empty()) l += ", ";
            l += v.name;
        }
        h += "      <CellData Scalars=\"" + scal + "\" Vectors=\"" + vect + "\">\n";
        for (size_t k = 0; k < f.vars.size(); ++k) {
            const Var& v = f.vars[k];
            h += "        " + data_array(v.name, type_name(v.out_type), v.dim_out, fmt, v.offset);
            if (fmt != BCLBM_VTU_BINARY) {
                ok &= put(fp, h);
                ok &= put(fp, vals[k].data(), vals[k].size());
                h.clear();
            }
            h += "</DataArray>\n";
        }
        h += "      </CellData>\n    </Piece>\n  </UnstructuredGrid>\n";
        ok &= put(fp, h);
        if (fmt == BCLBM_VTU_BINARY && f.offset > 0) {
            ok &= put(fp, std::string("  <AppendedData encoding=\"raw\">\n_"));
            for (const Block& b : o->grid_blocks) ok &= put(fp, b.bytes.data(), b.bytes.size());
            for (const auto& b : vals) ok &= put(fp, b.data(), b.size());
            ok &= put(fp, std::string("  </AppendedData>\n"));
        }
        ok &= put(fp, std::string("</VTKFile>\n"));
        ok &= std::fclose(fp) == 0;
        if (!ok) {
            err = "write to " + o->vtu_dir + vtu_name + " failed";
            return BCLBM_ERR_INVALID;
        }
    }
    // the PVTU: header, this rank's piece padded to 99 characters plus a newline
    // (the MPI_write_piece form, VTK.h:1289-1306, which the reference's MPI runs take), footer
    std::snprintf(num, sizeof num, "%s_%07d.pvtu", f.name.c_str(), nwrite);
    const std::string pvtu = o->dir + num;
    FILE* fp = std::fopen(pvtu.c_str(), "wb");
    if (!fp) {
        err = "cannot open " + pvtu;
        return BCLBM_ERR_INVALID;
    }
    char tbuf[40];
    std::snprintf(tbuf, sizeof tbuf, "%g", time);
    std::string h = "<?xml version=\"1.0\"?>\n<!-- Created " + timestring() + " -->\n<!-- time = " + tbuf +
                    " s -->\n<VTKFile type=\"PUnstructuredGrid\" version=\"0.1\" byte_order=\"LittleEndian\">\n"
                    "  <PUnstructuredGrid GhostLevel=\"0\">\n    <PPoints>\n"
                    "      <PDataArray type=\"Float32\" NumberOfComponents=\"3\" />\n    </PPoints>\n"
                    "    <PCellData>\n      <PDataArray type=\"Int32\" Name=\"connectivity\" />\n"
                    "      <PDataArray type=\"Int32\" Name=\"offsets\" />\n      <PDataArray type=\"Int32\" Name=\"types\" />\n"
                    "    </PCellData>\n    <PCellData>\n";
    for (const Var& v : f.vars)
        h += "      <PDataArray Name=\"" + v.name + "\" type=\"" + type_name(v.out_type) + "\" NumberOfComponents=\"" +
             std::to_string(v.dim_out) + "\" />\n";
    h += "    </PCellData>\n";
    std::string piece = "    <Piece Source=\"vtu/" + vtu_name + "\" />";
    if (piece.size() < 99) piece.append(99 - piece.size(), ' ');
    piece += '\n';
    piece.resize(100);
    h += piece;
    h += "  </PUnstructuredGrid>\n</VTKFile>\n";
    bool ok = put(fp, h);
    ok &= std::fclose(fp) == 0;
    if (!ok) {
        err = "write to " + pvtu + " failed";
        return BCLBM_ERR_INVALID;
    }
    return BCLBM_OK;
}

struct Snapshot {  // one write: the values of every file's variables and the write numbers
    std::vector<std::vector<std::vector<char>>> vals;
    std::vector<int> nwrite;
    double time = 0.0;
};

int take(bclbm_output* o, double time, Snapshot& s) {
    BCLBM_TRACE("bclbm_output_gather");
    if (o->grid_blocks.empty()) build_grid_blocks(o);
    s.time = time;
    for (File& f : o->files) {
        std::vector<std::vector<char>> v;
        for (const Var& var : f.vars) v.push_back(gather(o, var));
        s.vals.push_back(std::move(v));
        s.nwrite.push_back(f.nwrite++);
    }
    return BCLBM_OK;
}

int emit(const bclbm_output* o, const Snapshot& s, std::string& err) {
    BCLBM_TRACE("bclbm_output_write_files");
    for (size_t k = 0; k < o->files.size(); ++k) {
        const int rc = write_file(o, o->files[k], s.nwrite[k], s.time, s.vals[k], err);
        if (rc != BCLBM_OK) return rc;
    }
    return BCLBM_OK;
}

int join(bclbm_output* o) {
    if (o->writer.joinable()) o->writer.join();
    const int rc = o->async_status;
    o->async_status = BCLBM_OK;
    return rc;
}

int fail(bclbm_output* o, int rc, const std::string& what) {
    o->error = what;
    return rc;
}

}  // namespace

extern "C" {

int bclbm_output_create(int32_t nd, int64_t n_cells, const int32_t* pos, const int32_t* nodes, const char* dir,
                        int32_t rank, int32_t nproc, int32_t value_type, int32_t format, bclbm_output** out) {
    if (!out) return BCLBM_ERR_INVALID;
    *out = nullptr;
    if ((nd != 2 && nd != 3) || n_cells < 1 || !pos || !dir || !dir[0] || rank < 0 || nproc < 1 || rank >= nproc)
        return BCLBM_ERR_INVALID;
    if (value_type != BCLBM_VTU_FLOAT64 && value_type != BCLBM_VTU_FLOAT32 && value_type != BCLBM_VTU_INT32)
        return BCLBM_ERR_INVALID;
    if (format != BCLBM_VTU_BINARY && format != BCLBM_VTU_ASCII && format != BCLBM_VTU_BINARY64)
        return BCLBM_ERR_INVALID;
    if (nproc != 1) return BCLBM_ERR_UNSUPPORTED;  // PVTU pieces of several ranks share one file
    if (n_cells * (nd == 3 ? 8 : 4) > kInt32Max) return BCLBM_ERR_UNSUPPORTED;
    bclbm_output* o = new (std::nothrow) bclbm_output();
    if (!o) return BCLBM_ERR_NOMEM;
    int rc = BCLBM_OK;
    try {
        o->nd = nd;
        o->n_cells = n_cells;
        o->value_type = value_type;
        o->format = format == BCLBM_VTU_BINARY64 ? BCLBM_VTU_BINARY : format;
        o->force_wide = format == BCLBM_VTU_BINARY64;
        o->rank = rank;
        o->nproc = nproc;
        if (nodes) o->nodes.assign(nodes, nodes + n_cells);
        // File::File folder handling (VTK.h:1010-1019, 1060-1072): "<dir>/", then "<dir>/vtu/"
        o->dir = dir;
        if (o->dir.back() != '/') o->dir += '/';
        make_dir(o->dir);
        o->vtu_dir = o->dir + "vtu/";
        make_dir(o->vtu_dir);
        rc = build_mesh(o, pos);
        if (rc == BCLBM_OK) relayout(o);
    } catch (const std::bad_alloc&) {
        rc = BCLBM_ERR_NOMEM;
    }
    if (rc != BCLBM_OK) {
        delete o;
        return rc;
    }
    *out = o;
    return BCLBM_OK;
}

int bclbm_output_add_file(bclbm_output* o, const char* name) {
    if (!o || !name || !name[0]) return BCLBM_ERR_INVALID;
    const int rc = join(o);
    if (rc != BCLBM_OK) return rc;
    o->files.push_back(File{name, {}, 0, 0});
    relayout(o);
    return BCLBM_OK;
}

static int add_var(bclbm_output* o, Var v) {
    if (o->files.empty()) return fail(o, BCLBM_ERR_INVALID, "add an output file before adding variables");
    const int rc = join(o);
    if (rc != BCLBM_OK) return rc;
    o->files.back().vars.push_back(std::move(v));
    relayout(o);
    return BCLBM_OK;
}

int bclbm_output_add_field(bclbm_output* o, const char* name, const double* data, int32_t n_fields, int32_t dim,
                           int32_t field_no) {
    if (!o || !name || !name[0] || !data || n_fields < 1 || (dim != 1 && dim != o->nd)) return BCLBM_ERR_INVALID;
    if (field_no < -1 || field_no >= n_fields) return BCLBM_ERR_INVALID;
    if (o->nodes.empty()) return fail(o, BCLBM_ERR_INVALID, "the output was created without node numbers");
    for (int32_t i = field_no < 0 ? 0 : field_no; i < (field_no < 0 ? n_fields : field_no + 1); ++i) {
        Var v;
        // Output::add_variable__ appends the field number whenever there are several
        // fields, also to the names add_variable_with_names gives (Output.h:166-169)
        v.name = n_fields > 1 ? std::string(name) + std::to_string(i) : std::string(name);
        v.out_type = o->value_type;
        v.src = data;
        v.src_type = BCLBM_VTU_FLOAT64;
        v.field = true;
        v.n_fields = n_fields;
        v.field_no = i;
        v.dim = dim;
        v.dim_out = dim == 2 ? 3 : dim;
        v.length = o->n_cells * v.dim_out;
        const int rc = add_var(o, std::move(v));
        if (rc != BCLBM_OK) return rc;
    }
    return BCLBM_OK;
}

int bclbm_output_add_array(bclbm_output* o, const char* name, const void* data, int32_t data_type, int64_t length) {
    if (!o || !name || !name[0] || !data || length < 1) return BCLBM_ERR_INVALID;
    if (data_type != BCLBM_VTU_FLOAT64 && data_type != BCLBM_VTU_FLOAT32 && data_type != BCLBM_VTU_INT32)
        return BCLBM_ERR_INVALID;
    // VTK::Output::add_variable_ (VTK.h:1528-1547): the components per cell from the size
    const int64_t dim = length / o->n_cells;
    if (dim != 1 && dim != o->nd) return fail(o, BCLBM_ERR_INVALID, "wrong dimension: expected 1 or the lattice's");
    Var v;
    v.name = name;
    v.out_type = o->value_type;
    v.src = data;
    v.src_type = data_type;
    v.dim = static_cast<int32_t>(dim);
    v.dim_out = dim == 2 ? 3 : static_cast<int32_t>(dim);
    v.length = dim == 2 ? 3 * (length / 2) : length;
    return add_var(o, std::move(v));
}

int bclbm_output_write(bclbm_output* o, double time) {
    if (!o) return BCLBM_ERR_INVALID;
    int rc = join(o);
    if (rc != BCLBM_OK) return rc;
    try {
        Snapshot s;
        rc = take(o, time, s);
        if (rc == BCLBM_OK) rc = emit(o, s, o->error);
    } catch (const std::bad_alloc&) {
        rc = BCLBM_ERR_NOMEM;
    }
    return rc;
}

int bclbm_output_write_async(bclbm_output* o, double time) {
    if (!o) return BCLBM_ERR_INVALID;
    int rc = join(o);
    if (rc != BCLBM_OK) return rc;
    try {
        auto s = std::make_shared<Snapshot>();
        rc = take(o, time, *s);
        if (rc != BCLBM_OK) return rc;
        o->writer = std::thread([o, s] {
            std::string err;
            const int r = emit(o, *s, err);
            if (r != BCLBM_OK) {
                std::lock_guard<std::mutex> g(o->mu);
                o->error = err;
                o->async_status = r;
            }
        });
    } catch (const std::bad_alloc&) {
        rc = BCLBM_ERR_NOMEM;
    } catch (const std::system_error&) {
        rc = BCLBM_ERR_INVALID;
    }
    return rc;
}

int bclbm_output_wait(bclbm_output* o) {
    if (!o) return BCLBM_ERR_INVALID;
    return join(o);
}

int bclbm_output_info(const bclbm_output* o, int64_t* n_points, int64_t* n_cells, int32_t* n_files) {
    if (!o) return BCLBM_ERR_INVALID;
    if (n_points) *n_points = o->n_points;
    if (n_cells) *n_cells = o->n_cells;
    if (n_files) *n_files = static_cast<int32_t>(o->files.size());
    return BCLBM_OK;
}

const char* bclbm_output_last_error(const bclbm_output* o) { return o ? o->error.c_str() : ""; }

void bclbm_output_destroy(bclbm_output* o) {
    if (!o) return;
    join(o);
    delete o;
}

}  // extern "C"
