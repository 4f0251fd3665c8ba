// Particle file IO.  Asynchronous export: the reference's
// Simulation::exportParticles (src/simulation.cpp:231-245) and Exporter
// (src/exporter.cpp:10-167).  CSV import: MPS::importInitialCondition
// (src/mps.cpp:38-94).
//
// The reference copies every particle to its host vector each export step and
// formats the CSV and VTU files on the stepping thread.  Here an export is a
// snapshot: one gather kernel on the engine's stream puts the state into id
// order in a device buffer, a copy on a second stream moves it to pinned
// host memory, and the steps that follow run meanwhile.  The writers format
// the snapshot with std::to_chars on several threads (the same text as the
// reference's printf("%.6f") CSV fields and default-precision ostream VTU
// fields) and write each file with a few large writes.
#include <algorithm>
#include <charconv>
#include <cstdio>
#include <cstring>
#include <string>
#include <system_error>
#include <thread>
#include <vector>

#include "engine_impl.cuh"

using namespace mpsg;

namespace {

// slot k -> id order: pos/vel xyz-interleaved (planar engines: z = z0, v_z = 0)
__global__ void k_export_gather(int n, const int32_t* __restrict__ id, const double* __restrict__ x,
                                const double* __restrict__ y, const double* __restrict__ z, double z0,
                                const double* __restrict__ vx, const double* __restrict__ vy,
                                const double* __restrict__ vz, const double* __restrict__ p,
                                const double* __restrict__ ndr, const int8_t* __restrict__ type,
                                const int8_t* __restrict__ bc, size_t np, double* __restrict__ out,
                                int32_t* __restrict__ out_i) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const size_t o = (size_t)id[k];
    out[3 * o] = x[k];
    out[3 * o + 1] = y[k];
    out[3 * o + 2] = z ? z[k] : z0;
    out[3 * np + 3 * o] = vx[k];
    out[3 * np + 3 * o + 1] = vy[k];
    out[3 * np + 3 * o + 2] = vz ? vz[k] : 0.0;
    out[6 * np + o] = p[k];
    out[7 * np + o] = ndr[k];
    out_i[o] = type[k];
    out_i[np + o] = bc[k];
}

int err(int code, const std::string& m) {
    set_last_error(m);
    return code;
}

#define XCU(call)                                                                            \
    do {                                                                                     \
        cudaError_t err_ = (call);                                                           \
        if (err_ != cudaSuccess)                                                             \
            return err(MPS_ERR_CUDA, std::string(#call " failed: ") + cudaGetErrorString(err_)); \
    } while (0)

// ---------------------------------------------------------------- writers
// printf("%.6f") and ostream's default (printf "%g", 6 significant digits)
// are both defined as correctly rounded; std::to_chars with the same format
// and precision produces the same characters.
inline void put_fixed6(std::string& s, double v) {
    char b[400];
    const auto r = std::to_chars(b, b + sizeof b, v, std::chars_format::fixed, 6);
    s.append(b, r.ptr);
}
inline void put_general6(std::string& s, double v) {
    char b[64];
    const auto r = std::to_chars(b, b + sizeof b, v, std::chars_format::general, 6);
    s.append(b, r.ptr);
}
inline void put_int(std::string& s, long long v) {
    char b[24];
    const auto r = std::to_chars(b, b + sizeof b, v);
    s.append(b, r.ptr);
}

// Formats [0, n) in chunks on up to 16 threads (about row_bytes each) and
// writes them in order; chunks whose thread could not start run here.
template <typename F>
bool write_rows(std::FILE* f, int n, size_t row_bytes, F&& row) {
    const int hw = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    const int T = n >= 65536 ? hw : 1;
    std::vector<std::string> part(T);
    auto work = [&](int t) {
        const int b = (int)((long long)n * t / T), e = (int)((long long)n * (t + 1) / T);
        std::string& s = part[t];
        s.reserve((size_t)(e - b) * row_bytes);
        for (int i = b; i < e; i++) row(s, i);
    };
    std::vector<std::thread> th;
    int started = 1;
    try {
        for (int t = 1; t < T; t++, started++) th.emplace_back(work, t);
    } catch (const std::system_error&) {
    }
    work(0);
    for (int t = started; t < T; t++) work(t);
    for (auto& x : th) x.join();
    for (auto& s : part)
        if (!s.empty() && std::fwrite(s.data(), 1, s.size(), f) != s.size()) return false;
    return true;
}

bool put(std::FILE* f, const std::string& s) { return std::fwrite(s.data(), 1, s.size(), f) == s.size(); }

// Exporter::toCsv (src/exporter.cpp:10-55): Ghost particles skipped, the
// count line holds every particle.
int write_csv(const mps_snapshot& s, const char* path, double time) {
    std::FILE* f = std::fopen(path, "wb");
    if (!f) return err(MPS_ERR_ARG, std::string("Could not open target csv file: ") + path);
    std::string h = "Time (s),";
    put_fixed6(h, time);
    h += "\nNumber of Particles,";
    put_int(h, s.n);
    h += "\nID,Type,Position.x (m),Position.y (m),Position.z (m),Velocity.x (m/s),Velocity.y (m/s),"
         "Velocity.z (m/s),Pressure (Pa),Number Density Ratio\n";
    bool ok = put(f, h) && write_rows(f, s.n, 96, [&](std::string& o, int i) {
        if (s.type[i] == -1) return;
        put_int(o, i);
        o += ',';
        put_int(o, s.type[i]);
        for (int c = 0; c < 3; c++) {
            o += ',';
            put_fixed6(o, s.pos[3 * (size_t)i + c]);
        }
        for (int c = 0; c < 3; c++) {
            o += ',';
            put_fixed6(o, s.vel[3 * (size_t)i + c]);
        }
        o += ',';
        put_fixed6(o, s.pressure[i]);
        o += ',';
        put_fixed6(o, s.ndr[i]);
        o += '\n';
    });
    ok = (std::fclose(f) == 0) && ok;
    return ok ? MPS_OK : err(MPS_ERR_ARG, std::string("write failed: ") + path);
}

// Exporter::toVtu (src/exporter.cpp:57-167): every particle, one vertex cell
// each; the velocity's z is written as 0.
int write_vtu(const mps_snapshot& s, const char* path, double time) {
    std::FILE* f = std::fopen(path, "wb");
    if (!f) return err(MPS_ERR_ARG, std::string("Could not open target vtu file: ") + path);
    const int n = s.n;
    auto begin_array = [](const char* comps, const char* type, const char* name) {
        return std::string("<DataArray NumberOfComponents='") + comps + "' type='" + type + "' Name='" +
               name + "' format='ascii'>\n";
    };
    const std::string end_array = "</DataArray>\n";
    std::string h = "<?xml version='1.0' encoding='UTF-8'?>\n"
                    "<VTKFile byte_order='LittleEndian' version='0.1' type = 'UnstructuredGrid'>\n"
                    "<UnstructuredGrid>\n<FieldData>\n"
                    "<DataArray type='Float64' Name='Time' NumberOfComponents='1' NumberOfTuples='1' "
                    "format='ascii'>\n";
    put_general6(h, time);
    h += "\n</DataArray>\n</FieldData>\n<Piece NumberOfCells='";
    put_int(h, n);
    h += "' NumberOfPoints='";
    put_int(h, n);
    h += "'>\n<Points>\n<DataArray NumberOfComponents='3' type='Float64' Name='position' format='ascii'>\n";
    bool ok = put(f, h);
    ok = ok && write_rows(f, n, 36, [&](std::string& o, int i) {
        for (int c = 0; c < 3; c++) {
            put_general6(o, s.pos[3 * (size_t)i + c]);
            o += c < 2 ? ' ' : '\n';
        }
    });
    ok = ok && put(f, end_array + "</Points>\n<PointData>\n" + begin_array("1", "Int32", "Type"));
    ok = ok && write_rows(f, n, 3, [&](std::string& o, int i) {
        put_int(o, s.type[i]);
        o += '\n';
    });
    ok = ok && put(f, end_array + begin_array("3", "Float64", "Velocity"));
    ok = ok && write_rows(f, n, 28, [&](std::string& o, int i) {
        put_general6(o, s.vel[3 * (size_t)i]);
        o += ' ';
        put_general6(o, s.vel[3 * (size_t)i + 1]);
        o += " 0\n";
    });
    ok = ok && put(f, end_array + begin_array("1", "Float64", "Pressure"));
    ok = ok && write_rows(f, n, 12, [&](std::string& o, int i) {
        put_general6(o, s.pressure[i]);
        o += '\n';
    });
    ok = ok && put(f, end_array + begin_array("1", "Float64", "Number Density Ratio"));
    ok = ok && write_rows(f, n, 12, [&](std::string& o, int i) {
        put_general6(o, s.ndr[i]);
        o += '\n';
    });
    ok = ok && put(f, end_array + begin_array("1", "Int32", "Boundary Condition"));
    ok = ok && write_rows(f, n, 2, [&](std::string& o, int i) {
        put_int(o, s.bc[i]);
        o += '\n';
    });
    ok = ok && put(f, end_array + "</PointData>\n<Cells>\n<DataArray type='Int32' Name='connectivity' "
                                  "format='ascii'>\n");
    ok = ok && write_rows(f, n, 8, [&](std::string& o, int i) {
        put_int(o, i);
        o += '\n';
    });
    ok = ok && put(f, end_array + "<DataArray type='Int32' Name='offsets' format='ascii'>\n");
    ok = ok && write_rows(f, n, 8, [&](std::string& o, int i) {
        put_int(o, (long long)i + 1);
        o += '\n';
    });
    ok = ok && put(f, end_array + "<DataArray type='UInt8' Name='types' format='ascii'>\n");
    ok = ok && write_rows(f, n, 2, [&](std::string& o, int) { o += "1\n"; });
    ok = ok && put(f, end_array + "</Cells>\n</Piece>\n</UnstructuredGrid>\n</VTKFile>\n");
    ok = (std::fclose(f) == 0) && ok;
    return ok ? MPS_OK : err(MPS_ERR_ARG, std::string("write failed: ") + path);
}

// ------------------------------------------------------------- CSV import
// The file is read once; line starts are indexed in one pass; rows are parsed
// on up to 16 threads with std::from_chars (correctly rounded, so the values
// equal strtod's).
struct CsvFile {
    std::string text;
    std::vector<std::pair<size_t, size_t>> lines;  // [begin, end) without '\r'
};

bool read_all(const char* path, std::string& out) {
    std::FILE* f = std::fopen(path, "rb");
    if (!f) return false;
    std::fseek(f, 0, SEEK_END);
    const long len = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    if (len < 0) {
        std::fclose(f);
        return false;
    }
    out.resize((size_t)len);
    const bool ok = std::fread(out.data(), 1, out.size(), f) == out.size();
    std::fclose(f);
    return ok;
}

void index_lines(CsvFile& c) {
    const char* s = c.text.data();
    const size_t n = c.text.size();
    size_t b = 0;
    while (b < n) {
        const void* q = std::memchr(s + b, '\n', n - b);
        size_t e = q ? (size_t)((const char*)q - s) : n;
        const size_t next = q ? e + 1 : n;
        if (e > b && s[e - 1] == '\r') e--;
        c.lines.emplace_back(b, e);
        b = next;
    }
}

// fields of one line, split at commas
int split_fields(const char* b, const char* e, const char** fb, const char** fe, int cap) {
    int k = 0;
    const char* p = b;
    while (k < cap) {
        const char* q = (const char*)std::memchr(p, ',', (size_t)(e - p));
        fb[k] = p;
        fe[k] = q ? q : e;
        k++;
        if (!q) break;
        p = q + 1;
    }
    return k;
}

template <typename T>
bool parse_num(const char* b, const char* e, T& v) {
    while (b < e && *b == ' ') b++;
    while (e > b && e[-1] == ' ') e--;
    if (b < e && *b == '+') b++;
    const auto r = std::from_chars(b, e, v);
    return r.ec == std::errc() && r.ptr == e;
}

}  // namespace

extern "C" {

int mps_write_snapshot(const mps_snapshot* s, const char* csv_path, const char* vtu_path, double time) {
    if (!s || s->n < 0 || (s->n > 0 && (!s->pos || !s->vel || !s->pressure || !s->ndr || !s->type || !s->bc)))
        return err(MPS_ERR_ARG, "mps_write_snapshot: incomplete snapshot");
    try {  // no C++ exception crosses the C ABI
        if (csv_path) {
            const int rc = write_csv(*s, csv_path, time);
            if (rc) return rc;
        }
        if (vtu_path) {
            const int rc = write_vtu(*s, vtu_path, time);
            if (rc) return rc;
        }
    } catch (const std::exception& ex) {
        return err(MPS_ERR_ARG, std::string("mps_write_snapshot: ") + ex.what());
    }
    return MPS_OK;
}

int mps_export_begin(mps_engine* e) {
    if (!e) return err(MPS_ERR_ARG, "null engine");
    const size_t np = e->n_pad;
    if (!e->xdev) {
        // all or nothing: each resource is created once (mps_destroy frees
        // what exists), and the buffers count as ready only when all are
        if (!e->xst) XCU(cudaStreamCreateWithFlags(&e->xst, cudaStreamNonBlocking));
        if (!e->xev_ready) XCU(cudaEventCreateWithFlags(&e->xev_ready, cudaEventDisableTiming));
        if (!e->xev_done) XCU(cudaEventCreateWithFlags(&e->xev_done, cudaEventDisableTiming));
        if (!e->xhost) XCU(cudaMallocHost(&e->xhost, sizeof(double) * 8 * np));
        if (!e->xhost_i) XCU(cudaMallocHost(&e->xhost_i, sizeof(int32_t) * 2 * np));
        double* d = nullptr;
        if (!e->xdev_i && e->alloc(&e->xdev_i, 2 * np)) return err(MPS_ERR_CUDA, "cudaMalloc export buffers");
        if (e->alloc(&d, 8 * np)) return err(MPS_ERR_CUDA, "cudaMalloc export buffers");
        e->xdev = d;
    }
    // the device buffer is rewritten only after the last snapshot left it
    if (e->x_pending) XCU(cudaStreamWaitEvent(e->st, e->xev_done, 0));
    const StateBuf& s = e->S();
    const int n = e->n;
    const bool pl = e->c.planar;
    k_export_gather<<<(n + 255) / 256, 256, 0, e->st>>>(n, s.id, s.x, s.y, pl ? nullptr : s.z, e->c.z0,
                                                        s.vx, s.vy, pl ? nullptr : s.vz, s.p, s.ndr, s.type,
                                                        s.bc, np, e->xdev, e->xdev_i);
    ++g_launches;
    XCU(cudaGetLastError());
    XCU(cudaEventRecord(e->xev_ready, e->st));
    XCU(cudaStreamWaitEvent(e->xst, e->xev_ready, 0));
    XCU(cudaMemcpyAsync(e->xhost, e->xdev, sizeof(double) * 8 * np, cudaMemcpyDeviceToHost, e->xst));
    XCU(cudaMemcpyAsync(e->xhost_i, e->xdev_i, sizeof(int32_t) * 2 * np, cudaMemcpyDeviceToHost, e->xst));
    XCU(cudaEventRecord(e->xev_done, e->xst));
    e->x_pending = 1;
    return MPS_OK;
}

int mps_export_view(mps_engine* e, mps_snapshot* out) {
    if (!e || !out) return err(MPS_ERR_ARG, "mps_export_view: null argument");
    if (!e->x_pending) return err(MPS_ERR_ARG, "mps_export_view: no snapshot (call mps_export_begin)");
    XCU(cudaEventSynchronize(e->xev_done));
    const size_t np = e->n_pad;
    out->n = e->n;
    out->pos = e->xhost;
    out->vel = e->xhost + 3 * np;
    out->pressure = e->xhost + 6 * np;
    out->ndr = e->xhost + 7 * np;
    out->type = e->xhost_i;
    out->bc = e->xhost_i + np;
    return MPS_OK;
}

int mps_export_write(mps_engine* e, const char* csv_path, const char* vtu_path, double time) {
    mps_snapshot s;
    const int rc = mps_export_view(e, &s);
    if (rc) return rc;
    return mps_write_snapshot(&s, csv_path, vtu_path, time);
}

static int read_csv_impl(const char* path, int32_t capacity, int32_t* n, double* time, double* pos,
                         double* vel, int32_t* type);

int mps_read_csv(const char* path, int32_t capacity, int32_t* n, double* time, double* pos,
                 double* vel, int32_t* type) {
    if (!path || !n) return err(MPS_ERR_ARG, "mps_read_csv: null argument");
    try {  // no C++ exception crosses the C ABI
        return read_csv_impl(path, capacity, n, time, pos, vel, type);
    } catch (const std::exception& ex) {
        return err(MPS_ERR_ARG, std::string("mps_read_csv: ") + ex.what());
    }
}

static int read_csv_impl(const char* path, int32_t capacity, int32_t* n, double* time, double* pos,
                         double* vel, int32_t* type) {
    CsvFile c;
    if (!read_all(path, c.text))
        return err(MPS_ERR_ARG, std::string("Input file does not exist in the specified path: ") + path);
    index_lines(c);
    if (c.lines.size() < 3) return err(MPS_ERR_ARG, std::string("particle CSV too short: ") + path);
    const char* s = c.text.data();
    const char *fb[64], *fe[64];
    auto line_fields = [&](size_t r) {
        return split_fields(s + c.lines[r].first, s + c.lines[r].second, fb, fe, 64);
    };
    if (line_fields(0) < 2 || (time && !parse_num(fb[1], fe[1], *time)))
        return err(MPS_ERR_ARG, "particle CSV: bad time line");
    const int nh = line_fields(2);
    const char* need[8] = {"ID", "Type", "Position.x (m)", "Position.y (m)", "Position.z (m)",
                           "Velocity.x (m/s)", "Velocity.y (m/s)", "Velocity.z (m/s)"};
    int col[8];
    for (int k = 0; k < 8; k++) {
        col[k] = -1;
        for (int h = 0; h < nh; h++)
            if ((size_t)(fe[h] - fb[h]) == std::strlen(need[k]) && std::memcmp(fb[h], need[k], fe[h] - fb[h]) == 0)
                col[k] = h;
        if (col[k] < 0) return err(MPS_ERR_ARG, std::string("particle CSV lacks column ") + need[k]);
    }
    // data rows: non-empty lines after the header, in order
    std::vector<size_t> rows;
    rows.reserve(c.lines.size());
    for (size_t r = 3; r < c.lines.size(); r++)
        if (c.lines[r].second > c.lines[r].first) rows.push_back(r);
    if (rows.size() > (size_t)INT32_MAX) return err(MPS_ERR_ARG, "particle CSV: too many rows");
    *n = (int32_t)rows.size();
    if (rows.size() > (size_t)std::max(capacity, 0)) return MPS_ERR_CAPACITY;
    const int R = (int)rows.size();
    const int hw = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    const int T = R >= 65536 ? hw : 1;
    std::vector<long long> bad(T, -1);  // first bad row per thread
    auto work = [&](int t) {
        const char *b[64], *e[64];
        const int r0 = (int)((long long)R * t / T), r1 = (int)((long long)R * (t + 1) / T);
        for (int i = r0; i < r1; i++) {
            const auto& L = c.lines[rows[i]];
            const int nf = split_fields(s + L.first, s + L.second, b, e, 64);
            int id = -1, ty = 0;
            double v[6];
            bool ok = nf >= nh && parse_num(b[col[0]], e[col[0]], id) && id == i &&
                      parse_num(b[col[1]], e[col[1]], ty);
            for (int k = 0; ok && k < 6; k++) ok = parse_num(b[col[2 + k]], e[col[2 + k]], v[k]);
            if (!ok) {
                bad[t] = (long long)rows[i];
                return;
            }
            if (type) type[i] = ty;
            if (pos)
                for (int k = 0; k < 3; k++) pos[3 * (size_t)i + k] = v[k];
            if (vel)
                for (int k = 0; k < 3; k++) vel[3 * (size_t)i + k] = v[3 + k];
        }
    };
    std::vector<std::thread> th;
    int started = 1;
    try {
        for (int t = 1; t < T; t++, started++) th.emplace_back(work, t);
    } catch (const std::system_error&) {
    }
    work(0);
    for (int t = started; t < T; t++) work(t);
    for (auto& x : th) x.join();
    for (int t = 0; t < T; t++)
        if (bad[t] >= 0)
            return err(MPS_ERR_ARG, "particle CSV: bad row " + std::to_string(bad[t] + 1) +
                                        " (fields, numbers, or an ID that is not its row index)");
    return MPS_OK;
}

}  // extern "C"
