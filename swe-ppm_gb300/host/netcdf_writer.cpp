// NetCDF snapshot writer (C ABI in include/swe_gb300_host.h).
//
// Writes the variables and layout of the reference's NetCdfWriter
// (src/writer/NetCdfWriter.cpp:84-130, 153-234): dimensions time (unlimited),
// x, y; float variables time(time), x(x), y(y), ah(time, y, x), hu(time, y, x),
// hv(time, y, x) and b(y, x); CF-1.5 global attributes; cell-centre
// coordinates origin + dx/2 + i dx accumulated in float.  libnetcdf is not
// available, so the file is produced directly in the classic NetCDF format
// with 64-bit offsets ("CDF\2", the public format specification); every
// NetCDF reader (including scipy.io.netcdf_file) opens it.  The number of
// records in the header is rewritten after every time step, so a file that is
// cut short still holds every completed step.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/swe_gb300_host.h"

struct swe_nc_writer {
    FILE *f = nullptr;
    int nx = 0, ny = 0;
    long long recBegin = 0;   // file offset of the first record
    long long recSize = 0;    // bytes per record
    long long recOffH = 0, recOffHU = 0, recOffHV = 0;  // offsets of ah/hu/hv inside a record
    int records = 0;
    std::vector<unsigned char> buf;
};

namespace {

void be32(std::vector<unsigned char> &o, uint32_t v) {
    for (int i = 3; i >= 0; i--) o.push_back((unsigned char)(v >> (8 * i)));
}
void be64(std::vector<unsigned char> &o, uint64_t v) {
    for (int i = 7; i >= 0; i--) o.push_back((unsigned char)(v >> (8 * i)));
}
void pad4(std::vector<unsigned char> &o) {
    while (o.size() % 4) o.push_back(0);
}
void name(std::vector<unsigned char> &o, const char *s) {
    const uint32_t n = uint32_t(strlen(s));
    be32(o, n);
    o.insert(o.end(), s, s + n);
    pad4(o);
}
void textAttr(std::vector<unsigned char> &o, const char *key, const char *val) {
    name(o, key);
    be32(o, 2);  // NC_CHAR
    const uint32_t n = uint32_t(strlen(val));
    be32(o, n);
    o.insert(o.end(), val, val + n);
    pad4(o);
}
uint32_t floatBits(float v) {
    uint32_t u;
    memcpy(&u, &v, 4);
    return u;
}
/// interior of a Float2D array (a[x][y] = raw[x*ld + y], ghosts at 0 and n+1)
/// as a big-endian (y, x) slab, the order the reference writes column by column
void slab(const float *a, int ld, int nx, int ny, std::vector<unsigned char> &o) {
    o.resize(size_t(nx) * size_t(ny) * 4);
    unsigned char *p = o.data();
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) {
            const uint32_t u = floatBits(a[size_t(i + 1) * ld + size_t(j + 1)]);
            p[0] = (unsigned char)(u >> 24); p[1] = (unsigned char)(u >> 16);
            p[2] = (unsigned char)(u >> 8); p[3] = (unsigned char)u;
            p += 4;
        }
}

struct VarDef {
    const char *name;
    std::vector<int> dims;
    bool record;
    long long vsize;
    std::vector<std::pair<const char *, const char *>> attrs;
};

} // namespace

extern "C" {

int swe_nc_open(const char *path, int nx, int ny, float dx, float dy, float originX, float originY, const float *b,
                int ld, swe_nc_writer **out) {
    if (!path || !out || nx < 1 || ny < 1 || !b || ld < ny + 2) return -1;
    *out = nullptr;
    FILE *f = fopen(path, "wb");
    if (!f) return -2;
    auto *W = new swe_nc_writer();
    W->f = f;
    W->nx = nx;
    W->ny = ny;
    const long long slabBytes = 4LL * nx * ny;
    // dimension ids: 0 time (record), 1 x, 2 y; variables in the reference's definition order
    std::vector<VarDef> vars = {
        {"time", {0}, true, 4, {{"long_name", "Time"}, {"units", "seconds since simulation start"}}},
        {"x", {1}, false, 4LL * nx, {}},
        {"y", {2}, false, 4LL * ny, {}},
        {"ah", {0, 2, 1}, true, slabBytes, {}},
        {"hu", {0, 2, 1}, true, slabBytes, {}},
        {"hv", {0, 2, 1}, true, slabBytes, {}},
        {"b", {2, 1}, false, slabBytes, {}},
    };
    auto header = [&](std::vector<long long> begins, int numrecs) {
        std::vector<unsigned char> h;
        h.insert(h.end(), {'C', 'D', 'F', 2});
        be32(h, uint32_t(numrecs));
        be32(h, 0x0A);  // NC_DIMENSION
        be32(h, 3);
        name(h, "time"); be32(h, 0);
        name(h, "x"); be32(h, uint32_t(nx));
        name(h, "y"); be32(h, uint32_t(ny));
        be32(h, 0x0C);  // NC_ATTRIBUTE (global)
        be32(h, 5);
        textAttr(h, "Conventions", "CF-1.5");
        textAttr(h, "title", "Computed tsunami solution");
        textAttr(h, "history", "SWE");
        textAttr(h, "source", "swe-gb300 block step (GB300)");
        textAttr(h, "comment", "shallow-water state written from device snapshots");
        be32(h, 0x0B);  // NC_VARIABLE
        be32(h, uint32_t(vars.size()));
        for (size_t v = 0; v < vars.size(); v++) {
            name(h, vars[v].name);
            be32(h, uint32_t(vars[v].dims.size()));
            for (int d : vars[v].dims) be32(h, uint32_t(d));
            if (vars[v].attrs.empty()) {
                be32(h, 0); be32(h, 0);
            } else {
                be32(h, 0x0C);
                be32(h, uint32_t(vars[v].attrs.size()));
                for (auto &a : vars[v].attrs) textAttr(h, a.first, a.second);
            }
            be32(h, 5);  // NC_FLOAT
            be32(h, uint32_t(vars[v].vsize));
            be64(h, uint64_t(begins[v]));
        }
        return h;
    };
    // first pass for the header size, second with the data offsets
    std::vector<long long> begins(vars.size(), 0);
    const long long hsize = (long long)header(begins, 0).size();
    long long off = hsize;
    for (size_t v = 0; v < vars.size(); v++)
        if (!vars[v].record) {
            begins[v] = off;
            off += vars[v].vsize;
        }
    W->recBegin = off;
    long long roff = 0;
    for (size_t v = 0; v < vars.size(); v++)
        if (vars[v].record) {
            begins[v] = W->recBegin + roff;
            if (!strcmp(vars[v].name, "ah")) W->recOffH = roff;
            if (!strcmp(vars[v].name, "hu")) W->recOffHU = roff;
            if (!strcmp(vars[v].name, "hv")) W->recOffHV = roff;
            roff += vars[v].vsize;
        }
    W->recSize = roff;
    std::vector<unsigned char> h = header(begins, 0);
    // non-record data: x, y cell centres (float accumulation as the reference), b
    std::vector<unsigned char> d;
    float pos = originX + 0.5f * dx;
    for (int i = 0; i < nx; i++) {
        be32(d, floatBits(pos));
        pos += dx;
    }
    pos = originY + 0.5f * dy;
    for (int j = 0; j < ny; j++) {
        be32(d, floatBits(pos));
        pos += dy;
    }
    std::vector<unsigned char> bs;
    slab(b, ld, nx, ny, bs);
    d.insert(d.end(), bs.begin(), bs.end());
    if (fwrite(h.data(), 1, h.size(), f) != h.size() || fwrite(d.data(), 1, d.size(), f) != d.size()) {
        fclose(f);
        delete W;
        return -3;
    }
    fflush(f);
    *out = W;
    return 0;
}

/// appends one time step from big-endian (y, x) slabs of the interior
int swe_nc_write_step_slabs(swe_nc_writer *W, float t, const void *h, const void *hu, const void *hv) {
    if (!W || !h || !hu || !hv) return -1;
    const long long base = W->recBegin + (long long)W->records * W->recSize;
    const size_t slabBytes = size_t(4) * W->nx * W->ny;
    std::vector<unsigned char> tb;
    be32(tb, floatBits(t));
    // record layout: time, ah, hu, hv (each vsize, already multiples of 4)
    if (fseeko(W->f, base, SEEK_SET)) return -2;
    if (fwrite(tb.data(), 1, 4, W->f) != 4) return -3;
    if (fseeko(W->f, base + W->recOffH, SEEK_SET) || fwrite(h, 1, slabBytes, W->f) != slabBytes) return -3;
    if (fseeko(W->f, base + W->recOffHU, SEEK_SET) || fwrite(hu, 1, slabBytes, W->f) != slabBytes) return -3;
    if (fseeko(W->f, base + W->recOffHV, SEEK_SET) || fwrite(hv, 1, slabBytes, W->f) != slabBytes) return -3;
    W->records++;
    // numrecs lives right after the magic number
    std::vector<unsigned char> nr;
    be32(nr, uint32_t(W->records));
    if (fseeko(W->f, 4, SEEK_SET) || fwrite(nr.data(), 1, 4, W->f) != 4) return -3;
    fflush(W->f);
    return 0;
}

/// appends one time step from host Float2D arrays (interior written, ghosts skipped)
int swe_nc_write_step(swe_nc_writer *W, float t, const float *h, const float *hu, const float *hv, int ld) {
    if (!W || !h || !hu || !hv || ld < W->ny + 2) return -1;
    std::vector<unsigned char> a, b, c;
    slab(h, ld, W->nx, W->ny, a);
    slab(hu, ld, W->nx, W->ny, b);
    slab(hv, ld, W->nx, W->ny, c);
    return swe_nc_write_step_slabs(W, t, a.data(), b.data(), c.data());
}

int swe_nc_close(swe_nc_writer *W) {
    if (!W) return -1;
    const int rc = fclose(W->f) == 0 ? 0 : -3;
    delete W;
    return rc;
}

} // extern "C"
