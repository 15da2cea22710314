// host_io.cpp -- the reference's file formats on the host: keyword=value
// configuration (config.h), ESRI ASCII rasters (io.cc), GridConfig
// (grid_config.cpp), CSV series (source.cc) and hot<k>.bin restart files
// (simulator.cu:912-1090).  Errors are status codes with a message, never
// exit() or a read of standard input.
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/rift_host.h"
#include "host_internal.hpp"

namespace rift_host {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}

// ------------------------------------------------------------- ConfigFile
// config.h:45-209: ';' starts a comment; a line without '=' or with nothing
// but blanks after it is malformed; the key is the text before '=' cut at
// its first blank, the value the text after it, trimmed of blanks and tabs.
int Config::open(const std::string& path) {
    std::ifstream f(path);
    if (!f) return fail(RIFT_ERR_ARG, "config: cannot open " + path);
    std::string line;
    size_t lineNo = 0;
    while (std::getline(f, line)) {
        lineNo++;
        if (line.empty()) continue;
        size_t sc = line.find(';');
        if (sc != std::string::npos) line.erase(sc);
        if (line.find_first_not_of(' ') == std::string::npos) continue;
        size_t eq = line.find('=');
        if (eq == std::string::npos)
            return fail(RIFT_ERR_ARG, "config: no '=' on line " + std::to_string(lineNo));
        std::string t = line;
        t.erase(0, t.find_first_not_of("\t "));
        eq = t.find('=');
        bool valueOk = false;
        for (size_t i = eq + 1; i < t.size(); i++)
            if (t[i] != ' ') valueOk = true;
        if (t.empty() || t[0] == '=' || !valueOk)
            return fail(RIFT_ERR_ARG, "config: bad format on line " + std::to_string(lineNo));
        std::string key = t.substr(0, eq);
        size_t blank = key.find_first_of("\t ");
        if (blank != std::string::npos) key.erase(blank);
        std::string value = t.substr(eq + 1);
        value.erase(0, value.find_first_not_of("\t "));
        size_t last = value.find_last_not_of("\t ");
        value.erase(last == std::string::npos ? 0 : last + 1);
        if (kv.count(key)) return fail(RIFT_ERR_ARG, "config: duplicate key " + key);
        kv[key] = value;
    }
    return RIFT_OK;
}

bool Config::has(const std::string& key) const { return kv.count(key) != 0; }

// keyIsNumber: the value's first word holds only digits and '.'
bool Config::isNumber(const std::string& key) const {
    auto it = kv.find(key);
    if (it == kv.end()) return false;
    std::istringstream is(it->second);
    std::string w;
    is >> w;
    if (w.empty()) return false;
    for (char c : w)
        if (!(std::isdigit((unsigned char)c) || c == '.')) return false;
    return true;
}

int Config::getString(const std::string& key, std::string& out) const {
    auto it = kv.find(key);
    if (it == kv.end()) return fail(RIFT_ERR_ARG, "config: missing key " + key);
    // string_to_T<std::string>: the first whitespace-separated word
    std::istringstream is(it->second);
    if (!(is >> out)) return fail(RIFT_ERR_ARG, "config: empty value for " + key);
    return RIFT_OK;
}

int Config::getDouble(const std::string& key, double& out) const {
    auto it = kv.find(key);
    if (it == kv.end()) return fail(RIFT_ERR_ARG, "config: missing key " + key);
    std::istringstream is(it->second);
    if (!(is >> out)) return fail(RIFT_ERR_ARG, "config: not a number: " + key);
    return RIFT_OK;
}

int Config::getInt(const std::string& key, int& out) const {
    auto it = kv.find(key);
    if (it == kv.end()) return fail(RIFT_ERR_ARG, "config: missing key " + key);
    std::istringstream is(it->second);
    if (!(is >> out)) return fail(RIFT_ERR_ARG, "config: not an integer: " + key);
    return RIFT_OK;
}

// operator>> of bool: "0" or "1"
int Config::getBool(const std::string& key, bool& out) const {
    auto it = kv.find(key);
    if (it == kv.end()) return fail(RIFT_ERR_ARG, "config: missing key " + key);
    std::istringstream is(it->second);
    if (!(is >> out)) return fail(RIFT_ERR_ARG, "config: not 0 or 1: " + key);
    return RIFT_OK;
}

// operator>> of std::complex<double>: "(re,im)", "(re)" or "re"
int Config::getComplex(const std::string& key, double& re, double& im) const {
    auto it = kv.find(key);
    if (it == kv.end()) return fail(RIFT_ERR_ARG, "config: missing key " + key);
    std::string v = it->second;
    re = im = 0.0;
    if (!v.empty() && v[0] == '(') {
        size_t close = v.find(')');
        if (close == std::string::npos) return fail(RIFT_ERR_ARG, "config: bad pair: " + key);
        std::string in = v.substr(1, close - 1);
        size_t comma = in.find(',');
        std::istringstream a(in.substr(0, comma));
        if (!(a >> re)) return fail(RIFT_ERR_ARG, "config: bad pair: " + key);
        if (comma != std::string::npos) {
            std::istringstream b(in.substr(comma + 1));
            if (!(b >> im)) return fail(RIFT_ERR_ARG, "config: bad pair: " + key);
        }
        return RIFT_OK;
    }
    std::istringstream a(v);
    if (!(a >> re)) return fail(RIFT_ERR_ARG, "config: bad pair: " + key);
    return RIFT_OK;
}

// -------------------------------------------------------------- rasters
namespace {
// Six (name, value) header pairs; the names are not checked (io.cc:44-67).
int readHeader(std::istream& is, const std::string& path, int& ncols, int& nrows, double& xll,
               double& yll, double& cell, double& nodata) {
    std::string name;
    if (!(is >> name >> ncols) || !(is >> name >> nrows) || !(is >> name >> xll) ||
        !(is >> name >> yll) || !(is >> name >> cell) || !(is >> name >> nodata))
        return fail(RIFT_ERR_ARG, path + ": bad ESRI header");
    if (ncols <= 0 || nrows <= 0) return fail(RIFT_ERR_ARG, path + ": bad raster size");
    return RIFT_OK;
}
}  // namespace

int readRaster(const std::string& path, int ncols, int nrows, bool nodataOk,
               std::vector<double>& out, RasterHeader* hdr) {
    std::ifstream is(path);
    if (!is) return fail(RIFT_ERR_ARG, path + ": cannot open");
    RasterHeader h;
    int rc = readHeader(is, path, h.ncols, h.nrows, h.xll, h.yll, h.cellsize, h.nodata);
    if (rc) return rc;
    if (hdr) *hdr = h;
    if (ncols > 0 && (h.ncols != ncols || h.nrows != nrows))
        return fail(RIFT_ERR_ARG, path + ": incorrect size: got (" + std::to_string(h.nrows) + "x" +
                                      std::to_string(h.ncols) + ") expected (" +
                                      std::to_string(nrows) + "x" + std::to_string(ncols) + ")");
    out.assign((size_t)h.ncols * h.nrows, 0.0);
    // the first line is the north row: it lands in row nrows-1 (io.cc:79-91)
    for (int j = h.nrows - 1; j >= 0; j--)
        for (int i = 0; i < h.ncols; i++) {
            double v;
            if (!(is >> v))
                return fail(RIFT_ERR_ARG, path + ": read error at line " +
                                              std::to_string(7 + (h.nrows - 1 - j)));
            if (v == h.nodata) {
                if (!nodataOk) return fail(RIFT_ERR_ARG, path + ": NODATA value(s) present");
                v = kNodata;
            }
            out[(size_t)j * h.ncols + i] = v;
        }
    return RIFT_OK;
}

// writeGrid (io.cc:331-361): header with 15 significant digits, then the
// interior rows from north to south, values separated by one blank.
int writeHGrid(const std::string& path, const double* x, const rift_gridconfig& gc) {
    FILE* f = std::fopen(path.c_str(), "w");
    if (!f) return fail(RIFT_ERR_ARG, path + ": error: cannot open for writing");
    std::fprintf(f, "ncols         %d\n", gc.h_nx - 4);
    std::fprintf(f, "nrows         %d\n", gc.h_ny - 4);
    std::fprintf(f, "xllcorner     %.15g\n", gc.h_xll);
    std::fprintf(f, "yllcorner     %.15g\n", gc.h_yll);
    std::fprintf(f, "cellsize      %.15g\n", gc.cellsize_original);
    std::fprintf(f, "NODATA_value  %.15g\n", kNodata);
    std::string line;
    char buf[40];
    for (int j = gc.h_ny - 3; j >= 2; j--) {
        line.clear();
        for (int i = 2; i < gc.h_nx - 2; i++) {
            std::snprintf(buf, sizeof(buf), "%.15g ", x[(size_t)j * gc.h_nx + i]);
            line += buf;
        }
        line += '\n';
        std::fputs(line.c_str(), f);
    }
    bool ok = std::ferror(f) == 0;
    ok = (std::fclose(f) == 0) && ok;
    return ok ? RIFT_OK : fail(RIFT_ERR_ARG, path + ": write failed");
}

// ----------------------------------------------------------- GridConfig
namespace {
double haversineKm(double lon1, double lat1, double lon2, double lat2) {
    const double R = 6372.8, d2r = M_PI / 180.0;
    double la1 = lat1 * d2r, la2 = lat2 * d2r, dla = la2 - la1, dlo = (lon2 - lon1) * d2r;
    double s = std::sin(dla / 2) * std::sin(dla / 2) +
               std::cos(la1) * std::cos(la2) * std::sin(dlo / 2) * std::sin(dlo / 2);
    return 2 * R * std::asin(std::sqrt(s));
}
}  // namespace

// ComputeCellSize (grid_config.cpp:67-88)
void computeCellSize(rift_gridconfig& gc) {
    if (!gc.projected) {
        gc.cellsize = gc.cellsize_original * 6378137.0 * M_PI / 180.0;
        if (gc.square_cells) {
            gc.h_dx = gc.cellsize_original * (double)6378137.f * (double)M_PI / (double)180.f;
            gc.h_dy = gc.h_dx;
        } else {
            double w = gc.b_nx * gc.cellsize_original, hgt = gc.b_ny * gc.cellsize_original;
            double xc = gc.h_xll + w / 2.0, xmax = gc.h_xll + w;
            double yc = gc.h_yll + hgt / 2.0, ymax = gc.h_yll + hgt;
            gc.h_dx = haversineKm(gc.h_xll, yc, xmax, yc) / gc.b_nx * 1000.0;
            gc.h_dy = haversineKm(xc, gc.h_yll, xc, ymax) / gc.b_ny * 1000.0;
        }
    } else {
        gc.cellsize = gc.cellsize_original;
        gc.h_dx = gc.cellsize;
        gc.h_dy = gc.cellsize;
    }
    gc.h_nx = gc.b_nx + 4 - 1;
    gc.h_ny = gc.b_ny + 4 - 1;
}

int gridConfigFromDem(const std::string& dem, bool square, bool projected, rift_gridconfig& gc,
                      std::vector<double>* data) {
    std::vector<double> tmp;
    RasterHeader h;
    int rc = readRaster(dem, 0, 0, false, data ? *data : tmp, &h);
    if (rc) return rc;
    std::memset(&gc, 0, sizeof(gc));
    gc.b_nx = h.ncols;
    gc.b_ny = h.nrows;
    gc.b_xll = h.xll;
    gc.b_yll = h.yll;
    gc.cellsize_original = h.cellsize;
    gc.h_xll = gc.b_xll + gc.cellsize_original / 2.0;
    gc.h_yll = gc.b_yll + gc.cellsize_original / 2.0;
    gc.square_cells = square ? 1 : 0;
    gc.projected = projected ? 1 : 0;
    computeCellSize(gc);
    return RIFT_OK;
}

// Coord2Index (grid_config.cpp:104-115), including its j-check on i
bool coord2Index(const rift_gridconfig& gc, double X, double Y, int& i, int& j) {
    bool ok = true;
    i = (int)((X - gc.h_xll) / gc.cellsize_original + 0.5);
    if (i < 2 || i > gc.h_nx - 2) ok = false;
    j = (int)((Y - gc.h_yll) / gc.cellsize_original + 0.5);
    if (j < 2 || i > gc.h_ny - 2) ok = false;
    return ok;
}

// ------------------------------------------------------------- CSV series
// Source::ReadSource (source.cc:11-63): float arithmetic throughout.
int readCsv(const std::string& path, std::vector<float>& t, std::vector<float>& r) {
    std::ifstream f(path);
    if (!f) return fail(RIFT_ERR_ARG, path + ": error: cannot open");
    t.clear();
    r.clear();
    std::string line;
    while (std::getline(f, line)) {
        if (!line.empty() && line[0] == '#') continue;
        std::stringstream ls(line);
        std::string field;
        int count = 0;
        float value = 0.f;
        while (std::getline(ls, field, ',')) {
            std::stringstream(field) >> value;  // a blank field keeps the last value
            if (count == 0)
                t.push_back(value * 60 * 60);
            else
                r.push_back(value);
            count++;
        }
    }
    if (r.empty() || t.empty()) return fail(RIFT_ERR_ARG, path + ": no data");
    if (r.back() != 0.f) {
        float est = 0.f;
        for (size_t i = 1; i < t.size(); i++) est += t[i] - t[i - 1];
        est /= (float)t.size() - 1;
        t.push_back(t.back() + est);
        r.push_back(0.f);
    }
    return RIFT_OK;
}

// ---------------------------------------------------------------- hotstart
int32_t growGridSize(int h_nx, int h_ny) {
    const int nBX = (h_nx + 15) / 16, nBY = (h_ny + 13) / 14;
    return ((nBX + 15) / 16 * 16) * ((nBY + 13) / 14 * 14);
}

int64_t hotstartSize(const rift_gridconfig& gc, bool hasF) {
    const int64_t N = (int64_t)gc.h_nx * gc.h_ny;
    return 98 + 8 * N * (hasF ? 4 : 3) + 5 * (int64_t)growGridSize(gc.h_nx, gc.h_ny);
}

namespace {
template <typename T>
void put(std::ofstream& o, const T& v) {
    o.write(reinterpret_cast<const char*>(&v), sizeof(T));
}
template <typename T>
bool get(std::ifstream& i, T& v) {
    return (bool)i.read(reinterpret_cast<char*>(&v), sizeof(T));
}
}  // namespace

// GridConfig::write (grid_config.cpp:124-143): native byte order, no padding
void writeGridConfig(std::ofstream& o, const rift_gridconfig& gc) {
    put(o, gc.b_nx);
    put(o, gc.b_ny);
    put(o, gc.b_xll);
    put(o, gc.b_yll);
    put(o, gc.cellsize_original);
    put(o, gc.h_nx);
    put(o, gc.h_ny);
    put(o, gc.h_xll);
    put(o, gc.h_yll);
    put(o, gc.cellsize);
    put(o, gc.h_dx);
    put(o, gc.h_dy);
    put(o, gc.square_cells);
    put(o, gc.projected);
}

bool readGridConfig(std::ifstream& i, rift_gridconfig& gc) {
    return get(i, gc.b_nx) && get(i, gc.b_ny) && get(i, gc.b_xll) && get(i, gc.b_yll) &&
           get(i, gc.cellsize_original) && get(i, gc.h_nx) && get(i, gc.h_ny) &&
           get(i, gc.h_xll) && get(i, gc.h_yll) && get(i, gc.cellsize) && get(i, gc.h_dx) &&
           get(i, gc.h_dy) && get(i, gc.square_cells) && get(i, gc.projected);
}

int writeHotstart(const std::string& path, double t, double dt, const rift_gridconfig& gc,
                  const double* w, const double* hu, const double* hv, const double* F,
                  const uint8_t* wet, const int32_t* active) {
    std::ofstream o(path, std::ios::binary);
    if (!o.good()) return fail(RIFT_ERR_ARG, "Cannot open hotstart file \"" + path + "\" for writing");
    put(o, t);
    put(o, dt);
    writeGridConfig(o, gc);
    const size_t N = (size_t)gc.h_nx * gc.h_ny;
    for (const double* p : {w, hu, hv, F})
        if (p) o.write(reinterpret_cast<const char*>(p), (std::streamsize)(N * sizeof(double)));
    const int32_t G = growGridSize(gc.h_nx, gc.h_ny);
    o.write(reinterpret_cast<const char*>(wet), G);
    o.write(reinterpret_cast<const char*>(active), (std::streamsize)G * 4);
    o.flush();
    const bool ok = (bool)o;
    o.close();
    return ok ? RIFT_OK : fail(RIFT_ERR_ARG, path + ": write failed");
}

int readHotstart(const std::string& path, double& t, double& dt, rift_gridconfig& gc, bool hasF,
                 double* w, double* hu, double* hv, double* F, uint8_t* wet, int32_t* active) {
    std::ifstream i(path, std::ios::binary | std::ios::in);
    if (!i.good()) return fail(RIFT_ERR_ARG, "Cannot open hotstart file \"" + path + "\" for reading");
    if (!get(i, t) || !get(i, dt) || !readGridConfig(i, gc))
        return fail(RIFT_ERR_ARG, path + ": truncated hotstart header");
    if (!w) return RIFT_OK;  // header only
    const size_t N = (size_t)gc.h_nx * gc.h_ny;
    for (double* p : {w, hu, hv, hasF ? F : (double*)nullptr})
        if (p && !i.read(reinterpret_cast<char*>(p), (std::streamsize)(N * sizeof(double))))
            return fail(RIFT_ERR_ARG, path + ": truncated hotstart fields");
    const int32_t G = growGridSize(gc.h_nx, gc.h_ny);
    if (!i.read(reinterpret_cast<char*>(wet), G) ||
        !i.read(reinterpret_cast<char*>(active), (std::streamsize)G * 4))
        return fail(RIFT_ERR_ARG, path + ": truncated hotstart tile arrays");
    return RIFT_OK;
}

}  // namespace rift_host

// ------------------------------------------------------------------ C ABI
using namespace rift_host;

struct rift_config {
    Config c;
};

extern "C" {

const char* rift_host_last_error(void) { return g_err.c_str(); }

int rift_config_open(const char* path, rift_config** out) {
    if (!path || !out) return RIFT_ERR_ARG;
    *out = nullptr;
    rift_config* c = new rift_config();
    int rc = c->c.open(path);
    if (rc) {
        delete c;
        return rc;
    }
    *out = c;
    return RIFT_OK;
}

int rift_config_has(const rift_config* c, const char* key) {
    return (c && key && c->c.has(key)) ? 1 : 0;
}

int rift_config_get(const rift_config* c, const char* key, char* buf, size_t cap) {
    if (!c || !key || !buf || cap == 0) return RIFT_ERR_ARG;
    auto it = c->c.kv.find(key);
    if (it == c->c.kv.end()) return fail(RIFT_ERR_ARG, std::string("config: missing key ") + key);
    if (it->second.size() + 1 > cap) return fail(RIFT_ERR_TOO_LARGE, "config: buffer too small");
    std::memcpy(buf, it->second.c_str(), it->second.size() + 1);
    return RIFT_OK;
}

int rift_config_is_number(const rift_config* c, const char* key) {
    return (c && key && c->c.isNumber(key)) ? 1 : 0;
}

int rift_config_get_double(const rift_config* c, const char* key, double* v) {
    if (!c || !key || !v) return RIFT_ERR_ARG;
    return c->c.getDouble(key, *v);
}

void rift_config_close(rift_config* c) { delete c; }

int rift_esri_read_header(const char* path, int32_t* ncols, int32_t* nrows, double* xll,
                          double* yll, double* cellsize, double* nodata) {
    if (!path) return RIFT_ERR_ARG;
    std::ifstream is(path);
    if (!is) return fail(RIFT_ERR_ARG, std::string(path) + ": cannot open");
    int nc, nr;
    double a, b, c, d;
    int rc = readHeader(is, path, nc, nr, a, b, c, d);
    if (rc) return rc;
    if (ncols) *ncols = nc;
    if (nrows) *nrows = nr;
    if (xll) *xll = a;
    if (yll) *yll = b;
    if (cellsize) *cellsize = c;
    if (nodata) *nodata = d;
    return RIFT_OK;
}

int rift_esri_read(const char* path, int32_t ncols, int32_t nrows, int32_t nodata_ok,
                   double* out) {
    if (!path || !out || ncols <= 0 || nrows <= 0) return RIFT_ERR_ARG;
    std::vector<double> v;
    int rc = readRaster(path, ncols, nrows, nodata_ok != 0, v, nullptr);
    if (rc) return rc;
    std::memcpy(out, v.data(), v.size() * sizeof(double));
    return RIFT_OK;
}

int rift_esri_write_hgrid(const char* path, const double* x, const rift_gridconfig* gc) {
    if (!path || !x || !gc) return RIFT_ERR_ARG;
    return writeHGrid(path, x, *gc);
}

int rift_gridconfig_from_dem(const char* dem_path, int32_t square_cells, int32_t projected,
                             rift_gridconfig* gc) {
    if (!dem_path || !gc) return RIFT_ERR_ARG;
    return gridConfigFromDem(dem_path, square_cells != 0, projected != 0, *gc, nullptr);
}

int rift_gridconfig_coord2index(const rift_gridconfig* gc, double X, double Y, int32_t* i,
                                int32_t* j, int32_t* ok) {
    if (!gc || !i || !j) return RIFT_ERR_ARG;
    int ii, jj;
    bool good = coord2Index(*gc, X, Y, ii, jj);
    *i = ii;
    *j = jj;
    if (ok) *ok = good ? 1 : 0;
    return RIFT_OK;
}

int rift_csv_read(const char* path, float* times_s, float* rates, int32_t cap, int32_t* n) {
    if (!path || !n) return RIFT_ERR_ARG;
    std::vector<float> t, r;
    int rc = readCsv(path, t, r);
    if (rc) return rc;
    const size_t m = std::min(t.size(), r.size());
    *n = (int32_t)m;
    if (times_s && rates) {
        if ((int64_t)m > cap) return fail(RIFT_ERR_TOO_LARGE, "csv: more rows than capacity");
        std::memcpy(times_s, t.data(), m * sizeof(float));
        std::memcpy(rates, r.data(), m * sizeof(float));
    }
    return RIFT_OK;
}

int64_t rift_hotstart_size(const rift_gridconfig* gc, int32_t has_F) {
    return gc ? hotstartSize(*gc, has_F != 0) : -1;
}

int rift_hotstart_write(const char* path, double t, double dt, const rift_gridconfig* gc,
                        const double* w, const double* hu, const double* hv, const double* F,
                        const uint8_t* wet_blocks, const int32_t* active_blocks) {
    if (!path || !gc || !w || !hu || !hv || !wet_blocks || !active_blocks) return RIFT_ERR_ARG;
    return writeHotstart(path, t, dt, *gc, w, hu, hv, F, wet_blocks, active_blocks);
}

int rift_hotstart_read(const char* path, double* t, double* dt, rift_gridconfig* gc,
                       int32_t has_F, double* w, double* hu, double* hv, double* F,
                       uint8_t* wet_blocks, int32_t* active_blocks) {
    if (!path || !t || !dt || !gc) return RIFT_ERR_ARG;
    if (w && (!hu || !hv || !wet_blocks || !active_blocks || (has_F && !F))) return RIFT_ERR_ARG;
    return readHotstart(path, *t, *dt, *gc, has_F != 0, w, hu, hv, F, wet_blocks, active_blocks);
}

int32_t rift_grow_grid_size(int32_t h_nx, int32_t h_ny) { return growGridSize(h_nx, h_ny); }

}  // extern "C"
