// host_internal.hpp -- C++ pieces of the host drop-in layer shared by its
// translation units (host_io.cpp, grid_series.cpp, simulator.cpp).
#pragma once
#include <cstdint>
#include <fstream>
#include <map>
#include <string>
#include <vector>

#include "../../include/rift_host.h"

namespace rift_host {

constexpr double kNodata = -9999.0;  // GridConfig::nodata (grid_config.cpp:15)

int fail(int code, const std::string& msg);
extern thread_local std::string g_err;

struct Config {
    std::map<std::string, std::string> kv;
    int open(const std::string& path);
    bool has(const std::string& key) const;
    bool isNumber(const std::string& key) const;
    int getString(const std::string& key, std::string& out) const;
    int getDouble(const std::string& key, double& out) const;
    int getInt(const std::string& key, int& out) const;
    int getBool(const std::string& key, bool& out) const;
    int getComplex(const std::string& key, double& re, double& im) const;
};

struct RasterHeader {
    int ncols = 0, nrows = 0;
    double xll = 0, yll = 0, cellsize = 0, nodata = 0;
};

// ncols/nrows 0: any size (the header's)
int readRaster(const std::string& path, int ncols, int nrows, bool nodataOk,
               std::vector<double>& out, RasterHeader* hdr);
int writeHGrid(const std::string& path, const double* x, const rift_gridconfig& gc);
void computeCellSize(rift_gridconfig& gc);
int gridConfigFromDem(const std::string& dem, bool square, bool projected, rift_gridconfig& gc,
                      std::vector<double>* data);
bool coord2Index(const rift_gridconfig& gc, double X, double Y, int& i, int& j);
int readCsv(const std::string& path, std::vector<float>& t, std::vector<float>& r);
int32_t growGridSize(int h_nx, int h_ny);
int64_t hotstartSize(const rift_gridconfig& gc, bool hasF);
int writeHotstart(const std::string& path, double t, double dt, const rift_gridconfig& gc,
                  const double* w, const double* hu, const double* hv, const double* F,
                  const uint8_t* wet, const int32_t* active);
int readHotstart(const std::string& path, double& t, double& dt, rift_gridconfig& gc, bool hasF,
                 double* w, double* hu, double* hv, double* F, uint8_t* wet, int32_t* active);

}  // namespace rift_host
