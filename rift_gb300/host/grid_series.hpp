// grid_series.hpp -- host map series (GridSeries.cu) feeding the engine.
#pragma once
#include <string>
#include <vector>

#include "host_internal.hpp"

namespace rift_host {

class MapSeries {
public:
    // Hold: HyetographGridSeries (map k on [(k-1)dt, k dt), zeros after
    // tmax).  Interp: InterpolatedGridSeries (linear between maps
    // trunc(t/dt) and +1, the last map held after tmax).
    enum class Kind { Hold, Interp };

    MapSeries(Kind kind, const std::string& prefix, double scale, double deltat, double tmax,
              const rift_gridconfig& gc, bool allowNodata, int which);

    // Advance to time t; uploads to the engine slot when a new map is due.
    int update(double t, rift_handle* R);
    // Earliest t at which update() changes the maps (infinity when done).
    double nextEvent() const;
    // prefix-%03d.txt (GridSeries::p_grid_name)
    std::string fileName(int index) const;

private:
    int readMap(int index, std::vector<double>& out);
    int upload(rift_handle* R);

    Kind kind_;
    std::string prefix_;
    double scale_, dt_, tmax_;
    rift_gridconfig gc_;
    bool allowNodata_;
    int which_;
    double inTime_ = -9999.0, nextTime_ = 0.0;
    bool done_ = false;
    std::vector<double> cur_, t0_, t1_;
};

}  // namespace rift_host
