// grid_series.cpp -- gridded rain / drain / surge map series on the host
// (GridSeries, HyetographGridSeries, InterpolatedGridSeries,
// GridSeries.cu:91-403), feeding the engine's map slots.
//
// The engine evaluates a map at every cell of every step (hold: the map;
// interpolated: factor * (m1 - m0) + m0 with the reference's nodata rules,
// the factor following t between the two map times).  This class keeps the
// reference's file sequence and timing and uploads a map pair only when the
// reference would read a new file; nextEvent() is the next time at which
// that happens, so the host can run all steps up to it in one engine call.
#include <cmath>
#include <cstdio>
#include <limits>

#include "grid_series.hpp"

namespace rift_host {

MapSeries::MapSeries(Kind kind, const std::string& prefix, double scale, double deltat,
                     double tmax, const rift_gridconfig& gc, bool allowNodata, int which)
    : kind_(kind),
      prefix_(prefix),
      scale_(scale),
      // GridSeries takes the interval as `const int&` (GridSeries.cuh:29)
      dt_((double)(int)deltat),
      tmax_(tmax),
      gc_(gc),
      allowNodata_(allowNodata),
      which_(which) {
    const size_t N = (size_t)gc.h_nx * gc.h_ny;
    const double fill = allowNodata_ ? kNodata : 0.0;
    cur_.assign(N, fill);
    t0_.assign(N, fill);
    t1_.assign(N, fill);
}

// p_grid_name: prefix-%03d.txt
std::string MapSeries::fileName(int index) const {
    char buf[32];
    std::snprintf(buf, sizeof(buf), "-%03d.txt", index);
    return prefix_ + buf;
}

// p_read_grid + p_interp: corner map -> cell means over the corners that are
// not nodata, kept only where at least 3 are, times the scale.
int MapSeries::readMap(int index, std::vector<double>& out) {
    std::vector<double> corners;
    int rc = readRaster(fileName(index), gc_.b_nx, gc_.b_ny, allowNodata_, corners, nullptr);
    if (rc) return rc;
    out.assign((size_t)gc_.h_nx * gc_.h_ny, allowNodata_ ? kNodata : 0.0);
    for (int j = 2; j < gc_.h_ny - 2; j++)
        for (int i = 2; i < gc_.h_nx - 2; i++) {
            const int jt = j - 2, it = i - 2;
            int nnd = 0;
            double vsum = 0.0;
            for (int ni = 0; ni < 2; ++ni)
                for (int nj = 0; nj < 2; ++nj) {
                    const double v = corners[(size_t)(jt + nj) * gc_.b_nx + (it + ni)];
                    if (v != kNodata) {
                        nnd++;
                        vsum += v;
                    }
                }
            if (nnd > 2) {
                double m = vsum / (double)nnd;
                m *= scale_;
                out[(size_t)j * gc_.h_nx + i] = m;
            }
        }
    return RIFT_OK;
}

int MapSeries::upload(rift_handle* R) {
    int rc;
    if (kind_ == Kind::Hold) {
        rc = rift_set_map(R, which_, cur_.data(), nullptr, 0.0);
    } else {
        rc = rift_set_map(R, which_, t0_.data(), t1_.data(), 0.0);
        if (!rc) rc = rift_set_map_times(R, which_, inTime_, nextTime_);
    }
    if (rc) return fail(rc, std::string("engine map upload: ") + rift_last_error(R));
    return RIFT_OK;
}

// The reference calls update(t) at t0 and after every step.
int MapSeries::update(double t, rift_handle* R) {
    int rc;
    bool changed = false;
    if (kind_ == Kind::Hold) {
        // HyetographGridSeries::p_update (GridSeries.cu:261-293)
        if (inTime_ < 0.0) {
            inTime_ = t;  // GridSeries::p_update's first call reads map trunc(t/dt)...
            if (inTime_ < tmax_) {
                std::vector<double> first;
                if ((rc = readMap((int)std::trunc(inTime_ / dt_), first))) return rc;
                cur_ = first;
                changed = true;
            }
        }
        if (t >= tmax_) {
            if (!done_) {
                std::fill(cur_.begin(), cur_.end(), 0.0);
                changed = true;
            }
            done_ = true;
        } else if (t >= inTime_) {  // ...and the next map replaces it at once
            inTime_ += dt_;
            if ((rc = readMap((int)std::trunc(inTime_ / dt_), cur_))) return rc;
            changed = true;
        }
    } else {
        // InterpolatedGridSeries::p_update (GridSeries.cu:335-375)
        if (inTime_ < 0.0) {
            inTime_ = t;
            const int index = (int)std::trunc(inTime_ / dt_);
            if ((rc = readMap(index, t0_))) return rc;
            inTime_ = index * dt_;
            nextTime_ = inTime_ + dt_;
            if ((rc = readMap(index + 1, t1_))) return rc;
            changed = true;
        } else if (t >= tmax_) {
            if (!done_) {
                inTime_ = nextTime_;
                nextTime_ = inTime_ + dt_;
                t0_ = t1_;
                changed = true;
            }
            done_ = true;
        } else if (t >= nextTime_) {
            t0_ = t1_;
            inTime_ = nextTime_;
            nextTime_ = inTime_ + dt_;
            if ((rc = readMap((int)std::trunc(nextTime_ / dt_), t1_))) return rc;
            changed = true;
        }
    }
    if (changed && R) return upload(R);
    return RIFT_OK;
}

// Earliest t at which update() changes the maps.
double MapSeries::nextEvent() const {
    const double inf = std::numeric_limits<double>::infinity();
    if (done_) return inf;
    if (kind_ == Kind::Hold) return std::min(inTime_, tmax_);
    return std::min(nextTime_, tmax_);
}

}  // namespace rift_host
