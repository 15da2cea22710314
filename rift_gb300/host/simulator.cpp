// simulator.cpp -- the reference's Simulator life cycle (simulator.h:14-181,
// simulator.cu) on the GB300 engine: keyword=value parameters, ESRI / CSV
// inputs, gridded map series, outputs and hot<k>.bin restarts, with every
// device step going through the engine's C ABI (include/rift_gb300.h).
//
// The reference's per-step host work -- UpdateSource, the thrust reductions
// of ComputeTimestep, the D2H of dt -- runs on the device in the engine, so
// a run between two host events (an output time, a map switch, tf) is one
// engine call; the events fire at the same steps as in RunSimulation.
#include <algorithm>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdio>
#include <limits>
#include <memory>
#include <string>
#include <vector>

#include "../../include/rift_host.h"
#include "grid_series.hpp"
#include "host_internal.hpp"

namespace rift_host {

struct Simulator {
    // ---- user parameters (Simulator::ReadUserParams, simulator.cu:25-265)
    std::string DEM_file, output_file = "./", n_file, K_file, h_file, hydrograph_file;
    std::string hyetograph_file, drain_file, hyetograph_prefix, drain_prefix, surge_prefix;
    std::string read_hotstart;
    double t0 = 0.0, tf = 0.0, t = 0.0, dt = (double)0.0000001f, courant_max = 0.25;
    double n_const = 0.0, psi = 0.0, dtheta = 0.0, kappa = 0.0;
    double t_print = 0.0, dt_print = 0.0;
    double hyetograph_dt = 0.0, hyetograph_tf = 0.0, drain_dt = 0.0, drain_tf = 0.0;
    double surge_dt = 0.0, surge_tf = 0.0;
    bool euler_integration = false, n_gridded = false, infiltration = false, h_init = false;
    bool dambreak = false, rainfall_averaged = false, drain_averaged = false;
    bool rainfall_gridded = false, hyetograph_interp = false, drain_gridded = false;
    bool surge_gridded = false, h_print = false, ws_print = false, q_print = false;
    bool save_max = false, save_arrival_time = false, check_volume = false;
    bool save_hotstart = false, b_print = false, n_print = false, tile_acceleration = true;
    bool square_cells = true, projected = false;
    double source_X[2] = {0, 0}, source_Y[2] = {0, 0};  // (real, imag) of std::complex
    bool coupled_source = false;      // source cells whose rate the caller sets
    double flow_rate = 0.0;           // OpenSimulation's flowrate argument
    std::vector<double> source_rate;  // m/s per source cell (setSourceValue)
    double V_added = 0.0;             // setSourceValue's check_volume bookkeeping
    int device = 0, count_print = 0;
    long long count = 0;
    std::vector<float> hyeT, hyeR, drnT, drnR, hydT, hydR;

    // ---- grid and engine
    rift_gridconfig gc{};
    std::vector<double> BC, h_n;
    std::vector<int32_t> source_idx;
    rift_handle* R = nullptr;
    std::unique_ptr<MapSeries> rainS, drainS, surgeS;
    std::chrono::steady_clock::time_point start;
    std::string err;

    ~Simulator() {
        if (R) rift_destroy(R);
    }
    bool printing() const { return h_print || q_print || ws_print || check_volume; }
    size_t N() const { return (size_t)gc.h_nx * gc.h_ny; }
    int engineFail(int rc, const char* what) {
        return fail(rc, std::string(what) + ": " + (R ? rift_last_error(R) : ""));
    }

    int readUserParams(const std::string& path);
    int initSimulation();
    int openSimulation(const std::string& path);
    void setSourceValue(double value);
    int updateSources();
    int events();
    int runSimulation();
    int run(double tEnd, long long* steps);
    int printData();
    int printSummaryData();
    int writeHotstart();
    int readHotstart(const std::string& path);
    int closeSimulation();
    int getField(int which, std::vector<double>& out);
    int writeMap(const std::string& name, const std::vector<double>& x);
};

// ------------------------------------------------------- ReadUserParams
int Simulator::readUserParams(const std::string& path) {
    Config cfg;
    int rc;
    if ((rc = cfg.open(path))) return rc;
    if ((rc = cfg.getString("DEM", DEM_file)) || (rc = cfg.getDouble("t0", t0)) ||
        (rc = cfg.getDouble("tf", tf)))
        return rc;
    t = t0;
    dt = (double)0.0000001f;
    if (cfg.has("euler_integration") && (rc = cfg.getBool("euler_integration", euler_integration)))
        return rc;
    if (cfg.has("output") && (rc = cfg.getString("output", output_file))) return rc;
    n_gridded = false;
    n_const = 0.0;
    if (cfg.has("n")) {
        // keyIsNumber accepts only digits and '.': "-0.03" or "3e-2" name a file
        if (cfg.isNumber("n")) {
            if ((rc = cfg.getDouble("n", n_const))) return rc;
        } else {
            n_gridded = true;
            if ((rc = cfg.getString("n", n_file))) return rc;
        }
    }
    courant_max = 0.25;
    if (cfg.has("courant_limit")) {
        if ((rc = cfg.getDouble("courant_limit", courant_max))) return rc;
        if (courant_max <= 0 || courant_max >= 1.0) {
            std::fprintf(stderr, "Specified courant_limit (%g) is out of range, reverting to default\n",
                         courant_max);
            courant_max = 0.25;
        }
    }
    infiltration = cfg.has("K");
    if (infiltration && ((rc = cfg.getString("K", K_file)) || (rc = cfg.getDouble("psi", psi)) ||
                         (rc = cfg.getDouble("dtheta", dtheta))))
        return rc;
    h_init = cfg.has("h0");
    if (h_init && (rc = cfg.getString("h0", h_file))) return rc;
    dambreak = cfg.has("hydrograph");
    // A source location without a hydrograph CSV: the source of a 1D-2D
    // coupling, whose rate the caller sets (setSourceValue / updateSources).
    // The reference reads the location only with a hydrograph and would leave
    // such a source without cells.
    coupled_source = !dambreak && (cfg.has("source_rect_X") || cfg.has("source_pt") ||
                                   (cfg.has("source_X") && cfg.has("source_Y")));
    if (dambreak && ((rc = cfg.getString("hydrograph", hydrograph_file)) ||
                     (rc = readCsv(hydrograph_file, hydT, hydR))))
        return rc;
    if (dambreak || coupled_source) {
        if (cfg.has("source_rect_X")) {
            if ((rc = cfg.getComplex("source_rect_X", source_X[0], source_X[1])) ||
                (rc = cfg.getComplex("source_rect_Y", source_Y[0], source_Y[1])))
                return rc;
        } else if (cfg.has("source_pt")) {
            double x, y;
            if ((rc = cfg.getComplex("source_pt", x, y))) return rc;
            source_X[0] = source_X[1] = x;
            source_Y[0] = source_Y[1] = y;
        } else {
            double x, y;
            if ((rc = cfg.getDouble("source_X", x)) || (rc = cfg.getDouble("source_Y", y))) return rc;
            source_X[0] = source_X[1] = x;
            source_Y[0] = source_Y[1] = y;
        }
    }
    rainfall_averaged = cfg.has("hyetograph");
    if (rainfall_averaged && ((rc = cfg.getString("hyetograph", hyetograph_file)) ||
                              (rc = readCsv(hyetograph_file, hyeT, hyeR))))
        return rc;
    rainfall_gridded = cfg.has("hyetograph_prefix");
    if (rainfall_gridded) {
        if ((rc = cfg.getString("hyetograph_prefix", hyetograph_prefix))) return rc;
        hyetograph_interp = false;
        if (cfg.has("hyetograph_interp") && (rc = cfg.getBool("hyetograph_interp", hyetograph_interp)))
            return rc;
        if ((rc = cfg.getDouble("hyetograph_dt", hyetograph_dt)) ||
            (rc = cfg.getDouble("hyetograph_tf", hyetograph_tf)))
            return rc;
    }
    drain_averaged = cfg.has("drain");
    if (drain_averaged &&
        ((rc = cfg.getString("drain", drain_file)) || (rc = readCsv(drain_file, drnT, drnR))))
        return rc;
    drain_gridded = cfg.has("drain_prefix");
    if (drain_gridded && ((rc = cfg.getString("drain_prefix", drain_prefix)) ||
                          (rc = cfg.getDouble("drain_dt", drain_dt)) ||
                          (rc = cfg.getDouble("drain_tf", drain_tf))))
        return rc;
    surge_gridded = cfg.has("surge_prefix");
    if (surge_gridded && ((rc = cfg.getString("surge_prefix", surge_prefix)) ||
                          (rc = cfg.getDouble("surge_dt", surge_dt)) ||
                          (rc = cfg.getDouble("surge_tf", surge_tf))))
        return rc;
    struct {
        const char* key;
        bool* v;
    } flags[] = {{"h_print", &h_print},         {"ws_print", &ws_print},
                 {"save_max", &save_max},       {"save_arrival", &save_arrival_time},
                 {"q_print", &q_print},         {"check_volume", &check_volume},
                 {"save_hotstart", &save_hotstart}};
    for (auto& f : flags) {
        *f.v = false;
        if (cfg.has(f.key) && (rc = cfg.getBool(f.key, *f.v))) return rc;
    }
    read_hotstart.clear();
    if (cfg.has("read_hotstart") && (rc = cfg.getString("read_hotstart", read_hotstart))) return rc;
    if (h_print || q_print || ws_print || check_volume || save_hotstart) {
        t_print = t0;
        if ((rc = cfg.getDouble("dt_print", dt_print))) return rc;
        count_print = 0;
    }
    b_print = cfg.has("b_print");  // enabled by the key's presence
    n_print = cfg.has("n_print");
    device = 0;
    if (cfg.has("device") && (rc = cfg.getInt("device", device))) return rc;
    square_cells = true;
    if (cfg.has("square_cells") && (rc = cfg.getBool("square_cells", square_cells))) return rc;
    projected = false;
    if (cfg.has("projected") && (rc = cfg.getBool("projected", projected))) return rc;
    tile_acceleration = true;
    if (cfg.has("tile_acceleration") && (rc = cfg.getBool("tile_acceleration", tile_acceleration)))
        return rc;
    return RIFT_OK;
}

// ------------------------------------------------------- InitSimulation
int Simulator::initSimulation() {
    int rc;
    std::vector<double> B;  // raw corner DEM (ReadGrid; the min-shifted copy is unused)
    if ((rc = gridConfigFromDem(DEM_file, square_cells, projected, gc, &B))) return rc;
    const int h_nx = gc.h_nx, h_ny = gc.h_ny, b_nx = gc.b_nx, b_ny = gc.b_ny;
    // simulator.cu:281, in float
    kappa = (double)sqrtf(0.01f * fmaxf(1.f, fminf((float)gc.h_dx, (float)gc.h_dy)));

    std::vector<double> h_o, n_o, K_o;
    if (h_init && (rc = readRaster(h_file, b_nx, b_ny, false, h_o, nullptr))) return rc;
    if (n_gridded && (rc = readRaster(n_file, b_nx, b_ny, false, n_o, nullptr))) return rc;
    if (infiltration && (rc = readRaster(K_file, b_nx, b_ny, false, K_o, nullptr))) return rc;

    // InitializeSources (simulator.cu:858-885): Coord2Index, whose cell is
    // 2 cells west / south of the coordinate; its ok flag is not checked
    source_idx.clear();
    if (dambreak || coupled_source) {
        int imin, jmin, imax, jmax;
        coord2Index(gc, source_X[0], source_Y[0], imin, jmin);
        coord2Index(gc, source_X[1], source_Y[1], imax, jmax);
        for (int i = imin; i <= imax; ++i)
            for (int j = jmin; j <= jmax; ++j) source_idx.push_back(j * h_nx + i);
        for (int32_t idx : source_idx)
            if (idx < 0 || idx >= h_nx * h_ny)
                return fail(RIFT_ERR_ARG, "source location outside the grid");
    }

    // faces and cell fields (simulator.cu:384-431)
    std::vector<double> BX((size_t)h_ny * (h_nx + 1), 0.0), BY((size_t)(h_ny + 1) * h_nx, 0.0);
    std::vector<double> h_h(N(), 0.0), h_K(N(), 0.0);
    h_n.assign(N(), 0.0);
    for (int j = 2; j < h_ny - 2; j++)
        for (int i = 2; i < h_nx - 2; i++) {
            const int jt = j - 2, it = i - 2;
            const size_t bed = (size_t)j * (h_nx + 1) + i + 1, bwd = (size_t)j * (h_nx + 1) + i;
            const size_t bnd = (size_t)(j + 1) * h_nx + i, bsd = (size_t)j * h_nx + i;
            const size_t ll = (size_t)jt * b_nx + it, ul = (size_t)(jt + 1) * b_nx + it;
            const size_t ur = (size_t)(jt + 1) * b_nx + it + 1, lr = (size_t)jt * b_nx + it + 1;
            BX[bed] = 0.5 * (B[ur] + B[lr]);
            BX[bwd] = 0.5 * (B[ll] + B[ul]);
            BY[bnd] = 0.5 * (B[ul] + B[ur]);
            BY[bsd] = 0.5 * (B[ll] + B[lr]);
            if (i == 2) {
                BX[(size_t)j * (h_nx + 1) + (i - 1)] = BX[bed];
                BX[(size_t)j * (h_nx + 1) + (i - 2)] = BX[bwd];
            }
            if (i == h_nx - 3) BX[(size_t)j * (h_nx + 1) + (i + 2)] = BX[bwd];
            if (j == 2) {
                BY[(size_t)(j - 1) * h_nx + i] = BY[bnd];
                BY[(size_t)(j - 2) * h_nx + i] = BY[bsd];
            }
            if (j == h_ny - 3) BY[(size_t)(j + 2) * h_nx + i] = BY[bsd];
            const size_t c = (size_t)j * h_nx + i;
            if (h_init) h_h[c] = 0.25 * (h_o[ur] + h_o[lr] + h_o[ll] + h_o[ul]);
            h_n[c] = n_gridded ? 0.25 * (n_o[ur] + n_o[lr] + n_o[ll] + n_o[ul]) : n_const;
            if (infiltration) {
                h_K[c] = 0.25 * (K_o[ur] + K_o[lr] + K_o[ll] + K_o[ul]);
                h_K[c] /= (double)(3600.f * 1000.f);
            }
        }

    rift_grid_desc g{};
    g.h_nx = h_nx;
    g.h_ny = h_ny;
    g.dx = gc.h_dx;
    g.dy = gc.h_dy;
    g.kappa = kappa;
    g.nodata = kNodata;
    g.courant = courant_max;
    g.psi = psi;
    g.dtheta = dtheta;
    g.flags = (rainfall_averaged ? RIFT_F_RAIN_UNIFORM : 0) | (rainfall_gridded ? RIFT_F_RAIN_GRID : 0) |
              (drain_averaged ? RIFT_F_DRAIN_UNIFORM : 0) | (drain_gridded ? RIFT_F_DRAIN_GRID : 0) |
              (infiltration ? RIFT_F_INFILTRATION : 0) | (surge_gridded ? RIFT_F_SURGE_GRID : 0) |
              (euler_integration ? RIFT_F_EULER : 0) | (save_max ? RIFT_F_SAVE_MAX : 0) |
              (save_arrival_time ? RIFT_F_SAVE_ARRIVAL : 0) |
              (tile_acceleration ? RIFT_F_TILE_ACCEL : 0) |
              ((dambreak || coupled_source) ? RIFT_F_POINT_SOURCE : 0) |
              (h_init ? RIFT_F_H_INIT : 0) | (check_volume ? RIFT_F_CHECK_VOLUME : 0);
    g.device = device;
    if ((rc = rift_create(&g, &R))) return engineFail(rc, "rift_create");
    if ((rc = rift_upload_static(R, BX.data(), BY.data(), h_n.data(),
                                 infiltration ? h_K.data() : nullptr, h_init ? h_h.data() : nullptr)))
        return engineFail(rc, "rift_upload_static");
    if (rainfall_averaged &&
        (rc = rift_set_series(R, 0, hyeT.data(), hyeR.data(), (int32_t)hyeT.size())))
        return engineFail(rc, "hyetograph");
    if (drain_averaged && (rc = rift_set_series(R, 1, drnT.data(), drnR.data(), (int32_t)drnT.size())))
        return engineFail(rc, "drain");
    source_rate.assign(source_idx.size(), 0.0);
    if (dambreak || coupled_source) {
        if ((rc = rift_set_point_sources(R, source_idx.data(), source_rate.data(),
                                         (int32_t)source_idx.size())) ||
            (dambreak && (rc = rift_set_series(R, 2, hydT.data(), hydR.data(), (int32_t)hydT.size()))))
            return engineFail(rc, "point sources");
    }
    // gridded series at t0 (simulator.cu:329-365)
    const double rainScale = 1.0 / 3600.0 / 1000.0;
    if (rainfall_gridded)
        rainS.reset(new MapSeries(hyetograph_interp ? MapSeries::Kind::Interp : MapSeries::Kind::Hold,
                                  hyetograph_prefix, rainScale, hyetograph_dt, hyetograph_tf, gc,
                                  false, RIFT_MAP_RAIN));
    if (drain_gridded)
        drainS.reset(new MapSeries(MapSeries::Kind::Hold, drain_prefix, rainScale, drain_dt, drain_tf,
                                   gc, false, RIFT_MAP_DRAIN));
    if (surge_gridded)
        surgeS.reset(new MapSeries(MapSeries::Kind::Interp, surge_prefix, 1.0, surge_dt, surge_tf, gc,
                                   true, RIFT_MAP_SURGE));
    for (MapSeries* s : {rainS.get(), drainS.get(), surgeS.get()})
        if (s && (rc = s->update(t0, R))) return rc;
    if ((rc = rift_init(R, t0))) return engineFail(rc, "rift_init");
    if (b_print || ws_print) {
        if ((rc = getField(RIFT_FIELD_BC, BC))) return rc;
        if (b_print && (rc = writeMap("bc.txt", BC))) return rc;
    }
    if (n_print && (rc = writeMap("n.txt", h_n))) return rc;
    return RIFT_OK;
}

int Simulator::getField(int which, std::vector<double>& out) {
    out.assign(N(), 0.0);
    int rc = rift_get_field(R, which, out.data(), (size_t)gc.h_nx);
    return rc ? engineFail(rc, "rift_get_field") : RIFT_OK;
}

int Simulator::writeMap(const std::string& name, const std::vector<double>& x) {
    return writeHGrid(output_file + "/" + name, x.data(), gc);
}

// ------------------------------------------------------- OpenSimulation
int Simulator::openSimulation(const std::string& path) {
    int rc;
    if ((rc = readUserParams(path)) || (rc = initSimulation())) return rc;
    if (!read_hotstart.empty() && (rc = readHotstart(read_hotstart))) return rc;
    count = 0;
    start = std::chrono::steady_clock::now();
    return RIFT_OK;
}

// Simulator::setSourceValue (simulator.cu:891-901): a discharge in m^3/s
// spread over the source cells, as m/s of depth per cell; with check_volume
// each cell's rate times the current dt is added to V_added.
void Simulator::setSourceValue(double value) {
    const size_t n = source_idx.size();
    for (size_t k = 0; k < n; k++) {
        source_rate[k] = value / gc.h_dx / gc.h_dy / (double)n;
        if (check_volume) V_added += source_rate[k] * dt;
    }
}

// Simulator::updateSources (simulator.cu:903-907): the rates to the device.
int Simulator::updateSources() {
    int rc = rift_set_point_rates(R, source_rate.data(), (int32_t)source_rate.size());
    return rc ? engineFail(rc, "updateSources") : RIFT_OK;
}

// The host part of RunSimulation after a step (simulator.cu:819-849): map
// series to the new t, then the outputs once t passes t_print.
int Simulator::events() {
    int rc;
    for (MapSeries* s : {rainS.get(), drainS.get(), surgeS.get()})
        if (s && (rc = s->update(t, R))) return rc;
    if (printing() && t > t_print) {
        if ((rc = printData())) return rc;
        t_print += dt_print;
        const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - start).count();
        std::printf("%.17g\t%.17g", t, dt);
        if (check_volume) {
            double V = 0.0, added = 0.0;
            if ((rc = rift_mass_ledger(R, &V, &added))) return engineFail(rc, "rift_mass_ledger");
            const double cells = (double)(gc.h_nx - 4) * (gc.h_ny - 4) * (double)count;
            std::printf("\t%.17g\t%.17g\t%.17g\t%d\t%.6g\t%.6g", added * gc.h_dx * gc.h_dy,
                        V * gc.h_dx * gc.h_dy, added != 0.0 ? (V - added) / added : 0.0,
                        gc.b_nx * gc.b_ny, el, el > 0 ? cells / el / 1e6 : 0.0);
        }
        std::printf("\n");
        std::fflush(stdout);
    }
    return RIFT_OK;
}

// RunSimulation: one step and its host events.
int Simulator::runSimulation() {
    int rc = rift_step(R, &t, &dt);
    if (rc) return engineFail(rc, "rift_step");
    count++;
    return events();
}

// RunSimulation until t >= min(tEnd, tf): the steps between two host events
// run in one engine call that stops at the first step reaching the event
// time, where RunSimulation would act.
int Simulator::run(double tEnd, long long* steps) {
    const double inf = std::numeric_limits<double>::infinity();
    const double stop = std::min(tEnd, tf);
    long long done = 0;
    int rc;
    while (t < stop) {
        double next = stop;
        for (MapSeries* s : {rainS.get(), drainS.get(), surgeS.get()})
            if (s) next = std::min(next, s->nextEvent());
        if (printing()) next = std::min(next, t_print);
        int32_t ran = 0;
        if (next > t)
            rc = rift_run(R, INT_MAX, next, &t, &dt, &ran);
        else  // the event needs t strictly past its time: one more step
            rc = rift_run(R, 1, inf, &t, &dt, &ran);
        if (rc) return engineFail(rc, "rift_run");
        if (ran == 0) break;
        done += ran;
        count += ran;
        if ((rc = events())) return rc;
    }
    if (steps) *steps = done;
    return RIFT_OK;
}

// ---------------------------------------------------------- outputs
int Simulator::printData() {
    int rc;
    std::vector<double> h;
    if ((h_print || ws_print) && (rc = getField(RIFT_FIELD_H, h))) return rc;
    if (save_max && (rc = printSummaryData())) return rc;
    const std::string k = std::to_string(count_print);
    if (h_print && (rc = writeMap("h" + k + ".txt", h))) return rc;
    if (ws_print) {
        std::vector<double> ws(N());
        for (size_t c = 0; c < N(); c++) ws[c] = h[c] > 0.0 ? h[c] + BC[c] : kNodata;
        if ((rc = writeMap("ws" + k + ".txt", ws))) return rc;
    }
    if (save_hotstart && (rc = writeHotstart())) return rc;
    if (q_print) {
        std::vector<double> q;
        if ((rc = getField(RIFT_FIELD_Q, q)) || (rc = writeMap("q" + k + ".txt", q))) return rc;
    }
    count_print++;
    return RIFT_OK;
}

int Simulator::printSummaryData() {
    int rc;
    std::vector<double> x;
    if (save_max) {
        const struct {
            int field;
            const char* name;
        } maps[] = {{RIFT_FIELD_HMAX, "peak_flood_depth.txt"},
                    {RIFT_FIELD_QMAX, "peak_unit_flow.txt"},
                    {RIFT_FIELD_TPEAK, "time_to_peak.txt"},
                    {RIFT_FIELD_TDRY, "time_to_dry.txt"}};
        for (auto& m : maps)
            if ((rc = getField(m.field, x)) || (rc = writeMap(m.name, x))) return rc;
    }
    if (save_arrival_time &&
        ((rc = getField(RIFT_FIELD_TWET, x)) || (rc = writeMap("flood_wave_arrival.txt", x))))
        return rc;
    return RIFT_OK;
}

// WriteHotstart (simulator.cu:912-968).  F is written only with
// infiltration (the reference writes it whenever its F pointer is set,
// which it leaves uninitialised otherwise).  active_blocks: active ids
// ascending, then the inactive ones as -id; entries past GridSize are 0.
int Simulator::writeHotstart() {
    int rc;
    std::vector<double> w, hu, hv, F;
    if ((rc = getField(RIFT_FIELD_W, w)) || (rc = getField(RIFT_FIELD_HU, hu)) ||
        (rc = getField(RIFT_FIELD_HV, hv)))
        return rc;
    if (infiltration && (rc = getField(RIFT_FIELD_F, F))) return rc;
    int32_t nBX = 0, nBY = 0;
    if ((rc = rift_get_tile_grid(R, &nBX, &nBY))) return engineFail(rc, "rift_get_tile_grid");
    const int G = nBX * nBY, GG = growGridSize(gc.h_nx, gc.h_ny);
    std::vector<uint8_t> wet(GG, 0);
    std::vector<int32_t> act(G), blocks(GG, 0);
    int32_t nAct = 0;
    if ((rc = rift_get_tiles(R, wet.data(), act.data(), &nAct))) return engineFail(rc, "rift_get_tiles");
    std::vector<uint8_t> isAct(G, 0);
    int k = 0;
    for (int q = 0; q < nAct; q++) {
        blocks[k++] = act[q];
        isAct[act[q]] = 1;
    }
    for (int b = 0; b < G; b++)
        if (!isAct[b]) blocks[k++] = -b;
    const std::string path = output_file + "/hot" + std::to_string(count_print) + ".bin";
    return rift_host::writeHotstart(path, t, dt, gc, w.data(), hu.data(), hv.data(),
                                    infiltration ? F.data() : nullptr, wet.data(), blocks.data());
}

// ReadHotstart (simulator.cu:973-1090): the file's grid must match this one.
int Simulator::readHotstart(const std::string& path) {
    double ft, fdt;
    rift_gridconfig fg{};
    int rc = rift_host::readHotstart(path, ft, fdt, fg, infiltration, nullptr, nullptr, nullptr,
                                     nullptr, nullptr, nullptr);
    if (rc) return rc;
    std::string bad;
    if (fg.b_nx != gc.b_nx || fg.b_ny != gc.b_ny) bad += " domain size";
    if (fg.h_dx != gc.h_dx || fg.h_dy != gc.h_dy) bad += " internal cell sizes";
    if (fg.cellsize_original != gc.cellsize_original) bad += " original cell size";
    if (fg.cellsize != gc.cellsize) bad += " cell size";
    if ((fg.square_cells != 0) != square_cells || (fg.projected != 0) != projected)
        bad += " domain flags";
    if (!bad.empty()) return fail(RIFT_ERR_ARG, "Invalid hotstart:" + bad);
    const int GG = growGridSize(gc.h_nx, gc.h_ny);
    std::vector<double> w(N()), hu(N()), hv(N()), F(infiltration ? N() : 0);
    std::vector<uint8_t> wet(GG);
    std::vector<int32_t> blocks(GG);
    if ((rc = rift_host::readHotstart(path, ft, fdt, fg, infiltration, w.data(), hu.data(),
                                      hv.data(), infiltration ? F.data() : nullptr, wet.data(),
                                      blocks.data())))
        return rc;
    int32_t nBX = 0, nBY = 0;
    if ((rc = rift_get_tile_grid(R, &nBX, &nBY))) return engineFail(rc, "rift_get_tile_grid");
    const int G = nBX * nBY;
    // the active set: the non-negative entries (tile 0 encodes as 0)
    std::vector<uint8_t> isAct(G, 0);
    for (int q = 0; q < G; q++)
        if (blocks[q] >= 0 && blocks[q] < G) isAct[blocks[q]] = 1;
    std::vector<int32_t> act;
    for (int b = 0; b < G; b++)
        if (isAct[b]) act.push_back(b);
    if ((rc = rift_set_state(R, ft, fdt, w.data(), hu.data(), hv.data(),
                             infiltration ? F.data() : nullptr, wet.data(), act.data(),
                             (int32_t)act.size(), nullptr, nullptr)))
        return engineFail(rc, "rift_set_state");
    t = ft;
    dt = fdt;
    return RIFT_OK;
}

int Simulator::closeSimulation() {
    int rc = save_max ? printSummaryData() : RIFT_OK;
    if (R) {
        rift_destroy(R);
        R = nullptr;
    }
    return rc;
}

}  // namespace rift_host

// ------------------------------------------------------------------ C ABI
struct rift_sim {
    rift_host::Simulator s;
};

extern "C" {

int rift_sim_open(const char* config_path, rift_sim** out) {
    return rift_sim_open_flow(config_path, 0.0, out);
}

int rift_sim_open_flow(const char* config_path, double flow_rate, rift_sim** out) {
    if (!config_path || !out) return RIFT_ERR_ARG;
    *out = nullptr;
    rift_sim* s = new rift_sim();
    s->s.flow_rate = flow_rate;
    int rc = s->s.openSimulation(config_path);
    if (rc) {  // the message stays readable through rift_host_last_error()
        delete s;
        return rc;
    }
    *out = s;
    return RIFT_OK;
}

int rift_sim_step(rift_sim* s, double* t) {
    if (!s || !s->s.R) return RIFT_ERR_STATE;
    int rc = s->s.runSimulation();
    if (rc) s->s.err = rift_host::g_err;
    if (t) *t = s->s.t;
    return rc;
}

int rift_sim_run(rift_sim* s, double t_end, double* t, int64_t* steps) {
    if (!s || !s->s.R) return RIFT_ERR_STATE;
    long long n = 0;
    int rc = s->s.run(t_end, &n);
    if (rc) s->s.err = rift_host::g_err;
    if (t) *t = s->s.t;
    if (steps) *steps = n;
    return rc;
}

int rift_sim_time(rift_sim* s, double* t, double* dt, double* tf) {
    if (!s) return RIFT_ERR_ARG;
    if (t) *t = s->s.t;
    if (dt) *dt = s->s.dt;
    if (tf) *tf = s->s.tf;
    return RIFT_OK;
}

rift_handle* rift_sim_engine(rift_sim* s) { return s ? s->s.R : nullptr; }

int rift_sim_flow_rate(rift_sim* s, double* flow_rate) {
    if (!s || !flow_rate) return RIFT_ERR_ARG;
    *flow_rate = s->s.flow_rate;
    return RIFT_OK;
}

int rift_sim_num_sources(rift_sim* s, int32_t* n) {
    if (!s || !n) return RIFT_ERR_ARG;
    *n = (int32_t)s->s.source_idx.size();
    return RIFT_OK;
}

int rift_sim_set_source_value(rift_sim* s, double value) {
    if (!s || !s->s.R) return RIFT_ERR_STATE;
    s->s.setSourceValue(value);
    return RIFT_OK;
}

int rift_sim_update_sources(rift_sim* s) {
    if (!s || !s->s.R) return RIFT_ERR_STATE;
    int rc = s->s.updateSources();
    if (rc) s->s.err = rift_host::g_err;
    return rc;
}

int rift_sim_source_volume(rift_sim* s, double* v_added) {
    if (!s || !v_added) return RIFT_ERR_ARG;
    *v_added = s->s.V_added;
    return RIFT_OK;
}

int rift_sim_close(rift_sim* s) {
    if (!s) return RIFT_ERR_ARG;
    int rc = s->s.closeSimulation();
    delete s;
    return rc;
}

const char* rift_sim_last_error(rift_sim* s) { return s ? s->s.err.c_str() : "null simulator"; }

}  // extern "C"
