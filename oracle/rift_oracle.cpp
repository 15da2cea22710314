// rift_oracle.cpp -- CPU FP64 restatement of the reference RIFT step.
//
// TEST INFRASTRUCTURE ONLY: loaded by tests/, __graft_entry__.smoke() and the
// cpu_baseline / reference legs of bench.py as the checker.  The product path
// never links it.
//
// Every function cites the reference file:line whose behaviour it restates.
// State is kept in the reference's data model: FP64 water-surface elevation
// w, momenta hu/hv, face elevations BX/BY, cell-centre BC, per-tile flags and
// speed maxima.  Tiles are the reference's 16 x 14 blocks (grid.cu:18-19).

#include "rift_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr int TW = 16;  // BLOCK_COLS, grid.cu:19
constexpr int TH = 14;  // BLOCK_ROWS, grid.cu:18

// Physical constants are float literals widened to double (grid.cu:28-30).
const double kG = (double)9.80665f;
const double kEps = (double)1.19209e-07f;
const double kTheta = (double)1.3f;

// Mode-dependent rounding points.  In REF mode each float math call on a
// double argument rounds its argument(s) and result to float, as the
// reference's fminf/fmaxf/fabsf/sqrtf/powf calls do (grid.cu:75,83,134-135,
// 756-758, ...).
struct FM {
    bool ref;
    double fmin(double a, double b) const {
        return ref ? (double)fminf((float)a, (float)b) : std::fmin(a, b);
    }
    double fmax(double a, double b) const {
        return ref ? (double)fmaxf((float)a, (float)b) : std::fmax(a, b);
    }
    double fabs(double a) const { return ref ? (double)fabsf((float)a) : std::fabs(a); }
    double sqrt(double a) const { return ref ? (double)sqrtf((float)a) : std::sqrt(a); }
    double pow(double a, double b) const {
        return ref ? (double)powf((float)a, (float)b) : std::pow(a, b);
    }
};

// grid.cu:62-71.  `(int&)f` on a double reads the LOW 32-bit word, so the
// "sign" tests the low 31 mantissa bits and copies mantissa bit 31 into the
// low word of 1.0.  Result in {0, 1, 1+2^-21}; never negative.
double signf_lowword(double f) {
    uint64_t b;
    std::memcpy(&b, &f, 8);
    uint32_t lo = (uint32_t)b;
    if ((lo & 0x7FFFFFFFu) == 0) return 0.0;
    double r = 1.0;
    uint64_t rb;
    std::memcpy(&rb, &r, 8);
    rb |= (uint64_t)(lo & 0x80000000u);
    std::memcpy(&r, &rb, 8);
    return r;
}

// grid.cu:73-76
double minmod(const FM& m, double a, double b, double c) {
    double sa = signf_lowword(a), sb = signf_lowword(b), sc = signf_lowword(c);
    return 0.25 * sa * (sa + sb) * (sb + sc) * m.fmin(m.fmin(m.fabs(a), m.fabs(b)), m.fabs(c));
}

// grid.cu:78-80
double limiter(const FM& m, double U, double Up1, double Um1) {
    return 0.5 * minmod(m, kTheta * (Up1 - U), 0.5 * (Up1 - Um1), kTheta * (U - Um1));
}

// grid.cu:82-84
inline double velocity(const FM& m, double kappa, double h, double hz) {
    return 2.0 * h * hz / (h * h + m.fmax(h * h, kappa));
}

// grid.cu:86-89
inline double centralUpwind(double Uij, double Fij, double Ukh, double Fkh, double cm, double cp) {
    return (cp * Fij - cm * Fkh) / (cp - cm) + (cp * cm) / (cp - cm) * (Ukh - Uij);
}

struct Face3 {
    double w, hu, hv;
};

// grid.cu:91-116 -- reconstruction of one cell in one direction, with the
// wet/dry correction against the two face elevations.
void construct(const FM& m, double w, double hu, double hv, double wp1, double hup1,
               double hvp1, double wm1, double hum1, double hvm1, Face3& P, Face3& M,
               double Bp, double Bm) {
    double wz = limiter(m, w, wp1, wm1);
    double huz = limiter(m, hu, hup1, hum1);
    double hvz = limiter(m, hv, hvp1, hvm1);
    P.w = w + wz;
    M.w = w - wz;
    P.hu = hu + huz;
    M.hu = hu - huz;
    P.hv = hv + hvz;
    M.hv = hv - hvz;
    double wBar = P.w + M.w;
    if (P.w < Bp) {
        P.w = Bp;
        M.w = wBar - Bp;
    }
    if (M.w < Bm) {
        P.w = wBar - Bm;
        M.w = Bm;
    }
}

// grid.cu:118-165 (dir 0, getHX) and grid.cu:167-214 (dir 1, getHY).
// L is the upstream cell's face value, R the downstream cell's, B the face
// elevation.  Returns the three numerical fluxes and the local speed.
void faceFlux(const FM& m, double kappa, int dir, Face3 L, Face3 R, double B, double out[3],
              double& speed) {
    double hp = L.w - B;
    double hp1m = R.w - B;
    double up = velocity(m, kappa, hp, L.hu);
    double up1m = velocity(m, kappa, hp1m, R.hu);
    double vp = velocity(m, kappa, hp, L.hv);
    double vp1m = velocity(m, kappa, hp1m, R.hv);
    double hup = hp * up, hup1m = hp1m * up1m;
    double hvp = hp * vp, hvp1m = hp1m * vp1m;
    double sp = m.sqrt(kG * hp), sp1m = m.sqrt(kG * hp1m);
    double cp = dir == 0 ? up : vp, cp1m = dir == 0 ? up1m : vp1m;
    double ap = m.fmax(m.fmax(cp + sp, cp1m + sp1m), 0.0);
    double am = m.fmin(m.fmin(cp - sp, cp1m - sp1m), 0.0);
    double F0, F1, F2, R0, R1, R2;
    if (hp > 0.0) {
        if (dir == 0) {
            F0 = hup;
            F1 = hup * hup / hp + 0.5 * kG * hp * hp;
            F2 = hup * hvp / hp;
        } else {
            F0 = hvp;
            F1 = hup * hvp / hp;
            F2 = hvp * hvp / hp + 0.5 * kG * hp * hp;
        }
    } else {
        F0 = F1 = F2 = 0.0;
    }
    if (hp1m > 0.0) {
        if (dir == 0) {
            R0 = hup1m;
            R1 = hup1m * hup1m / hp1m + 0.5 * kG * hp1m * hp1m;
            R2 = hup1m * hvp1m / hp1m;
        } else {
            R0 = hvp1m;
            R1 = hup1m * hvp1m / hp1m;
            R2 = hvp1m * hvp1m / hp1m + 0.5 * kG * hp1m * hp1m;
        }
    } else {
        R0 = R1 = R2 = 0.0;
    }
    if (ap - am > 0.0) {
        out[0] = centralUpwind(L.w, F0, R.w, R0, am, ap);
        out[1] = centralUpwind(hup, F1, hup1m, R1, am, ap);
        out[2] = centralUpwind(hvp, F2, hvp1m, R2, am, ap);
    } else {
        out[0] = out[1] = out[2] = 0.0;
    }
    speed = m.fmax(ap, -am);
}

struct Series {
    std::vector<float> time, rate;
    float interp = 0.0f;  // Source::interpolated_rate (float, source.h:11)
    bool on = false;
    // source.cc:65-73 (evaluated at float(t), source.h:13)
    void interpolate(float t) {
        for (size_t i = 0; i + 1 < time.size(); i++) {
            if (t >= time[i] && t < time[i + 1]) {
                interp = rate[i] + (rate[i + 1] - rate[i]) / (time[i + 1] - time[i]) * (t - time[i]);
            }
        }
    }
};

struct Map {
    std::vector<double> t0, t1;
    double factor = 0.0;
    bool interp = false;
    bool set = false;
    bool timed = false;  // factor = (t - tA) / (tB - tA) at each step start
    double tA = 0.0, tB = 0.0;
};

}  // namespace

struct rift_oracle {
    rift_grid_desc g;
    FM m;
    int nx, ny, nBX, nBY, gridSize;
    bool have_static = false, inited = false;
    std::vector<double> BX, BY, BC, n, K, h0;
    std::vector<double> w, hu, hv, w_old, hu_old, hv_old, dw, dhu, dhv, G;
    std::vector<double> F, F_old, dF;
    std::vector<double> hmap, qmap, h_max, q_max, t_peak, t_dry, t_wet;
    std::vector<double> mx, my;
    std::vector<uint8_t> wet, active, prev_active;
    bool first_grow = true;
    double t = 0.0, dt = 0.0;
    double rain_rate = 0.0, drain_rate = 0.0;
    double v_added = 0.0;  // volume ledger, see rift_oracle_mass_ledger
    // full ledger (rift_oracle_mass_ledger_terms): terms since its start,
    // LED order drained, infiltrated, clamped, surge, boundary inflow; the
    // rates of the last flux pass (edge inflow, drain, infiltration) wait
    // for the dt the integrator applies them with
    double led[5] = {0, 0, 0, 0, 0};
    double pendRate[3] = {0, 0, 0};
    double vol0 = 0.0, soil0 = 0.0, added0 = 0.0;
    std::vector<int32_t> src_idx;
    std::vector<double> src_rate;
    Map maps[3];
    std::vector<double> cur_map[3];
    Series series[3];
    std::string err;

    bool has(uint32_t f) const { return (g.flags & f) != 0; }
    size_t c(int j, int i) const { return (size_t)j * nx + i; }
    double bx(int j, int i) const { return BX[(size_t)j * (nx + 1) + i]; }
    double by(int j, int i) const { return BY[(size_t)j * nx + i]; }
    bool interior(int j, int i) const { return i >= 2 && j >= 2 && i <= nx - 3 && j <= ny - 3; }
    // A tile's flags are written by its thread (0,0); the tile is "owned"
    // when that thread is an interior cell (Integrate_2_k:1061,1162-1170).
    bool tileHead(int b) const {
        int i0 = (b % nBX) * TW + 2, j0 = (b / nBX) * TH + 2;
        return i0 <= nx - 3 && j0 <= ny - 3;
    }
    // InitGrid_k:511-517: tiles whose thread (0,0) lies inside the h-grid.
    bool tileInGrid(int b) const {
        int i0 = (b % nBX) * TW + 2, j0 = (b / nBX) * TH + 2;
        return i0 < nx && j0 < ny;
    }
};

namespace {

double mapValue(const rift_oracle* o, int which, size_t idx) {
    return o->cur_map[which][idx];
}

// InterpGrid_k (grid.cu:292-311): nodata-aware linear interpolation.
void refreshMap(rift_oracle* o, int which) {
    Map& M = o->maps[which];
    std::vector<double>& cur = o->cur_map[which];
    if (!M.set) return;
    if (!M.interp) {
        cur = M.t0;
        return;
    }
    const double nd = o->g.nodata;
    for (size_t k = 0; k < cur.size(); k++) {
        double x0 = M.t0[k], x1 = M.t1[k];
        if (x1 == nd && x0 == nd)
            cur[k] = nd;
        else if (x1 == nd)
            cur[k] = x0;
        else if (x0 == nd)
            cur[k] = x1;
        else
            cur[k] = M.factor * (x1 - x0) + x0;
    }
}

// ApplyBoundariesX_k / ApplyBoundariesY_k (grid.cu:1325-1406): critical-depth
// outflow ghosts; X clamps HL at epsilon, Y does not; corners untouched.
void applyBoundaries(rift_oracle* o) {
    const FM& m = o->m;
    const int nx = o->nx, ny = o->ny;
    for (int j = 2; j <= ny - 3; j++) {
        size_t L = o->c(j, 2);
        double HL = m.fmin(m.pow(o->hu[L] * o->hu[L] / kG, 1.0 / 3.0), o->w[L] - o->BC[L]);
        HL = (HL > kEps) ? HL : 0.0;
        double wl = o->BC[L] + HL;
        o->w[o->c(j, 0)] = o->w[o->c(j, 1)] = wl;
        o->hu[o->c(j, 0)] = o->hu[o->c(j, 1)] = o->hu[L];
        o->hv[o->c(j, 0)] = o->hv[o->c(j, 1)] = o->hv[L];
        size_t R = o->c(j, nx - 3);
        double HR = m.fmin(m.pow(o->hu[R] * o->hu[R] / kG, 1.0 / 3.0), o->w[R] - o->BC[R]);
        HR = (HR > kEps) ? HR : 0.0;
        double wr = o->BC[R] + HR;
        o->w[o->c(j, nx - 1)] = o->w[o->c(j, nx - 2)] = wr;
        o->hu[o->c(j, nx - 1)] = o->hu[o->c(j, nx - 2)] = o->hu[R];
        o->hv[o->c(j, nx - 1)] = o->hv[o->c(j, nx - 2)] = o->hv[R];
    }
    for (int i = 2; i <= nx - 3; i++) {
        size_t B = o->c(2, i);
        double HB = m.fmin(m.pow(o->hv[B] * o->hv[B] / kG, 1.0 / 3.0), o->w[B] - o->BC[B]);
        double wb = o->BC[B] + HB;
        o->w[o->c(0, i)] = o->w[o->c(1, i)] = wb;
        o->hu[o->c(0, i)] = o->hu[o->c(1, i)] = o->hu[B];
        o->hv[o->c(0, i)] = o->hv[o->c(1, i)] = o->hv[B];
        size_t T = o->c(ny - 3, i);
        double HT = m.fmin(m.pow(o->hv[T] * o->hv[T] / kG, 1.0 / 3.0), o->w[T] - o->BC[T]);
        double wt = o->BC[T] + HT;
        o->w[o->c(ny - 1, i)] = o->w[o->c(ny - 2, i)] = wt;
        o->hu[o->c(ny - 1, i)] = o->hu[o->c(ny - 2, i)] = o->hu[T];
        o->hv[o->c(ny - 1, i)] = o->hv[o->c(ny - 2, i)] = o->hv[T];
    }
}

// Grow (grid.cu:1279-1322) with TrackRainfall_k / TrackSurge_k
// (grid.cu:1224-1276) and Grow_k (grid.cu:1188-1222).
void grow(rift_oracle* o) {
    const int nBX = o->nBX, nBY = o->nBY, nx = o->nx, ny = o->ny;
    const bool rg = o->has(RIFT_F_RAIN_GRID), sg = o->has(RIFT_F_SURGE_GRID);
    if (rg || sg) {
        // The entries that thrust::partition(is_negative) puts first are the
        // tiles encoded -id (inactive in the previous Grow; tile 0 encodes as
        // 0 and is never among them).  Before the first Grow the only
        // negative entries are the -1 fills of tiles InitGrid_k never
        // reached, which TrackRainfall_k maps to tile abs(-1) = 1.
        std::vector<int> tracked;
        if (o->first_grow) {
            bool anyOut = false;
            for (int b = 0; b < o->gridSize; b++)
                if (!o->tileInGrid(b)) anyOut = true;
            if (anyOut && o->gridSize > 1) tracked.push_back(1);
        } else {
            for (int b = 1; b < o->gridSize; b++)
                if (!o->prev_active[b]) tracked.push_back(b);
        }
        // The Track kernels take rows from blockY*BLOCK_COLS (16, not 14).
        auto track = [&](int which, bool surge) {
            std::vector<uint8_t> setw(o->gridSize, 0);
            for (int b : tracked) {
                if (o->wet[b]) continue;
                int bX = b % nBX, bY = b / nBX;
                bool hit = false;
                for (int ty = 0; ty < TH && !hit; ty++)
                    for (int tx = 0; tx < TW && !hit; tx++) {
                        int i = bX * TW + tx + 2, j = bY * TW + ty + 2;
                        if (i < 2 || j < 2 || i > nx - 3 || j > ny - 3) continue;
                        double v = mapValue(o, which, o->c(j, i));
                        if (surge) {
                            if (v != o->g.nodata && v > 0.0) hit = true;
                        } else if (v > kEps) {
                            hit = true;
                        }
                    }
                if (hit) setw[b] = 1;
            }
            for (int b = 0; b < o->gridSize; b++)
                if (setw[b]) o->wet[b] = 1;
        };
        if (rg) track(RIFT_MAP_RAIN, false);
        if (sg) track(RIFT_MAP_SURGE, true);
    }
    // Grow_k: 4-neighbour dilation, false outside the tile grid.  Tile 0
    // encodes as 0 either way and so is always kept by is_nonnegative.
    for (int bY = 0; bY < nBY; bY++)
        for (int bX = 0; bX < nBX; bX++) {
            int b = bY * nBX + bX;
            bool a = o->wet[b] || (bX > 0 && o->wet[b - 1]) || (bX < nBX - 1 && o->wet[b + 1]) ||
                     (bY > 0 && o->wet[b - nBX]) || (bY < nBY - 1 && o->wet[b + nBX]);
            o->active[b] = (a || b == 0) ? 1 : 0;
        }
    o->prev_active = o->active;
    o->first_grow = false;
}

// ComputeFluxes_k (grid.cu:564-839) over the active tiles.  Fluxes read the
// unclamped w of every cell; the w = BC clamp of grid.cu:748-749 is applied
// after all tiles are done (in the reference neighbours may read either value).
// clampWeight: the share of the step's result that the state entering this
// flux pass carries (1 for U^n, whose clamp both RK stages see; 1/2 for U*).
void computeFluxes(rift_oracle* o, double dtArg, double clampWeight) {
    const FM& m = o->m;
    const int nx = o->nx, ny = o->ny, nBX = o->nBX;
    const double kappa = o->g.kappa, dx = o->g.dx, dy = o->g.dy;
    std::vector<int> tiles;
    for (int b = 0; b < o->gridSize; b++)
        if (o->active[b]) tiles.push_back(b);
    std::vector<uint8_t> clampMask(o->w.size(), 0);
    const int ntiles = (int)tiles.size();
    // ledger partials per tile (summed in tile order afterwards): edge
    // inflow rate, drain rate, infiltration rate
    std::vector<double> part(3 * (size_t)ntiles, 0.0);

#pragma omp parallel for schedule(dynamic, 4)
    for (int k = 0; k < ntiles; k++) {
        const int b = tiles[k];
        const int bX = b % nBX, bY = b / nBX;
        const int i0 = bX * TW + 2, j0 = bY * TH + 2;
        double FX[TH][TW + 1][3], FY[TH + 1][TW][3];
        double SX[TH][TW], SY[TH][TW];
        for (int ty = 0; ty < TH; ty++)
            for (int tx = 0; tx < TW; tx++) SX[ty][tx] = SY[ty][tx] = 0.0;
        // x faces: face f sits between cells i0+f-1 and i0+f (f = 0..16)
        for (int ty = 0; ty < TH; ty++) {
            int j = j0 + ty;
            if (j > ny - 3) break;
            for (int f = 0; f <= TW; f++) {
                int il = i0 + f - 1, ir = i0 + f;
                if (il > nx - 3) break;
                Face3 Pl, Ml, Pr, Mr;
                size_t a = o->c(j, il), bb = o->c(j, ir);
                construct(m, o->w[a], o->hu[a], o->hv[a], o->w[a + 1], o->hu[a + 1], o->hv[a + 1],
                          o->w[a - 1], o->hu[a - 1], o->hv[a - 1], Pl, Ml, o->bx(j, il + 1),
                          o->bx(j, il));
                construct(m, o->w[bb], o->hu[bb], o->hv[bb], o->w[bb + 1], o->hu[bb + 1],
                          o->hv[bb + 1], o->w[bb - 1], o->hu[bb - 1], o->hv[bb - 1], Pr, Mr,
                          o->bx(j, ir + 1), o->bx(j, ir));
                double sp;
                faceFlux(m, kappa, 0, Pl, Mr, o->bx(j, ir), FX[ty][f], sp);
                if (f >= 1) SX[ty][f - 1] = sp;  // east face of cell il
            }
        }
        // y faces: face f sits between rows j0+f-1 and j0+f (f = 0..14)
        for (int tx = 0; tx < TW; tx++) {
            int i = i0 + tx;
            if (i > nx - 3) break;
            for (int f = 0; f <= TH; f++) {
                int jl = j0 + f - 1, jr = j0 + f;
                if (jl > ny - 3) break;
                Face3 Pl, Ml, Pr, Mr;
                size_t a = o->c(jl, i), bb = o->c(jr, i);
                construct(m, o->w[a], o->hu[a], o->hv[a], o->w[a + nx], o->hu[a + nx],
                          o->hv[a + nx], o->w[a - nx], o->hu[a - nx], o->hv[a - nx], Pl, Ml,
                          o->by(jl + 1, i), o->by(jl, i));
                construct(m, o->w[bb], o->hu[bb], o->hv[bb], o->w[bb + nx], o->hu[bb + nx],
                          o->hv[bb + nx], o->w[bb - nx], o->hu[bb - nx], o->hv[bb - nx], Pr, Mr,
                          o->by(jr + 1, i), o->by(jr, i));
                double sp;
                faceFlux(m, kappa, 1, Pl, Mr, o->by(jr, i), FY[f][tx], sp);
                if (f >= 1) SY[f - 1][tx] = sp;  // north face of cell jl
            }
        }
        // cell update, grid.cu:681-811
        double mxt = 0.0, myt = 0.0;
        for (int ty = 0; ty < TH; ty++) {
            int j = j0 + ty;
            if (j > ny - 3) break;
            for (int tx = 0; tx < TW; tx++) {
                int i = i0 + tx;
                if (i > nx - 3) break;
                size_t id = o->c(j, i);
                double dwv = -(FX[ty][tx + 1][0] - FX[ty][tx][0]) / dx;
                double dhuv = -(FX[ty][tx + 1][1] - FX[ty][tx][1]) / dx;
                double dhvv = -(FX[ty][tx + 1][2] - FX[ty][tx][2]) / dx;
                double S1 = (o->bx(j, i + 1) - o->bx(j, i)) / dx;
                double S2 = (o->by(j + 1, i) - o->by(j, i)) / dy;
                dwv += -(FY[ty + 1][tx][0] - FY[ty][tx][0]) / dy;
                dhuv += -(FY[ty + 1][tx][1] - FY[ty][tx][1]) / dy;
                dhvv += -(FY[ty + 1][tx][2] - FY[ty][tx][2]) / dy;
                double hC = o->w[id] - o->BC[id];
                if (!(hC > kEps)) clampMask[id] = 1;
                S1 *= -kG * hC;
                S2 *= -kG * hC;
                double nn = o->n[id];
                o->G[id] = -4.0 * kG * nn * nn * m.sqrt(o->hu[id] * o->hu[id] + o->hv[id] * o->hv[id]) *
                           m.pow(hC, (double)(5.f / 3.f)) / m.pow(hC * hC + m.fmax(hC * hC, kappa), 2.0);
                double S0 = 0.0;
                if (o->has(RIFT_F_RAIN_UNIFORM)) S0 += o->rain_rate;
                if (o->has(RIFT_F_RAIN_GRID)) S0 += mapValue(o, RIFT_MAP_RAIN, id);
                if (o->has(RIFT_F_DRAIN_UNIFORM)) {
                    double d = (o->drain_rate > hC / dtArg) ? hC / dtArg : o->drain_rate;
                    S0 -= d;
                    part[3 * k + 1] += d;
                }
                if (o->has(RIFT_F_DRAIN_GRID)) {
                    double d = mapValue(o, RIFT_MAP_DRAIN, id);
                    d = (d > hC / dtArg) ? hC / dtArg : d;
                    S0 -= d;
                    part[3 * k + 1] += d;
                }
                // flow through the domain edge (the critical-depth ghosts)
                if (i == 2) part[3 * k] += FX[ty][tx][0] / dx;
                if (i == nx - 3) part[3 * k] -= FX[ty][tx + 1][0] / dx;
                if (j == 2) part[3 * k] += FY[ty][tx][0] / dy;
                if (j == ny - 3) part[3 * k] -= FY[ty + 1][tx][0] / dy;
                if (o->has(RIFT_F_POINT_SOURCE) || !o->src_idx.empty()) {
                    for (size_t s = 0; s < o->src_idx.size(); s++)
                        S0 = ((long)j * nx + i == (long)o->src_idx[s]) ? S0 + o->src_rate[s] : S0;
                }
                if (o->has(RIFT_F_INFILTRATION)) {
                    double Kc = o->K[id], Fc = o->F[id];
                    double p1 = Kc * dtArg - 2.0 * Fc;
                    double p2 = Kc * (Fc + o->g.psi * o->g.dtheta);
                    double f = (p1 + m.sqrt(p1 * p1 + 8.0 * p2 * dtArg)) / (2.0 * dtArg);
                    f = (f > hC / dtArg) ? hC / dtArg : f;
                    f = (f > 0.0) ? f : 0.0;
                    o->dF[id] = f;
                    S0 -= f;
                    part[3 * k + 2] += f;
                }
                o->dw[id] = dwv + S0;
                o->dhu[id] = dhuv + S1;
                o->dhv[id] = dhvv + S2;
                mxt = m.fmax(mxt, SX[ty][tx]);
                myt = m.fmax(myt, SY[ty][tx]);
            }
        }
        o->mx[b] = mxt;
        o->my[b] = myt;
    }
    double clamped = 0.0;
    for (size_t id = 0; id < clampMask.size(); id++)
        if (clampMask[id]) {
            clamped += o->w[id] - o->BC[id];
            o->w[id] = o->BC[id];
        }
    o->led[2] += clampWeight * clamped;
    for (int q = 0; q < 3; q++) o->pendRate[q] = 0.0;
    for (int k = 0; k < ntiles; k++)
        for (int q = 0; q < 3; q++) o->pendRate[q] += part[3 * (size_t)k + q];
}

// The rates of the last flux pass applied for weight x dt: edge inflow,
// drain and infiltration into the ledger.
void ledgerRates(rift_oracle* o, double wdt) {
    o->led[4] += wdt * o->pendRate[0];
    o->led[0] += wdt * o->pendRate[1];
    o->led[1] += wdt * o->pendRate[2];
}

// Simulator::ComputeTimestep (simulator.cu:540-566): max over ALL tiles,
// stale entries of inactive tiles included.
void computeTimestep(rift_oracle* o) {
    const FM& m = o->m;
    double mxv = *std::max_element(o->mx.begin(), o->mx.end());
    double myv = *std::max_element(o->my.begin(), o->my.end());
    double cx = o->g.dx / m.fmax(mxv / o->g.courant, o->g.kappa);
    double cy = o->g.dy / m.fmax(myv / o->g.courant, o->g.kappa);
    o->dt = std::min(cx, cy);
    if (o->t == 0.0) o->dt = (double)0.000001f;
    o->t += o->dt;
}

double velocityOut(const FM& m, double kappa, double h, double hz) { return velocity(m, kappa, h, hz); }

// Integrate_1_k (grid.cu:856-1024)
void integrate1(rift_oracle* o) {
    const FM& m = o->m;
    const int nx = o->nx, nBX = o->nBX;
    const double t = o->t, dt = o->dt, kappa = o->g.kappa;
    const bool euler = o->has(RIFT_F_EULER);
    const double wHalf = euler ? 1.0 : 0.5;
    std::vector<int> tiles;
    for (int b = 0; b < o->gridSize; b++)
        if (o->active[b]) tiles.push_back(b);
    const int ntiles = (int)tiles.size();
    std::vector<double> part(2 * (size_t)ntiles, 0.0);  // clamp, surge
#pragma omp parallel for schedule(dynamic, 4)
    for (int k = 0; k < ntiles; k++) {
        const int b = tiles[k];
        const int bX = b % nBX, bY = b / nBX;
        bool anyWet = false;
        for (int ty = 0; ty < TH; ty++)
            for (int tx = 0; tx < TW; tx++) {
                int i = bX * TW + tx + 2, j = bY * TH + ty + 2;
                if (!o->interior(j, i)) continue;
                size_t id = o->c(j, i);
                o->w_old[id] = o->w[id];
                o->hu_old[id] = o->hu[id];
                o->hv_old[id] = o->hv[id];
                if (o->has(RIFT_F_SURGE_GRID)) {
                    double s = mapValue(o, RIFT_MAP_SURGE, id);
                    if (s != o->g.nodata && s > 0.0) {
                        double next_h = o->w[id] + o->dw[id] * dt - o->BC[id];
                        double d0 = o->dw[id];
                        o->dw[id] = (s - next_h) / dt;
                        part[2 * k + 1] += (o->dw[id] - d0) * dt;
                    }
                }
                o->w[id] += o->dw[id] * dt;
                o->hu[id] += o->dhu[id] * dt;
                o->hu[id] /= (1.0 - dt * o->G[id]);
                o->hv[id] += o->dhv[id] * dt;
                o->hv[id] /= (1.0 - dt * o->G[id]);
                double hC = (o->w[id] - o->BC[id] > kEps) ? o->w[id] - o->BC[id] : 0.0;
                if (!(hC > kEps)) part[2 * k] += o->w[id] - o->BC[id];
                o->w[id] = (hC > kEps) ? o->w[id] : o->BC[id];
                if (o->has(RIFT_F_INFILTRATION)) {
                    o->F_old[id] = o->F[id];
                    o->F[id] += o->dF[id] * dt;
                }
                if (euler) {
                    if (o->has(RIFT_F_SAVE_MAX)) {
                        double uC = velocityOut(m, kappa, hC, o->hu[id]);
                        double vC = velocityOut(m, kappa, hC, o->hv[id]);
                        o->t_peak[id] = (hC > o->h_max[id]) ? t : o->t_peak[id];
                        o->t_dry[id] = (hC > 0.0762) ? t : o->t_dry[id];
                        o->h_max[id] = m.fmax(o->h_max[id], hC);
                        o->q_max[id] = m.fmax(o->q_max[id], hC * m.sqrt(vC * vC + uC * uC));
                    }
                    o->hmap[id] = hC;
                    {
                        double uC = velocityOut(m, kappa, hC, o->hu[id]);
                        double vC = velocityOut(m, kappa, hC, o->hv[id]);
                        o->qmap[id] = hC * m.sqrt(vC * vC + uC * uC);
                    }
                    if (o->has(RIFT_F_SAVE_ARRIVAL)) {
                        if (o->t_wet[id] < 0.0 && hC > kEps) o->t_wet[id] = t;
                    }
                    bool wc = (o->w[id] - o->BC[id]) > kEps;
                    for (size_t s = 0; s < o->src_idx.size(); s++)
                        if ((long)j * nx + i == (long)o->src_idx[s]) wc = true;
                    if (o->has(RIFT_F_RAIN_UNIFORM) && o->rain_rate > 0.0) wc = true;
                    if (o->has(RIFT_F_RAIN_GRID) && mapValue(o, RIFT_MAP_RAIN, id) > 0.0) wc = true;
                    if (o->has(RIFT_F_SURGE_GRID)) {
                        double s = mapValue(o, RIFT_MAP_SURGE, id);
                        if (s != o->g.nodata && s > 0.0) wc = true;
                    }
                    anyWet = anyWet || wc;
                }
            }
        if (euler && o->tileHead(b)) o->wet[b] = (!o->has(RIFT_F_TILE_ACCEL)) || anyWet;
    }
    ledgerRates(o, wHalf * dt);
    for (int k = 0; k < ntiles; k++) {
        o->led[2] += wHalf * part[2 * (size_t)k];
        o->led[3] += wHalf * part[2 * (size_t)k + 1];
    }
}

// Integrate_2_k (grid.cu:1043-1171)
void integrate2(rift_oracle* o) {
    const FM& m = o->m;
    const int nx = o->nx, nBX = o->nBX;
    const double t = o->t, dt = o->dt, kappa = o->g.kappa;
    std::vector<int> tiles;
    for (int b = 0; b < o->gridSize; b++)
        if (o->active[b]) tiles.push_back(b);
    const int ntiles = (int)tiles.size();
    std::vector<double> part((size_t)ntiles, 0.0);  // clamp
#pragma omp parallel for schedule(dynamic, 4)
    for (int k = 0; k < ntiles; k++) {
        const int b = tiles[k];
        const int bX = b % nBX, bY = b / nBX;
        bool anyWet = false;
        for (int ty = 0; ty < TH; ty++)
            for (int tx = 0; tx < TW; tx++) {
                int i = bX * TW + tx + 2, j = bY * TH + ty + 2;
                if (!o->interior(j, i)) continue;
                size_t id = o->c(j, i);
                o->w[id] = 0.5 * (o->w_old[id] + o->w[id] + o->dw[id] * dt);
                o->hu[id] = 0.5 * (o->hu_old[id] + o->hu[id] + o->dhu[id] * dt);
                o->hv[id] = 0.5 * (o->hv_old[id] + o->hv[id] + o->dhv[id] * dt);
                double hC = (o->w[id] - o->BC[id] > kEps) ? o->w[id] - o->BC[id] : 0.0;
                if (!(hC > kEps)) part[k] += o->w[id] - o->BC[id];
                o->w[id] = (hC > kEps) ? o->w[id] : o->BC[id];
                if (o->has(RIFT_F_INFILTRATION))
                    o->F[id] = 0.5 * (o->F_old[id] + o->F[id] + o->dF[id] * dt);
                double uC = velocityOut(m, kappa, hC, o->hu[id]);
                double vC = velocityOut(m, kappa, hC, o->hv[id]);
                if (o->has(RIFT_F_SAVE_MAX)) {
                    o->h_max[id] = m.fmax(o->h_max[id], hC);
                    o->q_max[id] = m.fmax(o->q_max[id], hC * m.sqrt(vC * vC + uC * uC));
                }
                o->hmap[id] = hC;
                o->qmap[id] = hC * m.sqrt(vC * vC + uC * uC);
                if (o->has(RIFT_F_SAVE_ARRIVAL)) {
                    if (o->t_wet[id] < 0.0 && hC > kEps) o->t_wet[id] = t;
                }
                bool wc = hC > kEps;
                for (size_t s = 0; s < o->src_idx.size(); s++)
                    if ((long)j * nx + i == (long)o->src_idx[s]) wc = true;
                if (o->has(RIFT_F_RAIN_UNIFORM) && o->rain_rate > 0.0) wc = true;
                if (o->has(RIFT_F_RAIN_GRID) && mapValue(o, RIFT_MAP_RAIN, id) > 0.0) wc = true;
                anyWet = anyWet || wc;
            }
        if (o->tileHead(b)) o->wet[b] = (!o->has(RIFT_F_TILE_ACCEL)) || anyWet;
    }
    ledgerRates(o, 0.5 * dt);
    for (int k = 0; k < ntiles; k++) o->led[2] += part[(size_t)k];
}

// Simulator::UpdateSource (simulator.cu:500-538) for device-style series:
// interpolate at float(t), then divide the float rate in place (every step,
// so outside the CSV time range the rate keeps shrinking).
void updateSeries(rift_oracle* o) {
    const float tf = (float)o->t;
    if (o->series[2].on) {
        Series& s = o->series[2];
        s.interpolate(tf);
        s.interp /= 35.3147f;
        double v = (double)s.interp;
        long ns = (long)o->src_idx.size();
        for (long k = 0; k < ns; k++) o->src_rate[k] = v / o->g.dx / o->g.dy / (double)ns;
    }
    if (o->series[0].on) {
        Series& s = o->series[0];
        s.interpolate(tf);
        s.interp /= (3600.f * 1000.f);
        o->rain_rate = (double)s.interp;
    }
    if (o->series[1].on) {
        Series& s = o->series[1];
        s.interpolate(tf);
        s.interp /= (3600.f * 1000.f);
        o->drain_rate = (double)s.interp;
    }
}

void oneStep(rift_oracle* o) {
    updateSeries(o);
    // InterpolatedGridSeries::p_update (GridSeries.cu:398): the factor of the
    // map used during this step comes from the time at its start
    for (int w = 0; w < 3; w++)
        if (o->maps[w].set && o->maps[w].timed) {
            o->maps[w].factor = (o->t - o->maps[w].tA) / (o->maps[w].tB - o->maps[w].tA);
            refreshMap(o, w);
        }
    grow(o);
    computeFluxes(o, o->dt, 1.0);
    computeTimestep(o);
    // volume the sources add over this step (each rate applies for dt)
    double add = 0.0;
    if (o->has(RIFT_F_RAIN_UNIFORM)) add += o->rain_rate * (double)(o->nx - 4) * (o->ny - 4);
    for (double r : o->src_rate) add += r;
    if (o->has(RIFT_F_RAIN_GRID) && o->maps[RIFT_MAP_RAIN].set)
        for (int j = 2; j < o->ny - 2; j++)
            for (int i = 2; i < o->nx - 2; i++) add += o->cur_map[RIFT_MAP_RAIN][o->c(j, i)];
    o->v_added += add * o->dt;
    integrate1(o);
    applyBoundaries(o);
    if (!o->has(RIFT_F_EULER)) {
        computeFluxes(o, o->dt, 0.5);
        integrate2(o);
        applyBoundaries(o);
    }
}

}  // namespace

namespace {
// Interior sums of h = w - BC (as the state holds it) and of F, Kahan.
void stateSums(const rift_oracle* o, double* vol, double* soil) {
    double s = 0.0, cs = 0.0, f = 0.0, cf = 0.0;
    for (int j = 2; j <= o->ny - 3; j++)
        for (int i = 2; i <= o->nx - 3; i++) {
            size_t id = o->c(j, i);
            double y = (o->w[id] - o->BC[id]) - cs;
            double tt = s + y;
            cs = (tt - s) - y;
            s = tt;
            if (o->has(RIFT_F_INFILTRATION)) {
                double yf = o->F[id] - cf;
                double tf = f + yf;
                cf = (tf - f) - yf;
                f = tf;
            }
        }
    *vol = s;
    *soil = f;
}

void ledgerStart(rift_oracle* o) {
    for (double& x : o->led) x = 0.0;
    for (double& x : o->pendRate) x = 0.0;
    o->added0 = o->v_added;
    stateSums(o, &o->vol0, &o->soil0);
}
}  // namespace

extern "C" {

int rift_oracle_set_threads(int32_t n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

double rift_oracle_minmod(double a, double b, double c) {
    FM m{true};
    return minmod(m, a, b, c);
}

double rift_oracle_limiter(double U, double Up1, double Um1) {
    FM m{true};
    return limiter(m, U, Up1, Um1);
}

int rift_oracle_create(const rift_grid_desc* g, int32_t mode, rift_oracle** out) {
    if (!g || !out || g->h_nx < 5 || g->h_ny < 5 || g->dx <= 0 || g->dy <= 0) return RIFT_ERR_ARG;
    rift_oracle* o = new rift_oracle();
    o->g = *g;
    o->m.ref = (mode == RIFT_ORACLE_REF);
    o->nx = g->h_nx;
    o->ny = g->h_ny;
    o->nBX = (o->nx + TW - 1) / TW;
    o->nBY = (o->ny + TH - 1) / TH;
    o->gridSize = o->nBX * o->nBY;
    size_t N = (size_t)o->nx * o->ny;
    for (auto* v : {&o->BC, &o->n, &o->K, &o->h0, &o->w, &o->hu, &o->hv, &o->w_old, &o->hu_old,
                    &o->hv_old, &o->dw, &o->dhu, &o->dhv, &o->G, &o->F, &o->F_old, &o->dF,
                    &o->hmap, &o->qmap, &o->h_max, &o->q_max, &o->t_peak, &o->t_dry, &o->t_wet})
        v->assign(N, 0.0);
    for (int k = 0; k < 3; k++) o->cur_map[k].assign(N, 0.0);
    o->cur_map[RIFT_MAP_SURGE].assign(N, g->nodata);
    o->BX.assign((size_t)o->ny * (o->nx + 1), 0.0);
    o->BY.assign((size_t)(o->ny + 1) * o->nx, 0.0);
    o->mx.assign(o->gridSize, 0.0);
    o->my.assign(o->gridSize, 0.0);
    o->wet.assign(o->gridSize, 0);
    o->active.assign(o->gridSize, 0);
    o->prev_active.assign(o->gridSize, 0);
    *out = o;
    return RIFT_OK;
}

int rift_oracle_upload_static(rift_oracle* o, const double* BX, const double* BY, const double* n,
                              const double* K_mps, const double* h0) {
    if (!o || !BX || !BY || !n) return RIFT_ERR_ARG;
    std::copy(BX, BX + o->BX.size(), o->BX.begin());
    std::copy(BY, BY + o->BY.size(), o->BY.begin());
    std::copy(n, n + o->n.size(), o->n.begin());
    if (K_mps) std::copy(K_mps, K_mps + o->K.size(), o->K.begin());
    if (h0) std::copy(h0, h0 + o->h0.size(), o->h0.begin());
    o->have_static = true;
    return RIFT_OK;
}

// InitGrid_k (grid.cu:506-553) then ApplyBoundaries (simulator.cu:731).
int rift_oracle_init(rift_oracle* o, double t0) {
    if (!o || !o->have_static) return RIFT_ERR_STATE;
    const int nx = o->nx, ny = o->ny;
    o->v_added = 0.0;
    for (int j = 2; j < ny; j++)
        for (int i = 2; i < nx; i++) {
            size_t id = o->c(j, i);
            o->BC[id] = 0.25 * (o->bx(j, i + 1) + o->bx(j, i) + o->by(j + 1, i) + o->by(j, i));
            o->w[id] = o->w_old[id] = o->BC[id];
            o->hu[id] = o->hu_old[id] = 0.0;
            o->hv[id] = o->hv_old[id] = 0.0;
            o->G[id] = 0.0;
            if (o->has(RIFT_F_H_INIT)) {
                o->w[id] += o->h0[id];
                o->w_old[id] += o->h0[id];
            }
            if (o->has(RIFT_F_SAVE_ARRIVAL)) o->t_wet[id] = (double)-9999.f;
        }
    for (int b = 0; b < o->gridSize; b++) {
        bool in = o->tileInGrid(b);
        o->wet[b] = in ? 1 : 0;
        o->active[b] = in ? 1 : 0;
        o->prev_active[b] = in ? 1 : 0;
    }
    o->first_grow = true;
    o->t = t0;
    o->dt = (double)0.0000001f;  // simulator.cu:35
    applyBoundaries(o);
    o->inited = true;
    ledgerStart(o);
    return RIFT_OK;
}

int rift_oracle_set_uniform_rates(rift_oracle* o, double rain, double drain) {
    if (!o) return RIFT_ERR_ARG;
    o->rain_rate = rain;
    o->drain_rate = drain;
    return RIFT_OK;
}

int rift_oracle_set_point_sources(rift_oracle* o, const int32_t* idx, const double* rate, int32_t n) {
    if (!o || n < 0 || (n > 0 && (!idx || !rate))) return RIFT_ERR_ARG;
    o->src_idx.assign(idx, idx + n);
    o->src_rate.assign(rate, rate + n);
    return RIFT_OK;
}

int rift_oracle_set_map(rift_oracle* o, int32_t which, const double* t0map, const double* t1map,
                        double factor) {
    if (!o || which < 0 || which > 2 || !t0map) return RIFT_ERR_ARG;
    size_t N = (size_t)o->nx * o->ny;
    Map& M = o->maps[which];
    M.t0.assign(t0map, t0map + N);
    M.interp = (t1map != nullptr);
    if (t1map) M.t1.assign(t1map, t1map + N);
    M.factor = factor;
    M.set = true;
    refreshMap(o, which);
    return RIFT_OK;
}

int rift_oracle_set_map_factor(rift_oracle* o, int32_t which, double factor) {
    if (!o || which < 0 || which > 2 || !o->maps[which].set) return RIFT_ERR_ARG;
    o->maps[which].factor = factor;
    refreshMap(o, which);
    return RIFT_OK;
}

int rift_oracle_set_map_times(rift_oracle* o, int32_t which, double t0, double t1) {
    if (!o || which < 0 || which > 2 || !o->maps[which].set) return RIFT_ERR_ARG;
    o->maps[which].timed = t1 > t0;
    o->maps[which].tA = t0;
    o->maps[which].tB = t1;
    return RIFT_OK;
}

int rift_oracle_set_series(rift_oracle* o, int32_t which, const float* times, const float* rates,
                           int32_t n) {
    if (!o || which < 0 || which > 2 || n < 0 || (n > 0 && (!times || !rates))) return RIFT_ERR_ARG;
    Series& s = o->series[which];
    s.time.assign(times, times + n);
    s.rate.assign(rates, rates + n);
    s.interp = 0.0f;
    s.on = n > 0;
    return RIFT_OK;
}

int rift_oracle_step(rift_oracle* o, double* t, double* dt) {
    if (!o || !o->inited) return RIFT_ERR_STATE;
    oneStep(o);
    if (t) *t = o->t;
    if (dt) *dt = o->dt;
    return RIFT_OK;
}

int rift_oracle_run(rift_oracle* o, int32_t nsteps, double t_stop, double* t, double* dt,
                    int32_t* done) {
    if (!o || !o->inited) return RIFT_ERR_STATE;
    int32_t k = 0;
    while (k < nsteps && o->t < t_stop) {
        oneStep(o);
        k++;
    }
    if (t) *t = o->t;
    if (dt) *dt = o->dt;
    if (done) *done = k;
    return RIFT_OK;
}

int rift_oracle_get_field(rift_oracle* o, int32_t which, double* host, size_t ld) {
    if (!o || !host || ld < (size_t)o->nx) return RIFT_ERR_ARG;
    const std::vector<double>* src = nullptr;
    switch (which) {
        case RIFT_FIELD_W: src = &o->w; break;
        case RIFT_FIELD_HU: src = &o->hu; break;
        case RIFT_FIELD_HV: src = &o->hv; break;
        case RIFT_FIELD_F: src = &o->F; break;
        case RIFT_FIELD_H: src = &o->hmap; break;
        case RIFT_FIELD_Q: src = &o->qmap; break;
        case RIFT_FIELD_HMAX: src = &o->h_max; break;
        case RIFT_FIELD_QMAX: src = &o->q_max; break;
        case RIFT_FIELD_TPEAK: src = &o->t_peak; break;
        case RIFT_FIELD_TDRY: src = &o->t_dry; break;
        case RIFT_FIELD_TWET: src = &o->t_wet; break;
        case RIFT_FIELD_BC: src = &o->BC; break;
        default: return RIFT_ERR_ARG;
    }
    for (int j = 0; j < o->ny; j++)
        std::copy(src->begin() + (size_t)j * o->nx, src->begin() + (size_t)(j + 1) * o->nx,
                  host + (size_t)j * ld);
    return RIFT_OK;
}

int rift_oracle_get_tiles(rift_oracle* o, uint8_t* wet, int32_t* active, int32_t* n_active) {
    if (!o) return RIFT_ERR_ARG;
    if (wet) std::copy(o->wet.begin(), o->wet.end(), wet);
    int32_t k = 0;
    for (int b = 0; b < o->gridSize; b++)
        if (o->active[b]) {
            if (active) active[k] = b;
            k++;
        }
    if (n_active) *n_active = k;
    return RIFT_OK;
}

int rift_oracle_get_tile_speeds(rift_oracle* o, double* mx, double* my) {
    if (!o) return RIFT_ERR_ARG;
    if (mx) std::copy(o->mx.begin(), o->mx.end(), mx);
    if (my) std::copy(o->my.begin(), o->my.end(), my);
    return RIFT_OK;
}

int rift_oracle_set_state(rift_oracle* o, double t, double dt_prev, const double* w,
                          const double* hu, const double* hv, const double* F, const uint8_t* wet,
                          const int32_t* active_ids, int32_t n_active, const double* mx,
                          const double* my) {
    if (!o || !o->inited || !w || !hu || !hv) return RIFT_ERR_ARG;
    size_t N = (size_t)o->nx * o->ny;
    std::copy(w, w + N, o->w.begin());
    std::copy(hu, hu + N, o->hu.begin());
    std::copy(hv, hv + N, o->hv.begin());
    if (F) std::copy(F, F + N, o->F.begin());
    if (wet) std::copy(wet, wet + o->gridSize, o->wet.begin());
    if (active_ids && n_active >= 0) {
        std::fill(o->active.begin(), o->active.end(), 0);
        for (int32_t k = 0; k < n_active; k++)
            if (active_ids[k] >= 0 && active_ids[k] < o->gridSize) o->active[active_ids[k]] = 1;
    }
    if (mx) std::copy(mx, mx + o->gridSize, o->mx.begin());
    if (my) std::copy(my, my + o->gridSize, o->my.begin());
    o->t = t;
    o->dt = dt_prev;
    // a hotstart carries the tile lists; after it every tile id is encoded
    // (no -1 fills), so the first-Grow special case no longer applies
    o->first_grow = false;
    for (int b = 0; b < o->gridSize; b++) o->prev_active[b] = o->active[b];
    ledgerStart(o);
    return RIFT_OK;
}

int rift_oracle_get_time(rift_oracle* o, double* t, double* dt) {
    if (!o) return RIFT_ERR_ARG;
    if (t) *t = o->t;
    if (dt) *dt = o->dt;
    return RIFT_OK;
}

// Volume check of simulator.cu:609-637 over the interior: sum of (w - BC) [+ F]
// (the reference sums its dev_h map; here the clamped depth of the state).
int rift_oracle_volume(rift_oracle* o, double* volume) {
    if (!o || !volume) return RIFT_ERR_ARG;
    double s = 0.0, comp = 0.0;  // Kahan
    for (int j = o->ny - 3; j >= 2; j--)
        for (int i = 2; i < o->nx - 2; i++) {
            size_t id = o->c(j, i);
            double hC = (o->w[id] - o->BC[id] > kEps) ? o->w[id] - o->BC[id] : 0.0;
            double v = hC + (o->has(RIFT_F_INFILTRATION) ? o->F[id] : 0.0);
            double y = v - comp;
            double tt = s + y;
            comp = (tt - s) - y;
            s = tt;
        }
    *volume = s;
    return RIFT_OK;
}


int rift_oracle_mass_ledger_terms(rift_oracle* o, rift_ledger* out) {
    if (!o || !out || !o->inited) return RIFT_ERR_ARG;
    rift_ledger L{};
    stateSums(o, &L.volume, &L.soil);
    L.volume0 = o->vol0;
    L.soil0 = o->soil0;
    L.added = o->v_added - o->added0;
    L.drained = o->led[0];
    L.infiltrated = o->led[1];
    L.clamped = o->led[2];
    L.surge = o->led[3];
    L.boundary = o->led[4];
    *out = L;
    return RIFT_OK;
}

int rift_oracle_mass_ledger(rift_oracle* o, double* volume, double* added) {
    if (!o || !volume || !added) return RIFT_ERR_ARG;
    int rc = rift_oracle_volume(o, volume);
    *added = o->v_added;
    return rc;
}

int rift_oracle_get_tile_grid(rift_oracle* o, int32_t* nBX, int32_t* nBY) {
    if (!o) return RIFT_ERR_ARG;
    if (nBX) *nBX = o->nBX;
    if (nBY) *nBY = o->nBY;
    return RIFT_OK;
}

const char* rift_oracle_last_error(rift_oracle* o) { return o ? o->err.c_str() : "null handle"; }

void rift_oracle_destroy(rift_oracle* o) { delete o; }

}  // extern "C"
