// refrun.cu -- TEST INFRASTRUCTURE: a host driver that runs the REFERENCE's
// own kernels (from oracle/_ref/rift_ref_sm103a.fatbin, the reference's
// unmodified grid.cu compiled for sm_103a) through the CUDA driver API.
//
// The reference's host program cannot be built for the aarch64 GPU machine from
// here, so this file restates its host orchestration: the allocations of
// AllocateGrid (grid.cu:347-490), InitGrid + ApplyBoundaries
// (simulator.cu:433-462,731), and per step the order of
// Simulator::RunSimulation (simulator.cu:773-853): UpdateSource, Grow (with
// the same thrust::partition / count_if calls, grid.cu:1279-1322),
// ComputeFluxes, ComputeTimestep (thrust::max_element, simulator.cu:540-566),
// Integrate_1, ApplyBoundaries, ComputeFluxes, Integrate_2, ApplyBoundaries.
// Every kernel that touches the state is the reference's own.
//
// Usage:  refrun <fatbin> <case_dir> <out_dir>
//   case_dir/params.txt ("key value" lines) and raw little-endian arrays;
//   see tests/golden/refcase.py for the writer.

#include <cuda.h>
#include <cuda_runtime.h>
#include <thrust/count.h>
#include <thrust/device_ptr.h>
#include <thrust/extrema.h>
#include <thrust/partition.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#define CK(x)                                                                          \
    do {                                                                               \
        CUresult r_ = (x);                                                             \
        if (r_ != CUDA_SUCCESS) {                                                      \
            const char* s_ = nullptr;                                                  \
            cuGetErrorString(r_, &s_);                                                 \
            std::fprintf(stderr, "driver error %s at %s:%d\n", s_ ? s_ : "?", __FILE__, \
                         __LINE__);                                                    \
            std::exit(2);                                                              \
        }                                                                              \
    } while (0)
#define CR(x)                                                                          \
    do {                                                                               \
        cudaError_t e_ = (x);                                                          \
        if (e_ != cudaSuccess) {                                                       \
            std::fprintf(stderr, "runtime error %s at %s:%d\n", cudaGetErrorString(e_), \
                         __FILE__, __LINE__);                                          \
            std::exit(2);                                                              \
        }                                                                              \
    } while (0)

static const int BC_ = 16, BR_ = 14;  // BLOCK_COLS, BLOCK_ROWS

struct is_nonneg {
    __host__ __device__ bool operator()(const int x) { return x > -1; }
};
struct is_neg {
    __host__ __device__ bool operator()(const int x) { return x < 0; }
};

static std::map<std::string, std::string> readParams(const std::string& path) {
    std::map<std::string, std::string> p;
    std::ifstream f(path);
    std::string line;
    while (std::getline(f, line)) {
        std::istringstream ss(line);
        std::string k, v;
        if (ss >> k) {
            std::getline(ss, v);
            size_t a = v.find_first_not_of(" \t");
            p[k] = (a == std::string::npos) ? "" : v.substr(a);
        }
    }
    return p;
}

template <typename T>
static std::vector<T> readBin(const std::string& path, size_t n, bool required = true) {
    std::vector<T> v(n, T(0));
    std::ifstream f(path, std::ios::binary);
    if (!f) {
        if (required) {
            std::fprintf(stderr, "missing %s\n", path.c_str());
            std::exit(3);
        }
        return v;
    }
    f.read(reinterpret_cast<char*>(v.data()), n * sizeof(T));
    return v;
}

template <typename T>
static void writeBin(const std::string& path, const T* p, size_t n) {
    std::ofstream f(path, std::ios::binary);
    f.write(reinterpret_cast<const char*>(p), n * sizeof(T));
}

struct Series {  // Source (source.h:8-16), float time/rate
    std::vector<float> time, rate;
    float interp = 0.f;
    bool on = false;
    void interpolate(float t) {  // source.cc:65-73
        for (size_t i = 0; i + 1 < time.size(); i++)
            if (t >= time[i] && t < time[i + 1])
                interp = rate[i] + (rate[i + 1] - rate[i]) / (time[i + 1] - time[i]) * (t - time[i]);
    }
};

int main(int argc, char** argv) {
    if (argc < 4) {
        std::fprintf(stderr, "usage: refrun <fatbin> <case_dir> <out_dir>\n");
        return 1;
    }
    const std::string fat = argv[1], dir = argv[2], out = argv[3];
    auto P = readParams(dir + "/params.txt");
    auto geti = [&](const char* k, long d) { return P.count(k) ? std::stol(P[k]) : d; };
    auto getd = [&](const char* k, double d) { return P.count(k) ? std::stod(P[k]) : d; };

    CR(cudaSetDevice(0));
    CR(cudaFree(0));
    CUmodule mod;
    CK(cuModuleLoad(&mod, fat.c_str()));
    unsigned nf = 0;
    CK(cuModuleGetFunctionCount(&nf, mod));
    std::vector<CUfunction> fns(nf);
    CK(cuModuleEnumerateFunctions(fns.data(), nf, mod));
    auto fn = [&](const char* key) {
        for (auto f : fns) {
            const char* nm = nullptr;
            CK(cuFuncGetName(&nm, f));
            std::string s(nm);
            // mangled C++ names: _Z<len><name>...; extern "C" probes are bare
            std::string want = std::to_string(std::strlen(key)) + key;
            if (s == key || s.rfind("_Z" + want, 0) == 0) return f;
        }
        std::fprintf(stderr, "kernel %s not found\n", key);
        std::exit(4);
        return CUfunction{};
    };

    const std::string mode = P.count("mode") ? P["mode"] : "run";
    if (mode == "probe") {
        double kap = getd("kappa", 0.1);
        CUdeviceptr kp;
        size_t ksz;
        CK(cuModuleGetGlobal(&kp, &ksz, mod, "kappa"));
        CK(cuMemcpyHtoD(kp, &kap, 8));
        // probe tables: probe_a/b/c.bin (double), n entries
        int n = (int)geti("n", 0);
        auto a = readBin<double>(dir + "/probe_a.bin", n);
        auto b = readBin<double>(dir + "/probe_b.bin", n);
        auto c = readBin<double>(dir + "/probe_c.bin", n);
        double *da, *db, *dc, *dout;
        CR(cudaMalloc(&da, n * 8));
        CR(cudaMalloc(&db, n * 8));
        CR(cudaMalloc(&dc, n * 8));
        CR(cudaMalloc(&dout, n * 8));
        CR(cudaMemcpy(da, a.data(), n * 8, cudaMemcpyHostToDevice));
        CR(cudaMemcpy(db, b.data(), n * 8, cudaMemcpyHostToDevice));
        CR(cudaMemcpy(dc, c.data(), n * 8, cudaMemcpyHostToDevice));
        std::vector<double> res(n);
        unsigned grid = (n + 127) / 128;
        {
            void* args[] = {&da, &dout, &n};
            CK(cuLaunchKernel(fn("ref_probe_signf"), grid, 1, 1, 128, 1, 1, 0, 0, args, 0));
            CR(cudaMemcpy(res.data(), dout, n * 8, cudaMemcpyDeviceToHost));
            writeBin(out + "/probe_signf.bin", res.data(), n);
        }
        {
            void* args[] = {&da, &db, &dc, &dout, &n};
            CK(cuLaunchKernel(fn("ref_probe_minmod"), grid, 1, 1, 128, 1, 1, 0, 0, args, 0));
            CR(cudaMemcpy(res.data(), dout, n * 8, cudaMemcpyDeviceToHost));
            writeBin(out + "/probe_minmod.bin", res.data(), n);
        }
        {
            void* args[] = {&da, &db, &dc, &dout, &n};
            CK(cuLaunchKernel(fn("ref_probe_limiter"), grid, 1, 1, 128, 1, 1, 0, 0, args, 0));
            CR(cudaMemcpy(res.data(), dout, n * 8, cudaMemcpyDeviceToHost));
            writeBin(out + "/probe_limiter.bin", res.data(), n);
        }
        {
            void* args[] = {&da, &db, &dout, &n};
            CK(cuLaunchKernel(fn("ref_probe_velocity"), grid, 1, 1, 128, 1, 1, 0, 0, args, 0));
            CR(cudaMemcpy(res.data(), dout, n * 8, cudaMemcpyDeviceToHost));
            writeBin(out + "/probe_velocity.bin", res.data(), n);
        }
        std::printf("probe ok n=%d\n", n);
        return 0;
    }

    const int nx = (int)geti("nx", 0), ny = (int)geti("ny", 0);
    const unsigned flags = (unsigned)geti("flags", 0);
    const double dx = getd("dx", 1), dy = getd("dy", 1), kappa = getd("kappa", 0.1);
    const double nodata = getd("nodata", -9999.0), courant = getd("courant", 0.25);
    const double psi = getd("psi", 0), dtheta = getd("dtheta", 0);
    const int nsteps = (int)geti("nsteps", 1);
    const bool timing = geti("timing", 0) != 0;
    std::vector<int> dumps;
    if (P.count("dump")) {
        std::istringstream ss(P["dump"]);
        std::string tok;
        while (std::getline(ss, tok, ',')) dumps.push_back(std::stoi(tok));
    }
    auto F_ = [&](unsigned b) { return (flags & (1u << b)) != 0; };
    // flag bits as in include/rift_gb300.h
    const bool rainU = F_(0), rainG = F_(1), drainU = F_(2), drainG = F_(3), infil = F_(4),
               surgeG = F_(5), euler = F_(6), saveMax = F_(7), saveArr = F_(8), tileAcc = F_(9),
               dambreak = F_(10), hInit = F_(11);

    // ---- SetDeviceConstants (grid.cu:321-344)
    auto setSym = [&](const char* name, const void* src, size_t bytes) {
        CUdeviceptr p;
        size_t sz;
        CK(cuModuleGetGlobal(&p, &sz, mod, name));
        if (sz != bytes) {
            std::fprintf(stderr, "symbol %s size %zu != %zu\n", name, sz, bytes);
            std::exit(5);
        }
        CK(cuMemcpyHtoD(p, src, bytes));
    };
    const int nBX = (int)std::ceil((double)nx / BC_), nBY = (int)std::ceil((double)ny / BR_);
    setSym("nx", &nx, 4);
    setSym("ny", &ny, 4);
    setSym("dx", &dx, 8);
    setSym("dy", &dy, 8);
    setSym("kappa", &kappa, 8);
    setSym("nodata", &nodata, 8);
    setSym("nBlocksX", &nBX, 4);
    setSym("nBlocksY", &nBY, 4);
    const int GridSize = nBX * nBY;
    int nBlocks = GridSize;
    // ---- AllocateGrid flags (grid.cu:368-382)
    bool bcheck = false, bprint = true;
    setSym("dambreak", &dambreak, 1);
    setSym("rainfall_averaged", &rainU, 1);
    setSym("drain_averaged", &drainU, 1);
    setSym("rainfall_gridded", &rainG, 1);
    setSym("drain_gridded", &drainG, 1);
    setSym("infiltration", &infil, 1);
    setSym("surge_gridded", &surgeG, 1);
    setSym("euler_integration", &euler, 1);
    setSym("check_volume", &bcheck, 1);
    setSym("h_init", &hInit, 1);
    setSym("h_print", &bprint, 1);
    setSym("q_print", &bprint, 1);
    setSym("save_max", &saveMax, 1);
    setSym("save_arrival_time", &saveArr, 1);
    setSym("tile_acceleration", &tileAcc, 1);
    setSym("psi", &psi, 8);
    setSym("dtheta", &dtheta, 8);

    size_t width = (size_t)nBX * BC_ * 8, width_p1 = ((size_t)nBX * BC_ + 1) * 8;
    size_t height = (size_t)nBY * BR_, height_p1 = height + 1;
    // The reference kernels touch up to two rows past the allocated height and
    // two columns past the width (ComputeFluxes_k on the last tile row and
    // column, past the allocation).  Every pitched array here gets
    // PAD extra rows and columns so those accesses stay inside this
    // allocation; the reference's arithmetic on interior cells never reads
    // them.
    const size_t PADC = 4 * 8, PADR = 4;
    size_t pitch = 0, pitchBX = 0, pitchBY = 0;
    auto allocP = [&](double*& p) {
        size_t pt;
        CR(cudaMallocPitch((void**)&p, &pt, width + PADC, height + PADR));
        CR(cudaMemset2D(p, pt, 0, width + PADC, height + PADR));
        pitch = pt;
    };
    double *w, *hu, *hv, *w_old, *hu_old, *hv_old, *G, *dw, *dhu, *dhv, *BCd, *BXd, *BYd;
    double *hmap, *qmap, *rain, *drain, *surge, *F, *F_old, *dF, *K, *n, *h_max, *q_max, *t_peak,
        *t_dry, *t_wet;
    double *rain0, *rain1, *drain0, *drain1, *surge0, *surge1;
    for (double** p : {&w, &hu, &hv, &w_old, &hu_old, &hv_old, &G, &dw, &dhu, &dhv, &BCd, &hmap,
                       &qmap, &rain, &drain, &surge, &F, &F_old, &dF, &K, &n, &h_max, &q_max,
                       &t_peak, &t_dry, &t_wet, &rain0, &rain1, &drain0, &drain1, &surge0, &surge1})
        allocP(*p);
    CR(cudaMallocPitch((void**)&BXd, &pitchBX, width_p1 + PADC, height + PADR));
    CR(cudaMemset2D(BXd, pitchBX, 0, width_p1 + PADC, height + PADR));
    CR(cudaMallocPitch((void**)&BYd, &pitchBY, width + PADC, height_p1 + PADR));
    CR(cudaMemset2D(BYd, pitchBY, 0, width + PADC, height_p1 + PADR));

    dim3 GridDim(nBX, nBY);
    dim3 GrowGrid((unsigned)std::ceil((double)nBX / BC_), (unsigned)std::ceil((double)nBY / BR_));
    size_t GrowGridSize = (size_t)(GrowGrid.x * BC_) * (GrowGrid.y * BR_);
    bool* wet_blocks;
    int* active_blocks;
    double *mx, *my;
    CR(cudaMalloc(&wet_blocks, GrowGridSize));
    CR(cudaMalloc(&active_blocks, GrowGridSize * 4));
    CR(cudaMalloc(&mx, GrowGridSize * 8));
    CR(cudaMalloc(&my, GrowGridSize * 8));
    CR(cudaMemset(wet_blocks, 0, GridSize));
    CR(cudaMemset(active_blocks, 0xFF, GridSize * 4));
    CR(cudaMemset(mx, 0, GridSize * 8));
    CR(cudaMemset(my, 0, GridSize * 8));

    // ---- uploads (simulator.cu:433-450)
    const size_t N = (size_t)nx * ny;
    auto up = [&](double* d, const std::vector<double>& h, size_t cols, size_t rows, size_t pt) {
        CR(cudaMemcpy2D(d, pt, h.data(), cols * 8, cols * 8, rows, cudaMemcpyHostToDevice));
    };
    up(BXd, readBin<double>(dir + "/BX.bin", (size_t)ny * (nx + 1)), nx + 1, ny, pitchBX);
    up(BYd, readBin<double>(dir + "/BY.bin", (size_t)(ny + 1) * nx), nx, ny + 1, pitchBY);
    up(n, readBin<double>(dir + "/n.bin", N), nx, ny, pitch);
    if (infil) up(K, readBin<double>(dir + "/K.bin", N), nx, ny, pitch);
    if (hInit) up(hmap, readBin<double>(dir + "/h0.bin", N), nx, ny, pitch);
    int mrain = (int)geti("map_rain", 0), mdrain = (int)geti("map_drain", 0),
        msurge = (int)geti("map_surge", 0);
    double frain = getd("factor_rain", 0), fdrain = getd("factor_drain", 0),
           fsurge = getd("factor_surge", 0);
    CUfunction kFill = fn("FillGrid_k"), kInterp = fn("InterpGrid_k");
    if (msurge) {  // surge maps default to nodata (GridSeries allow_no_data)
        for (double* p : {surge, surge0, surge1}) {
            void* a[] = {&p, &pitch, (void*)&nodata};
            CK(cuLaunchKernel(kFill, GridDim.x, GridDim.y, 1, BC_, BR_, 1, 0, 0, a, 0));
        }
    }
    auto loadMap = [&](int m, const char* base, double* cur, double* t0, double* t1) {
        if (!m) return;
        std::string b(base);
        up(t0, readBin<double>(dir + "/" + b + "_t0.bin", N), nx, ny, pitch);
        if (m == 1) {
            up(cur, readBin<double>(dir + "/" + b + "_t0.bin", N), nx, ny, pitch);
        } else {
            up(t1, readBin<double>(dir + "/" + b + "_t1.bin", N), nx, ny, pitch);
        }
    };
    loadMap(mrain, "rain", rain, rain0, rain1);
    loadMap(mdrain, "drain", drain, drain0, drain1);
    loadMap(msurge, "surge", surge, surge0, surge1);
    // Interpolated maps: a fixed factor, or (map_times_<name> "t0 t1") the
    // factor (t - t0) / (t1 - t0) of InterpolatedGridSeries::update
    // (GridSeries.cu:393-398), evaluated with the time reached after each step
    // (simulator.cu:819-828) and at the start (simulator.cu:352-370).
    auto mapTimes = [&](const char* name, double& a, double& b) {
        std::string k = std::string("map_times_") + name;
        if (!P.count(k)) return false;
        std::istringstream ss(P[k]);
        ss >> a >> b;
        return b > a;
    };
    double trn0 = 0, trn1 = 0, tdr0 = 0, tdr1 = 0, tsg0 = 0, tsg1 = 0;
    const bool timedRain = mapTimes("rain", trn0, trn1), timedDrain = mapTimes("drain", tdr0, tdr1),
               timedSurge = mapTimes("surge", tsg0, tsg1);
    double tNow = getd("t0", 0.0);
    auto interpMaps = [&]() {
        auto one = [&](int m, double f, double* t0, double* t1, double* cur) {
            if (m != 2) return;
            void* a[] = {&f, &pitch, &t0, &t1, &cur};
            CK(cuLaunchKernel(kInterp, GridDim.x, GridDim.y, 1, BC_, BR_, 1, 0, 0, a, 0));
        };
        if (timedRain) frain = (tNow - trn0) / (trn1 - trn0);
        if (timedDrain) fdrain = (tNow - tdr0) / (tdr1 - tdr0);
        if (timedSurge) fsurge = (tNow - tsg0) / (tsg1 - tsg0);
        one(mrain, frain, rain0, rain1, rain);
        one(mdrain, fdrain, drain0, drain1, drain);
        one(msurge, fsurge, surge0, surge1, surge);
    };

    // sources
    int nsrc = (int)geti("nsrc", 0);
    auto srcIdxH = readBin<int>(dir + "/src_idx.bin", nsrc, nsrc > 0);
    std::vector<double> srcRateH(nsrc, 0.0);
    int* srcIdx = nullptr;
    double* srcRate = nullptr;
    CR(cudaMalloc(&srcIdx, std::max(nsrc, 1) * 4));
    CR(cudaMalloc(&srcRate, std::max(nsrc, 1) * 8));
    CR(cudaMemset(srcRate, 0, std::max(nsrc, 1) * 8));
    Series ser[3];
    for (int s = 0; s < 3; s++) {
        int ns = (int)geti(("series" + std::to_string(s)).c_str(), 0);
        if (ns > 0) {
            ser[s].time = readBin<float>(dir + "/series" + std::to_string(s) + "_t.bin", ns);
            ser[s].rate = readBin<float>(dir + "/series" + std::to_string(s) + "_r.bin", ns);
            ser[s].on = true;
        }
    }
    // fixed uniform rates when no series is given
    double rainRateFixed = getd("rain_rate", 0), drainRateFixed = getd("drain_rate", 0);
    std::vector<double> srcRateFixed;
    if (nsrc > 0 && !ser[2].on) srcRateFixed = readBin<double>(dir + "/src_rate.bin", nsrc);

    CUfunction kInit = fn("InitGrid_k"), kFlux = fn("ComputeFluxes_k"),
               kInt1 = fn("Integrate_1_k"), kInt2 = fn("Integrate_2_k"), kGrow = fn("Grow_k"),
               kBX = fn("ApplyBoundariesX_k"), kBY = fn("ApplyBoundariesY_k"),
               kTrackR = fn("TrackRainfall_k"), kTrackS = fn("TrackSurge_k");

    {  // InitGrid_k
        void* a[] = {&w,  &hu, &hv,         &w_old,         &hu_old,  &hv_old,  &BCd,    &BXd, &BYd,
                     &wet_blocks, &active_blocks, &pitch, &pitchBX, &pitchBY, &hmap, &t_wet, &G};
        CK(cuLaunchKernel(kInit, GridDim.x, GridDim.y, 1, BC_, BR_, 1, 0, 0, a, 0));
    }
    unsigned gX = (unsigned)std::ceil((double)ny / 48.0), gY = (unsigned)std::ceil((double)nx / 48.0);
    auto applyBC = [&]() {
        void* a[] = {&w, &hu, &hv, &BCd, &pitch};
        CK(cuLaunchKernel(kBX, gX, 1, 1, 48, 1, 1, 0, 0, a, 0));
        CK(cuLaunchKernel(kBY, gY, 1, 1, 48, 1, 1, 0, 0, a, 0));
    };
    applyBC();

    double t = getd("t0", 0.0), dt = (double)0.0000001f;
    if (P.count("dt0")) dt = getd("dt0", dt);
    if (geti("state", 0)) {
        // hotstart-like state: Simulator::ReadHotstart (simulator.cu:975-1090)
        // then ApplyBoundaries (simulator.cu:731)
        up(w, readBin<double>(dir + "/state_w.bin", N), nx, ny, pitch);
        up(hu, readBin<double>(dir + "/state_hu.bin", N), nx, ny, pitch);
        up(hv, readBin<double>(dir + "/state_hv.bin", N), nx, ny, pitch);
        if (infil) up(F, readBin<double>(dir + "/state_F.bin", N), nx, ny, pitch);
        auto wb = readBin<unsigned char>(dir + "/state_wet.bin", GridSize);
        CR(cudaMemcpy(wet_blocks, wb.data(), GridSize, cudaMemcpyHostToDevice));
        int na = (int)geti("state_nactive", 0);
        auto ids = readBin<int>(dir + "/state_active.bin", na);
        std::vector<int> enc(GridSize);
        std::vector<char> on(GridSize, 0);
        for (int k = 0; k < na; k++) on[ids[k]] = 1;
        for (int b = 0; b < GridSize; b++) enc[b] = on[b] ? b : -b;
        CR(cudaMemcpy(active_blocks, enc.data(), GridSize * 4, cudaMemcpyHostToDevice));
        nBlocks = na;
        auto m1 = readBin<double>(dir + "/state_mx.bin", GridSize);
        auto m2 = readBin<double>(dir + "/state_my.bin", GridSize);
        CR(cudaMemcpy(mx, m1.data(), GridSize * 8, cudaMemcpyHostToDevice));
        CR(cudaMemcpy(my, m2.data(), GridSize * 8, cudaMemcpyHostToDevice));
        applyBC();
    }
    tNow = t;
    interpMaps();
    double rainRate = rainRateFixed, drainRate = drainRateFixed;
    long numSources = nsrc;
    if (nsrc > 0) CR(cudaMemcpy(srcIdx, srcIdxH.data(), nsrc * 4, cudaMemcpyHostToDevice));

    auto dump = [&](int step) {
        char pre[64];
        std::snprintf(pre, sizeof pre, "/s%05d_", step);
        std::vector<double> buf(N);
        auto dl = [&](double* d, const char* nm) {
            CR(cudaMemcpy2D(buf.data(), nx * 8, d, pitch, nx * 8, ny, cudaMemcpyDeviceToHost));
            writeBin(out + pre + nm + ".bin", buf.data(), N);
        };
        dl(w, "w");
        dl(hu, "hu");
        dl(hv, "hv");
        if (infil) dl(F, "F");
        if (saveMax) {
            dl(h_max, "hmax");
            dl(q_max, "qmax");
        }
        if (saveArr) dl(t_wet, "twet");
        if (geti("dump_bc", 1)) dl(BCd, "BC");
        std::vector<unsigned char> wb(GridSize);
        CR(cudaMemcpy(wb.data(), wet_blocks, GridSize, cudaMemcpyDeviceToHost));
        writeBin(out + pre + "wet.bin", wb.data(), GridSize);
        std::vector<int> ab(GridSize);
        CR(cudaMemcpy(ab.data(), active_blocks, GridSize * 4, cudaMemcpyDeviceToHost));
        std::vector<int> act(ab.begin(), ab.begin() + nBlocks);
        std::sort(act.begin(), act.end());
        writeBin(out + pre + "active.bin", act.data(), act.size());
        std::vector<double> m(GridSize);
        CR(cudaMemcpy(m.data(), mx, GridSize * 8, cudaMemcpyDeviceToHost));
        writeBin(out + pre + "mx.bin", m.data(), GridSize);
        CR(cudaMemcpy(m.data(), my, GridSize * 8, cudaMemcpyDeviceToHost));
        writeBin(out + pre + "my.bin", m.data(), GridSize);
        double td[2] = {t, dt};
        writeBin(out + pre + "t.bin", td, 2);
    };
    if (std::find(dumps.begin(), dumps.end(), 0) != dumps.end()) dump(0);

    FILE* log = std::fopen((out + "/steps.txt").c_str(), "w");
    long cellsActive = 0;
    // One step in the order of Simulator::RunSimulation (simulator.cu:773-853).
    auto doStep = [&]() {
        // UpdateSource (simulator.cu:500-538)
        if (dambreak || rainU || drainU) {
            if (nsrc > 0) CR(cudaMemcpy(srcIdx, srcIdxH.data(), nsrc * 4, cudaMemcpyHostToDevice));
            if (dambreak) {
                if (ser[2].on) {
                    ser[2].interpolate((float)t);
                    ser[2].interp /= 35.3147f;
                    for (int k = 0; k < nsrc; k++)
                        srcRateH[k] = (double)ser[2].interp / dx / dy / (double)numSources;
                } else {
                    srcRateH = srcRateFixed;
                }
                if (nsrc > 0) CR(cudaMemcpy(srcRate, srcRateH.data(), nsrc * 8, cudaMemcpyHostToDevice));
            }
            if (rainU && ser[0].on) {
                ser[0].interpolate((float)t);
                ser[0].interp /= (3600.f * 1000.f);
                rainRate = (double)ser[0].interp;
            }
            if (drainU && ser[1].on) {
                ser[1].interpolate((float)t);
                ser[1].interp /= (3600.f * 1000.f);
                drainRate = (double)ser[1].interp;
            }
        }
        // Grow (grid.cu:1279-1322)
        thrust::device_ptr<int> dpa = thrust::device_pointer_cast(active_blocks);
        if (rainG || surgeG) {
            thrust::partition(dpa, dpa + GridSize, is_neg());
            int nneg = (int)thrust::count_if(dpa, dpa + GridSize, is_neg());
            if (nneg > 0) {
                if (rainG) {
                    void* a[] = {&wet_blocks, &active_blocks, &rain, &pitch};
                    CK(cuLaunchKernel(kTrackR, nneg, 1, 1, BC_, BR_, 1, 0, 0, a, 0));
                }
                if (surgeG) {
                    void* a[] = {&wet_blocks, &active_blocks, &surge, &pitch};
                    CK(cuLaunchKernel(kTrackS, nneg, 1, 1, BC_, BR_, 1, 0, 0, a, 0));
                }
            }
        }
        {
            void* a[] = {&wet_blocks, &active_blocks};
            CK(cuLaunchKernel(kGrow, GrowGrid.x, GrowGrid.y, 1, BC_, BR_, 1, 0, 0, a, 0));
        }
        thrust::partition(dpa, dpa + GridSize, is_nonneg());
        nBlocks = (int)thrust::count_if(dpa, dpa + GridSize, is_nonneg());
        cellsActive += (long)nBlocks * BC_ * BR_;
        auto flux = [&](double dtArg) {
            void* a[] = {&w,     &hu,     &hv,      &dw,       &dhu,     &dhv,     &mx,     &my,
                         &BCd,   &BXd,    &BYd,     &G,        &active_blocks, &dtArg, &pitch,
                         &pitchBX, &pitchBY, &n,   &rainRate, &drainRate, &rain, &drain, &F,
                         &F_old, &dF,     &K,       &srcIdx,   &srcRate, &numSources};
            CK(cuLaunchKernel(kFlux, nBlocks, 1, 1, BC_, BR_, 1, 0, 0, a, 0));
        };
        flux(dt);
        // ComputeTimestep (simulator.cu:540-566)
        {
            thrust::device_ptr<double> mxp(mx), myp(my);
            double max_x = *thrust::max_element(mxp, mxp + GridSize);
            double max_y = *thrust::max_element(myp, myp + GridSize);
            double c_x = dx / fmaxf(max_x / courant, kappa);
            double c_y = dy / fmaxf(max_y / courant, kappa);
            dt = std::min(c_x, c_y);
            dt = (t == 0.f) ? 0.000001f : dt;
            t += dt;
        }
        {
            void* a[] = {&w,     &hu,     &hv,   &w_old, &hu_old, &hv_old, &dw,    &dhu,   &dhv,
                         &BCd,   &G,      &wet_blocks, &active_blocks, &t, &dt, &pitch, &rainRate,
                         &rain,  &surge,  &F,    &F_old, &dF,     &K,      &hmap,  &qmap,  &h_max,
                         &q_max, &t_wet,  &srcIdx, &srcRate, &numSources, &t_peak, &t_dry};
            CK(cuLaunchKernel(kInt1, nBlocks, 1, 1, BC_, BR_, 1, 0, 0, a, 0));
        }
        applyBC();
        if (!euler) {
            flux(dt);
            void* a[] = {&w,   &hu,    &hv,    &w_old, &hu_old, &hv_old,     &dw,           &dhu,
                         &dhv, &BCd,   &G,     &wet_blocks, &active_blocks, &t, &dt, &pitch,
                         &rainRate, &rain, &F, &F_old, &dF,     &K,          &hmap,         &qmap,
                         &h_max, &q_max, &t_wet, &srcIdx, &srcRate, &numSources};
            CK(cuLaunchKernel(kInt2, nBlocks, 1, 1, BC_, BR_, 1, 0, 0, a, 0));
            applyBC();
        }
        tNow = t;
        interpMaps();  // GridSeries::update
    };
    // Spin-up / logged part: nsteps steps, or fewer when t reaches t_stop.
    const double tStop = getd("t_stop", 1e300);
    const bool dumpFinal = geti("dump_final", 0) != 0;
    const int timedSteps = (int)geti("timed_steps", 0);
    cudaEvent_t e0, e1;
    CR(cudaEventCreate(&e0));
    CR(cudaEventCreate(&e1));
    CR(cudaDeviceSynchronize());
    auto wall0 = std::chrono::steady_clock::now();
    CR(cudaEventRecord(e0));
    int step = 0;
    while (step < nsteps && t < tStop) {
        step++;
        doStep();
        if (!timing) {
            std::fprintf(log, "%d %.17g %.17g %d\n", step, t, dt, nBlocks);
            if (std::find(dumps.begin(), dumps.end(), step) != dumps.end()) dump(step);
        }
    }
    CR(cudaEventRecord(e1));
    CR(cudaEventSynchronize(e1));
    auto wall1 = std::chrono::steady_clock::now();
    float ms = 0;
    CR(cudaEventElapsedTime(&ms, e0, e1));
    double wall = std::chrono::duration<double>(wall1 - wall0).count();
    std::fclose(log);
    const int stepsRun = step;
    if (dumpFinal) dump(stepsRun);
    const double tSpin = t;
    // Timed part: timed_steps more steps after the spin-up, CUDA events on
    // the legacy stream around them and the host clock around the loop
    // (thrust's host synchronisations of every step included, as in the
    // reference's main loop).
    float msTimed = 0.f;
    double wallTimed = 0.0;
    long cellsTimed = 0;
    if (timedSteps > 0) {
        const long c0 = cellsActive;
        CR(cudaDeviceSynchronize());
        auto w0 = std::chrono::steady_clock::now();
        CR(cudaEventRecord(e0));
        for (int k = 0; k < timedSteps; k++) doStep();
        CR(cudaEventRecord(e1));
        CR(cudaEventSynchronize(e1));
        wallTimed = std::chrono::duration<double>(std::chrono::steady_clock::now() - w0).count();
        CR(cudaEventElapsedTime(&msTimed, e0, e1));
        cellsTimed = cellsActive - c0;
    }
    long interior = (long)(nx - 4) * (ny - 4);
    if (timedSteps > 0) {
        std::printf(
            "{\"steps\": %d, \"t\": %.9g, \"dt\": %.9g, \"spinup_steps\": %d, \"t_spinup\": %.9g, "
            "\"spinup_wall_s\": %.3f, \"gpu_ms\": %.4f, \"wall_s\": %.6f, "
            "\"domain_cell_updates_per_s\": %.6g, \"active_tile_cells\": %ld, \"n_active_last\": %d}\n",
            timedSteps, t, dt, stepsRun, tSpin, wall, msTimed, wallTimed,
            (double)interior * timedSteps / wallTimed, cellsTimed, nBlocks);
    } else {
        std::printf(
            "{\"steps\": %d, \"t\": %.9g, \"dt\": %.9g, \"gpu_ms\": %.4f, \"wall_s\": %.6f, "
            "\"domain_cell_updates_per_s\": %.6g, \"active_tile_cells\": %ld, \"n_active_last\": %d}\n",
            stepsRun, t, dt, ms, wall, (double)interior * stepsRun / wall, cellsActive, nBlocks);
    }
    return 0;
}
