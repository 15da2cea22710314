"""Seeded synthetic inputs for the RIFT workloads, and the host-side static
field construction the reference performs in Simulator::InitSimulation.

All arrays use the reference's host layout: corner rasters are (b_ny, b_nx)
with row 0 the SOUTH edge (the ESRI reader flips rows so j grows north,
io.cc:79-91); h-grid arrays are (h_ny, h_nx) with h_nx = b_nx + 3
(grid_config.cpp:84-85).
"""
from __future__ import annotations

import dataclasses

import numpy as np

F32 = np.float32


def kappa_for(dx: float, dy: float) -> float:
    """Desingularisation constant, simulator.cu:281 (float arithmetic)."""
    m = np.minimum(F32(dx), F32(dy))
    return float(np.sqrt(F32(0.01) * np.maximum(F32(1.0), m)))


def faces_from_corners(B: np.ndarray):
    """BX / BY face elevations from the corner DEM (simulator.cu:384-431).

    B has shape (b_ny, b_nx).  Returns BX (h_ny, h_nx+1), BY (h_ny+1, h_nx),
    including the ghost-face copies the reference makes for i == 2,
    i == h_nx-3, j == 2, j == h_ny-3; every other ghost face stays 0.
    """
    b_ny, b_nx = B.shape
    h_nx, h_ny = b_nx + 3, b_ny + 3
    BX = np.zeros((h_ny, h_nx + 1))
    BY = np.zeros((h_ny + 1, h_nx))
    ll = B[:-1, :-1]
    ul = B[1:, :-1]
    ur = B[1:, 1:]
    lr = B[:-1, 1:]
    J = slice(2, h_ny - 2)
    I = slice(2, h_nx - 2)
    # west faces of cells i (column i) and east faces (column i+1)
    BX[J, 3:h_nx - 1] = 0.5 * (ur + lr)
    BX[J, 2:h_nx - 2] = 0.5 * (ll + ul)
    BY[3:h_ny - 1, I] = 0.5 * (ul + ur)
    BY[2:h_ny - 2, I] = 0.5 * (ll + lr)
    # ghost faces (order of the reference loop: bed/bwd written for i, then
    # copies for i == 2 and i == h_nx-3)
    BX[J, 1] = BX[J, 3]
    BX[J, 0] = BX[J, 2]
    BX[J, h_nx - 1] = BX[J, h_nx - 3]
    BY[1, I] = BY[3, I]
    BY[0, I] = BY[2, I]
    BY[h_ny - 1, I] = BY[h_ny - 3, I]
    return BX, BY


def cell_mean(C: np.ndarray) -> np.ndarray:
    """Corner -> interior cell mean, 0.25f*(ur+lr+ll+ul) (simulator.cu:416-428)."""
    b_ny, b_nx = C.shape
    out = np.zeros((b_ny + 3, b_nx + 3))
    ll = C[:-1, :-1]
    ul = C[1:, :-1]
    ur = C[1:, 1:]
    lr = C[:-1, 1:]
    out[2:-2, 2:-2] = 0.25 * (((ur + lr) + ll) + ul)
    return out


def coord2index(X, Y, h_xll, h_yll, cellsize_original):
    """GridConfig::Coord2Index (grid_config.cpp:104-115)."""
    i = int((X - h_xll) / cellsize_original + 0.5)
    j = int((Y - h_yll) / cellsize_original + 0.5)
    return i, j


@dataclasses.dataclass
class Case:
    """One workload: static fields on the h-grid plus run settings."""
    name: str
    B: np.ndarray                  # corner DEM (b_ny, b_nx)
    cell: float                    # metres (projected)
    n: np.ndarray                  # (h_ny, h_nx) Manning n per cell
    K: np.ndarray | None = None    # (h_ny, h_nx) m/s
    h0: np.ndarray | None = None   # (h_ny, h_nx) m
    psi: float = 0.0
    dtheta: float = 0.0
    courant: float = 0.25
    t0: float = 0.0
    tf: float = 3600.0
    flags: int = 0
    series: dict = dataclasses.field(default_factory=dict)  # which -> (times_s f32, rates f32)
    src_idx: np.ndarray | None = None
    rain_maps: list | None = None  # two (h_ny, h_nx) maps in m/s bracketing the run
    map_times: tuple | None = None  # (t0, t1) of those two maps
    map_dt: float = 0.0

    @property
    def b_nx(self):
        return self.B.shape[1]

    @property
    def b_ny(self):
        return self.B.shape[0]

    @property
    def h_nx(self):
        return self.b_nx + 3

    @property
    def h_ny(self):
        return self.b_ny + 3

    @property
    def kappa(self):
        return kappa_for(self.cell, self.cell)

    def faces(self):
        return faces_from_corners(self.B)


# flag bits (include/rift_gb300.h)
RAIN_UNIFORM, RAIN_GRID, DRAIN_UNIFORM, DRAIN_GRID = 1, 2, 4, 8
INFILTRATION, SURGE_GRID, EULER, SAVE_MAX = 16, 32, 64, 128
SAVE_ARRIVAL, TILE_ACCEL, POINT_SOURCE, H_INIT = 256, 512, 1024, 2048
CHECK_VOLUME = 4096


def csv_series(hours, rates):
    """Source::ReadSource (source.cc:11-63): hours -> seconds in float, a zero
    appended at last + mean spacing when the last rate is not zero."""
    t = [F32(h) * F32(60) * F32(60) for h in hours]
    r = [F32(x) for x in rates]
    if r[-1] != F32(0):
        est = F32(0)
        for i in range(1, len(t)):
            est = F32(est + F32(t[i] - t[i - 1]))
        est = F32(est / F32(F32(len(t)) - F32(1)))
        t.append(F32(t[-1] + est))
        r.append(F32(0))
    return np.array(t, dtype=F32), np.array(r, dtype=F32)


def gaussian_bumps(X, Y, rng, count, amp, sigma, extent):
    z = np.zeros_like(X)
    for _ in range(count):
        a = rng.uniform(*amp)
        s = rng.uniform(*sigma)
        cx = rng.uniform(0, extent)
        cy = rng.uniform(0, extent)
        z += a * np.exp(-((X - cx) ** 2 + (Y - cy) ** 2) / (2.0 * s * s))
    return z


def config1(N=512, seed=0, cell=10.0, rim=True, tf=3600.0) -> Case:
    """Plain method, small: N x N cells at 10 m; plane dropping 0.001 toward
    +x plus 20 Gaussian bumps (amplitude U(1,8) m, sigma U(50,300) m); n =
    0.035; h0 = 0; uniform hyetograph 50 mm/hr for 0-1800 s then 0.

    The reference has no reflective boundary; `rim` raises the outer two
    corner rows/columns by 100 m so the domain is closed for both codes.
    """
    rng = np.random.default_rng(seed)
    x = np.arange(N + 1) * cell
    X, Y = np.meshgrid(x, x)
    extent = N * cell
    z = 20.0 - 0.001 * X + gaussian_bumps(X, Y, rng, 20, (1, 8), (50, 300), extent)
    if rim:
        z[:2, :] += 100.0
        z[-2:, :] += 100.0
        z[:, :2] += 100.0
        z[:, -2:] += 100.0
    b = z.shape
    n = np.zeros((b[0] + 3, b[1] + 3))
    n[2:-2, 2:-2] = 0.035
    t, r = csv_series([0, 0.5, 0.5, 1], [50, 50, 0, 0])
    return Case(name=f"config1_{N}", B=z, cell=cell, n=n, tf=tf,
                flags=RAIN_UNIFORM | TILE_ACCEL, series={0: (t, r)})


def _fft_len(n):
    """Smallest FFT length >= n with only small prime factors."""
    import scipy.fft as sf
    return sf.next_fast_len(int(n))


def fractal_surface(N, hurst, relief, rng):
    """Spectral (1/f^(H+1)) random surface on an (N+1)^2 corner grid: the
    field is synthesised on a periodic grid of a fast FFT length >= N+1 and
    cropped to the corner grid."""
    import scipy.fft as sf
    M = N + 1
    L = _fft_len(M)
    kx = np.fft.fftfreq(L)
    k = np.sqrt(kx[None, :] ** 2 + kx[:, None] ** 2)
    k[0, 0] = 1.0
    amp = k ** (-(hurst + 1.0))
    amp[0, 0] = 0.0
    phase = rng.uniform(0, 2 * np.pi, size=(L, L))
    spec = amp * np.exp(1j * phase)
    z = np.ascontiguousarray(np.real(sf.ifft2(spec, workers=-1))[:M, :M])
    z -= z.min()
    z *= relief / max(z.max(), 1e-12)
    return z


def config2(N=2048, seed=1, cell=5.0, tf=21600.0) -> Case:
    """Mostly dry point-source flood: fractal (Hurst 0.8, 40 m relief) with a
    20 m wide, 3 m deep meandering channel; triangular hydrograph 0 -> 500 cfs
    at 1 h -> 0 at 3 h at the channel head; n 0.03 / 0.08; Green-Ampt with
    lognormal K (median 5 mm/hr, sigma_ln 0.8), psi 0.11 m, dtheta 0.3."""
    rng = np.random.default_rng(seed)
    z = fractal_surface(N, 0.8, 40.0, rng) + 5.0
    x = np.arange(N + 1) * cell
    X, Y = np.meshgrid(x, x)
    # meander: centreline y = y0 + A sin(2 pi x / L), descending toward +x
    L = N * cell
    yc = 0.5 * L + 0.15 * L * np.sin(2 * np.pi * X / (0.6 * L))
    chan = np.abs(Y - yc) < 10.0
    # channel bed follows a smooth downstream slope below the local minimum
    zc = z.copy()
    zc[chan] = np.minimum(z[chan], (z.mean() + 10.0 - 0.004 * X[chan])) - 3.0
    z = zc
    nC = np.where(chan, 0.03, 0.08)
    Kc = np.exp(np.log(5.0) + 0.8 * rng.standard_normal(z.shape))  # mm/hr at corners
    b = z.shape
    from_c = cell_mean
    n = from_c(nC)
    K = from_c(Kc) / (3600.0 * 1000.0)
    # channel head: first channel cell column near x = 2 cells
    i_head = 4
    j_head = int(round(yc[0, i_head] / cell))
    h_nx = b[1] + 3
    # source cell index on the h-grid (the reference's -2-cell offset of
    # Coord2Index is applied by whoever converts coordinates; here the cell
    # is chosen directly on the h-grid)
    src = np.array([(j_head + 2) * h_nx + (i_head + 2)], dtype=np.int32)
    t, r = csv_series([0, 1, 3], [0, 500, 0])
    return Case(name=f"config2_{N}", B=z, cell=cell, n=n, K=K, psi=0.11, dtheta=0.3,
                tf=tf, flags=INFILTRATION | POINT_SOURCE | TILE_ACCEL,
                series={2: (t, r)}, src_idx=src)


def config3(N=8192, seed=2, cell=2.0, tf=10800.0, nblocks=4000) -> Case:
    """Large urban rainfall domain: fractal (15 m relief) + building blocks
    raised 10 m (10-40 m sides); uniform drain 5 mm/hr; n 0.015 / 0.05.
    Rain maps are produced separately (config3_rain_maps)."""
    rng = np.random.default_rng(seed)
    z = fractal_surface(N, 0.8, 15.0, rng) + 5.0
    M = N + 1
    roof = np.zeros(z.shape, dtype=bool)
    for _ in range(nblocks):
        w = int(rng.uniform(10, 40) / cell)
        hgt = int(rng.uniform(10, 40) / cell)
        i0 = int(rng.uniform(0, M - w))
        j0 = int(rng.uniform(0, M - hgt))
        roof[j0:j0 + hgt, i0:i0 + w] = True
    z = z + 10.0 * roof
    nC = np.where(roof, 0.015, 0.05)
    n = cell_mean(nC)
    t, r = csv_series([0, 3], [5, 5])
    case = Case(name=f"config3_{N}", B=z, cell=cell, n=n, tf=tf,
                flags=RAIN_GRID | DRAIN_UNIFORM | TILE_ACCEL, series={1: (t, r)}, map_dt=300.0)
    # the first two of the rain maps (every 300 s), interpolated in time
    maps = []
    for k in range(2):
        mm = rain_map_corners(z.shape, cell, np.random.default_rng(1000 + seed * 100 + k))
        maps.append(cell_mean(mm) / (3600.0 * 1000.0))
    case.rain_maps = maps
    case.map_times = (0.0, 300.0)
    return case


def config5(members=128, side=(256, 2048), seed=0, cell=5.0, tf=14400.0) -> list:
    """Batched ensemble: members on square domains of uneven size (side
    uniform in `side` cells at 5 m), each with its own fractal DEM (seed =
    member id); per member a uniform rain of lognormal scale (median 40
    mm/hr, sigma_ln 0.5) lasting 1-3 h; every second member also has a
    point hydrograph of 100-800 cfs (triangular, peak at 1 h, over 3 h) at
    the domain's lowest interior corner point."""
    rng = np.random.default_rng(seed)
    cases = []
    for m in range(members):
        N = int(rng.integers(side[0], side[1] + 1))
        mr = np.random.default_rng(m)
        z = fractal_surface(N, 0.8, 20.0, mr) + 5.0
        z[:2, :] += 30.0
        z[-2:, :] += 30.0
        z[:, :2] += 30.0
        z[:, -2:] += 30.0
        n = np.zeros((N + 4, N + 4))
        n[2:-2, 2:-2] = 0.035
        rate = float(np.exp(np.log(40.0) + 0.5 * rng.standard_normal()))
        hours = float(rng.uniform(1.0, 3.0))
        series = {0: csv_series([0, hours, hours, 4], [rate, rate, 0, 0])}
        flags = RAIN_UNIFORM | TILE_ACCEL
        src = None
        if m % 2 == 1:
            q = float(rng.uniform(100.0, 800.0))
            series[2] = csv_series([0, 1, 3], [0, q, 0])
            inner = z[4:-4, 4:-4]
            jj, ii = np.unravel_index(np.argmin(inner), inner.shape)
            src = np.array([(jj + 4 + 2) * (N + 4) + (ii + 4 + 2)], dtype=np.int32)
            flags |= POINT_SOURCE
        cases.append(Case(name=f"member{m}_{N}", B=z, cell=cell, n=n, tf=tf, flags=flags,
                          series=series, src_idx=src))
    return cases


def smooth_field(shape, corr_cells, rng):
    """Gaussian random field with Gaussian correlation (FFT filter on a
    periodic grid of fast FFT lengths, cropped to `shape`), unit variance."""
    import scipy.fft as sf
    ny, nx = shape
    Ly, Lx = _fft_len(ny), _fft_len(nx)
    ky = np.fft.fftfreq(Ly)
    kx = np.fft.rfftfreq(Lx)
    filt = np.exp(-2.0 * (np.pi ** 2) * (corr_cells ** 2) * (kx[None, :] ** 2 + ky[:, None] ** 2))
    noise = rng.standard_normal((Ly, Lx))
    f = sf.irfft2(sf.rfft2(noise, workers=-1) * filt, s=(Ly, Lx), workers=-1)[:ny, :nx]
    f = f - f.mean()
    s = f.std()
    return f / (s if s > 0 else 1.0)


def rain_map_corners(shape, cell, rng, mean=40.0, sigma=15.0, corr_m=500.0):
    """One rain-rate map in mm/hr on the corner grid, clipped at 0."""
    f = mean + sigma * smooth_field(shape, corr_m / cell, rng)
    return np.clip(f, 0.0, None)


def small_case(nx_cells=40, ny_cells=36, seed=7, cell=10.0, flags=None, rain_mmhr=50.0,
               h0_depth=0.0, rim=False) -> Case:
    """A small bumpy-plane case used by the parity tests."""
    rng = np.random.default_rng(seed)
    xs = np.arange(nx_cells + 1) * cell
    ys = np.arange(ny_cells + 1) * cell
    X, Y = np.meshgrid(xs, ys)
    ext = max(nx_cells, ny_cells) * cell
    z = 20.0 - 0.002 * X + 0.001 * Y + gaussian_bumps(X, Y, rng, 6, (0.5, 3), (20, 80), ext)
    if rim:
        z[:2, :] += 50.0
        z[-2:, :] += 50.0
        z[:, :2] += 50.0
        z[:, -2:] += 50.0
    n = np.zeros((ny_cells + 4, nx_cells + 4))
    n[2:-2, 2:-2] = 0.03
    fl = (RAIN_UNIFORM | TILE_ACCEL) if flags is None else flags
    case = Case(name="small", B=z, cell=cell, n=n, flags=fl)
    t, r = csv_series([0, 0.25, 0.5], [rain_mmhr, rain_mmhr, 0])
    case.series = {0: (t, r)}
    if h0_depth > 0:
        h0 = np.zeros_like(n)
        h0[2:-2, 2:-2] = h0_depth * rng.uniform(0.0, 1.0, size=(ny_cells, nx_cells))
        case.h0 = h0
        case.flags |= H_INIT
    return case
