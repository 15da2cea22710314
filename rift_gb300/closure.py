"""Learned sub-grid flux closure: host side over librift_closure.so.

The closure lets a grid coarsened 2x reproduce a fine run.  A three-layer
convolutional net (include/rift_closure.h) reads (h, hu, hv, b, n, rain)
around each coarse cell and predicts corrections to the mass and normal
momentum fluxes through the cell's east and north faces.  Between steps of
the plain coarse solve the corrections are applied as antisymmetric face
fluxes, so they move volume between cells without creating or destroying it.

Training targets come from the solver itself.  For a synthetic scenario,
the fine run is restricted to the coarse grid at a sample time (2x2 means of
h, hu, hv).  The coarse handle starts from that state.  Over a window both
runs integrate the central-upwind flux through every coarse face (the fine
run through the two fine faces that make it up).  The target is the fine
time-mean flux minus the coarse one: the part of the flux the coarse grid
misses.

PyTorch is used here as device memory only: tensors hold features, targets,
parameters and Adam moments, and their pointers go through the C ABI.  Every
kernel is in rift_gb300/csrc/rift_closure.cu.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import os
import time

import numpy as np

from . import capi, synth

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "librift_closure.so")

NPARAM = 14664
OFF_W1, OFF_B1, OFF_W2, OFF_B2, OFF_W3, OFF_B3 = 0, 5120, 5152, 14368, 14400, 14656
HALO = 3          # input cells beyond an output block on each side
PATCH = 64        # output cells per training patch side
RAIN_SCALE = 1.0 / (50.0 / 3.6e6)  # 50 mm/hr -> 1


class Src(C.Structure):
    """rift_closure_src (include/rift_closure.h)."""
    _fields_ = [("plane", C.c_void_p * 6), ("value", C.c_float * 6), ("scale", C.c_float * 6),
                ("sample_stride", C.c_int64), ("pitch", C.c_int32), ("H", C.c_int32),
                ("W", C.c_int32), ("oy0", C.c_int32), ("ox0", C.c_int32), ("OH", C.c_int32),
                ("OW", C.c_int32), ("samples", C.c_int32)]


_lib = None


def load():
    """The closure library; fails loudly when it is not built (no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise capi.RiftError(f"closure extension not built: {LIB_PATH} missing (run build())")
        lib = C.CDLL(LIB_PATH)
        P, F, I = C.c_void_p, C.c_float, C.c_int32
        sig = {
            "rift_closure_forward": [C.POINTER(Src), P, P, P],
            "rift_closure_train": [C.POINTER(Src), P, P, P, F, P, P, P],
            "rift_closure_adam": [P, P, P, P, I, F, F, F, F, F, F, P],
            "rift_closure_face_flux": [C.POINTER(capi.DeviceView), I, F, P, I, I, I, I],
            "rift_closure_apply": [C.POINTER(capi.DeviceView), C.POINTER(Src), P,
                                   C.POINTER(C.c_float), F, F, F, F, P, P, P],
            "rift_closure_selftest": [P, P],
            "rift_closure_check": [P],
        }
        for name, args in sig.items():
            fn = getattr(lib, name)
            fn.restype = C.c_int
            fn.argtypes = args
        lib.rift_closure_last_error.restype = C.c_char_p
        lib.rift_closure_last_error.argtypes = []
        _lib = lib
    return _lib


def _check(rc, what):
    if rc != capi.RIFT_OK:
        msg = load().rift_closure_last_error().decode()
        raise capi.RiftError(f"{what} failed: {capi.ERRORS.get(rc, rc)} {msg}")


def _torch():
    import torch
    return torch


def _stream():
    return C.c_void_p(_torch().cuda.current_stream().cuda_stream)


# --------------------------------------------------------------- parameters
def init_params(seed: int = 0) -> np.ndarray:
    """He-normal layers 1 and 2, layer 3 scaled by 0.1 (the net starts near
    zero corrections), zero biases, in the C layout."""
    rng = np.random.default_rng(seed)
    p = np.zeros(NPARAM, dtype=np.float32)
    w1 = np.zeros((32, 160), np.float32)
    w1[:, :150] = rng.standard_normal((32, 150)) * np.sqrt(2.0 / 150)
    p[OFF_W1:OFF_B1] = w1.ravel()
    p[OFF_W2:OFF_B2] = (rng.standard_normal((32, 288)) * np.sqrt(2.0 / 288)).ravel()
    w3 = np.zeros((8, 32), np.float32)
    w3[:4] = rng.standard_normal((4, 32)) * np.sqrt(1.0 / 32) * 0.1
    p[OFF_W3:OFF_B3] = w3.ravel()
    return p


def unpack(p):
    """Parameter vector -> torch conv2d weights (W1 [32,6,5,5], b1, W2
    [32,32,3,3], b2, W3 [4,32,1,1], b3); p is a numpy array or tensor."""
    torch = _torch()
    p = torch.as_tensor(p, dtype=torch.float32)
    W1 = p[OFF_W1:OFF_B1].view(32, 160)[:, :150].view(32, 5, 5, 6).permute(0, 3, 1, 2)
    W2 = p[OFF_W2:OFF_B2].view(32, 3, 3, 32).permute(0, 3, 1, 2)
    W3 = p[OFF_W3:OFF_B3].view(8, 32)[:4].view(4, 32, 1, 1)
    return W1, p[OFF_B1:OFF_W2], W2, p[OFF_B2:OFF_W3], W3, p[OFF_B3:OFF_B3 + 4]


def torch_forward(x, p):
    """FP32 PyTorch statement of the net on patches x (S, 6, H, W) of scaled
    inputs, valid convolutions: channel 3 enters relative to the bed of each
    layer-1 window's centre cell.  Output (S, 4, H-6, W-6)."""
    torch = _torch()
    F = torch.nn.functional
    # true FP32: PyTorch's defaults let cuDNN convolutions run on TF32
    prev = (torch.backends.cudnn.allow_tf32, torch.backends.cuda.matmul.allow_tf32)
    torch.backends.cudnn.allow_tf32 = False
    torch.backends.cuda.matmul.allow_tf32 = False
    try:
        W1, b1, W2, b2, W3, b3 = unpack(p.to(x.device))
        z1 = F.conv2d(x, W1) - x[:, 3:4, 2:-2, 2:-2] * W1[:, 3].sum(dim=(1, 2)).view(1, -1, 1, 1)
        a1 = torch.relu(z1 + b1.view(1, -1, 1, 1))
        a2 = torch.relu(F.conv2d(a1, W2) + b2.view(1, -1, 1, 1))
        return F.conv2d(a2, W3) + b3.view(1, -1, 1, 1)
    finally:
        torch.backends.cudnn.allow_tf32, torch.backends.cuda.matmul.allow_tf32 = prev


# ------------------------------------------------------------ device calls
def patch_src(feats, scale):
    """Src over a contiguous (S, 6, H, W) FP32 CUDA tensor of patches."""
    S, ch, H, W = feats.shape
    assert ch == 6 and feats.is_contiguous() and feats.dtype == _torch().float32
    s = Src()
    base = feats.data_ptr()
    for c in range(6):
        s.plane[c] = base + c * H * W * 4
        s.value[c] = 0.0
        s.scale[c] = float(scale[c])
    s.sample_stride, s.pitch, s.H, s.W = 6 * H * W, W, H, W
    s.oy0 = s.ox0 = HALO
    s.OH, s.OW, s.samples = H - 2 * HALO, W - 2 * HALO, S
    return s


def forward(feats, params, scale):
    """Raw net outputs (S, 4, H-6, W-6) of the patches feats."""
    torch = _torch()
    src = patch_src(feats, scale)
    out = torch.empty((src.samples, 4, src.OH, src.OW), device=feats.device, dtype=torch.float32)
    _check(load().rift_closure_forward(C.byref(src), params.data_ptr(), out.data_ptr(), _stream()),
           "rift_closure_forward")
    check(_stream())
    return out


def check(stream=None):
    """Wait for `stream` and raise if a tensor-core completion wait of the
    closure kernels gave up (rift_closure_check)."""
    _check(load().rift_closure_check(stream), "rift_closure_check")


def train_pass(feats, params, scale, target, weight, loss_scale, grad, loss):
    src = patch_src(feats, scale)
    _check(load().rift_closure_train(C.byref(src), params.data_ptr(), target.data_ptr(),
                                     weight.data_ptr(), float(loss_scale), grad.data_ptr(),
                                     loss.data_ptr(), _stream()), "rift_closure_train")


def adam(params, grad, m, v, step, lr, beta1=0.9, beta2=0.999, eps=1e-8):
    _check(load().rift_closure_adam(params.data_ptr(), grad.data_ptr(), m.data_ptr(), v.data_ptr(),
                                    params.numel(), lr, beta1, beta2, eps, 1.0 - beta1 ** step,
                                    1.0 - beta2 ** step, _stream()), "rift_closure_adam")


def face_flux(view, ratio, weight, acc, acc_nx, acc_ny):
    """acc (4, rows, pitch) += weight x face fluxes of view's U^n (on view's stream)."""
    _check(load().rift_closure_face_flux(C.byref(view), ratio, float(weight), acc.data_ptr(),
                                         acc.shape[2], acc.shape[1], acc_nx, acc_ny),
           "rift_closure_face_flux")


# ---------------------------------------------------------------- geometry
def coarse_case(fine: synth.Case) -> synth.Case:
    """The 2x-coarsened case: every other DEM corner, cell doubled, n (and K)
    as 2x2 means of the fine cells; same sources and settings."""
    N = fine.b_nx - 1
    assert N % 2 == 0 and fine.b_ny == fine.b_nx
    B = fine.B[::2, ::2].copy()

    def restrict_cells(a):
        if a is None:
            return None
        out = np.zeros((B.shape[0] + 3, B.shape[1] + 3))
        out[2:-2, 2:-2] = restrict(a[2:-2, 2:-2])
        return out

    src = None
    if fine.src_idx is not None:
        # a point source stays a volume rate at the coarse cell holding it
        ny_c, nx_c = B.shape[0] + 3, B.shape[1] + 3
        j, i = np.divmod(np.asarray(fine.src_idx, dtype=np.int64), fine.h_nx)
        J = np.clip(2 + (j - 2) // 2, 2, ny_c - 3)
        I = np.clip(2 + (i - 2) // 2, 2, nx_c - 3)
        src = (J * nx_c + I).astype(np.int32)
    return dataclasses.replace(fine, name=fine.name + "_coarse", B=B, cell=2.0 * fine.cell,
                               n=restrict_cells(fine.n), K=restrict_cells(fine.K),
                               h0=restrict_cells(fine.h0), src_idx=src, rain_maps=None)


def even_side(case: synth.Case) -> synth.Case:
    """The case cropped to an even number of cells per side (the last corner
    row and column dropped), so that it coarsens 2x."""
    N = case.b_nx - 1
    if N % 2 == 0:
        return case
    crop = lambda a: None if a is None else a[:-1, :-1].copy()
    src = None
    if case.src_idx is not None:
        j, i = np.divmod(np.asarray(case.src_idx, dtype=np.int64), case.h_nx)
        j, i = np.minimum(j, case.h_ny - 4), np.minimum(i, case.h_nx - 4)
        src = (j * (case.h_nx - 1) + i).astype(np.int32)
    return dataclasses.replace(case, B=case.B[:-1, :-1].copy(), n=crop(case.n), K=crop(case.K),
                               h0=crop(case.h0), src_idx=src)


def restrict(a):
    """2x2 means of an (2n, 2m) array."""
    n, m = a.shape[0] // 2, a.shape[1] // 2
    return a.reshape(n, 2, m, 2).mean(axis=(1, 3))


def face_mask(h, hmin):
    """(2, n, m) masks of the east and north faces of interior cells h (n, m)
    that the closure corrects: both cells deeper than hmin, both at least one
    cell inside the interior's edge."""
    n, m = h.shape
    wet = h > hmin
    inner = np.zeros_like(wet)
    inner[1:-1, 1:-1] = True
    ok = wet & inner
    east = np.zeros_like(wet)
    north = np.zeros_like(wet)
    east[:, :-1] = ok[:, :-1] & ok[:, 1:]
    north[:-1, :] = ok[:-1, :] & ok[1:, :]
    return east, north


def uniform_rate(case: synth.Case, t: float) -> float:
    """Uniform rain rate (m/s) of the case's hyetograph at time t (linear)."""
    if 0 not in case.series:
        return 0.0
    ts, rs = case.series[0]
    return float(np.interp(t, ts, rs)) / 3.6e6


def scenario(seed: int, N: int = 1024, cell: float = 2.0, tf: float = 3600.0) -> synth.Case:
    """A seeded rain scenario on a config-1 (plane and bumps) or config-2
    (fractal and channel) DEM, alternating by seed: uniform rain of
    U(30, 80) mm/hr for the first half hour, n from the generator."""
    rng = np.random.default_rng(10_000 + seed)
    if seed % 2 == 0:
        c = synth.config1(N=N, seed=seed, cell=cell, rim=True, tf=tf)
    else:
        c = synth.config2(N=N, seed=seed, cell=cell, tf=tf)
    r = float(rng.uniform(30.0, 80.0))
    t, rates = synth.csv_series([0, 0.5, 0.5, 1], [r, r, 0, 0])
    flags = synth.RAIN_UNIFORM | synth.TILE_ACCEL | synth.SAVE_MAX | synth.SAVE_ARRIVAL
    return dataclasses.replace(c, name=f"closure_s{seed}", K=None, psi=0.0, dtheta=0.0, flags=flags,
                               series={0: (t, rates)}, src_idx=None, tf=tf)


# --------------------------------------------------------- training data
@dataclasses.dataclass
class Dataset:
    feats: np.ndarray     # (P, 6, 70, 70) unscaled inputs
    target: np.ndarray    # (P, 4, 64, 64) flux corrections per unit width
    mask: np.ndarray      # (P, 4, 64, 64) 1 where the face is corrected


def _interior_fields(sim):
    """Interior h, hu, hv (FP64) of a handle."""
    w, bc = sim.field("W"), sim.field("BC")
    sl = (slice(2, -2), slice(2, -2))
    return (w - bc)[sl], sim.field("HU")[sl], sim.field("HV")[sl]


def _patches(planes, masks, targets, min_frac):
    """Cut (6, n, m) inputs into 64 x 64 output patches with a 3-cell halo
    (edge cells repeated past the interior), keeping patches with at least
    min_frac of their faces corrected."""
    n, m = planes.shape[1:]
    out = []
    for y0 in range(0, n - PATCH + 1, PATCH):
        for x0 in range(0, m - PATCH + 1, PATCH):
            mk = masks[:, y0:y0 + PATCH, x0:x0 + PATCH]
            if mk.mean() < min_frac:
                continue
            ys = np.clip(np.arange(y0 - HALO, y0 + PATCH + HALO), 0, n - 1)
            xs = np.clip(np.arange(x0 - HALO, x0 + PATCH + HALO), 0, m - 1)
            out.append((planes[:, ys][:, :, xs], targets[:, y0:y0 + PATCH, x0:x0 + PATCH], mk))
    return out


def generate(seeds, N=1024, cell=2.0, sample_times=(600.0, 1200.0, 1800.0, 2400.0), window=20.0,
             hmin=0.01, min_frac=0.05, log=None) -> Dataset:
    """Training patches from fine runs of the seeded scenarios (N x N cells
    at `cell` m) and coarse runs restarted from their restrictions."""
    torch = _torch()
    feats, targets, masks = [], [], []
    for seed in seeds:
        t0 = time.time()
        fc = scenario(seed, N, cell)
        cc = coarse_case(fc)
        fine = capi.Sim(fc).setup()
        coarse = capi.Sim(cc).setup()
        fv, cv = fine.device_view(), coarse.device_view()
        accF = torch.zeros((4, cv.rows, cv.pitch), device="cuda", dtype=torch.float32)
        accC = torch.zeros_like(accF)
        bc = coarse.field("BC")[2:-2, 2:-2]
        n_c = cc.n[2:-2, 2:-2]
        all_ids = np.arange(coarse.grid_size, dtype=np.int32)
        wet_all = np.ones(coarse.grid_size, dtype=np.uint8)
        got = 0
        for ts in sample_times:
            t, _, _ = fine.run(10 ** 9, ts)
            hF, uF, vF = _interior_fields(fine)
            h, hu, hv = restrict(hF), restrict(uF), restrict(vF)
            w = np.zeros((cc.h_ny, cc.h_nx))
            huf, hvf = np.zeros_like(w), np.zeros_like(w)
            w[2:-2, 2:-2] = bc + h
            huf[2:-2, 2:-2], hvf[2:-2, 2:-2] = hu, hv
            _, dt_prev = fine.time()
            coarse.set_state(t, dt_prev, w, huf, hvf, wet=wet_all, active=all_ids)
            torch.cuda.synchronize()
            accF.zero_()
            accC.zero_()
            torch.cuda.synchronize()
            tF = t
            while tF < t + window:
                tF, dt = fine.step()
                face_flux(fv, 2, dt, accF, cc.h_nx, cc.h_ny)
            tC = t
            while tC < t + window:
                tC, dt = coarse.step()
                face_flux(cv, 1, dt, accC, cc.h_nx, cc.h_ny)
            torch.cuda.synchronize()
            tgt = (accF / (tF - t) - accC / (tC - t))[:, 2:cc.h_ny - 2, 2:cc.h_nx - 2]
            tgt = tgt.cpu().numpy().astype(np.float32)
            east, north = face_mask(h, hmin)
            mk = np.stack([east, east, north, north]).astype(np.float32)
            rain = np.full_like(h, uniform_rate(fc, t))
            planes = np.stack([h, hu, hv, bc, n_c, rain]).astype(np.float32)
            for f, tg, m in _patches(planes, mk, tgt * mk, min_frac):
                feats.append(f)
                targets.append(tg)
                masks.append(m)
                got += 1
        fine.close()
        coarse.close()
        if log:
            log(f"scenario {seed}: {got} patches ({time.time() - t0:.1f} s)")
    if not feats:
        raise ValueError("no training patches: no 64 x 64 block had enough corrected faces "
                         "(more or larger scenarios, later sample times or a smaller min_frac)")
    return Dataset(np.stack(feats), np.stack(targets), np.stack(masks))


# ------------------------------------------------------------------- model
@dataclasses.dataclass
class Model:
    params: np.ndarray   # NPARAM FP32
    scale: np.ndarray    # 6 input scales
    oscale: np.ndarray   # 4 output scales (net output x oscale = correction)

    def save(self, path):
        np.savez(path, params=self.params, scale=self.scale, oscale=self.oscale)

    @staticmethod
    def load(path):
        z = np.load(path)
        return Model(z["params"], z["scale"], z["oscale"])


def input_scales(ds: Dataset) -> np.ndarray:
    wet = ds.feats[:, 0] > 0.0
    hs = max(float(ds.feats[:, 0][wet].std()), 1e-3) if wet.any() else 1.0
    qs = max(float(np.sqrt(0.5 * (ds.feats[:, 1][wet] ** 2 + ds.feats[:, 2][wet] ** 2).mean())), 1e-4) \
        if wet.any() else 1.0
    return np.array([1 / hs, 1 / qs, 1 / qs, 1.0, 1 / 0.05, RAIN_SCALE], dtype=np.float32)


def output_scales(ds: Dataset) -> np.ndarray:
    o = np.ones(4, dtype=np.float32)
    for c in range(4):
        m = ds.mask[:, c] > 0
        if m.any():
            o[c] = max(float(np.sqrt((ds.target[:, c][m] ** 2).mean())), 1e-7)
    return o


def loss_on(ds: Dataset, model: Model, batch=256) -> float:
    """Mean masked squared error of the scaled targets over a dataset (the
    training loss, without an optimiser step)."""
    torch = _torch()
    P = torch.as_tensor(model.params, device="cuda")
    G = torch.zeros_like(P)
    loss = torch.zeros(1, device="cuda", dtype=torch.float64)
    n = len(ds.feats)
    for a in range(0, n, batch):
        xb = torch.as_tensor(ds.feats[a:a + batch], device="cuda").contiguous()
        tb = torch.as_tensor(ds.target[a:a + batch] / model.oscale.reshape(1, 4, 1, 1), device="cuda")
        wb = torch.as_tensor(ds.mask[a:a + batch], device="cuda")
        train_pass(xb, P, model.scale, tb.contiguous(), wb.contiguous(), 1.0 / (n * PATCH * PATCH), G, loss)
    torch.cuda.synchronize()
    return float(loss.item())


def train(ds: Dataset, steps=1500, batch=256, lr=2e-3, seed=0, log=None, log_every=250):
    """Adam on the masked squared error of the scaled targets; returns the
    Model and the loss history (one value per step, FP64 from the device)."""
    torch = _torch()
    scale, oscale = input_scales(ds), output_scales(ds)
    dev = "cuda"
    X = torch.as_tensor(ds.feats, device=dev)
    T = torch.as_tensor(ds.target / oscale.reshape(1, 4, 1, 1), device=dev)
    W = torch.as_tensor(ds.mask, device=dev)
    P = torch.as_tensor(init_params(seed), device=dev)
    G = torch.zeros_like(P)
    M1 = torch.zeros_like(P)
    V2 = torch.zeros_like(P)
    loss = torch.zeros(steps, device=dev, dtype=torch.float64)
    gen = torch.Generator(device=dev)
    gen.manual_seed(seed)
    nP = X.shape[0]
    b = min(batch, nP)
    for k in range(steps):
        idx = torch.randint(0, nP, (b,), device=dev, generator=gen)
        xb, tb, wb = X[idx].contiguous(), T[idx].contiguous(), W[idx].contiguous()
        train_pass(xb, P, scale, tb, wb, 1.0 / (b * PATCH * PATCH), G, loss[k:k + 1])
        adam(P, G, M1, V2, k + 1, lr * (0.1 ** (k / max(steps, 1))))
        if log and (k + 1) % log_every == 0:
            torch.cuda.synchronize()
            log(f"step {k + 1}: loss {loss[max(0, k - log_every + 1):k + 1].mean().item():.4e}")
    torch.cuda.synchronize()
    return Model(P.cpu().numpy(), scale, oscale), loss.cpu().numpy()


# -------------------------------------------------------- coarse closure run
BLOCK = 16  # coarse cells per side of a closure block (k_closure's output block)


def patch_range(j0, j1, halo, n):
    """The coarse interior rows (or columns) [a, b) of a fine re-solve patch:
    the block's [j0, j1) widened by `halo` cells, clipped to the interior
    [2, n - 2) of an h-grid of n cells."""
    return max(2, j0 - halo), min(n - 2, j1 + halo)


def fine_patch_case(fine: synth.Case, Ja, Jb, Ia, Ib) -> synth.Case:
    """The fine case under coarse interior cells [Ja, Jb) x [Ia, Ib) of its 2x
    coarsening: the fine corner DEM of those cells, their n (and K), the same
    uniform series, and the point sources that fall inside."""
    fa, fb = 2 * (Ja - 2), 2 * (Jb - 2)  # fine interior rows (0-based) of the patch
    ga, gb = 2 * (Ia - 2), 2 * (Ib - 2)
    B = fine.B[fa:fb + 1, ga:gb + 1].copy()

    def cells(a):
        if a is None:
            return None
        out = np.zeros((fb - fa + 4, gb - ga + 4))
        out[2:-2, 2:-2] = a[2 + fa:2 + fb, 2 + ga:2 + gb]
        return out

    src = None
    flags = fine.flags & ~(synth.SAVE_MAX | synth.SAVE_ARRIVAL | synth.CHECK_VOLUME)
    if fine.src_idx is not None:
        j, i = np.divmod(np.asarray(fine.src_idx, dtype=np.int64), fine.h_nx)
        inside = (j >= 2 + fa) & (j < 2 + fb) & (i >= 2 + ga) & (i < 2 + gb)
        if inside.any():
            nx_p = gb - ga + 4
            src = ((j[inside] - fa) * nx_p + (i[inside] - ga)).astype(np.int32)
        else:
            flags &= ~synth.POINT_SOURCE
    return dataclasses.replace(fine, name=fine.name + f"_patch{Ja}_{Ia}", B=B, n=cells(fine.n),
                               K=cells(fine.K), h0=None, src_idx=src, rain_maps=None,
                               flags=flags & ~synth.H_INIT)


class FineFallback:
    """The plain fine-grid solve as the per-block fallback of the closure.

    A block whose residual indicator exceeds tau (k_closure's fallback test)
    is re-solved on the fine grid over the closure interval [t0, t1]: a patch
    of the fine case -- the block and `halo` coarse cells around it, at the
    fine resolution -- starts from the coarse state at t0 (each coarse cell's
    depth and momenta on its four fine cells; the bed is the fine bed), runs
    the plain solver to t1, and its 2x2 means replace the block's coarse
    cells at t1.  The block keeps the volume the coarse solve gave it (the
    fine depths are scaled to it over the wet cells), so the run stays
    conservative, and wet and dry cells keep their status, which the engine's
    tile activity requires; cells next to the domain edge keep the coarse
    values.  The halo absorbs the patch's own open edges over the interval.
    With `batch`, the patches of an interval run to t1 together as members of
    one ensemble launch (up to `cache` of them per launch)."""

    def __init__(self, coarse_sim: capi.Sim, fine: synth.Case, halo=4, max_blocks=256, cache=64,
                 batch=True):
        self.sim, self.fine, self.halo = coarse_sim, fine, halo
        self.max_blocks, self.cache, self.batch = max_blocks, cache, batch
        self.ensembles = 0  # ensemble launches that re-solved a group of patches
        self.patches = {}   # block -> (Sim, BC of the patch)
        self.refined = 0    # blocks re-solved so far
        self.skipped = 0    # fallen-back blocks beyond max_blocks in one interval

    def _patch(self, key, Ja, Jb, Ia, Ib):
        if key in self.patches:
            self.patches[key] = self.patches.pop(key)  # most recent last
            return self.patches[key]
        if len(self.patches) >= self.cache:
            old = next(iter(self.patches))
            self.patches.pop(old)[0].close()
        case = fine_patch_case(self.fine, Ja, Jb, Ia, Ib)
        sim = capi.Sim(case).setup()
        entry = (sim, sim.field("BC"))
        self.patches[key] = entry
        return entry

    def refine(self, fell, u0, t0, t1, dt0):
        """Re-solve the fallen-back blocks (fell: per-block flags, row-major
        over ceil((nx-4)/16) blocks) from the coarse state u0 = (h, hu, hv)
        at t0 (host arrays of the h-grid) to t1, writing the coarse state at t1
        through the handle's device view."""
        torch = _torch()
        v = self.sim.device_view()
        ny, nx = v.h_ny, v.h_nx
        tx = -(-(nx - 4) // BLOCK)
        blocks = np.nonzero(fell)[0]
        if len(blocks) > self.max_blocks:
            self.skipped += len(blocks) - self.max_blocks
            blocks = blocks[:self.max_blocks]
        if len(blocks) == 0:
            return 0
        planes = [_device_plane(ptr, v) for ptr in (v.h, v.hu, v.hv)]
        torch.cuda.synchronize()
        cur = [p[:ny, :nx].cpu().numpy() for p in planes]
        eps = 1.19209e-07
        # groups of at most `cache` blocks, so that no patch of a group is
        # evicted while the group runs
        group = max(1, self.cache)
        for g0 in range(0, len(blocks), group):
            work = []
            for b in blocks[g0:g0 + group]:
                by, bx = divmod(int(b), tx)
                j0, i0 = 2 + BLOCK * by, 2 + BLOCK * bx
                j1, i1 = min(j0 + BLOCK, ny - 2), min(i0 + BLOCK, nx - 2)
                Ja, Jb = patch_range(j0, j1, self.halo, ny)
                Ia, Ib = patch_range(i0, i1, self.halo, nx)
                psim, pbc = self._patch((j0, i0), Ja, Jb, Ia, Ib)
                # the coarse state at t0 on the fine cells of the patch
                hf = np.zeros(pbc.shape)
                huf, hvf = np.zeros(pbc.shape), np.zeros(pbc.shape)
                for a, src in ((hf, u0[0]), (huf, u0[1]), (hvf, u0[2])):
                    blk = src[Ja:Jb, Ia:Ib].astype(np.float64)
                    a[2:-2, 2:-2] = np.repeat(np.repeat(blk, 2, axis=0), 2, axis=1)
                hf = np.maximum(hf, 0.0)
                n_bx, n_by = psim.nBX, psim.nBY
                psim.set_state(t0, dt0, pbc + hf, huf, hvf, wet=np.ones(n_bx * n_by, np.uint8),
                               active=np.arange(n_bx * n_by, dtype=np.int32))
                work.append((psim, pbc, j0, i0, j1, i1, Ja, Ia))
            if self.batch and len(work) > 1:
                # every patch of the group to t1 in one ensemble launch, each
                # with its own dt (the ensemble kernel), instead of one patch
                # run after another
                ens = capi.Ensemble([w[0] for w in work])
                try:
                    ens.run(t_stop=t1)
                finally:
                    ens.close()
                self.ensembles += 1
            else:
                for w in work:
                    w[0].run(2 ** 31 - 1, t1)
            for psim, pbc, j0, i0, j1, i1, Ja, Ia in work:
                hp = (psim.field("W") - pbc)[2:-2, 2:-2]
                up, vp = psim.field("HU")[2:-2, 2:-2], psim.field("HV")[2:-2, 2:-2]
                # the block's cells in the patch, 2x2 means; the edge cells of
                # the domain keep the coarse values
                r0, c0 = 2 * (j0 - Ja), 2 * (i0 - Ia)
                sl = (slice(r0, r0 + 2 * (j1 - j0)), slice(c0, c0 + 2 * (i1 - i0)))
                Hf, Uf, Vf = restrict(hp[sl]), restrict(up[sl]), restrict(vp[sl])
                jj, ii = np.mgrid[j0:j1, i0:i1]
                keep = (jj >= 3) & (jj <= ny - 4) & (ii >= 3) & (ii <= nx - 4)
                Hc = cur[0][j0:j1, i0:i1].astype(np.float64)
                wet = (Hc > eps) & keep
                Hn = np.where(wet, np.maximum(Hf, 2 * eps), Hc)
                vol_c, vol_f = Hc[wet].sum(), Hn[wet].sum()
                if vol_f > 0:
                    Hn[wet] *= vol_c / vol_f
                    Hn[wet] = np.maximum(Hn[wet], 2 * eps)
                cur[0][j0:j1, i0:i1] = np.where(wet, Hn, Hc).astype(np.float32)
                cur[1][j0:j1, i0:i1] = np.where(wet, Uf, cur[1][j0:j1, i0:i1]).astype(np.float32)
                cur[2][j0:j1, i0:i1] = np.where(wet, Vf, cur[2][j0:j1, i0:i1]).astype(np.float32)
                self.refined += 1
        for p, c in zip(planes, cur):
            p[:ny, :nx].copy_(torch.as_tensor(c, device="cuda"))
        torch.cuda.synchronize()
        return len(blocks)

    def close(self):
        for sim, _ in self.patches.values():
            sim.close()
        self.patches.clear()


def _device_plane(ptr, v):
    """A (rows, pitch) FP32 CUDA tensor over a device-view plane (no copy)."""
    torch = _torch()

    class _Arr:
        __cuda_array_interface__ = {"shape": (v.rows, v.pitch), "typestr": "<f4",
                                    "data": (int(ptr), False), "version": 3, "strides": None}
    return torch.as_tensor(_Arr(), device="cuda")


class ClosureRun:
    """A coarse handle stepped by the engine, with the closure applied every
    `every` steps over the time those steps covered.  With `fine` (the fine
    case the coarse one was coarsened from), blocks that fall back are
    re-solved on the fine grid (FineFallback) instead of keeping the plain
    coarse solve."""

    def __init__(self, sim: capi.Sim, model: Model, every=4, hmin=0.01, lim=0.2, tau=0.5, gain=1.0,
                 fine: synth.Case | None = None, halo=4, fine_batch=True):
        torch = _torch()
        self.sim, self.model = sim, model
        self.every, self.hmin, self.lim, self.tau = every, hmin, lim, tau
        self.fallback = (FineFallback(sim, fine, halo=halo, batch=fine_batch)
                         if fine is not None else None)
        v = sim.device_view()
        self.view = v
        rows, pitch = v.rows, v.pitch
        bc = sim.field("BC")
        n = np.array(sim.case.n, dtype=np.float64)
        self.bed = torch.zeros((rows, pitch), device="cuda", dtype=torch.float32)
        self.nman = torch.zeros_like(self.bed)
        ny, nx = v.h_ny, v.h_nx
        jj = np.clip(np.arange(ny), 2, ny - 3)
        ii = np.clip(np.arange(nx), 2, nx - 3)
        self.bed[:ny, :nx] = torch.as_tensor(bc[jj][:, ii], dtype=torch.float32)
        self.nman[:ny, :nx] = torch.as_tensor(n[jj][:, ii], dtype=torch.float32)
        self.params = torch.as_tensor(model.params, device="cuda")
        self.corr = torch.zeros((4, rows, pitch), device="cuda", dtype=torch.float32)
        nb = -(-(v.h_nx - 4) // 16) * -(-(v.h_ny - 4) // 16)
        self.fell = torch.zeros(nb, device="cuda", dtype=torch.uint8)
        self.counters = torch.zeros(2, device="cuda", dtype=torch.int32)
        # gain: strength of each correction (east mass, east x momentum,
        # north mass, north y momentum), multiplying the output scales
        g = np.broadcast_to(np.asarray(gain, dtype=np.float64), (4,))
        self.osc = (C.c_float * 4)(*[float(x) for x in model.oscale * g])
        torch.cuda.synchronize()
        self.applies = 0

    def _src(self, rain):
        v = self.view
        s = Src()
        planes = [v.h, v.hu, v.hv, self.bed.data_ptr(), self.nman.data_ptr(), None]
        for c in range(6):
            s.plane[c] = planes[c]
            s.value[c] = rain if c == 5 else 0.0
            s.scale[c] = float(self.model.scale[c])
        s.sample_stride, s.pitch, s.H, s.W = 0, v.pitch, v.h_ny, v.h_nx
        s.oy0 = s.ox0 = 2
        s.OH, s.OW, s.samples = v.h_ny - 4, v.h_nx - 4, 1
        return s

    def apply(self, dtw, t):
        src = self._src(uniform_rate(self.sim.case, t))
        _check(load().rift_closure_apply(C.byref(self.view), C.byref(src), self.params.data_ptr(),
                                         self.osc, float(dtw), self.hmin, self.lim, self.tau,
                                         self.corr.data_ptr(), self.fell.data_ptr(),
                                         self.counters.data_ptr()),
               "rift_closure_apply")
        self.applies += 1

    def run(self, tf):
        t, dt = self.sim.time()
        while t < tf:
            u0 = self._state_copy() if self.fallback is not None else None
            t_new, dt_new, k = self.sim.run(self.every, tf)
            if k == 0:
                break
            self.apply(t_new - t, t_new)
            if self.fallback is not None:
                _torch().cuda.synchronize()  # the closure kernels ran on the handle's stream
                fell = self.fell.cpu().numpy()
                if fell.any():
                    v = self.view
                    u = [p[:v.h_ny, :v.h_nx].cpu().numpy() for p in u0]
                    self.fallback.refine(fell, u, t, t_new, 0.5 * dt)
            t, dt = t_new, dt_new
        check(self.view.stream)
        return t

    def _state_copy(self):
        """Device copy of the handle's h, hu, hv (the state at an interval's start)."""
        v = self.view
        _torch().cuda.synchronize()  # the handle's stream wrote the state
        return [_device_plane(p, v).clone() for p in (v.h, v.hu, v.hv)]

    def block_counts(self):
        """(blocks evaluated, blocks that fell back) over every apply."""
        _torch().cuda.synchronize()
        c = self.counters.cpu().numpy()
        return int(c[0]), int(c[1])


class EnsembleClosure:
    """An ensemble (capi.Ensemble) of coarse members with the closure: the
    persistent ensemble kernel advances every live member by `every` of its
    own steps, then each member that moved gets the closure over the time it
    covered; repeated until every member reaches t_stop."""

    def __init__(self, ens, sims, model: Model, every=8, **kw):
        self.ens, self.sims, self.every = ens, list(sims), every
        self.runs = [ClosureRun(s, model, every=every, **kw) for s in self.sims]
        self.chunks = 0  # ensemble launches (one kernel each)

    def run(self, t_stop):
        """Run every member to t_stop; finish_wall[m] is the host time from
        the call's start to the end of the chunk in which member m reached
        t_stop (its closure step included)."""
        import time
        torch = _torch()
        t_prev = np.array([s.time()[0] for s in self.sims])
        steps = np.zeros(len(self.sims), dtype=np.int64)
        self.finish_wall = np.zeros(len(self.sims))
        t0 = time.perf_counter()
        while True:
            t, k = self.ens.run(t_stop=t_stop, max_steps=self.every)
            self.chunks += 1
            if k.max() == 0:
                break
            steps += k
            for m in np.nonzero(t > t_prev)[0]:
                self.runs[m].apply(t[m] - t_prev[m], t[m])
            # the closure kernels run on the members' streams, the ensemble
            # kernel on its own: finish them before the next launch
            torch.cuda.synchronize()
            now = time.perf_counter() - t0
            for m in np.nonzero((t >= t_stop) & (t_prev < t_stop))[0]:
                self.finish_wall[m] = now
            t_prev = t
            if (t >= t_stop).all():
                break
        check(None)
        return t_prev, steps

    def launches(self):
        """Kernels launched: one ensemble kernel per chunk, two per closure step."""
        return self.chunks + 2 * sum(r.applies for r in self.runs)
