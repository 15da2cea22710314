"""Learned flux closure kernels on the GPU, each against an FP32 statement of
the same arithmetic: the net's forward pass and its parameter gradient
against PyTorch autograd (BF16 tensor-core operands, so the tolerances are
BF16-sized), Adam against its formula, the face-flux kernel against a numpy
FP32 restatement of the step's reconstruction and central-upwind flux, and
the closure step's volume conservation."""
import ctypes

import numpy as np
import pytest

from rift_gb300 import build as eb
from rift_gb300 import capi, closure, synth

pytestmark = pytest.mark.gpu

# BF16 operands (8-bit mantissa) in the tensor-core layers (1 and 2 in the
# forward and apply kernels on tcgen05, layer 3 there in FP32; all three in
# the training kernel on mma.sync), FP32 accumulation, against true FP32
# PyTorch (TF32 off).  Measured on GB300 with mma.sync everywhere: forward
# 5.1e-3, loss 2.5e-4, gradient blocks 1.6e-3 .. 2.5e-3; the bars keep 3-4x
# margin.
FWD_TOL = 1.5e-2    # max |out - ref| / max |ref|
LOSS_TOL = 2e-3     # relative loss difference
GRAD_TOL = 1e-2     # |g - g_ref| / |g_ref| per parameter block


@pytest.fixture(scope="module")
def torch():
    import torch
    eb.build()
    closure.load()
    return torch


def test_tcgen05_mma_layout_selftest(torch):
    """One tcgen05.mma (128 x 32 x 16) through the forward pass's operand
    descriptors and instruction descriptor, read back from tensor memory:
    the product of small exactly representable values must be exact."""
    out = torch.zeros(128 * 32, dtype=torch.float32, device="cuda")
    closure._check(closure.load().rift_closure_selftest(ctypes.c_void_p(out.data_ptr()), None),
                   "rift_closure_selftest")
    closure._check(closure.load().rift_closure_check(None), "rift_closure_check")
    r = np.arange(128)[:, None]
    n = np.arange(32)[:, None]
    k = np.arange(16)[None, :]
    A = (r % 7) - 3 + 0.25 * (k % 5)
    B = (n % 5) - 2 + 0.5 * (k % 3)
    ref = (A @ B.T).astype(np.float32)
    got = out.cpu().numpy().reshape(128, 32)
    assert np.array_equal(got, ref), np.abs(got - ref).max()


def _patches(rng, S=3, H=70):
    x = np.zeros((S, 6, H, H), np.float32)
    x[:, 0] = np.abs(rng.normal(0.3, 0.3, (S, H, H)))
    x[:, 1] = rng.normal(0, 0.2, (S, H, H))
    x[:, 2] = rng.normal(0, 0.2, (S, H, H))
    yy, xx = np.mgrid[0:H, 0:H]
    for s in range(S):
        x[s, 3] = 30.0 + 0.05 * xx - 0.03 * yy + rng.normal(0, 0.2, (H, H))
    x[:, 4] = rng.uniform(0.02, 0.08, (S, H, H))
    x[:, 5] = 1.4e-5
    return x


SCALE = np.array([2.0, 3.0, 3.0, 1.0, 20.0, closure.RAIN_SCALE], np.float32)


def _params(rng):
    p = closure.init_params(3)
    p[closure.OFF_B1:closure.OFF_W2] = rng.normal(0, 0.1, 32)
    p[closure.OFF_B2:closure.OFF_W3] = rng.normal(0, 0.1, 32)
    w3 = p[closure.OFF_W3:closure.OFF_B3].reshape(8, 32)
    w3[:4] *= 10.0
    p[closure.OFF_B3:closure.OFF_B3 + 4] = rng.normal(0, 0.1, 4)
    return p


def test_forward_matches_torch(torch):
    rng = np.random.default_rng(0)
    x = torch.as_tensor(_patches(rng), device="cuda")
    p = torch.as_tensor(_params(rng), device="cuda")
    out = closure.forward(x, p, SCALE)
    torch.cuda.synchronize()
    xs = x * torch.as_tensor(SCALE, device="cuda").view(1, 6, 1, 1)
    ref = closure.torch_forward(xs, p)
    assert out.shape == ref.shape == (3, 4, 64, 64)
    err = (out - ref).abs().max().item() / ref.abs().max().item()
    assert err < FWD_TOL, err


def test_forward_partial_blocks_and_clamped_edges(torch):
    """Output extents that are not multiples of 16 (the last block partial,
    its input reads clamped to the patch): every output cell matches torch."""
    rng = np.random.default_rng(1)
    H = 45  # 39 output cells per side: three blocks, the last one partial
    x = torch.as_tensor(_patches(rng, S=2, H=H), device="cuda")
    p = torch.as_tensor(_params(rng), device="cuda")
    out = closure.forward(x, p, SCALE)
    xs = x * torch.as_tensor(SCALE, device="cuda").view(1, 6, 1, 1)
    ref = closure.torch_forward(xs, p)
    assert out.shape == ref.shape == (2, 4, 39, 39)
    err = (out - ref).abs().max().item() / ref.abs().max().item()
    assert err < FWD_TOL, err


def test_gradient_matches_autograd(torch):
    rng = np.random.default_rng(2)
    x = torch.as_tensor(_patches(rng, S=4), device="cuda")
    pn = _params(rng)
    p = torch.as_tensor(pn, device="cuda")
    tgt = torch.as_tensor(rng.normal(0, 1, (4, 4, 64, 64)).astype(np.float32), device="cuda")
    w = torch.as_tensor((rng.uniform(0, 1, (4, 4, 64, 64)) > 0.3).astype(np.float32), device="cuda")
    ls = 1.0 / (4 * 64 * 64)
    grad = torch.zeros(closure.NPARAM, device="cuda")
    loss = torch.zeros(1, device="cuda", dtype=torch.float64)
    closure.train_pass(x, p, SCALE, tgt, w, ls, grad, loss)
    torch.cuda.synchronize()
    pr = p.clone().requires_grad_(True)
    xs = x * torch.as_tensor(SCALE, device="cuda").view(1, 6, 1, 1)
    ref = closure.torch_forward(xs, pr)
    lref = ls * (w * (ref - tgt) ** 2).sum()
    lref.backward()
    g = pr.grad
    assert abs(loss.item() - lref.item()) / lref.item() < LOSS_TOL
    blocks = {"W1": (closure.OFF_W1, closure.OFF_B1), "b1": (closure.OFF_B1, closure.OFF_W2),
              "W2": (closure.OFF_W2, closure.OFF_B2), "b2": (closure.OFF_B2, closure.OFF_W3),
              "W3": (closure.OFF_W3, closure.OFF_W3 + 128), "b3": (closure.OFF_B3, closure.OFF_B3 + 4)}
    for name, (a, b) in blocks.items():
        gk, gr = grad[a:b], g[a:b]
        rel = (gk - gr).norm().item() / gr.norm().item()
        assert rel < GRAD_TOL, (name, rel)
    # padding columns of W1 and rows 4..7 of W3 get no gradient
    assert grad[closure.OFF_W1:closure.OFF_B1].view(32, 160)[:, 150:].abs().max().item() == 0.0
    assert grad[closure.OFF_W3 + 128:closure.OFF_B3].abs().max().item() == 0.0


def test_adam_matches_formula(torch):
    rng = np.random.default_rng(3)
    n = 1000
    p0 = rng.normal(0, 1, n).astype(np.float32)
    g0 = rng.normal(0, 1, n).astype(np.float32)
    p, g = torch.as_tensor(p0, device="cuda"), torch.as_tensor(g0, device="cuda")
    m, v = torch.zeros_like(p), torch.zeros_like(p)
    closure.adam(p, g, m, v, 1, 1e-2)
    torch.cuda.synchronize()
    mm = 0.1 * g0
    vv = 0.001 * g0 * g0
    ref = p0 - 1e-2 * (mm / 0.1) / (np.sqrt(vv / 0.001) + 1e-8)
    np.testing.assert_allclose(p.cpu().numpy(), ref, rtol=1e-5, atol=1e-6)
    assert g.abs().max().item() == 0.0


# ------------------------------------------------------------- face fluxes
def _cudart():
    for name in ("libcudart.so", "libcudart.so.13", "libcudart.so.12"):
        try:
            lib = ctypes.CDLL(name)
            lib.cudaMemcpy.restype = ctypes.c_int
            lib.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
            return lib
        except OSError:
            continue
    pytest.skip("no CUDA runtime library to read device planes")


def _plane(view, ptr, k=0):
    out = np.zeros((view.rows, view.pitch), np.float32)
    src = ptr + k * view.rows * view.pitch * 4
    assert _cudart().cudaMemcpy(out.ctypes.data, src, out.nbytes, 2) == 0
    return out


def _np_flux(h, u, v, eM, eP, j, i, axis, kappa):
    """FP32 numpy statement of the step's reconstruction + face flux through
    the + face of cell (j, i) along axis (1: x, 0: y)."""
    f32 = np.float32
    G = f32(9.80665)

    def cell(k):
        jj, ii = (j, i + k) if axis == 1 else (j + k, i)
        return h[jj, ii], u[jj, ii], v[jj, ii], eM[jj, ii], eP[jj, ii]

    def slope(dp, dm):
        a = f32(1.3) * abs(dp)
        b = f32(0.5) * abs(f32(dp + dm))
        c = f32(1.3) * abs(dm)
        return f32(0.5) * min(min(a, b), c)

    def rec(k):
        h0, u0, v0, em, ep = cell(k)
        hp, up, vp, emp, _ = cell(k + 1)
        hm, um, vm, _, epm = cell(k - 1)
        sw = slope(f32(f32(ep - emp) + f32(hp - h0)), f32(f32(epm - em) + f32(h0 - hm)))
        su = slope(f32(up - u0), f32(u0 - um))
        sv = slope(f32(vp - v0), f32(v0 - vm))
        hP = f32(f32(h0 + sw) - ep)
        hM = f32(f32(h0 - sw) - em)
        hb = f32(f32(h0 + h0) - f32(ep + em))
        if hP < 0:
            hP, hM = f32(0), hb
        if hM < 0:
            hP, hM = hb, f32(0)
        return (hP, f32(u0 + su), f32(v0 + sv)), (hM, f32(u0 - su), f32(v0 - sv))

    L, _ = rec(0)
    _, R = rec(1)

    def side(hh, qu, qv):
        h2 = f32(hh * hh)
        r = f32(f32(2) * hh) / f32(h2 + max(h2, f32(kappa)))
        uu, vv = f32(qu * r), f32(qv * r)
        return hh, uu, vv, f32(hh * uu), f32(hh * vv), f32(np.sqrt(f32(G * hh)))

    hL, uL, vL, quL, qvL, cL = side(*L)
    hR, uR, vR, quR, qvR, cR = side(*R)
    nL, nR = (uL, uR) if axis == 1 else (vL, vR)
    ap = max(max(f32(nL + cL), f32(nR + cR)), f32(0))
    am = min(min(f32(nL - cL), f32(nR - cR)), f32(0))
    pL, pR = f32(f32(0.5) * G * hL * hL), f32(f32(0.5) * G * hR * hR)
    if axis == 1:
        FL = [quL, f32(quL * uL + pL), f32(quL * vL)]
        FR = [quR, f32(quR * uR + pR), f32(quR * vR)]
    else:
        FL = [qvL, f32(qvL * uL), f32(qvL * vL + pL)]
        FR = [qvR, f32(qvR * uR), f32(qvR * vR + pR)]
    if not hL > 0:
        FL = [f32(0)] * 3
    if not hR > 0:
        FR = [f32(0)] * 3
    d = f32(ap - am)
    if not d > 0:
        return [0.0, 0.0, 0.0]
    k = f32(ap * am / d)
    qs = [(hR, hL), (quR, quL), (qvR, qvL)]
    return [float(f32((ap * FL[c] - am * FR[c]) / d) + k * f32(qs[c][0] - qs[c][1])) for c in range(3)]


@pytest.fixture(scope="module")
def wet_small(torch):
    case = synth.small_case(nx_cells=40, ny_cells=36, seed=5, cell=10.0, rain_mmhr=400.0, rim=True)
    sim = capi.Sim(case).setup()
    sim.run(400)
    return sim


def test_face_flux_matches_numpy_statement(torch, wet_small):
    sim = wet_small
    v = sim.device_view()
    acc = torch.zeros((4, v.rows, v.pitch), device="cuda")
    torch.cuda.synchronize()
    closure.face_flux(v, 1, 1.0, acc, v.h_nx, v.h_ny)
    torch.cuda.synchronize()
    a = acc.cpu().numpy()
    h, u, w = _plane(v, v.h), _plane(v, v.hu), _plane(v, v.hv)
    eW, eE, eS, eN = (_plane(v, v.e, k) for k in range(4))
    rng = np.random.default_rng(4)
    wet = np.argwhere(h[3:v.h_ny - 3, 3:v.h_nx - 3] > 0.01) + 3
    assert len(wet) > 50
    pick = wet[rng.choice(len(wet), 40, replace=False)]
    worst = 0.0
    for j, i in pick:
        fx = _np_flux(h, u, w, eW, eE, j, i, 1, v.kappa)
        fy = _np_flux(h, u, w, eS, eN, j, i, 0, v.kappa)
        ref = [fx[0], fx[1], fy[0], fy[2]]
        got = a[:, j, i]
        for c in range(4):
            worst = max(worst, abs(got[c] - ref[c]) / (abs(ref[c]) + 1e-4))
    assert worst < 1e-4, worst


def test_face_flux_ratio2_is_the_mean_of_fine_faces(torch, wet_small):
    sim = wet_small
    v = sim.device_view()
    ncx, ncy = (v.h_nx - 4) // 2 + 4, (v.h_ny - 4) // 2 + 4
    fine = torch.zeros((4, v.rows, v.pitch), device="cuda")
    coarse = torch.zeros((4, ncy + 2, ncx + 2), device="cuda")
    torch.cuda.synchronize()
    closure.face_flux(v, 1, 1.0, fine, v.h_nx, v.h_ny)
    closure.face_flux(v, 2, 1.0, coarse, ncx, ncy)
    torch.cuda.synchronize()
    f, c = fine.cpu().numpy(), coarse.cpu().numpy()
    J, I = np.mgrid[2:ncy - 2, 2:ncx - 2]
    jf, i0 = 2 * (J - 2) + 2, 2 * (I - 2) + 2
    east = 0.5 * (f[0][jf, i0 + 1] + f[0][jf + 1, i0 + 1])
    north = 0.5 * (f[2][jf + 1, i0] + f[2][jf + 1, i0 + 1])
    np.testing.assert_allclose(c[0][2:ncy - 2, 2:ncx - 2], east, rtol=1e-5, atol=1e-7)
    np.testing.assert_allclose(c[2][2:ncy - 2, 2:ncx - 2], north, rtol=1e-5, atol=1e-7)


def test_face_flux_rejects_mismatched_grids(torch, wet_small):
    v = wet_small.device_view()
    acc = torch.zeros((4, v.rows, v.pitch), device="cuda")
    with pytest.raises(capi.RiftError):
        closure.face_flux(v, 2, 1.0, acc, v.h_nx, v.h_ny)


# ------------------------------------------------------------ closure step
def test_closure_step_conserves_volume(torch):
    """Corrections move volume between cells only: the total changes by
    rounding, no cell goes negative, dry cells stay untouched."""
    # 70 x 58 interior cells: the last block of each row and column is partial
    case = synth.small_case(nx_cells=70, ny_cells=58, seed=9, cell=4.0, rain_mmhr=600.0, rim=True)
    sim = capi.Sim(case).setup()
    sim.run(300)
    rng = np.random.default_rng(5)
    p = _params(rng)
    model = closure.Model(p, SCALE, np.array([2e-3, 2e-3, 2e-3, 2e-3], np.float32))
    run = closure.ClosureRun(sim, model, hmin=0.01, lim=0.2, tau=1e9)
    h0 = sim.field("W") - sim.field("BC")
    v0 = sim.volume()
    run.apply(2.0, sim.time()[0])
    torch.cuda.synchronize()
    h1 = sim.field("W") - sim.field("BC")
    v1 = sim.volume()
    ev, fb = run.block_counts()
    assert ev >= 1 and fb == 0
    changed = np.abs(h1 - h0)[2:-2, 2:-2] > 0
    assert changed.sum() > 10
    assert abs(v1 - v0) <= 1e-6 * v0, (v0, v1)
    inner = (slice(2, -2), slice(2, -2))
    assert (h1[inner] >= 0).all()
    dry = h0[inner] <= 0.01
    assert np.array_equal(h1[inner][dry], h0[inner][dry])


def test_closure_fallback_blocks_leave_the_state(torch):
    """With tau = 0 every evaluated block falls back: the step changes nothing."""
    case = synth.small_case(nx_cells=48, ny_cells=48, seed=9, cell=4.0, rain_mmhr=600.0, rim=True)
    sim = capi.Sim(case).setup()
    sim.run(300)
    rng = np.random.default_rng(6)
    model = closure.Model(_params(rng), SCALE, np.full(4, 2e-3, np.float32))
    run = closure.ClosureRun(sim, model, tau=0.0)
    w0 = sim.field("W")
    run.apply(2.0, sim.time()[0])
    ev, fb = run.block_counts()
    assert ev >= 1 and fb >= 1
    assert np.array_equal(sim.field("W"), w0)


def test_closure_mixed_fallback_isolates_blocks(torch):
    """Some blocks fall back, others not: every cell of a fallen-back block
    keeps the plain solve bit for bit, faces shared with a fallen-back block
    are not corrected from either side, and the other cells change by exactly
    the divergence of their own blocks' corrections (a numpy FP32 restatement
    of the apply step with the kernel's per-block flags)."""
    case = synth.small_case(nx_cells=80, ny_cells=64, seed=9, cell=4.0, rain_mmhr=600.0, rim=True)
    sim = capi.Sim(case).setup()
    sim.run(300)
    rng = np.random.default_rng(8)
    model = closure.Model(_params(rng), SCALE, np.full(4, 2e-3, np.float32))
    snap = sim.snapshot()
    bc = sim.field("BC")
    dtw = 2.0
    chosen = None
    for tau in np.geomspace(1e-5, 1e2, 36):
        sim.load_snapshot(snap)
        run = closure.ClosureRun(sim, model, hmin=0.01, lim=0.2, tau=float(tau))
        run.apply(dtw, sim.time()[0])
        ev, fb = run.block_counts()
        if 0 < fb < ev:
            chosen = run
            break
    assert chosen is not None, "no tau splits the blocks"
    run = chosen
    torch.cuda.synchronize()
    h0 = (snap["w"] - bc).astype(np.float64)
    h1 = sim.field("W") - bc
    v = run.view
    ny, nx = v.h_ny, v.h_nx
    tx = -(-(nx - 4) // 16)
    fell = run.fell.cpu().numpy().astype(bool)
    corr = run.corr.cpu().numpy()[:, :ny, :nx]
    jj, ii = np.mgrid[0:ny, 0:nx]
    blk = np.full((ny, nx), -1)
    inner = (jj >= 2) & (jj <= ny - 3) & (ii >= 2) & (ii <= nx - 3)
    blk[inner] = ((jj[inner] - 2) // 16) * tx + (ii[inner] - 2) // 16
    fb_cell = np.zeros((ny, nx), bool)
    fb_cell[inner] = fell[blk[inner]]
    # fallen-back blocks: bit-identical depths (the FP64 w of an unchanged FP32 h)
    assert fb_cell.any() and (~fb_cell & inner).any()
    np.testing.assert_array_equal(sim.field("W")[fb_cell], snap["w"][fb_cell])
    # restatement of the apply step
    sx = np.float32(dtw / case.cell)
    off = fb_cell.copy()
    exp = h0.astype(np.float32).copy()
    for j in range(3, ny - 3):
        for i in range(3, nx - 3):
            if fb_cell[j, i]:
                continue
            mE = 0.0 if off[j, i + 1] else corr[0, j, i]
            mW = 0.0 if off[j, i - 1] else corr[0, j, i - 1]
            mN = 0.0 if off[j + 1, i] else corr[2, j, i]
            mS = 0.0 if off[j - 1, i] else corr[2, j - 1, i]
            if mE == mW == mN == mS == 0.0:
                continue
            exp[j, i] = np.float32(exp[j, i] - (sx * np.float32(mE - mW) + sx * np.float32(mN - mS)))
    d = np.abs(h1 - exp.astype(np.float64))[inner]
    assert d.max() <= 1e-6, d.max()
    assert np.abs(h1 - h0)[inner & ~fb_cell].max() > 0
    v0 = float(h0[inner].sum())
    assert abs(float(h1[inner].sum()) - v0) <= 1e-6 * v0


def test_closure_rejects_limits_that_could_dry_a_cell(torch):
    case = synth.small_case(nx_cells=32, ny_cells=32, seed=9, cell=4.0)
    sim = capi.Sim(case).setup()
    model = closure.Model(closure.init_params(0), SCALE, np.full(4, 2e-3, np.float32))
    for kw in (dict(lim=0.25), dict(lim=0.3), dict(hmin=1e-7, lim=0.2)):
        run = closure.ClosureRun(sim, model, **kw)
        with pytest.raises(capi.RiftError):
            run.apply(1.0, 0.0)


def test_generate_train_and_run_end_to_end(torch):
    """Small-grid version of the whole closure workflow: training patches
    from the solver, a few Adam steps that lower the loss, a coarse run with
    the closure that stays finite and conserves the rain volume."""
    ds = closure.generate([0, 1], N=256, cell=4.0, sample_times=(600.0, 1200.0), window=10.0,
                          hmin=0.005, min_frac=0.02)
    assert ds.feats.shape[1:] == (6, 70, 70) and ds.target.shape[1:] == (4, 64, 64)
    assert len(ds.feats) >= 2 and np.isfinite(ds.target).all()
    model, loss = closure.train(ds, steps=60, batch=16, lr=3e-3)
    assert np.isfinite(loss).all() and loss[-10:].mean() < loss[:10].mean()
    cc = closure.coarse_case(closure.scenario(6, N=256, cell=4.0, tf=900.0))  # rimmed: closed
    sim = capi.Sim(cc).setup()
    run = closure.ClosureRun(sim, model, every=4)
    t = run.run(600.0)
    assert t >= 600.0 and run.applies > 0
    vol, added = sim.mass_ledger()
    assert abs(vol - added) <= 1e-5 * added


def test_ensemble_with_closure_matches_members_alone(torch):
    """Coarse members stepped by the ensemble kernel with the closure every
    4 steps end where each ends run alone with the same closure."""
    rng = np.random.default_rng(7)
    model = closure.Model(_params(rng), SCALE, np.full(4, 2e-3, np.float32))
    cases = [closure.coarse_case(closure.even_side(c))
             for c in synth.config5(members=3, side=(96, 160), tf=900.0)]
    alone = []
    for c in cases:
        sim = capi.Sim(c).setup()
        closure.ClosureRun(sim, model, every=4).run(600.0)
        alone.append((sim.time()[0], sim.field("W")))
        sim.close()
    sims = [capi.Sim(c).setup() for c in cases]
    ens = capi.Ensemble(sims)
    t, steps = closure.EnsembleClosure(ens, sims, model, every=4).run(600.0)
    for m, s in enumerate(sims):
        ta, wa = alone[m]
        assert abs(t[m] - ta) <= 1e-6 * ta
        d = np.abs(s.field("W") - wa)[2:-2, 2:-2].max()
        assert d < 1e-3, (m, d)
    ens.close()


def test_fine_fallback_resolves_blocks_on_the_fine_grid(torch):
    """The plain fine-grid solve as the per-block fallback: every block whose
    net output corrects a face falls back (tau = 0; a block runs the net when
    a cell of it is deeper than hmin, here the wetter blocks along the rim
    after 300 s of rain, and a block whose only deep cells sit on the domain
    edge corrects no face) and is re-solved from the coarse state at the
    interval's start on a fine patch (block + 4 coarse cells of halo, 2 m
    cells under 4 m ones).  The patches run together in ensemble launches and
    end where they end run one after another (within 1e-4).  The re-solve
    keeps each block's volume, keeps wet and dry cells as they were, changes
    the wet cells of the blocks, and leaves the edge cells of the domain
    alone; a run with the fallback on stays finite and its mass ledger
    closes."""
    fine = closure.scenario(6, N=256, cell=2.0, tf=900.0)  # rimmed plane with bumps
    cc = closure.coarse_case(fine)
    sim = capi.Sim(cc).setup()
    sim.run(2 ** 31 - 1, 300.0)
    rng = np.random.default_rng(9)
    model = closure.Model(_params(rng), SCALE, np.full(4, 2e-3, np.float32))
    run = closure.ClosureRun(sim, model, every=4, tau=0.0, fine=fine)
    bc = sim.field("BC")
    t0, dt0 = sim.time()
    u0 = [p[:run.view.h_ny, :run.view.h_nx].cpu().numpy() for p in run._state_copy()]
    t1, _, k = sim.run(4)
    run.apply(t1 - t0, t1)
    torch.cuda.synchronize()
    fell = run.fell.cpu().numpy()
    evaluated, fallen = run.block_counts()
    assert int(fell.sum()) == fallen and 8 <= fallen <= evaluated, (evaluated, fallen)
    h1 = sim.field("W") - bc
    v1 = sim.volume()
    v = run.view
    planes = [closure._device_plane(p, v) for p in (v.h, v.hu, v.hv)]
    before = [p[:v.h_ny, :v.h_nx].clone() for p in planes]
    n = run.fallback.refine(fell, u0, t0, t1, 0.5 * dt0)
    assert n == fallen and run.fallback.refined == n
    assert run.fallback.ensembles >= 1  # the patches ran together in ensemble launches
    h2 = sim.field("W") - bc
    # the same re-solve with one patch run after another ends in the same state
    after = [p[:v.h_ny, :v.h_nx].clone() for p in planes]
    for p, b in zip(planes, before):
        p[:v.h_ny, :v.h_nx].copy_(b)
    one_by_one = closure.FineFallback(sim, fine, batch=False)
    assert one_by_one.refine(fell, u0, t0, t1, 0.5 * dt0) == n and one_by_one.ensembles == 0
    for p, a in zip(planes, after):
        assert (p[:v.h_ny, :v.h_nx] - a).abs().max().item() <= 1e-4
        p[:v.h_ny, :v.h_nx].copy_(a)
    torch.cuda.synchronize()
    one_by_one.close()
    v2 = sim.volume()
    assert abs(v2 - v1) <= 1e-6 * v1, (v1, v2)
    eps = 1.19209e-07
    inner = (slice(2, -2), slice(2, -2))
    assert np.array_equal(h1[inner] > eps, h2[inner] > eps)
    d = np.abs(h2 - h1)
    assert d[3:-3, 3:-3].max() > 0
    assert d[2, :].max() == 0 and d[-3, :].max() == 0 and d[:, 2].max() == 0 and d[:, -3].max() == 0
    assert (h2[inner] >= 0).all() and d.max() < 1.0
    # a run with the fallback on
    t = run.run(400.0)
    assert t >= 400.0 and np.isfinite(sim.field("W")).all()
    vol, added = sim.mass_ledger()
    assert abs(vol - added) <= 1e-4 * added
    run.fallback.close()
