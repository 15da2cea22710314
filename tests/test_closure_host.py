"""Host-side logic of the learned flux closure (no GPU): the parameter
layout against PyTorch's convolution weights, the coarse-grid geometry, the
face masks and the patch cutter."""
import dataclasses

import numpy as np

from rift_gb300 import closure, synth


def test_parameter_layout_round_trips_through_torch_weights():
    import torch

    p = closure.init_params(1)
    assert p.shape == (closure.NPARAM,) and p.dtype == np.float32
    W1, b1, W2, b2, W3, b3 = closure.unpack(p)
    assert W1.shape == (32, 6, 5, 5) and W2.shape == (32, 32, 3, 3) and W3.shape == (4, 32, 1, 1)
    assert b1.shape == (32,) and b2.shape == (32,) and b3.shape == (4,)
    # W1[o][(dy*5 + dx)*6 + c] is torch's W1[o, c, dy, dx]
    w1 = p[closure.OFF_W1:closure.OFF_B1].reshape(32, 160)
    assert W1[7, 4, 2, 3].item() == w1[7, (2 * 5 + 3) * 6 + 4]
    assert (w1[:, 150:] == 0).all()
    w2 = p[closure.OFF_W2:closure.OFF_B2].reshape(32, 288)
    assert W2[5, 31, 1, 2].item() == w2[5, (1 * 3 + 2) * 32 + 31]
    assert (p[closure.OFF_W3 + 128:closure.OFF_B3] == 0).all()


def test_torch_statement_centres_the_bed_on_each_window():
    """Adding a constant to the bed channel leaves the net's output unchanged."""
    import torch

    rng = np.random.default_rng(0)
    x = torch.as_tensor(rng.normal(0, 1, (2, 6, 20, 20)).astype(np.float32))
    p = torch.as_tensor(closure.init_params(2))
    a = closure.torch_forward(x, p)
    x2 = x.clone()
    x2[:, 3] += 17.0
    b = closure.torch_forward(x2, p)
    assert a.shape == (2, 4, 14, 14)
    assert torch.allclose(a, b, atol=1e-4)


def test_coarse_case_geometry():
    f = closure.scenario(0, N=64, cell=2.0)
    c = closure.coarse_case(f)
    assert c.b_nx == 33 and c.cell == 4.0
    assert c.h_nx - 4 == (f.h_nx - 4) // 2
    assert np.array_equal(c.B, f.B[::2, ::2])
    np.testing.assert_allclose(c.n[2:-2, 2:-2], closure.restrict(f.n[2:-2, 2:-2]))
    assert c.flags == f.flags and c.series.keys() == f.series.keys()
    assert c.flags & synth.SAVE_MAX and c.flags & synth.SAVE_ARRIVAL


def test_scenarios_alternate_generators_and_rain():
    a, b = closure.scenario(0, N=64), closure.scenario(1, N=64)
    assert a.flags & synth.RAIN_UNIFORM and not a.flags & synth.INFILTRATION
    assert b.K is None and b.src_idx is None
    ra = closure.uniform_rate(a, 100.0)
    assert 30 / 3.6e6 <= ra <= 80 / 3.6e6
    assert closure.uniform_rate(a, 3000.0) == 0.0


def test_restrict_preserves_the_mean():
    a = np.arange(48, dtype=float).reshape(6, 8)
    r = closure.restrict(a)
    assert r.shape == (3, 4)
    assert r[0, 0] == np.mean([0, 1, 8, 9])
    assert np.isclose(r.mean(), a.mean())


def test_face_mask_follows_the_kernel_gate():
    h = np.zeros((6, 7))
    h[1:5, 1:6] = 0.05
    h[2, 3] = 0.001
    east, north = closure.face_mask(h, 0.01)
    # both cells deeper than hmin and one cell inside the interior's edge
    assert east[1, 1] and east[1, 4] and not east[1, 5]
    assert not east[2, 2] and not east[2, 3]
    assert north[1, 1] and not north[1, 3] and not north[4, 1]
    assert not east[0].any() and not north[:, 0].any()


def test_patch_cutter_repeats_edges_and_filters():
    n = 128
    planes = np.zeros((6, n, n), np.float32)
    planes[0] = np.arange(n)[None, :]
    masks = np.zeros((4, n, n), np.float32)
    masks[:, :64, :64] = 1.0
    tg = masks * 2.0
    out = closure._patches(planes, masks, tg, 0.05)
    assert len(out) == 1
    f, t, m = out[0]
    assert f.shape == (6, 70, 70) and t.shape == (4, 64, 64)
    assert f[0, 0, 0] == 0 and f[0, 0, 3] == 0 and f[0, 0, 4] == 1
    assert (t == 2).all() and (m == 1).all()


def test_even_side_and_coarse_point_sources():
    cases = synth.config5(members=2, side=(33, 33), tf=600.0)
    c = cases[1]                      # odd side, with a point source
    assert (c.b_nx - 1) % 2 == 1 and c.src_idx is not None
    e = closure.even_side(c)
    assert e.b_nx - 1 == 32 and e.n.shape == (e.h_ny, e.h_nx)
    j, i = divmod(int(c.src_idx[0]), c.h_nx)
    je, ie = divmod(int(e.src_idx[0]), e.h_nx)
    assert (je, ie) == (min(j, e.h_ny - 3), min(i, e.h_nx - 3))
    k = closure.coarse_case(e)
    J, I = divmod(int(k.src_idx[0]), k.h_nx)
    assert (J, I) == (2 + (je - 2) // 2, 2 + (ie - 2) // 2)
    assert 2 <= J <= k.h_ny - 3 and 2 <= I <= k.h_nx - 3


def test_fine_patch_geometry():
    """A fine re-solve patch covers the block and its halo of coarse cells at
    the fine resolution: its corner DEM is the fine DEM under those cells,
    its n the fine cells' n, and point sources inside it keep their cells."""
    from rift_gb300 import closure, synth
    fine = closure.scenario(0, N=128, cell=2.0)
    fine = dataclasses.replace(fine, src_idx=np.array([(40 + 2) * fine.h_nx + (50 + 2)], np.int32),
                               flags=fine.flags | synth.POINT_SOURCE)
    cc = closure.coarse_case(fine)
    ny = cc.h_ny
    j0, i0 = 2 + 16, 2 + 16  # block (1, 1)
    Ja, Jb = closure.patch_range(j0, j0 + 16, 4, ny)
    Ia, Ib = closure.patch_range(i0, i0 + 16, 4, ny)
    assert (Ja, Jb, Ia, Ib) == (14, 38, 14, 38)
    p = closure.fine_patch_case(fine, Ja, Jb, Ia, Ib)
    assert p.B.shape == (49, 49) and p.cell == fine.cell
    np.testing.assert_array_equal(p.B, fine.B[24:73, 24:73])
    np.testing.assert_array_equal(p.n[2:-2, 2:-2], fine.n[2 + 24:2 + 72, 2 + 24:2 + 72])
    # fine cell (40, 50) is patch cell (16, 26), plus the ghost ring
    assert list(p.src_idx) == [(16 + 2) * p.h_nx + (26 + 2)]
    # the edge of the domain clips the halo
    assert closure.patch_range(2, 18, 4, ny) == (2, 22)
    assert closure.patch_range(ny - 18, ny - 2, 4, ny) == (ny - 22, ny - 2)
