"""The operand layouts of the closure's tensor-core forward pass, on the CPU.

A numpy model of one 16 x 16 block as `k_forward` / `k_closure` compute it:
the shared-memory images the kernels build (the BF16 input cells, the
layer-1 weight blocks with their zero block, the layer-2 weight blocks, the
four 8-channel planes of the layer-1 activations), every tcgen05.mma read
through the descriptor arithmetic of `tcIssue1` / `tcIssue2` (K-major, no
swizzle: row r, column k of an operand at start + (r/8) SBO + (k/8) LBO +
(r%8) 16 + (k%8) 2 bytes), the two epilogues and layer 3.  The result is
compared with a direct statement of the convolutions with the same BF16
roundings, so a wrong offset, stride, weight block or plane shows as an O(1)
error; the GPU tests check the hardware's reading of the same descriptors
(`rift_closure_selftest`) and the whole kernel against PyTorch.
"""
import numpy as np

RI, XBC, A1C, OT = 22, 640, 432, 16
M1TC, M2TC, KS1, KS2 = 4, 3, 15, 18
MAP = [0, 1, 2, 3, 3, 4, 5, -1]  # BF16 input channel -> net input channel


def bf16(x):
    """Round FP32 to BF16 (nearest even), returned as FP32."""
    a = np.asarray(x, dtype=np.float32).copy()
    u = a.view(np.uint32)
    u += np.uint32(0x7FFF) + ((u >> 16) & 1)
    u &= np.uint32(0xFFFF0000)
    return a


def operand(mem, start, lbo, sbo, rows):
    """rows x 16 operand read from a flat BF16 image (element = 2 bytes)."""
    r = np.arange(rows)[:, None]
    k = np.arange(16)[None, :]
    byte = start + (r // 8) * sbo + (k // 8) * lbo + (r % 8) * 16 + (k % 8) * 2
    assert (byte % 2 == 0).all() and byte.max() < 2 * mem.size
    return mem[byte // 2]


def test_tensor_core_block_matches_the_convolutions():
    rng = np.random.default_rng(5)
    x = rng.normal(0, 1, (RI * RI, 6)).astype(np.float32)  # scaled inputs, cell-major
    x[:, 3] = 30 + rng.normal(0, 0.5, RI * RI).astype(np.float32)  # bed
    W1 = rng.normal(0, 0.2, (32, 25, 6)).astype(np.float32)  # [o][dy*5+dx][c]
    W2 = rng.normal(0, 0.1, (32, 9, 32)).astype(np.float32)  # [o][dy*3+dx][c]
    W3 = rng.normal(0, 0.3, (4, 32)).astype(np.float32)
    b1, b2, b3 = (rng.normal(0, 0.1, n).astype(np.float32) for n in (32, 32, 4))
    bref = x[(RI // 2) * RI + RI // 2, 3]

    # ---- shared-memory images (tcStoreInput, tcSetup) ----
    xb = np.zeros((XBC, 8), np.float32)
    br = x[:, 3] - bref
    bh = bf16(br)
    xb[:RI * RI] = np.stack([bf16(x[:, 0]), bf16(x[:, 1]), bf16(x[:, 2]), bh, bf16(br - bh),
                             bf16(x[:, 4]), bf16(x[:, 5]), np.zeros(RI * RI, np.float32)], 1)
    w1t = np.zeros((26, 32, 8), np.float32)
    for c8, c in enumerate(MAP):
        if c >= 0:
            w1t[:25, :, c8] = bf16(W1[:, :, c]).T
    w2t = np.zeros((36, 32, 8), np.float32)
    for blk in range(36):
        w2t[blk] = bf16(W2[:, blk >> 2, (blk & 3) * 8:(blk & 3) * 8 + 8])
    sbed = bf16(W1[:, :, 3]).sum(1)

    # ---- layer 1 (tcIssue1 + tcEpilogue1) ----
    xbm, w1m = xb.reshape(-1), w1t.reshape(-1)
    a1 = np.zeros((4, A1C, 8), np.float32)
    for mt in range(M1TC):
        D = np.zeros((128, 32), np.float64)
        for s in range(KS1):
            cell = mt * 128 + (s // 5) * 2 * RI + s % 5
            T0 = (s // 5) * 10 + s % 5
            T1 = T0 + 5 if s < 10 else 25
            A = operand(xbm, cell * 16, RI * 16, 128, 128)
            B = operand(w1m, T0 * 512, (T1 - T0) * 512, 128, 32)
            D += A.astype(np.float64) @ B.T.astype(np.float64)
        for r in range(128):
            m = mt * 128 + r
            if m >= A1C:
                continue
            cb = x[m + 2 * RI + 2, 3] - bref
            v = np.maximum(D[r].astype(np.float32) + b1 - cb * sbed, 0)
            a1[:, m, :] = bf16(v).reshape(4, 8)

    # ---- layer 2 (tcIssue2) and layer 3 (tcOutputs) ----
    a1m = a1.reshape(-1)
    out = np.full((OT, OT, 4), np.nan, np.float32)
    for mt in range(M2TC):
        D = np.zeros((128, 32), np.float64)
        for s in range(KS2):
            tap, kb = s >> 1, s & 1
            cell = kb * 2 * A1C + mt * 128 + (tap // 3) * RI + tap % 3
            A = operand(a1m, cell * 16, A1C * 16, 128, 128)
            B = operand(w2t.reshape(-1), (tap * 4 + 2 * kb) * 512, 512, 128, 32)
            D += A.astype(np.float64) @ B.T.astype(np.float64)
        for r in range(128):
            m = mt * 128 + r
            oy, ox = divmod(m, RI)
            if oy < OT and ox < OT:
                a2 = np.maximum(D[r].astype(np.float32) + b2, 0)
                out[oy, ox] = W3 @ a2 + b3
    assert not np.isnan(out).any()  # every output cell came from a valid MMA row

    # ---- direct statement: valid convolutions on the 22 x 22 block ----
    X = xb[:RI * RI].reshape(RI, RI, 8)
    Wf = np.zeros((32, 5, 5, 8), np.float32)
    for c8, c in enumerate(MAP):
        if c >= 0:
            Wf[..., c8] = bf16(W1[:, :, c]).reshape(32, 5, 5)
    z1 = np.zeros((18, 18, 32), np.float64)
    for dy in range(5):
        for dx in range(5):
            z1 += X[dy:dy + 18, dx:dx + 18].astype(np.float64) @ Wf[:, dy, dx].T.astype(np.float64)
    cb = x[:, 3].reshape(RI, RI)[2:20, 2:20] - bref
    A1 = bf16(np.maximum(z1.astype(np.float32) + b1 - cb[..., None] * sbed, 0))
    W2f = bf16(W2).reshape(32, 3, 3, 32)
    z2 = np.zeros((OT, OT, 32), np.float64)
    for dy in range(3):
        for dx in range(3):
            z2 += A1[dy:dy + OT, dx:dx + OT].astype(np.float64) @ W2f[:, dy, dx].T.astype(np.float64)
    ref = np.maximum(z2.astype(np.float32) + b2, 0) @ W3.T + b3
    err = np.abs(out - ref).max() / np.abs(ref).max()
    assert err < 1e-3, err  # summation order only (an activation's BF16 rounding may flip)
