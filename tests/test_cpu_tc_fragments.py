"""The index arithmetic of the tensor-core training kernels (waves_gb300/csrc/k_train.cu,
WAVES_NET_TENSOR) restated on the CPU with the fragment semantics of ldmatrix (plain and .trans)
and mma.sync m16n8k16 from the PTX ISA, against a numpy convolution: the B-fragment packing of
k_tc_frag, the halo staging and lane addresses of k_tc_conv (forward, last layer, input gradient
with the mirrored taps) and k_tc_grad_w (both operands transposed), every shared-memory row in
bounds and 16-byte aligned, every partial written.  Ragged sizes: two x blocks, a partial y block,
a partial z chunk."""
import numpy as np

def bf16(a):
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    return (((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16).astype(np.uint32).view(np.float32).astype(np.float64)

TX, TY, HX, HY, HZ, KS = 32, 4, 34, 6, 3, 24
KHALO = HX * HY * HZ
KZC = 4

def b1(v):
    return float(bf16(np.array([v]))[0])

def ldmatrix(smem, addrs, trans):
    """ldmatrix.x4 (.trans): lanes 8q..8q+7 address the eight 16-byte rows of block q; lane L
    receives row L/4, columns 2(L%4), 2(L%4)+1 of each block (transposed: rows 2(L%4), 2(L%4)+1 of
    column L/4)."""
    regs = np.zeros((32, 4, 2))
    for q in range(4):
        M = np.zeros((8, 8))
        for r in range(8):
            a = addrs[8 * q + r]
            assert a % 8 == 0, "16-byte row alignment"
            assert 0 <= a and a + 8 <= len(smem), ("smem bounds", a)
            M[r] = smem[a:a + 8]
        for L in range(32):
            if trans:
                regs[L, q] = (M[2 * (L % 4), L // 4], M[2 * (L % 4) + 1, L // 4])
            else:
                regs[L, q] = (M[L // 4, 2 * (L % 4)], M[L // 4, 2 * (L % 4) + 1])
    return regs

def mma(acc, a, b):
    """mma.sync m16n8k16: rebuild A (16x16) and B (16x8) from the lanes' fragments, D += A B."""
    A = np.full((16, 16), np.nan); B = np.full((16, 8), np.nan)
    for L in range(32):
        g, t = L // 4, L % 4
        for e in range(2):
            A[g, 2*t+e] = a[L][0][e]; A[g+8, 2*t+e] = a[L][1][e]
            A[g, 2*t+8+e] = a[L][2][e]; A[g+8, 2*t+8+e] = a[L][3][e]
            B[2*t+e, g] = b[L][0][e]; B[2*t+8+e, g] = b[L][1][e]
    assert not np.isnan(A).any() and not np.isnan(B).any()
    D = A @ B
    for L in range(32):
        g, t = L // 4, L % 4
        acc[L] += (D[g, 2*t], D[g, 2*t+1], D[g+8, 2*t], D[g+8, 2*t+1])

def frag_pack(w, ci_n, co_n, transpose):
    frag = np.zeros((27 * 2 * 32, 2, 2))
    for k in range(27 * 2 * 32):
        lane, j, tap = k & 31, (k >> 5) & 1, k >> 6
        n, t = 8 * j + (lane >> 2), lane & 3
        def val(kk):
            if transpose:
                return w[kk, 26 - tap, n] if (n < ci_n and kk < co_n) else 0.0
            return w[n, tap, kk] if (n < co_n and kk < ci_n) else 0.0
        frag[k, 0] = (b1(val(2*t)), b1(val(2*t+1)))
        frag[k, 1] = (b1(val(2*t+8)), b1(val(2*t+9)))
    return frag

def at(S, x, y, z):
    B, nz, ny, nx = S
    return (z * ny + y) * nx + x

def stage_halo(S, src_b, x0, y0, z):
    B, nz, ny, nx = S
    tile = np.zeros(KHALO * KS)
    for c in range(KHALO):
        hx, hy, hz = c % HX, (c // HX) % HY, c // (HX * HY)
        gx, gy, gz = x0 + hx - 1, y0 + hy - 1, z + hz - 1
        if 0 <= gx < nx and 0 <= gy < ny and 0 <= gz < nz:
            tile[c*KS:c*KS+16] = src_b[at(S, gx, gy, gz)]
    return tile

def conv(S, inp, frag, bias, n_bias, z_prev, NTILES, MODE):
    """inp [B*C][16]; returns out (FP channel-first) and out16 [B*C][16]"""
    B, nz, ny, nx = S
    C = nz * ny * nx
    out = np.full((B, 16 if MODE != 1 else 1, C), np.nan)
    out16 = np.full((B * C, 16), np.nan)
    gx_n, gy_n = (nx + TX - 1) // TX, (ny + TY - 1) // TY
    sb = np.array([(bias[i] if (MODE != 2 and i < n_bias) else 0.0) for i in range(16)])
    for bz in range(B * nz):
        z, b = bz % nz, bz // nz
        for bx in range(gx_n):
            for by in range(gy_n):
                x0, y0 = bx * TX, by * TY
                tile = stage_halo(S, inp[b*C:(b+1)*C], x0, y0, z)
                for warp in range(8):
                    wx, wy = (warp & 1) * 16, warp >> 1
                    acc = np.zeros((NTILES, 32, 4))
                    for tap in range(27):
                        kx, ky, kz = tap % 3, (tap // 3) % 3, tap // 9
                        addrs = []
                        for lane in range(32):
                            row = (lane & 7) + ((lane >> 3) & 1) * 8; half = (lane >> 4) * 8
                            cell = (kz * HY + wy + ky) * HX + wx + kx + row
                            addrs.append(cell * KS + half)
                        a = ldmatrix(tile, addrs, False)
                        for j in range(NTILES):
                            bfr = np.array([frag[(tap * 2 + j) * 32 + lane] for lane in range(32)])
                            mma(acc[j], a, bfr)
                    for lane in range(32):
                        g, t = lane >> 2, lane & 3
                        y = y0 + wy
                        for hrow in range(2):
                            x = x0 + wx + g + 8 * hrow
                            if x >= nx or y >= ny: continue
                            cell = at(S, x, y, z)
                            if MODE == 1:
                                if t == 0: out[b, 0, cell] = acc[0][lane][2*hrow] + sb[0]
                            else:
                                for j in range(NTILES):
                                    n = j * 8 + 2 * t
                                    v0 = acc[j][lane][2*hrow] + sb[n]; v1 = acc[j][lane][2*hrow+1] + sb[n+1]
                                    if MODE == 2:
                                        v0 = v0 if z_prev[b, n, cell] > 0 else 0.0
                                        v1 = v1 if z_prev[b, n+1, cell] > 0 else 0.0
                                        out16[b*C+cell, n:n+2] = (b1(v0), b1(v1))
                                    else:
                                        out16[b*C+cell, n:n+2] = (b1(max(v0, 0)), b1(max(v1, 0)))
                                    out[b, n, cell] = v0; out[b, n+1, cell] = v1
    return out, out16

def grad_w(S, g16, act):
    B, nz, ny, nx = S
    C = nz * ny * nx
    chunks = (nz + KZC - 1) // KZC
    gx_n, gy_n = (nx + TX - 1) // TX, (ny + TY - 1) // TY
    nblk = gx_n * gy_n * B * chunks
    part = np.full((nblk, 16 * 27 * 16), np.nan)
    for bz in range(B * chunks):
        for by in range(gy_n):
            for bx in range(gx_n):
                b, z0 = bz // chunks, (bz % chunks) * KZC
                z1 = min(z0 + KZC, nz)
                x0, y0 = bx * TX, by * TY
                accs = [np.zeros((4, 2, 32, 4)) for _ in range(8)]
                for z in range(z0, z1):
                    tile = stage_halo(S, act[b*C:(b+1)*C], x0, y0, z)
                    gt = np.zeros(TX * TY * KS)
                    for c in range(TX * TY):
                        gx, gy = x0 + c % TX, y0 + c // TX
                        if gx < nx and gy < ny:
                            gt[c*KS:c*KS+16] = g16[b*C + at(S, gx, gy, z)]
                    for warp in range(8):
                        ntaps = 4 if warp < 3 else 3
                        for seg in range(8):
                            wx, wy = (seg & 1) * 16, seg >> 1
                            aad, = [[((wy * TX + wx + ((l & 7) + (l >> 4) * 8)) * KS + ((l >> 3) & 1) * 8) for l in range(32)]]
                            a = ldmatrix(gt, aad, True)
                            for i in range(4):
                                if i >= ntaps: continue
                                tap = warp + 8 * i
                                kx, ky, kz = tap % 3, (tap // 3) % 3, tap // 9
                                bad = [((kz * HY + wy + ky) * HX + wx + kx + ((l & 7) + ((l >> 3) & 1) * 8)) * KS + (l >> 4) * 8 for l in range(32)]
                                bb = ldmatrix(tile, bad, True)
                                mma(accs[warp][i][0], a, bb[:, 0:2])
                                mma(accs[warp][i][1], a, bb[:, 2:4])
                blk = bx + gx_n * (by + gy_n * bz)
                for warp in range(8):
                    ntaps = 4 if warp < 3 else 3
                    for lane in range(32):
                        g, t = lane >> 2, lane & 3
                        for i in range(ntaps):
                            tap = warp + 8 * i
                            for j in range(2):
                                ci = j * 8 + 2 * t
                                acc = accs[warp][i][j][lane]
                                part[blk, (g*27+tap)*16+ci] = acc[0]; part[blk, (g*27+tap)*16+ci+1] = acc[1]
                                part[blk, ((g+8)*27+tap)*16+ci] = acc[2]; part[blk, ((g+8)*27+tap)*16+ci+1] = acc[3]
    assert not np.isnan(part).any(), "partial not fully written"
    return part.sum(axis=0).reshape(16, 27, 16)

# ---- numpy references ----
def offs():
    return [(t % 3 - 1, (t // 3) % 3 - 1, t // 9 - 1) for t in range(27)]

def shift(a, ox, oy, oz):
    """a[..., z, y, x] -> a[..., z+oz, y+oy, x+ox] with zero outside"""
    out = np.zeros_like(a)
    nz, ny, nx = a.shape[-3:]
    zs = slice(max(0, -oz), min(nz, nz - oz)); ys = slice(max(0, -oy), min(ny, ny - oy)); xs = slice(max(0, -ox), min(nx, nx - ox))
    zs2 = slice(zs.start + oz, zs.stop + oz); ys2 = slice(ys.start + oy, ys.stop + oy); xs2 = slice(xs.start + ox, xs.stop + ox)
    out[..., zs, ys, xs] = a[..., zs2, ys2, xs2]
    return out

def conv_ref(a, w, bias):
    """a [B][ci][z][y][x], w [co][27][ci] -> [B][co][z][y][x]"""
    co = w.shape[0]
    out = np.zeros((a.shape[0], co) + a.shape[2:]) + bias[None, :, None, None, None]
    for t, (ox, oy, oz) in enumerate(offs()):
        out += np.einsum('oc,bczyx->bozyx', w[:, t, :], shift(a, ox, oy, oz))
    return out

def test_tensor_core_training_kernels_index_arithmetic():
    rng = np.random.default_rng(0)
    B, nz, ny, nx = 1, 5, 6, 37
    S = (B, nz, ny, nx); C = nz * ny * nx
    CH = [(3, 16), (16, 16), (16, 16), (16, 1)]
    x = rng.normal(size=(B, 3, nz, ny, nx))
    ws = [rng.normal(0, 1/np.sqrt(27*ci), size=(co, 27, ci)) for ci, co in CH]
    bs = [rng.normal(0, .1, size=co) for ci, co in CH]
    # pack x
    act = [np.zeros((B*C, 16))]
    act[0][:, :3] = bf16(x.reshape(B, 3, C).transpose(0, 2, 1).reshape(B*C, 3))
    zs = []
    for l, (ci, co) in enumerate(CH):
        fw = frag_pack(ws[l], ci, co, 0)
        if l < 3:
            z, a16 = conv(S, act[l], fw, bs[l], co, None, 2, 0)
            act.append(a16)
        else:
            z, _ = conv(S, act[l], fw, bs[l], co, None, 1, 1)
        # reference from the same BF16 input
        ain = act[l][:, :ci].reshape(B, nz, ny, nx, ci).transpose(0, 4, 1, 2, 3)
        zr = conv_ref(ain, bf16(ws[l]), bs[l]).reshape(B, co, C)
        err = np.abs(z[:, :co] - zr).max()
        assert err < 1e-9
        zs.append(z[:, :co])
    # backward: g of layer 3 (1 channel)
    g3 = rng.normal(size=(B, 1, C))
    g16 = np.zeros((B*C, 16)); g16[:, 0] = bf16(g3.reshape(-1))
    for l in (3, 2, 1, 0):
        ci, co = CH[l]
        gw = grad_w(S, g16, act[l])
        gref = np.zeros((co, 27, ci))
        gg = g16[:, :co].reshape(B, nz, ny, nx, co).transpose(0, 4, 1, 2, 3)
        aa = act[l][:, :ci].reshape(B, nz, ny, nx, ci).transpose(0, 4, 1, 2, 3)
        for t, (ox, oy, oz) in enumerate(offs()):
            gref[:, t, :] = np.einsum('bozyx,bczyx->oc', gg, shift(aa, ox, oy, oz))
        err = np.abs(gw[:co, :, :ci] - gref).max(); pad = np.abs(gw).sum() - np.abs(gw[:co, :, :ci]).sum()
        assert err < 1e-9 * max(1, np.abs(gref).max()) and pad == 0
        if l == 0: break
        ft = frag_pack(ws[l], ci, co, 1)
        zp = np.concatenate([zs[l-1]], axis=1)
        ga, ga16 = conv(S, g16, ft, None, 0, zp, 2, 2)
        # reference: ga[ci][cell] = sum_t sum_co W[co][t][ci] g[co][cell - off_t], masked
        gref_a = np.zeros((B, ci, nz, ny, nx))
        wb = bf16(ws[l])
        for t, (ox, oy, oz) in enumerate(offs()):
            gref_a += np.einsum('oc,bozyx->bczyx', wb[:, t, :], shift(gg, -ox, -oy, -oz))
        gref_a = np.where(zs[l-1].reshape(B, ci, nz, ny, nx) > 0, gref_a, 0).reshape(B, ci, C)
        err = np.abs(ga - gref_a).max()
        assert err < 1e-9
        g16 = ga16

