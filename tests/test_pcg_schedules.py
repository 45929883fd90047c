"""Index schedules of the two warp-per-tile PCG kernels (vare_gb300/csrc/projection.cu),
restated lane by lane in numpy and checked on the CPU: every shared-memory read stays
inside the warp's buffers, and the schedules reproduce the plain forms they replace bit
for bit (same float32 operations in the same order).

* k_pcg_update: block-MIC(0) forward and backward sweeps; lane L owns tile rows L and
  L + 32, cell (i, j, k) is staged at i + 8 j + 73 k after 80 guard cells, and step u
  handles cell i = u - (j + k) - 1 of every row.
* k_pcg_direction: q = A d' with x neighbours from the lane's own registers, y and z
  neighbours by shuffles, and the face cells of the six neighbour tiles loaded by the
  boundary rows.

numpy evaluates a*b + c with two roundings; the reference forms below do the same, so
the comparison is exact (the kernels use fused multiply-adds in both places).
"""
import numpy as np

F = np.float32

# k_pcg_update constants (namespace micsweep)
PLANE, GUARD = 73, 80
BUF = GUARD + 7 * PLANE + 64 + PLANE + 7


def mic_wavefront(r, m):
    """z = M^-1 r over the tile's 22 planes i+j+k = p (forward, then backward)."""
    y = r.copy()
    for p in range(22):
        for k in range(8):
            for j in range(8):
                i = p - j - k
                if not 0 <= i < 8:
                    continue
                l = i + 8 * j + 64 * k
                t = F(y[l])
                if i:
                    t = F(m[l - 1] * y[l - 1] + t)
                if j:
                    t = F(m[l - 8] * y[l - 8] + t)
                if k:
                    t = F(m[l - 64] * y[l - 64] + t)
                y[l] = F(t * m[l])
    for p in range(21, -1, -1):
        for k in range(8):
            for j in range(8):
                i = p - j - k
                if not 0 <= i < 8:
                    continue
                l = i + 8 * j + 64 * k
                acc = F(0)
                if i < 7:
                    acc = F(acc + y[l + 1])
                if j < 7:
                    acc = F(acc + y[l + 8])
                if k < 7:
                    acc = F(acc + y[l + 64])
                y[l] = F(F(m[l] * acc + y[l]) * m[l])
    return y


def mic_lane_schedule(r, m):
    """The k_pcg_update schedule: per step, every lane reads its operands, then all lanes
    write (the __syncwarp between steps). Returns z and the range of buffer indices read."""
    V = np.zeros(BUF, F)
    P = np.zeros(BUF, F)
    lo, hi = BUF, -1

    def rd(a, idx):
        nonlocal lo, hi
        x = GUARD + idx
        lo, hi = min(lo, x), max(hi, x)
        assert 0 <= x < BUF
        return a[x]

    lanes = []
    for L in range(32):
        j, kq = L & 7, L >> 3
        sA = j + kq
        rA = 8 * j + PLANE * kq
        rB = rA + 4 * PLANE
        lanes.append(dict(j=j, kq=kq, sA=sA, oA=rA - sA - 1, oB=rB - (sA + 4) - 1))
        for i in range(8):  # staging: float4 c = lane + 32 m holds cells 4c..4c+3
            for k, base in ((kq, rA), (kq + 4, rB)):
                V[GUARD + base + i] = r[i + 8 * j + 64 * k]
                P[GUARD + base + i] = m[i + 8 * j + 64 * k]
    state = [dict(yA=F(0), mA=F(0), yB=F(0), mB=F(0)) for _ in range(32)]
    for u in range(1, 23):
        writes = []
        for L, d in enumerate(lanes):
            for row in "AB":
                if (row == "A" and u > 18) or (row == "B" and u < 5):
                    continue
                o = (d["oA"] if row == "A" else d["oB"]) + u
                s = d["sA"] + (0 if row == "A" else 4)
                zm = d["kq"] > 0 if row == "A" else True
                act = 0 <= u - s - 1 < 8
                st = state[L]
                t = F(st["m" + row] * st["y" + row] + rd(V, o))
                t = F((rd(P, o - 8) if d["j"] > 0 else F(0)) * rd(V, o - 8) + t)
                t = F((rd(P, o - PLANE) if zm else F(0)) * rd(V, o - PLANE) + t)
                mm = rd(P, o) if act else F(0)
                y = F(t * mm)
                st["y" + row], st["m" + row] = y, mm
                if act:
                    writes.append((o, y))
        for o, y in writes:
            V[GUARD + o] = y
    state = [dict(zA=F(0), zB=F(0)) for _ in range(32)]
    for u in range(22, 0, -1):
        writes = []
        for L, d in enumerate(lanes):
            for row in "BA":
                if (row == "A" and u > 18) or (row == "B" and u < 5):
                    continue
                o = (d["oA"] if row == "A" else d["oB"]) + u
                s = d["sA"] + (0 if row == "A" else 4)
                zp = d["kq"] < 3 if row == "B" else True
                act = 0 <= u - s - 1 < 8
                acc = F(0)
                acc = F(acc + state[L]["z" + row])
                acc = F(acc + (rd(V, o + 8) if d["j"] < 7 else F(0)))
                acc = F(acc + (rd(V, o + PLANE) if zp else F(0)))
                mm = rd(P, o) if act else F(0)
                z = F(F(mm * acc + rd(V, o)) * mm)
                state[L]["z" + row] = z
                if act:
                    writes.append((o, z))
        for o, z in writes:
            V[GUARD + o] = z
    out = np.zeros(512, F)
    for L, d in enumerate(lanes):
        j, kq = d["j"], d["kq"]
        for i in range(8):
            out[i + 8 * j + 64 * kq] = V[GUARD + 8 * j + PLANE * kq + i]
            out[i + 8 * j + 64 * (kq + 4)] = V[GUARD + 8 * j + PLANE * (kq + 4) + i]
    return out, lo, hi


def test_update_sweep_schedule_matches_wavefront():
    rng = np.random.default_rng(7)
    for _ in range(3):
        m = rng.uniform(0.2, 1.0, 512).astype(F)
        r = rng.standard_normal(512).astype(F)
        dead = rng.random(512) < 0.25  # non-fluid cells: pivot 0 and r = 0
        m[dead] = 0
        r[dead] = 0
        z, lo, hi = mic_lane_schedule(r, m)
        np.testing.assert_array_equal(z, mic_wavefront(r, m))
        assert lo >= 0 and hi < BUF


def test_update_staging_addresses():
    """The coalesced staging writes float4 c = lane + 32 m (cells 4c..4c+3) at
    4 lane + 9 (lane >> 4) + 146 m: the cell's i + 8 j + 73 k."""
    for lane in range(32):
        for mm in range(4):
            c = lane + 32 * mm
            for e in range(4):
                l = 4 * c + e
                i, j, k = l & 7, (l >> 3) & 7, l >> 6
                assert 4 * lane + 9 * (lane >> 4) + 146 * mm + e == i + 8 * j + PLANE * k


def test_direction_shuffle_schedule_matches_stencil():
    """q = diag d' - (sum of the six face neighbours' d', order -x +x -y +y -z +z) on a
    3^3 grid of tiles with inactive tiles, by direct indexing and by the lane schedule."""
    rng = np.random.default_rng(3)
    T = 3
    slot = -np.ones((T, T, T), int)
    pos, n = {}, 0
    for z in range(T):
        for y in range(T):
            for x in range(T):
                if rng.random() < 0.8:
                    slot[z, y, x] = n
                    pos[n] = (x, y, z)
                    n += 1
    d = rng.standard_normal(n * 512).astype(F)
    zz = rng.standard_normal(n * 512).astype(F)
    fluid = rng.random(n * 512) < 0.7
    d[~fluid] = 0
    zz[~fluid] = 0
    diag = rng.integers(0, 7, n * 512)
    beta = F(0.37)
    dn = (beta * d + zz).astype(F)

    def tile_at(x, y, z):
        return slot[z, y, x] if 0 <= x < T and 0 <= y < T and 0 <= z < T else -1

    def val(s, i, j, k):
        x, y, z = pos[s]
        g = (x * 8 + i, y * 8 + j, z * 8 + k)
        t = tile_at(g[0] // 8, g[1] // 8, g[2] // 8) if min(g) >= 0 else -1
        return F(0) if t < 0 else dn[t * 512 + g[0] % 8 + 8 * (g[1] % 8) + 64 * (g[2] % 8)]

    ref = np.zeros(n * 512, F)
    for s in range(n):
        for l in range(512):
            if not fluid[s * 512 + l]:
                continue
            i, j, k = l & 7, (l >> 3) & 7, l >> 6
            acc = F(0)
            for a, b, c in ((i - 1, j, k), (i + 1, j, k), (i, j - 1, k), (i, j + 1, k), (i, j, k - 1), (i, j, k + 1)):
                acc = F(acc + val(s, a, b, c))
            ref[s * 512 + l] = F(F(diag[s * 512 + l]) * dn[s * 512 + l] - acc)

    def face(s, dx, dy, dz):
        x, y, z = pos[s]
        return tile_at(x + dx, y + dy, z + dz)

    def h8(t, c):
        return [F(0)] * 8 if t < 0 else [dn[t * 512 + c + e] for e in range(8)]

    def h1(t, c):
        return F(0) if t < 0 else dn[t * 512 + c]

    got = np.zeros_like(ref)
    for s in range(n):
        smx, spx, smy, spy, smz, spz = (face(s, -1, 0, 0), face(s, 1, 0, 0), face(s, 0, -1, 0),
                                        face(s, 0, 1, 0), face(s, 0, 0, -1), face(s, 0, 0, 1))
        dA = [[dn[s * 512 + 8 * L + i] for i in range(8)] for L in range(32)]
        dB = [[dn[s * 512 + 256 + 8 * L + i] for i in range(8)] for L in range(32)]
        halo = []
        for L in range(32):
            j, kq = L & 7, L >> 3
            yt = smy if j == 0 else (spy if j == 7 else -1)
            yc = 8 * (L - j) + (56 if j == 0 else 0)
            zt = smz if kq == 0 else (spz if kq == 3 else -1)
            zc = 8 * j + (448 if kq == 0 else 0)
            halo.append(dict(xmA=h1(smx, 8 * L + 7), xpA=h1(spx, 8 * L), xmB=h1(smx, 256 + 8 * L + 7),
                             xpB=h1(spx, 256 + 8 * L), yA=h8(yt, yc), yB=h8(yt, yc + 256), z=h8(zt, zc)))
        for i in range(8):
            colA = [dA[L][i] for L in range(32)]
            colB = [dB[L][i] for L in range(32)]
            for L in range(32):
                j, kq, h = L & 7, L >> 3, halo[L]

                def up(col, dl):  # __shfl_up_sync: lanes below dl keep their own value
                    return col[L - dl] if L >= dl else col[L]

                def down(col, dl):  # __shfl_down_sync
                    return col[L + dl] if L + dl < 32 else col[L]

                ymA, ypA, ymB, ypB = up(colA, 1), down(colA, 1), up(colB, 1), down(colB, 1)
                if j == 0:
                    ymA, ymB = h["yA"][i], h["yB"][i]
                if j == 7:
                    ypA, ypB = h["yA"][i], h["yB"][i]
                zmA = h["z"][i] if kq == 0 else up(colA, 8)
                src = (L + 8) & 31
                zpA = colB[src] if (src >> 3) == 0 else colA[src]
                src = (L + 24) & 31
                zmB = colA[src] if (src >> 3) == 3 else colB[src]
                zpB = h["z"][i] if kq == 3 else down(colB, 8)
                xmA = dA[L][i - 1] if i > 0 else h["xmA"]
                xpA = dA[L][i + 1] if i < 7 else h["xpA"]
                xmB = dB[L][i - 1] if i > 0 else h["xmB"]
                xpB = dB[L][i + 1] if i < 7 else h["xpB"]
                for off, nbs, dd in ((0, (xmA, xpA, ymA, ypA, zmA, zpA), dA), (256, (xmB, xpB, ymB, ypB, zmB, zpB), dB)):
                    l = s * 512 + off + 8 * L + i
                    if not fluid[l]:
                        continue
                    acc = F(0)
                    for v in nbs:
                        acc = F(acc + v)
                    got[l] = F(F(diag[l]) * dd[L][i] - acc)
    np.testing.assert_array_equal(got, ref)


def test_p2g_dual_cells_each_taken_once():
    """k_p2g (p2g.cu) hands its threads the tile's 512 dual cells, then the 217 of its low-side
    halo, by item number: restated here, the items cover the 9^3 dual cells of tile-local
    coordinates -1..7 exactly once."""
    seen = set()
    for item in range(512 + 217):
        if item < 512:
            d = (item & 7, (item >> 3) & 7, item >> 6)
        else:
            hh = item - 512
            if hh < 81:
                d = (hh % 9 - 1, hh // 9 - 1, -1)
            elif hh < 153:
                u = hh - 81
                d = (u % 9 - 1, -1, u // 9)
            else:
                u = hh - 153
                d = (-1, u & 7, u >> 3)
        assert all(-1 <= c <= 7 for c in d)
        assert d not in seen
        seen.add(d)
    assert len(seen) == 9 ** 3
