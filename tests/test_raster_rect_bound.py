"""The raster forward's per-triangle candidate rectangle (photara_drender_gb300/csrc/raster_tile.cuh
pixel_rect) must contain every pixel of the tile whose sample passes the reference's edge tests
(rasterize_forward.hlsl: fl(cross(a - s, b - s)) * sign >= -1e-7 for the three edges), or else decline
(the kernel then enumerates the whole tile); on 16x8 tiles the per-row spans cut from the rectangle
(raster_tile.cuh row_spans) must contain every such pixel of their row; and the 16x8 binning
(bin_rect.cuh triangle_tile_rect) may leave out only sub-tiles none of whose pixels pass. Restated here in NumPy float32,
operation by operation, and checked against brute-force edge tests over whole tiles on triangles of
every scale: microscopic ones (whose tolerance reaches beyond their bounding box), slivers, large ones
crossing the tile, vertices on the sample lattice, and odd viewports."""
import numpy as np

f = np.float32
TILE = 16


def sample_ndc(p, v0, size):
    return ((p.astype(np.float32) - f(v0) + f(0.5)) * f(2.0) / f(size) - f(1.0)).astype(np.float32)


def pixel_rect(s, area, vp, x_org, y_org, x_end, y_end):
    """NumPy float32 restatement of pixel_rect for arrays of triangles s [n, 3, 2]; returns (large, none,
    x0, x1, y0, y1, err) with absolute pixel bounds and the per-sample edge-value error bound."""
    vp = [f(v) for v in vp]
    sx, sy = s[..., 0], s[..., 1]
    mnx, mxx = np.fmin(sx[:, 0], np.fmin(sx[:, 1], sx[:, 2])), np.fmax(sx[:, 0], np.fmax(sx[:, 1], sx[:, 2]))
    mny, mxy = np.fmin(sy[:, 0], np.fmin(sy[:, 1], sy[:, 2])), np.fmax(sy[:, 0], np.fmax(sy[:, 1], sy[:, 2]))
    pxw, pyw = f(2.0) / vp[2], f(2.0) / vp[3]
    ext = np.fmax(mxx - mnx, mxy - mny)
    tsx_lo = sample_ndc(np.array([x_org]), vp[0], vp[2])[0]
    tsx_hi = sample_ndc(np.array([x_end - 1]), vp[0], vp[2])[0]
    tsy_lo = sample_ndc(np.array([y_org]), vp[1], vp[3])[0]
    tsy_hi = sample_ndc(np.array([y_end - 1]), vp[1], vp[3])[0]
    L = f(1.01) * np.fmax(np.fmax(np.abs(mxx - tsx_lo), np.abs(tsx_hi - mnx)),
                          np.fmax(np.abs(mxy - tsy_lo), np.abs(tsy_hi - mny)))
    perim = (np.abs(sx[:, 1] - sx[:, 0]) + np.abs(sy[:, 1] - sy[:, 0]) + np.abs(sx[:, 2] - sx[:, 1]) +
             np.abs(sy[:, 2] - sy[:, 1]) + np.abs(sx[:, 0] - sx[:, 2]) + np.abs(sy[:, 0] - sy[:, 2]))
    err = f(2e-6) * L * L
    tau = f(1e-7) + err
    D = f(2.0) * tau * perim / np.abs(area)
    large = ~(D <= np.fmin(pxw, pyw)) | ~(np.abs(area) >= f(1e-4) * ext * ext)
    slx = f(0.05) + f(1e-6) * (vp[2] + abs(vp[0]))
    sly = f(0.05) + f(1e-6) * (vp[3] + abs(vp[1]))
    fx0 = np.ceil(((mnx - D) + f(1.0)) * f(0.5) * vp[2] + vp[0] - f(0.5) - slx)
    fx1 = np.floor(((mxx + D) + f(1.0)) * f(0.5) * vp[2] + vp[0] - f(0.5) + slx)
    fy0 = np.ceil(((mny - D) + f(1.0)) * f(0.5) * vp[3] + vp[1] - f(0.5) - sly)
    fy1 = np.floor(((mxy + D) + f(1.0)) * f(0.5) * vp[3] + vp[1] - f(0.5) + sly)
    cx0, cx1 = np.fmax(fx0, f(x_org)), np.fmin(fx1, f(x_end - 1))
    cy0, cy1 = np.fmax(fy0, f(y_org)), np.fmin(fy1, f(y_end - 1))
    none = ~(cx0 <= cx1) | ~(cy0 <= cy1)
    return large, none, cx0, cx1, cy0, cy1, err


def covered(s, sign, px, py, vp):
    """The reference's edge tests of every triangle at every pixel (px, py): [n, pixels] bool."""
    sx = sample_ndc(px, vp[0], vp[2])[None, :]
    sy = sample_ndc(py, vp[1], vp[3])[None, :]
    cr = lambda ax, ay, bx, by: ax * by - ay * bx  # noqa: E731
    a = [(s[:, k, 0:1], s[:, k, 1:2]) for k in range(3)]
    e0 = cr(a[1][0] - sx, a[1][1] - sy, a[2][0] - sx, a[2][1] - sy)
    e1 = cr(a[2][0] - sx, a[2][1] - sy, a[0][0] - sx, a[0][1] - sy)
    e2 = cr(a[0][0] - sx, a[0][1] - sy, a[1][0] - sx, a[1][1] - sy)
    c, sg = f(-1e-7), sign[:, None]
    return ~((e0 * sg < c) | (e1 * sg < c) | (e2 * sg < c))


def triangles(rng, n):
    """Projected vertices [n, 3, 2] float32 of mixed scales around the tile at NDC (-0.1 .. 0.1)."""
    out = []
    for scale in (1e-6, 1e-5, 1e-4, 1e-3, 1e-2, 0.05, 0.3, 3.0):
        c = rng.uniform(-0.12, 0.12, size=(n, 1, 2))
        out.append(c + rng.normal(scale=scale, size=(n, 3, 2)))
    a = rng.uniform(-0.12, 0.12, size=(n, 2))
    d = rng.normal(size=(n, 2))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    nrm = np.stack([-d[:, 1], d[:, 0]], 1)
    for width in (1e-7, 1e-5, 1e-3):
        ln = rng.uniform(0.01, 0.4, size=(n, 1))
        out.append(np.stack([a, a + d * ln, a + d * ln * 0.5 + nrm * width], 1))
    return np.concatenate(out).astype(np.float32)


def check(rng, vp, tiles):
    W, H = int(vp[2]), int(vp[3])
    s = triangles(rng, 600)
    # snap some vertices onto the sample lattice (edges through pixel centres)
    lat = rng.uniform(size=s.shape[:2]) < 0.2
    k = np.round((s[..., 0] + 1) * 0.5 * vp[2] + vp[0] - 0.5)
    s[..., 0] = np.where(lat, sample_ndc(k, vp[0], vp[2]), s[..., 0])
    area = ((s[:, 1, 0] - s[:, 0, 0]) * (s[:, 2, 1] - s[:, 0, 1]) -
            (s[:, 1, 1] - s[:, 0, 1]) * (s[:, 2, 0] - s[:, 0, 0])).astype(np.float32)
    keep = ~(np.abs(area) <= f(1e-12))  # the reference skips these before the edge tests
    s, area = s[keep], area[keep]
    sign = np.where(area > 0, f(1.0), f(-1.0))
    declined = total = 0
    for tx, ty in tiles:
        x_org, y_org = tx * TILE, ty * TILE
        x_end, y_end = min(x_org + TILE, W), min(y_org + TILE, H)
        px, py = np.meshgrid(np.arange(x_org, x_end), np.arange(y_org, y_end))
        px, py = px.reshape(-1), py.reshape(-1)
        cov = covered(s, sign, px, py, vp)
        large, none, x0, x1, y0, y1, _ = pixel_rect(s, area, vp, x_org, y_org, x_end, y_end)
        inside = ((px[None] >= x0[:, None]) & (px[None] <= x1[:, None]) & (py[None] >= y0[:, None]) &
                  (py[None] <= y1[:, None]) & ~none[:, None])
        missed = cov & ~inside & ~large[:, None]
        assert not missed.any(), f"tile {(tx, ty)}: {int(missed.sum())} covered pixels outside the rectangle"
        declined += int(large.sum())
        total += len(large)
    return declined, total


def test_rectangle_contains_every_covered_pixel():
    rng = np.random.default_rng(12)
    for vp, tiles in [((0.0, 0.0, 64.0, 64.0), [(1, 1), (2, 1), (1, 2), (2, 2)]),
                      ((-3.0, 2.5, 75.0, 58.0), [(0, 0), (1, 1), (2, 1), (3, 2)]),
                      ((0.0, 0.0, 1024.0, 1024.0), [(31, 31), (32, 32), (30, 33)])]:
        declined, total = check(rng, vp, tiles)
        assert 0 < declined < total  # both the rectangle and the fallback are exercised


def row_spans(s, sign, err, x0, x1, y0, y1, tsx, tsy, slx):
    """NumPy float32 restatement of raster_tile.cuh row_spans for arrays of triangles (tile-local
    rectangle bounds x0..y1, tile sample positions tsx / tsy): per triangle and row (up to 8), the first
    column and the width of the row's span (0: empty)."""
    n = len(s)
    sxa, sxb, sya, syc = tsx[x0], tsx[x1], tsy[y0], tsy[y1]
    nx = (x1 - x0).astype(np.uint32)
    fnx = nx.astype(np.float32)
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        inv_dy = np.where(y1 > y0, f(1.0) / (syc - sya), f(0.0)).astype(np.float32)
        al, ga, nb = [], [], []
        for ia, ib in ((1, 2), (2, 0), (0, 1)):
            ax, ay, bx, by = s[:, ia, 0], s[:, ia, 1], s[:, ib, 0], s[:, ib, 1]
            cr = lambda px, py, qx, qy: px * qy - py * qx  # noqa: E731
            e00 = cr(ax - sxa, ay - sya, bx - sxa, by - sya)
            e10 = cr(ax - sxb, ay - sya, bx - sxb, by - sya)
            e01 = cr(ax - sxa, ay - syc, bx - sxa, by - syc)
            mag = np.abs(e00) + np.abs(e10) + np.abs(e01)
            beta = np.where(nx > 0, sign * (e10 - e00), f(0.0)).astype(np.float32)
            ga.append(np.where(y1 > y0, sign * (e01 - e00), f(0.0)).astype(np.float32))
            al.append((sign * e00 + ((f(1e-7) + f(4.0) * err) + f(4e-6) * mag)).astype(np.float32))
            nb.append(np.where(beta != 0, f(-1.0) / beta, f(0.0)).astype(np.float32))
        c0 = np.zeros((n, 8), np.int64)
        w = np.zeros((n, 8), np.int64)
        for i in range(8):
            live = i <= (y1 - y0)
            yi = np.minimum(y0 + i, len(tsy) - 1)
            v = ((tsy[yi] - sya) * inv_dy).astype(np.float32)
            lo, hi = np.zeros(n, np.float32), np.ones(n, np.float32)
            empty = np.zeros(n, bool)
            for e in range(3):
                a = (al[e] + ga[e] * v).astype(np.float32)
                t = (a * nb[e]).astype(np.float32)
                lo = np.where(nb[e] < 0, np.fmax(lo, t), lo)
                hi = np.where(nb[e] > 0, np.fmin(hi, t), hi)
                empty |= (nb[e] == 0) & (a < 0)
            ok = live & ~empty & (lo <= hi)
            cl = np.fmax(np.ceil(lo * fnx - slx), f(0.0))
            ch = np.fmin(np.floor(hi * fnx + slx), fnx)
            ok &= cl <= ch
            c0[:, i] = np.where(ok, cl, 0).astype(np.int64)
            w[:, i] = np.where(ok, ch - cl + 1, 0).astype(np.int64)
    return c0, w


def test_row_spans_contain_every_covered_pixel():
    """16x8 tiles: the row spans of each triangle's rectangle (or of the whole tile where the rectangle
    declines) hold every pixel whose sample passes the edge tests, and cut the candidates well below the
    rectangles on the same triangles."""
    rng = np.random.default_rng(13)
    TW, TH = 16, 8
    spans_total = rect_total = 0
    for vp, tiles in [((0.0, 0.0, 64.0, 64.0), [(1, 2), (2, 3), (1, 4), (2, 4)]),
                      ((-3.0, 2.5, 75.0, 58.0), [(0, 0), (1, 2), (2, 3), (3, 5)]),
                      ((0.0, 0.0, 1024.0, 1024.0), [(31, 63), (32, 64), (30, 65)])]:
        W, H = int(vp[2]), int(vp[3])
        s = triangles(rng, 400)
        lat = rng.uniform(size=s.shape[:2]) < 0.2
        k = np.round((s[..., 0] + 1) * 0.5 * vp[2] + vp[0] - 0.5)
        s[..., 0] = np.where(lat, sample_ndc(k, vp[0], vp[2]), s[..., 0])
        area = ((s[:, 1, 0] - s[:, 0, 0]) * (s[:, 2, 1] - s[:, 0, 1]) -
                (s[:, 1, 1] - s[:, 0, 1]) * (s[:, 2, 0] - s[:, 0, 0])).astype(np.float32)
        keep = ~(np.abs(area) <= f(1e-12))
        s, area = s[keep], area[keep]
        sign = np.where(area > 0, f(1.0), f(-1.0))
        slx = f(0.05) + f(1e-6) * (f(vp[2]) + abs(f(vp[0])))
        for tx, ty in tiles:
            x_org, y_org = tx * TW, ty * TH
            x_end, y_end = min(x_org + TW, W), min(y_org + TH, H)
            tsx = sample_ndc(np.arange(x_org, x_end), vp[0], vp[2])
            tsy = sample_ndc(np.arange(y_org, y_end), vp[1], vp[3])
            px, py = np.meshgrid(np.arange(x_org, x_end), np.arange(y_org, y_end))
            px, py = px.reshape(-1), py.reshape(-1)
            cov = covered(s, sign, px, py, vp)
            large, none, cx0, cx1, cy0, cy1, err = pixel_rect(s, area, vp, x_org, y_org, x_end, y_end)
            use = ~none | large
            x0 = np.where(large, 0, np.where(none, 0, cx0 - x_org)).astype(np.int64)
            x1 = np.where(large, x_end - x_org - 1, np.where(none, 0, cx1 - x_org)).astype(np.int64)
            y0 = np.where(large, 0, np.where(none, 0, cy0 - y_org)).astype(np.int64)
            y1 = np.where(large, y_end - y_org - 1, np.where(none, 0, cy1 - y_org)).astype(np.int64)
            c0, w = row_spans(s, sign, err, x0, x1, y0, y1, tsx, tsy, slx)
            row = py[None, :] - y_org - y0[:, None]
            rowc = np.clip(row, 0, 7)
            first = x_org + x0[:, None] + np.take_along_axis(c0, rowc, 1)
            width = np.take_along_axis(w, rowc, 1)
            inside = use[:, None] & (row >= 0) & (row < 8) & (px[None] >= first) & (px[None] < first + width)
            missed = cov & ~inside
            assert not missed.any(), f"tile {(tx, ty)}: {int(missed.sum())} covered pixels outside the row spans"
            spans_total += int((w * use[:, None]).sum())
            rect_total += int((((x1 - x0 + 1) * (y1 - y0 + 1)) * use).sum())
    print(f"\nrow spans: {spans_total} candidates, rectangles: {rect_total}")
    assert spans_total < 0.8 * rect_total, (spans_total, rect_total)


def subtile_rows(s, area, vp, W, H):
    """NumPy float32 restatement of bin_rect.cuh triangle_tile_rect's row range for 16x8 sub-tiles: the
    reference's 16x16 rows expanded to sub-tile rows, then (when the bound holds) cut to the pixel box
    grown by one or two pixels. Returns (ref_row0, ref_row1, row0, row1) in 8-row sub-tiles."""
    vp = [f(v) for v in vp]
    sx, sy = s[..., 0], s[..., 1]
    min_x, max_x = sx.min(1), sx.max(1)
    min_y, max_y = sy.min(1), sy.max(1)
    px0 = np.floor((min_x * f(0.5) + f(0.5)) * vp[2] + vp[0]).astype(np.int64)
    px1 = np.ceil((max_x * f(0.5) + f(0.5)) * vp[2] + vp[0]).astype(np.int64) - 1
    py0 = np.floor((min_y * f(0.5) + f(0.5)) * vp[3] + vp[1]).astype(np.int64)
    py1 = np.ceil((max_y * f(0.5) + f(0.5)) * vp[3] + vp[1]).astype(np.int64) - 1
    x0, x1 = np.clip(px0, 0, W - 1), np.clip(px1, 0, W - 1)
    y0, y1 = np.clip(py0, 0, H - 1), np.clip(py1, 0, H - 1)
    ty_last = (H + 7) // 8 - 1
    ry0, ry1 = y0 // 16 * 2, np.minimum((y1 // 16 + 1) * 2 - 1, ty_last)
    ix, iy = f(2.0) / vp[2], f(2.0) / vp[3]
    tsx_lo = ((x0 // 16 * 16).astype(np.float32) - vp[0] + f(0.5)) * ix - f(1.0) - f(1e-5)
    tsx_hi = (np.minimum(x1 // 16 * 16 + 15, W - 1).astype(np.float32) - vp[0] + f(0.5)) * ix - f(1.0) + f(1e-5)
    tsy_lo = ((y0 // 16 * 16).astype(np.float32) - vp[1] + f(0.5)) * iy - f(1.0) - f(1e-5)
    tsy_hi = (np.minimum(y1 // 16 * 16 + 15, H - 1).astype(np.float32) - vp[1] + f(0.5)) * iy - f(1.0) + f(1e-5)
    L = f(1.01) * np.fmax(np.fmax(np.abs(max_x - tsx_lo), np.abs(tsx_hi - min_x)),
                          np.fmax(np.abs(max_y - tsy_lo), np.abs(tsy_hi - min_y)))
    perim = (np.abs(sx[:, 1] - sx[:, 0]) + np.abs(sy[:, 1] - sy[:, 0]) + np.abs(sx[:, 2] - sx[:, 1]) +
             np.abs(sy[:, 2] - sy[:, 1]) + np.abs(sx[:, 0] - sx[:, 2]) + np.abs(sy[:, 0] - sy[:, 2]))
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        D = f(2.0) * (f(1e-7) + f(2e-6) * L * L) * perim / np.abs(area)
    ext = np.fmax(max_x - min_x, max_y - min_y)
    S = max(vp[2] + abs(vp[0]), vp[3] + abs(vp[1]))
    bounded = (D <= np.fmin(ix, iy)) & (np.abs(area) >= f(1e-4) * ext * ext) & (S <= f(5e5))
    m = 1 if S <= 1e5 else 2
    row0 = np.where(bounded, np.maximum(ry0, np.maximum(y0 - m, 0) // 8), ry0)
    row1 = np.where(bounded, np.minimum(ry1, np.minimum(y1 + m, H - 1) // 8), ry1)
    inside = ~((max_x < -1) | (min_x > 1) | (max_y < -1) | (min_y > 1))
    return ry0, ry1, row0, row1, x0 // 16, x1 // 16, inside


def test_subtile_binning_leaves_out_only_unreachable_subtiles():
    """16x8 binning lists a triangle in the 8-row sub-tiles of the reference's 16x16 tiles, minus those the
    pixel box grown by one pixel (two for very large viewports) does not reach when the candidate
    rectangle's bound holds over the whole reference-tile rectangle. Every sub-tile left out is checked
    by brute force: no pixel of it passes the triangle's edge tests, so the (triangle, pixel) pairs tested
    stay the reference's."""
    rng = np.random.default_rng(14)
    left_out = 0
    for vp in [(0.0, 0.0, 64.0, 64.0), (-3.0, 2.5, 75.0, 58.0), (0.0, 0.0, 1024.0, 1024.0)]:
        W, H = int(vp[2]), int(vp[3])
        s = triangles(rng, 300)
        # also triangles in random places of the image, not only around one tile
        s = np.concatenate([s, (s + rng.uniform(-0.8, 0.8, size=(len(s), 1, 2))).astype(np.float32)])
        lat = rng.uniform(size=s.shape[:2]) < 0.2
        k = np.round((s[..., 0] + 1) * 0.5 * vp[2] + vp[0] - 0.5)
        s[..., 0] = np.where(lat, sample_ndc(k, vp[0], vp[2]), s[..., 0])
        area = ((s[:, 1, 0] - s[:, 0, 0]) * (s[:, 2, 1] - s[:, 0, 1]) -
                (s[:, 1, 1] - s[:, 0, 1]) * (s[:, 2, 0] - s[:, 0, 0])).astype(np.float32)
        keep = ~(np.abs(area) <= f(1e-12))
        s, area = s[keep], area[keep]
        sign = np.where(area > 0, f(1.0), f(-1.0))
        ry0, ry1, row0, row1, tx0, tx1, inside = subtile_rows(s, area, vp, W, H)
        for i in np.nonzero(inside)[0]:
            rows = [r for r in range(int(ry0[i]), int(ry1[i]) + 1) if r < row0[i] or r > row1[i]]
            if not rows:
                continue
            px, py = np.meshgrid(np.arange(int(tx0[i]) * 16, min(int(tx1[i]) * 16 + 16, W)),
                                 np.concatenate([np.arange(r * 8, min(r * 8 + 8, H)) for r in rows]))
            cov = covered(s[i:i + 1], sign[i:i + 1], px.reshape(-1), py.reshape(-1), vp)
            assert not cov.any(), (vp, i, rows)
            left_out += len(rows)
    assert left_out > 100  # the narrowing is exercised
