"""The oracle's triangle rasteriser (Rasterizer::fill_triangle, rasterizer.rs:731-1292) against a second,
independent restatement written here in plain Python integers, on small frames: every pixel's coverage,
texture coordinates, light and blend. No GPU."""
import numpy as np
import pytest

import oracle
import scenes
from sqwheel import abi, gpu

MASK32 = 0xFFFFFFFF


def i32(x):
    x &= MASK32
    return x - (1 << 32) if x >> 31 else x


def fmul(a, b):  # fixed16_mul: (i64 a * i64 b) >> 16 as i32
    return i32((a * b) >> 16)


def fdiv(a, b):  # fixed16_div: ((i64 a) << 16) / i64 b, truncating toward zero, as i32
    n = a << 16
    q = abs(n) // abs(b)
    return i32(q if (n >= 0) == (b > 0) else -q)


HALF, ONE = 1 << 15, 1 << 16


def c32_lanes(c):
    return [(c >> (8 * i)) & 255 for i in range(4)]


def to_pixel(lanes, fmt):
    if fmt == abi.SW_PIXEL_C64:
        return sum(min(v & MASK32, 65535) << (16 * i) for i, v in enumerate(lanes))
    return sum(min(v & MASK32, 255) << (8 * i) for i, v in enumerate(lanes))


def from_pixel(p, fmt):
    if fmt == abi.SW_PIXEL_C64:
        return [(p >> (16 * i)) & 0xFFFF for i in range(4)]
    return [(p >> (8 * i)) & 0xFF for i in range(4)]


def blend(dst, lit, texel, mode, fmt):
    bits, mx = (16, 0xFFFF) if fmt == abi.SW_PIXEL_C64 else (8, 0xFF)
    src = to_pixel(lit, fmt)
    if mode == abi.SW_BLEND_NONE:
        return src
    if mode == abi.SW_BLEND_AVERAGE:
        a, b = from_pixel(dst, fmt), from_pixel(src, fmt)
        return sum(((x + y) >> 1) << (bits * i) for i, (x, y) in enumerate(zip(a, b)))  # (a ^ b) >> 1 + (a & b)
    if mode == abi.SW_BLEND_ADDITIVE:
        a, b = from_pixel(dst, fmt), from_pixel(src, fmt)
        return sum(min(x + y, mx) << (bits * i) for i, (x, y) in enumerate(zip(a, b)))
    if mode == abi.SW_BLEND_ALPHA_TEST:
        return src if (texel >> 24) > 0x7F else dst
    alpha = texel >> 24
    d = from_pixel(dst, fmt)
    return to_pixel([i32(i32(d[i] * (255 - alpha)) + i32(lit[i] * alpha)) >> 8 for i in range(4)], fmt)


def fill_triangle(fb, fmt, vs, tex, tw, th, mode):
    w, h = fb.shape[1], fb.shape[0]
    ys = [v["y"] for v in vs]
    if ys[0] >= ys[1] and ys[0] >= ys[2]:
        up, lo = 0, (1 if ys[1] < ys[2] else 2)
    elif ys[1] >= ys[0] and ys[1] >= ys[2]:
        up, lo = 1, (0 if ys[0] < ys[2] else 2)
    else:
        up, lo = 2, (0 if ys[0] < ys[1] else 1)
    U, L, M = ([int(vs[k]["x"]), int(vs[k]["y"]), [int(t) for t in vs[k]["tc"]], [int(t) for t in vs[k]["light"]]]
               for k in (up, lo, 3 - up - lo))
    long_dy = max(i32(U[1] - L[1]), HALF)
    lower_dy = max(i32(M[1] - L[1]), HALF)
    upper_dy = max(i32(U[1] - M[1]), HALF)
    long_dx = fdiv(i32(U[0] - L[0]), long_dy)
    long_x_mid = i32(L[0] + fmul(long_dx, i32(M[1] - L[1])))
    lower_dx = fdiv(i32(M[0] - L[0]), lower_dy)
    upper_dx = fdiv(i32(U[0] - M[0]), upper_dy)

    def slopes(a, b, c, n):
        ld = [fdiv(i32(a[i] - b[i]), long_dy) for i in range(n)]
        lm = [i32(b[i] + fmul(ld[i], lower_dy)) for i in range(n)]
        dl = [fdiv(i32(c[i] - b[i]), lower_dy) for i in range(n)]
        du = [fdiv(i32(a[i] - c[i]), upper_dy) for i in range(n)]
        return ld, lm, dl, du

    ltc, ltcm, dtcl, dtcu = slopes(U[2], L[2], M[2], 2)
    lli, llim, dlil, dliu = slopes(U[3], L[3], M[3], 3)
    if long_x_mid >= M[0]:
        mdx = max(i32(long_x_mid - M[0]), HALF)
        dtx = [fdiv(i32(ltcm[i] - M[2][i]), mdx) for i in range(2)]
        dlx = [fdiv(i32(llim[i] - M[3][i]), mdx) for i in range(3)]
        parts = [(L[1], M[1], (L[0], lower_dx), (L[0], long_dx), L[2], dtcl, L[3], dlil),
                 (M[1], U[1], (M[0], upper_dx), (long_x_mid, long_dx), M[2], dtcu, M[3], dliu)]
    else:
        mdx = max(i32(M[0] - long_x_mid), HALF)
        dtx = [fdiv(i32(M[2][i] - ltcm[i]), mdx) for i in range(2)]
        dlx = [fdiv(i32(M[3][i] - llim[i]), mdx) for i in range(3)]
        parts = [(L[1], M[1], (L[0], long_dx), (L[0], lower_dx), L[2], ltc, L[3], lli),
                 (M[1], U[1], (long_x_mid, long_dx), (M[0], upper_dx), ltcm, ltc, llim, lli)]
    for y0, y1, ls, rs, tcs, dtcy, lis, dliy in parts:
        part(fb, fmt, y0, y1, ls, rs, tcs, list(dtcy), list(dtx), lis, list(dliy), list(dlx), tex, tw, th, mode, w, h)


def part(fb, fmt, y_start, y_end, ls, rs, tc_start, dtcy, dtx, li_start, dliy, dlx, tex, tw, th, mode, w, h):
    ys_int = max(i32(y_start + HALF) >> 16, 0)
    ye_int = min(i32(y_end + HALF) >> 16, h)
    if ys_int >= ye_int:
        return
    ysd = i32(i32((ys_int << 16) + HALF) - y_start)
    xl = i32(ls[0] + fmul(ysd, ls[1]) + HALF)
    xr = i32(rs[0] + fmul(ysd, rs[1]) + HALF)
    yed = i32(y_end - i32(y_start + ysd))
    dxl = max(i32(xr - xl), 0)
    dxu = max(i32(i32(xr + fmul(yed, rs[1])) - i32(xl + fmul(yed, ls[1]))), 0)
    tcl = [0, 0]
    for i, size in enumerate((tw, th)):
        mt = i32((size << 16) - 1)
        tcl[i] = min(max(i32(tc_start[i] + fmul(ysd, dtcy[i])), 0), mt)
        d = fmul(dtx[i], dxl)
        if d > mt:
            tcl[i], dtx[i] = 0, fdiv(mt, dxl)
        elif d < -mt:
            tcl[i], dtx[i] = mt, fdiv(-mt, dxl)
        else:
            r = i32(tcl[i] + d)
            if r > mt:
                tcl[i] = i32(tcl[i] - i32(r - mt))
            elif r < 0:
                tcl[i] = i32(tcl[i] - r)
        tul = min(max(i32(tcl[i] + fmul(yed, dtcy[i])), 0), mt)
        d = fmul(dtx[i], dxu)
        if d > mt:
            tul, dtx[i] = 0, fdiv(mt, dxu)
        elif d < -mt:
            tul, dtx[i] = mt, fdiv(-mt, dxu)
        else:
            r = i32(tul + d)
            if r > mt:
                tul = i32(tul - i32(r - mt))
            elif r < 0:
                tul = i32(tul - r)
        dtcy[i] = fdiv(i32(tul - tcl[i]), yed) if yed > 0 else 0
        tul2 = i32(tcl[i] + fmul(yed, dtcy[i]))
        r = i32(tul2 + fmul(dtx[i], dxu))
        if r < 0:
            dtx[i] = fdiv(-tul2, dxu) if dxu > 0 else 0
        elif r > mt:
            dtx[i] = fdiv(i32(mt - tul2), dxu) if dxu > 0 else 0
    lil = [0, 0, 0]
    for i in range(3):
        lil[i] = max(i32(li_start[i] + fmul(ysd, dliy[i])), 0)
        r = i32(lil[i] + fmul(dxl, dlx[i]))
        if r < 0:
            lil[i] = i32(lil[i] - r)
        lul = max(i32(lil[i] + fmul(yed, dliy[i])), 0)
        r = i32(lul + fmul(dxu, dlx[i]))
        if r < 0:
            lul = i32(lul - r)
        dliy[i] = fdiv(i32(lul - lil[i]), yed) if yed > 0 else 0
        lul2 = i32(lil[i] + fmul(yed, dliy[i]))
        if i32(lul2 + fmul(dxu, dlx[i])) < 0:
            dlx[i] = fdiv(-lul2, dxu) if dxu > 0 else 0
    for y in range(ys_int, ye_int):
        xs, xe = max(xl >> 16, 0), min(xr >> 16, w)
        if xs < xe:
            xsd = i32(i32((xs << 16) + ONE) - xl)
            tc = [i32(tcl[i] + fmul(xsd, dtx[i])) for i in range(2)]
            li = [i32(lil[i] + fmul(xsd, dlx[i])) for i in range(3)]
            for x in range(xs, xe):
                u, v = tc[0] >> 16, tc[1] >> 16
                texel = int(tex[u + v * tw])
                t = c32_lanes(texel)
                lit = [i32(t[0] * li[2]) >> 16, i32(t[1] * li[1]) >> 16, i32(t[2] * li[0]) >> 16, 0]
                fb[y, x] = blend(int(fb[y, x]), lit, texel, mode, fmt)
                tc = [i32(tc[i] + dtx[i]) for i in range(2)]
                li = [i32(li[i] + dlx[i]) for i in range(3)]
        xl, xr = i32(xl + ls[1]), i32(xr + rs[1])
        tcl = [i32(tcl[i] + dtcy[i]) for i in range(2)]
        lil = [i32(lil[i] + dliy[i]) for i in range(3)]


@pytest.mark.parametrize("fmt", [abi.SW_PIXEL_C32, abi.SW_PIXEL_C64])
def test_oracle_triangles_match_independent_restatement(built_libs, fmt):
    w, h = 48, 40
    lite, draws, tv = scenes.make_triangle_draws(11 + fmt, w, h, 40, max_texture_side=16, degenerate_frac=0.2)
    dt = np.uint64 if fmt == abi.SW_PIXEL_C64 else np.uint32
    rng = np.random.default_rng(5)
    start = rng.integers(0, 1 << 62 if fmt == abi.SW_PIXEL_C64 else 1 << 32, (h, w), dtype=np.uint64).astype(dt)
    want = start.copy()
    for d in draws:
        k = int(d["first_vertex"])
        off = int(d["tex_offset"])
        tw, th = int(d["tex_size"][0]), int(d["tex_size"][1])
        fill_triangle(want, fmt, tv[k:k + 3], lite[off:off + tw * th], tw, th, int(d["blend"]))
    got = start.copy()
    fp = gpu.frame_params(w, h, fmt, (0, 0, 0))
    assert oracle.rasterize(draws, None, None, fp, got, tri_vertices=tv, lite=lite) == 0
    assert np.array_equal(want, got), f"{(want != got).sum()} pixels differ"


def test_triangle_coverage_known_answer(built_libs):
    """A right triangle with vertices at (0,0), (8,0), (0,8): rows y in [0, 8), row y covers the pixels
    whose centres lie left of the hypotenuse x + y < 8 (x_left = 0.5 px bias included): x in [0, 8 - y)
    (rasterizer.rs:1000-1012, 1188-1196). Constant texture colour and light 1.0: the texel itself."""
    tv = np.zeros(3, abi.TRI_VERTEX)
    for k, (x, y) in enumerate(((0, 0), (8, 0), (0, 8))):
        tv[k]["x"], tv[k]["y"] = x << 16, y << 16
        tv[k]["tc"] = (1 << 15, 1 << 15)
        tv[k]["light"] = (1 << 16, 1 << 16, 1 << 16)
    d = np.zeros(1, abi.DRAW_CMD)
    d["vertex_count"], d["mode"], d["tex_size"], d["tex_source"] = 3, abi.SW_RASTER_TRIANGLE, (1, 1), abi.SW_TEXSRC_LITE
    lite = np.array([0xFF405060], np.uint32)
    fb = np.zeros((10, 10), np.uint32)
    oracle.rasterize(d, None, None, gpu.frame_params(10, 10, abi.SW_PIXEL_C32, (0, 0, 0)), fb, tri_vertices=tv, lite=lite)
    want = np.zeros((10, 10), np.uint32)
    for y in range(8):
        want[y, :8 - y] = 0x00405060  # the alpha lane is lit by 0
    assert np.array_equal(fb, want), fb
