"""Random, well-formed raster workloads for parity tests.

Builds planar quads in view space, projects them with a pinhole camera, derives the screen-space depth
and texture-coordinate equations the way prepare_polygon_surface does (src/square_wheel/
partial_renderer.rs:1531-1635: inverse-depth plane, tc/z planes, surface rect from the projected
vertices, equations shifted by tc_min), clips them to the frame, converts vertices to 16.16 fixed point
(draw_polygon, partial_renderer.rs:4065-4077) and applies the power-of-two z_scale of the
non-affine modes (partial_renderer.rs:4103-4109).
"""
import numpy as np

from sqwheel import abi


def clip_to_rect(pts, w, h):
    """Sutherland-Hodgman clip of a convex polygon against [0,w]x[0,h]."""
    def clip(poly, f):
        out = []
        n = len(poly)
        for i in range(n):
            a, b = poly[i - 1], poly[i]
            fa, fb = f(a), f(b)
            if fb >= 0:
                if fa < 0:
                    t = fa / (fa - fb)
                    out.append(a + (b - a) * t)
                out.append(b)
            elif fa >= 0:
                t = fa / (fa - fb)
                out.append(a + (b - a) * t)
        return out
    poly = [np.asarray(p, np.float64) for p in pts]
    for f in (lambda p: p[0], lambda p: w - p[0], lambda p: p[1], lambda p: h - p[1]):
        poly = clip(poly, f)
        if len(poly) < 3:
            return []
    return poly


def make_raster_scene(seed, width, height, num_quads, modes=(0, 1, 2), blends=(0,), pixel_format=abi.SW_PIXEL_C32,
                      texel_density=1.0, max_texture_side=256):
    """Returns (arena, draws, vertices): a random surface arena with one surface per quad, and draws."""
    rng = np.random.default_rng(seed)
    f = 0.5 * width / np.tan(np.pi * 0.375 * 0.5)
    cx, cy = width * 0.5, height * 0.5
    draws = []
    verts = []
    surfaces = []
    offset = 0
    tries = 0
    while len(draws) < num_quads and tries < num_quads * 20:
        tries += 1
        z0 = rng.uniform(40, 1500)
        center = np.array([rng.uniform(-1, 1) * z0 * cx / f, rng.uniform(-1, 1) * z0 * cy / f, z0])
        q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        n = q[2]
        if n @ center > 0:
            n = -n  # face the camera
        u_axis, v_axis = q[0], q[1]
        half = rng.uniform(5, 400, 2)
        corners = [center + u_axis * su * half[0] + v_axis * sv * half[1] for su, sv in ((-1, -1), (1, -1), (1, 1), (-1, 1))]
        if min(c[2] for c in corners) < 1.0:
            continue
        proj = [np.array([f * c[0] / c[2] + cx, f * c[1] / c[2] + cy]) for c in corners]
        poly = clip_to_rect(proj, width, height)
        if len(poly) < 3:
            continue
        # Clockwise on screen (y down): positive signed area with this formula.
        area = sum(poly[i - 1][0] * poly[i][1] - poly[i][0] * poly[i - 1][1] for i in range(len(poly)))
        if area < 0:
            poly = poly[::-1]
        if abs(area) < 1.0:
            continue
        d = float(n @ center)
        # 1/z = (n . q)/d with q = ((x-cx)/f, (y-cy)/f, 1)
        dz = np.array([n[0] / (f * d), n[1] / (f * d), (n[2] - n[0] * cx / f - n[1] * cy / f) / d])
        # tc = a . p + b per axis, density texels per unit, random shift
        tcs = []
        for axis in (u_axis, v_axis):
            a = axis * texel_density
            b = rng.uniform(-300, 300)
            tcs.append((a, b))
        # tc/z = a.q + b*(1/z)
        te = np.zeros(6)
        for i, (a, b) in enumerate(tcs):
            te[i] = a[0] / f + b * dz[0]
            te[2 + i] = a[1] / f + b * dz[1]
            te[4 + i] = (a[2] - a[0] * cx / f - a[1] * cy / f) + b * dz[2]
        # surface rect from the clipped vertices
        tcv = []
        for p in poly:
            inv_z = dz[0] * p[0] + dz[1] * p[1] + dz[2]
            tcv.append([(te[i] * p[0] + te[2 + i] * p[1] + te[4 + i]) / inv_z for i in range(2)])
        tcv = np.array(tcv)
        tmin = np.floor(tcv.min(axis=0) + 1.0 / 32)
        tmax = np.ceil(tcv.max(axis=0) - 1.0 / 32)
        size = np.maximum(tmax - tmin, 1).astype(np.int64)
        if size.max() > max_texture_side:
            continue
        for i in range(2):
            te[i] -= tmin[i] * dz[0]
            te[2 + i] -= tmin[i] * dz[1]
            te[4 + i] -= tmin[i] * dz[2]
        dz32 = dz.astype(np.float32)
        te32 = te.astype(np.float32)
        mode = int(rng.choice(modes))
        if mode != abi.SW_RASTER_AFFINE:
            max_inv_z = max(float(dz32[0] * p[0] + dz32[1] * p[1] + dz32[2]) for p in poly)
            z_scale = np.float32(2.0) ** np.float32(-5.0 - np.ceil(np.log2(max(max_inv_z, 2.0 ** -20))))
            dz32 = (dz32 * z_scale).astype(np.float32)
            te32 = (te32 * z_scale).astype(np.float32)
        first = len(verts)
        for p in poly:
            verts.append((int(np.trunc(np.float32(p[0]) * np.float32(65536.0))),
                          int(np.trunc(np.float32(p[1]) * np.float32(65536.0)))))
        dc = np.zeros((), abi.DRAW_CMD)
        dc["first_vertex"] = first
        dc["vertex_count"] = len(poly)
        dc["mode"] = mode
        dc["blend"] = int(rng.choice(blends))
        dc["depth_eq"] = dz32
        dc["tc_eq"] = te32
        dc["tex_size"] = size.astype(np.uint32)
        dc["tex_offset"] = offset
        draws.append(dc)
        surfaces.append((offset, size))
        offset += int(size[0] * size[1])
    dt = np.uint64 if pixel_format == abi.SW_PIXEL_C64 else np.uint32
    if pixel_format == abi.SW_PIXEL_C64:
        arena = rng.integers(0, 1 << 62, offset, dtype=np.uint64)
    else:
        arena = rng.integers(0, 1 << 32, offset, dtype=np.uint64).astype(np.uint32)
    draws = np.array(draws, dtype=abi.DRAW_CMD) if draws else np.zeros(0, abi.DRAW_CMD)
    vertices = np.array(verts, dtype=abi.VERTEX16) if verts else np.zeros(0, abi.VERTEX16)
    return arena.astype(dt), draws, vertices


def make_triangle_draws(seed, width, height, num_triangles, lite_offset=0, blends=(0, 1, 2, 3, 4), max_texture_side=64,
                        degenerate_frac=0.1):
    """Random triangle draws (SW_RASTER_TRIANGLE) the way decals, sprites and models emit them
    (f32_to_fixed16 positions, texture coordinates inside [1/32, size - 1/32], per-vertex light in 16.16,
    partial_renderer.rs:3028-3067): positions partly outside the frame, some thin or degenerate
    triangles, random Color32 textures with random alpha appended after lite_offset texels.
    Returns (lite_pixels, draws, tri_vertices)."""
    rng = np.random.default_rng(seed)
    lite = []
    draws = np.zeros(num_triangles, abi.DRAW_CMD)
    tv = np.zeros(num_triangles * 3, abi.TRI_VERTEX)
    offset = lite_offset
    for t in range(num_triangles):
        tw, th = (int(2 ** rng.integers(2, int(np.log2(max_texture_side)) + 1)) for _ in range(2))
        tex = rng.integers(0, 1 << 32, tw * th, dtype=np.uint64).astype(np.uint32)
        lite.append(tex)
        c = rng.uniform([-0.2 * width, -0.2 * height], [1.2 * width, 1.2 * height])
        r = rng.uniform(1, 0.4 * max(width, height))
        pts = c + rng.uniform(-r, r, (3, 2))
        if rng.random() < degenerate_frac:
            kind = rng.integers(3)
            if kind == 0:
                pts[1] = pts[0]  # two equal vertices
            elif kind == 1:
                pts[:, 1] = pts[0, 1]  # zero height
            else:
                pts[2] = pts[0] + (pts[1] - pts[0]) * rng.uniform(0, 1)  # collinear
        for k in range(3):
            v = tv[3 * t + k]
            v["x"] = int(np.trunc(np.float32(pts[k, 0]) * np.float32(65536.0)))
            v["y"] = int(np.trunc(np.float32(pts[k, 1]) * np.float32(65536.0)))
            tcf = rng.uniform([1.0 / 32, 1.0 / 32], [tw - 1.0 / 32, th - 1.0 / 32]).astype(np.float32)
            v["tc"] = (np.trunc(tcf * np.float32(65536.0))).astype(np.int32)
            light = rng.uniform(0.0, 3.0, 3).astype(np.float32)
            if rng.random() < 0.1:
                light[rng.integers(3)] = 0.0
            v["light"] = (np.trunc(light * np.float32(65536.0))).astype(np.int32)
        d = draws[t]
        d["first_vertex"] = 3 * t
        d["vertex_count"] = 3
        d["mode"] = abi.SW_RASTER_TRIANGLE
        d["blend"] = int(rng.choice(blends))
        d["tex_size"] = (tw, th)
        d["tex_source"] = abi.SW_TEXSRC_LITE
        d["tex_offset"] = offset
        offset += tw * th
    pixels = np.concatenate(lite) if lite else np.zeros(0, np.uint32)
    return pixels, draws, tv


def interleave(poly_draws, tri_draws, seed):
    """Polygon and triangle draws merged in a random order that keeps each list's own order (painter's
    order is observable through the blends)."""
    rng = np.random.default_rng(seed)
    out = np.zeros(poly_draws.size + tri_draws.size, abi.DRAW_CMD)
    take_tri = np.zeros(out.size, bool)
    take_tri[rng.choice(out.size, tri_draws.size, replace=False)] = True
    out[take_tri] = tri_draws
    out[~take_tri] = poly_draws
    return out


def make_small_draws(seed, width, height, n, modes=(0, 1, 2), blends=(0, 1, 2, 3, 4), pixel_format=abi.SW_PIXEL_C32,
                     max_radius=20.0):
    """Returns (arena, draws, vertices): n small convex polygons (3..6 vertices, radius 2..max_radius px)
    inside the frame, each textured by its own surface at constant depth (texture coordinates one texel
    per pixel from the polygon's corner, inside the surface), any mode and blend. Vectorised."""
    rng = np.random.default_rng(seed)
    r = rng.uniform(2.0, max_radius, n)
    cx = rng.uniform(r + 1, width - r - 1)
    cy = rng.uniform(r + 1, height - r - 1)
    k = rng.integers(3, 7, n)
    phase = rng.uniform(0, 2 * np.pi, n)
    draws = np.zeros(n, abi.DRAW_CMD)
    verts = []
    offset = 0
    inv_z = np.float32(1.0 / 64.0)
    sizes = np.ceil(2 * r).astype(np.int64) + 3
    for i in range(n):
        ang = phase[i] + 2 * np.pi * np.arange(k[i]) / k[i]
        px = (cx[i] + r[i] * np.cos(ang)).astype(np.float32)
        py = (cy[i] + r[i] * np.sin(ang)).astype(np.float32)
        area = float(np.sum(np.roll(px, 1) * py - px * np.roll(py, 1)))
        if area < 0:
            px, py = px[::-1], py[::-1]
        first = len(verts)
        verts.extend(zip(np.trunc(px * np.float32(65536.0)).astype(np.int64).tolist(),
                         np.trunc(py * np.float32(65536.0)).astype(np.int64).tolist()))
        x0, y0 = np.float32(cx[i] - r[i] - 1), np.float32(cy[i] - r[i] - 1)
        d = draws[i]
        d["first_vertex"], d["vertex_count"] = first, k[i]
        d["mode"], d["blend"] = int(rng.choice(modes)), int(rng.choice(blends))
        d["depth_eq"] = (0.0, 0.0, inv_z)
        # tc / z = (p - p0) / 64: tc = x - x0 and y - y0 (1..2r+2, inside the size 2r+3 surface)
        d["tc_eq"] = (inv_z, 0.0, 0.0, inv_z, -x0 * inv_z, -y0 * inv_z)
        d["tex_size"] = (sizes[i], sizes[i])
        d["tex_offset"] = offset
        offset += int(sizes[i] * sizes[i])
    dt = np.uint64 if pixel_format == abi.SW_PIXEL_C64 else np.uint32
    if pixel_format == abi.SW_PIXEL_C64:
        arena = rng.integers(0, 1 << 62, offset, dtype=np.uint64)
    else:
        arena = rng.integers(0, 1 << 32, offset, dtype=np.uint64).astype(np.uint32)
    return arena.astype(dt), draws, np.array(verts, dtype=abi.VERTEX16)
