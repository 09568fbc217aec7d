"""Portals on the CPU (prepare_view_portals_textures / build_view_portals_textures / draw_view_portal,
partial_renderer.rs:1834-2283, 3720-3772): the host's nested views are well formed (targets inside the
arena and apart from the surfaces and from each other, draws in their ranges, a view only sampling the
targets of views rendered before it, the portal draws sampling their view's texture), the depth limit
leaves views without draws, and the oracle's texture mix matches a numpy restatement of
mix_surface_with_texture (surfaces.rs:903-971) for every blending mode."""
import numpy as np
import pytest

import oracle
from sqwheel import abi, host

pytestmark = pytest.mark.usefixtures("built_libs")

PORTAL_MAP = dict(host.SMALL_MAP, num_portals=3, portals_depth=2, num_dynamic_lights=3, shadowed_lights=1)
FRAMES = list(range(28, 64, 2))


@pytest.fixture(scope="module")
def portal_scene():
    s = host.Scene(**PORTAL_MAP)
    yield s
    s.close()


def surface_ranges(surfaces):
    return [(int(d["out_offset"]), int(d["out_offset"]) + int(d["size"][0]) * int(d["size"][1])) for d in surfaces]


def test_views_well_formed(portal_scene):
    fr = host.Frame(portal_scene)
    opts = host.frame_options(640, 360, abi.SW_PIXEL_C32, directional=False)
    seen_views = seen_nested = 0
    for fi in FRAMES:
        fr.prepare(fi, opts)
        views, draws = fr.views, fr.draws
        seen_views += len(views)
        total = fr.total_texels
        assert fr.surface_texels <= total
        targets = [(int(v["target_offset"]), int(v["target_offset"]) + int(v["width"]) * int(v["height"])) for v in views]
        surf = surface_ranges(fr.surfaces)
        for i, (a, b) in enumerate(targets):
            assert fr.surface_texels <= a < b <= total
            assert all(b2 <= a or b <= a2 for a2, b2 in surf), "a view target overlaps a surface"
            assert all(b2 <= a or b <= a2 for j, (a2, b2) in enumerate(targets) if j != i), "two view targets overlap"
        assert fr.main_draws <= draws.size
        covered = np.zeros(draws.size, np.int32)
        for i, v in enumerate(views):
            first, n = int(v["first_draw"]), int(v["num_draws"])
            assert fr.main_draws <= first and first + n <= draws.size
            covered[first:first + n] += 1
            for d in draws[first:first + n]:
                if int(d["tex_source"]) != abi.SW_TEXSRC_SURFACE:
                    continue
                a = int(d["tex_offset"])
                b = a + int(d["tex_size"][0]) * int(d["tex_size"][1])
                for j, (ta, tb) in enumerate(targets):
                    if not (tb <= a or b <= ta):
                        assert j < i, "a view samples a target not rendered yet"
                        assert (a, b) == (ta, tb), "a portal draw samples part of a view"
                        seen_nested += 1
        assert (covered[fr.main_draws:] == 1).all(), "every nested draw belongs to exactly one view"
        # the frame's own portal draws sample whole view targets
        for d in draws[:fr.main_draws]:
            a = int(d["tex_offset"])
            if int(d["tex_source"]) == abi.SW_TEXSRC_SURFACE and a >= fr.surface_texels:
                assert (a, a + int(d["tex_size"][0]) * int(d["tex_size"][1])) in targets
        # light indices of every surface inside the combined light list, shadow descriptors parallel
        assert fr.light_shadows.size == fr.lights.size
        for d in fr.surfaces:
            assert (d["lights"][:int(d["num_lights"])] < fr.lights.size).all()
    assert seen_views > 0


def test_depth_limit_views_have_no_draws():
    s = host.Scene(**dict(PORTAL_MAP, portals_depth=0))
    fr = host.Frame(s)
    opts = host.frame_options(640, 360, abi.SW_PIXEL_C32, directional=False)
    seen = 0
    for fi in FRAMES:
        fr.prepare(fi, opts)
        seen += len(fr.views)
        assert (fr.views["num_draws"] == 0).all() and fr.main_draws == fr.draws.size
    assert seen > 0
    s.close()


def np_mix(region, v, lite, c64):
    """mix_surface_with_texture_impl over a region (h, w) in numpy."""
    h, w = region.shape
    sw, sh = int(v["mix_size"][0]), int(v["mix_size"][1])
    tex = lite[int(v["mix_offset"]):int(v["mix_offset"]) + sw * sh].reshape(sh, sw).astype(np.int64)
    ys = (int(v["mix_tc_min"][1]) + np.arange(h)) % sh
    xs = (int(v["mix_tc_min"][0]) + np.arange(w)) % sw
    t = tex[ys][:, xs]
    bits = 16 if c64 else 8
    lanes = lambda c, b: np.stack([(c >> (b * i)) & ((1 << b) - 1) for i in range(4)], -1).astype(np.int64)
    light = np.array([int(np.float32(v["mix_light"][2]) * np.float32(256)), int(np.float32(v["mix_light"][1]) * np.float32(256)),
                      int(np.float32(v["mix_light"][0]) * np.float32(256)), 0], np.int64)
    m = (lanes(t, 8) * light) >> 8
    d = lanes(region.astype(np.int64), bits)
    blend = int(v["mix_blend"])
    if blend == abi.SW_BLEND_NONE:
        out = m
    elif blend == abi.SW_BLEND_AVERAGE:
        out = (m + d) >> 1
    elif blend == abi.SW_BLEND_ADDITIVE:
        out = m + d
    elif blend == abi.SW_BLEND_ALPHA_TEST:
        out = np.where(((t & 0xFF000000) > 0x7F000000)[..., None], m, d)
    else:
        a = (t >> 24)[..., None]
        out = (m * a + d * (255 - a)) >> 8
    hi = (1 << bits) - 1
    out = np.where(out < 0, 1 << 40, out)  # (v as u32).min(max)
    out = np.minimum(out, hi)
    return sum(out[..., i].astype(np.uint64) << np.uint64(bits * i) for i in range(4)).astype(region.dtype)


@pytest.mark.parametrize("c64", [False, True])
def test_oracle_mix_against_numpy(c64):
    rng = np.random.default_rng(5)
    lite = rng.integers(0, 1 << 32, 64 * 32 + 100, dtype=np.uint64).astype(np.uint32)
    dt = np.uint64 if c64 else np.uint32
    for blend in range(5):
        for light in ([1.0, 1.0, 1.0], [0.5, 2.0, 0.0], [3.5, 0.25, 1.5]):
            v = np.zeros(1, abi.VIEW)
            v["width"], v["height"] = 37, 23
            v["mix_blend"], v["mix_offset"], v["mix_size"] = blend, 100, [64, 32]
            v["mix_tc_min"], v["mix_light"] = [int(rng.integers(-200, 200)), int(rng.integers(-200, 200))], light
            if c64:
                region = rng.integers(0, 1 << 62, (23, 37), dtype=np.uint64) & np.uint64(0x00FF00FF00FF00FF)
            else:
                region = rng.integers(0, 1 << 32, (23, 37), dtype=np.uint64).astype(np.uint32)
            region = region.astype(dt)
            want = np_mix(region.copy(), v[0], lite, c64)
            got = region.copy()
            assert oracle.load().orc_mix_view(abi.ptr(v), abi.ptr(got), abi.SW_PIXEL_C64 if c64 else abi.SW_PIXEL_C32,
                                              abi.ptr(lite), lite.size) == 0
            assert np.array_equal(got, want), (blend, light)
