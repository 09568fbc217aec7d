"""CPU tests of the skybox (draw_skybox, src/square_wheel/partial_renderer.rs:2311-2448): the side textures
and their mips as the reference builds them (make_skybox_side_texture{,64}, make_skybox_side_texture_mips,
src/square_wheel/textures.rs:183-290), the host's skybox draws, and whole frames with a sky rendered by the
oracle."""
import numpy as np
import pytest

import oracle
from sqwheel import abi, host


def _lanes(a, bits):
    m = (1 << bits) - 1
    return np.stack([(a.astype(np.uint64) >> np.uint64(bits * i)) & np.uint64(m) for i in range(4)], -1).astype(np.int64)


@pytest.fixture(scope="module")
def sky_scene(built_libs):
    return host.Scene(**host.SKY_MAP)


def test_skybox_textures_and_mips(sky_scene):
    t32, t64, offs, sizes = sky_scene.skybox()
    assert t32.size == t64.size > 0
    n = host.SKY_MAP["skybox_size"]
    assert sizes.tolist() == [[n >> m for m in range(5)]] * 6
    for side in range(6):
        for m in range(5):
            a = slice(int(offs[side, m]), int(offs[side, m]) + int(sizes[side, m]) ** 2)
            l32, l64 = _lanes(t32[a], 8), _lanes(t64[a], 16)
            assert (l32[:, 3] == 0).all() and (l64[:, 3] == 0).all()  # brightness vector (b, b, b, 0)
            if m == 0:
                # both formats scale the same 8-bit image; Color32 saturates at 255 (into_color32)
                assert np.array_equal(l32, np.minimum(l64, 255))
                assert l64.max() > 255  # brightness 2 gives HDR values in Color64
            else:
                s = int(sizes[side, m - 1])
                p = slice(int(offs[side, m - 1]), int(offs[side, m - 1]) + s * s)
                for lanes, bits, tex in ((l32, 8, t32), (l64, 16, t64)):
                    prev = _lanes(tex[p], bits).reshape(s, s, 4)
                    # shift_right::<2>(add(add(p00, p01), add(p10, p11))), textures.rs:269-278
                    want = ((prev[0::2, 0::2] + prev[1::2, 0::2]) + (prev[0::2, 1::2] + prev[1::2, 1::2])) >> 2
                    assert np.array_equal(lanes.reshape(s // 2, s // 2, 4), want), (side, m, bits)


def test_skybox_draws(sky_scene):
    _, _, offs, sizes = sky_scene.skybox()
    fr = host.Frame(sky_scene)
    seen = 0
    for fi in (0, 9, 30, 63):
        fr.prepare(fi, host.frame_options(640, 480, abi.SW_PIXEL_C32, directional=False))
        k = fr.skybox_draws
        seen += k
        d = fr.draws
        # the skybox is drawn first (perform_rasterization_for_viewport_part, :1285-1325), opaque
        assert (d["tex_source"][:k] == abi.SW_TEXSRC_SKYBOX).all()
        assert (d["tex_source"][k:] == abi.SW_TEXSRC_SURFACE).all()
        assert (d["blend"][:k] == abi.SW_BLEND_NONE).all()
        for cmd in d[:k]:
            side, mip = np.argwhere(offs == cmd["tex_offset"])[0]
            assert cmd["tex_size"].tolist() == [sizes[side, mip]] * 2
        # sky polygons are not surfaces: no surface uses the sky material's (stub) texture mips
        sky_material = sky_scene.info().materials - 1
        assert not np.isin(fr.surfaces["texture_mip"] // 5, [sky_material]).any()
    assert seen > 0


def test_scene_without_sky_is_unchanged(built_libs):
    """The sky options draw from their own generators: with sky_rooms = 0 the scene is the plain one."""
    a = host.Scene(**host.SMALL_MAP)
    b = host.Scene(**dict(host.SMALL_MAP, skybox_size=64, skybox_brightness=3.0))
    fa, fb = host.Frame(a), host.Frame(b)
    for fi in (0, 40):
        o = host.frame_options(320, 240, abi.SW_PIXEL_C32, directional=False)
        fa.prepare(fi, o)
        fb.prepare(fi, o)
        assert fa.skybox_draws == fb.skybox_draws == 0
        assert np.array_equal(fa.draws, fb.draws) and np.array_equal(fa.surfaces, fb.surfaces)
    assert b.skybox()[0].size == 0


def test_missing_side_is_skipped(built_libs):
    sc = host.Scene(**dict(host.SKY_MAP, skybox_missing_side=5))  # +Z (the sky's top) has no texture
    _, _, offs, sizes = sc.skybox()
    assert (sizes[5] == 0).all() and (sizes[:5] > 0).all()
    fr = host.Frame(sc)
    for fi in range(0, 64, 7):
        fr.prepare(fi, host.frame_options(320, 240, abi.SW_PIXEL_C32, directional=False))
        for cmd in fr.draws[:fr.skybox_draws]:
            assert cmd["tex_offset"] in offs[:5]


@pytest.mark.parametrize("fmt", [abi.SW_PIXEL_C32, abi.SW_PIXEL_C64])
def test_sky_frame_oracle(sky_scene, fmt):
    """A frame with a sky through the oracle: no fetch outside a texture, the open ceiling filled by sky
    texels, and split_rect rasterisation covering the same pixels as the single-rect one."""
    t32, t64, _, _ = sky_scene.skybox()
    st = sky_scene.static_data()
    fr = host.Frame(sky_scene).prepare(5, host.frame_options(320, 240, fmt, directional=False))
    assert fr.skybox_draws > 0
    arena = oracle.build_surfaces(st, fr.surfaces, fr.lights, fr.params, fr.total_texels, num_threads=4)
    sky = t64 if fmt == abi.SW_PIXEL_C64 else t32
    dt = np.uint64 if fmt == abi.SW_PIXEL_C64 else np.uint32
    marker = dt(0xFFFFFFFFFFFF) if fmt == abi.SW_PIXEL_C64 else dt(0xFFFFFFFF)
    a = np.full((240, 320), marker, dt)
    b = a.copy()
    assert oracle.rasterize(fr.draws, fr.vertices, arena, fr.params, a, num_threads=1, skybox=sky) == 0
    assert oracle.rasterize(fr.draws, fr.vertices, arena, fr.params, b, num_threads=4, skybox=sky) == 0
    assert np.array_equal(a == marker, b == marker)
    # Without the skybox draws the open ceiling stays empty; with them only the few crack pixels of the
    # synthetic geometry's T-junctions (present in frames without sky too) remain uncovered.
    c = np.full((240, 320), marker, dt)
    oracle.rasterize(fr.draws[fr.skybox_draws:], fr.vertices, arena, fr.params, c, skybox=sky)
    assert (c == marker).mean() > 0.05
    assert (a == marker).mean() < 1e-3
    assert np.isin(a[c == marker], sky).mean() > 0.99
    with pytest.raises(RuntimeError):  # skybox draws need the skybox texels
        oracle.rasterize(fr.draws, fr.vertices, arena, fr.params, a)
