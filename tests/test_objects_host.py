"""Sprites and decals on the host (draw_sprite, partial_renderer.rs:3290-3523; draw_polygon_decals and
subdivide_and_draw_decal_triangle, :2794-3080): the fill_triangle draws they emit, checked for the
reference's invariants - decal texture coordinates inside [1/32, size - 1/32], draws reading whole lite
mips of the objects' textures, triangles inside the frame - and the oracle rasterising them in bounds."""
import numpy as np
import pytest

import oracle
from sqwheel import abi, host

pytestmark = pytest.mark.usefixtures("built_libs")


@pytest.fixture(scope="module")
def scene():
    s = host.Scene(**dict(host.SMALL_MAP, num_sprites=60, num_decals=300, num_dynamic_lights=3))
    yield s
    s.close()


def test_object_draws(scene):
    fr = host.Frame(scene)
    lite = scene.lite_textures()
    w, h = 640, 480
    opts = host.frame_options(w, h, abi.SW_PIXEL_C32, directional=False)
    total = 0
    for fi in range(0, 64, 3):
        fr.prepare(fi, opts)
        tri = fr.draws[fr.draws["mode"] == abi.SW_RASTER_TRIANGLE]
        total += tri.size
        assert (tri["tex_source"] == abi.SW_TEXSRC_LITE).all()
        assert (tri["tex_offset"] + tri["tex_size"][:, 0].astype(np.uint64) * tri["tex_size"][:, 1] <= lite.size).all()
        tv = fr.tri_vertices
        if tv.size:
            # vertices inside the viewport (clipped by the leaf bounds), texture coordinates inside the mip
            assert (tv["x"] >= -16).all() and (tv["x"] <= (w << 16) + 16).all()  # clipping rounds within 1/4096 px
            assert (tv["y"] >= -16).all() and (tv["y"] <= (h << 16) + 16).all()
            sizes = np.repeat(tri["tex_size"], 3, axis=0)
            assert (tv["tc"] >= 0).all() and (tv["tc"] <= (sizes.astype(np.int64) << 16)).all()
    assert total > 500


def test_objects_rasterise_in_bounds(scene):
    fr = host.Frame(scene).prepare(0, host.frame_options(640, 480, abi.SW_PIXEL_C64, directional=False))
    st = scene.static_data()
    arena = oracle.build_surfaces(st, fr.surfaces, fr.lights, fr.params, fr.total_texels, num_threads=4)
    img = np.zeros((480, 640), np.uint64)
    assert oracle.rasterize(fr.draws, fr.vertices, arena, fr.params, img, tri_vertices=fr.tri_vertices,
                            lite=scene.lite_textures()) == 0
    assert fr.model_triangles > 0
