"""CPU tests of the host side: scene generation, visibility, surface preparation and draw setup, and a
whole frame rendered by the oracle from the host's outputs (closed map: every pixel covered, no texel
fetch outside its surface)."""
import ctypes
import os
import re

import numpy as np
import pytest

import oracle
from sqwheel import abi, host

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def small_scene(built_libs):
    return host.Scene(**host.SMALL_MAP)


def test_host_symbols_exported(built_libs):
    text = open(os.path.join(ROOT, "include", "swhost.h")).read()
    names = sorted(set(re.findall(r"^\s*(?:int|const char\*|SwCtx\*|SwhFrame\*)\s+(swh\w*)\s*\(", text, re.M)))
    lib = ctypes.CDLL(host.HOST_LIB_PATH)
    assert [n for n in names if not hasattr(lib, n)] == []
    assert sorted(host.HOST_EXPORTED) == names


def test_scene_is_deterministic(built_libs):
    a = host.Scene(**host.SMALL_MAP).info()
    b = host.Scene(**host.SMALL_MAP).info()
    assert [getattr(a, f) for f, _ in host.SceneInfo._fields_] == [getattr(b, f) for f, _ in host.SceneInfo._fields_]
    assert 1000 <= a.polygons <= 4000  # ~2k polygons for the 8-room map
    assert a.leafs == a.nodes + 1      # full binary tree
    c = host.Scene(**dict(host.SMALL_MAP, seed=9)).info()
    assert c.polygons != a.polygons or c.lightmap_elements != a.lightmap_elements


def test_scene_rejects_bad_config(built_libs):
    with pytest.raises(Exception):
        host.Scene(**dict(host.SMALL_MAP, room_min=100.0))
    with pytest.raises(Exception):
        host.Scene(**dict(host.SMALL_MAP, tile_size=1000.0))


def test_frame_outputs_invariants(small_scene):
    fr = host.Frame(small_scene)
    for fi in (0, 17, 33, 63):
        fr.prepare(fi, host.frame_options(640, 480, abi.SW_PIXEL_C32, directional=False))
        s = fr.surfaces
        assert s.size > 0 and fr.draws.size > 0
        # Surfaces are packed back to back in allocation order (partial_renderer.rs:1617-1618).
        area = s["size"][:, 0].astype(np.int64) * s["size"][:, 1]
        assert np.array_equal(s["out_offset"], np.concatenate([[0], np.cumsum(area)[:-1]]))
        assert int(area.sum()) == fr.total_texels
        # Draws reference their surface exactly and stay inside the arena.
        ends = fr.draws["tex_offset"] + fr.draws["tex_size"][:, 0].astype(np.uint64) * fr.draws["tex_size"][:, 1]
        assert (ends <= fr.total_texels).all()
        assert set(fr.draws["tex_offset"].tolist()) <= set(s["out_offset"].tolist())
        assert (fr.draws["vertex_count"] >= 3).all() and (fr.draws["vertex_count"] <= 24).all()
        # Lightmap reads stay inside each polygon's lightmap.
        sh = s["lightmap_tc_shift"].astype(np.int64)
        lg = s["lightmap_scale_log2"].astype(np.int64)
        lu = (s["size"][:, 0] - 1 + sh[:, 0]) >> lg
        lv = (s["size"][:, 1] - 1 + sh[:, 1]) >> lg
        assert (lu + 1 < s["lightmap_size"][:, 0]).all() and (lv + 1 < s["lightmap_size"][:, 1]).all()


def test_oracle_frame_covers_every_pixel(small_scene):
    """The map is closed and the camera stays inside it: the painter's algorithm must cover the frame."""
    st = small_scene.static_data()
    fr = host.Frame(small_scene)
    fr.prepare(5, host.frame_options(320, 240, abi.SW_PIXEL_C32, directional=False))
    arena = oracle.build_surfaces(st, fr.surfaces, fr.lights, fr.params, fr.total_texels, num_threads=4)
    fb = np.zeros((240, 320), np.uint32)
    bad = oracle.rasterize(fr.draws, fr.vertices, arena, fr.params, fb)
    assert bad == 0
    assert (fb != 0).all()


def test_oracle_single_vs_split_rect(small_scene):
    """Multi-thread rasterisation clips spans per region and changes texel addresses: the single-thread
    path is the parity contract, and split_rect covers the same pixels."""
    st = small_scene.static_data()
    fr = host.Frame(small_scene)
    fr.prepare(9, host.frame_options(320, 240, abi.SW_PIXEL_C32, directional=False))
    arena = oracle.build_surfaces(st, fr.surfaces, fr.lights, fr.params, fr.total_texels, num_threads=4)
    a = np.zeros((240, 320), np.uint32)
    b = np.zeros((240, 320), np.uint32)
    oracle.rasterize(fr.draws, fr.vertices, arena, fr.params, a, num_threads=1)
    oracle.rasterize(fr.draws, fr.vertices, arena, fr.params, b, num_threads=4)
    assert (a != 0).all() and (b != 0).all()


@pytest.mark.parametrize("cfg", ["small", "sky"])
def test_prepare_view_matches_prepare(built_libs, cfg):
    """The host half of a GPU-prepared frame (prepare_view) sees the same leafs as the host preparation: every
    visible polygon lies in a view leaf, the drawn leafs are draw_tree's (a permutation 0..n-1), leaf light
    lists index the frame's lights, and the skybox draws are identical."""
    scene = host.Scene(**(host.SMALL_MAP if cfg == "small" else host.SKY_MAP))
    fr = host.Frame(scene)
    fv = host.Frame(scene)
    opts = host.frame_options(800, 600, abi.SW_PIXEL_C64, directional=True)
    for fi in (0, 5, 30, 61, 90):
        fr.prepare(fi, opts)
        fv.prepare_view(fi, opts)
        leafs = fv.view_leafs
        assert leafs.size > 0
        order = leafs["draw_order"][leafs["draw_order"] != abi.SW_LEAF_NOT_DRAWN]
        assert sorted(order.tolist()) == list(range(order.size))
        assert order.size == fr.visible_leafs
        assert int(leafs["num_polygons"].sum()) >= fr.surfaces.size
        first, num = leafs["first_light"].astype(np.int64), leafs["num_lights"].astype(np.int64)
        assert (first + num <= fv.view_leaf_lights.size).all()
        assert (fv.view_leaf_lights < fr.lights.size).all()
        n_sky = fr.skybox_draws
        assert fv.draws.size == n_sky
        assert np.array_equal(fv.draws.view(np.uint8), fr.draws[:n_sky].view(np.uint8))
        sky_vertices = int(fr.draws[:n_sky]["vertex_count"].sum())
        assert np.array_equal(fv.vertices.view(np.uint8), fr.vertices[:sky_vertices].view(np.uint8))
        if cfg == "sky" and fi == 0:
            assert n_sky > 0
