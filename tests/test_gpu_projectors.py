"""Projector lights (ShadowMap::Projector, light.rs:53-60, 261-294) through the GPU path against the
oracle: the projector maps (drawn like a cube side with the light's matrices, then the corners outside the
inscribed circle set to 1e24, make_shadow_map_circle light.rs:135-156), surfaces lit through them
(projector_shadow_map_fetch) with light lists narrowed to the cone (polygon_is_affected_by_light,
partial_renderer.rs:3901-3944), and whole frames through both preparation paths - bit-exact."""
import numpy as np
import pytest

import oracle
from sqwheel import abi, gpu, host

pytestmark = pytest.mark.gpu

PROJ_MAP = dict(host.SMALL_MAP, num_dynamic_lights=5, shadowed_lights=1, projector_lights=3)


def oracle_storage(fr, storage):
    if storage.size < fr.shadow_texels:
        storage = np.concatenate([storage, np.zeros(fr.shadow_texels - storage.size, np.float32)])
    oracle.shadow_maps(fr.depth_draws, fr.depth_vertices, storage)
    for m in fr.light_shadows:
        if m["kind"] == abi.SW_SHADOW_PROJECTOR:
            oracle.shadow_map_circle(storage, int(m["offset"]), int(m["size"]))
    return storage


def test_projector_maps_and_surfaces(gpu_ok):
    scene = host.Scene(**PROJ_MAP)
    st = scene.static_data()
    fr = host.Frame(scene)
    r = gpu.GpuRenderer(st)
    storage = np.zeros(0, np.float32)
    projected = 0
    try:
        for fi in (0, 5, 20, 21, 33, 47, 60):
            fmt = abi.SW_PIXEL_C32 if fi == 5 else abi.SW_PIXEL_C64
            fr.prepare(fi, host.frame_options(640, 480, fmt, directional=True))
            kinds = fr.light_shadows["kind"]
            projected += int((kinds == abi.SW_SHADOW_PROJECTOR).sum())
            storage = oracle_storage(fr, storage)
            r.build_shadow_maps(fr.depth_draws, fr.depth_vertices, fr.shadow_texels)
            r.set_light_shadows(fr.light_shadows)  # applies the projector circles after the draws
            got = r.read_shadow_maps(storage.size)
            assert np.array_equal(got.view(np.uint32), storage.view(np.uint32)), \
                f"frame {fi}: {(got != storage).sum()} shadow-map texels differ"
            want = oracle.build_surfaces(st, fr.surfaces, fr.lights, fr.params, fr.total_texels, num_threads=8,
                                         shadows=fr.light_shadows, shadow_texels=storage)
            r.frame_begin(fr.params, fr.lights)
            r.submit_surfaces(fr.surfaces, fr.total_texels)
            assert np.array_equal(want, r.read_surfaces(fr.total_texels, fmt)), f"frame {fi}: surfaces differ"
        assert projected > 0
    finally:
        r.close()


@pytest.mark.parametrize("gpu_prep", [True, False])
def test_projector_frames_through_the_renderer(gpu_ok, gpu_prep):
    """render_frame with cube and projector lights: the GPU-side preparation narrows light lists with the
    projector cones exactly as the host does, and frames equal the oracle's."""
    scene = host.Scene(**PROJ_MAP)
    st = scene.static_data()
    fr = host.Frame(scene)
    hr = host.HostRenderer(scene)
    hr.set_gpu_prep(gpu_prep)
    w, h = 640, 480
    opts = host.frame_options(w, h, abi.SW_PIXEL_C64, directional=True, clear_background=True)
    storage = np.zeros(0, np.float32)
    try:
        for fi in (3, 21, 56, 60):
            fr.prepare(fi, opts)
            storage = oracle_storage(fr, storage)
            arena = oracle.build_surfaces(st, fr.surfaces, fr.lights, fr.params, fr.total_texels, num_threads=8,
                                          shadows=fr.light_shadows, shadow_texels=storage)
            want = np.zeros((h, w), np.uint64)
            oracle.clear_background(fr.params, want)
            assert oracle.rasterize(fr.draws, fr.vertices, arena, fr.params, want) == 0
            got = np.zeros((h, w), np.uint64)
            hr.render_frame(fi, opts, out=got)
            assert np.array_equal(want, got), f"frame {fi}: {(want != got).sum()} pixels differ"
            if gpu_prep:
                _, s, _, _ = hr.read_view_prep()
                assert s.tobytes() == fr.surfaces.tobytes(), f"frame {fi}: GPU light lists differ from the host's"
    finally:
        hr.close()
