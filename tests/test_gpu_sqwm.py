"""Compiled maps on the GPU: the compressed lightmap records decoded by sw_set_lightmaps_compressed equal
the oracle's decompression bit for bit (lightmap_compression.rs:64-68, 88-130), and frames of a map read
from a .sqwm file, whose lightmaps the renderer uploads compressed and decodes on the GPU, equal the
oracle's frames rendered from the host-decoded lightmaps."""
import numpy as np
import pytest

import oracle
from sqwheel import abi, gpu, host

pytestmark = pytest.mark.gpu


def special_records(rng, n_simple, n_dir):
    simple = rng.integers(0, 256, (n_simple, 4), dtype=np.uint8)
    simple[::9, 3] = 0     # scale 0
    simple[::13] = 255
    d = rng.integers(0, 256, (n_dir, 13), dtype=np.uint8)
    d[::5, 4:7] = 0        # zero direction: (0, 0, 1/1024)
    d[::7, 7] = 0          # zero vector scale
    d[::11, 4:7] = 0x80    # -128 components
    return simple, d


@pytest.mark.parametrize("n_simple,n_dir", [(1, 1), (255, 257), (4096, 12345), (100003, 70001)])
def test_gpu_lightmap_decode_bit_exact(gpu_ok, n_simple, n_dir):
    scene = host.Scene(**host.SMALL_MAP)
    r = gpu.GpuRenderer(scene.static_data())
    rng = np.random.default_rng(n_simple + n_dir)
    try:
        for _ in range(2):  # a second upload replaces the first in place
            simple, d = special_records(rng, n_simple, n_dir)
            r.set_lightmaps_compressed(simple, d)
            got, got_d = r.read_lightmaps(n_simple, n_dir)
            want = oracle.decompress_lightmaps(simple)
            want_d = oracle.decompress_directional_lightmaps(d)
            assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
            assert got_d.tobytes() == want_d.tobytes()
    finally:
        r.close()


def test_gpu_lightmaps_checked_against_the_map(gpu_ok):
    """Lightmaps shorter than the uploaded map's polygons read are refused and leave the old ones."""
    scene = host.Scene(**dict(host.SMALL_MAP, directional_lightmaps=1))
    glib = gpu.load_library()
    hr = host.HostRenderer(scene)
    try:
        ctx = hr.context()
        polys, verts = host.Frame(scene).map_data()
        assert glib.sw_set_map(ctx, abi.ptr(polys), polys.size, abi.ptr(verts), verts.shape[0]) == abi.SW_OK
        st = scene.static_data()
        rec = oracle.compress_lightmaps(st.lightmaps[:100])
        drec = oracle.compress_directional_lightmaps(st.directional_lightmaps[:100])
        assert glib.sw_set_lightmaps_compressed(ctx, abi.ptr(rec), 100, abi.ptr(drec), 100) == abi.SW_ERR_INVALID_ARGUMENT
        assert b"lightmaps shorter" in glib.sw_last_error(ctx)
        back = np.zeros(4, abi.DIR_LIGHTMAP_ELEMENT)
        assert glib.sw_read_lightmaps(ctx, None, 0, abi.ptr(back), 4) == abi.SW_OK
        assert back.tobytes() == st.directional_lightmaps[:4].tobytes()
    finally:
        hr.close()


@pytest.fixture(scope="module")
def map_bytes(tmp_path_factory):
    gen = host.Scene(**dict(host.SMALL_MAP, directional_lightmaps=1, num_materials=12))
    path = tmp_path_factory.mktemp("maps") / "small.sqwm"
    gen.save_map(str(path))
    gen.close()
    return path.read_bytes()


@pytest.mark.parametrize("gpu_prep,directional", [(True, True), (False, True), (True, False)])
def test_loaded_map_frames(gpu_ok, map_bytes, gpu_prep, directional):
    cfg = dict(host.SMALL_MAP, directional_lightmaps=1 if directional else 0, num_dynamic_lights=4,
               metal_frac=0.25, dielectric_frac=0.25, normal_maps=1)
    scene = host.Scene.load_map(map_bytes, **cfg)
    st = scene.static_data()
    fr = host.Frame(scene)
    hr = host.HostRenderer(scene)
    hr.set_gpu_prep(gpu_prep)
    glib = gpu.load_library()
    w, h = 640, 360
    opts = host.frame_options(w, h, abi.SW_PIXEL_C64, directional=directional, clear_background=True)
    try:
        # the renderer decoded the file's records on the GPU: the same values the host decoded
        ctx = hr.context()
        simple, d = scene.compressed_lightmaps()
        got = np.zeros((simple.shape[0], 3), np.float32)
        got_d = np.zeros(d.shape[0], abi.DIR_LIGHTMAP_ELEMENT)
        assert glib.sw_read_lightmaps(ctx, abi.ptr(got), got.shape[0], abi.ptr(got_d), got_d.size) == abi.SW_OK
        assert got.tobytes() == st.lightmaps.tobytes() and got_d.tobytes() == st.directional_lightmaps.tobytes()
        for fi in (0, 9, 30, 57):
            fr.prepare(fi, opts)
            arena = oracle.build_surfaces(st, fr.surfaces, fr.lights, fr.params, fr.total_texels, num_threads=8)
            want = np.zeros((h, w), np.uint64)
            oracle.clear_background(fr.params, want)
            assert oracle.rasterize(fr.draws, fr.vertices, arena, fr.params, want) == 0
            out = np.zeros((h, w), np.uint64)
            hr.render_frame(fi, opts, out=out)
            assert np.array_equal(want, out), f"frame {fi}: {(want != out).sum()} pixels differ"
    finally:
        hr.close()
        scene.close()
