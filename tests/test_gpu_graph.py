"""The whole frame as one CUDA graph (sw_draw_frame) and the launch configurations (sw_set_tuning,
sw_autotune): every path gives the oracle's frame bit for bit, including the exposure sequence."""
import numpy as np
import pytest

import oracle
from sqwheel import abi, gpu, host

pytestmark = pytest.mark.gpu


def _prepare(scene, frames, w, h, fmt, directional):
    fr = host.Frame(scene)
    out = []
    for fi in frames:
        fr.prepare(fi, host.frame_options(w, h, fmt, directional=directional))
        out.append(dict(surfaces=fr.surfaces, draws=fr.draws, vertices=fr.vertices, lights=fr.lights,
                        params=fr.params, total_texels=fr.total_texels))
    return out


def test_graph_frames_c32_match_oracle(gpu_ok):
    scene = host.Scene(**host.SMALL_MAP)
    st = scene.static_data()
    w, h = 640, 480
    frames = _prepare(scene, [0, 9, 33, 63], w, h, abi.SW_PIXEL_C32, False)
    r = gpu.GpuRenderer(st)
    try:
        for f in frames:
            got = np.zeros((h, w), np.uint32)
            r.draw_frame(r.frame_input(f["params"], f["lights"], f["surfaces"], f["total_texels"], f["draws"],
                                       f["vertices"], dst=got))
            arena = oracle.build_surfaces(st, f["surfaces"], f["lights"], f["params"], f["total_texels"], num_threads=8)
            want = np.zeros((h, w), np.uint32)
            oracle.rasterize(f["draws"], f["vertices"], arena, f["params"], want)
            assert np.array_equal(want, got)
    finally:
        r.close()


def test_graph_hdr_sequence_matches_per_call_path(gpu_ok):
    """Colour64 + bloom + tonemap over a frame sequence: the graph path and the per-call path give the
    same Color32 frames and exposures (the per-call path is checked against the oracle elsewhere), and
    the first frame matches the oracle."""
    scene = host.Scene(**dict(host.FULL_MAP, grid_x=4, grid_y=4))
    st = scene.static_data()
    w, h = 480, 270
    frames = _prepare(scene, [0, 30, 31, 32, 90], w, h, abi.SW_PIXEL_C64, True)
    cfg = abi.PostConfig.default()
    rg, rc = gpu.GpuRenderer(st), gpu.GpuRenderer(st)
    try:
        for i, f in enumerate(frames):
            got = np.zeros((h, w), np.uint32)
            rg.draw_frame(rg.frame_input(f["params"], f["lights"], f["surfaces"], f["total_texels"], f["draws"],
                                         f["vertices"], post_config=cfg, dst=got))
            rc.frame_begin(f["params"], f["lights"])
            rc.submit_surfaces(f["surfaces"], f["total_texels"])
            rc.submit_draws(f["draws"], f["vertices"])
            rc.render()
            want = np.zeros((h, w), np.uint32)
            rc.postprocess(cfg, 1.0 / 60.0, (1.0, 1.0, 1.0), out=want)
            assert np.array_equal(want, got), f"frame {i}"
            assert rg.exposure() == rc.exposure()
            if i == 0:
                arena = oracle.build_surfaces(st, f["surfaces"], f["lights"], f["params"], f["total_texels"], num_threads=8)
                hdr = np.zeros((h, w), np.uint64)
                oracle.rasterize(f["draws"], f["vertices"], arena, f["params"], hdr)
                want_ldr, _, _ = oracle.postprocess(cfg, hdr, 1.0 / 60.0, (1.0, 1.0, 1.0), 1.0)
                assert np.array_equal(want_ldr, got)
    finally:
        rg.close()
        rc.close()


def test_graph_device_output_and_direct_mode(gpu_ok):
    import torch
    scene = host.Scene(**host.SMALL_MAP)
    st = scene.static_data()
    w, h = 320, 240
    f = _prepare(scene, [17], w, h, abi.SW_PIXEL_C32, False)[0]
    r = gpu.GpuRenderer(st)
    try:
        dev = torch.zeros((h, w + 8), dtype=torch.int32, device="cuda:0")
        r.draw_frame(r.frame_input(f["params"], f["lights"], f["surfaces"], f["total_texels"], f["draws"], f["vertices"],
                                   dst_device_ptr=dev.data_ptr(), pitch=w + 8))
        r.sync()
        got_graph = dev[:, :w].cpu().numpy().view(np.uint32).copy()
        r.set_frame_graph(False)
        host_out = np.zeros((h, w), np.uint32)
        r.draw_frame(r.frame_input(f["params"], f["lights"], f["surfaces"], f["total_texels"], f["draws"], f["vertices"],
                                   dst=host_out))
        assert np.array_equal(got_graph, host_out)
        assert np.all(dev[:, w:].cpu().numpy() == 0)
    finally:
        r.close()


def test_every_tuning_gives_the_same_frame(gpu_ok):
    scene = host.Scene(**dict(host.FULL_MAP, grid_x=4, grid_y=4))
    st = scene.static_data()
    w, h = 480, 270
    f = _prepare(scene, [31], w, h, abi.SW_PIXEL_C64, True)[0]
    arena = oracle.build_surfaces(st, f["surfaces"], f["lights"], f["params"], f["total_texels"], num_threads=8)
    want = np.zeros((h, w), np.uint64)
    oracle.rasterize(f["draws"], f["vertices"], arena, f["params"], want)
    r = gpu.GpuRenderer(st)
    try:
        for tile in range(abi.SW_RASTER_TILE_VARIANTS):
            for blocks in (1, 8, 64):
                r.set_tuning(tile, blocks)
                got = np.zeros((h, w), np.uint64)
                r.draw_frame(r.frame_input(f["params"], f["lights"], f["surfaces"], f["total_texels"], f["draws"],
                                           f["vertices"], dst=got))
                assert np.array_equal(want, got), (tile, blocks)
        with pytest.raises(gpu.SwError):
            r.set_tuning(abi.SW_RASTER_TILE_VARIANTS, 8)
    finally:
        r.close()


def test_autotune_keeps_best_and_restores_exposure(gpu_ok):
    scene = host.Scene(**dict(host.FULL_MAP, grid_x=4, grid_y=4))
    st = scene.static_data()
    w, h = 480, 270
    f = _prepare(scene, [44], w, h, abi.SW_PIXEL_C64, True)[0]
    cfg = abi.PostConfig.default()
    r = gpu.GpuRenderer(st)
    try:
        out = np.zeros((h, w), np.uint32)
        fi = r.frame_input(f["params"], f["lights"], f["surfaces"], f["total_texels"], f["draws"], f["vertices"],
                           post_config=cfg, dst=out)
        r.set_exposure(1.5)
        best, ms = r.autotune(fi, reps=3)
        assert 0 <= best.raster_tile < abi.SW_RASTER_TILE_VARIANTS and best.surface_blocks_per_sm >= 1
        assert 0.0 < ms < 50.0
        t = r.tuning()
        assert (t.raster_tile, t.surface_blocks_per_sm) == (best.raster_tile, best.surface_blocks_per_sm)
        assert r.exposure() == np.float32(1.5)
    finally:
        r.close()
