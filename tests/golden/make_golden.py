"""Generates the golden fixtures in this directory: seeded inputs of the GPU path's stages and the outputs
of the oracle (the C++ restatement of the reference's CPU path, single-threaded) on them.

The reference ships no test vectors for this path and cannot be built here (no Rust toolchain), so these
fixtures anchor regressions of the oracle and of the GPU path alike: tests/test_golden.py checks that the
oracle still reproduces them bit for bit (CPU) and that the CUDA path does too (GPU).

Usage: python tests/golden/make_golden.py   (rewrites the .npz files)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (os.path.join(ROOT, "square-wheel_gb300"), os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)

import oracle  # noqa: E402
import scenes  # noqa: E402
from sqwheel import abi, gpu, host, synth  # noqa: E402

SURFACE_CASES = {
    # name: BatchedSurfaces arguments
    "surfaces_c64_directional": dict(seed=101, count=24, min_side=4, max_side=40, num_materials=4, texture_size=32,
                                     num_lights=4, emissive_frac=0.25, directional=True, pixel_format=abi.SW_PIXEL_C64),
    "surfaces_c32_simple": dict(seed=102, count=24, min_side=4, max_side=40, num_materials=4, texture_size=32,
                                num_lights=2, emissive_frac=0.25, directional=False, pixel_format=abi.SW_PIXEL_C32),
}
RASTER_CASES = {
    "raster_c32": dict(seed=201, width=160, height=120, num_quads=30, modes=(0, 1, 2), blends=(0, 1, 2, 3, 4),
                       pixel_format=abi.SW_PIXEL_C32, texel_density=0.2, max_texture_side=48),
    "raster_c64": dict(seed=202, width=160, height=120, num_quads=30, modes=(0, 1, 2), blends=(0, 1, 2, 3, 4),
                       pixel_format=abi.SW_PIXEL_C64, texel_density=0.2, max_texture_side=48),
}
# A frame of the sky map (draw_skybox first, then the world) at 160x120 Color64: skybox sides of 32 texels
# at HDR brightness 2, rotated by the frame's sky angle.
SKY_RASTER_CASES = {
    "raster_sky_c64": dict(scene=dict(host.SKY_MAP, skybox_size=32), frame=5, width=160, height=120,
                           pixel_format=abi.SW_PIXEL_C64),
}
POST_CASES = {
    # name: (PostConfig overrides, frames)
    "post_bloom_nearest": (dict(bloom_buffer_scale_log2=1, linear_bloom_filter=0, bloom_sigma=1.0), 2),
    "post_bloom_linear_s4": (dict(bloom_buffer_scale_log2=2, linear_bloom_filter=1, bloom_sigma=6.0), 2),
    "post_no_bloom": (dict(bloom_sigma=0.0), 2),
}


def frame_params_array(fp):
    return np.frombuffer(bytes(fp), np.uint8).copy()


def make_surfaces(name, kw):
    b = synth.BatchedSurfaces(**kw)
    st = b.static_data()
    fp = gpu.frame_params(64, 64, b.pixel_format, b.cam_pos, directional=b.directional)
    want = oracle.build_surfaces(st, b.surfaces, b.lights, fp, b.total_texels, num_threads=1)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), texels=st.texels, texture_mips=st.texture_mips,
                        emissive_pixels=st.emissive_pixels, emissive_mips=st.emissive_mips, lightmaps=st.lightmaps,
                        directional_lightmaps=st.directional_lightmaps, surfaces=b.surfaces, lights=b.lights,
                        frame_params=frame_params_array(fp), total_texels=np.uint64(b.total_texels), want=want)


def make_raster(name, kw):
    kw = dict(kw)
    w, h, fmt = kw.pop("width"), kw.pop("height"), kw["pixel_format"]
    arena, draws, verts = scenes.make_raster_scene(kw.pop("seed"), w, h, kw.pop("num_quads"), **kw)
    rng = np.random.default_rng(7)
    dt = np.uint64 if fmt == abi.SW_PIXEL_C64 else np.uint32
    if fmt == abi.SW_PIXEL_C64:
        fb0 = rng.integers(0, 1 << 16, (h, w, 4), dtype=np.uint64)
        fb0 = (fb0[..., 0] | (fb0[..., 1] << 16) | (fb0[..., 2] << 32) | (fb0[..., 3] << 48)).astype(dt)
    else:
        fb0 = rng.integers(0, 1 << 32, (h, w), dtype=np.uint64).astype(dt)
    fp = gpu.frame_params(w, h, fmt, (0.0, 0.0, 0.0))
    want = fb0.copy()
    bad = oracle.rasterize(draws, verts, arena, fp, want)
    assert bad == 0
    np.savez_compressed(os.path.join(HERE, name + ".npz"), arena=arena, draws=draws, vertices=verts,
                        frame_params=frame_params_array(fp), framebuffer_in=fb0, want=want)


def make_sky_raster(name, kw):
    sc = host.Scene(**kw["scene"])
    w, h, fmt = kw["width"], kw["height"], kw["pixel_format"]
    fr = host.Frame(sc).prepare(kw["frame"], host.frame_options(w, h, fmt, directional=False))
    assert fr.skybox_draws > 0
    t32, t64, _, _ = sc.skybox()
    arena = oracle.build_surfaces(sc.static_data(), fr.surfaces, fr.lights, fr.params, fr.total_texels, num_threads=1)
    rng = np.random.default_rng(9)
    dt = np.uint64 if fmt == abi.SW_PIXEL_C64 else np.uint32
    fb0 = rng.integers(0, 1 << 16, (h, w), dtype=np.uint64).astype(dt)
    want = fb0.copy()
    bad = oracle.rasterize(fr.draws, fr.vertices, arena, fr.params, want, skybox=t64 if fmt == abi.SW_PIXEL_C64 else t32)
    assert bad == 0
    np.savez_compressed(os.path.join(HERE, name + ".npz"), arena=arena, draws=fr.draws, vertices=fr.vertices,
                        frame_params=frame_params_array(fr.params), framebuffer_in=fb0, want=want, skybox32=t32,
                        skybox64=t64)


def make_post(name, overrides, frames):
    cfg = abi.PostConfig.default()
    for k, v in overrides.items():
        setattr(cfg, k, v)
    rng = np.random.default_rng(301)
    w, h = 96, 64
    # smooth HDR content with a few bright spots (exercises bloom and the exposure loop)
    yy, xx = np.mgrid[0:h, 0:w]
    hdrs, wants, exposures = [], [], []
    exposure = 1.0
    for f in range(frames):
        lanes = []
        for c in range(3):
            base = 120 + 110 * np.sin(xx / (9.0 + c + f) + yy / (13.0 - c)) + rng.integers(0, 40, (h, w))
            spots = (rng.random((h, w)) < 0.01) * rng.integers(2000, 30000, (h, w))
            lanes.append(np.clip(base + spots, 0, 65535).astype(np.uint64))
        hdr = (lanes[0] | (lanes[1] << 16) | (lanes[2] << 32)).astype(np.uint64)
        ldr, exposure_next, _ = oracle.postprocess(cfg, hdr, 1.0 / 60.0, (1.0, 0.9, 0.8), exposure)
        hdrs.append(hdr)
        wants.append(ldr)
        exposures.append(exposure_next)
        exposure = exposure_next
    np.savez_compressed(os.path.join(HERE, name + ".npz"), config=frame_params_array(cfg), hdr=np.stack(hdrs),
                        want=np.stack(wants), exposures=np.array(exposures, np.float32),
                        color_modulate=np.array([1.0, 0.9, 0.8], np.float32))


def main():
    oracle.build()
    for name, kw in SURFACE_CASES.items():
        make_surfaces(name, kw)
    for name, kw in RASTER_CASES.items():
        make_raster(name, kw)
    for name, kw in SKY_RASTER_CASES.items():
        make_sky_raster(name, kw)
    for name, (ov, n) in POST_CASES.items():
        make_post(name, ov, n)
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
