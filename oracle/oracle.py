"""Test infrastructure: ctypes binding of the CPU oracle (oracle/build/liboracle.so).

The oracle restates the reference's CPU renderer for the GPU path; only tests, the smoke check and
bench.py's CPU-baseline leg use it, as the checker. It takes the same descriptors as the GPU library.
"""
import ctypes
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "build", "liboracle.so")
sys.path.insert(0, os.path.join(HERE, "..", "square-wheel_gb300"))
from sqwheel import abi  # noqa: E402

_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE, "-j4"], check=True)
    return LIB_PATH


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        build()
    lib = ctypes.CDLL(LIB_PATH)
    vp, u32, u64, i32, f32 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int, ctypes.c_float
    lib.orc_build_surfaces.argtypes = [vp, vp, u32, vp, u32, vp, vp, u64, vp, vp, u64, u32]
    lib.orc_shadow_maps.argtypes = [vp, u32, vp, u32, vp, u64]
    lib.orc_rasterize.argtypes = [vp, u32, vp, u32, vp, u64, vp, u64, vp, vp, u32, u32, ctypes.POINTER(u64)]
    lib.orc_rasterize_ex.argtypes = [vp, u32, vp, u32, vp, u32, vp, u64, vp, u64, vp, u64, vp, vp, u32, u32,
                                     ctypes.POINTER(u64)]
    lib.orc_clear_background.argtypes = [vp, vp, u32]
    lib.orc_shadow_map_circle.argtypes = [vp, u64, u64, u32]
    lib.orc_postprocess.argtypes = [vp, vp, u32, u32, f32, vp, ctypes.POINTER(f32), vp, u32, vp]
    lib.orc_upscale.argtypes = [u32, u32, vp, vp, u32, u32, u32]
    lib.orc_gaussian_kernel.argtypes = [f32, u32, vp]
    lib.orc_turb_shifts.argtypes = [f32, f32, f32, f32, u32, u32, u32, vp, u32]
    lib.orc_apply_texture_passes.argtypes = [vp, u32, vp, u32, vp, u32, vp, vp, u32, vp]
    lib.orc_sim_effect_size.restype = u32
    lib.orc_sim_create.argtypes = [vp]
    lib.orc_sim_create.restype = vp
    lib.orc_sim_destroy.argtypes = [vp]
    lib.orc_sim_update.argtypes = [vp, f32, vp, u32, vp, vp, u32, vp, u32]
    lib.orc_sim_state.argtypes = [vp, vp, u64, vp, vp, vp]
    lib.orc_xoshiro_outputs.argtypes = [vp, vp, u32]
    lib.orc_small_rng_state.argtypes = [u64, vp]
    lib.orc_mix_view.argtypes = [vp, vp, u32, vp, u64]
    for name in ("orc_compress_lightmaps", "orc_decompress_lightmaps", "orc_compress_directional_lightmaps",
                 "orc_decompress_directional_lightmaps"):
        getattr(lib, name).argtypes = [vp, u64, vp]
    for fn in (lib.orc_build_surfaces, lib.orc_rasterize, lib.orc_rasterize_ex, lib.orc_clear_background, lib.orc_postprocess,
               lib.orc_upscale, lib.orc_gaussian_kernel, lib.orc_shadow_maps, lib.orc_shadow_map_circle):
        fn.restype = i32
    _lib = lib
    return lib


def _check(r, what):
    if r != 0:
        raise RuntimeError(f"{what} failed with status {r}")


def build_surfaces(static, surfaces, lights, frame_params, total_texels, num_threads=1, shadows=None, shadow_texels=None):
    """shadows: one SW LightShadow per light (abi.LIGHT_SHADOW) with the f32 cube maps in shadow_texels."""
    lib = load()
    ci = static.create_info()
    surfaces = np.ascontiguousarray(surfaces, dtype=abi.SURFACE_DESC)
    lights = np.ascontiguousarray(lights if lights is not None else np.zeros(0, abi.LIGHT), dtype=abi.LIGHT)
    dt = np.uint64 if frame_params.pixel_format == abi.SW_PIXEL_C64 else np.uint32
    arena = np.zeros(int(total_texels), dt)
    sh_ptr, tex_ptr, tex_n = None, None, 0
    if shadows is not None and len(shadows):
        shadows = np.ascontiguousarray(shadows, dtype=abi.LIGHT_SHADOW)
        assert shadows.size == lights.size
        shadow_texels = np.ascontiguousarray(shadow_texels, dtype=np.float32)
        sh_ptr, tex_ptr, tex_n = abi.ptr(shadows), abi.ptr(shadow_texels), shadow_texels.size
    _check(lib.orc_build_surfaces(ctypes.byref(ci), abi.ptr(surfaces), surfaces.size, abi.ptr(lights), lights.size,
                                  sh_ptr, tex_ptr, tex_n, ctypes.byref(frame_params), abi.ptr(arena), arena.size,
                                  num_threads),
           "orc_build_surfaces")
    return arena


def shadow_maps(draws, vertices, storage):
    """Draw the depth draws in order into `storage` (f32, in place; nothing is cleared)."""
    lib = load()
    draws = np.ascontiguousarray(draws, dtype=abi.DEPTH_DRAW)
    vertices = np.ascontiguousarray(vertices, dtype=abi.VERTEX16)
    assert storage.dtype == np.float32 and storage.flags["C_CONTIGUOUS"]
    _check(lib.orc_shadow_maps(abi.ptr(draws), draws.size, abi.ptr(vertices), vertices.size, abi.ptr(storage), storage.size),
           "orc_shadow_maps")
    return storage


def shadow_map_circle(storage, offset, size):
    """make_shadow_map_circle on the projector map at `offset` of the f32 storage, in place."""
    _check(load().orc_shadow_map_circle(abi.ptr(storage), storage.size, int(offset), int(size)), "orc_shadow_map_circle")


def rasterize(draws, vertices, arena, frame_params, framebuffer, num_threads=1, skybox=None, tri_vertices=None, lite=None):
    """Rasterise into `framebuffer` (height, pitch) in place; returns the count of bad texel fetches.
    skybox: the skybox texels (frame's pixel format) that SW_TEXSRC_SKYBOX draws read; tri_vertices and
    lite: the vertices and Color32 textures of SW_RASTER_TRIANGLE draws."""
    lib = load()
    draws = np.ascontiguousarray(draws, dtype=abi.DRAW_CMD)
    vertices = np.ascontiguousarray(vertices if vertices is not None else np.zeros(0, abi.VERTEX16), dtype=abi.VERTEX16)
    bad = ctypes.c_uint64(0)
    sky_ptr, sky_n = (None, 0) if skybox is None or len(skybox) == 0 else (abi.ptr(skybox), len(skybox))
    arena_ptr, arena_n = (None, 0) if arena is None else (abi.ptr(arena), arena.size)
    tv = np.ascontiguousarray(tri_vertices if tri_vertices is not None else np.zeros(0, abi.TRI_VERTEX), dtype=abi.TRI_VERTEX)
    lt = np.ascontiguousarray(lite if lite is not None else np.zeros(0, np.uint32), dtype=np.uint32).reshape(-1)
    _check(lib.orc_rasterize_ex(abi.ptr(draws), draws.size, abi.ptr(vertices), vertices.size, abi.ptr(tv), tv.size,
                                arena_ptr, arena_n, sky_ptr, sky_n, abi.ptr(lt), lt.size, ctypes.byref(frame_params),
                                abi.ptr(framebuffer), framebuffer.shape[1], num_threads, ctypes.byref(bad)),
           "orc_rasterize_ex")
    return bad.value


def clear_background(frame_params, framebuffer):
    _check(load().orc_clear_background(ctypes.byref(frame_params), abi.ptr(framebuffer), framebuffer.shape[1]),
           "orc_clear_background")


def postprocess(config, hdr, frame_duration_s, color_modulate, exposure, pitch=None):
    """Returns (ldr frame (h, pitch) uint32, new exposure, average colour lanes)."""
    lib = load()
    hdr = np.ascontiguousarray(hdr, dtype=np.uint64)
    h, w = hdr.shape
    pitch = pitch or w
    out = np.zeros((h, pitch), np.uint32)
    e = ctypes.c_float(exposure)
    avg = np.zeros(4, np.float32)
    mod = (ctypes.c_float * 3)(*[float(c) for c in color_modulate])
    _check(lib.orc_postprocess(ctypes.byref(config), abi.ptr(hdr), w, h, float(frame_duration_s), mod, ctypes.byref(e),
                               abi.ptr(out), pitch, abi.ptr(avg)), "orc_postprocess")
    return out, e.value, avg


def upscale(mode, scale, src, dst_width, dst_height):
    lib = load()
    src = np.ascontiguousarray(src, dtype=np.uint32)
    out = np.zeros((dst_height, dst_width), np.uint32)
    _check(lib.orc_upscale(mode, scale, abi.ptr(src), abi.ptr(out), dst_width, dst_height, dst_width), "orc_upscale")
    return out


def gaussian_kernel(sigma, radius):
    out = np.zeros(33, np.float32)
    _check(load().orc_gaussian_kernel(float(sigma), radius, abi.ptr(out)), "orc_gaussian_kernel")
    return out


def compress_lightmaps(rgb):
    """CompressedColor records (n, 4) uint8 of float32 (n, 3) lightmap elements."""
    rgb = np.ascontiguousarray(rgb, dtype=np.float32).reshape(-1, 3)
    out = np.zeros((rgb.shape[0], 4), np.uint8)
    _check(load().orc_compress_lightmaps(abi.ptr(rgb), rgb.shape[0], abi.ptr(out)), "orc_compress_lightmaps")
    return out


def decompress_lightmaps(records):
    records = np.ascontiguousarray(records, dtype=np.uint8).reshape(-1, 4)
    out = np.zeros((records.shape[0], 3), np.float32)
    _check(load().orc_decompress_lightmaps(abi.ptr(records), records.shape[0], abi.ptr(out)), "orc_decompress_lightmaps")
    return out


def compress_directional_lightmaps(elements):
    """13-byte records (n, 13) uint8 of abi.DIR_LIGHTMAP_ELEMENT elements."""
    elements = np.ascontiguousarray(elements, dtype=abi.DIR_LIGHTMAP_ELEMENT)
    out = np.zeros((elements.size, 13), np.uint8)
    _check(load().orc_compress_directional_lightmaps(abi.ptr(elements), elements.size, abi.ptr(out)),
           "orc_compress_directional_lightmaps")
    return out


def decompress_directional_lightmaps(records):
    records = np.ascontiguousarray(records, dtype=np.uint8).reshape(-1, 13)
    out = np.zeros(records.shape[0], abi.DIR_LIGHTMAP_ELEMENT)
    _check(load().orc_decompress_directional_lightmaps(abi.ptr(records), records.shape[0], abi.ptr(out)),
           "orc_decompress_directional_lightmaps")
    return out


def turb_shifts(amplitude, wave_length, frequency, time_s, width, height, mip, buffer):
    """make_turb_distortion's shift table into `buffer` (int32, len >= max(width, height)), in place."""
    assert buffer.dtype == np.int32 and buffer.flags["C_CONTIGUOUS"]
    _check(load().orc_turb_shifts(amplitude, wave_length, frequency, time_s, width, height, mip, abi.ptr(buffer),
                                  buffer.size), "orc_turb_shifts")
    return buffer


def apply_texture_passes(passes, shifts, static):
    """The texture effect passes applied in order to static.texels / static.emissive_pixels, in place."""
    passes = np.ascontiguousarray(passes, dtype=abi.TEXTURE_PASS)
    shifts = np.ascontiguousarray(shifts if shifts is not None else np.zeros(0, np.int32), dtype=np.int32)
    assert static.texels.flags["C_CONTIGUOUS"] and static.emissive_pixels.flags["C_CONTIGUOUS"]
    _check(load().orc_apply_texture_passes(abi.ptr(passes), passes.size, abi.ptr(shifts), shifts.size,
                                           abi.ptr(static.texture_mips), static.texture_mips.size, abi.ptr(static.texels),
                                           abi.ptr(static.emissive_mips), static.emissive_mips.size,
                                           abi.ptr(static.emissive_pixels)), "orc_apply_texture_passes")


class SimEffect:
    """A water or fire effect run whole on the CPU (orc_sim_*): created from the effect description's bytes
    (the host's SwhSimEffect layout), updated at frame times against a copy of the static texture data,
    into which each update writes the generated texture at the effect's output slot."""

    def __init__(self, effect):
        lib = load()
        raw = bytes(effect)
        assert len(raw) == lib.orc_sim_effect_size(), "effect description layout differs from the oracle's"
        self._buf = ctypes.create_string_buffer(raw, len(raw))
        self.handle = lib.orc_sim_create(self._buf)
        if not self.handle:
            raise RuntimeError("orc_sim_create refused the effect")
        self.area = 1 << (effect.resolution_log2[0] + effect.resolution_log2[1])

    def update(self, time_s, static, source_texture):
        """One GenerativeTextureEffect::update; True when it generated the texture this time."""
        r = load().orc_sim_update(self.handle, time_s, abi.ptr(static.texture_mips), static.texture_mips.size,
                                  abi.ptr(static.texels), abi.ptr(static.emissive_mips), static.emissive_mips.size,
                                  abi.ptr(static.emissive_pixels), source_texture)
        if r < 0:
            raise RuntimeError(f"orc_sim_update failed with status {r}")
        return r == 1

    def state(self):
        """(field words: f32 bits of the wave field or the heat values, update_step, generated, particles)."""
        words = np.zeros(self.area, np.uint32)
        v = [ctypes.c_uint32() for _ in range(3)]
        _check(load().orc_sim_state(self.handle, abi.ptr(words), words.size, *[ctypes.byref(x) for x in v]),
               "orc_sim_state")
        return words, int(v[0].value), int(v[1].value), int(v[2].value)

    def close(self):
        if self.handle:
            load().orc_sim_destroy(self.handle)
            self.handle = None

    def __del__(self):
        self.close()


def xoshiro_outputs(state, n):
    st = np.ascontiguousarray(state, dtype=np.uint64)
    out = np.zeros(n, np.uint64)
    load().orc_xoshiro_outputs(abi.ptr(st), abi.ptr(out), n)
    return out


def small_rng_state(seed):
    out = np.zeros(4, np.uint64)
    load().orc_small_rng_state(seed, abi.ptr(out))
    return out


def render_views(views, draws, vertices, arena, frame_params, tri_vertices=None, lite=None, skybox=None, num_threads=1):
    """The nested views of a whole frame (SwView), in order, into the arena: each region cleared to black,
    its background drawn when it says so, rasterised from its draws and mixed with its texture."""
    lt = np.ascontiguousarray(lite if lite is not None else np.zeros(1, np.uint32), dtype=np.uint32).reshape(-1)
    for v in np.atleast_1d(views):
        w, h = int(v["width"]), int(v["height"])
        params = abi.FrameParams()
        ctypes.pointer(params)[0] = frame_params
        params.width, params.height, params.clear_background = w, h, int(v["clear_background"])
        region = np.zeros((h, w), arena.dtype)
        if params.clear_background:
            clear_background(params, region)
        first, n = int(v["first_draw"]), int(v["num_draws"])
        if n:
            bad = rasterize(draws[first:first + n], vertices, arena, params, region, num_threads=num_threads,
                            skybox=skybox, tri_vertices=tri_vertices, lite=lt)
            assert bad == 0, "bad texel fetches in a view"
        one = np.ascontiguousarray(v).view(abi.VIEW)
        _check(load().orc_mix_view(abi.ptr(one), abi.ptr(region), frame_params.pixel_format, abi.ptr(lt), lt.size),
               "orc_mix_view")
        off = int(v["target_offset"])
        arena[off:off + w * h] = region.reshape(-1)
    return arena
