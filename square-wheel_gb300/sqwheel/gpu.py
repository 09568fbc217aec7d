"""Python binding of the GB300 rendering library (libswgpu.so, C ABI in include/swgpu.h).

`GpuRenderer` mirrors the reference's per-frame API for the GPU path:
  Renderer::new            -> GpuRenderer(scene)                  (src/square_wheel/renderer.rs:24-59)
  Renderer::prepare_frame  -> frame_begin + submit_surfaces        (renderer.rs:61-104)
  Renderer::draw_frame     -> submit_draws + render               (renderer.rs:106-124)
  Postprocessor::perform_postprocessing -> postprocess            (postprocessor.rs:68-204)
  FrameUpscaler::perform_upscale        -> upscale                (frame_upscaler.rs:42-70)
There is no CPU fallback: constructing a renderer without the built library or without a GPU raises.
"""
import ctypes
import os

import numpy as np

from . import abi

PKG_DIR = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG_DIR, "lib", "libswgpu.so")

EXPORTED = [
    "sw_create", "sw_destroy", "sw_last_error", "sw_sync", "sw_frame_begin", "sw_submit_surfaces", "sw_rebuild_surfaces", "sw_rebuild_surfaces_per_surface", "sw_set_surfaces", "sw_set_skybox", "sw_register_host_buffer", "sw_unregister_host_buffer",
    "sw_submit_draws", "sw_submit_draws_ex", "sw_set_lite_textures", "sw_set_lightmaps_compressed", "sw_read_lightmaps",
    "sw_update_textures", "sw_read_texels", "sw_reserve_simulation_state", "sw_update_simulations",
    "sw_read_simulation_state",
    "sw_render", "sw_postprocess", "sw_upscale", "sw_read_surfaces", "sw_read_framebuffer", "sw_get_exposure", "sw_set_exposure",
    "sw_set_framebuffer", "sw_get_stats", "sw_get_stream", "sw_abi_layout", "sw_enable_timing", "sw_get_timings",
    "sw_postprocess_noalloc", "sw_set_learned_upscaler", "sw_draw_frame", "sw_set_frame_graph", "sw_set_frames_in_flight", "sw_set_tuning",
    "sw_get_tuning", "sw_autotune", "sw_set_map", "sw_draw_frame_view", "sw_read_view_prep",
    "sw_build_shadow_maps", "sw_set_light_shadows", "sw_read_shadow_maps", "sw_build_shadow_maps_view",
    # learned upscaler (include/swlearn.h)
    "sw_upscaler_create", "sw_upscaler_destroy", "sw_upscaler_last_error", "sw_upscaler_get_params",
    "sw_upscaler_set_params", "sw_upscaler_gradients", "sw_upscaler_train_step", "sw_upscaler_steps",
    "sw_upscaler_infer", "sw_upscaler_psnr", "sw_upscaler_save", "sw_upscaler_load",
    "sw_monitor_init", "sw_monitor_plan", "sw_monitor_report", "sw_upscaler_set_fused", "sw_upscaler_check", "sw_upscaler_wait_probe",
]

_lib = None


class SwError(RuntimeError):
    pass


def load_library(path=LIB_PATH):
    """Load libswgpu.so (built by square-wheel_gb300/build.py). Raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise SwError(f"{path} is missing: build it with `python square-wheel_gb300/build.py`")
    lib = ctypes.CDLL(path)
    vp, u32, u64, i32, f32 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int, ctypes.c_float
    sig = {
        "sw_create": ([vp, ctypes.POINTER(vp)], i32),
        "sw_destroy": ([vp], i32),
        "sw_last_error": ([vp], ctypes.c_char_p),
        "sw_sync": ([vp], i32),
        "sw_frame_begin": ([vp, vp, vp, u32], i32),
        "sw_submit_surfaces": ([vp, vp, u32, u64], i32),
        "sw_rebuild_surfaces": ([vp], i32),
        "sw_rebuild_surfaces_per_surface": ([vp], i32),
        "sw_set_surfaces": ([vp, vp, u64], i32),
        "sw_set_skybox": ([vp, vp, vp, u64], i32),
        "sw_register_host_buffer": ([vp, vp, u64], i32),
        "sw_unregister_host_buffer": ([vp, vp], i32),
        "sw_submit_draws": ([vp, vp, u32, vp, u32], i32),
        "sw_submit_draws_ex": ([vp, vp, u32, vp, u32, vp, u32], i32),
        "sw_set_lite_textures": ([vp, vp, u64], i32),
        "sw_set_lightmaps_compressed": ([vp, vp, u64, vp, u64], i32),
        "sw_update_textures": ([vp, vp, u32, vp, u32], i32),
        "sw_read_texels": ([vp, vp, u64, vp, u64], i32),
        "sw_reserve_simulation_state": ([vp, u64], i32),
        "sw_update_simulations": ([vp, vp, u32, vp, u32], i32),
        "sw_read_simulation_state": ([vp, u64, u64, vp], i32),
        "sw_read_lightmaps": ([vp, vp, u64, vp, u64], i32),
        "sw_render": ([vp, vp, u32, i32], i32),
        "sw_postprocess": ([vp, vp, f32, vp, vp, u32, i32], i32),
        "sw_upscale": ([vp, u32, u32, vp, i32, vp, u32, u32, u32, i32], i32),
        "sw_read_surfaces": ([vp, vp, u64], i32),
        "sw_read_framebuffer": ([vp, vp, u64], i32),
        "sw_get_exposure": ([vp, ctypes.POINTER(f32)], i32),
        "sw_set_exposure": ([vp, f32], i32),
        "sw_set_framebuffer": ([vp, vp, u32, u32, u32, i32], i32),
        "sw_get_stats": ([vp, vp], i32),
        "sw_get_stream": ([vp, ctypes.POINTER(vp)], i32),
        "sw_abi_layout": ([ctypes.POINTER(u32), u32], i32),
        "sw_postprocess_noalloc": ([vp, u32, u32, vp, f32, vp, vp, u32, vp, vp], i32),
        "sw_enable_timing": ([vp, i32], i32),
        "sw_get_timings": ([vp, vp], i32),
        "sw_set_learned_upscaler": ([vp, vp], i32),
        "sw_draw_frame": ([vp, vp], i32),
        "sw_set_frame_graph": ([vp, i32], i32),
        "sw_set_frames_in_flight": ([vp, u32], i32),
        "sw_set_tuning": ([vp, vp], i32),
        "sw_get_tuning": ([vp, vp], i32),
        "sw_autotune": ([vp, vp, u32, vp, ctypes.POINTER(f32)], i32),
        "sw_set_map": ([vp, vp, u32, vp, u32], i32),
        "sw_draw_frame_view": ([vp, vp], i32),
        "sw_read_view_prep": ([vp, vp, vp, u32, vp, u32, vp, u32], i32),
        "sw_build_shadow_maps": ([vp, vp, u32, vp, u32, u64], i32),
        "sw_set_light_shadows": ([vp, vp, u32], i32),
        "sw_read_shadow_maps": ([vp, vp, u64], i32),
        "sw_build_shadow_maps_view": ([vp, vp, u32, vp, u32, u64], i32),
        "sw_upscaler_create": ([i32, u64, ctypes.POINTER(vp)], i32),
        "sw_upscaler_destroy": ([vp], i32),
        "sw_upscaler_last_error": ([vp], ctypes.c_char_p),
        "sw_upscaler_get_params": ([vp, vp, u32], i32),
        "sw_upscaler_set_params": ([vp, vp, u32], i32),
        "sw_upscaler_gradients": ([vp, vp, u32, vp, ctypes.POINTER(f32)], i32),
        "sw_upscaler_train_step": ([vp, vp, u32, f32, ctypes.POINTER(f32)], i32),
        "sw_upscaler_steps": ([vp, ctypes.POINTER(u64)], i32),
        "sw_upscaler_infer": ([vp, vp, u32, u32, u32, vp, u32, vp], i32),
        "sw_upscaler_psnr": ([vp, vp, u32, vp, u32, u32, u32, vp, ctypes.POINTER(ctypes.c_double)], i32),
        "sw_upscaler_save": ([vp, ctypes.c_char_p], i32),
        "sw_upscaler_load": ([vp, ctypes.c_char_p], i32),
        "sw_monitor_init": ([vp, u32, f32, u32], i32),
        "sw_upscaler_set_fused": ([vp, i32], i32),
        "sw_upscaler_check": ([vp], i32),
        "sw_upscaler_wait_probe": ([vp, u32, ctypes.POINTER(ctypes.c_int)], i32),
        "sw_monitor_plan": ([vp, ctypes.POINTER(u32)], i32),
        "sw_monitor_report": ([vp, ctypes.c_double], i32),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


def abi_layout():
    lib = load_library()
    sizes = (ctypes.c_uint32 * 32)()
    n = lib.sw_abi_layout(sizes, 32)
    return [int(sizes[i]) for i in range(n)]


class StaticData:
    """Static map data uploaded once: textures with mips, emissive textures, lightmaps."""

    def __init__(self, texels, texture_mips, emissive_pixels=None, emissive_mips=None, lightmaps=None,
                 directional_lightmaps=None):
        self.texels = np.ascontiguousarray(texels, dtype=np.uint64)
        self.texture_mips = np.ascontiguousarray(texture_mips, dtype=abi.TEXTURE_MIP)
        self.emissive_pixels = np.ascontiguousarray(
            emissive_pixels if emissive_pixels is not None else np.zeros(0, np.uint32), dtype=np.uint32)
        self.emissive_mips = np.ascontiguousarray(
            emissive_mips if emissive_mips is not None else np.zeros(0, abi.EMISSIVE_MIP), dtype=abi.EMISSIVE_MIP)
        self.lightmaps = np.ascontiguousarray(
            lightmaps if lightmaps is not None else np.zeros((1, 3), np.float32), dtype=np.float32).reshape(-1, 3)
        self.directional_lightmaps = np.ascontiguousarray(
            directional_lightmaps if directional_lightmaps is not None else np.zeros(0, abi.DIR_LIGHTMAP_ELEMENT),
            dtype=abi.DIR_LIGHTMAP_ELEMENT)

    def create_info(self, device=0):
        ci = abi.CreateInfo()
        ci.abi_version = abi.SWGPU_ABI_VERSION
        ci.device = device
        ci.texels = abi.ptr(self.texels)
        ci.num_texels = self.texels.size
        ci.texture_mips = abi.ptr(self.texture_mips)
        ci.num_texture_mips = self.texture_mips.size
        ci.emissive_pixels = abi.ptr(self.emissive_pixels)
        ci.num_emissive_pixels = self.emissive_pixels.size
        ci.emissive_mips = abi.ptr(self.emissive_mips)
        ci.num_emissive_mips = self.emissive_mips.size
        ci.lightmaps = abi.ptr(self.lightmaps)
        ci.num_lightmap_elements = self.lightmaps.shape[0]
        ci.directional_lightmaps = abi.ptr(self.directional_lightmaps)
        ci.num_directional_lightmap_elements = self.directional_lightmaps.size
        return ci


def frame_params(width, height, pixel_format, cam_pos, directional=True, clear_background=False):
    fp = abi.FrameParams()
    fp.pixel_format = pixel_format
    fp.width = width
    fp.height = height
    fp.use_directional_lightmaps = 1 if directional else 0
    for i in range(3):
        fp.cam_pos[i] = float(cam_pos[i])
    fp.clear_background = 1 if clear_background else 0
    return fp


class GpuRenderer:
    """One rendering context on one GPU (SwCtx)."""

    def __init__(self, static: StaticData, device=0):
        self.lib = load_library()
        self.static = static  # keep host arrays alive for the duration of sw_create
        self.ctx = ctypes.c_void_p()
        ci = static.create_info(device)
        r = self.lib.sw_create(ctypes.byref(ci), ctypes.byref(self.ctx))
        if r != abi.SW_OK:
            raise SwError(f"sw_create failed with status {r}")

    def _check(self, r, what):
        if r != abi.SW_OK:
            msg = self.lib.sw_last_error(self.ctx)
            raise SwError(f"{what} failed ({r}): {msg.decode() if msg else ''}")

    def close(self):
        if self.ctx:
            self.lib.sw_destroy(self.ctx)
            self.ctx = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def stream_handle(self):
        s = ctypes.c_void_p()
        self._check(self.lib.sw_get_stream(self.ctx, ctypes.byref(s)), "sw_get_stream")
        return s.value or 0

    def frame_begin(self, params, lights=None):
        lights = np.ascontiguousarray(lights if lights is not None else np.zeros(0, abi.LIGHT), dtype=abi.LIGHT)
        self._lights = lights
        self._check(self.lib.sw_frame_begin(self.ctx, ctypes.byref(params), abi.ptr(lights), lights.size), "sw_frame_begin")

    def submit_surfaces(self, surfaces, total_texels):
        surfaces = np.ascontiguousarray(surfaces, dtype=abi.SURFACE_DESC)
        self._check(self.lib.sw_submit_surfaces(self.ctx, abi.ptr(surfaces), surfaces.size, int(total_texels)),
                    "sw_submit_surfaces")

    def build_shadow_maps(self, depth_draws, depth_vertices, total_texels):
        d = np.ascontiguousarray(depth_draws, dtype=abi.DEPTH_DRAW)
        v = np.ascontiguousarray(depth_vertices, dtype=abi.VERTEX16)
        self._check(self.lib.sw_build_shadow_maps(self.ctx, abi.ptr(d), d.size, abi.ptr(v), v.size, int(total_texels)),
                    "sw_build_shadow_maps")

    def set_light_shadows(self, shadows):
        sh = np.ascontiguousarray(shadows if shadows is not None else np.zeros(0, abi.LIGHT_SHADOW), dtype=abi.LIGHT_SHADOW)
        self._shadows = sh
        self._check(self.lib.sw_set_light_shadows(self.ctx, abi.ptr(sh), sh.size), "sw_set_light_shadows")

    def build_shadow_maps_view(self, sides, leafs, total_texels):
        """Depth draws prepared on the GPU from the cube sides and their leafs (needs set_map)."""
        s = np.ascontiguousarray(sides, abi.SHADOW_SIDE)
        lf = np.ascontiguousarray(leafs, abi.SHADOW_LEAF)
        self._check(self.lib.sw_build_shadow_maps_view(self.ctx, abi.ptr(s), s.size, abi.ptr(lf), lf.size, int(total_texels)),
                    "sw_build_shadow_maps_view")

    def read_shadow_maps(self, texels):
        out = np.zeros(int(texels), np.float32)
        self._check(self.lib.sw_read_shadow_maps(self.ctx, abi.ptr(out), out.size), "sw_read_shadow_maps")
        return out

    def rebuild_surfaces_per_surface(self):
        """The last submitted surfaces again, one launch per surface (the unbatched baseline)."""
        self._check(self.lib.sw_rebuild_surfaces_per_surface(self.ctx), "sw_rebuild_surfaces_per_surface")

    def rebuild_surfaces(self):
        self._check(self.lib.sw_rebuild_surfaces(self.ctx), "sw_rebuild_surfaces")

    def set_surfaces(self, arena):
        arena = np.ascontiguousarray(arena)
        self._check(self.lib.sw_set_surfaces(self.ctx, abi.ptr(arena), arena.size), "sw_set_surfaces")

    def set_skybox(self, texels32, texels64):
        """Skybox side textures (all sides and mips, Color32 and Color64 copies of the same layout)."""
        t32 = np.ascontiguousarray(texels32, dtype=np.uint32)
        t64 = np.ascontiguousarray(texels64, dtype=np.uint64)
        if t32.size != t64.size:
            raise SwError("skybox texel arrays differ in size")
        self._check(self.lib.sw_set_skybox(self.ctx, abi.ptr(t32) if t32.size else None,
                                           abi.ptr(t64) if t64.size else None, t32.size), "sw_set_skybox")

    def set_lite_textures(self, pixels):
        """Color32 textures of triangle draws (SW_TEXSRC_LITE), one array."""
        pixels = np.ascontiguousarray(pixels, dtype=np.uint32).reshape(-1)
        self._check(self.lib.sw_set_lite_textures(self.ctx, abi.ptr(pixels), pixels.size), "sw_set_lite_textures")

    def set_lightmaps_compressed(self, simple, directional):
        """Replace the lightmaps with compressed records decoded on the GPU: simple (n, 4) and directional
        (m, 13) uint8 arrays as a compiled map holds them."""
        a = np.ascontiguousarray(simple, dtype=np.uint8).reshape(-1, 4)
        d = np.ascontiguousarray(directional, dtype=np.uint8).reshape(-1, 13)
        self._check(self.lib.sw_set_lightmaps_compressed(self.ctx, abi.ptr(a), a.shape[0], abi.ptr(d), d.shape[0]),
                    "sw_set_lightmaps_compressed")

    def update_textures(self, passes, shifts):
        """Run generative texture effect passes (abi.TEXTURE_PASS) with their turbulence shifts (int32)."""
        passes = np.ascontiguousarray(passes, dtype=abi.TEXTURE_PASS)
        shifts = np.ascontiguousarray(shifts if shifts is not None else np.zeros(0, np.int32), dtype=np.int32)
        self._check(self.lib.sw_update_textures(self.ctx, abi.ptr(passes), passes.size, abi.ptr(shifts), shifts.size),
                    "sw_update_textures")

    def reserve_simulation_state(self, words):
        self._check(self.lib.sw_reserve_simulation_state(self.ctx, int(words)), "sw_reserve_simulation_state")

    def update_simulations(self, passes, points):
        """Run simulated texture effect passes (abi.SIM_PASS, sorted by launch) with their points (abi.SIM_POINT)."""
        passes = np.ascontiguousarray(passes, dtype=abi.SIM_PASS)
        points = np.ascontiguousarray(points if points is not None else np.zeros(0, abi.SIM_POINT), dtype=abi.SIM_POINT)
        self._check(self.lib.sw_update_simulations(self.ctx, abi.ptr(passes), passes.size, abi.ptr(points), points.size),
                    "sw_update_simulations")

    def read_simulation_state(self, first, count):
        out = np.empty(int(count), np.uint32)
        self._check(self.lib.sw_read_simulation_state(self.ctx, int(first), out.size, abi.ptr(out)),
                    "sw_read_simulation_state")
        return out

    def read_texels(self, num_texels, num_emissive=0):
        """The context's material texels (uint64) and emissive pixels (uint32), e.g. after texture passes."""
        out = np.empty(int(num_texels), np.uint64)
        em = np.empty(int(num_emissive), np.uint32)
        self._check(self.lib.sw_read_texels(self.ctx, abi.ptr(out), out.size, abi.ptr(em), em.size), "sw_read_texels")
        return out, em

    def read_lightmaps(self, num_elements, num_directional):
        """The decoded lightmaps: (float32 (n, 3), DIR_LIGHTMAP_ELEMENT (m,))."""
        a = np.zeros((int(num_elements), 3), np.float32)
        d = np.zeros(int(num_directional), abi.DIR_LIGHTMAP_ELEMENT)
        self._check(self.lib.sw_read_lightmaps(self.ctx, abi.ptr(a), a.shape[0], abi.ptr(d), d.size), "sw_read_lightmaps")
        return a, d

    def submit_draws_ex(self, draws, vertices, tri_vertices):
        """Draws with triangle draws among them (SW_RASTER_TRIANGLE, vertices in tri_vertices)."""
        draws = np.ascontiguousarray(draws, dtype=abi.DRAW_CMD)
        vertices = np.ascontiguousarray(vertices if vertices is not None else np.zeros(0, abi.VERTEX16), dtype=abi.VERTEX16)
        tv = np.ascontiguousarray(tri_vertices if tri_vertices is not None else np.zeros(0, abi.TRI_VERTEX),
                                  dtype=abi.TRI_VERTEX)
        self._check(self.lib.sw_submit_draws_ex(self.ctx, abi.ptr(draws), draws.size, abi.ptr(vertices), vertices.size,
                                                abi.ptr(tv), tv.size), "sw_submit_draws_ex")

    def submit_draws(self, draws, vertices):
        draws = np.ascontiguousarray(draws, dtype=abi.DRAW_CMD)
        vertices = np.ascontiguousarray(vertices, dtype=abi.VERTEX16)
        self._check(self.lib.sw_submit_draws(self.ctx, abi.ptr(draws), draws.size, abi.ptr(vertices), vertices.size),
                    "sw_submit_draws")

    def render(self, out=None, device_ptr=None, pitch=None):
        """Rasterise. `out` = host numpy array (height, pitch) to receive the frame, or device_ptr."""
        if out is not None:
            p = pitch or out.shape[1]
            self._check(self.lib.sw_render(self.ctx, abi.ptr(out), p, 0), "sw_render")
        elif device_ptr is not None:
            self._check(self.lib.sw_render(self.ctx, ctypes.c_void_p(device_ptr), pitch, 1), "sw_render")
        else:
            self._check(self.lib.sw_render(self.ctx, None, 0, 0), "sw_render")

    def set_framebuffer(self, frame, pixel_format):
        frame = np.ascontiguousarray(frame)
        h, w = frame.shape
        self._check(self.lib.sw_set_framebuffer(self.ctx, abi.ptr(frame), w, h, pixel_format, 0), "sw_set_framebuffer")

    def postprocess(self, config, frame_duration_s, color_modulate, out=None, device_ptr=None, pitch=None):
        mod = (ctypes.c_float * 3)(*[float(c) for c in color_modulate])
        if out is not None:
            r = self.lib.sw_postprocess(self.ctx, ctypes.byref(config), float(frame_duration_s), mod, abi.ptr(out),
                                        pitch or out.shape[1], 0)
        else:
            r = self.lib.sw_postprocess(self.ctx, ctypes.byref(config), float(frame_duration_s), mod,
                                        ctypes.c_void_p(device_ptr), pitch, 1)
        self._check(r, "sw_postprocess")

    def upscale(self, mode, scale, src, out):
        src = np.ascontiguousarray(src, dtype=np.uint32)
        h, w = out.shape
        self._check(self.lib.sw_upscale(self.ctx, mode, scale, abi.ptr(src), 0, abi.ptr(out), w, h, w, 0), "sw_upscale")

    def upscale_device(self, mode, scale, src_ptr, dst_ptr, width, height, pitch):
        self._check(self.lib.sw_upscale(self.ctx, mode, scale, ctypes.c_void_p(src_ptr), 1, ctypes.c_void_p(dst_ptr),
                                        width, height, pitch, 1), "sw_upscale")

    def frame_input(self, params, lights, surfaces, total_texels, draws, vertices, post_config=None,
                    frame_duration_s=1.0 / 60.0, color_modulate=(1.0, 1.0, 1.0), dst=None, dst_device_ptr=None, pitch=None,
                    tri_vertices=None):
        """SwFrameInput for draw_frame / autotune (keeps the arrays it points to alive on the object)."""
        fi = abi.FrameInput()
        fi.params = params
        keep = []
        def arr(a, dt):
            a = np.ascontiguousarray(a if a is not None else np.zeros(0, dt), dtype=dt)
            keep.append(a)
            return a
        lights = arr(lights, abi.LIGHT)
        surfaces = arr(surfaces, abi.SURFACE_DESC)
        draws = arr(draws, abi.DRAW_CMD)
        vertices = arr(vertices, abi.VERTEX16)
        fi.num_lights, fi.lights = lights.size, abi.ptr(lights)
        fi.num_surfaces, fi.surfaces, fi.total_texels = surfaces.size, abi.ptr(surfaces), int(total_texels)
        fi.num_draws, fi.draws = draws.size, abi.ptr(draws)
        fi.num_vertices, fi.vertices = vertices.size, abi.ptr(vertices)
        tv = arr(tri_vertices, abi.TRI_VERTEX)
        fi.num_tri_vertices, fi.tri_vertices = tv.size, abi.ptr(tv)
        if post_config is not None:
            fi.postprocess = 1
            fi.post = post_config
        fi.frame_duration_s = frame_duration_s
        fi.color_modulate = (ctypes.c_float * 3)(*color_modulate)
        if dst is not None:
            keep.append(dst)
            fi.dst, fi.dst_pitch, fi.dst_is_device = abi.ptr(dst), pitch or dst.shape[1], 0
        elif dst_device_ptr is not None:
            fi.dst, fi.dst_pitch, fi.dst_is_device = ctypes.c_void_p(dst_device_ptr), pitch, 1
        fi._keep = keep
        return fi

    def draw_frame(self, frame_input):
        """One whole frame through sw_draw_frame (one CUDA graph unless disabled)."""
        self._check(self.lib.sw_draw_frame(self.ctx, ctypes.byref(frame_input)), "sw_draw_frame")

    def set_frames_in_flight(self, frames):
        self._check(self.lib.sw_set_frames_in_flight(self.ctx, int(frames)), "sw_set_frames_in_flight")

    def set_frame_graph(self, enable):
        self._check(self.lib.sw_set_frame_graph(self.ctx, 1 if enable else 0), "sw_set_frame_graph")

    def tuning(self):
        t = abi.Tuning()
        self._check(self.lib.sw_get_tuning(self.ctx, ctypes.byref(t)), "sw_get_tuning")
        return t

    def set_tuning(self, raster_tile, surface_blocks_per_sm, surface_texels_per_thread=0):
        t = abi.Tuning(raster_tile, surface_blocks_per_sm, surface_texels_per_thread, 0)
        self._check(self.lib.sw_set_tuning(self.ctx, ctypes.byref(t)), "sw_set_tuning")

    def autotune(self, frame_input, reps=5):
        """Returns (Tuning, median ms per frame) of the fastest configuration, which stays selected."""
        t = abi.Tuning()
        ms = ctypes.c_float()
        self._check(self.lib.sw_autotune(self.ctx, ctypes.byref(frame_input), reps, ctypes.byref(t), ctypes.byref(ms)),
                    "sw_autotune")
        return t, ms.value

    def attach_upscaler(self, ups):
        """Use a learned upscaler (sqwheel.learned.Upscaler, or None) for SW_UPSCALE_LEARNED."""
        self._check(self.lib.sw_set_learned_upscaler(self.ctx, ups.h if ups is not None else None),
                    "sw_set_learned_upscaler")

    def read_surfaces(self, total_texels, pixel_format):
        dt = np.uint64 if pixel_format == abi.SW_PIXEL_C64 else np.uint32
        out = np.empty(int(total_texels), dt)
        self._check(self.lib.sw_read_surfaces(self.ctx, abi.ptr(out), out.nbytes), "sw_read_surfaces")
        return out

    def read_framebuffer(self, width, height, pixel_format):
        """The context's frame buffer (the last rasterised frame) as a height x width array."""
        dt = np.uint64 if pixel_format == abi.SW_PIXEL_C64 else np.uint32
        out = np.empty((int(height), int(width)), dt)
        self._check(self.lib.sw_read_framebuffer(self.ctx, abi.ptr(out), out.nbytes), "sw_read_framebuffer")
        return out

    def exposure(self):
        e = ctypes.c_float()
        self._check(self.lib.sw_get_exposure(self.ctx, ctypes.byref(e)), "sw_get_exposure")
        return e.value

    def set_exposure(self, e):
        self._check(self.lib.sw_set_exposure(self.ctx, float(e)), "sw_set_exposure")

    def stats(self):
        s = abi.Stats()
        self._check(self.lib.sw_get_stats(self.ctx, ctypes.byref(s)), "sw_get_stats")
        return s

    def enable_timing(self, on=True):
        self._check(self.lib.sw_enable_timing(self.ctx, 1 if on else 0), "sw_enable_timing")

    def timings(self):
        """Device ms of the last surface build, raster, postprocess, upscale and whole frame."""
        t = (ctypes.c_float * 5)()
        self._check(self.lib.sw_get_timings(self.ctx, t), "sw_get_timings")
        return list(t)

    def sync(self):
        self._check(self.lib.sw_sync(self.ctx), "sw_sync")
