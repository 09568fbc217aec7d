"""Python binding of the host library (libswhost.so, C ABI in include/swhost.h): synthetic scenes and the
per-frame host work (visibility, surface preparation, draw setup) that produces the GPU path's inputs."""
import ctypes
import os

import numpy as np

from . import abi
from .gpu import PKG_DIR, SwError, load_library

HOST_LIB_PATH = os.path.join(PKG_DIR, "lib", "libswhost.so")
_lib = None


class SceneConfig(ctypes.Structure):
    _fields_ = [
        ("seed", ctypes.c_uint64), ("grid_x", ctypes.c_uint32), ("grid_y", ctypes.c_uint32),
        ("room_min", ctypes.c_float), ("room_max", ctypes.c_float), ("tile_size", ctypes.c_float),
        ("texture_size", ctypes.c_uint32), ("num_materials", ctypes.c_uint32),
        ("metal_frac", ctypes.c_float), ("dielectric_frac", ctypes.c_float),
        ("normal_maps", ctypes.c_uint32), ("directional_lightmaps", ctypes.c_uint32),
        ("lights_per_room", ctypes.c_uint32), ("num_dynamic_lights", ctypes.c_uint32),
        ("num_frames", ctypes.c_uint32), ("emissive_frac", ctypes.c_float),
        ("sky_rooms", ctypes.c_uint32), ("skybox_size", ctypes.c_uint32), ("skybox_brightness", ctypes.c_float),
        ("skybox_missing_side", ctypes.c_int32), ("sky_rotation_speed", ctypes.c_float),
        ("camera_pitch", ctypes.c_float), ("shadowed_lights", ctypes.c_uint32), ("scrolling_materials", ctypes.c_uint32),
        ("animated_materials", ctypes.c_uint32), ("projector_lights", ctypes.c_uint32), ("num_models", ctypes.c_uint32), ("model_triangles", ctypes.c_uint32),
        ("model_frames", ctypes.c_uint32), ("turb_materials", ctypes.c_uint32), ("layered_materials", ctypes.c_uint32), ("num_sprites", ctypes.c_uint32),
        ("num_decals", ctypes.c_uint32), ("water_materials", ctypes.c_uint32), ("fire_materials", ctypes.c_uint32),
        ("num_portals", ctypes.c_uint32), ("portals_depth", ctypes.c_uint32), ("light_grid", ctypes.c_uint32),
    ]


class SceneInfo(ctypes.Structure):
    _fields_ = [("nodes", ctypes.c_uint32), ("leafs", ctypes.c_uint32), ("polygons", ctypes.c_uint32),
                ("portals", ctypes.c_uint32), ("materials", ctypes.c_uint32), ("frames", ctypes.c_uint32),
                ("dynamic_lights", ctypes.c_uint32), ("reserved", ctypes.c_uint32),
                ("lightmap_elements", ctypes.c_uint64), ("texels", ctypes.c_uint64),
                ("skybox_texels", ctypes.c_uint64)]


class TextureEffectInfo(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_uint32), ("output_texture", ctypes.c_int32), ("num_layers", ctypes.c_uint32),
                ("turb", ctypes.c_float * 3)]


class TimeFunction(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_uint32), ("a", ctypes.c_float), ("b", ctypes.c_float), ("c", ctypes.c_float),
                ("d", ctypes.c_float)]


class RandomValue(ctypes.Structure):
    _fields_ = [("value", TimeFunction), ("deviation", TimeFunction)]


class SimSource(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_uint32), ("points", (ctypes.c_uint32 * 2) * 2), ("offsets", (TimeFunction * 2) * 2),
                ("frequency", ctypes.c_float), ("phase", ctypes.c_float), ("amplitude", ctypes.c_float),
                ("offset", ctypes.c_float), ("radius", ctypes.c_float), ("ramp", ctypes.c_uint32),
                ("fire_offsets", (RandomValue * 2) * 2), ("heat", RandomValue), ("angle", RandomValue),
                ("speed", RandomValue), ("gravity", RandomValue), ("spawn_angle", RandomValue),
                ("spawn_distance", RandomValue), ("lifetime", RandomValue)]


MAX_SIM_SOURCES = 8
EFFECT_WATER, EFFECT_FIRE = 3, 4


class SimEffect(ctypes.Structure):
    """SwhSimEffect: a material's water or fire effect, flattened (the oracle takes the same bytes)."""
    _fields_ = [("kind", ctypes.c_uint32), ("resolution_log2", ctypes.c_uint32 * 2), ("update_frequency", ctypes.c_float),
                ("attenuation_param", ctypes.c_float), ("color_mode", ctypes.c_uint32), ("slow", ctypes.c_uint32),
                ("has_color", ctypes.c_uint32), ("color", ctypes.c_float * 3), ("roughness", ctypes.c_float),
                ("output_texture", ctypes.c_int32), ("output_emissive", ctypes.c_int32),
                ("source_emissive", ctypes.c_int32), ("num_sources", ctypes.c_uint32), ("state_offset", ctypes.c_uint64),
                ("sources", SimSource * MAX_SIM_SOURCES)]


class FrameOptions(ctypes.Structure):
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("pixel_format", ctypes.c_uint32),
                ("use_directional_lightmaps", ctypes.c_uint32), ("clear_background", ctypes.c_uint32),
                ("fov", ctypes.c_float), ("mip_bias", ctypes.c_float), ("shadows_quality", ctypes.c_float)]


class FrameOutputs(ctypes.Structure):
    _fields_ = [("surfaces", ctypes.c_void_p), ("num_surfaces", ctypes.c_uint32), ("num_draws", ctypes.c_uint32),
                ("total_texels", ctypes.c_uint64), ("draws", ctypes.c_void_p), ("vertices", ctypes.c_void_p),
                ("num_vertices", ctypes.c_uint32), ("num_lights", ctypes.c_uint32), ("lights", ctypes.c_void_p),
                ("params", abi.FrameParams), ("visible_leafs", ctypes.c_uint32), ("camera_leaf", ctypes.c_uint32),
                ("skybox_draws", ctypes.c_uint32), ("light_shadows", ctypes.c_void_p), ("depth_draws", ctypes.c_void_p),
                ("num_depth_draws", ctypes.c_uint32), ("num_depth_vertices", ctypes.c_uint32),
                ("depth_vertices", ctypes.c_void_p), ("shadow_texels", ctypes.c_uint64),
                ("shadow_sides", ctypes.c_void_p), ("num_shadow_sides", ctypes.c_uint32),
                ("num_shadow_leafs", ctypes.c_uint32), ("shadow_leafs", ctypes.c_void_p),
                ("tri_vertices", ctypes.c_void_p), ("num_tri_vertices", ctypes.c_uint32),
                ("model_triangles", ctypes.c_uint32), ("texture_passes", ctypes.c_void_p),
                ("num_texture_passes", ctypes.c_uint32), ("num_texture_shifts", ctypes.c_uint32),
                ("texture_shifts", ctypes.c_void_p), ("sim_passes", ctypes.c_void_p),
                ("num_sim_passes", ctypes.c_uint32), ("num_sim_points", ctypes.c_uint32), ("sim_points", ctypes.c_void_p),
                ("views", ctypes.c_void_p), ("num_views", ctypes.c_uint32), ("main_draws", ctypes.c_uint32),
                ("surface_texels", ctypes.c_uint64)]


def load_host_library():
    global _lib
    if _lib is not None:
        return _lib
    load_library()  # libswgpu.so first (dependency)
    if not os.path.exists(HOST_LIB_PATH):
        raise SwError(f"{HOST_LIB_PATH} is missing: build it with `python square-wheel_gb300/build.py`")
    lib = ctypes.CDLL(HOST_LIB_PATH)
    vp, u32, i32 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int
    sig = {
        "swh_scene_create": ([vp, ctypes.POINTER(vp)], i32), "swh_scene_destroy": ([vp], i32),
        "swh_scene_info": ([vp, vp], i32), "swh_scene_create_info": ([vp, u32, vp], i32),
        "swh_last_error": ([], ctypes.c_char_p), "swh_frame_create": ([vp, ctypes.POINTER(vp)], i32),
        "swh_frame_destroy": ([vp], i32), "swh_frame_prepare": ([vp, u32, vp], i32),
        "swh_frame_outputs": ([vp, vp], i32), "swh_renderer_create": ([vp, u32, ctypes.POINTER(vp)], i32),
        "swh_renderer_destroy": ([vp], i32), "swh_renderer_prepare_frame": ([vp, u32, vp], i32),
        "swh_renderer_draw_frame": ([vp, vp, u32, i32], i32), "swh_renderer_context": ([vp], vp),
        "swh_renderer_frame": ([vp], vp),
        "swh_scene_skybox": ([vp, ctypes.POINTER(vp), ctypes.POINTER(vp), ctypes.POINTER(ctypes.c_uint64), vp, vp], i32),
        "swh_renderer_render_frame": ([vp, u32, vp, vp, ctypes.c_float, vp, vp, u32, i32], i32),
        "swh_frame_prepare_view": ([vp, u32, vp], i32), "swh_frame_view_input": ([vp, vp], i32),
        "swh_renderer_set_gpu_prep": ([vp, i32], i32),
        "swh_renderer_set_frames_in_flight": ([vp, u32], i32),
        "swh_scene_lite_textures": ([vp, ctypes.POINTER(vp), ctypes.POINTER(ctypes.c_uint64)], i32),
        "swh_frame_map": ([vp, ctypes.POINTER(vp), ctypes.POINTER(u32), ctypes.POINTER(vp), ctypes.POINTER(u32)], i32),
        "swh_scene_load_map": ([ctypes.c_char_p, vp, ctypes.POINTER(vp)], i32),
        "swh_scene_load_map_memory": ([vp, ctypes.c_uint64, vp, ctypes.POINTER(vp)], i32),
        "swh_scene_save_map": ([vp, ctypes.c_char_p], i32),
        "swh_scene_texture_effect": ([vp, u32, vp], i32),
        "swh_scene_simulated_effect": ([vp, u32, vp], i32),
        "swh_scene_simulation_words": ([vp, ctypes.POINTER(ctypes.c_uint64)], i32),
        "swh_scene_light_grid": ([vp, vp, vp, vp, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)], i32),
        "swh_scene_fetch_light": ([vp, vp, vp], i32),
        "swh_frame_effect_state": ([vp, u32, ctypes.POINTER(u32), ctypes.POINTER(u32), ctypes.POINTER(u32),
                                    ctypes.POINTER(u32)], i32),
        "swh_scene_compressed_lightmaps": ([vp, ctypes.POINTER(vp), ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(vp),
                                            ctypes.POINTER(ctypes.c_uint64)], i32),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


HOST_EXPORTED = ["swh_scene_create", "swh_scene_destroy", "swh_scene_info", "swh_scene_create_info", "swh_last_error",
                 "swh_frame_create", "swh_frame_destroy", "swh_frame_prepare", "swh_frame_outputs",
                 "swh_renderer_create", "swh_renderer_destroy", "swh_renderer_prepare_frame",
                 "swh_renderer_draw_frame", "swh_renderer_context", "swh_renderer_frame", "swh_scene_skybox",
                 "swh_renderer_render_frame", "swh_frame_prepare_view", "swh_frame_view_input",
                 "swh_renderer_set_gpu_prep", "swh_frame_map", "swh_renderer_set_frames_in_flight",
                 "swh_scene_lite_textures", "swh_scene_load_map", "swh_scene_load_map_memory", "swh_scene_save_map",
                 "swh_scene_compressed_lightmaps", "swh_scene_texture_effect", "swh_scene_simulated_effect",
                 "swh_scene_simulation_words", "swh_frame_effect_state", "swh_scene_light_grid", "swh_scene_fetch_light"]

# The two map configurations of the benchmark plan.
SMALL_MAP = dict(seed=1, grid_x=4, grid_y=2, tile_size=128.0, texture_size=128, num_materials=16, metal_frac=0.0,
                 dielectric_frac=0.0, normal_maps=0, directional_lightmaps=0, lights_per_room=1,
                 num_dynamic_lights=0, num_frames=64)
FULL_MAP = dict(seed=2, grid_x=8, grid_y=8, tile_size=80.0, texture_size=256, num_materials=32, metal_frac=0.25,
                dielectric_frac=0.25, normal_maps=1, directional_lightmaps=1, lights_per_room=2,
                num_dynamic_lights=8, num_frames=256)
# The full-size map with triangle models: 200 per-vertex animated models of about 2k triangles and 8
# keyframes each on the rooms' floors (the stress configuration's models).
MODEL_MAP = dict(FULL_MAP, num_models=200, model_triangles=2000, model_frames=8)
# The stress configuration's map: 128 rooms (16 x 8) of the full-size configuration with portals
# (mirrors, cameras, parallax windows; two nested levels), translucent (averaging animated frames),
# alpha-blended and alpha-tested (layered) surfaces, 2k decals, sprites and the 200 models, all lit from
# a seeded light grid.
STRESS_MAP = dict(FULL_MAP, seed=5, grid_x=16, grid_y=8, num_models=200, model_triangles=2000, model_frames=8,
                  num_decals=2000, num_sprites=64, num_portals=12, portals_depth=2, light_grid=1,
                  layered_materials=4, animated_materials=4)
# The small map with a sky: three rooms open to a skybox (the sky material's six 128x128 sides, HDR
# brightness 2, rotating slowly), the camera looking 0.45 rad up so ceilings are in view.
SKY_MAP = dict(SMALL_MAP, sky_rooms=3, skybox_size=128, skybox_brightness=2.0, sky_rotation_speed=0.01,
               camera_pitch=0.45)


def _check(lib, r, what):
    if r != 0:
        msg = lib.swh_last_error()
        raise SwError(f"{what} failed ({r}): {msg.decode() if msg else ''}")


class Scene:
    def __init__(self, _map=None, **kw):
        """A generated scene (keyword arguments: SceneConfig fields), or with _map (a path or the bytes of a
        compiled .sqwm map) the scene swh_scene_load_map makes of that map."""
        self.lib = load_host_library()
        c = SceneConfig(seed=1, grid_x=4, grid_y=2, room_min=256.0, room_max=1024.0, tile_size=128.0, texture_size=128,
                        num_materials=16, metal_frac=0.0, dielectric_frac=0.0, normal_maps=0, directional_lightmaps=0,
                        lights_per_room=1, num_dynamic_lights=0, num_frames=64, emissive_frac=0.0, sky_rooms=0,
                        skybox_size=128, skybox_brightness=1.0, skybox_missing_side=-1, sky_rotation_speed=0.01,
                        camera_pitch=0.0, shadowed_lights=0, scrolling_materials=0,
                        animated_materials=0, projector_lights=0, num_models=0, model_triangles=2000, model_frames=8)
        for k, v in kw.items():
            setattr(c, k, v)
        self.config = c
        self.handle = ctypes.c_void_p()
        if _map is None:
            _check(self.lib, self.lib.swh_scene_create(ctypes.byref(c), ctypes.byref(self.handle)), "swh_scene_create")
        elif isinstance(_map, (bytes, bytearray)):
            buf = ctypes.create_string_buffer(bytes(_map), len(_map))
            _check(self.lib, self.lib.swh_scene_load_map_memory(buf, len(_map), ctypes.byref(c), ctypes.byref(self.handle)),
                   "swh_scene_load_map_memory")
        else:
            _check(self.lib, self.lib.swh_scene_load_map(os.fsencode(_map), ctypes.byref(c), ctypes.byref(self.handle)),
                   "swh_scene_load_map")

    @classmethod
    def load_map(cls, path_or_bytes, **kw):
        return cls(_map=path_or_bytes, **kw)

    def texture_effect(self, material):
        """(kind, output_texture, num_layers, (amplitude, wave_length, frequency)) of a material's generative
        texture effect (kind 0 none, 1 turbulence, 2 layered)."""
        e = TextureEffectInfo()
        _check(self.lib, self.lib.swh_scene_texture_effect(self.handle, material, ctypes.byref(e)), "swh_scene_texture_effect")
        return int(e.kind), int(e.output_texture), int(e.num_layers), tuple(e.turb)

    def simulated_effect(self, material):
        """The material's water / fire effect as a SimEffect (kind 0 for other materials)."""
        e = SimEffect()
        _check(self.lib, self.lib.swh_scene_simulated_effect(self.handle, material, ctypes.byref(e)),
               "swh_scene_simulated_effect")
        return e

    def simulation_words(self):
        n = ctypes.c_uint64()
        _check(self.lib, self.lib.swh_scene_simulation_words(self.handle, ctypes.byref(n)), "swh_scene_simulation_words")
        return int(n.value)

    def light_grid(self):
        """(header: cell size, start and size arrays; columns (n, 3) u32; samples (m, 24) f32)."""
        nc, ns = ctypes.c_uint64(), ctypes.c_uint64()
        _check(self.lib, self.lib.swh_scene_light_grid(self.handle, None, None, None, ctypes.byref(nc), ctypes.byref(ns)),
               "swh_scene_light_grid")
        hdr = np.zeros(9, np.float32)
        cols = np.zeros((nc.value, 3), np.uint32)
        samples = np.zeros((ns.value, 24), np.float32)
        _check(self.lib, self.lib.swh_scene_light_grid(self.handle, hdr.ctypes.data, cols.ctypes.data, samples.ctypes.data,
                                                       ctypes.byref(nc), ctypes.byref(ns)), "swh_scene_light_grid")
        header = dict(cell_size=hdr[0:3].copy(), start=hdr[3:6].copy(), size=hdr[6:9].view(np.uint32).copy())
        return header, cols, samples

    def fetch_light(self, pos):
        p = np.asarray(pos, np.float32)
        out = np.zeros(24, np.float32)
        _check(self.lib, self.lib.swh_scene_fetch_light(self.handle, p.ctypes.data, out.ctypes.data), "swh_scene_fetch_light")
        return out

    def save_map(self, path):
        _check(self.lib, self.lib.swh_scene_save_map(self.handle, os.fsencode(path)), "swh_scene_save_map")

    def compressed_lightmaps(self):
        """(simple, directional) compressed lightmap records of a loaded map as uint8 arrays of shape (n, 4)
        and (n, 13); empty for generated scenes."""
        p, n, pd, nd = ctypes.c_void_p(), ctypes.c_uint64(), ctypes.c_void_p(), ctypes.c_uint64()
        _check(self.lib, self.lib.swh_scene_compressed_lightmaps(self.handle, ctypes.byref(p), ctypes.byref(n),
                                                                 ctypes.byref(pd), ctypes.byref(nd)),
               "swh_scene_compressed_lightmaps")

        def arr(ptr, count, width):
            if not ptr.value or count.value == 0:
                return np.zeros((0, width), np.uint8)
            return np.ctypeslib.as_array(ctypes.cast(ptr, ctypes.POINTER(ctypes.c_uint8)),
                                         shape=(int(count.value) * width,)).copy().reshape(-1, width)
        return arr(p, n, 4), arr(pd, nd, 13)

    def info(self):
        i = SceneInfo()
        _check(self.lib, self.lib.swh_scene_info(self.handle, ctypes.byref(i)), "swh_scene_info")
        return i

    def create_info(self, device=0):
        ci = abi.CreateInfo()
        _check(self.lib, self.lib.swh_scene_create_info(self.handle, device, ctypes.byref(ci)), "swh_scene_create_info")
        return ci

    def skybox(self):
        """(texels32, texels64, mip_offsets[6, 5], mip_sizes[6, 5]) numpy copies; empty arrays without sky."""
        t32, t64, n = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_uint64()
        offs = np.zeros(30, np.uint64)
        sizes = np.zeros(30, np.uint32)
        _check(self.lib, self.lib.swh_scene_skybox(self.handle, ctypes.byref(t32), ctypes.byref(t64), ctypes.byref(n),
                                                   abi.ptr(offs), abi.ptr(sizes)), "swh_scene_skybox")
        count = int(n.value)

        def arr(p, dt):
            if not p.value or count == 0:
                return np.zeros(0, dt)
            return np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(ctypes.c_uint8)),
                                         shape=(count * np.dtype(dt).itemsize,)).view(dt).copy()
        return arr(t32, np.uint32), arr(t64, np.uint64), offs.reshape(6, 5), sizes.reshape(6, 5)

    def lite_textures(self):
        """The models' Color32 skins with their mips (one uint32 array, sw_set_lite_textures)."""
        p, n = ctypes.c_void_p(), ctypes.c_uint64()
        _check(self.lib, self.lib.swh_scene_lite_textures(self.handle, ctypes.byref(p), ctypes.byref(n)),
               "swh_scene_lite_textures")
        if not p.value or n.value == 0:
            return np.zeros(0, np.uint32)
        return np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(ctypes.c_uint32)), shape=(int(n.value),)).copy()

    def static_data(self):
        """numpy copies of the static data (for the oracle and GpuRenderer)."""
        from .gpu import StaticData
        ci = self.create_info()

        def arr(p, n, dt):
            if not p or n == 0:
                return np.zeros(0, dt)
            return np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(ctypes.c_uint8)),
                                         shape=(int(n) * np.dtype(dt).itemsize,)).view(dt).copy()
        return StaticData(arr(ci.texels, ci.num_texels, np.uint64), arr(ci.texture_mips, ci.num_texture_mips, abi.TEXTURE_MIP),
                          arr(ci.emissive_pixels, ci.num_emissive_pixels, np.uint32),
                          arr(ci.emissive_mips, ci.num_emissive_mips, abi.EMISSIVE_MIP),
                          arr(ci.lightmaps, ci.num_lightmap_elements * 3, np.float32),
                          arr(ci.directional_lightmaps, ci.num_directional_lightmap_elements, abi.DIR_LIGHTMAP_ELEMENT))

    def close(self):
        if self.handle:
            self.lib.swh_scene_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def frame_options(width, height, pixel_format, directional=True, clear_background=False, fov=0.0, mip_bias=0.0,
                  shadows_quality=0.0):
    return FrameOptions(width, height, pixel_format, 1 if directional else 0, 1 if clear_background else 0, fov, mip_bias,
                        shadows_quality)


class Frame:
    """Per-frame host work; outputs are copied into numpy arrays."""

    def __init__(self, scene):
        self.scene = scene
        self.lib = scene.lib
        self.handle = ctypes.c_void_p()
        _check(self.lib, self.lib.swh_frame_create(scene.handle, ctypes.byref(self.handle)), "swh_frame_create")

    def prepare(self, frame_index, options):
        _check(self.lib, self.lib.swh_frame_prepare(self.handle, frame_index, ctypes.byref(options)), "swh_frame_prepare")
        return self._outputs()

    def effect_state(self, material):
        """(update_step, current_buffer, generated, particles) of a simulated effect after the last prepared frame."""
        v = [ctypes.c_uint32() for _ in range(4)]
        _check(self.lib, self.lib.swh_frame_effect_state(self.handle, material, *[ctypes.byref(x) for x in v]),
               "swh_frame_effect_state")
        return tuple(int(x.value) for x in v)

    def map_data(self):
        """Copies of the map's world polygons (abi.MAP_POLYGON) and vertices (float32, n x 3) as sw_set_map
        takes them."""
        pp, vp_ = ctypes.c_void_p(), ctypes.c_void_p()
        n, nv = ctypes.c_uint32(), ctypes.c_uint32()
        _check(self.lib, self.lib.swh_frame_map(self.handle, ctypes.byref(pp), ctypes.byref(n), ctypes.byref(vp_),
                                                ctypes.byref(nv)), "swh_frame_map")
        polys = np.ctypeslib.as_array(ctypes.cast(pp, ctypes.POINTER(ctypes.c_uint8)),
                                      shape=(n.value * abi.MAP_POLYGON.itemsize,)).view(abi.MAP_POLYGON).copy()
        verts = np.ctypeslib.as_array(ctypes.cast(vp_, ctypes.POINTER(ctypes.c_float)), shape=(nv.value * 3,)).copy()
        return polys, verts.reshape(-1, 3)

    def _outputs(self):
        o = FrameOutputs()
        _check(self.lib, self.lib.swh_frame_outputs(self.handle, ctypes.byref(o)), "swh_frame_outputs")

        def arr(p, n, dt):
            if not p or n == 0:
                return np.zeros(0, dt)
            return np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(ctypes.c_uint8)),
                                         shape=(int(n) * np.dtype(dt).itemsize,)).view(dt).copy()
        self.surfaces = arr(o.surfaces, o.num_surfaces, abi.SURFACE_DESC)
        self.draws = arr(o.draws, o.num_draws, abi.DRAW_CMD)
        self.vertices = arr(o.vertices, o.num_vertices, abi.VERTEX16)
        self.tri_vertices = arr(o.tri_vertices, o.num_tri_vertices, abi.TRI_VERTEX)
        self.model_triangles = int(o.model_triangles)
        self.texture_passes = arr(o.texture_passes, o.num_texture_passes, abi.TEXTURE_PASS)
        self.texture_shifts = arr(o.texture_shifts, o.num_texture_shifts, np.int32)
        self.sim_passes = arr(o.sim_passes, o.num_sim_passes, abi.SIM_PASS)
        self.sim_points = arr(o.sim_points, o.num_sim_points, abi.SIM_POINT)
        self.views = arr(o.views, o.num_views, abi.VIEW)
        self.main_draws = int(o.main_draws) if o.num_views else int(o.num_draws)
        self.surface_texels = int(o.surface_texels)
        self.lights = arr(o.lights, o.num_lights, abi.LIGHT)
        self.total_texels = int(o.total_texels)
        self.params = abi.FrameParams()
        ctypes.pointer(self.params)[0] = o.params
        self.visible_leafs = int(o.visible_leafs)
        self.camera_leaf = int(o.camera_leaf)
        self.skybox_draws = int(o.skybox_draws)
        self.light_shadows = arr(o.light_shadows, o.num_lights, abi.LIGHT_SHADOW)
        self.depth_draws = arr(o.depth_draws, o.num_depth_draws, abi.DEPTH_DRAW)
        self.depth_vertices = arr(o.depth_vertices, o.num_depth_vertices, abi.VERTEX16)
        self.shadow_texels = int(o.shadow_texels)
        self.shadow_sides = arr(o.shadow_sides, o.num_shadow_sides, abi.SHADOW_SIDE)
        self.shadow_leafs = arr(o.shadow_leafs, o.num_shadow_leafs, abi.SHADOW_LEAF)
        return self

    def prepare_view(self, frame_index, options):
        """Host half of a GPU-prepared frame: returns its SwViewFrameInput (pointers into this frame) and
        copies of the visible leafs and their light lists."""
        _check(self.lib, self.lib.swh_frame_prepare_view(self.handle, frame_index, ctypes.byref(options)),
               "swh_frame_prepare_view")
        vin = abi.ViewFrameInput()
        _check(self.lib, self.lib.swh_frame_view_input(self.handle, ctypes.byref(vin)), "swh_frame_view_input")

        def arr(p, n, dt):
            if not p or n == 0:
                return np.zeros(0, dt)
            return np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(ctypes.c_uint8)),
                                         shape=(int(n) * np.dtype(dt).itemsize,)).view(dt).copy()
        self._outputs()  # lights, shadow maps and their sides' leafs
        self.view_leafs = arr(vin.leafs, vin.num_leafs, abi.VIEW_LEAF)
        self.view_leaf_lights = arr(vin.leaf_lights, vin.num_leaf_lights, np.uint16)
        self.draws = arr(vin.draws, vin.num_draws, abi.DRAW_CMD)
        self.vertices = arr(vin.vertices, vin.num_vertices, abi.VERTEX16)
        return vin

    def close(self):
        if self.handle:
            self.lib.swh_frame_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class HostRenderer:
    """Renderer API mirror driving the GPU library from C++ (swh_renderer_*)."""

    def __init__(self, scene, device=0):
        self.scene = scene
        self.lib = scene.lib
        self.handle = ctypes.c_void_p()
        _check(self.lib, self.lib.swh_renderer_create(scene.handle, device, ctypes.byref(self.handle)), "swh_renderer_create")

    def _err(self, r, what):
        if r != 0:
            glib = load_library()
            ctx = self.lib.swh_renderer_context(self.handle)
            msg = glib.sw_last_error(ctx) if ctx else b""
            raise SwError(f"{what} failed ({r}): {msg.decode() if msg else ''}")

    def prepare_frame(self, frame_index, options):
        self._err(self.lib.swh_renderer_prepare_frame(self.handle, frame_index, ctypes.byref(options)), "prepare_frame")

    def draw_frame(self, out=None, device_ptr=None, pitch=None):
        if out is not None:
            self._err(self.lib.swh_renderer_draw_frame(self.handle, abi.ptr(out), pitch or out.shape[1], 0), "draw_frame")
        elif device_ptr is not None:
            self._err(self.lib.swh_renderer_draw_frame(self.handle, ctypes.c_void_p(device_ptr), pitch, 1), "draw_frame")
        else:
            self._err(self.lib.swh_renderer_draw_frame(self.handle, None, 0, 0), "draw_frame")

    def render_frame(self, frame_index, options, out=None, device_ptr=None, pitch=None, post=None,
                     frame_duration_s=1.0 / 60.0, color_modulate=(1.0, 1.0, 1.0)):
        """Host work + the whole frame as one graph (sw_draw_frame); with `post` (an abi.PostConfig) the
        Color32 result, else the frame, lands in `out` (host) or at device_ptr."""
        mod = (ctypes.c_float * 3)(*[float(c) for c in color_modulate])
        post_p = ctypes.byref(post) if post is not None else None
        if out is not None:
            dst, pitch, dev = abi.ptr(out), pitch or out.shape[1], 0
        elif device_ptr is not None:
            dst, dev = ctypes.c_void_p(device_ptr), 1
        else:
            dst, pitch, dev = None, 0, 0
        self._err(self.lib.swh_renderer_render_frame(self.handle, frame_index, ctypes.byref(options), post_p,
                                                     frame_duration_s, mod, dst, pitch or 0, dev), "render_frame")

    def set_frames_in_flight(self, frames):
        """2: render_frame returns once its frame is enqueued and the previous frame is in its buffer."""
        self._err(self.lib.swh_renderer_set_frames_in_flight(self.handle, int(frames)), "set_frames_in_flight")

    def sync(self):
        """Wait until every frame in flight is in its buffer."""
        self._err(load_library().sw_sync(self.context()), "sync")

    def set_gpu_prep(self, enable):
        """render_frame's preparation: True = on the GPU (default), False = on the host."""
        self._err(self.lib.swh_renderer_set_gpu_prep(self.handle, 1 if enable else 0), "set_gpu_prep")

    def read_view_prep(self, max_surfaces=1 << 16, max_draws=1 << 16, max_vertices=1 << 20):
        """Counts, surface descriptors, draws and vertices of the last GPU-prepared frame (synchronises)."""
        glib = load_library()
        k = abi.ViewCounts()
        s = np.zeros(max_surfaces, abi.SURFACE_DESC)
        d = np.zeros(max_draws, abi.DRAW_CMD)
        v = np.zeros(max_vertices, abi.VERTEX16)
        self._err(glib.sw_read_view_prep(self.context(), ctypes.byref(k), abi.ptr(s), max_surfaces, abi.ptr(d), max_draws,
                                         abi.ptr(v), max_vertices), "read_view_prep")
        return k, s[:k.num_surfaces].copy(), d[:k.num_draws].copy(), v[:k.num_vertices].copy()

    def register_host_buffer(self, arr):
        """Page-lock `arr` (reused for frames) so frames are copied straight into it."""
        self._err(load_library().sw_register_host_buffer(self.context(), abi.ptr(arr), arr.nbytes), "register")

    def unregister_host_buffer(self, arr):
        self._err(load_library().sw_unregister_host_buffer(self.context(), abi.ptr(arr)), "unregister")

    def context(self):
        return self.lib.swh_renderer_context(self.handle)

    def close(self):
        if self.handle:
            self.lib.swh_renderer_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
