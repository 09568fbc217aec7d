"""numpy / ctypes mirrors of the structs in include/swgpu.h.

Arrays of descriptors are numpy structured arrays (aligned like the C structs) so that they can be
handed to the C ABI by pointer; single parameter blocks are ctypes Structures.
"""
import ctypes

import numpy as np

SWGPU_ABI_VERSION = 2

SW_OK = 0
SW_ERR_INVALID_ARGUMENT = -1
SW_ERR_OUT_OF_MEMORY = -2
SW_ERR_CUDA = -3
SW_ERR_LIMIT = -4
SW_ERR_NO_DEVICE = -5
SW_ERR_STATE = -6

SW_PIXEL_C32 = 0
SW_PIXEL_C64 = 1

SW_BLEND_NONE, SW_BLEND_AVERAGE, SW_BLEND_ADDITIVE, SW_BLEND_ALPHA_TEST, SW_BLEND_ALPHA_BLEND = range(5)
SW_RASTER_FULL_PERSPECTIVE, SW_RASTER_LINE_Z_CORRECTED, SW_RASTER_AFFINE, SW_RASTER_TRIANGLE = range(4)
SW_TEXSRC_SURFACE, SW_TEXSRC_SKYBOX, SW_TEXSRC_LITE = range(3)
SW_UPSCALE_NEAREST, SW_UPSCALE_AVG2X, SW_UPSCALE_LEARNED = range(3)

SW_TEX_HAS_NORMAL_MAP = 1
SW_TEX_HAS_NON_ONE_ROUGHNESS = 2
SW_TEX_IS_METAL = 4

SW_MAX_POLYGON_LIGHTS = 6
SW_MAX_POLYGON_VERTICES = 24
SW_NO_LIGHTMAP = 0
SW_NO_EMISSIVE = 0xFFFFFFFF
SW_SURF_DIFFUSE_LAYER = 1
SW_POLY_DRAW, SW_POLY_SKY, SW_POLY_DIFFUSE_LAYER, SW_POLY_SHADOW = 1, 2, 4, 8
SW_LEAF_NOT_DRAWN = 0xFFFFFFFF
SW_SHADOW_NONE, SW_SHADOW_CUBE, SW_SHADOW_PROJECTOR = 0, 1, 2

TEXTURE_MIP = np.dtype([("offset", "<u8"), ("width", "<u4"), ("height", "<u4"), ("flags", "<u4"), ("reserved", "<u4")], align=True)
EMISSIVE_MIP = np.dtype([("offset", "<u8"), ("width", "<u4"), ("height", "<u4")], align=True)
DIR_LIGHTMAP_ELEMENT = np.dtype(
    [("ambient_light", "<f4", 3), ("light_direction_vector_scaled", "<f4", 3), ("directional_light_deviation", "<f4"),
     ("directional_light_color", "<f4", 3)], align=True)
LIGHT = np.dtype([("position", "<f4", 3), ("radius", "<f4"), ("inv_square_radius", "<f4"), ("color", "<f4", 3)], align=True)
SURFACE_DESC = np.dtype([
    ("basis_u", "<f4", 3), ("basis_v", "<f4", 3), ("basis_start", "<f4", 3), ("basis_normal", "<f4", 3),
    ("size", "<u4", 2), ("tc_start", "<i4", 2), ("texture_mip", "<u4"), ("emissive_mip", "<u4"),
    ("lightmap_offset", "<u4"), ("lightmap_size", "<u4", 2), ("lightmap_scale_log2", "<u4"),
    ("lightmap_tc_shift", "<u4", 2), ("flags", "<u4"), ("num_lights", "<u4"), ("lights", "<u2", 6),
    ("emissive_light", "<f4", 3), ("out_offset", "<u8")], align=True)
VERTEX16 = np.dtype([("x", "<i4"), ("y", "<i4")], align=True)
TEXTURE_PASS = np.dtype([("kind", "<u4"), ("dst_mip", "<u4"), ("src_mip", "<u4"), ("blending_mode", "<u4"),
                         ("shift", "<i4", 2), ("light", "<f4", 3), ("shifts_offset", "<u4")], align=True)
SW_TEXPASS_TURB, SW_TEXPASS_LAYER, SW_TEXPASS_EMISSIVE = 1, 2, 0x100
# SwView: a nested view of a whole frame (a portal's texture rendered before the frame's own draws)
VIEW = np.dtype([("target_offset", "<u8"), ("width", "<u4"), ("height", "<u4"), ("first_draw", "<u4"),
                 ("num_draws", "<u4"), ("clear_background", "<u4"), ("mix_blend", "<u4"), ("mix_offset", "<u8"),
                 ("mix_size", "<u4", 2), ("mix_tc_min", "<i4", 2), ("mix_light", "<f4", 3), ("reserved", "<u4")])
SW_VIEW_NO_MIX = 0xFFFFFFFF
# SwSimPass / SwSimPoint (sw_update_simulations): simulated water and fire effects
SIM_PASS = np.dtype([("kind", "<u4"), ("launch", "<u4"), ("size_log2", "<u4", 2), ("state_src", "<u8"),
                     ("state_dst", "<u8"), ("first_point", "<u4"), ("num_points", "<u4"), ("dst_mip", "<u4"),
                     ("src_mip", "<u4"), ("flags", "<u4"), ("param", "<u4"), ("base_color", "<u4"), ("reserved", "<u4")])
SIM_POINT = np.dtype([("address", "<u4"), ("value", "<u4")])
(SW_SIM_WATER_POINTS, SW_SIM_WATER_STEP, SW_SIM_FIRE_STEP, SW_SIM_FIRE_POINTS, SW_SIM_WATER_TEXTURE,
 SW_SIM_FIRE_TEXTURE, SW_SIM_TEXTURE_MIP, SW_SIM_EMISSIVE_MIP) = range(1, 9)
SW_SIM_FIRE_SLOW, SW_SIM_WATER_INIT_DIFFUSE, SW_SIM_COLOR_MODE_SHIFT = 1, 2, 8
TRI_VERTEX = np.dtype([("x", "<i4"), ("y", "<i4"), ("tc", "<i4", 2), ("light", "<i4", 3), ("reserved", "<i4")], align=True)
DRAW_CMD = np.dtype([
    ("first_vertex", "<u4"), ("vertex_count", "<u4"), ("mode", "<u4"), ("blend", "<u4"), ("depth_eq", "<f4", 3),
    ("tc_eq", "<f4", 6), ("tex_size", "<u4", 2), ("tex_source", "<u4"), ("tex_offset", "<u8")], align=True)

MAP_POLYGON = np.dtype([
    ("plane", "<f4", 4), ("tex_coord_equation", "<f4", (2, 4)), ("basis_u", "<f4", 3), ("basis_v", "<f4", 3),
    ("basis_start", "<f4", 3), ("basis_normal", "<f4", 3), ("tex_coord_min", "<i4", 2), ("tex_coord_max", "<i4", 2),
    ("first_vertex", "<u4"), ("num_vertices", "<u4"), ("texture", "<u4"), ("lightmap_data_offset", "<u4"),
    ("flags", "<u4"), ("blending_mode", "<u4"), ("emissive_texture", "<u4"), ("emissive_light", "<f4", 3)], align=True)
LIGHT_SHADOW = np.dtype([("kind", "<u4"), ("size", "<u4"), ("offset", "<u8"), ("basis_x", "<f4", 3), ("basis_y", "<f4", 3),
                         ("basis_z", "<f4", 3), ("reserved", "<u4")], align=True)
DEPTH_DRAW = np.dtype([("first_vertex", "<u4"), ("vertex_count", "<u4"), ("map_size", "<u4"), ("reserved", "<u4"),
                       ("map_offset", "<u8"), ("depth_eq", "<f4", 3), ("reserved2", "<u4")], align=True)
MATERIAL_FRAME = np.dtype([("shift", "<i4", 2), ("texture", "<u4"), ("flags", "<u4"), ("blending_mode", "<u4"),
                           ("emissive_texture", "<u4"), ("emissive_light", "<f4", 3), ("reserved", "<u4")], align=True)
SHADOW_SIDE = np.dtype([("view_matrix", "<f4", 16), ("planes_matrix", "<f4", 16), ("map_size", "<u4"),
                        ("reserved", "<u4"), ("map_offset", "<u8")], align=True)
SHADOW_LEAF = np.dtype([("side", "<u4"), ("first_polygon", "<u4"), ("num_polygons", "<u4"), ("reserved", "<u4"),
                        ("clip_planes", "<f4", (8, 3))], align=True)
VIEW_LEAF = np.dtype([
    ("first_polygon", "<u4"), ("num_polygons", "<u4"), ("first_light", "<u4"), ("num_lights", "<u4"),
    ("draw_order", "<u4"), ("reserved", "<u4"), ("clip_planes", "<f4", (8, 3)), ("draw_clip_planes", "<f4", (8, 3))],
    align=True)


class CreateInfo(ctypes.Structure):
    _fields_ = [
        ("abi_version", ctypes.c_uint32), ("device", ctypes.c_uint32),
        ("texels", ctypes.c_void_p), ("num_texels", ctypes.c_uint64),
        ("texture_mips", ctypes.c_void_p), ("num_texture_mips", ctypes.c_uint32), ("num_emissive_mips", ctypes.c_uint32),
        ("emissive_pixels", ctypes.c_void_p), ("num_emissive_pixels", ctypes.c_uint64), ("emissive_mips", ctypes.c_void_p),
        ("lightmaps", ctypes.c_void_p), ("num_lightmap_elements", ctypes.c_uint64),
        ("directional_lightmaps", ctypes.c_void_p), ("num_directional_lightmap_elements", ctypes.c_uint64),
        ("max_surface_texels", ctypes.c_uint64), ("max_surfaces", ctypes.c_uint32), ("max_draws", ctypes.c_uint32),
    ]


class FrameParams(ctypes.Structure):
    _fields_ = [
        ("pixel_format", ctypes.c_uint32), ("width", ctypes.c_uint32), ("height", ctypes.c_uint32),
        ("use_directional_lightmaps", ctypes.c_uint32), ("cam_pos", ctypes.c_float * 3),
        ("clear_background", ctypes.c_uint32), ("reserved", ctypes.c_uint32),
    ]


class PostConfig(ctypes.Structure):
    """PostprocessorConfig after synchronize_config clamping (postprocessor.rs:958-977)."""
    _fields_ = [
        ("exposure_update_speed", ctypes.c_float), ("base_brightness", ctypes.c_float),
        ("zero_level_brightness", ctypes.c_float), ("brightness_scale_power", ctypes.c_float),
        ("min_exposure", ctypes.c_float), ("max_exposure", ctypes.c_float), ("bloom_sigma", ctypes.c_float),
        ("bloom_buffer_scale_log2", ctypes.c_uint32), ("bloom_scale", ctypes.c_float),
        ("linear_bloom_filter", ctypes.c_uint32),
    ]

    @classmethod
    def default(cls):
        """Defaults of postprocessor_config.rs:13-41 (bloom on, sigma 1, scale log2 1)."""
        return cls(1.0, 1.0, 1.0, 0.25, 1.0 / 65536.0, 128.0, 1.0, 1, 0.25, 0)


class Stats(ctypes.Structure):
    _fields_ = [("surfaces", ctypes.c_uint64), ("surface_texels", ctypes.c_uint64), ("draws", ctypes.c_uint64),
                ("bad_texel_fetches", ctypes.c_uint64), ("pixel_writes", ctypes.c_uint64),
                ("upload_bytes", ctypes.c_uint64)]


# Order reported by sw_abi_layout.
class FrameInput(ctypes.Structure):
    """SwFrameInput: one whole frame for sw_draw_frame."""
    _fields_ = [("params", FrameParams), ("num_lights", ctypes.c_uint32), ("lights", ctypes.c_void_p),
                ("surfaces", ctypes.c_void_p), ("total_texels", ctypes.c_uint64), ("num_surfaces", ctypes.c_uint32),
                ("num_draws", ctypes.c_uint32), ("draws", ctypes.c_void_p), ("vertices", ctypes.c_void_p),
                ("num_vertices", ctypes.c_uint32), ("postprocess", ctypes.c_uint32), ("post", PostConfig),
                ("frame_duration_s", ctypes.c_float), ("color_modulate", ctypes.c_float * 3), ("dst", ctypes.c_void_p),
                ("dst_pitch", ctypes.c_uint32), ("dst_is_device", ctypes.c_int32), ("tri_vertices", ctypes.c_void_p),
                ("num_tri_vertices", ctypes.c_uint32), ("num_views", ctypes.c_uint32), ("views", ctypes.c_void_p),
                ("main_draws", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]


class ViewFrameInput(ctypes.Structure):
    """SwViewFrameInput: one whole frame for sw_draw_frame_view (GPU-side surface and draw preparation)."""
    _fields_ = [("params", FrameParams), ("num_lights", ctypes.c_uint32), ("lights", ctypes.c_void_p),
                ("view_matrix", ctypes.c_float * 16), ("planes_matrix", ctypes.c_float * 16), ("mip_bias", ctypes.c_float),
                ("num_leafs", ctypes.c_uint32), ("leafs", ctypes.c_void_p), ("num_leaf_lights", ctypes.c_uint32),
                ("leaf_lights", ctypes.c_void_p), ("num_draws", ctypes.c_uint32), ("draws", ctypes.c_void_p),
                ("vertices", ctypes.c_void_p), ("num_vertices", ctypes.c_uint32), ("postprocess", ctypes.c_uint32),
                ("post", PostConfig), ("frame_duration_s", ctypes.c_float), ("color_modulate", ctypes.c_float * 3),
                ("dst", ctypes.c_void_p), ("dst_pitch", ctypes.c_uint32), ("dst_is_device", ctypes.c_int32),
                ("num_material_frames", ctypes.c_uint32), ("material_frames", ctypes.c_void_p)]


class ViewCounts(ctypes.Structure):
    """SwViewCounts: what the last sw_draw_frame_view prepared."""
    _fields_ = [("num_surfaces", ctypes.c_uint32), ("num_draws", ctypes.c_uint32), ("num_vertices", ctypes.c_uint32),
                ("error", ctypes.c_uint32), ("total_texels", ctypes.c_uint64), ("num_rows", ctypes.c_uint64)]


class Tuning(ctypes.Structure):
    """SwTuning: launch configuration (raster tile shape, surface-build blocks per SM)."""
    _fields_ = [("raster_tile", ctypes.c_uint32), ("surface_blocks_per_sm", ctypes.c_uint32),
                ("surface_texels_per_thread", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]


SW_RASTER_TILE_VARIANTS = 5

LAYOUT_ORDER = [
    ("SwCreateInfo", ctypes.sizeof(CreateInfo)), ("SwTextureMip", TEXTURE_MIP.itemsize),
    ("SwEmissiveMip", EMISSIVE_MIP.itemsize), ("SwDirectionalLightmapElement", DIR_LIGHTMAP_ELEMENT.itemsize),
    ("SwLight", LIGHT.itemsize), ("SwSurfaceDesc", SURFACE_DESC.itemsize), ("SwVertex16", VERTEX16.itemsize),
    ("SwDrawCmd", DRAW_CMD.itemsize), ("SwFrameParams", ctypes.sizeof(FrameParams)),
    ("SwPostConfig", ctypes.sizeof(PostConfig)), ("SwStats", ctypes.sizeof(Stats)),
    ("SwFrameInput", ctypes.sizeof(FrameInput)), ("SwTuning", ctypes.sizeof(Tuning)),
    ("SwMapPolygon", MAP_POLYGON.itemsize), ("SwViewLeaf", VIEW_LEAF.itemsize),
    ("SwViewFrameInput", ctypes.sizeof(ViewFrameInput)), ("SwViewCounts", ctypes.sizeof(ViewCounts)),
    ("SwLightShadow", LIGHT_SHADOW.itemsize), ("SwDepthDraw", DEPTH_DRAW.itemsize),
    ("SwShadowSide", SHADOW_SIDE.itemsize), ("SwShadowLeaf", SHADOW_LEAF.itemsize),
    ("SwMaterialFrame", MATERIAL_FRAME.itemsize), ("SwTriVertex", TRI_VERTEX.itemsize),
    ("SwTexturePass", TEXTURE_PASS.itemsize), ("SwSimPass", SIM_PASS.itemsize), ("SwSimPoint", SIM_POINT.itemsize),
    ("SwView", VIEW.itemsize),
]


def ptr(a):
    """Raw pointer of a contiguous numpy array (or None for an empty/None array)."""
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"], "array must be C-contiguous"
    return ctypes.c_void_p(a.ctypes.data) if a.size else None
