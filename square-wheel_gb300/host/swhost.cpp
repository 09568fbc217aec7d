// C ABI of the host library (include/swhost.h).
#include "../../include/swhost.h"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>

#include "frame.h"
#include "scene.h"
#include "sqwm.h"

using namespace swhost;

struct SwhScene
{
	Scene scene;
};
struct SwhFrame
{
	explicit SwhFrame(const Scene& s) : scene(s), prep(s) {}
	const Scene& scene;
	FramePrep prep;
};
struct SwhRenderer;
namespace
{
int submit_shadows(SwhRenderer* r, const FramePrep& p);
}
struct SwhRenderer
{
	const SwhScene* scene = nullptr;
	SwCtx* ctx = nullptr;
	SwhFrame* frame = nullptr;
	bool gpu_prep = true; // render_frame: surfaces and world draws prepared on the GPU (sw_draw_frame_view)
	bool shadows_set = false; // sw_set_light_shadows holds descriptors from an earlier frame
};

namespace
{
// The frame's texture effect passes (update_animations, map_materials_processor.rs:249-303), then
// build_shadow_maps (partial_renderer.rs:525-592) for the frame and its lights' shadow maps.
int submit_shadows(SwhRenderer* r, const FramePrep& p)
{
	// the generative texture effects of the frame first: the surfaces read their output textures
	if (!p.texture_passes.empty())
	{
		const int st = sw_update_textures(r->ctx, p.texture_passes.data(), uint32_t(p.texture_passes.size()),
			p.texture_shifts.data(), uint32_t(p.texture_shifts.size()));
		if (st) return st;
	}
	if (!p.simulations.passes.empty())
	{
		const int st = sw_update_simulations(r->ctx, p.simulations.passes.data(), uint32_t(p.simulations.passes.size()),
			p.simulations.points.data(), uint32_t(p.simulations.points.size()));
		if (st) return st;
	}
	if (p.shadow_texels == 0)
	{
		if (!r->shadows_set) return SW_OK;
		r->shadows_set = false;
		return sw_set_light_shadows(r->ctx, nullptr, 0);
	}
	// prepare_view lists sides and leafs (the GPU prepares their polygons); prepare lists depth draws
	int st = !p.shadow_sides.empty()
		? sw_build_shadow_maps_view(r->ctx, p.shadow_sides.data(), uint32_t(p.shadow_sides.size()), p.shadow_leafs.data(),
			  uint32_t(p.shadow_leafs.size()), p.shadow_texels)
		: sw_build_shadow_maps(r->ctx, p.depth_draws.data(), uint32_t(p.depth_draws.size()), p.depth_vertices.data(),
			  uint32_t(p.depth_vertices.size()), p.shadow_texels);
	if (st) return st;
	r->shadows_set = true;
	return sw_set_light_shadows(r->ctx, p.light_shadows.data(), uint32_t(p.light_shadows.size()));
}
} // namespace

namespace
{
thread_local std::string g_error;

// textures_mip_bias as Renderer::synchronize_config leaves it before every frame (renderer.rs:222-233).
float clamped_mip_bias(float b)
{
	if (b < -1.0f) b = -1.0f;
	if (b > 2.0f) b = 2.0f;
	return b;
}

FrameOptions to_options(const SwhFrameOptions* o)
{
	FrameOptions f;
	f.width = o->width;
	f.height = o->height;
	f.pixel_format = o->pixel_format;
	f.use_directional_lightmaps = o->use_directional_lightmaps != 0;
	f.clear_background = o->clear_background != 0;
	if (o->fov > 0.0f) f.fov = o->fov;
	f.mip_bias = clamped_mip_bias(o->mip_bias);
	// Renderer::synchronize_config, renderer.rs:235-244 (a NaN passes both comparisons unchanged)
	f.shadows_quality = o->shadows_quality;
	if (f.shadows_quality < -1.0f) f.shadows_quality = -1.0f;
	if (f.shadows_quality > 1.0f) f.shadows_quality = 1.0f;
	return f;
}

bool valid_options(const SwhFrameOptions* o)
{
	return o && o->width > 0 && o->height > 0 && o->width <= 16384 && o->height <= 16384 && o->pixel_format <= SW_PIXEL_C64;
}
} // namespace

extern "C" {

const char* swh_last_error(void) { return g_error.c_str(); }

namespace
{
int scene_config_from(const SwhSceneConfig* c, SceneConfig& cfg)
{
	cfg.seed = c->seed;
	cfg.grid_x = c->grid_x;
	cfg.grid_y = c->grid_y;
	cfg.room_min = c->room_min;
	cfg.room_max = c->room_max;
	cfg.tile_size = c->tile_size;
	cfg.texture_size = c->texture_size;
	cfg.num_materials = c->num_materials;
	cfg.metal_frac = c->metal_frac;
	cfg.dielectric_frac = c->dielectric_frac;
	cfg.normal_maps = c->normal_maps != 0;
	cfg.directional_lightmaps = c->directional_lightmaps != 0;
	cfg.lights_per_room = c->lights_per_room;
	cfg.num_dynamic_lights = c->num_dynamic_lights;
	cfg.num_frames = c->num_frames ? c->num_frames : 1;
	cfg.emissive_frac = c->emissive_frac;
	cfg.sky_rooms = c->sky_rooms;
	cfg.skybox_size = c->skybox_size ? c->skybox_size : 128;
	cfg.skybox_brightness = c->skybox_brightness > 0.0f ? c->skybox_brightness : 1.0f;
	cfg.skybox_missing_side = c->skybox_missing_side;
	cfg.sky_rotation_speed = c->sky_rotation_speed;
	cfg.camera_pitch = c->camera_pitch;
	cfg.shadowed_lights = c->shadowed_lights;
	cfg.scrolling_materials = c->scrolling_materials;
	cfg.animated_materials = c->animated_materials;
	cfg.projector_lights = c->projector_lights;
	cfg.num_models = c->num_models;
	cfg.model_triangles = c->model_triangles ? c->model_triangles : 2000;
	cfg.model_frames = c->model_frames ? c->model_frames : 8;
	cfg.turb_materials = c->turb_materials;
	cfg.num_sprites = c->num_sprites;
	cfg.num_decals = c->num_decals;
	cfg.layered_materials = c->layered_materials;
	cfg.water_materials = c->water_materials;
	cfg.fire_materials = c->fire_materials;
	cfg.num_portals = c->num_portals;
	cfg.portals_depth = std::min(c->portals_depth, 8u);
	cfg.light_grid = c->light_grid;
	if (cfg.num_portals > 4096)
	{
		g_error = "too many portals";
		return SW_ERR_INVALID_ARGUMENT;
	}
	if (cfg.num_models > 100000 || cfg.model_triangles > 200000 || cfg.model_frames > 256 || cfg.num_sprites > 1000000 ||
		cfg.num_decals > 1000000)
	{
		g_error = "too many models, model triangles, frames or sprites";
		return SW_ERR_INVALID_ARGUMENT;
	}
	return SW_OK;
}
} // namespace

int swh_scene_create(const SwhSceneConfig* c, SwhScene** out)
{
	if (!c || !out) return SW_ERR_INVALID_ARGUMENT;
	*out = nullptr;
	SceneConfig cfg;
	const int st = scene_config_from(c, cfg);
	if (st != SW_OK) return st;
	SwhScene* s = new (std::nothrow) SwhScene();
	if (!s) return SW_ERR_OUT_OF_MEMORY;
	try
	{
		if (!generate_scene(cfg, s->scene, g_error))
		{
			delete s;
			return SW_ERR_INVALID_ARGUMENT;
		}
	}
	catch (const std::bad_alloc&)
	{
		delete s;
		g_error = "out of host memory";
		return SW_ERR_OUT_OF_MEMORY;
	}
	*out = s;
	return SW_OK;
}

int swh_scene_destroy(SwhScene* s)
{
	if (!s) return SW_ERR_INVALID_ARGUMENT;
	delete s;
	return SW_OK;
}

int swh_scene_load_map_memory(const void* data, uint64_t size, const SwhSceneConfig* c, SwhScene** out)
{
	if (!data || !c || !out) return SW_ERR_INVALID_ARGUMENT;
	*out = nullptr;
	SceneConfig cfg;
	int st = scene_config_from(c, cfg);
	if (st != SW_OK) return st;
	try
	{
		SqwmMap map;
		std::string error;
		if (sqwm_parse(static_cast<const uint8_t*>(data), size_t(size), map, error) != SQWM_OK)
		{
			g_error = error;
			return SW_ERR_INVALID_ARGUMENT;
		}
		SwhScene* s = new SwhScene();
		if (!scene_from_map(map, cfg, s->scene, g_error))
		{
			delete s;
			return SW_ERR_INVALID_ARGUMENT;
		}
		*out = s;
		return SW_OK;
	}
	catch (const std::bad_alloc&)
	{
		g_error = "out of host memory";
		return SW_ERR_OUT_OF_MEMORY;
	}
}

int swh_scene_load_map(const char* path, const SwhSceneConfig* c, SwhScene** out)
{
	if (!path || !c || !out) return SW_ERR_INVALID_ARGUMENT;
	*out = nullptr;
	std::FILE* f = std::fopen(path, "rb");
	if (!f)
	{
		g_error = std::string("can't open ") + path;
		return SW_ERR_INVALID_ARGUMENT;
	}
	std::vector<uint8_t> bytes;
	try
	{
		uint8_t buf[1 << 16];
		size_t n;
		while ((n = std::fread(buf, 1, sizeof(buf), f)) > 0) bytes.insert(bytes.end(), buf, buf + n);
	}
	catch (const std::bad_alloc&)
	{
		std::fclose(f);
		g_error = "out of host memory";
		return SW_ERR_OUT_OF_MEMORY;
	}
	const bool read_error = std::ferror(f) != 0;
	std::fclose(f);
	if (read_error)
	{
		g_error = std::string("can't read ") + path;
		return SW_ERR_INVALID_ARGUMENT;
	}
	return swh_scene_load_map_memory(bytes.data(), bytes.size(), c, out);
}

int swh_scene_save_map(const SwhScene* s, const char* path)
{
	if (!s || !path) return SW_ERR_INVALID_ARGUMENT;
	try
	{
		SqwmMap map;
		map_from_scene(s->scene, map);
		std::vector<uint8_t> bytes;
		sqwm_serialize(map, bytes);
		std::FILE* f = std::fopen(path, "wb");
		if (!f)
		{
			g_error = std::string("can't create ") + path;
			return SW_ERR_INVALID_ARGUMENT;
		}
		const bool ok = std::fwrite(bytes.data(), 1, bytes.size(), f) == bytes.size();
		if (std::fclose(f) != 0 || !ok)
		{
			g_error = std::string("can't write ") + path;
			return SW_ERR_INVALID_ARGUMENT;
		}
		return SW_OK;
	}
	catch (const std::bad_alloc&)
	{
		g_error = "out of host memory";
		return SW_ERR_OUT_OF_MEMORY;
	}
}

int swh_scene_compressed_lightmaps(const SwhScene* s, const void** out_lightmaps, uint64_t* out_count,
	const void** out_directional, uint64_t* out_directional_count)
{
	if (!s || !out_lightmaps || !out_count || !out_directional || !out_directional_count) return SW_ERR_INVALID_ARGUMENT;
	const Scene& sc = s->scene;
	*out_lightmaps = sc.lightmaps_compressed.data();
	*out_count = sc.lightmaps_compressed.size() / SW_LIGHTMAP_COMPRESSED_BYTES;
	*out_directional = sc.directional_lightmaps_compressed.data();
	*out_directional_count = sc.directional_lightmaps_compressed.size() / SW_DIR_LIGHTMAP_COMPRESSED_BYTES;
	return SW_OK;
}

int swh_scene_texture_effect(const SwhScene* s, uint32_t material, SwhTextureEffect* out)
{
	if (!s || !out || material >= s->scene.materials.size()) return SW_ERR_INVALID_ARGUMENT;
	const Material& m = s->scene.materials[material];
	out->kind = m.effect;
	out->output_texture = m.effect_texture;
	out->num_layers = uint32_t(m.layers.size());
	out->turb[0] = m.turb_amplitude;
	out->turb[1] = m.turb_wave_length;
	out->turb[2] = m.turb_frequency;
	return SW_OK;
}

namespace
{
SwhTimeFunction flat_function(const TimeFunction& f) { return SwhTimeFunction{f.kind, f.a, f.b, f.c, f.d}; }
SwhRandomValue flat_random(const RandomValue& v) { return SwhRandomValue{flat_function(v.value), flat_function(v.deviation)}; }
} // namespace

int swh_scene_simulated_effect(const SwhScene* s, uint32_t material, SwhSimEffect* out)
{
	if (!s || !out || material >= s->scene.materials.size()) return SW_ERR_INVALID_ARGUMENT;
	const Material& m = s->scene.materials[material];
	std::memset(out, 0, sizeof(*out));
	out->output_texture = m.effect_texture;
	out->output_emissive = m.effect_emissive;
	out->source_emissive = m.emissive;
	out->roughness = m.roughness;
	out->state_offset = m.sim_state;
	if (m.effect == Material::WATER)
	{
		const WaterEffect& w = m.water;
		out->kind = m.effect;
		out->resolution_log2[0] = w.resolution_log2[0];
		out->resolution_log2[1] = w.resolution_log2[1];
		out->update_frequency = w.update_frequency;
		out->attenuation_param = w.fluidity;
		out->color_mode = w.color_mode;
		if (w.sources.size() > SWH_MAX_SIM_SOURCES) return SW_ERR_LIMIT;
		out->num_sources = uint32_t(w.sources.size());
		for (size_t i = 0; i < w.sources.size(); ++i)
		{
			const WaveSource& a = w.sources[i];
			SwhSimSource& o = out->sources[i];
			o.kind = a.kind;
			for (int p = 0; p < 2; ++p)
				for (int c = 0; c < 2; ++c)
				{
					o.points[p][c] = a.points[p][c];
					o.offsets[p][c] = flat_function(a.offsets[p][c]);
				}
			o.frequency = a.frequency;
			o.phase = a.phase;
			o.amplitude = a.amplitude;
			o.offset = a.offset;
			o.radius = a.radius;
		}
	}
	else if (m.effect == Material::FIRE)
	{
		const FireEffect& f = m.fire;
		out->kind = m.effect;
		out->resolution_log2[0] = f.resolution_log2[0];
		out->resolution_log2[1] = f.resolution_log2[1];
		out->update_frequency = f.update_frequency;
		out->attenuation_param = f.heat_conductivity;
		out->slow = f.slow ? 1u : 0u;
		out->has_color = f.has_color ? 1u : 0u;
		for (int c = 0; c < 3; ++c) out->color[c] = f.color[c];
		if (f.sources.size() > SWH_MAX_SIM_SOURCES) return SW_ERR_LIMIT;
		out->num_sources = uint32_t(f.sources.size());
		for (size_t i = 0; i < f.sources.size(); ++i)
		{
			const HeatSource& a = f.sources[i];
			SwhSimSource& o = out->sources[i];
			o.kind = a.kind;
			for (int p = 0; p < 2; ++p)
				for (int c = 0; c < 2; ++c)
				{
					o.points[p][c] = a.points[p][c];
					o.fire_offsets[p][c] = flat_random(a.offset[p][c]);
				}
			o.frequency = a.frequency;
			o.ramp = a.ramp ? 1u : 0u;
			o.heat = flat_random(a.heat);
			o.angle = flat_random(a.angle);
			o.speed = flat_random(a.speed);
			o.gravity = flat_random(a.gravity);
			o.spawn_angle = flat_random(a.spawn_angle);
			o.spawn_distance = flat_random(a.spawn_distance);
			o.lifetime = flat_random(a.lifetime);
		}
	}
	return SW_OK;
}

int swh_scene_simulation_words(const SwhScene* s, uint64_t* out)
{
	if (!s || !out) return SW_ERR_INVALID_ARGUMENT;
	*out = s->scene.sim_state_words;
	return SW_OK;
}

int swh_scene_light_grid(const SwhScene* s, void* out_header, uint32_t* out_columns, float* out_samples, uint64_t* num_columns,
	uint64_t* num_samples)
{
	if (!s || !num_columns || !num_samples) return SW_ERR_INVALID_ARGUMENT;
	const Scene& sc = s->scene;
	*num_columns = sc.light_grid_columns.size();
	*num_samples = sc.light_grid_samples.size();
	static_assert(sizeof(LightGridHeader) == 36 && sizeof(LightGridColumn) == 12 && sizeof(LightGridElement) == 96, "grid layout");
	if (out_header) std::memcpy(out_header, &sc.light_grid_header, sizeof(LightGridHeader));
	if (out_columns && !sc.light_grid_columns.empty())
		std::memcpy(out_columns, sc.light_grid_columns.data(), sc.light_grid_columns.size() * sizeof(LightGridColumn));
	if (out_samples && !sc.light_grid_samples.empty())
		std::memcpy(out_samples, sc.light_grid_samples.data(), sc.light_grid_samples.size() * sizeof(LightGridElement));
	return SW_OK;
}

int swh_scene_fetch_light(const SwhScene* s, const float pos[3], float out_sample[24])
{
	if (!s || !pos || !out_sample) return SW_ERR_INVALID_ARGUMENT;
	const LightGridElement e = s->scene.fetch_light_from_grid(v3(pos[0], pos[1], pos[2]));
	std::memcpy(out_sample, &e, sizeof(e));
	return SW_OK;
}

int swh_scene_info(const SwhScene* s, SwhSceneInfo* out)
{
	if (!s || !out) return SW_ERR_INVALID_ARGUMENT;
	const Scene& sc = s->scene;
	out->nodes = uint32_t(sc.nodes.size());
	out->leafs = uint32_t(sc.leafs.size());
	out->polygons = uint32_t(sc.polygons.size());
	out->portals = uint32_t(sc.portals.size());
	out->materials = uint32_t(sc.materials.size());
	out->frames = uint32_t(sc.camera_path.size());
	out->dynamic_lights = uint32_t(sc.dynamic_lights.size());
	out->reserved = 0;
	out->lightmap_elements = sc.lightmap_elements;
	out->texels = sc.texels.size();
	out->skybox_texels = sc.skybox32.size();
	return SW_OK;
}

int swh_scene_skybox(const SwhScene* s, const uint32_t** t32, const uint64_t** t64, uint64_t* count,
	uint64_t mip_offsets[30], uint32_t mip_sizes[30])
{
	if (!s || !t32 || !t64 || !count) return SW_ERR_INVALID_ARGUMENT;
	const Scene& sc = s->scene;
	*t32 = sc.skybox32.data();
	*t64 = sc.skybox64.data();
	*count = sc.skybox32.size();
	for (uint32_t side = 0; side < 6; ++side)
		for (uint32_t m = 0; m < NUM_MIPS; ++m)
		{
			if (mip_offsets) mip_offsets[side * NUM_MIPS + m] = sc.skybox_mips[side][m].offset;
			if (mip_sizes) mip_sizes[side * NUM_MIPS + m] = sc.skybox_mips[side][m].size;
		}
	return SW_OK;
}

int swh_scene_create_info(const SwhScene* s, uint32_t device, SwCreateInfo* out)
{
	if (!s || !out) return SW_ERR_INVALID_ARGUMENT;
	*out = s->scene.create_info(device);
	return SW_OK;
}

int swh_scene_lite_textures(const SwhScene* s, const uint32_t** out_pixels, uint64_t* out_count)
{
	if (!s || !out_pixels || !out_count) return SW_ERR_INVALID_ARGUMENT;
	*out_pixels = s->scene.lite_pixels.data();
	*out_count = s->scene.lite_pixels.size();
	return SW_OK;
}

int swh_frame_create(const SwhScene* s, SwhFrame** out)
{
	if (!s || !out) return SW_ERR_INVALID_ARGUMENT;
	*out = new (std::nothrow) SwhFrame(s->scene);
	return *out ? SW_OK : SW_ERR_OUT_OF_MEMORY;
}

int swh_frame_map(const SwhFrame* f, const SwMapPolygon** out_polygons, uint32_t* out_num_polygons, const float** out_vertices,
	uint32_t* out_num_vertices)
{
	if (!f || !out_polygons || !out_num_polygons || !out_vertices || !out_num_vertices) return SW_ERR_INVALID_ARGUMENT;
	*out_polygons = f->prep.map_polygons_base.data();
	*out_num_polygons = uint32_t(f->prep.map_polygons_base.size());
	*out_vertices = reinterpret_cast<const float*>(f->scene.vertices.data());
	*out_num_vertices = uint32_t(f->scene.vertices.size());
	return SW_OK;
}

int swh_frame_destroy(SwhFrame* f)
{
	if (!f) return SW_ERR_INVALID_ARGUMENT;
	delete f;
	return SW_OK;
}

int swh_frame_prepare(SwhFrame* f, uint32_t frame_index, const SwhFrameOptions* o)
{
	if (!f || !valid_options(o)) return SW_ERR_INVALID_ARGUMENT;
	try
	{
		f->prep.prepare(frame_index, to_options(o));
	}
	catch (const std::bad_alloc&)
	{
		g_error = "out of host memory";
		return SW_ERR_OUT_OF_MEMORY;
	}
	return SW_OK;
}

int swh_frame_prepare_view(SwhFrame* f, uint32_t frame_index, const SwhFrameOptions* o)
{
	if (!f || !valid_options(o)) return SW_ERR_INVALID_ARGUMENT;
	try
	{
		f->prep.prepare_view(frame_index, to_options(o));
	}
	catch (const std::bad_alloc&)
	{
		g_error = "out of host memory";
		return SW_ERR_OUT_OF_MEMORY;
	}
	return SW_OK;
}

int swh_frame_view_input(const SwhFrame* f, SwViewFrameInput* out)
{
	if (!f || !out) return SW_ERR_INVALID_ARGUMENT;
	const FramePrep& p = f->prep;
	std::memset(out, 0, sizeof(*out));
	out->params = p.params;
	out->num_lights = uint32_t(p.lights.size());
	out->lights = p.lights.data();
	const CameraMatrices& cam = p.camera();
	for (int c = 0; c < 4; ++c)
	{
		const Vec4* cols[2] = {&cam.view_matrix.c[c], &cam.planes_matrix.c[c]};
		float* dst[2] = {out->view_matrix + c * 4, out->planes_matrix + c * 4};
		for (int m = 0; m < 2; ++m)
		{
			dst[m][0] = cols[m]->x;
			dst[m][1] = cols[m]->y;
			dst[m][2] = cols[m]->z;
			dst[m][3] = cols[m]->w;
		}
	}
	out->num_leafs = uint32_t(p.view_leafs.size());
	out->leafs = p.view_leafs.data();
	out->num_leaf_lights = uint32_t(p.view_leaf_lights.size());
	out->leaf_lights = p.view_leaf_lights.data();
	out->num_draws = uint32_t(p.draws.size());
	out->draws = p.draws.data();
	out->vertices = p.vertices.data();
	out->num_vertices = uint32_t(p.vertices.size());
	out->num_material_frames = p.animated ? uint32_t(p.material_frames.size()) : 0u;
	out->material_frames = p.animated ? p.material_frames.data() : nullptr;
	return SW_OK;
}

int swh_frame_effect_state(const SwhFrame* f, uint32_t material, uint32_t* out_update_step, uint32_t* out_current_buffer,
	uint32_t* out_generated, uint32_t* out_particles)
{
	if (!f || !out_update_step || !out_current_buffer || !out_generated || !out_particles) return SW_ERR_INVALID_ARGUMENT;
	const EffectSim* e = f->prep.effect_sim(material);
	if (!e) return SW_ERR_INVALID_ARGUMENT;
	*out_update_step = e->update_step();
	*out_current_buffer = e->current_buffer();
	*out_generated = e->generated() ? 1u : 0u;
	*out_particles = e->num_particles();
	return SW_OK;
}

int swh_frame_outputs(const SwhFrame* f, SwhFrameOutputs* out)
{
	if (!f || !out) return SW_ERR_INVALID_ARGUMENT;
	const FramePrep& p = f->prep;
	out->surfaces = p.surfaces.data();
	out->num_surfaces = uint32_t(p.surfaces.size());
	out->total_texels = p.total_texels;
	out->draws = p.draws.data();
	out->num_draws = uint32_t(p.draws.size());
	out->vertices = p.vertices.data();
	out->num_vertices = uint32_t(p.vertices.size());
	out->lights = p.lights.data();
	out->num_lights = uint32_t(p.lights.size());
	out->params = p.params;
	out->visible_leafs = p.stats.visible_leafs;
	out->camera_leaf = p.stats.camera_leaf;
	out->skybox_draws = p.stats.skybox_draws;
	out->light_shadows = p.light_shadows.data();
	out->depth_draws = p.depth_draws.data();
	out->num_depth_draws = uint32_t(p.depth_draws.size());
	out->num_depth_vertices = uint32_t(p.depth_vertices.size());
	out->depth_vertices = p.depth_vertices.data();
	out->shadow_texels = p.shadow_texels;
	out->shadow_sides = p.shadow_sides.data();
	out->num_shadow_sides = uint32_t(p.shadow_sides.size());
	out->num_shadow_leafs = uint32_t(p.shadow_leafs.size());
	out->shadow_leafs = p.shadow_leafs.data();
	out->tri_vertices = p.tri_vertices.data();
	out->num_tri_vertices = uint32_t(p.tri_vertices.size());
	out->model_triangles = p.stats.model_triangles;
	out->texture_passes = p.texture_passes.data();
	out->num_texture_passes = uint32_t(p.texture_passes.size());
	out->texture_shifts = p.texture_shifts.data();
	out->num_texture_shifts = uint32_t(p.texture_shifts.size());
	out->sim_passes = p.simulations.passes.data();
	out->num_sim_passes = uint32_t(p.simulations.passes.size());
	out->sim_points = p.simulations.points.data();
	out->num_sim_points = uint32_t(p.simulations.points.size());
	out->views = p.views.data();
	out->num_views = uint32_t(p.views.size());
	out->main_draws = p.main_draws;
	out->surface_texels = p.surface_texels;
	return SW_OK;
}

int swh_renderer_create(const SwhScene* s, uint32_t device, SwhRenderer** out)
{
	if (!s || !out) return SW_ERR_INVALID_ARGUMENT;
	*out = nullptr;
	SwhRenderer* r = new (std::nothrow) SwhRenderer();
	if (!r) return SW_ERR_OUT_OF_MEMORY;
	r->scene = s;
	SwCreateInfo ci = s->scene.create_info(device);
	// a loaded map's lightmaps go up compressed, as the file holds them, and are decoded on the GPU
	const Scene& sc = s->scene;
	const bool compressed = !sc.lightmaps_compressed.empty() || !sc.directional_lightmaps_compressed.empty();
	if (compressed)
	{
		ci.lightmaps = nullptr;
		ci.num_lightmap_elements = 0;
		ci.directional_lightmaps = nullptr;
		ci.num_directional_lightmap_elements = 0;
	}
	int st = sw_create(&ci, &r->ctx);
	if (st != SW_OK)
	{
		g_error = "sw_create failed";
		delete r;
		return st;
	}
	if (compressed &&
		(st = sw_set_lightmaps_compressed(r->ctx, sc.lightmaps_compressed.data(),
			 sc.lightmaps_compressed.size() / SW_LIGHTMAP_COMPRESSED_BYTES, sc.directional_lightmaps_compressed.data(),
			 sc.directional_lightmaps_compressed.size() / SW_DIR_LIGHTMAP_COMPRESSED_BYTES)) != SW_OK)
	{
		g_error = std::string("sw_set_lightmaps_compressed failed: ") + sw_last_error(r->ctx);
		sw_destroy(r->ctx);
		delete r;
		return st;
	}
	if (!s->scene.lite_pixels.empty() &&
		(st = sw_set_lite_textures(r->ctx, s->scene.lite_pixels.data(), s->scene.lite_pixels.size())) != SW_OK)
	{
		g_error = "sw_set_lite_textures failed";
		sw_destroy(r->ctx);
		delete r;
		return st;
	}
	if (!s->scene.skybox32.empty() &&
		(st = sw_set_skybox(r->ctx, s->scene.skybox32.data(), s->scene.skybox64.data(), s->scene.skybox32.size())) != SW_OK)
	{
		g_error = "sw_set_skybox failed";
		sw_destroy(r->ctx);
		delete r;
		return st;
	}
	if (s->scene.sim_state_words && (st = sw_reserve_simulation_state(r->ctx, s->scene.sim_state_words)) != SW_OK)
	{
		g_error = std::string("sw_reserve_simulation_state failed: ") + sw_last_error(r->ctx);
		sw_destroy(r->ctx);
		delete r;
		return st;
	}
	r->frame = new (std::nothrow) SwhFrame(s->scene);
	if (!r->frame)
	{
		sw_destroy(r->ctx);
		delete r;
		return SW_ERR_OUT_OF_MEMORY;
	}
	const std::vector<SwMapPolygon>& mp = r->frame->prep.map_polygons_base;
	if ((st = sw_set_map(r->ctx, mp.data(), uint32_t(mp.size()), reinterpret_cast<const float*>(s->scene.vertices.data()),
			 uint32_t(s->scene.vertices.size()))) != SW_OK)
	{
		g_error = std::string("sw_set_map failed: ") + sw_last_error(r->ctx);
		sw_destroy(r->ctx);
		delete r->frame;
		delete r;
		return st;
	}
	*out = r;
	return SW_OK;
}

int swh_renderer_destroy(SwhRenderer* r)
{
	if (!r) return SW_ERR_INVALID_ARGUMENT;
	if (r->ctx) sw_destroy(r->ctx);
	delete r->frame;
	delete r;
	return SW_OK;
}

int swh_renderer_prepare_frame(SwhRenderer* r, uint32_t frame_index, const SwhFrameOptions* o)
{
	if (!r) return SW_ERR_INVALID_ARGUMENT;
	int st = swh_frame_prepare(r->frame, frame_index, o);
	if (st) return st;
	const FramePrep& p = r->frame->prep;
	if ((st = submit_shadows(r, p))) return st;
	st = sw_frame_begin(r->ctx, &p.params, p.lights.data(), uint32_t(p.lights.size()));
	if (st) return st;
	return sw_submit_surfaces(r->ctx, p.surfaces.data(), uint32_t(p.surfaces.size()), p.total_texels);
}

int swh_renderer_draw_frame(SwhRenderer* r, void* dst, uint32_t pitch, int dst_is_device)
{
	if (!r) return SW_ERR_INVALID_ARGUMENT;
	const FramePrep& p = r->frame->prep;
	if (!p.views.empty())
	{
		g_error = "a frame with portal views renders through swh_renderer_render_frame";
		return SW_ERR_STATE;
	}
	int st = sw_submit_draws_ex(r->ctx, p.draws.data(), uint32_t(p.draws.size()), p.vertices.data(), uint32_t(p.vertices.size()),
		p.tri_vertices.data(), uint32_t(p.tri_vertices.size()));
	if (st) return st;
	return sw_render(r->ctx, dst, pitch, dst_is_device);
}

int swh_renderer_render_frame(SwhRenderer* r, uint32_t frame_index, const SwhFrameOptions* o, const SwPostConfig* post,
	float frame_duration_s, const float color_modulate[3], void* dst, uint32_t pitch, int dst_is_device)
{
	if (!r || (post && (!dst || !color_modulate))) return SW_ERR_INVALID_ARGUMENT;
	// The GPU-side preparation emits each leaf's polygons only; a scene with triangle models, sprites, decals
	// or portals (drawn after their leaf's polygons) takes the host-prepared draw list.
	const Scene& scene = r->scene->scene;
	if (r->gpu_prep && scene.models.empty() && scene.sprites.empty() && scene.decals.empty() && scene.view_portals.empty())
	{
		int st = swh_frame_prepare_view(r->frame, frame_index, o);
		if (st) return st;
		if ((st = submit_shadows(r, r->frame->prep))) return st;
		SwViewFrameInput vin;
		swh_frame_view_input(r->frame, &vin);
		vin.mip_bias = clamped_mip_bias(o->mip_bias);
		if (post)
		{
			vin.postprocess = 1;
			vin.post = *post;
			vin.frame_duration_s = frame_duration_s;
			for (int i = 0; i < 3; ++i) vin.color_modulate[i] = color_modulate[i];
		}
		vin.dst = dst;
		vin.dst_pitch = pitch;
		vin.dst_is_device = dst_is_device;
		return sw_draw_frame_view(r->ctx, &vin);
	}
	int st = swh_frame_prepare(r->frame, frame_index, o);
	if (st) return st;
	const FramePrep& p = r->frame->prep;
	if ((st = submit_shadows(r, p))) return st;
	SwFrameInput in;
	std::memset(&in, 0, sizeof(in));
	in.params = p.params;
	in.num_lights = uint32_t(p.lights.size());
	in.lights = p.lights.data();
	in.surfaces = p.surfaces.data();
	in.total_texels = p.total_texels;
	in.num_surfaces = uint32_t(p.surfaces.size());
	in.num_draws = uint32_t(p.draws.size());
	in.draws = p.draws.data();
	in.vertices = p.vertices.data();
	in.num_vertices = uint32_t(p.vertices.size());
	in.tri_vertices = p.tri_vertices.data();
	in.num_tri_vertices = uint32_t(p.tri_vertices.size());
	in.num_views = uint32_t(p.views.size());
	in.views = p.views.data();
	in.main_draws = p.main_draws;
	if (post)
	{
		in.postprocess = 1;
		in.post = *post;
		in.frame_duration_s = frame_duration_s;
		for (int i = 0; i < 3; ++i) in.color_modulate[i] = color_modulate[i];
	}
	in.dst = dst;
	in.dst_pitch = pitch;
	in.dst_is_device = dst_is_device;
	return sw_draw_frame(r->ctx, &in);
}

int swh_renderer_set_frames_in_flight(SwhRenderer* r, uint32_t frames)
{
	if (!r) return SW_ERR_INVALID_ARGUMENT;
	return sw_set_frames_in_flight(r->ctx, frames);
}

int swh_renderer_set_gpu_prep(SwhRenderer* r, int enable)
{
	if (!r) return SW_ERR_INVALID_ARGUMENT;
	r->gpu_prep = enable != 0;
	return SW_OK;
}

SwCtx* swh_renderer_context(SwhRenderer* r) { return r ? r->ctx : nullptr; }
SwhFrame* swh_renderer_frame(SwhRenderer* r) { return r ? r->frame : nullptr; }

} // extern "C"
