"""Simulated water and fire texture effects on the GPU (sw_update_simulations) against the oracle's whole
restatement of the effects: the device wave fields and heat maps, and the generated texture and emissive
mips, equal the oracle's bit for bit frame after frame; whole frames of a map with water and fire
materials through both preparation paths equal the oracle's frames rendered from the oracle's own
effect textures; malformed pass lists are refused before anything runs."""
import numpy as np
import pytest

import oracle
from sqwheel import abi, gpu, host

pytestmark = pytest.mark.gpu

SIM_MAP = dict(host.SMALL_MAP, water_materials=4, fire_materials=3)
FRAME_SEQUENCE = [0, 1, 2, 3, 5, 8, 13, 14, 30, 31, 90, 91, 60, 92, 93]


def frame_time(fi):
    return float(np.float32(np.float32(fi) * np.float32(1.0 / 60.0)))


def effects_of(scene):
    out = {m: scene.simulated_effect(m) for m in range(scene.info().materials)}
    return {m: e for m, e in out.items() if e.kind}


def slot_range(mips, slot):
    first, last = mips[slot * 5], mips[slot * 5 + 4]
    return int(first["offset"]), int(last["offset"]) + int(last["width"]) * int(last["height"])


def test_simulation_state_and_textures_bit_exact(gpu_ok):
    scene = host.Scene(**SIM_MAP)
    st = scene.static_data()
    effects = effects_of(scene)
    sims = {m: oracle.SimEffect(e) for m, e in effects.items()}
    work = type(st)(st.texels.copy(), st.texture_mips, st.emissive_pixels.copy(), st.emissive_mips, st.lightmaps,
                    st.directional_lightmaps)
    r = gpu.GpuRenderer(st)
    fr = host.Frame(scene)
    opts = host.frame_options(320, 240, abi.SW_PIXEL_C32, directional=False)
    try:
        r.reserve_simulation_state(scene.simulation_words())
        for fi in FRAME_SEQUENCE:
            fr.prepare(fi, opts)
            r.update_simulations(fr.sim_passes, fr.sim_points)
            for m, sim in sims.items():
                sim.update(frame_time(fi), work, m)
            texels, em = r.read_texels(st.texels.size, st.emissive_pixels.size)
            for m, sim in sims.items():
                e = effects[m]
                words, _, generated, _ = sim.state()
                area = words.size
                cur = fr.effect_state(m)[1]
                got = r.read_simulation_state(e.state_offset + cur * area, area)
                assert np.array_equal(got, words), f"frame {fi} material {m}: {(got != words).sum()} words differ"
                if e.kind == host.EFFECT_WATER:
                    a, b = slot_range(st.texture_mips, e.output_texture)
                    diff = texels[a:b] != work.texels[a:b]
                else:
                    a, b = slot_range(st.emissive_mips, e.output_emissive)
                    diff = em[a:b] != work.emissive_pixels[a:b]
                assert not diff.any(), f"frame {fi} material {m}: {diff.sum()} generated texels differ"
        # nothing else in the static data changed
        assert np.array_equal(texels, work.texels) and np.array_equal(em, work.emissive_pixels)
    finally:
        r.close()


@pytest.mark.parametrize("gpu_prep,fmt", [(True, abi.SW_PIXEL_C64), (False, abi.SW_PIXEL_C32)])
def test_simulated_effect_frames(gpu_ok, gpu_prep, fmt):
    scene = host.Scene(**dict(SIM_MAP, num_dynamic_lights=2, normal_maps=1))
    st = scene.static_data()
    effects = effects_of(scene)
    sims = {m: oracle.SimEffect(e) for m, e in effects.items()}
    work = type(st)(st.texels.copy(), st.texture_mips, st.emissive_pixels.copy(), st.emissive_mips, st.lightmaps,
                    st.directional_lightmaps)
    fr = host.Frame(scene)
    hr = host.HostRenderer(scene)
    hr.set_gpu_prep(gpu_prep)
    w, h = 480, 270
    opts = host.frame_options(w, h, fmt, directional=False)
    outputs = {e.output_texture for e in effects.values()} | {e.output_emissive for e in effects.values()}
    seen = 0
    try:
        for fi in range(0, 64, 3):  # in order: the effects' state carries from frame to frame
            fr.prepare(fi, opts)
            for m, sim in sims.items():
                sim.update(frame_time(fi), work, m)
            s = fr.surfaces
            seen += int(np.isin(s["texture_mip"] // 5, list(outputs)).sum() +
                        np.isin(s["emissive_mip"][s["emissive_mip"] != 0xFFFFFFFF] // 5, list(outputs)).sum())
            arena = oracle.build_surfaces(work, s, fr.lights, fr.params, fr.total_texels, num_threads=8)
            want = np.zeros((h, w), np.uint64 if fmt == abi.SW_PIXEL_C64 else np.uint32)
            assert oracle.rasterize(fr.draws, fr.vertices, arena, fr.params, want) == 0
            got = np.zeros_like(want)
            hr.render_frame(fi, opts, out=got)
            assert np.array_equal(want, got), f"frame {fi}: {(want != got).sum()} pixels differ"
        assert seen > 0
    finally:
        hr.close()


def test_malformed_simulation_passes_refused(gpu_ok):
    scene = host.Scene(**SIM_MAP)
    st = scene.static_data()
    effects = effects_of(scene)
    r = gpu.GpuRenderer(st)
    try:
        words = scene.simulation_words()
        r.reserve_simulation_state(words)
        water = next(e for e in effects.values() if e.kind == host.EFFECT_WATER and e.resolution_log2[0] == 7)
        area = 1 << 14
        base = np.zeros(1, abi.SIM_PASS)
        base["kind"], base["size_log2"] = abi.SW_SIM_WATER_STEP, [7, 7]
        base["state_src"], base["state_dst"] = water.state_offset, water.state_offset + area
        base["param"] = np.float32(0.99).view(np.uint32)
        r.update_simulations(base, None)  # well-formed
        before = r.read_simulation_state(0, words)
        cases = []
        q = base.copy(); q["state_dst"] = words - area + 1; cases.append((q, None, "state out of range"))
        q = base.copy(); q["state_dst"] = q["state_src"]; cases.append((q, None, "state out of range"))
        q = base.copy(); q["size_log2"] = [1, 7]; cases.append((q, None, "field size"))
        q = base.copy(); q["kind"] = 99; cases.append((q, None, "unknown kind"))
        q = np.concatenate([base, base]); q["launch"] = [1, 0]; cases.append((q, None, "out of order"))
        pts = np.zeros(2, abi.SIM_POINT); pts["address"] = [5, area]
        q = base.copy(); q["kind"], q["num_points"] = abi.SW_SIM_WATER_POINTS, 2; cases.append((q, pts, "outside the field"))
        q = base.copy(); q["kind"], q["num_points"] = abi.SW_SIM_FIRE_POINTS, 3; cases.append((q, pts, "points out of range"))
        q = base.copy(); q["kind"], q["dst_mip"] = abi.SW_SIM_WATER_TEXTURE, 0  # a 128x128 mip, not the output slot
        q["src_mip"] = 5; q["flags"] = 4 << abi.SW_SIM_COLOR_MODE_SHIFT; cases.append((q, None, "colour mode"))
        q = base.copy(); q["kind"], q["num_points"] = abi.SW_SIM_FIRE_TEXTURE, 10; q["dst_mip"] = 0
        cases.append((q, np.zeros(10, abi.SIM_POINT), "palette"))
        q = base.copy(); q["kind"], q["dst_mip"], q["src_mip"] = abi.SW_SIM_TEXTURE_MIP, 0, 1
        cases.append((q, None, "half the source"))
        q = base.copy(); q["kind"], q["param"] = abi.SW_SIM_FIRE_STEP, (1 << 18) + 1; cases.append((q, None, "attenuation"))
        for passes, points, msg in cases:
            with pytest.raises(gpu.SwError, match=msg):
                r.update_simulations(passes, points)
        assert np.array_equal(r.read_simulation_state(0, words), before)
        with pytest.raises(gpu.SwError, match="outside the simulation state"):
            r.read_simulation_state(words - 4, 8)
    finally:
        r.close()
