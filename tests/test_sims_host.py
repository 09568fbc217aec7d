"""Simulated water and fire texture effects on the CPU. The oracle's random engine against xoshiro256++'s
published reference outputs; the host's per-frame pass lists (sw_update_simulations) replayed by a numpy
restatement of the passes' per-word semantics give the wave fields and heat maps of the oracle's whole
restatement of the effects (generative_texture_effect_water.rs, generative_texture_effect_fire.rs) bit
for bit, frame after frame, with the same update steps, particles and first generation."""
import numpy as np
import pytest

import oracle
from sqwheel import abi, host

pytestmark = pytest.mark.usefixtures("built_libs")

SIM_MAP = dict(host.SMALL_MAP, water_materials=4, fire_materials=3)
# frame indices in the order they are prepared: single steps, skipped frames (several steps), a jump of
# more than 10 steps, and a step back in time (no step)
FRAME_SEQUENCE = [0, 1, 2, 3, 5, 8, 13, 14, 30, 31, 90, 91, 60, 92, 93]


def test_xoshiro_reference_outputs():
    # xoshiro256plusplus.c's first outputs from the state {1, 2, 3, 4}
    want = [41943041, 58720359, 3588806011781223, 3591011842654386, 9228616714210784205, 9973669472204895162,
            14011001112246962877, 12406186145184390807, 15849039046786891736, 10450023813501588000]
    assert oracle.xoshiro_outputs([1, 2, 3, 4], 10).tolist() == want
    # seed_from_u64: PCG32 (multiplier 6364136223846793005, increment 11634580027462260723, XSH RR output)
    # filling the seed's little-endian u32 words
    seed = 0b1001100000111010100101010101010111000111010110100101111001010101
    words, st = [], seed
    for _ in range(8):
        st = (st * 6364136223846793005 + 11634580027462260723) % (1 << 64)
        xs, rot = (((st >> 18) ^ st) >> 27) & 0xFFFFFFFF, st >> 59
        words.append(((xs >> rot) | (xs << ((32 - rot) % 32))) & 0xFFFFFFFF)
    assert oracle.small_rng_state(seed).tolist() == [words[2 * i] | (words[2 * i + 1] << 32) for i in range(4)]


def replay(passes, points, state):
    """The per-word semantics of the simulation passes (include/swgpu.h), in numpy, on `state` (uint32)."""
    f32 = state.view(np.float32)
    for p in passes:
        kind, lx, ly = int(p["kind"]), int(p["size_log2"][0]), int(p["size_log2"][1])
        w, h = 1 << lx, 1 << ly
        src, dst = int(p["state_src"]), int(p["state_dst"])
        pts = points[int(p["first_point"]):int(p["first_point"]) + int(p["num_points"])]
        if kind == abi.SW_SIM_WATER_POINTS:
            for q in pts:
                v = np.uint32(q["value"]).view(np.float32)
                f32[src + q["address"]] = np.float32(f32[src + q["address"]] + v)
                f32[dst + q["address"]] = np.float32(f32[dst + q["address"]] - v)
        elif kind == abi.SW_SIM_WATER_STEP:
            s = f32[src:src + w * h].reshape(h, w)
            d = f32[dst:dst + w * h].reshape(h, w)
            total = ((np.roll(s, 1, 1) + np.roll(s, -1, 1)) + np.roll(s, 1, 0)) + np.roll(s, -1, 0)
            d[:] = (total * np.float32(0.5) - d) * np.uint32(p["param"]).view(np.float32)
        elif kind == abi.SW_SIM_FIRE_STEP:
            s = state[src:src + w * h].reshape(h, w).astype(np.uint64)
            d = state[dst:dst + w * h].reshape(h, w)
            att = int(p["param"])
            if int(p["flags"]) & abi.SW_SIM_FIRE_SLOW:
                for y in range(h - 1):
                    row, below, new = s[y], s[y + 1], np.zeros(w, np.uint64)
                    new[0] = ((row[w - 1] + row[0] + row[1] + below[0]) * att) >> 20
                    for x in range(1, w - 1):
                        new[x] = ((new[x - 1] + row[x] + row[x + 1] + below[x]) * att) >> 20
                    new[w - 1] = ((new[w - 2] + row[w - 1] + new[0] + below[w - 1]) * att) >> 20
                    d[y] = new & 0xFF
            else:
                r1 = s[1:]
                r2 = np.concatenate([s[2:], s[h - 1:h]])
                total = np.roll(r1, 1, 1) + r1 + np.roll(r1, -1, 1) + r2
                d[:h - 1] = ((total * att) >> 20) & 0xFF
            d[h - 1] = 0
        elif kind == abi.SW_SIM_FIRE_POINTS:
            np.maximum.at(state[dst:dst + w * h], pts["address"].astype(np.int64), pts["value"])
    return state


@pytest.fixture(scope="module")
def sim_scene():
    s = host.Scene(**SIM_MAP)
    yield s
    s.close()


def test_pass_lists_replay_to_oracle_fields(sim_scene):
    scene = sim_scene
    st = scene.static_data()
    effects = {m: scene.simulated_effect(m) for m in range(scene.info().materials)}
    effects = {m: e for m, e in effects.items() if e.kind}
    kinds = sorted(e.kind for e in effects.values())
    assert kinds.count(host.EFFECT_WATER) == 4 and kinds.count(host.EFFECT_FIRE) == 3
    assert {e.color_mode for e in effects.values() if e.kind == host.EFFECT_WATER} == {0, 1, 2, 3}
    assert {e.slow for e in effects.values() if e.kind == host.EFFECT_FIRE} == {0, 1}
    sims = {m: oracle.SimEffect(e) for m, e in effects.items()}
    work = type(st)(st.texels.copy(), st.texture_mips, st.emissive_pixels.copy(), st.emissive_mips, st.lightmaps,
                    st.directional_lightmaps)
    state = np.zeros(scene.simulation_words(), np.uint32)
    fr = host.Frame(scene)
    opts = host.frame_options(320, 240, abi.SW_PIXEL_C32, directional=False)
    total_kinds = np.zeros(9, np.int64)
    for fi in FRAME_SEQUENCE:
        fr.prepare(fi, opts)
        passes, points = fr.sim_passes, fr.sim_points
        assert (np.diff(passes["launch"].astype(np.int64)) >= 0).all()
        total_kinds += np.bincount(passes["kind"], minlength=9)
        replay(passes, points, state)
        t = float(np.float32(np.float32(fi) * np.float32(1.0 / 60.0)))
        for m, sim in sims.items():
            generated_now = sim.update(t, work, m)
            words, step, generated, particles = sim.state()
            h_step, h_cur, h_gen, h_particles = fr.effect_state(m)
            assert (h_step, h_gen, h_particles) == (step, generated, particles), (fi, m)
            e = effects[m]
            area = 1 << (e.resolution_log2[0] + e.resolution_log2[1])
            cur = state[e.state_offset + h_cur * area:e.state_offset + (h_cur + 1) * area]
            assert np.array_equal(cur, words), f"frame {fi} material {m}: {(cur != words).sum()} words differ"
            # a texture pass exactly when the effect generated this frame
            dst = e.output_texture * 5 if e.kind == host.EFFECT_WATER else e.output_emissive * 5
            kind = abi.SW_SIM_WATER_TEXTURE if e.kind == host.EFFECT_WATER else abi.SW_SIM_FIRE_TEXTURE
            tex = passes[(passes["kind"] == kind) & (passes["dst_mip"] == dst)]
            assert tex.size == (1 if generated_now else 0), (fi, m)
    # every kind ran, and fountains kept particles alive
    assert (total_kinds[1:] > 0).all()
    assert any(fr.effect_state(m)[3] > 0 for m, e in effects.items() if e.kind == host.EFFECT_FIRE)


def test_surfaces_switch_to_generated_textures(sim_scene):
    """get_texture / get_emissive_texture: the material's own texture until the effect's first generation."""
    scene = sim_scene
    effects = {m: scene.simulated_effect(m) for m in range(scene.info().materials)}
    water_out = {e.output_texture for e in effects.values() if e.kind == host.EFFECT_WATER}
    fire_out = {e.output_emissive for e in effects.values() if e.kind == host.EFFECT_FIRE}
    fr = host.Frame(scene)
    opts = host.frame_options(320, 240, abi.SW_PIXEL_C32, directional=False)
    seen_tex, seen_em = set(), set()
    for fi in range(0, 90, 1):
        fr.prepare(fi, opts)
        tex = set((fr.surfaces["texture_mip"] // 5).tolist())
        em = set((fr.surfaces["emissive_mip"][fr.surfaces["emissive_mip"] != 0xFFFFFFFF] // 5).tolist())
        if fi <= 1:  # no update step yet: nothing generated
            assert not (tex & water_out) and not (em & fire_out)
        seen_tex |= tex & water_out
        seen_em |= em & fire_out
    assert seen_tex and seen_em
