"""CPU tests of scrolling textures in the host's preparation (MapMaterialsProcessor::update_shifts and
get_texture_shift, map_materials_processor.rs:229-247, 330-334, applied in build_polygons_surfaces,
partial_renderer.rs:1687-1693): the shift of a scrolling material at the frame's time moves its
surfaces' texture start by shift >> mip and nothing else of the frame."""
import numpy as np
import pytest

from sqwheel import abi, host

SCROLLING = 6


def expected_shift(material, frame_index, size):
    # speeds of the generator's scrolling materials; `(speed * t) as i32` (saturating), rem_euclid(size)
    speed = [np.float32(24.0 + 8.0 * material), np.float32(-13.5 if material & 1 else 6.25)]
    t = np.float32(np.float32(frame_index) * np.float32(1.0 / 60.0))
    out = []
    for s in speed:
        x = np.float32(s * t)
        v = int(np.clip(np.trunc(x), -2**31, 2**31 - 1))
        out.append(v % size)
    return out


@pytest.mark.parametrize("frame_index", [0, 1, 59, 61, 1234, 100000])
def test_scrolling_moves_only_the_texture_start(built_libs, frame_index):
    cfg = dict(host.SMALL_MAP, num_dynamic_lights=2)
    plain = host.Frame(host.Scene(**cfg))
    scroll = host.Frame(host.Scene(**dict(cfg, scrolling_materials=SCROLLING)))
    opts = host.frame_options(640, 480, abi.SW_PIXEL_C64, directional=False)
    a = plain.prepare(frame_index, opts)
    b = scroll.prepare(frame_index, opts)
    assert a.surfaces.size == b.surfaces.size and a.total_texels == b.total_texels
    assert np.array_equal(a.draws.view(np.uint8), b.draws.view(np.uint8))  # the draws do not move
    size = host.SMALL_MAP["texture_size"]
    moved = 0
    for sa, sb in zip(a.surfaces, b.surfaces):
        material, mip = divmod(int(sa["texture_mip"]), 5)
        want = [0, 0]
        if material < SCROLLING:
            want = [x >> mip for x in expected_shift(material, frame_index, size)]
        assert list(sb["tc_start"] - sa["tc_start"]) == want
        moved += want != [0, 0]
        for f in abi.SURFACE_DESC.names:
            if f not in ("tc_start", "basis_start"):
                assert np.atleast_1d(sa[f]).tobytes() == np.atleast_1d(sb[f]).tobytes(), f
    if frame_index == 0:
        assert moved == 0
    elif frame_index >= 59:  # at least ~23 texels of mip 0 by then: visible at every mip in use
        assert moved > 0


def restated_mapping(num_materials, animated, times):
    """textures_mapping_table after each update (map_materials_processor.rs:184-227) for the generator's
    framed animations: material m < animated cycles m -> a -> b -> m with a, b appended after the
    num_materials materials (durations 0.25, 0.4, 0.3 s), in float32."""
    base = num_materials
    total = base + 2 * animated

    def next_of(x):
        if x < animated:
            return base + 2 * x
        if x >= base:
            m, j = divmod(x - base, 2)
            return base + 2 * m + 1 if j == 0 else m
        return None

    def duration(x):
        return np.float32(0.25 if x < animated else (0.4 if (x - base) % 2 == 0 else 0.3))

    mapping = list(range(total))
    change = [np.float32(0.0)] * total
    out = []
    for t in times:
        for m in range(total):
            n = next_of(mapping[m])
            if n is not None and t >= change[m]:
                mapping[m] = n
                change[m] = np.float32(change[m] + duration(n))
                if change[m] < t:
                    change[m] = t
        out.append(list(mapping))
    return out


def test_framed_animations_follow_the_mapping_table(built_libs):
    animated = 5
    cfg = dict(host.SMALL_MAP, num_dynamic_lights=1)
    plain = host.Frame(host.Scene(**cfg))
    anim = host.Frame(host.Scene(**dict(cfg, animated_materials=animated)))
    opts = host.frame_options(640, 480, abi.SW_PIXEL_C64, directional=False)
    frames = [0, 1, 2, 15, 16, 30, 31, 45, 100, 101, 5000, 5001, 5002]
    times = [np.float32(np.float32(f) * np.float32(1.0 / 60.0)) for f in frames]
    want = restated_mapping(host.SMALL_MAP["num_materials"], animated, times)
    seen = set()
    for fi, mapping in zip(frames, want):
        a = plain.prepare(fi, opts)
        b = anim.prepare(fi, opts)
        assert a.surfaces.size == b.surfaces.size
        for sa, sb in zip(a.surfaces, b.surfaces):
            if not sa["flags"] & abi.SW_SURF_DIFFUSE_LAYER:
                continue
            material, mip = divmod(int(sa["texture_mip"]), 5)
            assert int(sb["texture_mip"]) == mapping[material] * 5 + mip, f"frame {fi}, material {material}"
            if material < animated:
                seen.add(mapping[material] - material if mapping[material] == material else 1 + (mapping[material] - 16) % 2)
            sa_rest = sa.copy()
            sa_rest["texture_mip"] = sb["texture_mip"]
            if material < animated and mapping[material] != material and (mapping[material] - 16) % 2 == 0:
                # the cycle's first extra frame carries an emissive layer of its own (get_emissive_texture
                # through the mapping table)
                assert int(sb["emissive_mip"]) != 0xFFFFFFFF and int(sb["emissive_mip"]) % 5 == mip
                assert list(sb["emissive_light"]) == [1.5, 0.75, 0.25]
                sa_rest["emissive_mip"], sa_rest["emissive_light"] = sb["emissive_mip"], sb["emissive_light"]
            assert sa_rest.tobytes() == sb.tobytes()
    assert seen == {0, 1, 2}  # every frame of the cycle was shown
