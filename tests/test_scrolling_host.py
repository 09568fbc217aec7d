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
