"""GPU parity of the surface builder against the oracle: bit-exact for every variant
(simple / directional lightmap, normal map or not, no specular / dielectric / metal, dynamic lights,
emissive layer, Color32 and Color64)."""
import numpy as np
import pytest

import oracle
from sqwheel import abi, gpu, synth

pytestmark = pytest.mark.gpu


def build_both(b, use_directional=True):
    fp = gpu.frame_params(64, 64, b.pixel_format, b.cam_pos, directional=use_directional)
    want = oracle.build_surfaces(b.static_data(), b.surfaces, b.lights, fp, b.total_texels, num_threads=8)
    r = gpu.GpuRenderer(b.static_data())
    try:
        r.frame_begin(fp, b.lights)
        r.submit_surfaces(b.surfaces, b.total_texels)
        got = r.read_surfaces(b.total_texels, b.pixel_format)
    finally:
        r.close()
    return want, got


def assert_exact(want, got, b):
    if np.array_equal(want, got):
        return
    bad = np.nonzero(want != got)[0]
    starts = b.surfaces["out_offset"].astype(np.int64)
    s = int(np.searchsorted(starts, bad[0], side="right") - 1)
    raise AssertionError(f"{bad.size} texels differ; first at {bad[0]} (surface {s}, desc {b.surfaces[s]}): "
                         f"want {want[bad[0]]:#x} got {got[bad[0]]:#x}")


@pytest.mark.parametrize("fmt", [abi.SW_PIXEL_C32, abi.SW_PIXEL_C64])
@pytest.mark.parametrize("directional", [True, False])
def test_surfaces_bit_exact(gpu_ok, fmt, directional):
    b = synth.BatchedSurfaces(seed=11 + fmt + 2 * directional, count=160, max_side=96, num_lights=5,
                              emissive_frac=0.2, directional=directional, pixel_format=fmt)
    want, got = build_both(b, directional)
    assert_exact(want, got, b)


def test_surfaces_all_material_kinds(gpu_ok):
    """Every texture-flag combination appears: plain, normal-mapped, dielectric, metal."""
    b = synth.BatchedSurfaces(seed=5, count=96, max_side=64, num_lights=6, pixel_format=abi.SW_PIXEL_C64)
    flags = b.texture_mips["flags"][b.surfaces["texture_mip"]]
    kinds = set((int(f) & 6) for f in flags)
    assert {0, 2, 6} <= kinds
    want, got = build_both(b)
    assert_exact(want, got, b)


def test_surfaces_large_lightmaps(gpu_ok):
    """Surfaces up to 512 texels: lightmap rows longer than the reference's 19-entry line buffer."""
    b = synth.BatchedSurfaces(seed=9, count=12, min_side=300, max_side=512, pixel_format=abi.SW_PIXEL_C64)
    assert b.surfaces["lightmap_size"][:, 0].max() > 19
    want, got = build_both(b)
    assert_exact(want, got, b)


def test_surfaces_invalid_descriptor_rejected(gpu_ok):
    b = synth.BatchedSurfaces(seed=2, count=8, max_side=32)
    r = gpu.GpuRenderer(b.static_data())
    try:
        r.frame_begin(gpu.frame_params(64, 64, b.pixel_format, b.cam_pos), b.lights)
        s = b.surfaces.copy()
        s["lightmap_size"][3, 0] = 1  # reads past the lightmap row
        with pytest.raises(gpu.SwError):
            r.submit_surfaces(s, b.total_texels)
        s = b.surfaces.copy()
        s["out_offset"][5] = b.total_texels  # outside the arena
        with pytest.raises(gpu.SwError):
            r.submit_surfaces(s, b.total_texels)
        # The context stays usable after a rejected call.
        r.submit_surfaces(b.surfaces, b.total_texels)
        r.sync()
    finally:
        r.close()
