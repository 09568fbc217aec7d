"""Generative texture effects on the GPU (sw_update_textures) against the oracle: random turbulence and
layer passes over material and emissive textures (every blending mode, modulation, skipped additive
layers, tiling with negative offsets), texels equal bit for bit over consecutive calls; whole frames of a
map with turbulent and layered materials through both preparation paths equal the oracle's frames
rendered from the oracle's own effect outputs; malformed pass lists are refused before any launch."""
import numpy as np
import pytest

import oracle
from sqwheel import abi, gpu, host

pytestmark = pytest.mark.gpu

EFFECT_MAP = dict(host.SMALL_MAP, turb_materials=3, layered_materials=3, emissive_frac=0.5)


def random_passes(rng, st, n_materials):
    """Turbulence passes (material and emissive) and layer groups with disjoint destinations and sources."""
    mats = rng.permutation(n_materials)
    dst_mats, src_mats = mats[: n_materials // 2], mats[n_materials // 2:]
    passes, shifts = [], []
    for k, dm in enumerate(dst_mats):
        for mip in range(5):
            dst = int(dm) * 5 + mip
            if k % 3 == 0:  # turbulence from a source of the same size
                p = np.zeros(1, abi.TEXTURE_PASS)
                p["kind"], p["dst_mip"], p["src_mip"] = abi.SW_TEXPASS_TURB, dst, int(src_mats[k % len(src_mats)]) * 5 + mip
                n = int(max(st.texture_mips[dst]["width"], st.texture_mips[dst]["height"]))
                p["shifts_offset"] = sum(len(s) for s in shifts)
                shifts.append(rng.integers(-40, 40, n).astype(np.int32))
                passes.append(p)
            else:  # a layer group: 1..5 layers of any source mip
                for _ in range(int(rng.integers(1, 6))):
                    p = np.zeros(1, abi.TEXTURE_PASS)
                    p["kind"], p["dst_mip"] = abi.SW_TEXPASS_LAYER, dst
                    p["src_mip"] = int(rng.choice(src_mats)) * 5 + int(rng.integers(0, 5))
                    p["blending_mode"] = int(rng.integers(0, 5))
                    p["shift"] = rng.integers(-1000, 1000, 2)
                    p["light"] = rng.choice([1.0, 0.0, 0.005, 0.99, 0.5, 3.0, 127.0], 3)
                    passes.append(p)
    em = st.emissive_mips
    ne = em.size // 5
    if ne >= 2:
        for mip in range(5):
            p = np.zeros(1, abi.TEXTURE_PASS)
            p["kind"] = abi.SW_TEXPASS_TURB | abi.SW_TEXPASS_EMISSIVE
            p["dst_mip"], p["src_mip"] = mip, 5 + mip
            n = int(max(em[mip]["width"], em[mip]["height"]))
            p["shifts_offset"] = sum(len(s) for s in shifts)
            shifts.append(rng.integers(-1000, 1000, n).astype(np.int32))
            passes.append(p)
    return np.concatenate(passes), np.concatenate(shifts) if shifts else np.zeros(0, np.int32)


def test_random_passes_bit_exact(gpu_ok):
    scene = host.Scene(**EFFECT_MAP)
    st = scene.static_data()
    r = gpu.GpuRenderer(st)
    rng = np.random.default_rng(21)
    work = type(st)(st.texels.copy(), st.texture_mips, st.emissive_pixels.copy(), st.emissive_mips, st.lightmaps,
                    st.directional_lightmaps)
    try:
        assert st.emissive_mips.size >= 10
        for call in range(3):  # consecutive calls build on the previous outputs
            passes, shifts = random_passes(rng, st, 16)
            r.update_textures(passes, shifts)
            oracle.apply_texture_passes(passes, shifts, work)
            texels, em = r.read_texels(st.texels.size, st.emissive_pixels.size)
            assert np.array_equal(texels, work.texels), f"call {call}: {(texels != work.texels).sum()} texels differ"
            assert np.array_equal(em, work.emissive_pixels), f"call {call}: emissive pixels differ"
    finally:
        r.close()


def test_malformed_passes_refused(gpu_ok):
    scene = host.Scene(**EFFECT_MAP)
    st = scene.static_data()
    r = gpu.GpuRenderer(st)
    try:
        before = r.read_texels(st.texels.size)[0]
        p = np.zeros(2, abi.TEXTURE_PASS)
        p["kind"] = abi.SW_TEXPASS_LAYER
        p["dst_mip"], p["src_mip"], p["light"] = [0, 10], [5, 0], 1.0  # pass 2 reads pass 1's destination
        cases = [(p, "reads a mip that another pass writes")]
        q = p.copy()
        q["dst_mip"], q["src_mip"] = [0, 0], [5, 10]  # two groups (a layer, a turbulence) writing mip 0
        q["kind"] = [abi.SW_TEXPASS_LAYER, abi.SW_TEXPASS_TURB]
        cases.append((q, "same mip"))
        q = p[:1].copy()
        q["light"] = [1.0, float("nan"), 1.0]
        cases.append((q, "light outside"))
        q = p[:1].copy()
        q["src_mip"] = st.texture_mips.size
        cases.append((q, "bad layer mip"))
        q = p[:1].copy()
        q["kind"] = abi.SW_TEXPASS_TURB
        q["src_mip"] = 6  # a different size
        cases.append((q, "equal power-of-two sizes"))
        for passes, msg in cases:
            with pytest.raises(gpu.SwError, match=msg):
                r.update_textures(passes, np.zeros(512, np.int32))
        assert np.array_equal(r.read_texels(st.texels.size)[0], before)
    finally:
        r.close()


@pytest.mark.parametrize("gpu_prep", [True, False])
def test_effect_frames(gpu_ok, gpu_prep):
    scene = host.Scene(**dict(EFFECT_MAP, emissive_frac=0.0, num_dynamic_lights=2))
    st = scene.static_data()
    work = type(st)(st.texels.copy(), st.texture_mips, st.emissive_pixels.copy(), st.emissive_mips, st.lightmaps,
                    st.directional_lightmaps)
    fr = host.Frame(scene)
    hr = host.HostRenderer(scene)
    hr.set_gpu_prep(gpu_prep)
    glib = gpu.load_library()
    w, h = 480, 270
    opts = host.frame_options(w, h, abi.SW_PIXEL_C64, directional=False)
    info = scene.info()
    outputs = {scene.texture_effect(m)[1] for m in range(info.materials)} - {-1}
    seen = 0
    try:
        for fi in range(0, 48, 3):  # in order: the effects' state carries from frame to frame
            fr.prepare(fi, opts)
            oracle.apply_texture_passes(fr.texture_passes, fr.texture_shifts, work)
            seen += int(np.isin(fr.surfaces["texture_mip"] // 5, list(outputs)).sum())
            arena = oracle.build_surfaces(work, fr.surfaces, fr.lights, fr.params, fr.total_texels, num_threads=8)
            want = np.zeros((h, w), np.uint64)
            assert oracle.rasterize(fr.draws, fr.vertices, arena, fr.params, want) == 0
            got = np.zeros((h, w), np.uint64)
            hr.render_frame(fi, opts, out=got)
            assert np.array_equal(want, got), f"frame {fi}: {(want != got).sum()} pixels differ"
            texels = np.empty(st.texels.size, np.uint64)
            assert glib.sw_read_texels(hr.context(), abi.ptr(texels), texels.size, None, 0) == abi.SW_OK
            assert np.array_equal(texels, work.texels), f"frame {fi}: effect outputs differ"
        assert seen > 0
    finally:
        hr.close()
