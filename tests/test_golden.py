"""Golden fixtures (tests/golden/*.npz, made by tests/golden/make_golden.py) and known-answer tests.

CPU: the oracle reproduces every fixture bit for bit, and small cases whose answers follow by hand from
the reference's formulas (coverage rule, blend modes, tonemapping, exposure update, a lightmapped
surface) come out of the oracle as computed here.
GPU: the CUDA path reproduces every fixture through the C ABI.
"""
import glob
import os

import numpy as np
import pytest

import oracle
from sqwheel import abi, gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))


def _load(path):
    return dict(np.load(path))


def _static(d):
    return gpu.StaticData(d["texels"], d["texture_mips"], d["emissive_pixels"], d["emissive_mips"], d["lightmaps"],
                          d["directional_lightmaps"])


def _frame_params(b):
    return abi.FrameParams.from_buffer_copy(bytes(b))


def _post_config(b):
    return abi.PostConfig.from_buffer_copy(bytes(b))


def _kind(path):
    return os.path.basename(path).split("_")[0]


def test_fixtures_present():
    kinds = {_kind(p) for p in GOLDEN}
    assert kinds == {"surfaces", "raster", "post"}, GOLDEN


# ---------------------------------------------------------------- oracle regression (CPU)

@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
def test_oracle_reproduces_fixture(built_libs, path):
    d = _load(path)
    kind = _kind(path)
    if kind == "surfaces":
        got = oracle.build_surfaces(_static(d), d["surfaces"], d["lights"], _frame_params(d["frame_params"]),
                                    int(d["total_texels"]), num_threads=3)
        assert np.array_equal(got, d["want"])
    elif kind == "raster":
        fb = d["framebuffer_in"].copy()
        fp = _frame_params(d["frame_params"])
        sky = d.get("skybox64" if fp.pixel_format == abi.SW_PIXEL_C64 else "skybox32")
        bad = oracle.rasterize(d["draws"], d["vertices"], d["arena"], fp, fb, skybox=sky)
        assert bad == 0 and np.array_equal(fb, d["want"])
    else:
        cfg = _post_config(d["config"])
        exposure = 1.0
        for i in range(d["hdr"].shape[0]):
            ldr, exposure, _ = oracle.postprocess(cfg, d["hdr"][i], 1.0 / 60.0, tuple(d["color_modulate"]), exposure)
            assert np.array_equal(ldr, d["want"][i])
            assert np.float32(exposure) == d["exposures"][i]


# ---------------------------------------------------------------- known answers (CPU)

def _quad_draw(mode, blend, x0=10, y0=10, x1=20, y1=20, tex=(10, 10)):
    """Axis-aligned quad (x0, y0)-(x1, y1) in pixels, clockwise (y down), sampling a tex-sized surface at
    offset 0 with tc = (x - x0, y - y0); equations pre-scaled by z_scale = 1/32 as draw_polygon does
    for inv_z = 1 (partial_renderer.rs:4106-4109)."""
    d = np.zeros(1, abi.DRAW_CMD)
    d["first_vertex"], d["vertex_count"], d["mode"], d["blend"] = 0, 4, mode, blend
    s = np.float32(1.0 / 32.0)
    d["depth_eq"] = (0.0, 0.0, s)
    d["tc_eq"] = (s, 0.0, 0.0, s, -x0 * s, -y0 * s)
    d["tex_size"] = tex
    v = np.zeros(4, abi.VERTEX16)
    v["x"] = [x0 << 16, x1 << 16, x1 << 16, x0 << 16]
    v["y"] = [y0 << 16, y0 << 16, y1 << 16, y1 << 16]
    return d, v


@pytest.mark.parametrize("mode", [abi.SW_RASTER_FULL_PERSPECTIVE, abi.SW_RASTER_LINE_Z_CORRECTED, abi.SW_RASTER_AFFINE])
def test_known_answer_coverage(built_libs, mode):
    """A span covers pixels whose centres lie inside: rows [round(y0), round(y1)), columns
    [floor(x_left + 1/2), floor(x_right + 1/2)) (rasterizer.rs:316-331), so the quad (10,10)-(20,20)
    fills exactly the 10 x 10 pixels [10, 20) x [10, 20)."""
    c = np.uint32(0x11223344)
    arena = np.full(100, c, np.uint32)
    d, v = _quad_draw(mode, 0)
    fp = gpu.frame_params(32, 32, abi.SW_PIXEL_C32, (0, 0, 0))
    fb = np.zeros((32, 32), np.uint32)
    assert oracle.rasterize(d, v, arena, fp, fb) == 0
    want = np.zeros((32, 32), np.uint32)
    want[10:20, 10:20] = c
    assert np.array_equal(fb, want)


def _lanes(c):
    return [(int(c) >> s) & 255 for s in (0, 8, 16, 24)]


def _pack(l):
    return np.uint32(l[0] | (l[1] << 8) | (l[2] << 16) | (l[3] << 24))


def _blend_answer(blend, dst, src):
    """write_into_framebuffer's blends (rasterizer.rs:1511-1536) with the generic colour primitives:
    average rounds down per byte (color.rs:46-49), additive saturates per byte, alpha test passes when
    A > 0x7F (abstract_color.rs:42-46), alpha blend (dst*(255 - a) + src*a) >> 8 per lane with a = src
    alpha (abstract_color.rs:30-40)."""
    D, S = _lanes(dst), _lanes(src)
    if blend == abi.SW_BLEND_NONE:
        return src
    if blend == abi.SW_BLEND_AVERAGE:
        return _pack([(x + y) >> 1 for x, y in zip(D, S)])
    if blend == abi.SW_BLEND_ADDITIVE:
        return _pack([min(x + y, 255) for x, y in zip(D, S)])
    if blend == abi.SW_BLEND_ALPHA_TEST:
        return src if S[3] > 0x7F else dst
    a = S[3]
    return _pack([min((x * (255 - a) + y * a) >> 8, 255) for x, y in zip(D, S)])


@pytest.mark.parametrize("blend", [abi.SW_BLEND_NONE, abi.SW_BLEND_AVERAGE, abi.SW_BLEND_ADDITIVE, abi.SW_BLEND_ALPHA_TEST,
                                   abi.SW_BLEND_ALPHA_BLEND])
@pytest.mark.parametrize("src", [0x80FF00FA, 0x7FFF00FA, 0xFF0A0B0C, 0x00FFFFFF])
def test_known_answer_blends(built_libs, blend, src):
    dst = np.uint32(0x40C86432)
    src = np.uint32(src)
    arena = np.full(100, src, np.uint32)
    d, v = _quad_draw(abi.SW_RASTER_AFFINE, blend)
    fp = gpu.frame_params(32, 32, abi.SW_PIXEL_C32, (0, 0, 0))
    fb = np.full((32, 32), dst, np.uint32)
    assert oracle.rasterize(d, v, arena, fp, fb) == 0
    assert fb[15, 15] == _blend_answer(blend, dst, src), hex(int(fb[15, 15]))
    assert fb[5, 5] == dst


def test_known_answer_tonemap_and_exposure(built_libs):
    """Without bloom, a uniform HDR frame c maps to c / (c/255 + 1/(exposure*modulate)) per lane
    (postprocessor.rs:997-1024) truncated to a byte, alpha 255: c = 255 at exposure 1 gives 127.
    The exposure then follows update_exposure (postprocessor.rs:206-223, 1047-1051)."""
    cfg = abi.PostConfig.default()
    cfg.bloom_sigma = 0.0
    hdr = np.full((16, 24), np.uint64(255 | (255 << 16) | (255 << 32)), np.uint64)
    ldr, exposure, avg = oracle.postprocess(cfg, hdr, 1.0 / 60.0, (1.0, 1.0, 1.0), 1.0)
    assert np.all(ldr == np.uint32(0xFF7F7F7F))
    assert np.all(avg[:3] == 255.0)
    f32 = np.float32
    b_raw = f32(f32(f32(255.0) + f32(255.0)) + f32(255.0)) * f32(0.33)
    b = f32(min(max(b_raw, f32(1.0 / 1024.0)), f32(65536.0))) / f32(255.0)
    target = f32(f32(f32(b / f32(cfg.zero_level_brightness)) ** f32(cfg.brightness_scale_power)) * f32(0.5)
                 * f32(cfg.base_brightness) / b)
    clamped = f32(min(max(target, f32(cfg.min_exposure)), f32(cfg.max_exposure)))
    mix = np.exp(f32(-cfg.exposure_update_speed) * f32(1.0 / 60.0), dtype=np.float32)
    want = np.exp(f32(np.log(f32(1.0)) * mix + np.log(clamped) * f32(f32(1.0) - mix)), dtype=np.float32)
    assert exposure == pytest.approx(float(want), rel=2e-6)
    zero = np.zeros((16, 24), np.uint64)
    ldr0, _, _ = oracle.postprocess(cfg, zero, 1.0 / 60.0, (1.0, 1.0, 1.0), 1.0)
    assert np.all(ldr0 == np.uint32(0xFF000000))


def test_known_answer_lightmapped_surface(built_libs):
    """A diffuse-only surface under a constant simple lightmap L = 2 (no normal map, no lights): every
    texel is diffuse x L per colour lane (surfaces.rs:551-572, 833-842), truncated to a byte."""
    from sqwheel import synth
    diffuse = np.full((8, 8), np.uint32(0xFF193264), np.uint32)  # a=255, r=25, g=50, b=100
    packed = synth.pack_normal_roughness(np.tile(np.array([0.0, 0.0, 1.0], np.float32), (8, 8, 1)),
                                         np.ones((8, 8), np.float32))
    texels = synth.make_texels(diffuse, packed).ravel()
    mips = np.zeros(1, abi.TEXTURE_MIP)
    mips[0] = (0, 8, 8, 0, 0)
    lightmaps = np.full((10, 3), 2.0, np.float32)
    st = gpu.StaticData(texels, mips, lightmaps=lightmaps)
    s = np.zeros(1, abi.SURFACE_DESC)
    s["basis_u"], s["basis_v"], s["basis_normal"] = (1, 0, 0), (0, 1, 0), (0, 0, 1)
    s["size"] = (6, 5)
    s["texture_mip"] = 0
    s["emissive_mip"] = abi.SW_NO_EMISSIVE
    s["lightmap_offset"], s["lightmap_size"], s["lightmap_scale_log2"] = 1, (3, 3), 4
    s["flags"] = abi.SW_SURF_DIFFUSE_LAYER
    fp = gpu.frame_params(64, 64, abi.SW_PIXEL_C32, (0, 0, 100), directional=False)
    out = oracle.build_surfaces(st, s, None, fp, 30, num_threads=1)
    rgb = out & np.uint32(0x00FFFFFF)
    assert np.all(rgb == np.uint32((50 << 16) | (100 << 8) | 200)), [hex(int(x)) for x in out[:4]]


# Out-of-range configurations and what Postprocessor::synchronize_config (postprocessor.rs:958-977)
# clamps them to before every frame.
CLAMP_CASES = [
    (dict(bloom_sigma=100.0), dict(bloom_sigma=40.0)),
    (dict(bloom_sigma=-3.0), dict(bloom_sigma=0.0)),
    (dict(bloom_buffer_scale_log2=0), dict(bloom_buffer_scale_log2=1)),
    (dict(bloom_buffer_scale_log2=7), dict(bloom_buffer_scale_log2=3)),
    (dict(bloom_scale=0.001), dict(bloom_scale=1.0 / 16.0)),
    (dict(bloom_scale=3.0), dict(bloom_scale=0.5)),
    (dict(min_exposure=100.0, max_exposure=0.1), dict(min_exposure=16.0, max_exposure=1.0)),
    (dict(exposure_update_speed=float("nan"), base_brightness=9.0), dict(exposure_update_speed=0.5, base_brightness=2.0)),
    (dict(zero_level_brightness=1e-6, brightness_scale_power=4.0), dict(zero_level_brightness=1.0 / 16.0, brightness_scale_power=0.5)),
]


def _config(**kw):
    c = abi.PostConfig.default()
    for k, v in kw.items():
        setattr(c, k, v)
    return c


@pytest.mark.parametrize("given,clamped", CLAMP_CASES)
def test_oracle_clamps_config(built_libs, given, clamped):
    """An out-of-range configuration gives exactly the frames and exposures of its clamped form."""
    rng = np.random.default_rng(5)
    lanes = rng.integers(0, 3000, (60, 88, 4), dtype=np.uint64)
    hdr = lanes[..., 0] | (lanes[..., 1] << 16) | (lanes[..., 2] << 32) | (np.uint64(255) << 48)
    e_a = e_b = 1.0
    for _ in range(3):
        a, e_a, _ = oracle.postprocess(_config(**given), hdr, 1.0 / 60.0, (1.0, 1.0, 1.0), e_a)
        b, e_b, _ = oracle.postprocess(_config(**clamped), hdr, 1.0 / 60.0, (1.0, 1.0, 1.0), e_b)
        assert np.array_equal(a, b)
        assert e_a == e_b


@pytest.mark.gpu
@pytest.mark.parametrize("given,clamped", CLAMP_CASES)
def test_gpu_clamps_config(gpu_ok, given, clamped):
    """The GPU postprocessor clamps the same way: frames and exposures equal the oracle's."""
    from sqwheel import synth
    rng = np.random.default_rng(6)
    lanes = rng.integers(0, 3000, (60, 88, 4), dtype=np.uint64)
    hdr = lanes[..., 0] | (lanes[..., 1] << 16) | (lanes[..., 2] << 32) | (np.uint64(255) << 48)
    cfg = _config(**given)
    r = gpu.GpuRenderer(synth.BatchedSurfaces(seed=1, count=1, max_side=8).static_data())
    exposure = 1.0
    try:
        for _ in range(3):
            want, exposure, _ = oracle.postprocess(cfg, hdr, 1.0 / 60.0, (1.0, 1.0, 1.0), exposure)
            r.set_framebuffer(hdr, abi.SW_PIXEL_C64)
            got = np.zeros_like(want)
            r.postprocess(cfg, 1.0 / 60.0, (1.0, 1.0, 1.0), out=got)
            assert np.array_equal(want, got)
            assert r.exposure() == np.float32(exposure)
    finally:
        r.close()


# ---------------------------------------------------------------- CUDA path (GPU)

@pytest.mark.gpu
@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
def test_gpu_reproduces_fixture(gpu_ok, path):
    d = _load(path)
    kind = _kind(path)
    if kind == "surfaces":
        st = _static(d)
        r = gpu.GpuRenderer(st)
        try:
            fp = _frame_params(d["frame_params"])
            r.frame_begin(fp, d["lights"])
            r.submit_surfaces(d["surfaces"], int(d["total_texels"]))
            assert np.array_equal(r.read_surfaces(int(d["total_texels"]), fp.pixel_format), d["want"])
        finally:
            r.close()
        return
    r = gpu.GpuRenderer(gpu.StaticData(np.zeros(1, np.uint64), np.zeros(0, abi.TEXTURE_MIP)))
    try:
        if kind == "raster":
            fp = _frame_params(d["frame_params"])
            fp.use_directional_lightmaps = 0  # no lightmaps in this context; the raster pass does not read them
            fb_in = d["framebuffer_in"]
            r.frame_begin(fp, None)
            r.set_framebuffer(fb_in, fp.pixel_format)
            r.set_surfaces(d["arena"])
            if "skybox32" in d:
                r.set_skybox(d["skybox32"], d["skybox64"])
            r.submit_draws(d["draws"], d["vertices"])
            got = np.zeros_like(fb_in)
            r.render(got)
            assert np.array_equal(got, d["want"])
        else:
            cfg = _post_config(d["config"])
            for i in range(d["hdr"].shape[0]):
                r.set_framebuffer(d["hdr"][i], abi.SW_PIXEL_C64)
                got = np.zeros(d["want"][i].shape, np.uint32)
                r.postprocess(cfg, 1.0 / 60.0, tuple(float(x) for x in d["color_modulate"]), out=got)
                assert np.array_equal(got, d["want"][i])
                assert np.float32(r.exposure()) == d["exposures"][i]
    finally:
        r.close()
