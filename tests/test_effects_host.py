"""Generative texture effects on the CPU: the oracle's turbulence shift table against a float64
restatement, the host's per-frame pass lists against the oracle (turbulence tables bit for bit, layered
animation passes by their invariants), surfaces of effect materials reading the effects' output
textures, and the oracle's pass application against a numpy restatement of the layer blending."""
import math

import numpy as np
import pytest

import oracle
from sqwheel import abi, host

pytestmark = pytest.mark.usefixtures("built_libs")

EFFECT_MAP = dict(host.SMALL_MAP, turb_materials=3, layered_materials=3)
TAU = np.float32(2 * math.pi)


def test_turb_shift_table_against_float64():
    rng = np.random.default_rng(3)
    checked = 0
    for _ in range(60):
        amp, wl, fq, t = (float(np.float32(v)) for v in (rng.uniform(1, 9), rng.uniform(8, 100), rng.uniform(0.1, 2), rng.uniform(0, 30)))
        mip = int(rng.integers(0, 5))
        w = 1 << int(rng.integers(2, 9))
        buf = np.full(w, 12345, np.int32)
        oracle.turb_shifts(amp, wl, fq, t, w, w, mip, buf)
        ms = np.float32(1) / np.float32(1 << mip)
        amp_c = np.float32(ms * np.float32(amp))
        fs = np.float32(TAU / np.float32(np.float32(wl) * ms))
        ts = np.float32(np.float32(np.float32(t) * np.float32(fq)) * TAU)
        arg = (np.arange(w, dtype=np.float32) * fs + ts).astype(np.float32)
        v = np.sin(arg.astype(np.float64)) * float(amp_c)
        near_half = np.abs(np.abs(v) % 1.0 - 0.5) < 1e-3
        want = np.where(v >= 0, np.floor(v + 0.5), -np.floor(-v + 0.5)).astype(np.int32)
        assert np.array_equal(buf[~near_half], want[~near_half])
        checked += int((~near_half).sum())
    assert checked > 1000
    # entries at and beyond w keep what the buffer held (the effect's buffer persists between calls)
    buf = np.full(64, 7, np.int32)
    oracle.turb_shifts(3.0, 20.0, 1.0, 0.5, 16, 64, 0, buf)
    assert (buf[16:] == 7).all() and not (buf[:16] == 7).all()


@pytest.fixture(scope="module")
def effect_scene():
    s = host.Scene(**EFFECT_MAP)
    yield s
    s.close()


def test_host_turb_tables_match_oracle(effect_scene):
    scene = effect_scene
    info = scene.info()
    st = scene.static_data()
    effects = {m: scene.texture_effect(m) for m in range(info.materials)}
    turb = {m: e for m, e in effects.items() if e[0] == 1}
    layered = {m: e for m, e in effects.items() if e[0] == 2}
    assert len(turb) == 3 and len(layered) == 3
    fr = host.Frame(scene)
    for fi in (0, 7, 33):
        fr.prepare(fi, host.frame_options(320, 240, abi.SW_PIXEL_C32, directional=False))
        t = np.float32(np.float32(fi) * np.float32(1.0 / 60.0))  # the frame's time, frame_index / 60 in f32
        passes, shifts = fr.texture_passes, fr.texture_shifts
        for m, (_, out_tex, _, (amp, wl, fq)) in turb.items():
            for mip in range(5):
                sel = passes[passes["dst_mip"] == out_tex * 5 + mip]
                assert sel.size == 1 and sel["kind"][0] == abi.SW_TEXPASS_TURB and sel["src_mip"][0] == m * 5 + mip
                w, h = (int(v) for v in st.texture_mips[m * 5 + mip][["width", "height"]])
                want = np.zeros(max(w, h), np.int32)
                oracle.turb_shifts(amp, wl, fq, float(t), w, h, mip, want)
                off = int(sel["shifts_offset"][0])
                assert np.array_equal(shifts[off:off + max(w, h)], want), (fi, m, mip)
        for m, (_, out_tex, nl, _) in layered.items():
            per_mip = [passes[passes["dst_mip"] == out_tex * 5 + mip] for mip in range(5)]
            assert all(p.size == nl for p in per_mip) and nl == 4
            for mip in range(5):
                p = per_mip[mip]
                assert (p["kind"] == abi.SW_TEXPASS_LAYER).all()
                assert np.array_equal(p["shift"], per_mip[0]["shift"] >> mip)  # (f(t) as i32) >> mip
                assert np.array_equal(p["light"], per_mip[0]["light"]) and (p["light"] >= 0).all() and (p["light"] <= 127).all()
                assert list(p["blending_mode"]) == [abi.SW_BLEND_NONE, abi.SW_BLEND_ADDITIVE, abi.SW_BLEND_ALPHA_BLEND,
                                                    abi.SW_BLEND_ALPHA_TEST]
                assert p["src_mip"][0] == m * 5 + mip
            assert (per_mip[0]["light"][0] == 1.0).all()  # the base layer is not modulated


def test_effect_surfaces_read_output_textures(effect_scene):
    scene = effect_scene
    info = scene.info()
    outputs = {scene.texture_effect(m)[1] for m in range(info.materials)} - {-1}
    fr = host.Frame(scene)
    seen = set()
    for fi in range(0, 64, 3):
        fr.prepare(fi, host.frame_options(320, 240, abi.SW_PIXEL_C32, directional=False))
        tex = set((fr.surfaces["texture_mip"] // 5).tolist())
        # effect materials' surfaces read the effect's output slot, never past it
        assert all(t < info.materials or t in outputs for t in tex)
        seen |= tex & outputs
    assert seen, "no effect material in view"


def _np_layer(dst, src, shift, light, blend):
    """numpy restatement of apply_texture_layer_impl_2 over one mip (dst, src: 2-D uint64 arrays)."""
    dh, dw = dst.shape
    sh, sw = src.shape
    ys = (shift[1] + np.arange(dh)) % sh
    xs = (shift[0] + np.arange(dw)) % sw
    t = src[ys][:, xs]
    td = (t & 0xFFFFFFFF).astype(np.int64)
    dd = (dst & 0xFFFFFFFF).astype(np.int64)
    lanes = lambda c: np.stack([(c >> (8 * i)) & 0xFF for i in range(4)], -1)
    modulate = any(l < np.float32(0.98) or l > np.float32(1.02) for l in light)
    lv = np.array([int(np.float32(light[2]) * np.float32(256)), int(np.float32(light[1]) * np.float32(256)),
                   int(np.float32(light[0]) * np.float32(256)), 0], np.int64)
    m = (lanes(td) * lv) >> 8 if modulate else lanes(td)
    d = lanes(dd)
    pack = lambda l: sum(np.clip(np.where(l[..., i] < 0, 1 << 40, l[..., i]), 0, 255) << (8 * i) for i in range(4))
    tn, dn = t >> np.uint64(32), dst >> np.uint64(32)
    if blend == abi.SW_BLEND_NONE:
        out_d, out_n = pack(m), tn
    elif blend == abi.SW_BLEND_AVERAGE:
        out_d = pack((m + d) >> 1) if modulate else (((td ^ dd) & 0xFEFEFEFE) >> 1) + (td & dd)
        out_n = dn
    elif blend == abi.SW_BLEND_ADDITIVE:
        out_d, out_n = pack(m + d), dn
    elif blend == abi.SW_BLEND_ALPHA_TEST:
        keep = (td & 0xFF000000) > 0x7F000000
        out_d = np.where(keep, pack(m), dd)
        out_n = np.where(keep, tn, dn)
    else:
        a = (td >> 24)[..., None]
        out_d, out_n = pack((m * a + d * (255 - a)) >> 8), dn
    return (np.asarray(out_n, np.uint64) << np.uint64(32)) | np.asarray(out_d, np.uint64)


def test_oracle_layers_against_numpy(effect_scene):
    st = effect_scene.static_data()
    rng = np.random.default_rng(11)
    mips = st.texture_mips
    dst_mip, src_mip = 5, 9  # material 1 mip 0 (128 x 128) <- material 1 mip 4 (8 x 8): tiling
    for blend in range(5):
        for light in ([1.0, 1.0, 1.0], [0.5, 2.0, 0.0], [1.01, 0.99, 1.0], [0.004, 0.003, 0.0]):
            shift = [int(rng.integers(-300, 300)), int(rng.integers(-300, 300))]
            texels = st.texels.copy()
            texels[:] ^= rng.integers(0, 1 << 62, texels.size, dtype=np.uint64) & np.uint64(0xFF000000)  # random alpha
            d = mips[dst_mip]
            s = mips[src_mip]
            dst = texels[int(d["offset"]):int(d["offset"]) + int(d["width"] * d["height"])].reshape(int(d["height"]), int(d["width"]))
            src = texels[int(s["offset"]):int(s["offset"]) + int(s["width"] * s["height"])].reshape(int(s["height"]), int(s["width"]))
            zero = all(l <= 1 / 128 for l in light)
            want = dst.copy() if (blend == abi.SW_BLEND_ADDITIVE and zero) else _np_layer(dst.copy(), src.copy(), shift, light, blend)
            p = np.zeros(1, abi.TEXTURE_PASS)
            p["kind"], p["dst_mip"], p["src_mip"], p["blending_mode"] = abi.SW_TEXPASS_LAYER, dst_mip, src_mip, blend
            p["shift"], p["light"] = shift, light
            work = type(st)(texels, st.texture_mips, st.emissive_pixels.copy(), st.emissive_mips, st.lightmaps, st.directional_lightmaps)
            oracle.apply_texture_passes(p, None, work)
            got = work.texels[int(d["offset"]):int(d["offset"]) + int(d["width"] * d["height"])].reshape(dst.shape)
            assert np.array_equal(got, want), (blend, light)
