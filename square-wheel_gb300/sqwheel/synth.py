"""Seeded synthetic inputs for the GB300 rendering path.

No map, texture or lightmap assets ship with the reference (its demo textures and compiled maps are not
in its repository), so every input here is generated from a seed:
  - material textures: value noise + checker diffuse, height-field normal maps, roughness; packed as the
    reference's TextureElement and mip-mapped as build_texture_mip does (src/square_wheel/textures.rs:
    288-362);
  - directional lightmap texels with the distributions of the batched-surface workload (ambient
    U[0,4], tangent-space direction x intensity U[0,8], deviation U[0,1], normalised colour);
  - batched surface descriptors: sides log-uniform in [4, 512], mips 0..3.
"""
import numpy as np

from . import abi

NUM_MIPS = 5  # MAX_MIP + 1, textures.rs:6-7


# ---- TextureElement packing (textures.rs:20-62, fast_math.rs:419-438 generic) ----

def pack_normal_roughness(n, roughness):
    """PackedNormalRoughness::pack with the generic pack_f32x4_into_bytes (truncating)."""
    v = np.stack([n[..., 0], n[..., 1], n[..., 2], roughness], axis=-1).astype(np.float32) * np.float32(127.0)
    v = np.clip(v, np.float32(-127.0), np.float32(127.0))
    b = np.trunc(v).astype(np.int32) & 0xFF
    return (b[..., 0] | (b[..., 1] << 8) | (b[..., 2] << 16) | (b[..., 3] << 24)).astype(np.uint32)


def unpack_normal_roughness(p):
    p = p.astype(np.uint32)
    out = []
    for i in range(4):
        s = ((p << np.uint32(24 - 8 * i)).astype(np.int32) >> 24).astype(np.float32)
        out.append(s * np.float32(1.0 / 127.0))
    return np.stack(out[:3], axis=-1), out[3]


def make_texels(diffuse, packed):
    return (diffuse.astype(np.uint64) | (packed.astype(np.uint64) << np.uint64(32))).astype(np.uint64)


def average4(c):
    """Color32::get_average_4 over the 2x2 blocks of a (h, w) uint32 image (color.rs:51-71)."""
    p = [c[0::2, 0::2], c[1::2, 0::2], c[0::2, 1::2], c[1::2, 1::2]]
    s0 = sum((x & 0xFF).astype(np.uint64) for x in p)
    s1 = sum((x & 0xFF00).astype(np.uint64) for x in p)
    s2 = sum((x & 0xFF0000).astype(np.uint64) for x in p)
    s3 = sum(((x & 0xFF000000) >> 2).astype(np.uint64) for x in p)
    r = (s0 >> 2) | ((s1 >> 2) & 0xFF00) | ((s2 >> 2) & 0xFF0000) | (s3 & 0xFF000000)
    return r.astype(np.uint32)


def build_mip(diffuse, packed):
    """build_texture_mip (textures.rs:309-362) for one level."""
    d = average4(diffuse)
    normals, rough = unpack_normal_roughness(packed)
    q = [(0, 0), (1, 0), (0, 1), (1, 1)]  # p00, p01, p10, p11 in the reference's naming
    ns = None
    rs = None
    for dy, dx in q:
        n = normals[dy::2, dx::2]
        r = rough[dy::2, dx::2]
        ns = n if ns is None else ns + n
        rs = r if rs is None else rs + r
    ln = np.sqrt((ns[..., 0] * ns[..., 0] + ns[..., 1] * ns[..., 1]) + ns[..., 2] * ns[..., 2]).astype(np.float32)
    ln = np.maximum(ln, np.float32(1e-6))
    nn = ns / ln[..., None]
    half_dev_cos = ln * np.float32(0.25)
    dev = (np.float32(1.0) - half_dev_cos) / np.float32(0.5)
    r = np.clip(rs * np.float32(0.25) + dev, np.float32(1.0 / 126.0), np.float32(1.0)).astype(np.float32)
    return d, pack_normal_roughness(nn.astype(np.float32), r)


def value_noise(rng, size, cells):
    g = rng.random((cells + 1, cells + 1), dtype=np.float32)
    x = np.linspace(0, cells, size, endpoint=False, dtype=np.float32)
    i = x.astype(np.int32)
    f = x - i
    f = f * f * (3 - 2 * f)
    a = g[i][:, i]
    b = g[i][:, i + 1]
    c = g[i + 1][:, i]
    d = g[i + 1][:, i + 1]
    fy = f[:, None]
    fx = f[None, :]
    return (a * (1 - fx) + b * fx) * (1 - fy) + (c * (1 - fx) + d * fx) * fy


def make_texture(rng, size, normal_map=True, roughness=1.0, metal=False):
    """One material: mip chain of (diffuse, packed) arrays plus flags."""
    n1 = value_noise(rng, size, 8)
    n2 = value_noise(rng, size, 32)
    yy, xx = np.mgrid[0:size, 0:size]
    checker = (((xx // (size // 8)) + (yy // (size // 8))) & 1).astype(np.float32)
    base = rng.random(3, dtype=np.float32) * 0.6 + 0.3
    lum = 0.55 + 0.3 * n1 + 0.15 * n2 - 0.12 * checker
    rgb = np.clip(lum[..., None] * base[None, None, :] * 255.0, 0, 255).astype(np.uint32)
    alpha = np.full((size, size), 255, np.uint32)
    diffuse = (alpha << 24) | (rgb[..., 0] << 16) | (rgb[..., 1] << 8) | rgb[..., 2]
    h = n1 * 2.0 + n2 * 0.5 + checker * 0.5
    gx = (np.roll(h, -1, 1) - np.roll(h, 1, 1)) * (size / 64.0)
    gy = (np.roll(h, -1, 0) - np.roll(h, 1, 0)) * (size / 64.0)
    if normal_map:
        n = np.stack([-gx, -gy, np.ones_like(gx)], axis=-1).astype(np.float32)
        n /= np.linalg.norm(n, axis=-1, keepdims=True)
    else:
        n = np.zeros((size, size, 3), np.float32)
        n[..., 2] = 1.0
    rough = np.clip(np.float32(roughness) * (0.8 + 0.2 * n2), 1.0 / 126.0, 1.0).astype(np.float32)
    if roughness >= 1.0:
        rough = np.ones_like(rough)
    packed = pack_normal_roughness(n.astype(np.float32), rough)
    flags = 0
    if normal_map:
        flags |= abi.SW_TEX_HAS_NORMAL_MAP
    if roughness < 1.0:
        flags |= abi.SW_TEX_HAS_NON_ONE_ROUGHNESS
    if metal:
        flags |= abi.SW_TEX_IS_METAL
    mips = [(diffuse.astype(np.uint32), packed)]
    for _ in range(NUM_MIPS - 1):
        mips.append(build_mip(*mips[-1]))
    return mips, flags


def make_material_set(seed, count, size, metal_frac=0.25, dielectric_frac=0.25, normal_maps=True):
    """Textures of `count` materials with full mip chains, packed into one texel array + mip table."""
    rng = np.random.default_rng(seed)
    texel_chunks = []
    mips = []
    offset = 0
    for m in range(count):
        u = m / max(count, 1)
        if u < metal_frac:
            rough, metal = 0.35, True
        elif u < metal_frac + dielectric_frac:
            rough, metal = 0.5, False
        else:
            rough, metal = 1.0, False
        chain, flags = make_texture(rng, size, normal_map=normal_maps, roughness=rough, metal=metal)
        for d, p in chain:
            t = make_texels(d, p).ravel()
            texel_chunks.append(t)
            mips.append((offset, d.shape[1], d.shape[0], flags, 0))
            offset += t.size
    texels = np.concatenate(texel_chunks)
    table = np.array(mips, dtype=abi.TEXTURE_MIP)
    return texels, table


def make_emissive_set(seed, count, size):
    """Color32 emissive textures with mips (make_texture_lite_mips, textures.rs:364-415)."""
    rng = np.random.default_rng(seed)
    chunks, mips, offset = [], [], 0
    for _ in range(count):
        img = rng.integers(0, 256, (size, size, 4), dtype=np.uint32)
        img[..., 3] = np.where(rng.random((size, size)) < 0.5, 255, 0)
        c = (img[..., 3] << 24) | (img[..., 0] << 16) | (img[..., 1] << 8) | img[..., 2]
        level = c.astype(np.uint32)
        for _m in range(NUM_MIPS):
            chunks.append(level.ravel())
            mips.append((offset, level.shape[1], level.shape[0]))
            offset += level.size
            if level.shape[0] >= 2:
                level = average4(level)
    return np.concatenate(chunks), np.array(mips, dtype=abi.EMISSIVE_MIP)


def random_directional_lightmap(rng, n):
    """Directional lightmap texels: ambient U[0,4], direction (tangent space, z>=0) x U[0,8],
    deviation U[0,1], colour normalised to max component 1."""
    e = np.zeros(n, abi.DIR_LIGHTMAP_ELEMENT)
    e["ambient_light"] = rng.uniform(0, 4, (n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d[:, 2] = np.abs(d[:, 2]) + 0.05
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    e["light_direction_vector_scaled"] = (d * rng.uniform(0.05, 8, (n, 1))).astype(np.float32)
    e["directional_light_deviation"] = rng.uniform(0, 1, n).astype(np.float32)
    c = rng.uniform(0.2, 1.0, (n, 3)).astype(np.float32)
    e["directional_light_color"] = c / c.max(axis=1, keepdims=True)
    return e


def random_lights(rng, n, center=(0.0, 0.0, 0.0), spread=256.0):
    l = np.zeros(n, abi.LIGHT)
    l["position"] = (np.asarray(center, np.float32) + rng.uniform(-spread, spread, (n, 3))).astype(np.float32)
    r = rng.uniform(128, 512, n).astype(np.float32)
    l["radius"] = r
    l["inv_square_radius"] = (np.float32(1.0) / (r * r)).astype(np.float32)
    l["color"] = rng.uniform(0, 2e5, (n, 3)).astype(np.float32)
    return l


def random_frame_basis(rng):
    q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
    return q.astype(np.float32)


class BatchedSurfaces:
    """The batched-surface workload: `count` surfaces with log-uniform sides in [min_side, max_side],
    mips 0..3, random directional (or simple) lightmaps, normal-mapped specular materials."""

    def __init__(self, seed=3, count=4096, min_side=4, max_side=512, num_materials=16, texture_size=256,
                 num_lights=0, emissive_frac=0.0, directional=True, pixel_format=abi.SW_PIXEL_C64):
        rng = np.random.default_rng(seed)
        self.seed = seed
        self.pixel_format = pixel_format
        self.directional = directional
        self.texels, self.texture_mips = make_material_set(seed + 1, num_materials, texture_size)
        self.emissive_pixels, self.emissive_mips = make_emissive_set(seed + 2, 2, 64)
        sides = np.exp(rng.uniform(np.log(min_side), np.log(max_side + 1), (count, 2))).astype(np.int64)
        sides = np.clip(sides, min_side, max_side)
        mips = rng.integers(0, 4, count)
        log2 = 4 - mips
        shifts = rng.integers(0, 1 << 16, (count, 2)) & ((1 << log2[:, None]) - 1)
        lm_size = ((sides - 1 + shifts) >> log2[:, None]) + 2
        lm_count = lm_size[:, 0] * lm_size[:, 1]
        lm_offsets = 1 + np.concatenate([[0], np.cumsum(lm_count)[:-1]])
        total_lm = int(1 + lm_count.sum())
        if directional:
            self.directional_lightmaps = random_directional_lightmap(rng, total_lm)
            self.lightmaps = np.zeros((1, 3), np.float32)
        else:
            self.directional_lightmaps = np.zeros(0, abi.DIR_LIGHTMAP_ELEMENT)
            self.lightmaps = rng.uniform(0, 4, (total_lm, 3)).astype(np.float32)
        self.cam_pos = rng.uniform(-512, 512, 3).astype(np.float32)
        self.lights = random_lights(rng, max(num_lights, 0))

        d = np.zeros(count, abi.SURFACE_DESC)
        for i in range(count):
            b = random_frame_basis(rng)
            scale = np.float32(1 << int(mips[i]))
            d["basis_u"][i] = b[0] * scale
            d["basis_v"][i] = b[1] * scale
            d["basis_normal"][i] = b[2]
            d["basis_start"][i] = rng.uniform(-256, 256, 3)
        d["size"] = sides.astype(np.uint32)
        d["tc_start"] = rng.integers(-2048, 2048, (count, 2)).astype(np.int32)
        tex = rng.integers(0, num_materials, count)
        d["texture_mip"] = (tex * NUM_MIPS + mips).astype(np.uint32)
        d["emissive_mip"] = abi.SW_NO_EMISSIVE
        em = rng.random(count) < emissive_frac
        d["emissive_mip"][em] = rng.integers(0, self.emissive_mips.size, int(em.sum())).astype(np.uint32)
        d["emissive_light"] = rng.uniform(0, 2, (count, 3)).astype(np.float32)
        d["lightmap_offset"] = lm_offsets.astype(np.uint32)
        d["lightmap_size"] = lm_size.astype(np.uint32)
        d["lightmap_scale_log2"] = log2.astype(np.uint32)
        d["lightmap_tc_shift"] = shifts.astype(np.uint32)
        d["flags"] = abi.SW_SURF_DIFFUSE_LAYER
        if num_lights > 0:
            nl = rng.integers(0, min(num_lights, abi.SW_MAX_POLYGON_LIGHTS) + 1, count)
            d["num_lights"] = nl.astype(np.uint32)
            for i in range(count):
                d["lights"][i, :nl[i]] = rng.choice(num_lights, nl[i], replace=False)
        area = sides[:, 0] * sides[:, 1]
        d["out_offset"] = np.concatenate([[0], np.cumsum(area)[:-1]]).astype(np.uint64)
        self.surfaces = d
        self.total_texels = int(area.sum())
        self.lightmap_elements_touched = int(lm_count.sum())

    def static_data(self):
        from .gpu import StaticData
        return StaticData(self.texels, self.texture_mips, self.emissive_pixels, self.emissive_mips, self.lightmaps,
                          self.directional_lightmaps)

    def algorithmic_bytes(self):
        """Bytes one build of all surfaces must move: texture texel (8 B) + output texel per surface texel,
        plus every lightmap element of each surface once."""
        out_b = 8 if self.pixel_format == abi.SW_PIXEL_C64 else 4
        lm_b = 40 if self.directional else 12
        return self.total_texels * (8 + out_b) + self.lightmap_elements_touched * lm_b
