"""Seeded synthetic scenes for the meshlet raster pipeline.

The reference loads glTF assets and splits them with meshoptimizer (src/SwRast/Scene.cpp:156-368);
neither the assets of the benchmark scenes nor those libraries exist here, so scenes are generated
directly in the reference's ``Meshlet`` record layout (src/SwRast/Scene.h:15-30, 1728 bytes).

Every meshlet is a closed, genus-0 "icosphere-like" patch: 64 points of a spherical Fibonacci
lattice triangulated by their convex hull (2*64-4 = 124 triangles), outward-facing triangles wound
counter-clockwise (the reference's FaceCullMode::FrontCCW keeps them), radially displaced by
Gaussian noise (sigma 0.02) per meshlet. Cameras follow the reference's reversed-Z infinite
projection (src/SwRast/Camera.h:38-48).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

MESHLET_SIZE = 1728

MESHLET_DTYPE = np.dtype({
    "names": ["BoundCenter", "BoundRadius", "ConeApex", "ConeAxis", "ConeCutoff", "NumVertices",
              "NumTriangles", "AlphaCutoff", "MaterialId", "TangentHandedness", "Positions",
              "TexCoords", "NormalTangents", "Indices"],
    "formats": [("<f4", 3), "<f4", ("<f4", 3), ("<f4", 3), "<f4", "u1", "u1", "u1", "<u4", "<u8",
                ("<f4", (3, 64)), ("<u4", 64), ("<u4", 64), ("u1", (3, 128))],
    "offsets": [0, 12, 16, 28, 40, 44, 45, 46, 48, 56, 64, 832, 1088, 1344],
    "itemsize": MESHLET_SIZE,
})

MATERIAL_DTYPE = np.dtype([("texture", "<u4"), ("is_double_sided", "u1"), ("alpha_cutoff", "u1"),
                           ("pad", "u1", 2)])


def concat_meshlets(parts) -> np.ndarray:
    """Concatenates meshlet arrays keeping the 1728-byte record (np.concatenate would canonicalise
    the structured dtype and drop the trailing padding)."""
    n = sum(len(p) for p in parts)
    out = np.zeros(n, dtype=MESHLET_DTYPE)
    i = 0
    for p in parts:
        out[i:i + len(p)] = p
        i += len(p)
    return out


# --------------------------------------------------------------------------- meshlet template
def _fibonacci_sphere(n: int) -> np.ndarray:
    i = np.arange(n, dtype=np.float64) + 0.5
    phi = np.arccos(1.0 - 2.0 * i / n)
    theta = math.pi * (1.0 + 5.0 ** 0.5) * i
    return np.stack([np.cos(theta) * np.sin(phi), np.cos(phi), np.sin(theta) * np.sin(phi)], axis=1)


def _hull_triangles(p: np.ndarray) -> np.ndarray:
    """Convex hull of points on a sphere, wound so (b-a)x(c-a) points outward."""
    from scipy.spatial import ConvexHull

    tris = ConvexHull(p).simplices.astype(np.int64)
    a, b, c = p[tris[:, 0]], p[tris[:, 1]], p[tris[:, 2]]
    n = np.cross(b - a, c - a)
    flip = np.einsum("ij,ij->i", n, (a + b + c) / 3.0) < 0
    tris[flip] = tris[flip][:, [0, 2, 1]]
    # deterministic, spatially coherent order: by latitude band then longitude of the centroid
    cen = (p[tris[:, 0]] + p[tris[:, 1]] + p[tris[:, 2]]) / 3.0
    band = np.floor((cen[:, 1] + 1.0) * 4.0)
    lon = np.arctan2(cen[:, 2], cen[:, 0])
    order = np.lexsort((lon, band))
    return tris[order]


_TEMPLATE: tuple[np.ndarray, np.ndarray] | None = None


def meshlet_template() -> tuple[np.ndarray, np.ndarray]:
    """(64x3 unit positions, 124x3 triangle indices)."""
    global _TEMPLATE
    if _TEMPLATE is None:
        p = _fibonacci_sphere(64)
        _TEMPLATE = (p, _hull_triangles(p))
    return _TEMPLATE


_PATCH: tuple[np.ndarray, np.ndarray] | None = None


def patch_template(cap_degrees: float = 20.0) -> tuple[np.ndarray, np.ndarray]:
    """An open patch of the unit sphere: the 64 points of a Fibonacci lattice on the cap within
    cap_degrees of +y, triangulated by the cap's part of the convex hull of those points and a point
    far below the cap (the hull's other triangles touch that point and are dropped), wound so
    (b-a)x(c-a) points outward. Returns (64x3 positions, triangles)."""
    global _PATCH
    if _PATCH is None:
        from scipy.spatial import ConvexHull

        n = 64
        i = np.arange(n, dtype=np.float64) + 0.5
        ymin = math.cos(math.radians(cap_degrees))
        y = 1.0 - (1.0 - ymin) * i / n
        r = np.sqrt(1.0 - y * y)
        th = math.pi * (1.0 + 5.0 ** 0.5) * i
        p = np.stack([np.cos(th) * r, y, np.sin(th) * r], axis=1)
        hull = ConvexHull(np.concatenate([p, [[0.0, -10.0, 0.0]]]))
        tris = hull.simplices[(hull.simplices < n).all(axis=1)].astype(np.int64)
        a, b, c = p[tris[:, 0]], p[tris[:, 1]], p[tris[:, 2]]
        flip = np.einsum("ij,ij->i", np.cross(b - a, c - a), (a + b + c) / 3.0) < 0
        tris[flip] = tris[flip][:, [0, 2, 1]]
        cen = (a + b + c) / 3.0
        tris = tris[np.lexsort((np.arctan2(cen[:, 2], cen[:, 0]), np.floor(cen[:, 1] * 8.0)))]
        _PATCH = (p, tris)
    return _PATCH


def normal_cones(world: np.ndarray, tris: np.ndarray, centers: np.ndarray, min_dot: float = 0.1):
    """Normal cones of meshlets in meshoptimizer's convention, as the reference stores them
    (ConeApex, ConeAxis, ConeCutoff, Scene.cpp:240-244): every triangle faces away from a camera at e
    when dot(normalize(apex - e), axis) >= cutoff. Axis = normalised mean of the unit triangle
    normals; with m the least cosine between a normal and the axis, cutoff = sqrt(1 - m^2) and the
    apex is the point centre - t*axis behind every triangle's plane (t = the largest distance along
    the axis from the centre back to a plane). A cone with m <= min_dot is degenerate: cutoff 1,
    axis 0, apex = centre. world: (n, verts, 3) float64 positions; returns float32 arrays."""
    a, b, c = world[:, tris[:, 0]], world[:, tris[:, 1]], world[:, tris[:, 2]]
    nrm = np.cross(b - a, c - a)
    ln = np.linalg.norm(nrm, axis=2, keepdims=True)
    nrm = np.where(ln > 0, nrm / np.where(ln > 0, ln, 1.0), 0.0)
    axis = nrm.sum(axis=1)
    al = np.linalg.norm(axis, axis=1, keepdims=True)
    axis = np.where(al > 0, axis / np.where(al > 0, al, 1.0), 0.0)
    m = np.einsum("ntk,nk->nt", nrm, axis).min(axis=1)
    dn = np.einsum("ntk,nk->nt", nrm, axis)
    dc = np.einsum("ntk,ntk->nt", centers[:, None, :] - a, nrm)
    t = np.where(dn > 0, dc / np.where(dn > 0, dn, 1.0), 0.0).max(axis=1).clip(min=0.0)
    ok = m > min_dot
    apex = np.where(ok[:, None], centers - axis * t[:, None], centers)
    cutoff = np.where(ok, np.sqrt(np.clip(1.0 - m * m, 0.0, 1.0)), 1.0)
    return apex.astype(np.float32), np.where(ok[:, None], axis, 0.0).astype(np.float32), cutoff.astype(np.float32)


def _random_rotations(rng: np.random.Generator, n: int) -> np.ndarray:
    """Uniformly distributed rotation matrices from normalised Gaussian quaternions, (n, 3, 3)."""
    q = rng.standard_normal((n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q.T
    return np.stack([np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)], axis=1),
                     np.stack([2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)], axis=1),
                     np.stack([2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], axis=1)], axis=1)


def build_patch_meshlets(centers: np.ndarray, scales: np.ndarray, material_ids: np.ndarray, rng: np.random.Generator,
                         sigma: float = 0.002, uv_repeat: float = 2.0) -> np.ndarray:
    """Open sphere patches (patch_template), one per meshlet: radially displaced, randomly rotated,
    scaled and translated, with bounding spheres and normal cones (normal_cones). The displacement
    is smaller than the closed meshlets' (sigma 0.002 instead of 0.02): on triangles this small,
    sigma 0.02 tilts some normals by 30 degrees or more, which widens every cone until it culls
    almost nothing."""
    n = len(centers)
    base, tris = patch_template()
    nv, nt = base.shape[0], tris.shape[0]
    out = np.zeros(n, dtype=MESHLET_DTYPE)
    disp = 1.0 + sigma * rng.standard_normal((n, nv))
    local = base[None, :, :] * disp[:, :, None]
    rot = _random_rotations(rng, n)
    world = np.einsum("nij,nvj->nvi", rot, local) * scales[:, None, None] + centers[:, None, :]
    world32 = world.astype(np.float32)
    out["Positions"] = np.transpose(world32, (0, 2, 1))
    out["NumVertices"] = nv
    out["NumTriangles"] = nt
    out["AlphaCutoff"] = 255
    out["MaterialId"] = material_ids.astype(np.uint32)
    out["BoundCenter"] = centers.astype(np.float32)
    d = np.linalg.norm(world32.astype(np.float64) - centers[:, None, :], axis=2).max(axis=1)
    out["BoundRadius"] = (d * (1.0 + 1e-6)).astype(np.float32)
    out["ConeApex"], out["ConeAxis"], out["ConeCutoff"] = normal_cones(world32.astype(np.float64), tris,
                                                                         centers.astype(np.float32).astype(np.float64))
    idx = np.zeros((3, 128), dtype=np.uint8)
    idx[:, :nt] = tris.T
    out["Indices"] = idx[None]
    uv = (base[:, [0, 2]] * 0.5 + 0.5) * uv_repeat
    uv16 = uv.astype(np.float16).view(np.uint16).astype(np.uint32)
    out["TexCoords"][:, :nv] = (uv16[:, 0] | (uv16[:, 1] << 16))[None]
    normal = local / np.linalg.norm(local, axis=2, keepdims=True)
    nrm = np.einsum("nij,nvj->nvi", rot, normal)
    up = np.array([0.0, 1.0, 0.0])
    tan = np.cross(up[None, None, :], nrm)
    tl = np.linalg.norm(tan, axis=2, keepdims=True)
    tan = np.where(tl > 1e-6, tan / np.maximum(tl, 1e-12), np.array([1.0, 0.0, 0.0]))
    on, ot = _pack_unorm8(_oct_encode(nrm)), _pack_unorm8(_oct_encode(tan))
    out["NormalTangents"][:, :nv] = on[..., 0] | (on[..., 1] << 8) | (ot[..., 0] << 16) | (ot[..., 1] << 24)
    return out


def _oct_encode(n: np.ndarray) -> np.ndarray:
    """Octahedral map of unit vectors to [0,1]^2 (the reference's MapOctahedron, Texture.h:282-288)."""
    w = 1.0 / (np.abs(n[..., 0]) + np.abs(n[..., 1]) + np.abs(n[..., 2]))
    t = np.maximum(-n[..., 2] * w, 0.0)
    u = n[..., 0] * w + np.copysign(t, n[..., 0])
    v = n[..., 1] * w + np.copysign(t, n[..., 1])
    return np.stack([u, v], axis=-1) * 0.5 + 0.5


def _pack_unorm8(v: np.ndarray) -> np.ndarray:
    return np.round(np.clip(v, 0.0, 1.0) * 255.0).astype(np.uint32)


def build_meshlets(centers: np.ndarray, scales: np.ndarray, yaws: np.ndarray, material_ids: np.ndarray,
                   rng: np.random.Generator, sigma: float = 0.02, uv_repeat: float = 2.0) -> np.ndarray:
    """Instantiates the template once per meshlet: displaced, scaled, yawed and translated."""
    n = len(centers)
    base, tris = meshlet_template()
    nv, nt = base.shape[0], tris.shape[0]
    out = np.zeros(n, dtype=MESHLET_DTYPE)

    disp = 1.0 + sigma * rng.standard_normal((n, nv))
    local = base[None, :, :] * disp[:, :, None]                       # (n, 64, 3) object space
    c, s = np.cos(yaws), np.sin(yaws)
    rx = c[:, None] * local[:, :, 0] + s[:, None] * local[:, :, 2]
    rz = -s[:, None] * local[:, :, 0] + c[:, None] * local[:, :, 2]
    world = np.stack([rx, local[:, :, 1], rz], axis=2) * scales[:, None, None] + centers[:, None, :]
    world32 = world.astype(np.float32)

    out["Positions"] = np.transpose(world32, (0, 2, 1))
    out["NumVertices"] = nv
    out["NumTriangles"] = nt
    out["AlphaCutoff"] = 255
    out["MaterialId"] = material_ids.astype(np.uint32)
    out["BoundCenter"] = centers.astype(np.float32)
    d = np.linalg.norm(world32.astype(np.float64) - centers[:, None, :], axis=2).max(axis=1)
    out["BoundRadius"] = (d * (1.0 + 1e-6)).astype(np.float32)
    out["ConeApex"] = centers.astype(np.float32)
    out["ConeAxis"] = np.array([0.0, 1.0, 0.0], dtype=np.float32)
    out["ConeCutoff"] = 1.0
    idx = np.zeros((3, 128), dtype=np.uint8)
    idx[:, :nt] = tris.T
    out["Indices"] = idx[None]

    # texture coordinates: planar projection of the unit template, as float16 pairs
    uv = (base[:, [0, 1]] * 0.5 + 0.5) * uv_repeat
    uv16 = uv.astype(np.float16).view(np.uint16).astype(np.uint32)
    tc = uv16[:, 0] | (uv16[:, 1] << 16)
    out["TexCoords"][:, :nv] = tc[None]

    # oct-encoded normal / tangent pairs (packUnorm4x8 order: nx, ny, tx, ty)
    normal = local / np.linalg.norm(local, axis=2, keepdims=True)
    nrm = np.stack([c[:, None] * normal[:, :, 0] + s[:, None] * normal[:, :, 2], normal[:, :, 1],
                    -s[:, None] * normal[:, :, 0] + c[:, None] * normal[:, :, 2]], axis=2)
    up = np.array([0.0, 1.0, 0.0])
    tan = np.cross(up[None, None, :], nrm)
    tl = np.linalg.norm(tan, axis=2, keepdims=True)
    tan = np.where(tl > 1e-6, tan / np.maximum(tl, 1e-12), np.array([1.0, 0.0, 0.0]))
    on, ot = _pack_unorm8(_oct_encode(nrm)), _pack_unorm8(_oct_encode(tan))
    out["NormalTangents"][:, :nv] = on[..., 0] | (on[..., 1] << 8) | (ot[..., 0] << 16) | (ot[..., 1] << 24)
    out["TangentHandedness"] = 0
    return out


# --------------------------------------------------------------------------------- cameras
def look_at(eye, target, up=(0.0, 1.0, 0.0)) -> np.ndarray:
    """Right-handed view matrix (camera looks down -z), column-major float32[16]."""
    eye, target, up = (np.asarray(v, dtype=np.float64) for v in (eye, target, up))
    f = target - eye
    f /= np.linalg.norm(f)
    r = np.cross(f, up)
    r /= np.linalg.norm(r)
    u = np.cross(r, f)
    m = np.eye(4)
    m[0, :3], m[1, :3], m[2, :3] = r, u, -f
    m[0, 3], m[1, 3], m[2, 3] = -r @ eye, -u @ eye, f @ eye
    return m.T.astype(np.float32).reshape(16)  # row-major math -> glm column-major storage


def proj_reversed_z(fov_deg: float, aspect: float, near: float) -> np.ndarray:
    """Camera::GetProjMatrix (Camera.h:38-48): infinite reversed-Z, y flipped, column-major."""
    f = 1.0 / math.tan(math.radians(fov_deg) / 2.0)
    m = np.zeros((4, 4), dtype=np.float32)  # [col][row]
    m[0, 0] = f / aspect
    m[1, 1] = -f
    m[2, 3] = -1.0
    m[3, 2] = near
    return m.reshape(16)


def mat_mul(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Column-major float32 product with the summation order of the host matrix helpers."""
    A, B = a.reshape(4, 4), b.reshape(4, 4)
    r = np.zeros((4, 4), dtype=np.float32)
    for c in range(4):
        for row in range(4):
            s = np.float32(A[0, row] * B[c, 0])
            s = np.float32(s + np.float32(A[1, row] * B[c, 1]))
            s = np.float32(s + np.float32(A[2, row] * B[c, 2]))
            s = np.float32(s + np.float32(A[3, row] * B[c, 3]))
            r[c, row] = s
    return r.reshape(16)


IDENTITY = np.eye(4, dtype=np.float32).reshape(16)


@dataclass
class View:
    width: int
    height: int
    view: np.ndarray
    proj: np.ndarray
    eye: np.ndarray
    depth_only: bool = False

    @property
    def world_to_clip(self) -> np.ndarray:
        return mat_mul(self.proj, self.view)


def make_view(width, height, eye, target, fov=60.0, near=0.1, depth_only=False) -> View:
    return View(width, height, look_at(eye, target), proj_reversed_z(fov, width / height, near),
                np.asarray(eye, dtype=np.float32), depth_only)


# ---------------------------------------------------------------------------------- textures
def _lattice_rgba(size: int, lat: np.ndarray) -> np.ndarray:
    """Bilinear interpolation (8-bit fractions) of a wrapping cells x cells x 4 lattice, int64[size, size, 4]."""
    cells = lat.shape[0]
    step = size // cells
    t = (np.arange(size) % step) * 256 // step                       # 8-bit fraction
    i0 = np.arange(size) // step
    i1 = (i0 + 1) % cells
    ty, tx = t[:, None, None], t[None, :, None]
    a = lat[i0[:, None], i0[None, :]]
    b = lat[i0[:, None], i1[None, :]]
    c = lat[i1[:, None], i0[None, :]]
    d = lat[i1[:, None], i1[None, :]]
    top = a * (256 - tx) + b * tx
    bot = c * (256 - tx) + d * tx
    return (top * (256 - ty) + bot * ty) >> 16


def value_noise_rgba(size: int, seed: int, cells: int = 32, layer: int = 0, detail: bool = False,
                     cutout: bool = False) -> np.ndarray:
    """Seeded RGBA8 value noise (bilinear over a cells x cells lattice, wrapping), uint32[size, size].
    With detail, a second octave with 8-texel cells is blended in at 1/4 weight. Layer 0 is opaque
    (alpha 255) unless cutout, where its alpha is noise too (for alpha-tested materials)."""
    # layer 1 = tangent-space normal XY (centred near 128), metallic, roughness (Scene.h:8-10)
    v = _lattice_rgba(size, _noise_lattice(seed, cells, layer))
    if detail:
        v = (3 * v + _lattice_rgba(size, _noise_lattice(seed + 104729, size // 8, layer))) >> 2
    v = v.astype(np.uint32)
    if layer == 0 and not cutout:
        v[..., 3] = 255
    return v[..., 0] | (v[..., 1] << 8) | (v[..., 2] << 16) | (v[..., 3] << 24)


def _noise_lattice(seed: int, cells: int, layer: int) -> np.ndarray:
    rng = np.random.default_rng(seed * 7919 + layer)
    lat = rng.integers(0, 256, size=(cells, cells, 4), dtype=np.int64)
    if layer == 1:
        lat[..., 0] = 128 + (lat[..., 0] - 128) // 3
        lat[..., 1] = 128 + (lat[..., 1] - 128) // 3
        # roughness in [ROUGHNESS_MIN, 255]: no mirror-like texels (their one-LSB changes swing the
        # GGX lobe by 2x and dominate any image comparison)
        lat[..., 3] = ROUGHNESS_MIN + lat[..., 3] * (255 - ROUGHNESS_MIN) // 255
    return lat


ROUGHNESS_MIN = 51  # 0.2


def value_noise_rgba_torch(size: int, seed: int, cells: int = 32, layer: int = 0, device="cuda", detail: bool = False,
                           cutout: bool = False):
    """value_noise_rgba computed on the device with torch (same integer arithmetic, same texels);
    returns an int32 tensor of shape (size, size) holding the packed RGBA8 words."""
    import torch

    def lattice(lat_np):
        lat = torch.from_numpy(lat_np).to(device)
        c = lat.shape[0]
        step = size // c
        ar = torch.arange(size, device=device)
        t = (ar % step) * 256 // step
        i0 = ar // step
        i1 = (i0 + 1) % c
        ty, tx = t[:, None, None], t[None, :, None]
        a = lat[i0[:, None], i0[None, :]]
        b = lat[i0[:, None], i1[None, :]]
        cc = lat[i1[:, None], i0[None, :]]
        d = lat[i1[:, None], i1[None, :]]
        top = a * (256 - tx) + b * tx
        bot = cc * (256 - tx) + d * tx
        return (top * (256 - ty) + bot * ty) >> 16

    v = lattice(_noise_lattice(seed, cells, layer))
    if detail:
        v = (3 * v + lattice(_noise_lattice(seed + 104729, size // 8, layer))) >> 2
    if layer == 0 and not cutout:
        v[..., 3] = 255
    packed = v[..., 0] | (v[..., 1] << 8) | (v[..., 2] << 16) | (v[..., 3] << 24)
    return (packed - ((packed >> 31) << 32)).to(torch.int32)


def env_map_r11g11b10(size: int, seed: int) -> np.ndarray:
    """Octahedral sky radiance: a smooth gradient plus noise quantised to 8 bits, then packed
    R11G11B10 (HdrTexture2D, Texture.h:216) with the reference's clamp-only packing."""
    u = (np.arange(size) + 0.5) / size
    uu, vv = np.meshgrid(u, u)
    noise = (value_noise_rgba(size, seed, cells=16) & 0xFF).astype(np.float64) / 255.0
    base = np.stack([0.3 + 0.5 * vv, 0.5 + 0.3 * uu, 0.9 - 0.2 * vv], axis=-1) * (0.75 + 0.5 * noise[..., None])
    q = np.round(np.clip(base, 0, 1) * 255.0) / 255.0 * 4.0            # 8-bit quantised, HDR scale 4
    q = q.astype(np.float32)

    def pack(x, mbits):
        x = np.maximum(x, np.float32(1.0 / (1 << 15)))
        x = np.minimum(x, np.float32(130048.0 if mbits == 6 else 129024.0))
        b = x.view(np.uint32)
        if mbits == 6:
            return ((b >> 17) & 0x3FFF) - 0x1C00
        return ((b >> 18) & 0x1FFF) - 0x0E00
    return (pack(q[..., 0], 6) << 21) | (pack(q[..., 1], 6) << 10) | pack(q[..., 2], 5)


# ------------------------------------------------------------------------------------ scenes
@dataclass
class Scene:
    meshlets: np.ndarray                      # MESHLET_DTYPE[n]
    materials: np.ndarray                     # MATERIAL_DTYPE[m]
    texture_size: int
    texture_layers: int
    views: list = field(default_factory=list)
    texture_seed: int = 0
    env_size: int = 0
    name: str = ""
    texture_detail: bool = False              # second noise octave with 8-texel cells


    @property
    def num_meshlets(self) -> int:
        return len(self.meshlets)

    def texture_cutout(self, i: int, layer: int) -> bool:
        """Layer 0 of an alpha-tested material carries a noise alpha channel."""
        return layer == 0 and int(self.materials["alpha_cutoff"][i]) < 255

    def texture_pixels(self, i: int, layer: int) -> np.ndarray:
        return value_noise_rgba(self.texture_size, self.texture_seed + i, layer=layer, detail=self.texture_detail,
                                cutout=self.texture_cutout(i, layer))


def grid_scene(n_side: int = 32, width: int = 1280, height: int = 720, seed: int = 1,
               texture_size: int = 512) -> Scene:
    """Small plain-path scene: n_side^2 meshlets on a grid over [-16,16]^2 with random yaw,
    one value-noise material (full mips), one camera."""
    rng = np.random.default_rng(seed)
    g = (np.arange(n_side) + 0.5) / n_side * 32.0 - 16.0
    gx, gz = np.meshgrid(g, g)
    centers = np.stack([gx.ravel(), np.zeros(gx.size), gz.ravel()], axis=1)
    n = len(centers)
    scales = np.full(n, 1.0)
    m = build_meshlets(centers, scales, rng.uniform(0, 2 * math.pi, n), np.zeros(n, np.int64), rng)
    mats = np.zeros(1, dtype=MATERIAL_DTYPE)
    mats["alpha_cutoff"] = 255
    view = make_view(width, height, eye=(0.0, 14.0, 24.0), target=(0.0, 0.0, -2.0))
    return Scene(m, mats, texture_size, 1, [view], texture_seed=seed, name=f"grid{n}@{width}x{height}")


def _round4(v: float) -> int:
    return max(4, int(round(v / 4.0)) * 4)


def frustum_visible_count(meshlets: np.ndarray, view: "View") -> int:
    """Meshlets whose bounding sphere passes frustum planes 0..4 of the view (CullMeshlets'
    frustum test, Shading.cpp:797-809, in float64; for choosing cameras, not for parity)."""
    m = mat_mul(view.proj, view.view).astype(np.float64).reshape(4, 4)  # [column, row]
    rows = m.T
    c = meshlets["BoundCenter"].astype(np.float64)
    r = meshlets["BoundRadius"].astype(np.float64)
    vis = np.ones(len(meshlets), bool)
    for i in range(3):
        for sgn in (1.0, -1.0):
            if i == 2 and sgn < 0:
                continue  # the far plane is not tested
            p = rows[3] + sgn * rows[i]
            p = p / np.linalg.norm(p[:3])
            vis &= c @ p[:3] + p[3] > -r
    return int(vis.sum())


def multiview_scene(n: int = 200_000, n_cameras: int = 58, seed: int = 3, cube_size: int = 1024,
                    min_res=(256, 256), max_res=(2560, 1440), min_visible: int | None = None,
                    max_visible: int | None = None) -> Scene:
    """Batched multi-view workload: n meshlets of the grid construction (spacing 1, radius 1,
    random yaw) seen by 6 depth-only cube-face views (cube_size^2, 90 degrees) from a point above the
    grid's centre plus n_cameras cameras at random positions and heights whose resolutions are
    drawn log-uniformly between min_res and max_res (rounded to multiples of 4). The cube is turned
    so that its diagonal is vertical: every face then sees part of the grid (an axis-aligned cube's
    upward face would see nothing). Cameras whose frustum holds fewer than min_visible or more than
    max_visible meshlets (default n/200 and 3n/4: 1k and 150k for 200k meshlets) are drawn again, so
    the views' loads range over that interval."""
    rng = np.random.default_rng(seed)
    min_visible = max(1, n // 200) if min_visible is None else min_visible
    max_visible = (3 * n) // 4 if max_visible is None else max_visible
    side = int(math.ceil(math.sqrt(n)))
    g = np.arange(side) - (side - 1) / 2.0
    gx, gz = np.meshgrid(g, g)
    centers = np.stack([gx.ravel(), np.zeros(gx.size), gz.ravel()], axis=1)[:n]
    m = build_meshlets(centers, np.ones(n), rng.uniform(0, 2 * math.pi, n), np.zeros(n, np.int64), rng)
    mats = np.zeros(1, dtype=MATERIAL_DTYPE)
    mats["alpha_cutoff"] = 255
    views = []
    eye = np.array([0.0, 3.0, 0.0])
    # rotation taking the cube diagonal (1, 1, 1) / sqrt(3) to +y
    d = np.array([1.0, 1.0, 1.0]) / math.sqrt(3.0)
    axis = np.cross(d, [0.0, 1.0, 0.0])
    ang = math.acos(d[1])
    k = axis / np.linalg.norm(axis)
    K = np.array([[0, -k[2], k[1]], [k[2], 0, -k[0]], [-k[1], k[0], 0]])
    R = np.eye(3) + math.sin(ang) * K + (1 - math.cos(ang)) * K @ K
    faces = [((1, 0, 0), (0, 1, 0)), ((-1, 0, 0), (0, 1, 0)), ((0, 1, 0), (0, 0, 1)), ((0, -1, 0), (0, 0, 1)),
             ((0, 0, 1), (0, 1, 0)), ((0, 0, -1), (0, 1, 0))]
    for fd, up in faces:
        fd, up = R @ np.array(fd, float), R @ np.array(up, float)
        v = View(cube_size, cube_size, look_at(eye, eye + fd, up), proj_reversed_z(90.0, 1.0, 0.1),
                 eye.astype(np.float32), depth_only=True)
        views.append(v)
    half = side / 2.0
    tries = 0
    while len(views) < 6 + n_cameras:
        tries += 1
        if tries > 100 * (n_cameras + 1):
            raise ValueError("multiview_scene: no camera placement meets the visible-meshlet bounds")
        w = _round4(math.exp(rng.uniform(math.log(min_res[0]), math.log(max_res[0]))))
        h = _round4(math.exp(rng.uniform(math.log(min_res[1]), math.log(max_res[1]))))
        height = math.exp(rng.uniform(math.log(1.5), math.log(80.0)))
        e = np.array([rng.uniform(-half, half), height, rng.uniform(-half, half)])
        yaw, pitch = rng.uniform(0, 2 * math.pi), math.radians(rng.uniform(-70, -8))
        dv = np.array([math.cos(pitch) * math.cos(yaw), math.sin(pitch), math.cos(pitch) * math.sin(yaw)])
        v = make_view(w, h, eye=e, target=e + dv)
        if min_visible <= frustum_visible_count(m, v) <= max_visible:
            views.append(v)
    return Scene(m, mats, 0, 1, views, name=f"multiview{n}x{len(views)}")


def volume_scene(n: int = 100_000, width: int = 1920, height: int = 1080, n_materials: int = 64,
                 seed: int = 2, texture_size: int = 2048, extent: float = 100.0,
                 env_size: int = 1024, alpha_every: int = 0, alpha_cutoff: int = 128) -> Scene:
    """Large plain-path scene: n meshlets scattered in a (2*extent)^3 volume with log-uniform
    scale 0.1-10 and random yaw, n_materials materials of two RGBA8 layers, seen by a camera on
    the volume's -z face looking in (plus a perturbed second camera for the Hi-Z frame).
    With alpha_every = k > 0, every k-th material is alpha-tested (cutoff alpha_cutoff, double-sided,
    noise alpha in layer 0), like foliage cards."""
    rng = np.random.default_rng(seed)
    centers = rng.uniform(-extent, extent, size=(n, 3))
    scales = np.exp(rng.uniform(math.log(0.1), math.log(10.0), n))
    yaws = rng.uniform(0, 2 * math.pi, n)
    mat_ids = rng.integers(0, n_materials, n)
    m = build_meshlets(centers, scales, yaws, mat_ids, rng)
    mats = np.zeros(n_materials, dtype=MATERIAL_DTYPE)
    mats["texture"] = np.arange(n_materials)
    mats["alpha_cutoff"] = 255
    if alpha_every > 0:
        mats["alpha_cutoff"][::alpha_every] = alpha_cutoff
        mats["is_double_sided"][::alpha_every] = 1
    eye = np.array([0.0, 0.0, -1.3 * extent])
    v0 = make_view(width, height, eye=eye, target=(0.0, 0.0, 0.0))
    v1 = make_view(width, height, eye=eye + np.array([0.4, 0.2, 0.6]), target=(1.0, 0.5, 0.0))
    return Scene(m, mats, texture_size, 2, [v0, v1], texture_seed=seed * 1000, env_size=env_size, texture_detail=True,
                 name=f"volume{n}@{width}x{height}")


def patch_scene(n: int = 100_000, width: int = 1920, height: int = 1080, n_materials: int = 64, seed: int = 2,
                texture_size: int = 2048, extent: float = 100.0, env_size: int = 1024) -> Scene:
    """The volume construction (volume_scene) with open sphere patches instead of closed hulls:
    n randomly rotated patches (build_patch_meshlets) scattered in a (2*extent)^3 volume with
    log-uniform scale 0.1-10, each carrying its normal cone, so that about half of them face away
    from any camera as a whole (what backface-cone culling removes)."""
    rng = np.random.default_rng(seed)
    centers = rng.uniform(-extent, extent, size=(n, 3))
    scales = np.exp(rng.uniform(math.log(0.1), math.log(10.0), n))
    mat_ids = rng.integers(0, n_materials, n)
    m = build_patch_meshlets(centers, scales, mat_ids, rng)
    mats = np.zeros(n_materials, dtype=MATERIAL_DTYPE)
    mats["texture"] = np.arange(n_materials)
    mats["alpha_cutoff"] = 255
    eye = np.array([0.0, 0.0, -1.3 * extent])
    v0 = make_view(width, height, eye=eye, target=(0.0, 0.0, 0.0))
    v1 = make_view(width, height, eye=eye + np.array([0.4, 0.2, 0.6]), target=(1.0, 0.5, 0.0))
    return Scene(m, mats, texture_size, 2, [v0, v1], texture_seed=seed * 1000, env_size=env_size, texture_detail=True,
                 name=f"patches{n}@{width}x{height}")


def combined_scene(copies: int = 10, base_n: int = 100_000, n_materials: int = 256, n_views: int = 16, seed: int = 5,
                   texture_size: int = 2048, env_size: int = 1024, extent: float = 100.0) -> Scene:
    """Combined stress workload: `copies` translated copies of the volume construction (base_n
    meshlets in a (2*extent)^3 cube each) side by side on a grid in x and z, copy c using materials
    (m % 64) + 64 * (c % (n_materials / 64)), seen by n_views cameras above the field looking at
    its centre, with 16:9 sizes log-uniform between 1280x720 and 2880x1620 (multiples of 4; the first two
    views take the two ends)."""
    rng = np.random.default_rng(seed)
    base = volume_scene(n=base_n, width=1280, height=720, n_materials=64, seed=seed, extent=extent).meshlets
    cols = int(math.ceil(math.sqrt(copies)))
    rows = int(math.ceil(copies / cols))
    groups = max(1, n_materials // 64)
    out = np.zeros(copies * base_n, dtype=MESHLET_DTYPE)
    for c in range(copies):
        ox = (c % cols - (cols - 1) / 2.0) * 2.0 * extent
        oz = (c // cols - (rows - 1) / 2.0) * 2.0 * extent
        part = out[c * base_n:(c + 1) * base_n]
        part[:] = base
        part["Positions"][:, 0, :] += np.float32(ox)
        part["Positions"][:, 2, :] += np.float32(oz)
        for f in ("BoundCenter", "ConeApex"):
            part[f][:, 0] += np.float32(ox)
            part[f][:, 2] += np.float32(oz)
        part["MaterialId"] = (base["MaterialId"] % 64) + 64 * (c % groups)
    mats = np.zeros(n_materials, dtype=MATERIAL_DTYPE)
    mats["texture"] = np.arange(n_materials)
    mats["alpha_cutoff"] = 255
    half_x, half_z = cols * extent, rows * extent
    views = []
    for i in range(n_views):
        s = math.exp(rng.uniform(0.0, math.log(2880.0 / 1280.0)))
        if i < 2:  # the interval's two ends are always among the sizes
            s = 1.0 if i == 0 else 2880.0 / 1280.0
        w, h = _round4(1280 * s), _round4(720 * s)
        ang = 2 * math.pi * i / n_views + rng.uniform(-0.2, 0.2)
        r = rng.uniform(0.6, 1.2) * max(half_x, half_z)
        eye = (r * math.cos(ang), rng.uniform(0.3, 1.0) * extent, r * math.sin(ang))
        views.append(make_view(w, h, eye=eye, target=(rng.uniform(-0.3, 0.3) * half_x, 0.0, rng.uniform(-0.3, 0.3) * half_z)))
    return Scene(out, mats, texture_size, 2, views, texture_seed=seed * 1000, env_size=env_size, texture_detail=True,
                 name=f"combined{copies * base_n}x{n_views}")
