"""Seeded synthetic scenes for the hybrid pass.

The reference's meshes and environment maps (sphere.obj, lucy.obj,
DamagedHelmet.gltf, the LA_Downtown HDR/JPG) are not part of its repository,
so seeded synthetic scenes of the stated shapes stand in for them:

* ``small``   256x256, 20x20 ground quad + 16 icospheres (subdivision 2),
              one point light (2,6,2) intensity 20 + one directional light,
              1 shadow ray per light per pixel, 1 mirror bounce.
* ``hd``      1920x1080, 512x512-vertex fBm terrain (522,242 triangles) +
              48 icospheres (subdivision 5, 20,480 triangles each): 1,505,282
              triangles, 256 materials, 4 spherical area lights (radius 0.5,
              intensity U[10, 50]), 16 shadow samples per light per pixel,
              1 mirror bounce.
* ``diff``    512x512, ground + 64 icospheres (subdivision 3), 64 materials,
              8 point lights, 16 shadow samples.

Materials: albedo U[0,1]^3, roughness U[0,1], metallic Bernoulli(0.3);
shading model 3 (mirror) when roughness < 0.3, else 0 (PBR).  Draws come
from numpy's PCG64 generator in the order written below.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .scene import (DIRECTIONAL_LIGHT, POINT_LIGHT, SHADING_MIRROR, SHADING_PBR, Camera, Light, Material,
                    Mesh, Object, Scene)


# ---- meshes ----------------------------------------------------------------------
def _vertices(pos, nrm, uv) -> np.ndarray:
    n = len(pos)
    v = np.zeros((n, 11), np.float32)
    v[:, 0:3] = pos
    v[:, 3:6] = nrm
    v[:, 6:9] = 1.0
    v[:, 9:11] = uv
    return v


def icosphere(subdiv: int) -> Mesh:
    """Unit icosphere: 20 * 4^subdiv triangles, outward normals."""
    t = (1.0 + 5 ** 0.5) / 2.0
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
             (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
             (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5),
             (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    v = np.array(verts, np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array(faces, np.int64)
    for _ in range(subdiv):
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
        e.sort(axis=1)
        uniq, inv = np.unique(e, axis=0, return_inverse=True)
        mid = (v[uniq[:, 0]] + v[uniq[:, 1]]) * 0.5
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        base = len(v)
        v = np.concatenate([v, mid])
        nf = len(f)
        a = base + inv[:nf]
        b = base + inv[nf:2 * nf]
        c = base + inv[2 * nf:]
        f = np.concatenate([np.stack([f[:, 0], a, c], 1), np.stack([f[:, 1], b, a], 1),
                            np.stack([f[:, 2], c, b], 1), np.stack([a, b, c], 1)])
    uv = np.stack([0.5 + np.arctan2(v[:, 0], v[:, 2]) / (2 * np.pi), 0.5 - np.arcsin(np.clip(v[:, 1], -1, 1)) / np.pi], 1)
    return Mesh(_vertices(v, v, uv), f.reshape(-1).astype(np.uint32))


def geodesic_sphere(freq: int) -> Mesh:
    """Unit geodesic icosphere: each icosahedron face cut into freq^2 triangles on a
    barycentric grid and projected onto the sphere (20 freq^2 triangles: 2,000 at
    freq 10; freq 2^k is icosphere(k)'s triangle count), outward normals."""
    t = (1.0 + 5 ** 0.5) / 2.0
    ico = np.array([(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t),
                    (0, 1, -t), (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)], np.float64)
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
             (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5),
             (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    key_to_index, pos, tris = {}, [], []

    def vert(a, b, c, i, j):
        # grid point i steps from a toward b, j steps toward c; shared edge points get one key
        w = {a: freq - i - j, b: i, c: j}
        key = tuple(sorted((k, v) for k, v in w.items() if v))
        if key not in key_to_index:
            p = sum(ico[k] * v for k, v in w.items()) / freq
            key_to_index[key] = len(pos)
            pos.append(p / np.linalg.norm(p))
        return key_to_index[key]

    for a, b, c in faces:
        for i in range(freq):
            for j in range(freq - i):
                v0, v1, v2 = vert(a, b, c, i, j), vert(a, b, c, i + 1, j), vert(a, b, c, i, j + 1)
                tris.append((v0, v1, v2))
                if i + j < freq - 1:
                    tris.append((v1, vert(a, b, c, i + 1, j + 1), v2))
    v = np.array(pos)
    uv = np.stack([0.5 + np.arctan2(v[:, 0], v[:, 2]) / (2 * np.pi), 0.5 - np.arcsin(np.clip(v[:, 1], -1, 1)) / np.pi], 1)
    return Mesh(_vertices(v, v, uv), np.array(tris, np.int64).reshape(-1).astype(np.uint32))


def quad(size: float) -> Mesh:
    h = size / 2.0
    pos = np.array([[-h, 0, -h], [h, 0, -h], [h, 0, h], [-h, 0, h]], np.float64)
    nrm = np.tile([0.0, 1.0, 0.0], (4, 1))
    uv = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float64)
    return Mesh(_vertices(pos, nrm, uv), np.array([0, 2, 1, 0, 3, 2], np.uint32))


def _value_noise(rng: np.random.Generator, n: int, cells: int) -> np.ndarray:
    g = rng.random((cells + 1, cells + 1))
    x = np.linspace(0, cells, n, endpoint=False)
    i = np.floor(x).astype(np.int64)
    f = x - i
    f = f * f * (3 - 2 * f)
    a = g[i][:, i]
    b = g[i][:, i + 1]
    c = g[i + 1][:, i]
    d = g[i + 1][:, i + 1]
    fx = f[None, :]
    fy = f[:, None]
    return (a * (1 - fx) + b * fx) * (1 - fy) + (c * (1 - fx) + d * fx) * fy


def terrain(rng: np.random.Generator, n: int = 512, extent: float = 50.0, amplitude: float = 2.0,
            octaves: int = 6) -> Mesh:
    """n x n vertex fBm heightfield over [-extent, extent]^2: 2 (n-1)^2 triangles."""
    h = np.zeros((n, n))
    amp, cells, norm = 1.0, 4, 0.0
    for _ in range(octaves):
        h += amp * (_value_noise(rng, n, cells) - 0.5)
        norm += amp
        amp *= 0.5   # gain
        cells *= 2   # lacunarity
    h *= amplitude / norm * 2.0
    xs = np.linspace(-extent, extent, n)
    X, Z = np.meshgrid(xs, xs)
    pos = np.stack([X, h, Z], -1).reshape(-1, 3)
    dx = xs[1] - xs[0]
    gx = np.gradient(h, dx, axis=1)
    gz = np.gradient(h, dx, axis=0)
    nrm = np.stack([-gx, np.ones_like(h), -gz], -1).reshape(-1, 3)
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    uv = np.stack([(X + extent) / (2 * extent), (Z + extent) / (2 * extent)], -1).reshape(-1, 2)
    i = np.arange(n - 1)
    I, J = np.meshgrid(i, i)
    a = (J * n + I).reshape(-1)
    b = a + 1
    c = a + n
    d = c + 1
    idx = np.stack([a, c, b, b, c, d], 1).reshape(-1).astype(np.uint32)
    return Mesh(_vertices(pos, nrm, uv), idx), h


def trs(t=(0, 0, 0), s=1.0) -> np.ndarray:
    """Translate * uniform scale in glm storage (m[col][row])."""
    m = np.eye(4) * s
    m[3, 3] = 1.0
    m[3, 0:3] = t
    return m


def random_materials(rng: np.random.Generator, n: int) -> list:
    out = []
    for _ in range(n):
        albedo = rng.random(3)
        rough = float(rng.random())
        metal = float(rng.random() < 0.3)
        model = SHADING_MIRROR if rough < 0.3 else SHADING_PBR
        out.append(Material(shading_model=model, diffuse_color=(*albedo, 1.0), metallic_factor=metal,
                            roughness_factor=rough, ior=1.0))
    return out


def env_map(rng: np.random.Generator, w: int = 1024, h: int = 512, sun=True) -> np.ndarray:
    """Procedural equirect RGBA8 sky: vertical gradient, low-frequency noise, a sun disk."""
    v = (np.arange(h) + 0.5) / h
    u = (np.arange(w) + 0.5) / w
    U, V = np.meshgrid(u, v)
    elev = (0.5 - V) * np.pi
    sky = np.stack([0.35 + 0.3 * np.sin(elev).clip(0), 0.55 + 0.25 * np.sin(elev).clip(0), 0.85 + 0.1 * np.sin(elev)], -1)
    ground = np.array([0.25, 0.22, 0.2])
    col = np.where((elev > 0)[..., None], sky, ground)
    col = col * (0.85 + 0.3 * _value_noise(rng, max(w, h), 8)[:h, :w][..., None])
    if sun:
        su, sv = rng.random() , 0.25 + 0.1 * rng.random()
        d = np.hypot((U - su) * 2, V - sv)
        col = col + (d < 0.02)[..., None] * 1.0
    rgba = np.concatenate([np.clip(col, 0, 1), np.ones((h, w, 1))], -1)
    return np.round(rgba * 255).astype(np.uint8)


# ---- configurations ---------------------------------------------------------------
@dataclass
class Workload:
    name: str
    scene: Scene
    width: int
    height: int
    spp: int
    max_bounces: int
    rng_mode: int   # HY_RNG_*

    def camera(self, frame: float = 0.0) -> np.ndarray:
        return self.scene.camera.rt_camera(self.width, self.height, frame)


def small(seed: int = 0, width: int = 256, height: int = 256) -> Workload:
    rng = np.random.default_rng(seed)
    sc = Scene()
    sc.entities.append(Object(quad(20.0), 0, trs()))
    ico = icosphere(2)
    for i in range(16):
        r = rng.uniform(0.3, 0.8)
        c = (rng.uniform(-5, 5), rng.uniform(0.5, 1.5), rng.uniform(-5, 5))
        sc.entities.append(Object(ico, i + 1, trs(c, r)))
    sc.materials = random_materials(rng, 17)
    sc.lights = [Light(POINT_LIGHT, (1, 1, 1), (2, 6, 2), 20.0, 500.0, 0.1),
                 Light(DIRECTIONAL_LIGHT, (1, 1, 1), (0.3, 1.0, 0.2), 1.0, 500.0, 0.1)]
    sc.camera = Camera((0.0, 4.0, 10.0), (0.0, 0.0, 0.0), 60.0)
    sc.env = [env_map(rng), env_map(rng, sun=False)]
    return Workload("small-256x256-5k", sc, width, height, 1, 1, 0)


def hd(seed: int = 1, width: int = 1920, height: int = 1080, n_spheres: int = 48, sphere_subdiv: int = 5,
       terrain_n: int = 512, spp: int = 16) -> Workload:
    rng = np.random.default_rng(seed)
    sc = Scene()
    ter, hmap = terrain(rng, terrain_n)
    sc.materials = random_materials(rng, 256)
    sc.entities.append(Object(ter, int(rng.integers(256)), trs()))
    ico = icosphere(sphere_subdiv)
    for _ in range(n_spheres):
        s = rng.uniform(0.5, 3.0)
        x, z = rng.uniform(-40, 40), rng.uniform(-40, 40)
        sc.entities.append(Object(ico, int(rng.integers(256)), trs((x, s + 1.0, z), s)))
    sc.lights = [Light(POINT_LIGHT, (1, 1, 1), (rng.uniform(-30, 30), rng.uniform(8, 16), rng.uniform(-30, 30)),
                       float(rng.uniform(10, 50)), 500.0, 0.5) for _ in range(4)]
    sc.camera = Camera((0.0, 18.0, 55.0), (0.0, 0.0, 0.0), 60.0)
    sc.env = [env_map(rng), env_map(rng, sun=False)]
    return Workload(f"hd-{width}x{height}-{sc.num_tris // 1000}k", sc, width, height, spp, 1, 1)


def small_glass(width: int = 48, height: int = 48) -> Workload:
    """The small scene with glass spheres (ior 1.5), mirror spheres and a mirror
    floor, 8 bounces: exercises every shading model of hybridHit.rchit."""
    wl = small(0, width, height)
    for i in (2, 5, 9):
        wl.scene.materials[i] = Material(4, (0.9, 0.95, 1.0, 1), 1.0, 0.0, 1.5)
    for i in (3, 7):
        wl.scene.materials[i] = Material(3, (0.8, 0.8, 0.8, 1), 1.0, 0.05, 1.0)
    wl.scene.materials[0] = Material(3, (0.6, 0.6, 0.6, 1), 1.0, 0.1, 1.0)
    wl.max_bounces = 8
    wl.name = f"small-glass-{width}x{height}"
    return wl


def checker_texture(n: int, cells: int, a, b) -> np.ndarray:
    y, x = np.mgrid[0:n, 0:n]
    m = ((x * cells // n + y * cells // n) % 2).astype(bool)
    img = np.where(m[..., None], np.array(a, np.float64), np.array(b, np.float64))
    return np.round(np.concatenate([img, np.ones((n, n, 1))], -1) * 255).astype(np.uint8)


def small_textured(width: int = 64, height: int = 48) -> Workload:
    """The small scene with material textures (Texture::_textures, RGBA8 NEAREST/REPEAT):
    a checker diffuse texture on the floor (UVs 0..4, so REPEAT wraps) and on spheres, a
    metallic-roughness texture, an emissive texture, tinted vertex colours on the floor,
    textured mirror and glass spheres; 4 bounces."""
    rng = np.random.default_rng(5)
    wl = small(0, width, height)
    sc = wl.scene
    sc.textures = [checker_texture(64, 8, (0.9, 0.8, 0.2), (0.1, 0.3, 0.8)),
                   np.concatenate([rng.integers(0, 256, (32, 32, 3)), np.full((32, 32, 1), 255)], -1).astype(np.uint8),
                   checker_texture(16, 4, (0.6, 0.1, 0.1), (0.0, 0.0, 0.0))]
    floor = sc.entities[0].mesh
    v = floor.vertices.copy()
    v[:, 9:11] *= 4.0
    v[:, 6:9] = [[1.0, 0.7, 0.7], [0.7, 1.0, 0.7], [0.7, 0.7, 1.0], [1.0, 1.0, 0.5]]
    sc.entities[0].mesh = type(floor)(v, floor.indices)
    m = sc.materials
    m[0] = Material(0, (0.5, 0.5, 0.5, 1), 0.0, 0.6, 1.0, diffuse_texture=0)
    m[1] = Material(0, (0.5, 0.5, 0.5, 1), 0.5, 0.5, 1.0, diffuse_texture=0, metallic_roughness_texture=1)
    m[2] = Material(0, (0.8, 0.2, 0.2, 1), 0.0, 0.4, 1.0, emissive_texture=2)
    m[3] = Material(3, (0.8, 0.8, 0.8, 1), 1.0, 0.05, 1.0, diffuse_texture=0)
    m[4] = Material(4, (0.9, 0.95, 1.0, 1), 1.0, 0.0, 1.5, diffuse_texture=0, metallic_roughness_texture=1)
    m[5] = Material(0, (0.3, 0.6, 0.3, 1), 0.0, 0.5, 1.0, diffuse_texture=0, emissive_texture=2,
                    metallic_roughness_texture=1)
    wl.max_bounces = 4
    wl.width, wl.height = width, height
    wl.name = f"small-textured-{width}x{height}"
    return wl


def diff(seed: int = 3, width: int = 512, height: int = 512) -> Workload:
    rng = np.random.default_rng(seed)
    sc = Scene()
    sc.entities.append(Object(quad(30.0), 0, trs()))
    ico = icosphere(3)
    sc.materials = random_materials(rng, 64)
    for i in range(64):
        r = rng.uniform(0.3, 0.8)
        c = (rng.uniform(-8, 8), rng.uniform(0.5, 1.5), rng.uniform(-8, 8))
        sc.entities.append(Object(ico, int(rng.integers(64)), trs(c, r)))
    sc.lights = [Light(POINT_LIGHT, (1, 1, 1), (rng.uniform(-8, 8), rng.uniform(4, 8), rng.uniform(-8, 8)),
                       float(rng.uniform(10, 50)), 500.0, 0.3) for _ in range(8)]
    sc.camera = Camera((0.0, 8.0, 16.0), (0.0, 0.0, 0.0), 60.0)
    sc.env = [env_map(rng), env_map(rng, sun=False)]
    return Workload("diff-512x512-82k", sc, width, height, 16, 1, 1)


# ---- the large combined configuration ----------------------------------------------------
def torus(rng: np.random.Generator, nu: int = 32, nv: int = 32, R: float = 1.0, r: float = 0.35,
          displacement: float = 0.06) -> Mesh:
    """Torus of 2 nu nv triangles (2048 at 32 x 32) with a seeded radial displacement of the tube."""
    u = np.arange(nu) * 2 * np.pi / nu
    v = np.arange(nv) * 2 * np.pi / nv
    U, V = np.meshgrid(u, v, indexing="ij")
    bumps = 1.0 + displacement * (_value_noise(rng, max(nu, nv), 4)[:nu, :nv] - 0.5) * 2.0
    rr = r * bumps
    pos = np.stack([(R + rr * np.cos(V)) * np.cos(U), rr * np.sin(V), (R + rr * np.cos(V)) * np.sin(U)], -1)
    nrm = np.stack([np.cos(V) * np.cos(U), np.sin(V), np.cos(V) * np.sin(U)], -1)
    uv = np.stack([U / (2 * np.pi), V / (2 * np.pi)], -1)
    i, j = np.meshgrid(np.arange(nu), np.arange(nv), indexing="ij")
    a = i * nv + j
    b = ((i + 1) % nu) * nv + j
    c = i * nv + (j + 1) % nv
    d = ((i + 1) % nu) * nv + (j + 1) % nv
    idx = np.stack([a, c, b, b, c, d], -1).reshape(-1).astype(np.uint32)
    return Mesh(_vertices(pos.reshape(-1, 3), nrm.reshape(-1, 3), uv.reshape(-1, 2)), idx)


def _rotation(q: np.ndarray) -> np.ndarray:
    w, x, y, z = q / np.linalg.norm(q)
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def large(seed: int = 4, width: int = 3840, height: int = 2160, n_instances: int = 4096, terrain_n: int = 512,
          n_materials: int = 1024, n_lights: int = 64) -> Workload:
    """3840x2160: 4096 instances of 8 base meshes of ~2k triangles (4 geodesic icospheres of
    2,000 triangles and 4 displaced tori of 2,048) under random rotations, scale U[0.2, 4]
    and positions over the terrain, flattened into one BVH (~8.3M triangles) plus the 1080p
    configuration's 512x512 terrain (~8.8M in all); 1024 materials; 64 area lights (radius
    0.5, intensity U[10, 50]); 64 shadow samples per pixel spread over the lights (1 per
    light, DECORRELATED); 2 reflection bounces."""
    rng = np.random.default_rng(seed)
    sc = Scene()
    ter, hmap = terrain(rng, terrain_n)
    sc.materials = random_materials(rng, n_materials)
    sc.entities.append(Object(ter, int(rng.integers(n_materials)), trs()))
    bases = [geodesic_sphere(10) for _ in range(4)] + [torus(rng) for _ in range(4)]
    n = hmap.shape[0]
    for _ in range(n_instances):
        mesh = bases[int(rng.integers(len(bases)))]
        s = float(rng.uniform(0.2, 4.0))
        x, z = rng.uniform(-45, 45, 2)
        gi = int(np.clip((x + 50) / 100 * (n - 1), 0, n - 1))
        gj = int(np.clip((z + 50) / 100 * (n - 1), 0, n - 1))
        m = np.eye(4)
        m[:3, :3] = _rotation(rng.normal(size=4)) * s
        m[:3, 3] = (x, hmap[gj, gi] + s, z)
        sc.entities.append(Object(mesh, int(rng.integers(n_materials)), m.T.copy()))  # glm storage m[col][row]
    sc.lights = [Light(POINT_LIGHT, (1, 1, 1), (rng.uniform(-40, 40), rng.uniform(10, 20), rng.uniform(-40, 40)),
                       float(rng.uniform(10, 50)), 500.0, 0.5) for _ in range(n_lights)]
    sc.camera = Camera((0.0, 22.0, 62.0), (0.0, 0.0, 0.0), 60.0)
    sc.env = [env_map(rng), env_map(rng, sun=False)]
    return Workload(f"large-{width}x{height}-{sc.num_tris // 1000}k", sc, width, height, 1, 2, 1)


# ---- the mixed batch ------------------------------------------------------------------
BATCH_RESOLUTIONS = ((320, 240), (640, 480), (1280, 720), (1920, 1080))
BATCH_SPP = (1, 4, 16, 64)


def batch_scene(rng: np.random.Generator, n_tris: int) -> Scene:
    """A scene generated as the 1080p one (fBm terrain + icospheres of subdivision 5,
    20,480 triangles each, scale U[0.5, 3]; 256 materials; area lights of radius 0.5,
    intensity U[10, 50]) with about n_tris triangles (35 % terrain, 65 % spheres) and 8
    lights (a view uses the first 1..8)."""
    sc = Scene()
    n_ter = max(8, int(round(np.sqrt(0.35 * n_tris / 2.0))) + 1)
    ter, _ = terrain(rng, n_ter)
    sc.materials = random_materials(rng, 256)
    sc.entities.append(Object(ter, int(rng.integers(256)), trs()))
    ico = icosphere(5)
    for _ in range(max(1, int(round(0.65 * n_tris / ico.num_tris)))):
        s = rng.uniform(0.5, 3.0)
        x, z = rng.uniform(-40, 40), rng.uniform(-40, 40)
        sc.entities.append(Object(ico, int(rng.integers(256)), trs((x, s + 1.0, z), s)))
    sc.lights = [Light(POINT_LIGHT, (1, 1, 1), (rng.uniform(-30, 30), rng.uniform(8, 16), rng.uniform(-30, 30)),
                       float(rng.uniform(10, 50)), 500.0, 0.5) for _ in range(8)]
    sc.env = [env_map(rng), env_map(rng, sun=False)]
    return sc


def batch(seed: int = 2, n_scenes: int = 8, n_views: int = 64, tri_range=(50_000, 2_000_000)):
    """64 views over 8 scenes: triangle counts log-uniform in [50k, 2M],
    resolution uniform in {320x240, 640x480, 1280x720, 1920x1080}, shadow spp
    uniform in {1, 4, 16, 64} (DECORRELATED), light count uniform in [1, 8],
    cameras on a ring around each scene.  Returns (scenes, view specs); a view
    spec holds scene, width, height, spp, lights, camera (Camera)."""
    rng = np.random.default_rng(seed)
    lo, hi = np.log(tri_range[0]), np.log(tri_range[1])
    counts = np.exp(rng.uniform(lo, hi, n_scenes)).astype(int)
    scs = [batch_scene(rng, int(n)) for n in counts]
    views = []
    for _ in range(n_views):
        si = int(rng.integers(n_scenes))
        w, h = BATCH_RESOLUTIONS[int(rng.integers(len(BATCH_RESOLUTIONS)))]
        spp = BATCH_SPP[int(rng.integers(len(BATCH_SPP)))]
        nl = int(rng.integers(1, 9))
        ang = rng.uniform(0, 2 * np.pi)
        cam = Camera((55.0 * np.sin(ang), float(rng.uniform(12, 24)), 55.0 * np.cos(ang)), (0.0, 0.0, 0.0), 60.0)
        views.append(dict(scene=si, width=w, height=h, spp=spp, lights=nl, camera=cam))
    return scs, views
