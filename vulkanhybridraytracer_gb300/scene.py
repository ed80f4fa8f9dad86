"""Host-side mirror of the reference's scene model, packed for the C ABI.

The classes follow VkPinut's data model so a user of the reference finds the
same fields with the same defaults:

* ``Material``  src/material.h:12-37; ``to_shader`` is
  Material::materialToShader (src/material.cpp:19-26).
* ``Light``     src/entity.h:56-69 (type, colour, position, intensity 1000,
  maxDistance 500, radius 1); ``to_ubo`` is the uboLight packing of
  VulkanEngine::update (src/vk_engine.cpp:146-164).
* ``Mesh`` / ``Object``  src/vk_mesh.h:21-33 (44-byte Vertex) and
  src/entity.h:38-52; one Object = one Primitive of its Prefab.
* ``Camera``    src/camera.h:25 / src/camera.cpp:49-58 (fov 60, near 0.1,
  far 1000) with the Vulkan Y flip of src/vk_engine.cpp:695 and the
  RTCameraData inverse matrices of src/vk_engine.cpp:727-733.
* ``Scene``     src/scene.h:7-22.

``Scene.pack`` produces the arrays of hy_scene_set_geometry /
hy_scene_set_materials / hy_scene_set_lights.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

POINT_LIGHT = 0
DIRECTIONAL_LIGHT = 1

SHADING_PBR = 0      # metallic-roughness, no reflection rays in the hybrid pass
SHADING_MIRROR = 3   # "MIRALL" (hybridHit.rchit:347)
SHADING_GLASS = 4    # "VIDRE"  (hybridHit.rchit:357)


@dataclass
class Material:
    shading_model: int = 0
    diffuse_color: tuple = (1.0, 1.0, 1.0, 1.0)
    metallic_factor: float = 1.0
    roughness_factor: float = 1.0
    ior: float = 1.0
    uv_factor: float = 1.0
    diffuse_texture: int = -1
    metallic_roughness_texture: int = -1
    emissive_texture: int = -1
    normal_texture: int = -1

    def to_shader(self, index: int) -> np.ndarray:
        """GPUMaterial: diffuse = (rgb, ior), textures, smr = (model, metallic, roughness, index)."""
        d = self.diffuse_color
        return np.array([d[0], d[1], d[2], self.ior,
                         self.diffuse_texture, self.normal_texture, self.emissive_texture,
                         self.metallic_roughness_texture,
                         self.shading_model, self.metallic_factor, self.roughness_factor, index], np.float32)


@dataclass
class Light:
    type: int = POINT_LIGHT
    color: tuple = (1.0, 1.0, 1.0)
    position: tuple = (0.0, 0.0, 0.0)
    intensity: float = 1000.0
    max_distance: float = 500.0
    radius: float = 1.0

    def to_ubo(self) -> np.ndarray:
        """uboLight: pos = (xyz, maxDistance or -1), color = (rgb, intensity), radius.

        For a directional light the reference leaves ``radius`` untouched
        (src/vk_engine.cpp:151-154); it is never read because directional
        lights are never traced, so it is packed as the light's radius.
        """
        w = -1.0 if self.type == DIRECTIONAL_LIGHT else self.max_distance
        p, c = self.position, self.color
        return np.array([p[0], p[1], p[2], w, c[0], c[1], c[2], self.intensity,
                         self.radius, 0, 0, 0], np.float32)


@dataclass
class Mesh:
    """Vertices (N, 11) float32 = pos3 normal3 color3 uv2; indices uint32."""
    vertices: np.ndarray
    indices: np.ndarray

    @property
    def num_tris(self) -> int:
        return len(self.indices) // 3


@dataclass
class Object:
    mesh: Mesh
    material_idx: int = 0
    matrix: np.ndarray = field(default_factory=lambda: np.eye(4, dtype=np.float32))


def look_at(eye, center, up=(0.0, 1.0, 0.0)) -> np.ndarray:
    """glm::lookAt (right-handed); returns the matrix as M[col][row] like glm."""
    eye, center, up = (np.asarray(v, np.float64) for v in (eye, center, up))
    f = center - eye
    f /= np.linalg.norm(f)
    s = np.cross(f, up)
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    m = np.eye(4)
    m[0, 0], m[1, 0], m[2, 0] = s
    m[0, 1], m[1, 1], m[2, 1] = u
    m[0, 2], m[1, 2], m[2, 2] = -f
    m[3, 0] = -s.dot(eye)
    m[3, 1] = -u.dot(eye)
    m[3, 2] = f.dot(eye)
    return m


def perspective(fovy_rad: float, aspect: float, near: float, far: float) -> np.ndarray:
    """glm::perspective (right-handed, clip z in [-1, 1]) as M[col][row]."""
    t = np.tan(fovy_rad / 2.0)
    m = np.zeros((4, 4))
    m[0, 0] = 1.0 / (aspect * t)
    m[1, 1] = 1.0 / t
    m[2, 2] = -(far + near) / (far - near)
    m[2, 3] = -1.0
    m[3, 2] = -(2.0 * far * near) / (far - near)
    return m


@dataclass
class Camera:
    position: tuple = (0.0, 0.0, 0.0)
    target: tuple = (0.0, 0.0, -1.0)
    fov: float = 60.0
    near: float = 0.1
    far: float = 1000.0

    def view(self) -> np.ndarray:
        return look_at(self.position, self.target)

    def projection(self, aspect: float) -> np.ndarray:
        p = perspective(np.radians(self.fov), aspect, self.near, self.far)
        p[1, 1] *= -1.0  # src/vk_engine.cpp:695
        return p

    def rt_camera(self, width: int, height: int, frame: float = 0.0) -> np.ndarray:
        """RTCameraData as 36 float32: invView (16), invProj (16), frame vec4."""
        iv = np.linalg.inv(self.view().T).T   # M[col][row] storage: invert the row-major view
        ip = np.linalg.inv(self.projection(width / height).T).T
        out = np.zeros(36, np.float32)
        out[0:16] = iv.astype(np.float32).reshape(-1)   # column-major (M[col] contiguous)
        out[16:32] = ip.astype(np.float32).reshape(-1)
        out[32:36] = frame
        return out


@dataclass
class Scene:
    entities: list = field(default_factory=list)
    lights: list = field(default_factory=list)
    materials: list = field(default_factory=list)
    camera: Camera = field(default_factory=Camera)
    env: list = field(default_factory=list)   # [sky, irradiance], each (h, w, 4) uint8
    # Texture::_textures in load order: (h, w, 4) uint8 RGBA8 images; a material's
    # *_texture field is an index into this list (-1: none)
    textures: list = field(default_factory=list)

    def pack(self):
        """Arrays for the C ABI: verts (N,11) f32, idx u32, prims (P,6) u32,
        transforms (T,16) f32 column-major, materials (M,12) f32, lights (L,12) f32."""
        verts, idx, prims, xf = [], [], [], []
        vofs = iofs = 0
        placed = {}  # a mesh shared by several entities is packed once (its Prefab's buffers)
        for e_i, ob in enumerate(self.entities):
            m = ob.mesh
            if id(m) not in placed:
                placed[id(m)] = (iofs, vofs)
                verts.append(np.asarray(m.vertices, np.float32))
                idx.append(np.asarray(m.indices, np.uint32))
                vofs += len(m.vertices)
                iofs += len(m.indices)
            fi, vo = placed[id(m)]
            prims.append([fi, len(m.indices), vo, ob.material_idx, e_i, e_i])
            xf.append(np.asarray(ob.matrix, np.float64).astype(np.float32).reshape(-1))
        mats = np.stack([mt.to_shader(i) for i, mt in enumerate(self.materials)])
        lights = (np.stack([l.to_ubo() for l in self.lights]) if self.lights
                  else np.zeros((0, 12), np.float32))
        return (np.ascontiguousarray(np.concatenate(verts)), np.ascontiguousarray(np.concatenate(idx)),
                np.ascontiguousarray(np.array(prims, np.uint32)), np.ascontiguousarray(np.stack(xf)),
                np.ascontiguousarray(mats), np.ascontiguousarray(lights))

    @property
    def num_tris(self) -> int:
        return sum(e.mesh.num_tris for e in self.entities)
