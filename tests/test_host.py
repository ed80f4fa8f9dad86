"""CPU tests of the host side: the C-ABI library loads and exports every
entry point hybridrt.h declares, struct layouts, scene packing against the
reference's packing code, camera matrices and the synthetic workloads."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from vulkanhybridraytracer_gb300 import _lib as L
from vulkanhybridraytracer_gb300 import build, scenes
from vulkanhybridraytracer_gb300.scene import DIRECTIONAL_LIGHT, Camera, Light, Material

ROOT = Path(__file__).resolve().parent.parent


def header_functions():
    src = (ROOT / "include" / "hybridrt.h").read_text()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(hy_\w+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    build.build_cuda()
    return L.load()


def test_library_exports_every_header_symbol(lib):
    names = header_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(L.PROTOTYPES), "ctypes prototypes and the header disagree"
    assert lib.hy_get_abi_version() == 5


def test_error_strings(lib):
    for code in range(0, -12, -1):
        s = lib.hy_error_string(code).decode()
        assert s and s != "unknown error"


def test_null_arguments_rejected(lib):
    assert lib.hy_create(None, None) == L.HY_ERR_INVALID_ARG
    assert lib.hy_scene_set_materials(None, None, 0) == L.HY_ERR_INVALID_ARG
    assert lib.hy_hybrid_forward(None, None, None, None, None, None, None, None) == L.HY_ERR_INVALID_ARG
    assert lib.hy_scene_set_anyhit_order(None, L.HY_ANYHIT_FAR_FIRST) == L.HY_ERR_INVALID_ARG
    assert lib.hy_scene_anyhit_order(None, None) == L.HY_ERR_INVALID_ARG
    assert lib.hy_bvh_build(None, None) == L.HY_ERR_INVALID_ARG
    lib.hy_destroy(None)


def test_create_without_gpu_fails_cleanly(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    info = L.HyCreateInfo(0, 0, None, 0)
    assert lib.hy_create(C.byref(h), C.byref(info)) == L.HY_ERR_CUDA
    assert not h.value


def test_struct_layouts():
    assert C.sizeof(L.HyLight) == 48          # uboLight, std140
    assert C.sizeof(L.HyMaterial) == 48       # GPUMaterial
    assert C.sizeof(L.HyVertex) == 44         # Vertex (src/vk_mesh.h:21-33)
    assert C.sizeof(L.HyCamera) == 144        # RTCameraData
    assert C.sizeof(L.HyPrimitive) == 24
    assert C.sizeof(L.HyStats) == 48
    assert C.sizeof(L.HyPassConfig) == 44
    assert C.sizeof(L.HyBvhLayout) == 32
    assert L.HyGBuffer.plane.offset == 8


def test_material_to_shader():
    """Material::materialToShader (src/material.cpp:19-26)."""
    m = Material(shading_model=3, diffuse_color=(0.1, 0.2, 0.3, 1), metallic_factor=0.7, roughness_factor=0.2,
                 ior=1.5, diffuse_texture=4, normal_texture=5, emissive_texture=6, metallic_roughness_texture=7)
    v = m.to_shader(9)
    np.testing.assert_array_equal(v, np.float32([0.1, 0.2, 0.3, 1.5, 4, 5, 6, 7, 3, 0.7, 0.2, 9]))
    d = Material()
    assert (d.metallic_factor, d.roughness_factor, d.ior) == (1.0, 1.0, 1.0)   # src/material.h:17-29


def test_light_to_ubo():
    """VulkanEngine::update light packing (src/vk_engine.cpp:146-164)."""
    p = Light(position=(1, 2, 3), color=(0.5, 0.5, 1), intensity=30, max_distance=40, radius=0.25).to_ubo()
    np.testing.assert_array_equal(p[:9], np.float32([1, 2, 3, 40, 0.5, 0.5, 1, 30, 0.25]))
    d = Light(DIRECTIONAL_LIGHT, position=(0, 1, 0)).to_ubo()
    assert d[3] == -1
    dflt = Light()
    assert (dflt.intensity, dflt.max_distance, dflt.radius) == (1000.0, 500.0, 1.0)  # src/entity.h:64


def test_camera_matrices():
    cam = Camera((0, 4, 10), (0, 0, 0), 60)
    m = cam.rt_camera(256, 256, 3.0)
    iv = m[0:16].reshape(4, 4)   # glm storage: iv[col][row]
    np.testing.assert_allclose(iv[3, :3], [0, 4, 10], atol=1e-5)   # camera position = column 3
    # centre ray: invProj * (0, 0, 1, 1) points down -z in view space
    ip = m[16:32].reshape(4, 4)
    t = ip.T @ np.array([0, 0, 1, 1.0])
    d = t[:3] / np.linalg.norm(t[:3])
    np.testing.assert_allclose(d, [0, 0, -1], atol=1e-6)
    # the Vulkan Y flip: NDC y = +1 maps to view-space -y
    t = ip.T @ np.array([0, 1, 1, 1.0])
    assert t[1] < 0
    assert m[32] == 3.0


def test_workload_sizes():
    """Triangle counts of the configurations."""
    assert scenes.small(0).scene.num_tris == 2 + 16 * 320
    assert scenes.diff(3).scene.num_tris == 2 + 64 * 1280
    assert scenes.icosphere(5).num_tris == 20480
    ter, _ = scenes.terrain(np.random.default_rng(0), 512)
    assert ter.num_tris == 511 * 511 * 2
    # the 4K configuration: 4096 instances of 8 base meshes of ~2k triangles + the terrain
    assert scenes.geodesic_sphere(10).num_tris == 2000
    assert scenes.torus(np.random.default_rng(0)).num_tris == 2048
    large = scenes.large()
    assert len(large.scene.entities) == 4097
    assert 8.2e6 < large.scene.num_tris - 511 * 511 * 2 < 8.4e6
    # the mixed batch: 8 scenes of log-uniform [50k, 2M] triangles
    scs, views = scenes.batch(2)
    assert len(scs) == 8 and len(views) == 64
    assert all(45_000 < sc.num_tris < 2_100_000 for sc in scs)


def test_geodesic_sphere_is_closed_and_outward():
    g = scenes.geodesic_sphere(7)
    f = g.indices.reshape(-1, 3).astype(np.int64)
    e = np.sort(np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]]), 1)
    _, counts = np.unique(e, axis=0, return_counts=True)
    assert g.num_tris == 20 * 49 and set(counts.tolist()) == {2}   # every edge shared by two triangles
    v = g.vertices[:, :3].astype(np.float64)
    n = np.cross(v[f[:, 1]] - v[f[:, 0]], v[f[:, 2]] - v[f[:, 0]])
    assert np.all((n * (v[f[:, 0]] + v[f[:, 1]] + v[f[:, 2]])).sum(1) > 0)
    np.testing.assert_allclose(np.linalg.norm(v, axis=1), 1.0, atol=1e-6)


def test_scene_pack_roundtrip():
    wl = scenes.small(0)
    verts, idx, prims, xf, mats, lights = wl.scene.pack()
    assert verts.shape[1] == 11 and verts.dtype == np.float32
    assert prims.shape == (17, 6)
    assert int(prims[:, 1].sum()) // 3 == wl.scene.num_tris
    assert np.all(idx[prims[0, 0]:prims[0, 0] + prims[0, 1]] < 4)
    assert mats.shape == (17, 12) and lights.shape == (2, 12)
    assert lights[1, 3] == -1  # directional


def _bench():
    import importlib.util
    root = Path(__file__).resolve().parent.parent
    spec = importlib.util.spec_from_file_location("bench_under_test", root / "bench.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_bench_source_hash_ignores_comments():
    """The ncu evidence in profiles/ is tied to a hash of the kernels' code with
    comments and blank lines stripped: a comment edit keeps it, a code edit does not."""
    b = _bench()
    src = {f: (b.ROOT / "vulkanhybridraytracer_gb300" / "csrc" / f).read_text() for f in b.KERNEL_SOURCES}
    base = b.kernel_source_sha(src.__getitem__)
    assert base == b.kernel_source_sha()
    f0 = b.KERNEL_SOURCES[0]
    commented = dict(src)
    commented[f0] = "// a new comment\n\n/* and a block\n   comment */\n" + src[f0].replace("\n", "  // note\n", 3)
    assert b.kernel_source_sha(commented.__getitem__) == base
    changed = dict(src)
    changed[f0] = src[f0] + "\nstatic int kUnused = 1;\n"
    assert b.kernel_source_sha(changed.__getitem__) != base
    assert b.code_of("a; // x\n\n  /* y */ b;\n") == "a;\n   b;"


def test_bench_profile_records():
    """Every key bench.py reads from the dominant kernel's ncu summaries is there."""
    b = _bench()
    rec = b.profile_records("k_shadow_stream<accum>")
    for k in ("source_sha", "case", "dram_bytes_1920x1080", "dram_gbs", "issue_active_pct", "lanes_per_inst",
              "alu_pipe_pct", "l2_gbs", "l2_bytes"):
        assert k in rec, k
    assert len(rec["source_sha"][0]) == 16
    assert rec["dram_bytes_1920x1080"][1].startswith("profiles/")
    assert b.profile_records("no_such_kernel") == {}
