"""Milton scene-file loader (milton_gb300/sceneloader.py): the reference loader's grammar, key
order, scene-graph flattening, transforms, meshes and the GPU path's refusals.  CPU only."""
import math
import os
import struct
from pathlib import Path

import numpy as np
import pytest

from milton_gb300 import sceneloader as L

HERE = Path(__file__).resolve().parent
# the reference tree, when present (MILTON_REFERENCE, as for the oracle built from its sources)
REF_SCENES = Path(os.environ.get("MILTON_REFERENCE", "/root/reference")) / "mlt" / "src" / "exec" / "scenes"


def _scene(body: str, extra: str = "") -> str:
    return '{ "scenefile" : { ' + extra + ' "scene" : { ' + body + ' } } }'


def test_grammar_comments_trailing_commas_repeats_and_numbers():
    root = L.parse_text('{ /* c */ "a" : 1, "b" : 1.5, "c" : [1, 2., .5, -3e2, ], "a" : "x", "d" : { }, '
                        '"e" : [ ], "f" : null, "g" : true, }')
    assert [k for k, _ in root.items()] == ["a", "a", "b", "c", "d", "e", "f", "g"]
    assert root.find("a") == 1 and isinstance(root.find("a"), int)
    assert isinstance(root.find("b"), float)
    c = root.find("c")
    assert c == [1, 2.0, 0.5, -300.0] and isinstance(c[0], int) and all(isinstance(x, float) for x in c[1:])
    assert root.find("f") is None and root.find("g") is True
    with pytest.raises(L.SceneFileError):
        L.parse_text('{ "a" : [1 2] }')
    with pytest.raises(L.SceneFileError):
        L.parse_text('[1, 2]')


def test_reading_joins_lines_like_the_reference(tmp_path):
    p = tmp_path / "s.js"
    p.write_text('{ "a" : 1, // comment\n "b" : 2 }\n')
    # lines are joined without separators: the // comment swallows the rest of the file
    with pytest.raises(L.SceneFileError):
        L.parse_text(L.read_scene_text(str(p)))
    p.write_text('{ "a" : 1,\n "b" : 2 }')  # no newline at the end: the last line is dropped
    assert L.read_scene_text(str(p)) == '{ "a" : 1,'
    p.write_text('{ "a" : "' + "x" * 300 + '" }\n')
    with pytest.raises(L.SceneFileError, match="characters"):
        L.read_scene_text(str(p))


def test_keys_are_visited_in_multimap_order():
    text = _scene('"triangle" : { "vertices" : [0,0,0, 1,0,0, 0,0,1] }, '
                  '"material" : { "bsdf" : { "type" : "diffuse", "kd" : 0.25 }, '
                  '"triangle" : { "vertices" : [0,1,0, 1,1,0, 0,1,1] } }, '
                  '"plane" : { "vertices" : [0,2,0, 1,2,0, 1,2,1, 0,2,1] }')
    sf = L.loads(text)
    s = sf.scene
    # material (its triangle) first, then plane (two triangles), then the top-level triangle
    assert s.ntri == 4
    assert np.allclose(s.tri_v[0, 0], [0, 1, 0]) and np.allclose(s.tri_v[1:3, :, 1], 2.0)
    assert np.allclose(s.tri_v[3, 0], [0, 0, 0])
    assert s.tri_mat.tolist() == [1, 0, 0, 0]
    assert s.materials[1, 1] == np.float32(0.25) and s.materials[0, 1] == np.float32(0.5)
    # planes given by vertices are the culled triangles (v1 v2 v3), (v1 v3 v4)
    assert np.allclose(s.tri_v[1], [[0, 2, 0], [1, 2, 0], [1, 2, 1]])
    assert np.allclose(s.tri_v[2], [[0, 2, 0], [1, 2, 1], [0, 2, 1]])
    assert (s.tri_flags[:4] & 1).tolist() == [1, 1, 1, 1]


def test_material_inside_a_shape_applies_to_nothing():
    text = _scene('"triangle" : { "vertices" : [0,0,0, 1,0,0, 0,0,1], '
                  '"material" : { "bsdf" : { "type" : "diffuse", "kd" : 0.1 } } }')
    s = L.loads(text).scene
    assert s.tri_mat.tolist() == [0]


def test_nested_shape_sets_never_reach_the_scene():
    text = _scene('"shapeSet" : { "triangle" : { "vertices" : [0,0,0, 1,0,0, 0,0,1] } }, '
                  '"triangle" : { "vertices" : [0,1,0, 1,1,0, 0,1,1] }')
    s = L.loads(text).scene
    assert s.ntri == 1 and np.allclose(s.tri_v[0, 0], [0, 1, 0])


def _rodrigues(axis, deg):
    k = np.asarray(axis, float) / np.linalg.norm(axis)
    a = math.radians(deg)
    K = np.array([[0, -k[2], k[1]], [k[2], 0, -k[0]], [-k[1], k[0], 0]])
    return np.eye(3) + math.sin(a) * K + (1 - math.cos(a)) * K @ K


def test_rotation_matches_the_axis_angle_formula():
    rng = np.random.default_rng(0)
    for _ in range(20):
        axis, deg, p = rng.normal(size=3), rng.uniform(-360, 360), rng.normal(size=3)
        m = L.rotation(p, axis, deg)
        R = _rodrigues(axis, deg)
        assert np.allclose(m[:3, :3], R, atol=1e-12)
        assert np.allclose(m[:3, :3] @ p + m[:3, 3], p, atol=1e-12)  # the point stays fixed


def test_transform_is_translate_rotate_scale_and_unit_plane_light():
    text = _scene('"material" : { "emitter" : { "type" : "oriented", "power" : [2, 4, 6] }, '
                  '"transform" : { "scale" : [2, 1, 3], "translate" : [1, 5, 0], '
                  '"rotate" : [0, 0, 0, 1, 0, 0, 180], "plane" : { } } }')
    s = L.loads(text).scene
    assert s.ntri == 2 and s.tri_light.tolist() == [0, 0] and (s.tri_flags & 1).tolist() == [0, 0]
    rec = s.lights[0]
    # p = T R S p_obj: the unit square scaled to 2 x 3, turned upside down, moved to (1, 5, 0)
    assert np.allclose(rec[0:3], [1, 5, 0], atol=1e-6)
    assert np.allclose(rec[3:6], [2, 0, 0], atol=1e-6) and np.allclose(rec[6:9], [0, 0, -3], atol=1e-6)
    assert np.allclose(rec[9:12], [0, -1, 0], atol=1e-6)  # +y turned to -y
    assert rec[12] == pytest.approx(6.0)
    assert np.allclose(rec[13:16], np.array([2, 4, 6]) / (6.0 * math.pi))  # Le = power / (area pi)
    assert np.allclose(np.sort(s.tri_v[:, :, 1].ravel()), 5.0, atol=1e-6)


def test_cube_and_obj_mesh_with_quads_negative_indices_and_normals(tmp_path):
    (tmp_path / "q.obj").write_text("v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nvn 0 0 2\n"
                                    "f -4//1 -3//1 -2//1 -1//1\n")
    (tmp_path / "s.js").write_text(_scene('"mesh" : { "path" : "q.obj" }, "cube" : { }') + "\n")
    s = L.load(str(tmp_path / "s.js")).scene
    assert s.ntri == 12 + 2
    assert [sh[0] for sh in s.shapes] == ["cube", "q.obj"]  # "cube" < "mesh"
    q = s.tri_v[12:]
    assert np.allclose(q[0], [[0, 0, 0], [1, 0, 0], [1, 1, 0]]) and np.allclose(q[1], [[0, 0, 0], [1, 1, 0], [0, 1, 0]])
    assert np.allclose(s.tri_n[12:], [0, 0, 2])  # file normals, not normalised (Milton interpolates raw)
    c = s.tri_v[:12]
    assert np.allclose(np.abs(c), 0.5)
    fn = np.cross(c[:, 1] - c[:, 0], c[:, 2] - c[:, 0])
    assert np.all(np.einsum("ij,ij->i", fn, s.tri_n[:12, 0]) > 0)  # normals point out of the cube


def test_mesh_normals_computed_like_milton_and_ply(tmp_path):
    verts, faces, normals, nf = L.load_mesh(str(HERE / "scenes" / "octahedron.obj"))
    assert normals is None and faces.shape == (8, 3)
    vn = L.mesh_vertex_normals(verts, faces)
    assert np.allclose(vn, verts / np.linalg.norm(verts, axis=1, keepdims=True))
    # PLY, ascii and binary little endian, float32 vertices and 'list uchar int' faces
    hdr = "ply\nformat {}\nelement vertex 4\nproperty float x\nproperty float y\nproperty float z\n" \
          "element face 1\nproperty list uchar int vertex_indices\nend_header\n"
    (tmp_path / "a.ply").write_text(hdr.format("ascii 1.0") + "0 0 0\n1 0 0\n1 1 0\n0 1 0\n4 0 1 2 3\n")
    body = struct.pack("<12f", 0, 0, 0, 1, 0, 0, 1, 1, 0, 0, 1, 0) + struct.pack("<B4i", 4, 0, 1, 2, 3)
    (tmp_path / "b.ply").write_bytes(hdr.format("binary_little_endian 1.0").encode() + body)
    for name in ("a.ply", "b.ply"):
        v, f, n, _ = L.load_mesh(str(tmp_path / name))
        assert f.tolist() == [[0, 1, 2], [0, 2, 3]] and np.allclose(v[2], [1, 1, 0]) and n is None
    (tmp_path / "c.ply").write_text(hdr.format("ascii 1.0").replace("property float x", "property double x")
                                    + "0 0 0\n1 0 0\n1 1 0\n0 1 0\n4 0 1 2 3\n")
    with pytest.raises(L.SceneFileError, match="float32"):
        L.load_mesh(str(tmp_path / "c.ply"))


def test_camera_defaults_and_output_size():
    sf = L.loads(_scene('"triangle" : { }', '"camera" : { "type" : "pinhole", "eye" : [0, 0, 5] }, '
                                            '"output" : { "size" : [64, 32] },'))
    cam = sf.scene.camera
    assert np.allclose(cam[0:3], [0, 0, 5]) and np.allclose(cam[3:6], [0, 0, -1])
    assert np.allclose(cam[6:9], np.array([-1, 2, -1]) / math.sqrt(6), atol=1e-6)  # default camera's v axis
    assert cam[9] == 45.0 and cam[10] == 1.0
    assert (sf.width, sf.height) == (64, 32)
    assert (L.loads(_scene('"triangle" : { }')).width, L.loads(_scene('"triangle" : { }')).height) == (480, 480)


@pytest.mark.parametrize("body,extra,msg", [
    ('"transform" : { "scale" : [1, 2, 1], "sphere" : { "radius" : 1 } }', "", "non-uniform scale"),
    ('"cylinder" : { }', "", "not supported"),
    ('"material" : { "emitter" : { "type" : "oriented", "power" : 1 }, "cube" : { } }', "", "emitting cube"),
    ('"transform" : { "translate" : [0, 0, 0], "name" : "x", "plane" : { } }', "", "unknown key"),
    ('"triangle" : { }', '"renderer" : { "type" : "pathTracer" }, "renderer" : { "type" : "pathTracer" },',
     "multiple renderer definitions"),
    ('"material" : { "bsdf" : { "type" : "diffuse", "kd" : 2 } }', "", "clampedSpectrum"),
    ('"material" : { "bsdf" : { "type" : "glass" } }', "", "invalid bsdf type"),
])
def test_refusals_name_the_element(body, extra, msg):
    with pytest.raises(L.SceneFileError, match=msg):
        L.loads(_scene(body, extra))


def test_missing_scene_is_an_error():
    with pytest.raises(L.SceneFileError, match="missing required key 'scene'"):
        L.loads('{ "scenefile" : { "version" : 0.1 } }')


def test_box_scene_file_and_path_tracer_settings():
    sf = L.load(str(HERE / "scenes" / "box.js"))
    s = sf.scene
    assert s.ntri == 2 + 10 + 12 + 8 + 1 and len(s.lights) == 1
    assert (sf.width, sf.height) == (48, 40)
    r = L.path_tracer(sf)
    st = r.settings()
    assert (st.width, st.height, st.spp, st.max_depth, st.rr_start_depth) == (48, 40, 16, 5, 3)
    assert s.materials[s.tri_mat[-9], 0] == 2 and s.materials[s.tri_mat[-9], 8] == np.float32(1.5)


@pytest.mark.skipif(not REF_SCENES.exists(), reason="reference scene files not present")
def test_reference_cornell_box_file():
    sf = L.load(str(REF_SCENES / "cornellBox.js"))
    s = sf.scene
    # one unit-plane light (2 triangles) and 15 planes given by vertices (30 culled triangles)
    assert s.ntri == 32 and len(s.lights) == 1 and int((s.tri_flags & 1).sum()) == 30
    rec = s.lights[0]
    assert rec[12] == pytest.approx(140 * 125)
    assert np.allclose(rec[13:16], np.array([2e6, 2e6, 1.6e6]) / (140 * 125 * math.pi), rtol=1e-6)
    assert np.allclose(rec[9:12], [0, -1, 0], atol=1e-6)
    assert sf.renderer["type"] == "preview" and sf.renderer["noSuperSamples"] == 1024


def test_triangle_and_mesh_emitters():
    sf = L.load(str(HERE / "scenes" / "emitters.js"))
    s = sf.scene
    ext = s.light_ext
    kinds = ext[:, 0].astype(int).tolist()
    # in flatten order: the ceiling's two Triangles, the triangle shape, the mesh, the unit plane
    assert kinds == [1, 1, 1, 2, 0]
    # ceiling triangles: object-space area 0.18 each, uv frames of Milton's plane split
    assert np.allclose(s.lights[0:2, 12], 0.18) and np.allclose(ext[0, 1:8], [0, 0, 0, 1, 1, 1, 1])
    assert np.allclose(ext[1, 1:8], [0, 0, 1, 1, 1, 0, 1])
    assert np.allclose(s.lights[0, 13:16], np.array([3, 3, 2.5]) / (0.18 * math.pi))
    # the mesh light covers its 8 triangles, area = world-space area of the scaled octahedron
    first, count = ext[3].view(np.uint32)[8:10]
    assert count == 8 and np.all(s.tri_light[first:first + count] == 3)
    oct_area = 8 * 0.5 * np.linalg.norm(np.cross([-1, 1, 0], [-1, 0, 1])) * 0.25 ** 2
    assert s.lights[3, 12] == pytest.approx(oct_area, rel=1e-6)
    # every emitting triangle points at its light record
    assert sorted(set(s.tri_light.tolist()) - {-1}) == [0, 1, 2, 3, 4]


def test_thin_lens_camera_record():
    sf = L.loads(_scene('"triangle" : { }', '"camera" : { "type" : "thinlens", "eye" : [0, 0, 5], '
                                            '"aperture" : 50, "fstop" : 10, "focalDistance" : 4.5 },'))
    cam = sf.scene.camera
    assert cam[11] == pytest.approx(0.05) and cam[12] == pytest.approx(0.5) and cam[13] == pytest.approx(4.5)
    # no focalDistance: autofocus on the scene centre, fallback 1 (resolved once resident)
    cam = L.loads(_scene('"triangle" : { }', '"camera" : { "type" : "thinlens" },')).scene.camera
    assert cam[11] == pytest.approx(0.035) and cam[12] == pytest.approx(0.49)
    assert cam[13] == -1.0 and tuple(cam[14:16]) == (0.5, 0.5)
    # a pinhole camera ignores its aperture key
    cam = L.loads(_scene('"triangle" : { }', '"camera" : { "type" : "pinhole", "aperture" : 100 },')).scene.camera
    assert cam[11] == 0.0


def test_output_filters():
    sf = L.loads(_scene('"triangle" : { }', '"output" : { "type" : "default", "width" : 8, "height" : 8 },'))
    assert sf.output["filter"] == ("lanczosSinc", 2.0, {"tau": 3.0})
    sf = L.loads(_scene('"triangle" : { }', '"output" : { "filter" : { "type" : "gaussian", "support" : 3, '
                                            '"sigma" : 0.7 } },'))
    assert sf.output["type"] == "reconstruction" and sf.output["filter"] == ("gaussian", 3.0, {"sigma": 0.7})
    sf = L.loads(_scene('"triangle" : { }', '"output" : { "type" : "naive", "width" : 8 },'))
    assert "filter" not in sf.output
    assert L.path_tracer(L.loads(_scene('"triangle" : { }', '"renderer" : { "type" : "pathTracer" }, '
                                        '"output" : { "filter" : "mitchell" },'))).output_filter == \
        ("mitchell", 2.0, {"B": 1 / 3, "C": 1 / 3})
    with pytest.raises(L.SceneFileError, match="invalid filter"):
        L.loads(_scene('"triangle" : { }', '"output" : { "filter" : { "type" : "sharp" } },'))


def test_instances_copy_named_shapes():
    text = _scene('"material" : { "bsdf" : { "type" : "diffuse", "kd" : 0.2 }, '
                  '"triangle" : { "name" : "t", "vertices" : [0,0,0, 1,0,0, 0,0,1] } }, '
                  '"transform" : { "translate" : [0, 5, 0], "shape" : { "instance" : "t" } }, '
                  '"material" : { "bsdf" : { "type" : "diffuse", "kd" : 0.7 }, '
                  '"transform" : { "translate" : [3, 0, 0], "shape" : { "instance" : "t" } } }')
    s = L.loads(text).scene
    assert s.ntri == 3
    # materials first: the original, then the instance under the second material, then the one
    # under the top-level transform (default material)
    assert np.allclose(s.tri_v[0, 0], [0, 0, 0]) and np.allclose(s.tri_v[1, 0], [3, 0, 0])
    assert np.allclose(s.tri_v[2, 0], [0, 5, 0])
    assert s.materials[s.tri_mat[0], 1] == np.float32(0.2) and s.materials[s.tri_mat[1], 1] == np.float32(0.7)
    assert s.tri_mat[2] == 0
    with pytest.raises(L.SceneFileError, match="not found"):
        L.loads(_scene('"shape" : { "instance" : "nope" }'))
    with pytest.raises(L.SceneFileError, match="duplicate"):
        L.loads(_scene('"triangle" : { "name" : "a" }, "plane" : { "name" : "a" }'))


def test_spheres_analytic_or_tessellated():
    body = ('"transform" : { "translate" : [0, 1, 0], "rotate" : [0, 0, 0, 0, 1, 0, 90], '
            '"sphere" : { "position" : [2, 0, 0], "radius" : 0.75 } }')
    a = L.loads(_scene(body)).scene
    # analytic: T(0, 1, 0) R_y(90) T(2, 0, 0) S(1.5): centre R (2, 0, 0) + (0, 1, 0) = (0, 1, -2)
    assert a.ntri == 0 and len(a.spheres) == 1
    assert np.allclose(a.spheres[0, :3], (0, 1, -2), atol=1e-6) and np.isclose(a.spheres[0, 3], 0.75)
    # the record rotates world directions into the object frame: R^T (0, 0, -1) = (1, 0, 0)
    from milton_gb300 import scene as Sc
    q = a.spheres[0, 4:8].astype(np.float64)
    u, w = q[:3], q[3]
    v = np.array([0.0, 0.0, -1.0])
    t = 2 * np.cross(u, v)
    assert np.allclose(v + w * t + np.cross(u, t), (1, 0, 0), atol=1e-6)
    body = ('"transform" : { "translate" : [0, 1, 0], '
            '"sphere" : { "position" : [2, 0, 0], "radius" : 0.75 } }')
    s = L.loads(_scene(body), tessellate=(16, 9)).scene
    assert s.ntri == 16 * 9 * 2 - 2 * 16
    # graph transform after the sphere's own T(position) S(2 radius) on a unit-diameter sphere
    v = s.tri_v.reshape(-1, 3).astype(np.float64)
    r = np.linalg.norm(v - [2, 1, 0], axis=1)
    assert np.allclose(r, 0.75, atol=1e-5)
    # mesh normals keep the inverse-transpose length (normalised per hit after interpolation)
    n = s.tri_n.reshape(-1, 3).astype(np.float64)
    assert np.allclose(n / np.linalg.norm(n, axis=1, keepdims=True), (v - [2, 1, 0]) / 0.75, atol=1e-5)


def test_point_lights_and_omni_emitters():
    text = _scene('"material" : { "emitter" : { "type" : "omni", "power" : [4, 8, 12] }, '
                  '"transform" : { "translate" : [1, 2, 3], "point" : { } } }, '
                  '"material" : { "emitter" : { "type" : "oriented", "power" : 2 }, "point" : { } }, '
                  '"material" : { "emitter" : { "type" : "omni", "power" : 1 }, '
                  '"transform" : { "scale" : [2, 1, 2], "plane" : { } } }, '
                  '"point" : { }')
    s = L.loads(text).scene
    # materials in file order: the two points, then the plane; the bare point is no light
    assert len(s.lights) == 3 and s.ntri == 2
    assert s.light_ext[2, 0] == 0 and s.light_ext[2, 15] == 1  # omni plane: area 4
    assert np.allclose(s.lights[2, 13:16], 1 / (4 * 4 * math.pi))
    p1, p2 = s.lights[0], s.lights[1]
    assert s.light_ext[0, 0] == 3 and s.light_ext[1, 0] == 3
    # an omni point: power / 4 pi; an oriented point: power / pi (its stand-in normal dot is 1)
    assert np.allclose(p1[0:3], (1, 2, 3)) and np.allclose(p1[13:16], np.array([4, 8, 12]) / (4 * math.pi))
    assert np.allclose(p2[0:3], 0) and np.allclose(p2[13:16], 2 / math.pi)
    assert np.all(s.tri_light == 2)


def test_per_channel_ior_is_dispersion():
    s = L.loads(_scene('"material" : { "bsdf" : { "type" : "dielectric", "ior" : [1.4, 1.5, 1.6] }, "triangle" : { } }, '
                       '"material" : { "bsdf" : { "type" : "dielectric", "ior" : 1.5 }, "triangle" : { } }')).scene
    d, g = s.materials[s.tri_mat[0]], s.materials[s.tri_mat[1]]
    assert np.allclose([d[8], d[14], d[15]], [1.4, 1.5, 1.6])
    assert g[8] == np.float32(1.5) and g[14] == 0 and g[15] == 0


def test_emitting_sphere_light_record():
    s = L.loads(_scene('"material" : { "emitter" : { "type" : "oriented", "power" : [3, 6, 9] }, '
                       '"transform" : { "translate" : [1, 2, 3], "sphere" : { "radius" : 0.5 } } }')).scene
    assert len(s.spheres) == 1 and len(s.lights) == 1 and s.sphere_light.tolist() == [0]
    assert s.light_ext[0, 0] == 4 and np.isclose(s.light_ext[0, 5], 0.5) and np.isclose(s.lights[0, 12], math.pi)
    # Le = power / (area pi) with the object-space area pi (Sphere::_getSurfaceArea)
    assert np.allclose(s.lights[0, 13:16], np.array([3, 6, 9]) / math.pi ** 2)
    assert np.allclose(s.lights[0, 0:3], (1, 2, 3))
