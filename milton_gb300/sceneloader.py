"""Milton scene files -> the flattened triangle scene the GPU path tracer renders.

Reads the scene-file dialect of Milton's loader (mlt/src/milton/loaders/MiltonJSONSceneLoader.cpp)
and flattens its scene graph the way SceneGraph::flatten does (mlt/src/milton/loaders/
SceneGraph.cpp:23-181), producing a `Scene` (world-space triangle soup, materials, lights,
camera) plus the renderer / camera / output property maps.  The behaviours that decide which
triangles exist, in which order (the global primitive id is the index in that order) and with
which material are kept as the reference has them:

* Reading (MiltonJSONSceneLoader::parse, :131-161): the file is read line by line and the lines
  are joined without separators, so a ``//`` comment runs to the end of the file and a last
  line without a terminating newline is dropped.  A line of 255 or more characters, on which
  the reference's read loop never terminates, is an error here.
* Grammar (third-party/tinyjson/tinyjson.hpp:460-560): JSON with C comments, trailing commas
  and repeated keys; a number with a '.' or an exponent is a real, otherwise an int.
* Objects are std::multimaps, so every object's keys are visited in byte order of the key,
  repeated keys in file order (JSONVisitor::visit, :66-130).  In a scene all "material" blocks
  come before "mesh", "plane", ..., "transform", "triangle" entries, whatever the file order.
* A material applies to the shapes nested in it; a "material" nested inside a shape object
  applies to nothing (the shape is flattened before its children, SceneGraph.cpp:52-76).
* A transform composes translate * rotate * scale (SceneGraph.h:68-70), repeated keys of one
  kind multiplied in order; rotate = [point, axis, degrees] (Matrix.cpp:83-99).
* A "plane" with "vertices" is two back-face-culled Triangles (v1 v2 v3), (v1 v3 v4)
  (:611-626); a "plane" without them is Milton's unit plane y = 0, |x|, |z| <= 1/2 under its
  transform (Plane.cpp), two-sided.  Meshes (OBJ, PLY) are two-sided MeshTriangles with
  per-vertex normals (computed as Mesh::computeNormals does when the file has none,
  Mesh.cpp:335-377).  Normals go to world space with the inverse transpose
  (Transformable.inl:37-48).
* A nested "shapeSet" is parsed but its shapes never reach the scene: SceneNodeShape::flatten
  (SceneGraph.cpp:99-133) makes it the active set without adding it to its parent.

Emitters: a unit plane becomes a parallelogram light, a Triangle a triangle light with its uv
frame and object-space area, a mesh one mesh light over its triangles (include/mgpu.h,
``light_ext``), a sphere a sphere light sampled as Sphere::getPosition does.  What the GPU path
cannot render is refused with a SceneFileError naming the element: cylinders, cones and blobs,
emitting cubes, oriented backgrounds, bump-mapped emitters, per-channel Phong exponents.  A
per-channel IOR disperses: a path refracts with its colour channel's IOR.
Emitters are oriented (one-sided, power / (area pi)) or omni (both sides, power / (area 4 pi))
on planes, triangles, meshes and spheres, and point lights (a "point" shape with either emitter:
one light sample, no area).  A scene's background is taken: an environment map
(latitude-longitude image: PNG, PPM / PGM or Radiance HDR) or an omni background's constant
radiance, added where a ray leaves the scene.  Image maps are taken: a material's kd / ks / transparency given as a file name and
its bumpMap become textures (PNG, PPM / PGM) with the material's filter, repeatU / repeatV and
bumpIntensity, and every triangle carries the uvs of Shape::_getUV for the shape it came from
(Plane, Triangle, Cube -- from the world position, as the reference does -- and Mesh: the first
vertex's texture coordinate for the whole triangle).  An image that fails to load leaves the
key at 0.7 or the normal unbumped, as the reference's Material does.  Spheres are analytic:
centre, radius and frame of Milton's T(position) S(2 radius) (:596-611) under the graph's
transform, which must then be a similarity; with tessellate=(nu, nv) they become nu x nv UV
spheres with radial normals instead (an approximation, for many or distorted spheres).  Instances of named shapes are copied (their geometry
under the instance's transform chain, with the material active at the instance).  A thin-lens
camera keeps its aperture, f-stop and focal distance; its autofocus is resolved against the
resident scene (pathtracer.resolve_autofocus).  A "cube" becomes the 12 triangles of Milton's
unit cube (Cube.cpp), which is the same surface but 12 primitive ids instead of one.
"""
from __future__ import annotations

import math
import os
import warnings
from dataclasses import dataclass, field

import numpy as np

from . import scene as S
from .imageio import read_image


class SceneFileError(ValueError):
    """A scene file the loader (or the GPU path) cannot take; the message names the element."""


# ------------------------------------------------------------------------------------------
# reading and parsing

def read_scene_text(path: str) -> str:
    """The text the reference parses: lines joined without separators, the last line kept
    only if a newline ends it (MiltonJSONSceneLoader::parse, :139-151)."""
    with open(path, "rb") as f:
        data = f.read().decode("latin-1")
    pieces = data.split("\n")[:-1]
    for k, line in enumerate(pieces):
        if len(line) >= 255:
            raise SceneFileError(f"{path}:{k + 1}: line of {len(line)} characters (at most 254 are read)")
    return "".join(pieces)


class JObj:
    """A JSON object as the reference holds it: a multimap, iterated in key order with repeated
    keys in file order; find() returns the first of a repeated key."""

    def __init__(self, pairs):
        self.pairs = list(pairs)

    def items(self):
        return sorted(self.pairs, key=lambda kv: kv[0].encode("latin-1"))

    def find(self, key):
        for k, v in self.pairs:
            if k == key:
                return v
        return _MISSING

    def __contains__(self, key):
        return self.find(key) is not _MISSING


_MISSING = object()


class _Parser:
    def __init__(self, text: str):
        self.s = text
        self.i = 0

    def error(self, msg):
        raise SceneFileError(f"error parsing file (ill-formed JSON): {msg} at offset {self.i}")

    def skip(self):
        s, n = self.s, len(self.s)
        while self.i < n:
            c = s[self.i]
            if c in " \t\r\n\f\v":
                self.i += 1
            elif s.startswith("/*", self.i):
                j = s.find("*/", self.i + 2)
                if j < 0:
                    self.error("unterminated comment")
                self.i = j + 2
            elif s.startswith("//", self.i):
                j = s.find("\n", self.i)
                self.i = n if j < 0 else j + 1
            else:
                break

    def peek(self):
        self.skip()
        return self.s[self.i] if self.i < len(self.s) else ""

    def expect(self, c):
        if self.peek() != c:
            self.error(f"expected '{c}'")
        self.i += 1

    def value(self):
        c = self.peek()
        if c == "{":
            return self.obj()
        if c == "[":
            return self.arr()
        if c == '"':
            return self.string()
        for word, val in (("true", True), ("false", False), ("null", None)):
            if self.s.startswith(word, self.i):
                self.i += len(word)
                return val
        return self.number()

    def _list(self, close, item):
        out = []
        if self.peek() == close:
            self.i += 1
            return out
        while True:
            out.append(item())
            c = self.peek()
            if c == ",":
                self.i += 1
                if self.peek() == close:  # trailing comma
                    self.i += 1
                    return out
            elif c == close:
                self.i += 1
                return out
            else:
                self.error(f"expected ',' or '{close}'")

    def obj(self):
        self.expect("{")

        def pair():
            k = self.string()
            self.expect(":")
            return (k, self.value())
        return JObj(self._list("}", pair))

    def arr(self):
        self.expect("[")
        return self._list("]", self.value)

    def string(self):
        if self.peek() != '"':
            self.error("expected a string")
        s, i = self.s, self.i + 1
        out = []
        esc = {'"': '"', "\\": "\\", "/": "/", "b": "\b", "f": "\f", "n": "\n", "r": "\r", "t": "\t"}
        while i < len(s) and s[i] != '"':
            if s[i] == "\\":
                if i + 1 >= len(s):
                    break
                e = s[i + 1]
                if e in esc:
                    out.append(esc[e])
                    i += 2
                elif e == "u" and i + 5 < len(s):
                    out.append(chr(int(s[i + 2:i + 6], 16)))
                    i += 6
                else:
                    self.error("bad escape")
            else:
                out.append(s[i])
                i += 1
        if i >= len(s):
            self.error("unterminated string")
        self.i = i + 1
        return "".join(out)

    def number(self):
        s, i = self.s, self.i
        j = i
        if j < len(s) and s[j] in "+-":
            j += 1
        d0 = j
        while j < len(s) and s[j].isdigit():
            j += 1
        intpart = j > d0
        real = False
        if j < len(s) and s[j] == ".":
            k = j + 1
            while k < len(s) and s[k].isdigit():
                k += 1
            if intpart or k > j + 1:
                real, j = True, k
        if (intpart or real) and j < len(s) and s[j] in "eE":
            k = j + 1
            if k < len(s) and s[k] in "+-":
                k += 1
            if k < len(s) and s[k].isdigit():
                while k < len(s) and s[k].isdigit():
                    k += 1
                real, j = True, k
        if not (intpart or real):
            self.error("expected a value")
        self.i = j
        return float(s[i:j]) if real else int(s[i:j])


def parse_text(text: str) -> JObj:
    p = _Parser(text)
    root = p.value()
    if not isinstance(root, JObj):
        raise SceneFileError("error parsing file (ill-formed JSON)")
    return root


# ------------------------------------------------------------------------------------------
# typed properties (MiltonJSONSceneLoader::_parse_properties, :1166-1338)

def _tname(v):
    if v is None:
        return "null"
    if isinstance(v, bool):
        return "bool"
    if isinstance(v, int):
        return "int"
    if isinstance(v, float):
        return "double"
    if isinstance(v, str):
        return "string"
    if isinstance(v, list):
        return "array"
    return "object"


def _real(v, key):
    if isinstance(v, bool) or not isinstance(v, (int, float)):
        raise SceneFileError(f"{key} must be of type 'real_t', found '{_tname(v)}'")
    return float(v)


def _properties(req: dict, obj: JObj, out: dict):
    """Constrained keys converted to their type, then every other key as is (arrays of length
    3 as vectors, other arrays and objects skipped); duplicate constrained keys are errors."""
    def add(key, val):
        if key in out:
            raise SceneFileError(f"duplicate key '{key}' found")
        out[key] = val

    for key in sorted(req):
        exp = req[key]
        v = obj.find(key)
        if v is _MISSING:
            continue
        if v is None:
            if exp != "null":
                raise SceneFileError(f"{key} must be of type '{exp}', found 'null'")
            add(key, None)
        elif isinstance(v, bool):
            if exp != "bool":
                raise SceneFileError(f"{key} must be of type '{exp}', found 'bool'")
            add(key, v)
        elif isinstance(v, (int, float)):
            x = float(v)
            if exp in ("int", "uint"):
                if isinstance(v, float) and math.floor(v) != v:
                    raise SceneFileError("expected integer; found real_t")
                add(key, int(x))
            elif exp == "real_t":
                add(key, x)
            elif exp == "clampedSpectrum":
                if not 0.0 <= x <= 1.0:
                    raise SceneFileError("clampedSpectrum must have value within [0, 1]")
                add(key, (x, x, x))
            elif exp == "spectrum":
                add(key, (x, x, x))
            else:
                raise SceneFileError(f"{key} must be of type '{exp}', found '{_tname(v)}'")
        elif isinstance(v, str):
            if exp not in ("string", "clampedSpectrum"):
                raise SceneFileError(f"{key} must be of type '{exp}', found 'string'")
            add(key, v)
        elif isinstance(v, list):
            if exp in ("point3", "vector3", "color3", "spectrum", "clampedSpectrum"):
                if len(v) != 3:
                    raise SceneFileError(f"'{key}' expects an array of length 3")
                d = tuple(_real(a, key) for a in v)
                if exp == "clampedSpectrum" and any(not 0.0 <= a <= 1.0 for a in d):
                    raise SceneFileError("clampedSpectrum expects values within [0, 1]")
                if exp == "color3" and any(not 0.0 <= a <= 1.0 for a in d):
                    raise SceneFileError(f"'{key}' expects a color3 with components in [0, 1]")
                add(key, d)
            elif exp.startswith("vector"):
                n = int(exp[6:])
                if len(v) != n:
                    raise SceneFileError(f"'{key}' expects an array of length {n}")
                add(key, tuple(_real(a, key) for a in v))
            else:
                raise SceneFileError(f"{key} must be of type '{exp}', found 'array'")
        else:
            raise SceneFileError(f"{key} must be of type '{exp}', found 'object'")
    for key, v in obj.items():
        if key in req or key in out:
            continue
        if isinstance(v, JObj):
            continue
        if isinstance(v, list):
            if len(v) != 3:
                continue
            try:
                v = tuple(float(a) for a in v)
            except (TypeError, ValueError):
                continue
        out[key] = v


# ------------------------------------------------------------------------------------------
# matrices (Matrix.cpp:30-160)

def _trans(v):
    m = np.eye(4)
    m[:3, 3] = v
    return m


def _scale(v):
    return np.diag([v[0], v[1], v[2], 1.0])


def _rot_x(a):
    c, s = math.cos(a), math.sin(a)
    return np.array([[1, 0, 0, 0], [0, c, -s, 0], [0, s, c, 0], [0, 0, 0, 1.0]])


def _rot_y(a):
    c, s = math.cos(a), math.sin(a)
    return np.array([[c, 0, s, 0], [0, 1, 0, 0], [-s, 0, c, 0], [0, 0, 0, 1.0]])


def _rot_z(a):
    c, s = math.cos(a), math.sin(a)
    return np.array([[c, -s, 0, 0], [s, c, 0, 0], [0, 0, 1, 0], [0, 0, 0, 1.0]])


def rotation(point, axis, degrees) -> np.ndarray:
    """Rotation by `degrees` about the axis through `point` (getRotMat, Matrix.cpp:83-99):
    the axis is turned onto +x (about y, then z), the rotation is about x, and undone."""
    v = np.asarray(axis, np.float64)
    v = v / np.linalg.norm(v)
    theta = math.atan2(v[2], v[0])
    phi = -math.atan2(v[1], math.sqrt(v[0] * v[0] + v[2] * v[2]))
    p = np.asarray(point, np.float64)
    return (_trans(p) @ _rot_y(-theta) @ _rot_z(-phi) @ _rot_x(math.radians(degrees)) @ _rot_z(phi)
            @ _rot_y(theta) @ _trans(-p))


# ------------------------------------------------------------------------------------------
# scene graph

@dataclass
class _Node:
    kind: str                      # "set", "material", "transform", "shape"
    payload: object = None
    children: list = field(default_factory=list)


@dataclass
class _Material:
    props: dict = field(default_factory=dict)
    filter: tuple | None = None  # the material's "filter" object (texture lookups); None = triangle, 2


@dataclass
class _Transform:
    translation: np.ndarray = field(default_factory=lambda: np.eye(4))
    rotation: np.ndarray = field(default_factory=lambda: np.eye(4))
    scale: np.ndarray = field(default_factory=lambda: np.eye(4))
    transform: np.ndarray = field(default_factory=lambda: np.eye(4))

    def matrix(self):
        return self.transform @ self.translation @ self.rotation @ self.scale


@dataclass
class _Shape:
    kind: str                      # "triangle", "plane", "mesh", "cube", "set"
    data: dict = field(default_factory=dict)
    local: np.ndarray = field(default_factory=lambda: np.eye(4))


class _Loader:
    SHAPES = ("blob", "cube", "cone", "cylinder", "mesh", "plane", "point", "shape", "sphere", "shapeSet",
              "triangle")

    def __init__(self, base_dir: str, tessellate=None):
        self.tessellate = tessellate
        self.bg = None  # the background element's material
        self.base_dir = base_dir
        self.stack: list[_Node] = []
        self.root: _Node | None = None
        self.renderer = None
        self.camera = None
        self.output = None
        self.output_props: dict = {}
        self.version = None
        self.named: dict = {}

    # -- scene graph stack (SceneGraph::beginNode / endNode)
    def begin(self, node: _Node):
        if self.stack:
            self.stack[-1].children.append(node)
        else:
            self.root = node
        self.stack.append(node)

    def end(self):
        self.stack.pop()

    # -- visitor (JSONVisitor::visit): keys in multimap order
    def visit(self, obj: JObj, fns: dict, strict: bool, required=(), repeats=True):
        seen = {}
        for key, val in obj.items():
            fn = fns.get(key)
            if fn is None:
                if key in fns:
                    continue
                if strict:
                    raise SceneFileError(f"encountered unknown key '{key}'")
                continue
            fn(val)
            seen[key] = seen.get(key, 0) + 1
            if seen[key] > 1 and not repeats:
                raise SceneFileError(f"found multiple definitions of key '{key}'")
        for key in required:
            if key not in seen:
                raise SceneFileError(f"missing required key '{key}'")

    def node_fns(self):
        f = {"material": self.material, "transform": self.transform}
        for s in self.SHAPES:
            f[s] = (lambda kind: (lambda v: self.shape_variant(kind, v)))(s)
        f["shape"] = self.shape
        f["shapeSet"] = self.shape_set
        return f

    # -- top level
    def root_obj(self, obj):
        if not isinstance(obj, JObj):
            raise SceneFileError("root must be of type 'object'")
        self.visit(obj, {"scenefile": self.scenefile}, strict=True, required=("scenefile",), repeats=False)

    def scenefile(self, v):
        if not isinstance(v, JObj):
            raise SceneFileError(f"scenefile must be of type 'object', found '{_tname(v)}'")
        self.visit(v, {"renderer": self.parse_renderer, "camera": self.parse_camera, "output": self.parse_output,
                       "scene": self.scene, "version": self.parse_version}, strict=True, required=("scene",),
                   repeats=False)

    def parse_version(self, v):
        self.version = _real(v, "version")

    def parse_renderer(self, v):
        if not isinstance(v, JObj):
            raise SceneFileError(f"renderer must be of type 'object', found '{_tname(v)}'")
        t = v.find("type")
        if t is _MISSING:
            raise SceneFileError("unable to infer renderer type")
        if self.renderer is not None:
            raise SceneFileError("multiple renderer definitions")
        if not isinstance(t, str):
            raise SceneFileError(f"renderer.type must be of type 'string', found '{_tname(t)}'")
        req = {"noDirectSamples": "uint", "noRenderThreads": "uint", "noSuperSamples": "uint",
               "directSampleGenerator": "string", "generator": "string"}
        if t in ("rayCaster",):
            req["ambient"] = "spectrum"
        elif t in ("rayTracer",):
            req.update(maxDepth="uint", ambient="spectrum")
        elif t in ("mlt", "MLT"):
            req.update(maxDepth="uint", maxConsequtiveRejections="uint", mltBidirPathMutationProb="real_t",
                       mltLensSubpathMutationProb="real_t", mltPerturbationPathMutationProb="real_t")
        elif t not in ("preview", "OpenGL", "pathTracer", "bidirectionalPathTracer", "bidirPathTracer", "dynamic"):
            raise SceneFileError("invalid renderer type")
        props = {}
        _properties(req, v, props)
        self.renderer = props

    def parse_output(self, v):
        if not isinstance(v, JObj):
            raise SceneFileError(f"output must be of type 'object', found '{_tname(v)}'")
        if self.output is not None:
            raise SceneFileError("multiple output definitions")
        req = {"width": "uint", "height": "uint", "size": "vector2", "dimensions": "vector2"}
        t = v.find("type")
        if t is not _MISSING or "filter" in v:
            kind = "reconstruction" if t is _MISSING else t
            if not isinstance(kind, str):
                raise SceneFileError("output.type must be of type 'string'")
            if kind not in ("naive", "default", "reconstruction", "dynamic"):
                raise SceneFileError("invalid output type")
            req["tonemap"] = "string"
            self.output = {"type": kind}
            # the reconstruction filter: an explicit "filter" object, or DefaultRenderOutput's
            # Lanczos-sinc of support 2 (DefaultRenderOutput.cpp:20); "naive" has none
            if kind != "naive":
                fv = v.find("filter")
                if fv is not _MISSING:
                    self.output["filter"] = parse_filter(fv)
                elif kind == "default":
                    self.output["filter"] = ("lanczosSinc", 2.0, {"tau": 3.0})
        props = {}
        _properties(req, v, props)
        self.output_props.update(props)
        if self.output is None:
            self.output = {}

    def parse_camera(self, v):
        if not isinstance(v, JObj):
            raise SceneFileError(f"camera must be of type 'object', found '{_tname(v)}'")
        t = v.find("type")
        if t is _MISSING:
            raise SceneFileError("unable to infer camera type")
        if not isinstance(t, str):
            raise SceneFileError(f"camera.type must be of type 'string', found '{_tname(t)}'")
        if self.camera is not None:
            raise SceneFileError("multiple camera definitions")
        if t not in ("pinhole", "thinlens", "dynamic"):
            raise SceneFileError("invalid camera type")
        req = {"eye": "point3", "look": "vector3", "focus": "point3", "up": "vector3", "heightAngle": "real_t",
               "aspectRatio": "real_t", "near": "real_t", "far": "real_t"}
        if t == "thinlens":
            req.update(aperture="real_t", fstop="real_t", focalDistance="real_t", focalPoint="vector2")
        props = {}
        _properties(req, v, props)
        self.camera = props

    # -- scene graph builders
    def scene(self, v):
        if not isinstance(v, JObj):
            raise SceneFileError(f"scene must be of type 'object', found '{_tname(v)}'")
        self.shape_set(v, root=True)

    def shape_set(self, v, root=False):
        if not isinstance(v, JObj):
            raise SceneFileError(f"shapeSet must be of type 'object', found '{_tname(v)}'")
        fns = self.node_fns()
        fns["background"] = self.background if root else None
        fns["spatialAccel"] = None
        self.begin(_Node("shape", _Shape("set", {"root": root})))
        _properties({}, v, {})
        self.visit(v, fns, strict=False)
        if not root:
            self.end()

    def background(self, v):
        """MiltonJSONSceneLoader::_parse_background (:1693-1720): at most one, holding exactly one
        emitter, which may be an environment map (latitude-longitude image, `path`)."""
        if not isinstance(v, JObj):
            raise SceneFileError(f"background must be of type 'object', found '{_tname(v)}'")
        if self.bg is not None:
            raise SceneFileError("scene may contain at most one background element")
        if len(v.pairs) == 0:
            self.bg = _Material()
            return
        e = v.find("emitter")
        if len(v.pairs) > 1 or e is _MISSING:
            raise SceneFileError("background element must have exactly one child emitter element")
        mat = _Material()
        if not isinstance(e, JObj):
            raise SceneFileError(f"emitter must be of type 'object', found '{_tname(e)}'")
        t = e.find("type")
        if t is _MISSING:
            raise SceneFileError("unable to infer emitter type")
        if not isinstance(t, str):
            raise SceneFileError("emitter.type must be of type 'string'")
        req = {}
        if t == "null":
            mat.props["emitter"] = "null"
        elif t in ("omni", "oriented", "environment"):
            mat.props["emitter"] = t
            req.update(power="spectrum", glDiffuseColor="color3", glSpecularColor="color3", glAttenuation="vector3")
            if t == "environment":
                req.update(coords="string", path="string")
        else:
            raise SceneFileError("invalid emitter type")
        _properties(req, e, mat.props)
        if t == "environment" and "path" not in mat.props:
            raise SceneFileError("environment map must contain a 'path' child element specifying an absolute or "
                                 "relative path to an environment texture")
        if t == "oriented":
            raise SceneFileError("an oriented background emitter is not supported by the GPU path (it has no "
                                 "surface normal to orient by)")
        self.bg = mat

    def material(self, v):
        mat = _Material()
        if v is None:
            self.begin(_Node("material", mat))
            self.end()
            return
        if not isinstance(v, JObj):
            raise SceneFileError(f"material must be of type 'object', found '{_tname(v)}'")
        fns = self.node_fns()
        fns.update(bsdf=lambda b: self.bsdf(mat, b), emitter=lambda e: self.emitter(mat, e),
                   medium=lambda m: self.medium(mat, m), filter=lambda f: setattr(mat, "filter", parse_filter(f)))
        _properties({"bumpMap": "string", "bumpIntensity": "real_t", "repeatU": "real_t", "repeatV": "real_t"},
                    v, mat.props)
        self.begin(_Node("material", mat))
        self.visit(v, fns, strict=False)
        self.end()

    def bsdf(self, mat: _Material, v):
        if not isinstance(v, JObj):
            raise SceneFileError(f"bsdf must be of type 'object', found '{_tname(v)}'")
        t = v.find("type")
        if t is _MISSING:
            raise SceneFileError("unable to infer bsdf type")
        if not isinstance(t, str):
            raise SceneFileError("bsdf.type must be of type 'string'")
        if "bsdf" in mat.props:
            raise SceneFileError("multiple bsdf definitions")
        req = {}
        if t == "diffuse":
            mat.props["bsdf"] = "diffuse"
            req["kd"] = "clampedSpectrum"
        elif t in ("specular", "transmissive"):
            mat.props["bsdf"] = "dielectric"
            req["ks"] = "clampedSpectrum"
        elif t == "dielectric":
            mat.props["bsdf"] = "dielectric"
            req.update(ks="clampedSpectrum", transparency="clampedSpectrum")
        elif t == "absorbent":
            mat.props["bsdf"] = "absorbent"
        elif t in ("modifiedPhong", "phong"):
            mat.props["bsdf"] = t
            req.update(kd="clampedSpectrum", ks="clampedSpectrum", n="spectrum")
        else:
            raise SceneFileError("invalid bsdf type")
        _properties(req, v, mat.props)
        if t == "specular":
            mat.props["transparency"] = 0.0
        elif t == "transmissive":
            mat.props["transparency"] = 1.0

    def emitter(self, mat: _Material, v):
        if not isinstance(v, JObj):
            raise SceneFileError(f"emitter must be of type 'object', found '{_tname(v)}'")
        t = v.find("type")
        if t is _MISSING:
            raise SceneFileError("unable to infer emitter type")
        if not isinstance(t, str):
            raise SceneFileError("emitter.type must be of type 'string'")
        if "emitter" in mat.props:
            raise SceneFileError("multiple emitter definitions")
        req = {}
        if t == "null":
            mat.props["emitter"] = "null"
        elif t in ("omni", "oriented"):
            mat.props["emitter"] = t
            req.update(power="spectrum", glDiffuseColor="color3", glSpecularColor="color3", glAttenuation="vector3")
        elif t == "environment":
            raise SceneFileError("environment map emitters may only be placed in the scene's "
                                 "\"background.emitter\" element")
        else:
            raise SceneFileError("invalid emitter type")
        _properties(req, v, mat.props)

    def medium(self, mat: _Material, v):
        if not isinstance(v, JObj):
            raise SceneFileError(f"medium must be of type 'object', found '{_tname(v)}'")
        t = v.find("type")
        t = "homogenous" if t is _MISSING else t
        if "medium" in mat.props:
            raise SceneFileError("multiple medium definitions")
        if t != "homogenous":
            raise SceneFileError("invalid medium type")
        mat.props["medium"] = t
        _properties({"ior": "spectrum"}, v, mat.props)

    def transform(self, v):
        if not isinstance(v, JObj):
            raise SceneFileError(f"transform must be of type 'object', found '{_tname(v)}'")
        tr = _Transform()

        def arr(val, n, msg):
            if not isinstance(val, list) or len(val) != n:
                raise SceneFileError(msg)
            return [_real(a, msg) for a in val]

        def arbitrary(val):
            tr.transform = tr.transform @ np.array(arr(val, 16, "arbitraryTransform expects 16 doubles in "
                                                             "row-major order")).reshape(4, 4)

        def translate(val):
            tr.translation = tr.translation @ _trans(arr(val, 3, "translate transformation expects 3 doubles"))

        def rotate(val):
            d = arr(val, 7, "rotate expects 7 doubles: [ px, py, pz, vx, vy, vz, degrees ]")
            tr.rotation = tr.rotation @ rotation(d[0:3], d[3:6], d[6])

        def scale(val):
            tr.scale = tr.scale @ _scale(arr(val, 3, "scale expects 3 doubles"))

        fns = self.node_fns()
        fns.update(arbitraryTransform=arbitrary, translate=translate, rotate=rotate, scale=scale)
        self.begin(_Node("transform", tr))
        self.visit(v, fns, strict=True)
        self.end()

    def shape_variant(self, kind, v):
        if not isinstance(v, JObj):
            raise SceneFileError(f"{kind} must be of type 'object', found '{_tname(v)}'")
        self.shape(JObj(v.pairs + [("type", kind)]))

    def shape(self, v):
        if not isinstance(v, JObj):
            raise SceneFileError(f"shape must be of type 'object', found '{_tname(v)}'")
        inst = v.find("instance")
        if inst is not _MISSING:
            # an instance of a named shape (SceneNodeInstance, SceneGraph.cpp:135-181): resolved
            # when the graph is flattened, so the name may be defined anywhere in the file
            if not isinstance(inst, str):
                raise SceneFileError(f"shape.instance must be of type 'string', found '{_tname(inst)}'")
            props = {}
            _properties({"name": "string"}, v, props)
            node = _Node("instance", inst)
            self.name_node(props, node)
            self.begin(node)
            self.visit(v, {"material": self.material}, strict=False)
            self.end()
            return
        t = v.find("type")
        if t is _MISSING:
            raise SceneFileError("unable to infer shape type")
        if not isinstance(t, str):
            raise SceneFileError(f"shape.type must be of type 'string', found '{_tname(t)}'")
        req = {"name": "string"}
        if t == "plane":
            req["vertices"] = "vector12"
        elif t == "mesh":
            req.update(path="string", normalize="bool")
        elif t == "triangle":
            req.update(vertices="vector9", normals="vector9", normal="vector3", uvs="vector6")
        elif t == "shapeSet":
            return self.shape_set(v)
        elif t in ("cube", "point"):
            pass
        elif t == "sphere":
            req.update(position="point3", radius="real_t")
        elif t in ("cylinder", "cone", "blob", "dynamic"):
            raise SceneFileError(f"shape '{t}' is not supported by the GPU path (planes, cubes, triangles, "
                                 "meshes, spheres and points are)")
        else:
            raise SceneFileError("invalid shape type")
        props = {}
        _properties(req, v, props)
        if t == "plane" and "vertices" in props:
            d = np.array(props["vertices"], np.float64).reshape(4, 3)
            self.begin(_Node("shape", _Shape("triangle", {"v": d[[0, 1, 2]], "uvs": (0, 0, 0, 1, 1, 1)})))
            self.end()
            node = _Node("shape", _Shape("triangle", {"v": d[[0, 2, 3]], "uvs": (0, 0, 1, 1, 1, 0)}))
        elif t == "plane":
            node = _Node("shape", _Shape("plane"))
        elif t == "triangle":
            verts = np.array(props.get("vertices", (0, 0, 0, 0, 0, 0.5, 0.5, 0, 0)), np.float64).reshape(3, 3)
            node = _Node("shape", _Shape("triangle", {"v": verts, "uvs": props.get("uvs", (0, 0, 1, 0, 0, 1))}))
        elif t == "cube":
            node = _Node("shape", _Shape("cube"))
        elif t == "point":
            node = _Node("shape", _Shape("point"))
        elif t == "sphere":
            # Milton's Sphere: a unit-diameter sphere under T(position) S(2 radius) (:575-589),
            # here an nu x nv UV sphere with radial normals -- an approximation of the analytic
            # surface, used only when the caller asks for it
            local = np.eye(4)
            pos = props.get("position")
            if pos is not None:
                local = local @ _trans(pos)
            if "radius" in props:
                local = local @ _scale([2.0 * props["radius"]] * 3)
            if not self.tessellate:
                node = _Node("shape", _Shape("sphere", {}, local))
                self.name_node(props, node)
                self.begin(node)
                self.visit(v, {"material": self.material, "spatialAccel": None}, strict=False)
                self.end()
                return
            tris, nrm, uv = _unit_sphere(*self.tessellate)
            node = _Node("shape", _Shape("mesh", {"v": tris.reshape(-1, 3).astype(np.float64),
                                                  "f": np.arange(tris.shape[0] * 3).reshape(-1, 3),
                                                  "n": nrm.reshape(-1, 3).astype(np.float64),
                                                  "nf": np.arange(tris.shape[0] * 3).reshape(-1, 3),
                                                  "uv": uv, "path": "sphere"}, local))
        else:  # mesh
            if "path" not in props:
                raise SceneFileError("missing required key 'path' in 'mesh' (path to mesh data file)")
            path = props["path"]
            if not os.path.isabs(path) and not os.path.exists(path):
                path = os.path.join(self.base_dir, path)  # the reference opens it from the cwd
            verts, faces, normals, nfaces, face_uv = load_mesh(path, with_uv=True)
            if props.get("normalize"):
                lo, hi = verts.min(0), verts.max(0)
                center = (lo + hi) * 0.5
                diag = hi - lo
                diag = diag + (diag == 0)
                verts = (verts - center) / diag
            node = _Node("shape", _Shape("mesh", {"v": verts, "f": faces, "n": normals, "nf": nfaces,
                                                  "uv": np.repeat(face_uv[:, None, :], 3, axis=1),
                                                  "path": props["path"]}))
        self.name_node(props, node)
        self.begin(node)
        self.visit(v, {"material": self.material, "spatialAccel": None}, strict=False)
        self.end()

    def name_node(self, props: dict, node: "_Node"):
        """Records a 'name'd node for instancing (MiltonJSONSceneLoader.cpp:634-648).  For a plane
        given by vertices that is its second triangle node, as in the reference."""
        if "name" in props:
            if props["name"] in self.named:
                raise SceneFileError(f"error: duplicate definitions for named node '{props['name']}'")
            self.named[props["name"]] = node


# ------------------------------------------------------------------------------------------
# meshes (MeshLoader.cpp:21-42; OBJ: MeshLoaderOBJ.cpp with obj-parser-0.1 triangulating
# faces as fans; PLY: MeshLoaderPLY.cpp reads float32 vertex x/y/z and fan-triangulates
# face vertex_indices lists)

def parse_filter(v) -> tuple:
    """MiltonJSONSceneLoader::_parse_filter (:1340-1382) -> (kind, support, params) with
    KernelFilter::create's defaults (support 2, sigma 1, B = C = 1/3, tau 3)."""
    if isinstance(v, str):
        v = JObj([("type", v)])
    if not isinstance(v, JObj):
        raise SceneFileError(f"filter must be of type 'object', found '{_tname(v)}'")
    t = v.find("type")
    if t is _MISSING:
        raise SceneFileError("unable to infer filter type")
    req = {"support": "uint"}
    if t == "gaussian":
        req["sigma"] = "real_t"
    elif t == "mitchell":
        req.update(B="real_t", C="real_t")
    elif t == "lanczosSinc":
        req["tau"] = "real_t"
    elif t not in ("box", "triangle"):
        raise SceneFileError("invalid filter type")
    props = {}
    _properties(req, v, props)
    params = {}
    if t == "gaussian":
        params["sigma"] = float(props.get("sigma", 1.0))
    elif t == "mitchell":
        params.update(B=float(props.get("B", 1.0 / 3.0)), C=float(props.get("C", 1.0 / 3.0)))
    elif t == "lanczosSinc":
        params["tau"] = float(props.get("tau", 3.0))
    return (t, float(props.get("support", 2)), params)


def load_mesh(path: str, with_uv: bool = False):
    """(vertices (V, 3) float64, triangles (T, 3) int, normals (N, 3) or None, normal indices
    (T, 3) or None), and with_uv: each triangle's uv (T, 2) -- Mesh::_getUV takes the uv of the
    triangle's first texture index for the whole triangle (Mesh.cpp:408-416), index 0 for faces
    without texture indices (MeshLoaderOBJ.cpp:117-162), (0, 0) for meshes without uvs."""
    suffix = path[path.rfind(".") + 1:]
    if suffix in ("obj", "OBJ"):
        r = _load_obj(path)
    elif suffix in ("ply", "PLY"):
        r = _load_ply(path) + (np.zeros((0, 2)), None)
    else:
        raise SceneFileError(f"mesh '{path}' failed to load (unable to infer mesh type '{suffix}')")
    if not with_uv:
        return r[:4]
    verts, faces, normals, nfaces, uvs, t_first = r
    if len(uvs) == 0:
        face_uv = np.zeros((len(faces), 2))
    else:
        if t_first.min() < 0 or t_first.max() >= len(uvs):
            raise SceneFileError(f"mesh '{path}': texture index out of range")
        face_uv = uvs[t_first]
    return verts, faces, normals, nfaces, face_uv


def _load_obj(path):
    if not os.path.exists(path):
        raise SceneFileError(f"mesh '{path}' failed to load")
    v, vn, vt, tris, ntris, tfirst = [], [], [], [], [], []
    with open(path, "r", encoding="latin-1") as f:
        for ln, line in enumerate(f, 1):
            parts = line.split()
            if not parts or parts[0].startswith("#"):
                continue
            tag = parts[0]
            if tag == "v":
                v.append([float(x) for x in parts[1:4]])
            elif tag == "vn":
                vn.append([float(x) for x in parts[1:4]])
            elif tag == "vt":
                vt.append([float(x) for x in parts[1:3]])
            elif tag == "f":
                idx = []
                for p in parts[1:]:
                    fs = p.split("/")
                    if len(fs) == 2 or (len(fs) == 3 and fs[2] == ""):
                        raise SceneFileError(f"{path}:{ln}: faces with texture but no normal indices are not "
                                             "supported by the reference's OBJ loader")
                    vi = int(fs[0])
                    ni = int(fs[2]) if len(fs) == 3 else None
                    ti = int(fs[1]) if len(fs) == 3 and fs[1] != "" else None
                    vi = vi - 1 if vi > 0 else len(v) + vi
                    if ni is not None:
                        ni = ni - 1 if ni > 0 else len(vn) + ni
                    if ti is not None:
                        ti = ti - 1 if ti > 0 else len(vt) + ti
                    idx.append((vi, ni, ti))
                if len(idx) < 3:
                    raise SceneFileError(f"{path}:{ln}: face with fewer than 3 vertices")
                for k in range(1, len(idx) - 1):
                    a, b, c = idx[0], idx[k], idx[k + 1]
                    tris.append((a[0], b[0], c[0]))
                    ntris.append((a[1], b[1], c[1]))
                    tfirst.append(a[2] if a[2] is not None else 0)
    verts = np.array(v, np.float64).reshape(-1, 3)
    faces = np.array(tris, np.int64).reshape(-1, 3)
    if len(faces) == 0 or len(verts) == 0:
        raise SceneFileError(f"mesh '{path}' failed to load (no triangles)")
    if faces.min() < 0 or faces.max() >= len(verts):
        raise SceneFileError(f"mesh '{path}': vertex index out of range")
    if vn and all(t[0] is not None for t in ntris):
        nf = np.array(ntris, np.int64)
        if nf.min() < 0 or nf.max() >= len(vn):
            raise SceneFileError(f"mesh '{path}': normal index out of range")
        return verts, faces, np.array(vn, np.float64), nf, np.array(vt, np.float64).reshape(-1, 2), np.array(tfirst)
    return verts, faces, None, None, np.array(vt, np.float64).reshape(-1, 2), np.array(tfirst)


_PLY_TYPES = {"char": "i1", "int8": "i1", "uchar": "u1", "uint8": "u1", "short": "i2", "int16": "i2",
              "ushort": "u2", "uint16": "u2", "int": "i4", "int32": "i4", "uint": "u4", "uint32": "u4",
              "float": "f4", "float32": "f4", "double": "f8", "float64": "f8"}


def _load_ply(path):
    if not os.path.exists(path):
        raise SceneFileError(f"mesh '{path}' failed to load")
    with open(path, "rb") as f:
        raw = f.read()
    end = raw.find(b"end_header")
    if not raw.startswith(b"ply") or end < 0:
        raise SceneFileError(f"mesh '{path}' failed to load (not a PLY file)")
    nl = raw.find(b"\n", end)
    header = raw[:end].decode("latin-1").splitlines()
    body = raw[nl + 1:]
    fmt = None
    elements = []
    for line in header:
        p = line.split()
        if not p:
            continue
        if p[0] == "format":
            fmt = p[1]
        elif p[0] == "element":
            elements.append([p[1], int(p[2]), []])
        elif p[0] == "property" and elements:
            if p[1] == "list":
                if elements[-1][0] == "face" and p[4] == "vertex_indices" and (
                        _PLY_TYPES[p[2]] != "u1" or _PLY_TYPES[p[3]] != "i4"):
                    raise SceneFileError(f"mesh '{path}': face vertex_indices must be 'list uchar int' "
                                         "(the reference binds no other list type)")
                elements[-1][2].append(("list", p[4], _PLY_TYPES[p[2]], _PLY_TYPES[p[3]]))
            else:
                elements[-1][2].append(("scalar", p[2], _PLY_TYPES[p[1]]))
    if fmt not in ("ascii", "binary_little_endian", "binary_big_endian"):
        raise SceneFileError(f"mesh '{path}': unknown PLY format {fmt}")
    verts, faces = [], []
    if fmt == "ascii":
        toks = body.decode("latin-1").split()
        pos = 0
        for name, count, props in elements:
            for _ in range(count):
                rec = {}
                for pr in props:
                    if pr[0] == "list":
                        n = int(toks[pos])
                        pos += 1
                        rec[pr[1]] = [int(float(t)) for t in toks[pos:pos + n]]
                        pos += n
                    else:
                        rec[pr[1]] = (pr[2], float(toks[pos]))
                        pos += 1
                _ply_record(name, rec, verts, faces)
    else:
        end_ch = "<" if fmt == "binary_little_endian" else ">"
        pos = 0
        for name, count, props in elements:
            for _ in range(count):
                rec = {}
                for pr in props:
                    if pr[0] == "list":
                        ct = np.dtype(end_ch + pr[2])
                        n = int(np.frombuffer(body, ct, 1, pos)[0])
                        pos += ct.itemsize
                        it = np.dtype(end_ch + pr[3])
                        rec[pr[1]] = [int(x) for x in np.frombuffer(body, it, n, pos)]
                        pos += it.itemsize * n
                    else:
                        dt = np.dtype(end_ch + pr[2])
                        rec[pr[1]] = (pr[2], float(np.frombuffer(body, dt, 1, pos)[0]))
                        pos += dt.itemsize
                _ply_record(name, rec, verts, faces)
    vv = np.array(verts, np.float64).reshape(-1, 3)
    ff = np.array(faces, np.int64).reshape(-1, 3)
    if len(ff) == 0 or len(vv) == 0:
        raise SceneFileError(f"mesh '{path}' failed to load (no triangles)")
    if ff.min() < 0 or ff.max() >= len(vv):
        raise SceneFileError(f"mesh '{path}': vertex index out of range")
    return vv, ff, None, None


def _ply_record(name, rec, verts, faces):
    if name == "vertex":
        # the reference binds float32 x, y, z only (MeshLoaderPLY.cpp scalar callbacks)
        xyz = []
        for k in ("x", "y", "z"):
            t = rec.get(k)
            if t is None or t[0] != "f4":
                raise SceneFileError(f"PLY vertex property '{k}' must be a float32")
            xyz.append(float(np.float32(t[1])))
        verts.append(xyz)
    elif name == "face" and "vertex_indices" in rec:
        idx = rec["vertex_indices"]
        for k in range(2, len(idx)):
            faces.append((idx[0], idx[k - 1], idx[k]))


def mesh_vertex_normals(verts: np.ndarray, faces: np.ndarray) -> np.ndarray:
    """Mesh::computeNormals: per vertex, the normalised sum of the unit normals of its faces."""
    a, b, c = verts[faces[:, 0]], verts[faces[:, 1]], verts[faces[:, 2]]
    fn = np.cross(b - a, c - a)
    ln = np.linalg.norm(fn, axis=1, keepdims=True)
    fn = np.where(ln > 0, fn / np.where(ln > 0, ln, 1.0), 0.0)
    acc = np.zeros_like(verts)
    for k in range(3):
        np.add.at(acc, faces[:, k], fn)
    ln = np.linalg.norm(acc, axis=1, keepdims=True)
    return np.where(ln > 0, acc / np.where(ln > 0, ln, 1.0), acc)


# ------------------------------------------------------------------------------------------
# flattening (SceneGraph::flatten)

_CUBE_FACES = [  # (normal axis, sign): two triangles per face of [-.5, .5]^3
    ((1, 0, 0), [(0.5, -0.5, -0.5), (0.5, 0.5, -0.5), (0.5, 0.5, 0.5), (0.5, -0.5, 0.5)]),
    ((-1, 0, 0), [(-0.5, -0.5, -0.5), (-0.5, -0.5, 0.5), (-0.5, 0.5, 0.5), (-0.5, 0.5, -0.5)]),
    ((0, 1, 0), [(-0.5, 0.5, -0.5), (-0.5, 0.5, 0.5), (0.5, 0.5, 0.5), (0.5, 0.5, -0.5)]),
    ((0, -1, 0), [(-0.5, -0.5, -0.5), (0.5, -0.5, -0.5), (0.5, -0.5, 0.5), (-0.5, -0.5, 0.5)]),
    ((0, 0, 1), [(-0.5, -0.5, 0.5), (0.5, -0.5, 0.5), (0.5, 0.5, 0.5), (-0.5, 0.5, 0.5)]),
    ((0, 0, -1), [(-0.5, -0.5, -0.5), (-0.5, 0.5, -0.5), (0.5, 0.5, -0.5), (0.5, -0.5, -0.5)]),
]


def _cube_uv(q_world, n_obj):
    """Cube::_getUV (Cube.cpp:84-105) at the corners of one face: it reads the hit position in
    world space (not object space) and the face's normalCase (axis, 4 + axis on the negative
    side, Cube.cpp:27-48); affine in the position, so corner values interpolate exactly."""
    axis = int(np.flatnonzero(np.asarray(n_obj))[0])
    case = axis if n_obj[axis] > 0 else 4 + axis
    side = case & 3
    out = np.zeros((len(q_world), 2))
    for k, P in enumerate(q_world):
        v = P[side + 1 - 3 * (side == 2)] + 0.5
        u = P[side + 2 - 3 * (side >= 1)] + 0.5
        if side == 2:
            u, v = 1 - v, u
        if case & 4:
            v = 1 - v
        if not (case & 5):
            u, v = 1 - u, 1 - v
        out[k] = (u, v)
    return out


def _xf_points(m, p):
    p = np.asarray(p, np.float64).reshape(-1, 3)
    return p @ m[:3, :3].T + m[:3, 3]


def _xf_normals(m, n):
    """Inverse transpose of the upper 3x3 (Transformable::_transformVector3ObjToWorld), normalised."""
    inv = np.linalg.inv(m)
    w = np.asarray(n, np.float64).reshape(-1, 3) @ inv[:3, :3]
    ln = np.linalg.norm(w, axis=1, keepdims=True)
    return w / np.where(ln > 0, ln, 1.0)


class _Flattener:
    def __init__(self, named=None, base_dir: str = "."):
        self.named = named or {}
        self.base_dir = base_dir
        self.depth = 0
        self.b = S.SceneBuilder()
        self.mat_index = {}   # id(_Material) -> material record index
        self.tex_index = {}   # (file, kind, filter, repeat, intensity) -> texture slot
        self.images = {}      # file -> (H, W, 3) float32 or None (ResourceManager's image cache)
        self.default = _Material()
        self.active = self.default
        self.in_root = True   # shapes go to the root ShapeSet (nested sets are never attached)

    def material_record(self, mat: _Material) -> int:
        key = id(mat)
        if key not in self.mat_index:
            slots = self.texture_slots(mat)
            rec = material_record(mat.props)
            rec[10:14] = slots
            self.mat_index[key] = self.b.material(rec)
        return self.mat_index[key]

    def image(self, name: str):
        """ResourceManager::getImage (ResourceManager.h:48-66): the image or None when it fails
        to load (the reference logs the failure and renders on)."""
        if name not in self.images:
            path = name
            if not os.path.isabs(path) and not os.path.exists(path):
                path = os.path.join(self.base_dir, path)  # the reference opens it from the cwd
            try:
                self.images[name] = read_image(path)
            except (OSError, ValueError) as e:
                warnings.warn(f"failed to load image '{name}': {e}")
                self.images[name] = None
        return self.images[name]

    def texture_slots(self, mat: _Material) -> list[float]:
        """Texture slots [kd, ks, transparency, bump map] of a material record.  A textured key
        whose image fails to load is the constant 0.7 (Material::getSpectralSampleSet,
        Material.cpp:281), a bump map that fails leaves the normal alone (:189-193)."""
        props = mat.props
        flt = mat.filter or ("triangle", 2.0, {})
        ru, rv = float(props.get("repeatU", 1.0)), float(props.get("repeatV", 1.0))
        intensity = float(props.get("bumpIntensity", 5.0))
        slots = [0.0, 0.0, 0.0, 0.0]
        keys = {"diffuse": ("kd",), "modifiedPhong": ("kd", "ks"), "phong": ("kd", "ks"),
                "dielectric": ("ks", "transparency")}.get(props.get("bsdf", "diffuse"), ())
        for k, key in enumerate(("kd", "ks", "transparency")):
            name = props.get(key)
            if key in keys and isinstance(name, str):
                img = self.image(name)
                if img is None:
                    props[key] = 0.7
                    continue
                slots[k] = self.texture(name, img, S.TEX_COLOR, flt, ru, rv, intensity)
        bump = props.get("bumpMap")
        if isinstance(bump, str) and bump:
            img = self.image(bump)
            if img is not None:
                slots[3] = self.texture(bump, img, S.TEX_BUMP, flt, ru, rv, intensity)
        return slots

    def background(self, mat: "_Material | None"):
        """The scene's background (Scene::setBackground, MiltonJSONSceneLoader.cpp:325-327): an
        environment map is a colour map with the background material's default filter and
        repeat (EnvironmentMap.cpp:21-56); an omni background is power / 4 pi
        (OmniEmitter.cpp; the null surface point has no area)."""
        if mat is None or mat.props.get("emitter", "null") == "null":
            return
        if mat.props["emitter"] == "environment":
            name = mat.props["path"]
            img = self.image(name)
            if img is None:
                # the reference asserts and then dereferences the missing image
                raise SceneFileError(f"failed to load environment map image '{name}'")
            self.b.background(tex=self.texture(name, img, S.TEX_COLOR, ("triangle", 2.0, {}), 1.0, 1.0, 5.0))
        else:  # omni
            power = np.broadcast_to(np.asarray(mat.props.get("power", 0.0), np.float64), 3)
            self.b.background(le=power / (4.0 * math.pi))

    def texture(self, name, img, kind, flt, ru, rv, intensity) -> int:
        key = (name, kind, repr(flt) if kind == S.TEX_COLOR else "", ru, rv, intensity)
        if key not in self.tex_index:
            self.tex_index[key] = self.b.texture(S.Texture(img, kind=kind, filter=flt, repeat_u=ru, repeat_v=rv,
                                                           bump_intensity=intensity))
        return self.tex_index[key]

    def run(self, root: _Node):
        self.material_record(self.default)
        self.flatten(root, np.eye(4))

    def flatten(self, node: _Node, trans: np.ndarray):
        if node.kind == "transform":
            trans = trans @ node.payload.matrix()
        elif node.kind == "material":
            self.active = node.payload
        elif node.kind == "shape":
            self.shape(node.payload, trans)
        elif node.kind == "instance":
            # the named node flattened again here: an InstancedShape undoes the instancee's own
            # transform and applies the instance's (InstancedShape.cpp:16-40), so the copy is the
            # named shape's object-space geometry under this node's transform chain
            target = self.named.get(node.payload)
            if target is None or target.kind != "shape":
                raise SceneFileError(f"error: instanced node '{node.payload}' not found")
            if self.depth > 64:
                raise SceneFileError("instances nested more than 64 deep (a cycle?)")
            active, in_root = self.active, self.in_root
            self.depth += 1
            self.flatten(target, trans)
            self.depth -= 1
            self.active, self.in_root = active, in_root
        active, in_root = self.active, self.in_root
        for child in node.children:
            self.flatten(child, trans)
            self.active, self.in_root = active, in_root

    def shape(self, sh: _Shape, trans: np.ndarray):
        if sh.kind == "set":
            # the root set receives every shape; a nested set becomes the active set without
            # being added to the scene, and so do the shapes below it
            self.in_root = bool(sh.data.get("root"))
            return
        if not self.in_root:
            return
        props = self.active.props
        emitter = props.get("emitter", "null")
        if emitter not in ("null", "oriented", "omni"):
            raise SceneFileError(f"'{emitter}' emitters are not supported by the GPU path (oriented and omni "
                                 "emitters are)")
        # OrientedEmitter: Le = power / (area pi) on the normal's side; OmniEmitter: power / (area
        # 4 pi) in every direction (Emitter.cpp:34-50, OrientedEmitter.cpp:17-23, OmniEmitter.cpp)
        per_sr = math.pi if emitter == "oriented" else 4.0 * math.pi
        omni_ext = np.zeros(16, np.float32)
        omni_ext[15] = 1.0 if emitter == "omni" else 0.0
        if sh.kind == "sphere":
            # an analytic sphere beside the soup: the object frame of T R S must be a similarity
            # (a uniformly scaled rotation) for the centre / radius / rotation record
            msph = trans @ sh.local
            A = msph[:3, :3]
            k = float(np.linalg.norm(A[:, 0]))
            if k <= 0 or not np.allclose(A.T @ A, k * k * np.eye(3), rtol=1e-6, atol=1e-9 * k * k) or \
                    np.linalg.det(A) <= 0:
                raise SceneFileError("a sphere under a non-uniform scale or a reflection is not supported by the "
                                     "GPU path as an analytic sphere (load with tessellate=(nu, nv))")
            mi = self.material_record(self.active)
            if emitter != "null" and self.b.materials[mi][13] != 0:
                raise SceneFileError("a bump-mapped emitter is not supported by the GPU path")
            radiance = None
            if emitter != "null":
                # Sphere::_getSurfaceArea is pi whatever the transform (Sphere.cpp:131-134)
                power = np.broadcast_to(np.asarray(props.get("power", (1.0, 1.0, 1.0)), np.float64), 3)
                radiance = power / (math.pi * per_sr)
            self.b.add_sphere(msph[:3, 3], 0.5 * k, mi, rotation=A / k, radiance=radiance, omni=emitter == "omni")
            return
        if sh.kind == "point":
            # PointShape (PointShape.cpp): its position; area 0, so Le = power / pi or power / 4 pi
            if emitter != "null":
                power = np.broadcast_to(np.asarray(props.get("power", (1.0, 1.0, 1.0)), np.float64), 3)
                rec = np.zeros(16, np.float32)
                rec[0:3] = _xf_points(trans @ sh.local, [(0.0, 0.0, 0.0)])[0]
                rec[9:12] = (0.0, 1.0, 0.0)
                rec[13:16] = power / per_sr
                ext = omni_ext.copy()
                ext[0] = 3
                self.b.add_light(rec, ext)
            return
        mi = self.material_record(self.active)
        if emitter != "null" and self.b.materials[mi][13] != 0:
            raise SceneFileError("a bump-mapped emitter is not supported by the GPU path (its light samples "
                                 "would need the bumped normal)")
        m = trans @ sh.local
        name = sh.kind
        if sh.kind == "plane":
            corners = _xf_points(m, [(-0.5, 0, -0.5), (0.5, 0, -0.5), (0.5, 0, 0.5), (-0.5, 0, 0.5)])
            nrm = _xf_normals(m, [(0.0, 1.0, 0.0)])[0]
            if emitter != "null":
                center = _xf_points(m, [(0, 0, 0)])[0]
                ex = m[:3, :3] @ np.array([1.0, 0.0, 0.0])
                ez = m[:3, :3] @ np.array([0.0, 0.0, 1.0])
                area = float(np.linalg.norm(np.cross(ex, ez)))
                power = np.broadcast_to(np.asarray(props.get("power", (1.0, 1.0, 1.0)), np.float64), 3)
                rec = S.quad_light(center, ex, ez, power / (area * per_sr))
                rec[9:12] = nrm  # emitting side: the transformed +y (inverse transpose)
                li = self.b.add_light(rec, omni_ext)
            else:
                li = -1
            tris = np.array([corners[[0, 3, 2]], corners[[0, 2, 1]]], np.float64)
            # Plane::_getUV (Plane.cpp:52-59): (x + 1/2, z + 1/2) in object space
            cuv = np.array([(0, 0), (1, 0), (1, 1), (0, 1)], np.float64)
            self.b.add(name, tris, np.broadcast_to(nrm, (2, 3, 3)), mi, light=li,
                       uv=np.array([cuv[[0, 3, 2]], cuv[[0, 2, 1]]]))
            return
        power = np.broadcast_to(np.asarray(props.get("power", (1.0, 1.0, 1.0)), np.float64), 3)
        if sh.kind == "triangle":
            vo = sh.data["v"]
            v = _xf_points(m, vo)
            n_obj = np.cross(vo[1] - vo[0], vo[2] - vo[0])
            nrm = _xf_normals(m, [n_obj / np.linalg.norm(n_obj)])[0]
            vi = v[[0, 2, 1]] if np.linalg.det(m[:3, :3]) < 0 else v  # culling follows the object-space winding
            li = -1
            if emitter != "null":
                # Triangle::_getSurfaceArea is the object-space area (Triangle.cpp:356-362)
                obj_area = 0.5 * float(np.linalg.norm(n_obj))
                uv = np.asarray(sh.data["uvs"], np.float64).reshape(3, 2)
                a, b = uv[1] - uv[0], uv[2] - uv[0]
                cross = abs(a[0] * b[1] - a[1] * b[0])
                if cross == 0:
                    raise SceneFileError("an emitting triangle needs a non-degenerate uv frame")
                rec = np.zeros(16, np.float32)
                rec[0:3], rec[3:6], rec[6:9], rec[9:12] = v[0], v[1] - v[0], v[2] - v[0], nrm
                rec[12] = obj_area
                rec[13:16] = power / (obj_area * per_sr)
                ext = omni_ext.copy()
                ext[0] = 1
                ext[1:3], ext[3:5], ext[5:7], ext[7] = uv[0], a, b, 1.0 / cross
                li = self.b.add_light(rec, ext)
            tuv = np.asarray(sh.data["uvs"], np.float64).reshape(3, 2)
            tuv = tuv[[0, 2, 1]] if np.linalg.det(m[:3, :3]) < 0 else tuv
            self.b.add(name, vi[None], np.broadcast_to(nrm, (1, 3, 3)), mi, light=li, culled=True, uv=tuv[None])
            return
        if emitter != "null" and sh.kind != "mesh":
            raise SceneFileError(f"an emitting {sh.kind} is not supported by the GPU path (emitters must be "
                                 "planes, triangles, meshes, spheres or points)")
        if sh.kind == "cube":
            tris, nrms, uvs = [], [], []
            for n_obj, q in _CUBE_FACES:
                q = _xf_points(m, q)
                nw = _xf_normals(m, [n_obj])[0]
                fu = _cube_uv(q, n_obj)
                tris += [q[[0, 1, 2]], q[[0, 2, 3]]]
                nrms += [np.broadcast_to(nw, (3, 3))] * 2
                uvs += [fu[[0, 1, 2]], fu[[0, 2, 3]]]
            self.b.add(name, np.array(tris), np.array(nrms), mi, uv=np.array(uvs))
        elif sh.kind == "mesh":
            verts, faces, normals, nfaces = sh.data["v"], sh.data["f"], sh.data["n"], sh.data["nf"]
            if normals is None:
                normals, nfaces = mesh_vertex_normals(verts, faces), faces
            vw = _xf_points(m, verts)
            inv = np.linalg.inv(m)
            nw = normals @ inv[:3, :3]  # not normalised: interpolated, then normalised per hit
            fuv = sh.data.get("uv")
            if emitter != "null":
                tv = vw[faces]
                area = 0.5 * float(np.linalg.norm(np.cross(tv[:, 1] - tv[:, 0], tv[:, 2] - tv[:, 0]), axis=1).sum())
                li = self.b.add_mesh_light(sh.data["path"], tv, nw[nfaces], power / (area * per_sr), mi, uv=fuv)
                self.b.light_ext[li][15] = omni_ext[15]
            else:
                self.b.add(sh.data["path"], vw[faces], nw[nfaces], mi, uv=fuv)


def material_record(props: dict) -> np.ndarray:
    """Milton material properties -> the 16-float record (defaults of Material.h:61-64,
    DiffuseBSDF, ModifiedPhongBSDF, DielectricBSDF; IndexOfRefraction::AIR)."""
    kind = props.get("bsdf", "diffuse")

    def spec(key, default):
        v = props.get(key, default)
        if isinstance(v, str):
            return np.zeros(3)  # an image map (texture slot) replaces the constant
        return np.broadcast_to(np.asarray(v, np.float64), 3)

    def scalar(key, default):
        v = props.get(key, default)
        if isinstance(v, str):
            if key == "transparency":
                return 1.0  # an image map (texture slot) replaces the constant
            raise SceneFileError(f"'{key}' = '{v}' is not supported by the GPU path")
        a = np.broadcast_to(np.asarray(v, np.float64), 3)
        if not (a[0] == a[1] == a[2]):
            raise SceneFileError(f"per-channel '{key}' {tuple(a)} is not supported by the GPU path")
        return float(a[0])

    ior_v = props.get("ior", S.AIR_IOR)
    if isinstance(ior_v, str):
        raise SceneFileError(f"'ior' = '{ior_v}' is not supported by the GPU path")
    ior = np.broadcast_to(np.asarray(ior_v, np.float64), 3)  # per channel: dispersion
    if kind == "diffuse":
        rec = S.diffuse(spec("kd", 0.5))
    elif kind == "absorbent":
        rec = S.diffuse(0.0)  # black: no reflection, NEE contributes 0, the path ends
    elif kind in ("modifiedPhong", "phong"):
        # ModifiedPhongBSDF::init (:48-60): with ks given kd defaults to black, with only kd
        # given ks does; with neither both are 0.5
        if "ks" in props:
            kd, ks = spec("kd", 0.0), spec("ks", 0.0)
        elif "kd" in props:
            kd, ks = spec("kd", 0.0), spec("ks", 0.0)
        else:
            kd, ks = spec("kd", 0.5), spec("ks", 0.5)
        rec = S.phong(kd, ks, scalar("n", 1.0))
    elif kind == "dielectric":
        rec = S.dielectric(ior=ior, transparency=scalar("transparency", 1.0), ks=spec("ks", 1.0))
    else:
        raise SceneFileError(f"invalid material (BSDF type): {kind}")
    S.set_ior(rec, ior)
    return rec


def camera_record(props: dict, width: int, height: int) -> np.ndarray:
    """ThinLensCamera::init (ThinLensCamera.cpp:62-86, 241-259): defaults eye (2, 2, 2), look
    toward focus (default origin), up = the default camera's v axis."""
    eye = np.asarray(props.get("eye", (2.0, 2.0, 2.0)), np.float64)
    focus = np.asarray(props.get("focus", (0.0, 0.0, 0.0)), np.float64)
    if "look" in props:
        look = np.asarray(props["look"], np.float64)
    else:
        d = focus - eye
        look = d / np.linalg.norm(d)
    n0 = np.array([1.0, 1.0, 1.0]) / math.sqrt(3.0)
    u0 = np.cross(np.array([0.0, 1.0, 0.0]), n0)
    u0 /= np.linalg.norm(u0)
    up = np.asarray(props.get("up", np.cross(n0, u0)), np.float64)
    ln = look / np.linalg.norm(look)
    if abs(abs(float(ln @ (up / np.linalg.norm(up)))) - 1.0) < 1e-7:
        up = np.array([0.0, 1.0, 0.0]) if not np.array_equal(up, [0.0, 1.0, 0.0]) else np.array([0.0, 0.0, 1.0])
    cam = np.zeros(16, np.float32)
    cam[0:3] = eye
    cam[3:6] = ln
    cam[6:9] = up
    cam[9] = props.get("heightAngle", 45.0)
    cam[10] = props.get("aspectRatio", 1.0)
    cam[13] = 1.0
    # PinholeCamera::init forces aperture 0 (PinholeCamera.cpp); a thin lens defaults to a 35 mm
    # aperture and f/14, focal length = fstop x aperture (ThinLensCamera.cpp:88-95)
    if props.get("type") == "thinlens":
        aperture = float(props.get("aperture", 35.0)) / 1000.0
        cam[11] = aperture
        cam[12] = float(props.get("fstop", 14.0)) * aperture
        if "focalPoint" in props or "focalDistance" not in props:
            # autofocus on the scene (ThinLensCamera.cpp:97-121): resolved once the scene is
            # resident (pathtracer.resolve_autofocus); -fallback marks it, the point follows
            fp = props.get("focalPoint", (0.5, 0.5))
            cam[13] = -float(props.get("focalDistance", 1.0))
            cam[14], cam[15] = fp[0], fp[1]
        else:
            cam[13] = float(props["focalDistance"])
    return cam


@dataclass
class SceneFile:
    scene: S.Scene
    renderer: dict
    camera: dict
    output: dict
    width: int
    height: int
    source: str = ""

    def path_tracer_props(self) -> dict:
        """The renderer's PropertyMap for pathtracer.PathTracer (type 'pathTracer' or a dynamic
        renderer plugin)."""
        t = self.renderer.get("type")
        if t not in ("pathTracer", "dynamic"):
            raise SceneFileError(f"renderer '{t}' is not the path tracer")
        return {k: v for k, v in self.renderer.items() if k not in ("type", "path")}


def _unit_sphere(nu: int, nv: int):
    """The UV sphere of scenegen (radius 1/2) with Sphere::_getUV at its vertices
    (Sphere.cpp:78-85: u = 1 - atan2(z, x) / 2 pi, v = 1/2 - asin(2 y) / pi), u taken continuous
    in the longitude so that no triangle straddles the seam (the fractional part, which is all
    a lookup uses, is the reference's)."""
    from .scenegen import _uv_sphere_fast
    tris, nrm = _uv_sphere_fast((0.0, 0.0, 0.0), 0.5, nu, nv)
    th = np.linspace(0.0, np.pi, nv + 1)
    ph = np.linspace(0.0, 2 * np.pi, nu + 1)
    T, PH = np.meshgrid(th, ph, indexing="ij")
    uvg = np.stack([1.0 - PH / (2 * np.pi), T / np.pi], -1)
    i, j = np.meshgrid(np.arange(nv), np.arange(nu), indexing="ij")
    a, b, cc, d = (i, j), (i, j + 1), (i + 1, j + 1), (i + 1, j)
    u1 = np.stack([uvg[a], uvg[d], uvg[b]], -2)
    u2 = np.stack([uvg[b], uvg[d], uvg[cc]], -2)
    keep = np.stack([i != 0, i != nv - 1], 2)
    return tris, nrm, np.stack([u1, u2], 2)[keep].astype(np.float32)


def loads(text: str, base_dir: str = ".", source: str = "<string>", tessellate=None) -> SceneFile:
    """Parses already-read scene text (see read_scene_text for how a file becomes text).
    tessellate=(nu, nv) turns spheres into UV spheres of that resolution (an approximation of
    Milton's Sphere; without it they are analytic spheres)."""
    ld = _Loader(base_dir, tessellate)
    ld.root_obj(parse_text(text))
    fl = _Flattener(ld.named, base_dir)
    fl.run(ld.root)
    fl.background(ld.bg)
    out = dict(ld.output_props)
    w, h, found = 480, 480, False
    for key in ("size", "dimensions"):
        if key in out:
            nw, nh = int(out[key][0]), int(out[key][1])
            if found and (nw, nh) != (w, h):
                raise SceneFileError("conflicting declarations of output size")
            w, h, found = nw, nh, True
    if "width" in out:
        if found and out["width"] != w:
            raise SceneFileError("conflicting definitions for output width")
        w = out["width"]
    if "height" in out:
        h = out["height"]
    out["width"], out["height"] = w, h
    if ld.output:
        out.update(ld.output)
    cam_props = dict(ld.camera or {"type": "pinhole"})
    cam = camera_record(cam_props, w, h)
    scene = fl.b.build(cam, name=os.path.basename(source))
    if not scene.textures:
        scene.tri_uv = None  # uvs only matter to image maps
    return SceneFile(scene=scene, renderer=dict(ld.renderer or {"type": "preview"}), camera=cam_props, output=out,
                     width=w, height=h, source=source)


def load(path: str, tessellate=None) -> SceneFile:
    """Loads a Milton scene file (MiltonJSONSceneLoader::parse); mesh paths are taken relative
    to the scene file's directory when not absolute."""
    return loads(read_scene_text(path), base_dir=os.path.dirname(os.path.abspath(path)), source=path,
                 tessellate=tessellate)


def path_tracer(sf: SceneFile):
    """A pathtracer.PathTracer set up from a loaded scene file (scene, output size and the
    renderer's keys), as Milton's loader hands scene, camera and output to the renderer
    (MiltonJSONSceneLoader::_finalizeData, :229-336)."""
    from .pathtracer import PathTracer
    r = PathTracer(sf.path_tracer_props())
    r.set_scene(sf.scene)
    r.set_output(sf.width, sf.height)
    r.output_filter = sf.output.get("filter")
    return r
