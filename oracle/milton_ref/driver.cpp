// driver.cpp -- test-oracle driver around Milton's own intersection code.
//
// Test infrastructure only: this program is linked with the reference's unmodified
// kdTreeAccel / Mesh / MeshTriangle / Triangle / ShapeSet / NaiveSpatialAccel sources
// (compiled from the reference tree by oracle/milton_ref/build.py) and answers ray queries the
// way Milton's Scene does:
//   closest   Scene::getIntersection -> ShapeSet::getIntersection (mlt/src/milton/core/Scene.cpp:104-108,
//             mlt/src/milton/shapes/ShapeSet.cpp:102-111), a kd-tree over the shapes and one per Mesh
//             (mlt/src/milton/shapes/Mesh.cpp:210-250, mlt/src/milton/accel/kdTreeAccel.cpp:893-1016)
//   any       Scene::intersects(ray, tMax) = ShapeSet::intersects(ray, tMax - EPSILON)
//             (mlt/src/milton/core/Scene.cpp:110-114, mlt/src/milton/accel/kdTreeAccel.cpp:1018-1094)
// With "_naive" appended the ShapeSet and every Mesh use NaiveSpatialAccel ("spatialAccel":
// "naive", mlt/src/milton/shapes/Mesh.cpp:222-233): Milton's own brute force.
//
// The scene is the flattened soup in ShapeSet order: each shape is either a Milton Mesh
// (two-sided MeshTriangles, identity transform) or a run of standalone, back-face culled Milton
// Triangles.  A hit reports the global primitive id = the shape's first id + the triangle's
// index inside the Mesh (the (pt.shape, pt.index) pair, kdTreeAccel.cpp:991-993).
//
// kdTreeAccel stores child pointers in 32 bits (kdTreeAccel.cpp:78-85, 117-126), so the program
// is linked without PIE (its malloc heap then starts below 4 GiB) and refuses to answer if the
// heap ended above 4 GiB.
//
// Files (little endian):
//   scene  "MRSC" u32 version(1) u32 nshapes, kd params (u32 minPrims, u32 maxDepth,
//          f64 costTraversal, f64 emptyBias), then per shape: u32 kind (0 Mesh, 1 culled
//          Triangles), u32 ntri, u64 first id, ntri*9 f64 vertices, ntri*9 f64 normals
//   rays   "MRRY" u32 version(1) u64 n, n * 7 f64: origin, direction, tMax (any-hit only)
//   out    closest: n * (f64 t, i64 id) (t = inf, id = -1 on a miss); any: n * u8
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include <map>
#include <string>
#include <vector>

#include <Material.h>
#include <Mesh.h>
#include <ResourceManager.h>
#include <ShapeSet.h>
#include <SurfacePoint.h>
#include <Triangle.h>
#include <common/image/Image.h>
#include <core/Ray.h>

using namespace milton;

namespace {

struct Reader {
  FILE *f;
  explicit Reader(const char *path) : f(fopen(path, "rb")) {
    if (!f) die("cannot open", path);
  }
  ~Reader() { fclose(f); }
  template <typename T> T get() {
    T v;
    if (fread(&v, sizeof(T), 1, f) != 1) die("short read", "");
    return v;
  }
  void getn(void *dst, size_t bytes) {
    if (bytes && fread(dst, 1, bytes, f) != bytes) die("short read", "");
  }
  [[noreturn]] static void die(const char *what, const char *arg) {
    fprintf(stderr, "milton_ref: %s %s\n", what, arg);
    exit(2);
  }
};

struct SceneBuild {
  ShapeSet *set = nullptr;
  std::map<const Shape *, int64_t> base;  // shape -> first global id
  std::map<const Shape *, bool> is_mesh;
};

SceneBuild load_scene(const char *path, bool naive) {
  Reader r(path);
  char magic[4];
  r.getn(magic, 4);
  if (memcmp(magic, "MRSC", 4) != 0 || r.get<uint32_t>() != 1) Reader::die("bad scene file", path);
  uint32_t nshapes = r.get<uint32_t>();
  uint32_t min_prims = r.get<uint32_t>(), max_depth = r.get<uint32_t>();
  double cost_trav = r.get<double>(), empty_bias = r.get<double>();
  SceneBuild sb;
  sb.set = new ShapeSet();
  sb.set->setMaterial(new Material());
  const std::string accel = naive ? "naive" : "kdTree";
  auto kd_props = [&](PropertyMap &m) {
    m["spatialAccel"] = accel;
    m["kdMinPrimitives"] = (unsigned)min_prims;
    m["kdMaxDepth"] = (unsigned)max_depth;
    m["kdCostTraversal"] = (real_t)cost_trav;
    m["kdEmptyBias"] = (real_t)empty_bias;
  };
  kd_props(*sb.set);
  for (uint32_t s = 0; s < nshapes; ++s) {
    uint32_t kind = r.get<uint32_t>(), ntri = r.get<uint32_t>();
    int64_t first = (int64_t)r.get<uint64_t>();
    std::vector<double> v(9 * (size_t)ntri), n(9 * (size_t)ntri);
    r.getn(v.data(), v.size() * sizeof(double));
    r.getn(n.data(), n.size() * sizeof(double));
    if (kind == 0) {
      MeshData md;
      md.vertices.resize(3 * (size_t)ntri);
      md.normals.resize(3 * (size_t)ntri);
      for (size_t k = 0; k < 3 * (size_t)ntri; ++k) {
        md.vertices[k] = Vertex(v[3 * k], v[3 * k + 1], v[3 * k + 2]);
        md.normals[k] = Normal(n[3 * k], n[3 * k + 1], n[3 * k + 2]);
      }
      for (uint32_t t = 0; t < ntri; ++t)
        md.triangles.push_back(MeshTriangle(3 * t, 3 * t + 1, 3 * t + 2, 3 * t, 3 * t + 1, 3 * t + 2));
      Mesh *mesh = new Mesh(md);
      mesh->setMaterial(new Material());
      kd_props(*mesh);
      sb.set->push_back(mesh);
      sb.base[mesh] = first;
      sb.is_mesh[mesh] = true;
    } else if (kind == 1) {
      for (uint32_t t = 0; t < ntri; ++t) {
        Vertex vs[3];
        Normal ns[3];
        for (int k = 0; k < 3; ++k) {
          const double *p = &v[9 * (size_t)t + 3 * k], *q = &n[9 * (size_t)t + 3 * k];
          vs[k] = Vertex(p[0], p[1], p[2]);
          ns[k] = Normal(q[0], q[1], q[2]);
        }
        Triangle *tri = new Triangle(vs, ns);
        tri->setMaterial(new Material());
        sb.set->push_back(tri);
        sb.base[tri] = first + t;
        sb.is_mesh[tri] = false;
      }
    } else {
      Reader::die("unknown shape kind", path);
    }
  }
  sb.set->init();
  return sb;
}

}  // namespace

int main(int argc, char **argv) {
  if (argc != 5) {
    fprintf(stderr, "usage: milton_ref closest|any[_naive] scene.bin rays.bin out.bin\n");
    return 2;
  }
  const std::string mode = argv[1];
  const bool naive = mode.size() > 6 && mode.compare(mode.size() - 6, 6, "_naive") == 0;
  const bool any = mode.rfind("any", 0) == 0;
  if (!any && mode.rfind("closest", 0) != 0) Reader::die("unknown mode", argv[1]);
  SceneBuild sb = load_scene(argv[2], naive);
  // every kd node came from malloc's brk heap, which must end below 4 GiB for the 32-bit
  // child pointers of kdTreeAccel to hold
  if ((uintptr_t)sbrk(0) >= ((uintptr_t)1 << 32)) Reader::die("heap above 4 GiB: kd child pointers truncated", "");

  Reader rr(argv[3]);
  char magic[4];
  rr.getn(magic, 4);
  if (memcmp(magic, "MRRY", 4) != 0 || rr.get<uint32_t>() != 1) Reader::die("bad ray file", argv[3]);
  uint64_t n = rr.get<uint64_t>();
  std::vector<double> rays(7 * n);
  rr.getn(rays.data(), rays.size() * sizeof(double));
  FILE *out = fopen(argv[4], "wb");
  if (!out) Reader::die("cannot write", argv[4]);
  std::vector<unsigned char> buf;
  buf.reserve(any ? n : 16 * n);
  for (uint64_t i = 0; i < n; ++i) {
    const double *q = &rays[7 * i];
    Ray ray(Point3(q[0], q[1], q[2]), Vector3(q[3], q[4], q[5]));
    if (any) {
      buf.push_back(sb.set->intersects(ray, q[6] - EPSILON) ? 1 : 0);
      continue;
    }
    SurfacePoint pt;
    double t = sb.set->getIntersection(ray, pt);
    int64_t id = -1;
    if (Ray::isValid(t)) {
      auto it = sb.base.find(pt.shape);
      if (it == sb.base.end()) Reader::die("hit an unknown shape", "");
      id = it->second + (sb.is_mesh[pt.shape] ? (int64_t)pt.index : 0);
    } else {
      t = INFINITY;
    }
    const unsigned char *pb = reinterpret_cast<const unsigned char *>(&t);
    buf.insert(buf.end(), pb, pb + 8);
    pb = reinterpret_cast<const unsigned char *>(&id);
    buf.insert(buf.end(), pb, pb + 8);
  }
  if (fwrite(buf.data(), 1, buf.size(), out) != buf.size()) Reader::die("short write", argv[4]);
  fclose(out);
  return 0;
}
